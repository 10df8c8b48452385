"""The allocation-free solve entry point against the regular one.

ikr_linear_solver_solve_noalloc serves callers that may not allocate device memory once they are running
(a device-memory budget fixed at start-up, or allocations that must all go through the caller's own
allocator): its CG work set lives in a fixed device array inside the library.  The caller still provides
the right-hand side and the solution buffer.  This test calls it through the C ABI twice in a row and
compares both results with ikr_linear_solver_solve on the same assembled tangent, checks the residual of
each result against the oracle's FP64 tangent, and checks that the second call leaves the device's free
memory unchanged (the first call on a device may still commit the library's fixed array when CUDA loads
device code lazily).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _solve_noalloc(ikr, asm, b_dev, x_dev, rtol, max_iter=100000):
    its = C.c_int32()
    code = ikr.lib().ikr_linear_solver_solve_noalloc(asm.h, C.c_void_p(b_dev), C.c_void_p(x_dev), rtol, max_iter,
                                                     C.byref(its))
    return code, its.value


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_solve_matches_regular_solve_twice(ikr, precision):
    torch = pytest.importorskip("torch")
    p = problems.cantilever(12, 3, 3, jitter=0.1, seed=4)
    fes, asm = problems.build_gpu(p, precision=precision)
    u = 0.01 * np.random.default_rng(1).standard_normal(p.n_dofs) * (1 - p.fixed)
    req = ikr.FERequirements(fes, u, 0.5)
    asm.matrix(req, dbc=ikr.DBCOption.Full, export=False)
    b = np.random.default_rng(2).standard_normal(p.n_dofs) * (1 - p.fixed)
    rtol = RTOL if precision == 0 else 1e-5

    ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol)
    ls.compute(asm)
    x_ref = ls.solve(asm, b)

    # the oracle's FP64 tangent at the same state: K x - b of every result
    sp = pytest.importorskip("scipy.sparse")
    cp, ri, v, n = oracle.from_problem(p).assemble_matrix_csc(u, 0.5)
    K = sp.csc_matrix((v, ri, cp), shape=(n, n))
    # FP64: the CG's own tolerance plus round-off; FP32: the FP32 tangent's rounding (entries within 2e-6 of the
    # FP64 ones) times this small system's condition number adds to the 1e-5 of the FP32 CG
    res_tol = 1e-11 if precision == 0 else 1e-3

    b_dev = torch.tensor(b, dtype=torch.float64, device="cuda")
    for call in range(2):  # the shared scratch keeps the previous call's contents; results must not depend on it
        x_dev = torch.full((p.n_dofs,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        code, its = _solve_noalloc(ikr, asm, b_dev.data_ptr(), x_dev.data_ptr(), rtol)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert code == 0, (call, code)
        assert its > 0
        if call == 1:
            assert free_after == free_before, (free_before, free_after)
        x = x_dev.cpu().numpy()
        tol = 1e-10 if precision == 0 else 1e-4
        assert np.abs(x - x_ref).max() <= tol * np.abs(x_ref).max(), call
        rel = np.linalg.norm(K @ x - b) / np.linalg.norm(b)
        print(f"noalloc precision {precision} call {call}: ||K64 x - b|| / ||b|| = {rel:.3e} ({its} iterations)")
        assert rel <= res_tol, (call, rel)


def test_noalloc_rejects_systems_above_its_limit(ikr):
    torch = pytest.importorskip("torch")
    p = problems.cantilever(40, 30, 30)  # 41 * 31 * 31 = 39401 nodes > 32768
    fes, asm = problems.build_gpu(p)
    b = torch.zeros(p.n_dofs, dtype=torch.float64, device="cuda")
    x = torch.zeros(p.n_dofs, dtype=torch.float64, device="cuda")
    code, _ = _solve_noalloc(ikr, asm, b.data_ptr(), x.data_ptr(), 1e-8)
    assert code == -1
    buf = C.create_string_buffer(512)
    ikr.lib().ikr_last_error(buf, 512)
    assert b"at most 32768 nodes" in buf.value
