"""FP64 outer solve of the mixed form (flexible GMRES on the FP64 tangent, preconditioned by the FP32 CG on its
FP32 rounding) against the oracle: linear solves reach FP64 accuracy with respect to the oracle's FP64 tangent, and
a nearly incompressible EAS load path (nu = 0.4999) converges to the oracle's solution."""
import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu
sp = pytest.importorskip("scipy.sparse")


def small_block(load_steps=3, pressure=10.0):
    return problems.eas_block(nx=12, ny=12, nz=3, pressure=pressure, load_steps=load_steps)


def test_fp64_outer_solve_reaches_fp64_residual_of_the_oracle_tangent(ikr, parity_log):
    p = small_block()
    o = oracle.from_problem(p)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(p.n_dofs) * (1 - p.fixed)
    cp, ri, v, n = o.assemble_matrix_csc(None, 0.0)
    K = sp.csc_matrix((v, ri, cp), shape=(n, n))
    fes, asm = problems.build_gpu(p, precision=1)
    req = ikr.FERequirements(fes)
    # FP32 CG alone: its residual against the FP64 tangent stalls at the FP32 tangent's rounding error
    ls32 = ikr.LinearSolver(rtol=1e-10, max_iter=20000)
    asm.matrix(req, dbc=ikr.DBCOption.Full, export=False)
    ls32.compute(asm)
    try:
        x32 = ls32.solve(asm, b)
        r32 = np.linalg.norm(K @ x32 - b) / np.linalg.norm(b)
    except ikr.IkarusError:  # the FP32 CG may also break down on its way to 1e-10
        r32 = np.inf
    # FP64 outer solve (the twin is assembled after analyzePattern switched it on)
    ls = ikr.LinearSolver(rtol=1e-10)
    ls.set_fp64_outer(restart=20, inner_rtol=1e-2)
    ls.analyzePattern(asm)
    asm.matrix(req, dbc=ikr.DBCOption.Full, export=False)
    ls.factorize(asm)
    x = ls.solve(asm, b)
    rel = np.linalg.norm(K @ x - b) / np.linalg.norm(b)
    outer, cycles = ls.outer_info()
    inner, rel_dev = ls.last_info()
    print(f"FP32 CG alone: {r32:.3e}; FP64 outer: {rel:.3e} ({outer} outer, {cycles} cycles, {inner} inner CG)")
    assert rel_dev <= 1e-10 and outer > 0 and inner > 0
    assert parity_log("fp64-outer solve: ||K64_oracle x - b|| / ||b||", rel, 2e-10)
    # repeat: bit-identical
    assert np.array_equal(ls.solve(asm, b), x)


def test_fp64_outer_without_the_twin_is_an_invalid_state(ikr):
    p = small_block()
    fes, asm = problems.build_gpu(p, precision=1)
    req = ikr.FERequirements(fes)
    ls = ikr.LinearSolver(rtol=1e-8)
    asm.matrix(req, dbc=ikr.DBCOption.Full, export=False)
    ls.compute(asm)
    ls.set_fp64_outer(restart=10)
    with pytest.raises(ikr.IkarusError, match="INVALID_STATE"):
        ls.solve(asm, np.ones(p.n_dofs) * (1 - p.fixed))
    with pytest.raises(ikr.IkarusError, match="ARG"):
        ls.set_fp64_outer(restart=64)


def test_mixed_nearly_incompressible_eas_path_matches_oracle(ikr, parity_log):
    """12x12x3 block, GL-E9, nu = 0.4999, 3 load steps: mixed form with the FP64 outer solve and
    Eisenstat-Walker forcing reaches ||R|| <= 1e-10 ||R0|| every step and the oracle's displacement within 1e-8."""
    p = small_block()
    ref = oracle.from_problem(p).load_control(p.load_steps, tol=1e-10, tol_mode=1, max_iter=40)
    fes, asm = problems.build_gpu(p, precision=1)
    req = ikr.FERequirements(fes)
    ls = ikr.LinearSolver()
    ls.set_fp64_outer(restart=20, inner_rtol=1e-2)
    st = ikr.NRSettings(tol=1e-10, maxIter=40, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-12)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ls))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    u = req.globalSolution()
    err = np.abs(u - ref["u"]).max() / np.abs(ref["u"]).max()
    print("Newton iterations per step: device", [s.iterations for s in info.solverInfos], "oracle",
          list(ref["iterations"]))
    assert parity_log("nearly incompressible EAS 12x12x3, mixed + FP64 outer: max|u - u_oracle| / max|u_oracle|",
                      err, 1e-8)
