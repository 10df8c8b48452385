"""Every CG kernel choice (direct-load SpMV, the bulk-copy staged SpMV variants, the persistent cooperative CG,
with and without the L2 keep policy) and both launch modes (CUDA graphs, kernel by kernel) solve the same
system to the same tolerance, each run to run bit-identical; the tuner picks one of them and reports it."""
import numpy as np
import pytest

from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu

def true_residual_bound(fp32):
    """Relative true residual |K x - b| / |b| (FP64 arithmetic on the stored tangent) a converged solve reaches.
    FP64: the CG tolerance.  FP32: the recursively updated CG residual drifts from the true one by about
    eps_32 * cond(K) (6e-8 * 2.4e5 here), so the bound is 2e-3; the FP64 Newton residual corrects this."""
    return 2e-3 if fp32 else 1e-10


# 0 direct-load SpMV, 1-4 staged SpMV variants, 5-11 persistent CG variants, 12-13 one-reduction persistent CG;
# keep = L2 evict_last share
KINDS = [(0, 0.0), (1, 0.0), (2, 0.0), (3, 0.0), (4, 0.0), (1, 0.5), (2, 0.75), (5, 0.0), (6, 0.0), (7, 0.0),
         (8, 0.0), (9, 0.0), (10, 0.0), (11, 0.0), (5, 0.4), (12, 0.0), (13, 0.0), (12, 0.45)]


@pytest.fixture(scope="module", params=[0, 1], ids=["fp64", "fp32"])
def system(request, ikr):
    # 12x5x3 elements: 13 * 6 * 4 = 312 nodes, so ten slices of 32 rows with a ragged last slice
    p = problems.cantilever(12, 5, 3, L=6.0, jitter=0.1, seed=3)
    fes, asm = problems.build_gpu(p, precision=request.param)
    # a random state small enough that the tangent stays positive definite (min eigenvalue 0.018 at 0.003)
    req = ikr.FERequirements(fes, 0.003 * np.random.default_rng(1).standard_normal(p.n_dofs) * (1 - p.fixed), 0.3)
    K = asm.matrix(req, dbc=ikr.DBCOption.Full)
    b = np.random.default_rng(0).standard_normal(p.n_dofs) * (1 - p.fixed)
    return request.param, p, asm, K, b


@pytest.mark.parametrize("kind,keep", KINDS)
@pytest.mark.parametrize("graphs", [True, False], ids=["graphs", "direct"])
def test_spmv_kernel_solves(ikr, system, kind, keep, graphs):
    fp32, p, asm, K, b = system
    rtol = 1e-5 if fp32 else 1e-11
    ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol, max_iter=20000)
    ls.set_kernel(kind, keep)
    ls.set_launch(use_graphs=graphs, chunk_len=8)
    ls.compute(asm)
    assert ls.kernel_info()[0] == kind
    x1 = ls.solve(asm, b)
    it1, rel1 = ls.last_info()
    x2 = ls.solve(asm, b)
    assert np.array_equal(x1, x2), "repeated solve is not bit-identical"
    assert 0 < it1 and rel1 <= rtol
    assert np.linalg.norm(K @ x1 - b) <= true_residual_bound(fp32) * np.linalg.norm(b)


def test_tuner_choice_is_reported(ikr, system):
    fp32, p, asm, K, b = system
    ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=1e-5 if fp32 else 1e-11)
    ls.compute(asm)
    kind, keep, us = ls.kernel_info()
    assert 0 <= kind <= 13 and 0.0 <= keep < 1.0 and us > 0.0
    x = ls.solve(asm, b)
    assert np.linalg.norm(K @ x - b) <= true_residual_bound(fp32) * np.linalg.norm(b)


@pytest.mark.parametrize("kind", [5, 6, 7, 8, 9, 10, 11])
def test_two_rhs_persistent_solve_matches_two_solves(ikr, system, kind):
    """Two right-hand sides in one persistent launch (the matrix streamed once per iteration for both) give
    bit-identical solutions and the same iteration counts as two single solves: each RHS keeps its own scalars and
    the reductions sum in the same order."""
    fp32, p, asm, K, b = system
    b2 = np.random.default_rng(5).standard_normal(p.n_dofs) * (1 - p.fixed)
    rtol = 1e-5 if fp32 else 1e-11
    ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol, max_iter=20000)
    ls.set_kernel(kind, 0.0)
    ls.compute(asm)
    xa = ls.solve(asm, b)
    ita = ls.last_info()[0]
    xb = ls.solve(asm, b2)
    itb = ls.last_info()[0]
    X = ls.solve(asm, np.stack([b, b2], axis=1))
    assert ls.last_info()[0] == ita + itb
    assert np.array_equal(X[:, 0], xa) and np.array_equal(X[:, 1], xb)
    ls.set_multi_rhs(False)
    Y = ls.solve(asm, np.stack([b, b2], axis=1))
    assert np.array_equal(X, Y)
