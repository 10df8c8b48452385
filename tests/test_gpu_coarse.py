"""GPU tests of the CG's coarse correction (coarse.cu, LinearSolver.set_coarse_space): an additive two-level
preconditioner, block Jacobi plus P A_c^-1 P^T with the rigid-body modes of slabs of nodes.

It changes the preconditioner only, so a converged solve is the same solution: FP64 solves within 1e-9 of the
oracle's direct solve (relative to the largest entry), FP32 solves within their own tolerance, Newton runs the
same iterations as the plain block-Jacobi CG and ends within 1e-8 of the oracle's load path.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu


def _system(ikr, p, precision, lam=0.1):
    """Tangent at u = 0 (Full DBC) on the device, a load vector and the oracle's direct FP64 solution."""
    fes, asm = problems.build_gpu(p, precision=precision)
    req = ikr.FERequirements(fes)
    req.insertParameter(lam)
    asm.matrix(req, dbc=ikr.DBCOption.Full)
    o = oracle.from_problem(p)
    cp, ri, va, n = o.assemble_matrix_csc(np.zeros(p.n_dofs), lam)
    b = -o.assemble_vector(np.zeros(p.n_dofs), lam)
    x_ref = sla.spsolve(sp.csc_matrix((va, ri, cp), shape=(n, n)), b)
    return fes, asm, req, b, x_ref


def _solve(ikr, asm, b, slabs, rtol):
    ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol)
    ls.set_coarse_space(slabs)
    ls.compute(asm)
    x = ls.solve(asm, b)
    it, rel = ls.last_info()
    return x, it, rel, ls


# FP32: rounding the tangent to FP32 alone moves this system's solution by 2.9e-4 of its largest entry (kappa
# about 1.1e6), so the FP32 solves are compared with the FP64 solution at 2e-3 and with each other at 1e-3
@pytest.mark.parametrize("precision,rtol,tol,tol_pair", [(0, 1e-12, 1e-9, 1e-9), (1, 1e-5, 2e-3, 1e-3)],
                         ids=["fp64", "fp32"])
def test_coarse_correction_gives_the_same_solution_in_fewer_iterations(ikr, precision, rtol, tol, tol_pair):
    p = problems.cantilever(32, 4, 4, jitter=0.1, seed=3)
    fes, asm, req, b, x_ref = _system(ikr, p, precision)
    x0, it0, rel0, _ = _solve(ikr, asm, b, 0, rtol)
    x1, it1, rel1, ls = _solve(ikr, asm, b, 8, rtol)
    scale = np.abs(x_ref).max()
    assert np.abs(x0 - x_ref).max() <= tol * scale
    assert np.abs(x1 - x_ref).max() <= tol * scale
    assert np.abs(x1 - x0).max() <= tol_pair * scale
    assert rel1 <= rtol
    assert it1 < 0.5 * it0, (it0, it1)
    info = ls.coarse_info()
    assert info["slabs"] == 8 and info["coarse_dofs"] == 48 and info["colours"] == 3
    # the clamped end keeps free interior nodes in its slab: no mode is dependent
    assert info["dropped_modes"] == 0
    # fixed-order sums: the same solve twice is bit-identical
    x2 = ls.solve(asm, b)
    np.testing.assert_array_equal(x1, x2)
    # constrained dofs stay zero
    assert np.all(x1[p.fixed == 1] == 0.0)


@pytest.mark.parametrize("precision,rtol,tol_pair", [(0, 1e-12, 1e-9), (1, 1e-5, 1e-3)], ids=["fp64", "fp32"])
def test_fused_coarse_kernel_matches_the_two_kernel_form(ikr, precision, rtol, tol_pair):
    """The persistent kernel with the coarse correction in the same launch (cg_coarse.cu) applies the same
    preconditioner as the two-kernel form (coarse.cu): the same solution to the solve tolerance, about the same
    iteration count, the requested tolerance reached, bit-identical repeats, and the tuner picks it."""
    p = problems.cantilever(32, 4, 4, jitter=0.1, seed=3)
    fes, asm, req, b, x_ref = _system(ikr, p, precision)
    kinds = ikr.LinearSolver.kind_ranges()
    ls2 = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol)
    ls2.set_kernel(1, 0.0)  # a two-kernel (staged) form
    ls2.set_coarse_space(8)
    ls2.compute(asm)
    x2 = ls2.solve(asm, b)
    it2, _ = ls2.last_info()
    for variant in range(kinds["coarse_fused"], kinds["count"]):
        lsf = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol)
        lsf.set_kernel(variant, 0.45)
        lsf.set_coarse_space(8)
        lsf.compute(asm)
        xf = lsf.solve(asm, b)
        itf, relf = lsf.last_info()
        scale = np.abs(x_ref).max()
        assert np.abs(xf - x2).max() <= tol_pair * scale, variant
        assert relf <= rtol
        assert abs(itf - it2) <= max(3, 0.1 * it2), (variant, itf, it2)
        np.testing.assert_array_equal(lsf.solve(asm, b), xf)
        assert np.all(xf[p.fixed == 1] == 0.0)
    lst = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol)
    lst.set_coarse_space(8)
    lst.compute(asm)
    assert lst.kernel_info()[0] >= kinds["coarse_fused"]
    # a fused kind without a coarse space is an argument error
    lsb = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=rtol)
    lsb.set_kernel(kinds["coarse_fused"], 0.0)
    with pytest.raises(ikr.IkarusError):
        lsb.compute(asm)


def test_coarse_correction_with_single_slab_and_many_slabs(ikr):
    """One slab (the six global rigid-body modes) and one slab per node layer, where the clamped layer has no free
    dof and its six modes are dropped."""
    p = problems.cantilever(16, 2, 2, jitter=0.1, seed=4)
    fes, asm, req, b, x_ref = _system(ikr, p, 0)
    for slabs, dropped in ((1, 0), (17, 6)):
        x, it, rel, ls = _solve(ikr, asm, b, slabs, 1e-12)
        assert np.abs(x - x_ref).max() <= 1e-9 * np.abs(x_ref).max(), slabs
        info = ls.coarse_info()
        assert info["slabs"] == slabs and info["dropped_modes"] == dropped


def test_newton_with_coarse_correction_matches_the_oracle(ikr):
    p = problems.config1()
    o = oracle.from_problem(p)
    ref = o.load_control(p.load_steps, tol=p.tol)
    fes, asm = problems.build_gpu(p, precision=0)
    req = ikr.FERequirements(fes)
    ls = ikr.LinearSolver(rtol=1e-12)
    ls.set_coarse_space(4)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(tol=p.tol, linear_rtol=1e-12), ls))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    assert [s.iterations for s in info.solverInfos] == list(ref["iterations"])
    u = req.globalSolution()
    assert np.abs(u - ref["u"]).max() <= 1e-8 * np.abs(ref["u"]).max()


def test_mixed_newton_with_coarse_correction(ikr):
    p = problems.config1()
    o = oracle.from_problem(p)
    ref = o.load_control(p.load_steps, tol=1e-8, tol_mode=1)
    fes, asm = problems.build_gpu(p, precision=1)
    req = ikr.FERequirements(fes)
    st = ikr.NRSettings(tol=1e-8, relative=True, eisenstat_walker=True, linear_rtol=1e-2, linear_rtol_min=1e-6)
    ls = ikr.LinearSolver(rtol=1e-4)
    ls.set_coarse_space(4)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ls))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    assert np.abs(req.globalSolution() - ref["u"]).max() <= 1e-6 * np.abs(ref["u"]).max()


def test_coarse_correction_argument_errors(ikr):
    ls = ikr.LinearSolver()
    for bad in (-1, 129):
        with pytest.raises(ikr.IkarusError):
            ls.set_coarse_space(bad)
    assert ls.coarse_info() == {"slabs": 0, "coarse_dofs": 0, "dropped_modes": 0, "colours": 0}
    with pytest.raises(ikr.IkarusError) as e:
        ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_Batched).set_coarse_space(4)
    assert e.value.code == -2
    # persistent CG kinds do not take the correction
    p = problems.cantilever(8, 2, 2)
    fes, asm = problems.build_gpu(p, precision=1)
    req = ikr.FERequirements(fes)
    asm.matrix(req, dbc=ikr.DBCOption.Full)
    ls = ikr.LinearSolver()
    ls.set_kernel(5, 0.0)
    ls.set_coarse_space(2)
    with pytest.raises(ikr.IkarusError):
        ls.compute(asm)
