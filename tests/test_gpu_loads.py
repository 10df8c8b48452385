"""Loads given as functions f(X, lambda) against the oracle's restatement: VolumeLoad (loads/volume.hh:86-106) at the
element's Gauss points and neumannBoundaryLoad with a general traction function (loads/traction.hh:105-138), alone
and together with the lambda-linear traction, for element vectors, energies, the assembled force vector at two load
factors (the functions are re-evaluated when lambda changes) and a load path whose load is not linear in lambda; and
inhomogeneous Dirichlet values given as a function of (X, lambda)."""
import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems
from ikarus_gb300.mesh import boundary_faces

pytestmark = pytest.mark.gpu
FP64_RTOL = 1e-12


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def body(X, lam):
    return np.stack([0.0 * X[:, 0], 0.1 * lam * np.sin(X[:, 0]), -lam ** 2 * (1.0 + X[:, 2])], axis=1)


def top(X, lam):
    return np.stack([0.2 * lam * X[:, 0], 0.0 * X[:, 0], -0.5 * lam ** 3 + 0.1 * X[:, 1]], axis=1)


def with_function_loads(p, target, scale=1.0):
    target.add_volume_load(lambda X, lam: scale * body(X, lam))
    fe, fl = boundary_faces(p.mesh, "z+")
    target.add_neumann_function(fe, fl, lambda X, lam: scale * top(X, lam))


@pytest.mark.parametrize("eas,n", [(0, 0), (1, 9)])
def test_function_loads_match_oracle(ikr, eas, n, parity_log):
    p = problems.cantilever(5, 3, 2, L=4.0, jitter=0.15, seed=4, eas=eas, n_eas=n)
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    with_function_loads(p, fes)
    with_function_loads(p, o)
    u = 0.01 * np.random.default_rng(3).standard_normal(p.n_dofs) * (1 - p.fixed)
    for lam in (0.3, 0.8):
        req = ikr.FERequirements(fes, u, lam)
        ev = ikr.calculateVector(fes, req)
        ref = np.array([o.element_vector(e, u, lam) for e in range(p.mesh.n_elems)])
        assert parity_log(f"function loads eas={eas} lambda={lam}: element vectors", rel_err(ev, ref), FP64_RTOL)
        R = asm.vector(req, dbc=ikr.DBCOption.Full)
        assert parity_log(f"function loads eas={eas} lambda={lam}: assembled force", rel_err(R, o.assemble_vector(u, lam)),
                          FP64_RTOL)
        if eas == 0:
            en = ikr.calculateScalar(fes, req)
            ref_e = np.array([o.element_energy(e, u, lam) for e in range(p.mesh.n_elems)])
            assert rel_err(en, ref_e) <= FP64_RTOL
    fes.clear_volume_loads()
    fes.clear_neumann()
    assert not asm.vector(ikr.FERequirements(fes), dbc=ikr.DBCOption.Full).any()  # no load left, undeformed


def test_load_path_with_loads_not_linear_in_lambda_matches_oracle(ikr, parity_log):
    p = problems.cantilever(8, 2, 2, traction=(0.0, 0.0, -0.3), load_steps=4, tol=1e-10)
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    with_function_loads(p, fes, 0.05)  # at full scale the cantilever's elements invert in the first step
    with_function_loads(p, o, 0.05)
    ref = o.load_control(p.load_steps, tol=p.tol, max_iter=30)
    req = ikr.FERequirements(fes)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(tol=p.tol, maxIter=30, linear_rtol=1e-13),
                                                         ikr.LinearSolver(rtol=1e-13)))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    assert [s.iterations for s in info.solverInfos] == list(ref["iterations"])
    assert parity_log("function loads load path: max|u - u_oracle| / max|u_oracle|",
                      rel_err(req.globalSolution(), ref["u"]), 1e-8)


def test_dirichlet_values_given_as_a_function_match_oracle(ikr, parity_log):
    """storeInhomogeneousBoundaryCondition(f) with f not linear in lambda (dirichletvalues.hh:213-282): the tip face
    is pulled down by w(X, lambda) = -(1.5 lambda + 0.5 lambda^2)(1 + 0.1 y); the device Newton adds the IDBC forces
    from df/dlambda at lambda = 1 and imposes f at every load factor like the oracle's restatement; iterations per
    step and the displacement match, the prescribed entries end exactly at f(X, 1)."""
    p = problems.cantilever(8, 2, 2, traction=(0.0, 0.0, 0.0), load_steps=4, tol=1e-10)
    X = p.mesh.coords
    L = p.mesh.lengths[0]
    tip = np.nonzero(np.abs(X[:, 0] - L) < 1e-8)[0]
    p.fixed = p.fixed.copy()
    p.fixed[3 * tip + 2] = 1
    on_tip = np.abs(X[:, 0] - L) < 1e-8

    def value(Xp, lam):
        out = np.zeros_like(Xp)
        sel = np.abs(Xp[:, 0] - L) < 1e-8
        out[sel, 2] = -(1.5 * lam + 0.5 * lam ** 2) * (1.0 + 0.1 * Xp[sel, 1])
        return out

    def derivative(Xp, lam):
        out = np.zeros_like(Xp)
        sel = np.abs(Xp[:, 0] - L) < 1e-8
        out[sel, 2] = -(1.5 + lam) * (1.0 + 0.1 * Xp[sel, 1])
        return out

    o = oracle.from_problem(p)
    o.set_dirichlet_function(value, derivative)
    ref = o.load_control(p.load_steps, tol=p.tol, max_iter=30)
    fes, asm = problems.build_gpu(p)
    asm.set_dirichlet_function(value, derivative)
    req = ikr.FERequirements(fes)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(tol=p.tol, maxIter=30, linear_rtol=1e-13),
                                                         ikr.LinearSolver(rtol=1e-13)))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    u = req.globalSolution()
    assert np.array_equal(u.reshape(-1, 3)[on_tip, 2], value(X, 1.0)[on_tip, 2])
    assert [s.iterations for s in info.solverInfos] == list(ref["iterations"])
    assert parity_log("Dirichlet value function: max|u - u_oracle| / max|u_oracle|", rel_err(u, ref["u"]), 1e-8)
    with pytest.raises(ikr.IkarusError, match="NOT_IMPLEMENTED"):  # path following takes lambda-linear values only
        ikr.PathFollowing(nr, 2, 0.1).run(ikr.FERequirements(fes))
