"""CPU tests of the oracle: pinned to the reference's goldens and to finite-difference consistency.

The reference cannot be compiled here (Dune, Eigen, dune-localfefunctions, autodiff are absent), so the oracle
is pinned by (a) the reference's end-to-end cantilever goldens, tests/src/testcantileverbeamEAS.cpp:60-96,
(b) derivative consistency as in tests/src/checkfebyautodiff.hh:56-86 (K = dR/dd, R = dPi/dd) with central
finite differences in place of autodiff, and (c) the sparsity sizes of the benchmark meshes.
"""
import json
import os

import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
EAS_KINDS = {"GreenLagrangeStrain": oracle.EAS_GL, "DisplacementGradient": oracle.EAS_H,
             "DisplacementGradientTransposed": oracle.EAS_HT}


MATERIALS = {"NeoHooke": oracle.MATERIAL_NEOHOOKE, "StVenantKirchhoff": oracle.MATERIAL_SVK,
             "BlatzKo": oracle.MATERIAL_BLATZKO}


@pytest.mark.parametrize("material", sorted(MATERIALS))
@pytest.mark.parametrize("es", sorted(EAS_KINDS))
def test_cantilever_goldens(es, material):
    g = GOLD["cantilever_3d"]
    want = g["results"][es][material]
    p = problems.cantilever_golden(EAS_KINDS[es], g["eas_parameters"][es], material=MATERIALS[material])
    o = oracle.from_problem(p)
    r = o.load_control(g["load_steps"], 0.0, 1.0, tol=g["tol"])
    assert r["success"]
    assert r["total_iterations"] == want["iterations"]
    max_disp = np.abs(r["u"]).max()
    assert abs(max_disp - want["max_disp"]) <= 1e-10 * want["max_disp"]  # FloatCmp tolerance of the test
    assert abs(r["lam"] - 1.0) <= 1e-10


def _distorted(eas=0, n=0, nu=0.3):
    offs = GOLD["fixed_distortion_3d"]
    return problems.single_element(offs, E=1000.0, nu=nu, eas=eas, n_eas=n)


def _relax_alpha(o, u):
    # local Newton on the internal variables at fixed u: alpha -= D^{-1} R~ (update with a zero correction)
    for _ in range(30):
        o.update_state(u, np.zeros_like(u))


@pytest.mark.parametrize("eas,n", [(0, 0), (oracle.EAS_GL, 9), (oracle.EAS_GL, 21), (oracle.EAS_H, 9),
                                   (oracle.EAS_HT, 9)])
def test_tangent_is_derivative_of_residual(eas, n):
    p = _distorted(eas, n)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(7)
    u = 0.05 * rng.standard_normal(24)
    if n:
        _relax_alpha(o, u)
    K = o.element_matrix(0, u)
    h = 1e-6
    Kfd = np.zeros((24, 24))
    for j in range(24):
        e = np.zeros(24)
        e[j] = h
        Kfd[:, j] = (o.element_vector(0, u + e) - o.element_vector(0, u - e)) / (2 * h)
    assert np.abs(K - Kfd).max() <= 1e-6 * np.abs(K).max()
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()


def test_residual_is_derivative_of_energy():
    p = _distorted()
    o = oracle.from_problem(p)
    rng = np.random.default_rng(3)
    u = 0.05 * rng.standard_normal(24)
    R = o.element_vector(0, u)
    h = 1e-6
    Rfd = np.array([(o.element_energy(0, u + h * np.eye(24)[j]) - o.element_energy(0, u - h * np.eye(24)[j])) / (2 * h)
                    for j in range(24)])
    assert np.abs(R - Rfd).max() <= 1e-7 * np.abs(R).max()


def test_green_lagrange_at_zero_is_linear_elasticity():
    # tests/src/testnonlinearelasticity.hh:194-246: at d = 0 the nonlinear K equals the linear-elastic K
    p = _distorted()
    o = oracle.from_problem(p)
    K = o.element_matrix(0, np.zeros(24))
    lam, mu = p.lam, p.mu
    Cl = np.zeros((6, 6))
    Cl[:3, :3] = lam
    Cl[np.arange(3), np.arange(3)] += 2 * mu
    Cl[np.arange(3, 6), np.arange(3, 6)] = mu
    X = p.mesh.coords[p.mesh.conn[0]]
    a, b = 0.5 - 0.5 / np.sqrt(3), 0.5 + 0.5 / np.sqrt(3)
    Klin = np.zeros((24, 24))
    for z in (a, b):
        for y in (a, b):
            for x in (a, b):
                xi = np.array([x, y, z])
                dN = np.zeros((8, 3))
                for v in range(8):
                    bits = [(v >> d) & 1 for d in range(3)]
                    f = [xi[d] if bits[d] else 1 - xi[d] for d in range(3)]
                    s = [1 if bits[d] else -1 for d in range(3)]
                    dN[v] = [s[0] * f[1] * f[2], f[0] * s[1] * f[2], f[0] * f[1] * s[2]]
                J = X.T @ dN
                G = dN @ np.linalg.inv(J)
                B = np.zeros((6, 24))
                for v in range(8):
                    g = G[v]
                    B[0, 3 * v], B[1, 3 * v + 1], B[2, 3 * v + 2] = g
                    B[3, 3 * v + 1], B[3, 3 * v + 2] = g[2], g[1]
                    B[4, 3 * v], B[4, 3 * v + 2] = g[2], g[0]
                    B[5, 3 * v], B[5, 3 * v + 1] = g[1], g[0]
                Klin += B.T @ Cl @ B * 0.125 * np.linalg.det(J)
    assert np.abs(K - Klin).max() <= 1e-8 * np.abs(K).max()


@pytest.mark.parametrize("nx,ny,nz", [(16, 4, 4), (10, 1, 1), (5, 3, 2)])
def test_pattern_sizes(nx, ny, nz):
    # n_b = prod(3(n_d+1) - 2) for structured hexahedral grids (8281 for the 16x4x4 mesh); scalar nnz = 9 n_b
    want = np.prod([3 * (n + 1) - 2 for n in (nx, ny, nz)])
    p = problems.cantilever(nx, ny, nz)
    o = oracle.from_problem(p)
    assert o.assemble_matrix_csc(dbc=oracle.DBC_FULL)[1].size == 9 * want


def test_reduced_is_full_restricted():
    # tests/src/testassembler.cpp:30-287: Reduced = Raw restricted to free dofs; Full has identity rows/cols
    p = problems.cantilever(4, 2, 2)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(1)
    u = 0.01 * rng.standard_normal(p.n_dofs) * (1 - p.fixed)
    Kf = o.assemble_matrix_dense(u, 0.3, oracle.DBC_FULL)
    Kr = o.assemble_matrix_dense(u, 0.3, oracle.DBC_RAW)
    Kred = o.assemble_matrix_dense(u, 0.3, oracle.DBC_REDUCED)
    free = p.fixed == 0
    assert np.array_equal(Kred, Kr[np.ix_(free, free)])
    assert np.array_equal(Kf[np.ix_(free, free)], Kred)
    fx = np.nonzero(p.fixed)[0]
    assert np.array_equal(Kf[np.ix_(fx, fx)], np.eye(len(fx)))
    assert not Kf[np.ix_(fx, np.nonzero(free)[0])].any()
    Rf = o.assemble_vector(u, 0.3, oracle.DBC_FULL)
    Rr = o.assemble_vector(u, 0.3, oracle.DBC_REDUCED)
    assert np.array_equal(Rf[free], Rr) and not Rf[fx].any()


def test_oracle_cg_matches_a_direct_solve():
    """The oracle's Jacobi-preconditioned CG (the reference's si_ConjugateGradient, the CPU baseline's CG) solves
    the assembled Full-DBC tangent to its tolerance."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    p = problems.cantilever(8, 2, 2, jitter=0.1, seed=4)
    o = oracle.from_problem(p)
    cp, ri, v, n = o.assemble_matrix_csc(None, 0.0)
    b = np.random.default_rng(0).standard_normal(n) * (1 - p.fixed)
    x, its, ok = oracle.cg_jacobi(cp, ri, v, b, 1e-12, 5000)
    A = sp.csc_matrix((v, ri, cp), shape=(n, n))
    assert ok and 0 < its < 5000
    assert np.abs(x - sla.spsolve(A, b)).max() <= 1e-8 * np.abs(x).max()


def _prescribed_tip(p, uz):
    """The cantilever's tip face z-displacements prescribed as lambda * uz (inhomogeneous Dirichlet values)."""
    tip = np.nonzero(np.abs(p.mesh.coords[:, 0] - p.mesh.lengths[0]) < 1e-8)[0]
    fixed = p.fixed.copy()
    fixed[3 * tip + 2] = 1
    rate = np.zeros(p.n_dofs)
    rate[3 * tip + 2] = uz
    p.fixed = fixed
    return rate


def test_oracle_inhomogeneous_dirichlet_values():
    """storeInhomogeneousBoundaryCondition semantics (dirichletvalues.hh:213-282, nonlinearsolverfactory.hh:45-52):
    the constrained entries end at lambda * rate, the free residual vanishes, and the equilibrium does not depend
    on the number of load steps."""
    res = []
    for steps in (4, 8):
        p = problems.cantilever(8, 2, 2, traction=(0.0, 0.0, 0.0), load_steps=steps, tol=1e-10)
        rate = _prescribed_tip(p, -2.0)
        o = oracle.from_problem(p)
        o.set_dirichlet_values(rate)
        r = o.load_control(steps, tol=1e-10, max_iter=30)
        u = r["u"]
        assert np.array_equal(u[rate != 0], rate[rate != 0])
        R = o.assemble_vector(u, 1.0)
        assert np.abs(R[p.fixed == 0]).max() <= 1e-9
        res.append(u)
    assert np.abs(res[0] - res[1]).max() <= 1e-8 * np.abs(res[1]).max()


@pytest.mark.parametrize("material", [oracle.MATERIAL_SVK, oracle.MATERIAL_BLATZKO], ids=["SVK", "BlatzKo"])
@pytest.mark.parametrize("eas,n", [(0, 0), (oracle.EAS_GL, 9), (oracle.EAS_H, 9)])
def test_svk_tangent_and_residual_are_consistent(eas, n, material):
    """StVenantKirchhoff (svk.hh:63-163) and BlatzKo (blatzko.hh) in the oracle: K = dR/dd and
    (displacement-based) R = dPsi/dd by central differences, as checkfebyautodiff.hh does for the reference's
    elements."""
    p = _distorted(eas, n)
    p.material = material
    o = oracle.from_problem(p)
    rng = np.random.default_rng(8)
    u = 0.05 * rng.standard_normal(24)
    if n:
        _relax_alpha(o, u)
    K = o.element_matrix(0, u)
    h = 1e-6
    Kfd = np.zeros((24, 24))
    for j in range(24):
        e = np.zeros(24)
        e[j] = h
        Kfd[:, j] = (o.element_vector(0, u + e) - o.element_vector(0, u - e)) / (2 * h)
    assert np.abs(K.reshape(24, 24, order="F") - Kfd).max() <= 1e-6 * np.abs(K).max()
    if n == 0:
        R = o.element_vector(0, u)
        Rfd = np.array([(o.element_energy(0, u + h * np.eye(24)[j]) - o.element_energy(0, u - h * np.eye(24)[j]))
                        / (2 * h) for j in range(24)])
        assert np.abs(R - Rfd).max() <= 1e-6 * np.abs(R).max()


# ---- path following (pathfollowing.inl, newtonraphsonwithscalarsubsidiaryfunction.hh) -------------------------
PF_CASES = {"simple2DOperatorArcLengthTest": (oracle.PF_ARC_LENGTH, False),
            "simple2DOperatorArcLengthTestWithIDBC": (oracle.PF_ARC_LENGTH, True),
            "simple2DOperatorLoadControlTestPF": (oracle.PF_LOAD_CONTROL, False),
            "simple2DOperatorDisplacementControlTest": (oracle.PF_DISPLACEMENT_CONTROL, False)}


@pytest.mark.parametrize("case", sorted(PF_CASES))
def test_path_following_two_dof_goldens(case):
    """The oracle's path-following routine on the reference's two-dof operator reproduces testpathfollowing.cpp:
    Newton iterations of every solve, final (u, w) (every step's for the load control) and final lambda, within the
    test's FloatCmp tolerance scaled to 1e-12."""
    g = GOLD["path_following_2dof"]
    want = g["cases"][case]
    kind, idbc = PF_CASES[case]
    r = oracle.path_following_toy(kind, idbc, steps=g["load_steps"], step_size=g["step_size"], tol=g["tol"],
                                  max_iter=g["max_iter"])
    assert r["iterations"] == want["iterations"]
    if len(want["displacement"]) == 2:
        np.testing.assert_allclose(r["d"], want["displacement"], rtol=1e-12, atol=0)
    else:
        per_step = np.asarray(want["displacement"]).reshape(2, -1)
        np.testing.assert_allclose(r["d_steps"].T, per_step, rtol=1e-12, atol=1e-15)
    assert abs(r["lam"] - want["lambda"]) <= 1e-12 * abs(want["lambda"])


def test_path_following_iteration_based_step_sizing():
    """AdaptiveStepSizing::IterationBased (adaptivestepsizing.hh:36-47): with a target of one iteration the step
    size shrinks by sqrt(1 / iterations) after every step that took more, so the path advances less."""
    g = GOLD["path_following_2dof"]
    noop = oracle.path_following_toy(oracle.PF_ARC_LENGTH, steps=5, step_size=0.1)
    ad = oracle.path_following_toy(oracle.PF_ARC_LENGTH, steps=5, step_size=0.1, target_iterations=1)
    assert noop["iterations"] == g["cases"]["simple2DOperatorArcLengthTest"]["iterations"]
    assert ad["lam"] < noop["lam"]
    assert np.all(np.diff(ad["lambdas"][1:]) < np.diff(noop["lambdas"][1:]) + 1e-15)


def test_oracle_path_following_load_control_matches_load_control():
    """The load-control subsidiary function walks lambda = s, 2s, ... like LoadControl over [0, N s]: both reach the
    same equilibria (tolerance-level differences only)."""
    p = problems.cantilever(4, 2, 2, load_steps=4, traction=(0.0, 0.0, -5.0))
    o = oracle.from_problem(p)
    lc = o.load_control(4, 0.0, 1.0, tol=1e-11)
    pf = oracle.from_problem(p).path_following(4, 0.25, kind=oracle.PF_LOAD_CONTROL, tol=1e-11)
    assert pf["success"] and lc["success"]
    np.testing.assert_allclose(pf["lambdas"], [0.0, 0.25, 0.5, 0.75, 1.0], atol=1e-14)
    np.testing.assert_allclose(pf["u"], lc["u"], rtol=0, atol=1e-9 * np.abs(lc["u"]).max())


def test_oracle_arc_length_constraint_and_equilibrium():
    """Every converged arc-length step is an equilibrium and lies on the sphere ||DD||^2 + psi^2 Dlambda^2 = s^2
    around the previous one (pathfollowingfunctions.hh:102-115)."""
    p = problems.cantilever(4, 2, 2, load_steps=4, traction=(0.0, 0.0, -5.0))
    s = 0.5
    us, lams = [], []
    for steps in (1, 2, 3):
        r = oracle.from_problem(p).path_following(steps, s, tol=1e-11)
        assert r["success"]
        us.append(r["u"])
        lams.append(r["lam"])
        o = oracle.from_problem(p)
        R = o.assemble_vector(r["u"], r["lam"])
        assert np.linalg.norm(R) <= 1e-11
    psi = oracle.from_problem(p).path_following(3, s, tol=1e-11)["psi"]
    for k in (1, 2):
        dd = us[k] - us[k - 1]
        dl = lams[k] - lams[k - 1]
        assert abs(np.sqrt(dd @ dd + psi * psi * dl * dl) - s) <= 1e-10


def test_oracle_stresses_reproduce_reference_q1_goldens():
    """tests/src/teststresscomputation.cpp ("Q1", planeStrain(StVenantKirchhoff(E = 1000, nu = 0.49)), unit square,
    the test's displacements and local point): the extruded hex (in-plane displacements on both faces, w = 0, so
    F33 = 1 and the in-plane stresses are the plane-strain ones) reproduces PK2, Kirchhoff and Cauchy stress."""
    g = GOLD["stress_q1_plane_strain_svk"]
    p = problems.single_element(None, E=g["E"], nu=g["nu"])
    o = oracle.from_problem(p)
    o.set_material(oracle.MATERIAL_SVK)
    d = np.asarray(g["d"]).reshape(4, 2)
    u = np.zeros(24)
    for v in range(8):
        u[3 * v:3 * v + 2] = d[v & 3]
    for t, key in enumerate(("PK2", "kirchhoff", "cauchy")):
        r = o.calculate_at(0, u, t, (g["position"][0], g["position"][1], 0.5))
        got = np.array([[r[0], r[5]], [r[5], r[1]]])
        want = np.asarray(g[key])
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), key


@pytest.mark.parametrize("eas,n", [(1, 9), (2, 9), (3, 9)])
def test_oracle_eas_stresses_at_zero_alpha_are_the_displacement_ones(eas, n):
    """With alpha = 0 the enhanced element's calculateAt is the displacement-based one (EAS(0) = NonLinearElastic,
    testnonlineareas.cpp:145-189 for the element quantities)."""
    p = problems.cantilever(3, 2, 2, L=3.0, jitter=0.1, seed=5)
    pe = problems.cantilever(3, 2, 2, L=3.0, jitter=0.1, seed=5, eas=eas, n_eas=n)
    o, oe = oracle.from_problem(p), oracle.from_problem(pe)
    u = 0.02 * np.random.default_rng(3).standard_normal(p.n_dofs)
    for e in range(p.mesh.n_elems):
        for t in range(3):
            np.testing.assert_allclose(oe.calculate_at(e, u, t, (0.3, 0.6, 0.2)), o.calculate_at(e, u, t, (0.3, 0.6, 0.2)),
                                       rtol=1e-13, atol=1e-13)
