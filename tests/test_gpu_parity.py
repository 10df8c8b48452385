"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on the same seeded inputs.

Tolerances: FP64 element and assembled residual / stiffness within 1e-12 relative
(max-norm, relative to the largest entry of the oracle's result); sparsity patterns and Dirichlet maps
bit-exact; FP32 tangents within 1e-6 relative; converged displacements within 1e-8 relative.
"""
import json
import os

import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
VARIANTS = [(0, 0), (1, 9), (1, 21), (2, 9), (3, 9)]  # (EAS kind, parameters)
FP64_RTOL = 1e-12


def rel_err(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def small_mesh_problem(eas=0, n=0, seed=0):
    p = problems.cantilever(3, 2, 2, L=3.0, jitter=0.15, seed=seed, eas=eas, n_eas=n)
    return p


def alpha_scale(eas):
    # GL modes are strains scaled by T0^{-1}/detJ (large on small elements); H modes are displacement gradients
    return 2e-4 if eas == 1 else 5e-3


def test_nonpositive_detc_is_reported_like_the_oracle(ikr):
    """checkPositiveOrAbort (materialhelpers.hh:119-126) aborts the reference; both the oracle and the device
    path return the NONPOSITIVE_DETC status for the same state instead."""
    p = small_mesh_problem(1, 9, seed=5)
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(12)
    u = 0.02 * rng.standard_normal(p.n_dofs)
    alpha = 0.005 * rng.standard_normal((p.mesh.n_elems, 9))  # far outside the admissible range
    fes.alpha = alpha
    o.alpha = alpha
    with pytest.raises(oracle.OracleError):
        o.assemble_vector(u, 0.5)
    req = ikr.FERequirements(fes, u, 0.5)
    with pytest.raises(ikr.IkarusError, match="NONPOSITIVE_DETC"):
        asm.vector(req, dbc=ikr.DBCOption.Full)
    fes.alpha = np.zeros_like(alpha)  # the handle stays usable after the error
    assert np.isfinite(asm.vector(req, dbc=ikr.DBCOption.Full)).all()


def test_undeformed_residual_is_exactly_zero(ikr):
    p = problems.config1()
    fes, asm = problems.build_gpu(p)
    req = ikr.FERequirements(fes)
    assert not asm.vector(req, dbc=ikr.DBCOption.Full).any()


@pytest.mark.parametrize("eas,n", VARIANTS)
def test_element_vector_matrix_single_distorted(ikr, eas, n):
    p = problems.single_element(GOLD["fixed_distortion_3d"], eas=eas, n_eas=n)
    fes, _ = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(11)
    u = 0.05 * rng.standard_normal(24)
    if n:
        alpha = 0.01 * rng.standard_normal((1, n))
        fes.alpha = alpha
        o.alpha = alpha
    req = ikr.FERequirements(fes, u, 0.0)
    Rg = ikr.calculateVector(fes, req)[0]
    Kg = ikr.calculateMatrix(fes, req)[0]
    assert rel_err(Rg, o.element_vector(0, u)) <= FP64_RTOL
    assert rel_err(Kg, o.element_matrix(0, u)) <= FP64_RTOL


@pytest.mark.parametrize("eas,n", VARIANTS)
def test_element_level_on_jittered_mesh_with_traction(ikr, eas, n):
    p = small_mesh_problem(eas, n, seed=5)
    fes, _ = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(12)
    u = 0.02 * rng.standard_normal(p.n_dofs)
    if n:
        alpha = alpha_scale(eas) * rng.standard_normal((p.mesh.n_elems, n))
        fes.alpha = alpha
        o.alpha = alpha
    req = ikr.FERequirements(fes, u, 0.7)
    R = ikr.calculateVector(fes, req)
    K = ikr.calculateMatrix(fes, req)
    for e in range(p.mesh.n_elems):
        assert rel_err(R[e], o.element_vector(e, u, 0.7)) <= FP64_RTOL
        assert rel_err(K[e], o.element_matrix(e, u, 0.7)) <= FP64_RTOL
    # element range batching
    R2 = ikr.calculateVector(fes, req, elements=(3, 7))
    assert np.array_equal(R2, R[3:7])


def test_element_energy(ikr):
    p = small_mesh_problem()
    fes, _ = problems.build_gpu(p)
    o = oracle.from_problem(p)
    u = 0.02 * np.random.default_rng(4).standard_normal(p.n_dofs)
    req = ikr.FERequirements(fes, u, 0.4)
    E = ikr.calculateScalar(fes, req)
    ref = np.array([o.element_energy(e, u, 0.4) for e in range(p.mesh.n_elems)])
    assert rel_err(E, ref) <= FP64_RTOL


def test_eas_scalar_is_not_implemented(ikr):
    p = small_mesh_problem(1, 9)
    fes, _ = problems.build_gpu(p)
    req = ikr.FERequirements(fes)
    with pytest.raises(ikr.IkarusError, match="NOT_IMPLEMENTED"):
        ikr.calculateScalar(fes, req)


@pytest.mark.parametrize("eas,n", VARIANTS)
def test_assembled_vector_and_matrix(ikr, eas, n):
    p = small_mesh_problem(eas, n, seed=9)
    p.pl_dofs = np.array([3 * (p.mesh.n_nodes - 1) + 1, 1], dtype=np.int32)  # dof 1 is constrained (x = 0)
    p.pl_values = np.array([1.5, -0.25])
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(21)
    u = 0.02 * rng.standard_normal(p.n_dofs) * (1 - p.fixed)
    if n:
        alpha = alpha_scale(eas) * rng.standard_normal((p.mesh.n_elems, n))
        fes.alpha = alpha
        o.alpha = alpha
    req = ikr.FERequirements(fes, u, 0.6)
    asm.bind(req, ikr.DBCOption.Full)
    for dbc, odbc in [(ikr.DBCOption.Full, oracle.DBC_FULL), (ikr.DBCOption.Raw, oracle.DBC_RAW),
                      (ikr.DBCOption.Reduced, oracle.DBC_REDUCED)]:
        Rg = asm.vector(req, dbc=dbc)
        Ro = o.assemble_vector(u, 0.6, odbc)
        assert rel_err(Rg, Ro) <= FP64_RTOL, dbc
        Kg = asm.matrix(req, dbc=dbc)
        cp, ri, v, nn = o.assemble_matrix_csc(u, 0.6, odbc)
        Kg.sort_indices()
        assert np.array_equal(Kg.indptr.astype(np.int64), cp), dbc   # pattern bit-exact
        assert np.array_equal(Kg.indices, ri), dbc
        assert rel_err(Kg.data, v) <= FP64_RTOL, dbc
        if dbc == ikr.DBCOption.Full:  # Dirichlet map bit-exact: unit diagonal, zero rows and columns
            fx = np.nonzero(p.fixed)[0]
            Kd = Kg.toarray()
            assert np.array_equal(Kd[np.ix_(fx, fx)], np.eye(len(fx)))
            assert not Kd[fx][:, p.fixed == 0].any() and not Kd[p.fixed == 0][:, fx].any()


def test_assembly_is_deterministic(ikr):
    p = problems.cantilever(8, 3, 3, jitter=0.1, seed=3)
    fes, asm = problems.build_gpu(p)
    u = 0.01 * np.random.default_rng(2).standard_normal(p.n_dofs)
    req = ikr.FERequirements(fes, u, 1.0)
    a = [asm.matrix(req, dbc=ikr.DBCOption.Full).data.copy() for _ in range(2)]
    b = [asm.vector(req, dbc=ikr.DBCOption.Full) for _ in range(2)]
    assert np.array_equal(a[0], a[1]) and np.array_equal(b[0], b[1])


def test_fp32_tangent(ikr):
    p = problems.cantilever(6, 2, 2, jitter=0.1, seed=8)
    u = 0.02 * np.random.default_rng(6).standard_normal(p.n_dofs)
    fes64, asm64 = problems.build_gpu(p, precision=0)
    fes32, asm32 = problems.build_gpu(p, precision=1)
    K64 = asm64.matrix(ikr.FERequirements(fes64, u, 1.0), dbc=ikr.DBCOption.Full)
    K32 = asm32.matrix(ikr.FERequirements(fes32, u, 1.0), dbc=ikr.DBCOption.Full)
    assert rel_err(K32.data, K64.data) <= 2e-6


@pytest.mark.parametrize("eas,n", [(1, 9), (2, 9), (3, 9)])
def test_update_state(ikr, eas, n):
    p = small_mesh_problem(eas, n, seed=2)
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(31)
    u = 0.02 * rng.standard_normal(p.n_dofs)
    du = 0.005 * rng.standard_normal(p.n_dofs)
    alpha = alpha_scale(eas) * rng.standard_normal((p.mesh.n_elems, n))
    fes.alpha = alpha
    o.alpha = alpha
    req = ikr.FERequirements(fes, u, 0.0)
    ikr.updateState(fes, req, du)
    o.update_state(u, du)
    assert rel_err(fes.alpha, o.alpha) <= 1e-11
    with pytest.raises(ikr.IkarusError, match="NOT_IMPLEMENTED"):  # reduced-size correction
        ikr.updateState(fes, req, du[p.fixed == 0])


def test_linear_solver(ikr):
    p = problems.cantilever(8, 2, 2)
    fes, asm = problems.build_gpu(p)
    req = ikr.FERequirements(fes)
    K = asm.matrix(req, dbc=ikr.DBCOption.Full)
    b = np.random.default_rng(0).standard_normal(p.n_dofs) * (1 - p.fixed)
    ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=1e-12)
    ls.compute(asm)
    x = ls.solve(asm, b)
    assert np.linalg.norm(K @ x - b) <= 1e-11 * np.linalg.norm(b)
    it, rel = ls.last_info()
    assert 0 < it and rel <= 1e-12


@pytest.mark.parametrize("material", ["NeoHooke", "StVenantKirchhoff", "BlatzKo"])
@pytest.mark.parametrize("es", ["GreenLagrangeStrain", "DisplacementGradient", "DisplacementGradientTransposed"])
def test_cantilever_goldens_on_gpu(ikr, es, material):
    """tests/src/testcantileverbeamEAS.cpp:60-124 through the device path: 80 Newton iterations, max |d|, for
    the NeoHooke, StVenantKirchhoff and BlatzKo materials of the reference test."""
    g = GOLD["cantilever_3d"]
    want = g["results"][es][material]
    kind = {"GreenLagrangeStrain": 1, "DisplacementGradient": 2, "DisplacementGradientTransposed": 3}[es]
    p = problems.cantilever_golden(kind, g["eas_parameters"][es],
                                   material={"NeoHooke": 0, "StVenantKirchhoff": 1, "BlatzKo": 2}[material])
    fes, asm = problems.build_gpu(p)
    req = ikr.FERequirements(fes)
    asm.bind(req, ikr.DBCOption.Full)
    ls = ikr.LinearSolver(ikr.SolverTypeTag.gpu_PCG_BlockJacobi, rtol=1e-13)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(tol=g["tol"], linear_rtol=1e-13), ls))
    msgs = []
    lc = ikr.LoadControl(nr, g["load_steps"], (0.0, 1.0))
    lc.subscribe(lambda m, s: msgs.append(m))
    info = lc.run(req)
    assert info.success
    assert info.totalIterations == want["iterations"]
    d = req.globalSolution()
    assert abs(np.abs(d).max() - want["max_disp"]) <= 1e-10 * want["max_disp"]
    assert abs(req.parameter() - 1.0) <= 1e-12
    assert msgs.count(ikr.ControlMessages.STEP_ENDED) == g["load_steps"] + 1
    assert all(si.residualNorm <= g["tol"] for si in info.solverInfos)


def test_config1_plain_fp64_matches_oracle(ikr, parity_log):
    p = problems.config1()
    o = oracle.from_problem(p)
    ref = o.load_control(p.load_steps, tol=p.tol)
    fes, asm = problems.build_gpu(p, precision=0)
    req = ikr.FERequirements(fes)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(tol=p.tol, linear_rtol=1e-12),
                                                         ikr.LinearSolver(rtol=1e-12)))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    assert [s.iterations for s in info.solverInfos] == list(ref["iterations"])
    assert parity_log("config1 FP64: max|u - u_oracle| / max|u_oracle|", rel_err(req.globalSolution(), ref["u"]),
                      1e-8)


def test_config1_mixed_precision_reaches_fp64_tolerance(ikr, parity_log):
    p = problems.config1()
    o = oracle.from_problem(p)
    ref = o.load_control(p.load_steps, tol=1e-10, tol_mode=1)
    fes, asm = problems.build_gpu(p, precision=1)
    req = ikr.FERequirements(fes)
    st = ikr.NRSettings(tol=1e-8, relative=True, eisenstat_walker=True, linear_rtol=1e-2, linear_rtol_min=1e-6)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(rtol=1e-4)))
    norms = []
    nr.subscribe(lambda m, s: norms.append((m, s["residualNorm"])))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    # the FP64 residual of every load step reached 1e-8 of its starting value
    for si in info.solverInfos[1:]:
        assert si.success
    assert parity_log("config1 mixed: max|u - u_oracle| / max|u_oracle|", rel_err(req.globalSolution(), ref["u"]),
                      1e-8)


@pytest.mark.parametrize("es", ["GreenLagrangeStrain", "DisplacementGradient", "DisplacementGradientTransposed"])
def test_cpp_facade_cantilever_goldens(ikr, es, tmp_path):
    """The reference's cantilever test written in C++ against include/ikarus_gb300.hpp (tests/cpp/)."""
    import subprocess
    from ikarus_gb300 import build
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "cantilever_eas")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "cantilever_eas.cpp"), "-L" + build.OUT, "-likarus_gb300",
                    "-Wl,-rpath," + build.OUT, "-o", exe], check=True)
    g = GOLD["cantilever_3d"]
    want = g["results"][es]["NeoHooke"]
    kind = {"GreenLagrangeStrain": 1, "DisplacementGradient": 2, "DisplacementGradientTransposed": 3}[es]
    r = subprocess.run([exe, str(kind), str(g["eas_parameters"][es]), str(want["iterations"]), repr(want["max_disp"])],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_backtracking_recovers_a_step_the_reference_aborts(ikr):
    """8x2x2 cantilever, tip traction 5 in ONE load step: the reference's Newton (and the oracle's) meets
    det C <= 0 on the way and aborts.  With max_backtracks the device Newton halves the corrections that invert
    an element and converges to the equilibrium the oracle reaches in 10 load steps."""
    p1 = problems.cantilever(8, 2, 2, traction=(0.0, 0.0, -5.0), load_steps=1, tol=1e-8, relative=True)
    with pytest.raises(oracle.OracleError):
        oracle.from_problem(p1).load_control(1, tol=1e-8, tol_mode=1, max_iter=60)
    ref = oracle.from_problem(p1).load_control(10, tol=1e-10, tol_mode=1, max_iter=60)

    def run(backtracks):
        fes, asm = problems.build_gpu(p1, precision=0)
        req = ikr.FERequirements(fes)
        st = ikr.NRSettings(tol=1e-10, maxIter=100, relative=True, linear_rtol=1e-12, backtracks=backtracks)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(rtol=1e-12)))
        info = ikr.LoadControl(nr, 1).run(req)
        return info, req.globalSolution()

    with pytest.raises(ikr.IkarusError, match="NONPOSITIVE_DETC"):
        run(0)
    info, u = run(30)
    assert info.success
    assert np.abs(u - ref["u"]).max() <= 1e-7 * np.abs(ref["u"]).max()


@pytest.mark.parametrize("eas,n", [(0, 0), (1, 9)])
def test_inhomogeneous_dirichlet_values_match_oracle(ikr, eas, n):
    """Prescribed tip displacement lambda * (-2) (storeInhomogeneousBoundaryCondition) under LoadControl: the
    device Newton adds the IDBC forces K_raw rate * stepSize to its first residual and re-imposes the values
    after every update like the reference; iteration counts per step and the converged displacement match the
    oracle, the constrained entries end exactly at lambda * rate, and the mixed form reaches the same state."""
    p = problems.cantilever(8, 2, 2, traction=(0.0, 0.0, 0.0), load_steps=4, tol=1e-10, eas=eas, n_eas=n)
    tip = np.nonzero(np.abs(p.mesh.coords[:, 0] - p.mesh.lengths[0]) < 1e-8)[0]
    fixed = p.fixed.copy()
    fixed[3 * tip + 2] = 1
    rate = np.zeros(p.n_dofs)
    rate[3 * tip + 2] = -2.0
    p.fixed = fixed
    o = oracle.from_problem(p)
    o.set_dirichlet_values(rate)
    ref = o.load_control(4, tol=1e-10, max_iter=30)
    for precision in (0, 1):
        fes, asm = problems.build_gpu(p, precision=precision)
        asm.set_dirichlet_values(rate)
        req = ikr.FERequirements(fes)
        if precision == 0:
            st = ikr.NRSettings(tol=1e-10, maxIter=30, linear_rtol=1e-13)
        else:
            st = ikr.NRSettings(tol=1e-10, maxIter=40, eisenstat_walker=True, linear_rtol=1e-2, linear_rtol_min=1e-6)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(rtol=1e-13)))
        info = ikr.LoadControl(nr, 4).run(req)
        assert info.success
        u = req.globalSolution()
        assert np.array_equal(u[rate != 0], rate[rate != 0])
        assert np.abs(u - ref["u"]).max() <= 1e-8 * np.abs(ref["u"]).max()
        if precision == 0:
            assert [s.iterations for s in info.solverInfos] == list(ref["iterations"])


@pytest.mark.parametrize("material", [0, 2], ids=["NeoHooke", "BlatzKo"])
def test_calculate_at_stresses_match_oracle(ikr, material):
    """calculateAt<PK2Stress / kirchhoffStress / cauchyStress> (nonlinearelastic.hh:237-271) at random local
    points of every element, FP64 within 1e-12 of the oracle; zero at the undeformed state."""
    p = problems.cantilever(4, 3, 2, L=4.0, jitter=0.15, seed=9)
    p.material = material
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(4)
    u = 0.01 * rng.standard_normal(p.n_dofs)
    req = ikr.FERequirements(fes, u, 0.0)
    local = rng.uniform(0.0, 1.0, (p.mesh.n_elems, 3))
    for rt in ikr.ResultTypes:
        got = ikr.calculateAt(fes, req, rt, local)
        ref = np.array([o.calculate_at(e, u, int(rt), local[e]) for e in range(p.mesh.n_elems)])
        assert rel_err(got, ref) <= FP64_RTOL, rt
        centre = ikr.calculateAt(fes, req, rt, elements=(2, 5))
        ref_c = np.array([o.calculate_at(e, u, int(rt)) for e in range(2, 5)])
        assert rel_err(centre, ref_c) <= FP64_RTOL
    assert np.abs(ikr.calculateAt(fes, ikr.FERequirements(fes), ikr.ResultTypes.cauchyStress)).max() == 0.0


@pytest.mark.parametrize("material", [0, 1, 2], ids=["NeoHooke", "SVK", "BlatzKo"])
@pytest.mark.parametrize("eas,n", [(1, 9), (1, 21), (2, 9), (3, 9)])
def test_eas_calculate_at_matches_oracle(ikr, eas, n, material):
    """calculateAt of EAS elements (enhancedassumedstrains.hh:127-188) with a stored alpha: the GL ansatz enhances
    the strain, H9 / H9T the displacement gradient (and with it F); FP64 within 1e-12 of the oracle."""
    p = problems.cantilever(4, 3, 2, L=4.0, jitter=0.15, seed=9, eas=eas, n_eas=n)
    p.material = material
    fes, asm = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(21)
    u = 0.01 * rng.standard_normal(p.n_dofs)
    alpha = alpha_scale(eas) * rng.standard_normal((p.mesh.n_elems, n))
    fes.alpha = alpha
    o.alpha = alpha
    req = ikr.FERequirements(fes, u, 0.0)
    local = rng.uniform(0.0, 1.0, (p.mesh.n_elems, 3))
    for rt in ikr.ResultTypes:
        got = ikr.calculateAt(fes, req, rt, local)
        ref = np.array([o.calculate_at(e, u, int(rt), local[e]) for e in range(p.mesh.n_elems)])
        assert rel_err(got, ref) <= FP64_RTOL, rt


def test_calculate_at_reproduces_reference_q1_stresses(ikr):
    """tests/src/teststresscomputation.cpp ("Q1"): planeStrain(StVenantKirchhoff(E = 1000, nu = 0.49)) on the unit
    square with the test's nodal displacements, PK2 / Kirchhoff / Cauchy stress at the test's local point.  The hex
    extruded along z with the in-plane displacements on both faces and w = 0 has F33 = 1, so its in-plane stresses
    are the plane-strain ones (the golden's own tolerance is 1e-8; met to 1e-12)."""
    g = GOLD["stress_q1_plane_strain_svk"]
    p = problems.single_element(None, E=g["E"], nu=g["nu"])
    p.material = 1
    fes, _ = problems.build_gpu(p)
    d = np.asarray(g["d"]).reshape(4, 2)
    u = np.zeros(24)
    for v in range(8):
        u[3 * v:3 * v + 2] = d[v & 3]
    req = ikr.FERequirements(fes, u, 0.0)
    loc = (g["position"][0], g["position"][1], 0.5)
    for rt, key in zip(ikr.ResultTypes, ("PK2", "kirchhoff", "cauchy")):
        r = ikr.calculateAt(fes, req, rt, loc)[0]
        got = np.array([[r[0], r[5]], [r[5], r[1]]])
        want = np.asarray(g[key])
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), key


@pytest.mark.parametrize("material", [1, 2], ids=["SVK", "BlatzKo"])
@pytest.mark.parametrize("eas,n", [(0, 0), (1, 9), (2, 9), (3, 9)])
def test_svk_element_and_assembly_match_oracle(ikr, eas, n, material):
    """StVenantKirchhoff (svk.hh:63-163) and BlatzKo (blatzko.hh) in the element kernels: element vectors and
    matrices, the assembled residual and tangent (FP64) within 1e-12 of the oracle, the FP32 tangent within 2e-6,
    energy for the displacement-based element."""
    p = problems.cantilever(4, 2, 2, L=4.0, jitter=0.15, seed=11, eas=eas, n_eas=n)
    p.material = material
    o = oracle.from_problem(p)
    rng = np.random.default_rng(5)
    u = 0.02 * rng.standard_normal(p.n_dofs)
    for precision in (0, 1):
        fes, asm = problems.build_gpu(p, precision=precision)
        req = ikr.FERequirements(fes, u, 0.4)
        if precision == 0:
            ev = ikr.calculateVector(fes, req)
            ref_v = np.array([o.element_vector(e, u, 0.4) for e in range(p.mesh.n_elems)])
            assert rel_err(ev, ref_v) <= FP64_RTOL
            em = ikr.calculateMatrix(fes, req)
            for e in range(p.mesh.n_elems):
                assert rel_err(em[e], o.element_matrix(e, u, 0.4)) <= FP64_RTOL
            if eas == 0:
                en = ikr.calculateScalar(fes, req)
                ref_e = np.array([o.element_energy(e, u, 0.4) for e in range(p.mesh.n_elems)])
                assert rel_err(en, ref_e) <= FP64_RTOL
            R = asm.vector(req, dbc=ikr.DBCOption.Full)
            assert rel_err(R, o.assemble_vector(u, 0.4)) <= FP64_RTOL
        K = asm.matrix(req, dbc=ikr.DBCOption.Full).toarray()
        Kref = o.assemble_matrix_dense(u, 0.4)
        assert rel_err(K, Kref) <= (2e-6 if precision else FP64_RTOL)


def test_newton_on_a_reduced_binding_gives_the_full_iterates(ikr):
    """DBCOption::Reduced bound to the assembler (the reference then solves the reduced system and expands the
    correction, nonlinearsolverfactory.hh:32-56): the reduced system is the Full one without its identity rows and
    columns, so the device Newton, which solves the Full system for every binding, gives the same iterations,
    norms and displacement; the constrained dofs stay at zero."""
    p = problems.cantilever(8, 2, 2, traction=(0.0, 0.0, -0.5), load_steps=3, tol=1e-10)
    results = []
    for dbc in (ikr.DBCOption.Full, ikr.DBCOption.Reduced):
        fes, asm = problems.build_gpu(p)
        req = ikr.FERequirements(fes)
        asm.bind(req, dbc)
        st = ikr.NRSettings(tol=1e-10, maxIter=30, linear_rtol=1e-13)
        nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver(rtol=1e-13)))
        info = ikr.LoadControl(nr, 3).run(req)
        assert info.success
        results.append((info, req.globalSolution()))
    (i0, u0), (i1, u1) = results
    assert [s.iterations for s in i0.solverInfos] == [s.iterations for s in i1.solverInfos]
    assert [s.residualNorm for s in i0.solverInfos] == [s.residualNorm for s in i1.solverInfos]
    assert np.array_equal(u0, u1)
    assert np.all(u1[p.fixed.astype(bool)] == 0.0)
    ref = oracle.from_problem(p).load_control(3, tol=1e-10, max_iter=30)
    assert np.abs(u1 - ref["u"]).max() <= 1e-8 * np.abs(ref["u"]).max()


@pytest.mark.parametrize("path", [1, 2, 3], ids=["coloured", "rows", "element-blocks"])
def test_fp32_tangent_kernels_match_oracle(ikr, path):
    """The three FP32 tangent kernels of the displacement-based NeoHooke element -- coloured element kernel, row
    kernel (a thread per node row adds its row of every adjacent element's tangent) and element blocks + gather --
    give the oracle's tangent within the FP32 bound, with Full Dirichlet rows and columns (and Raw without them); the
    timed choice picks one of them."""
    p = problems.cantilever(5, 3, 2, L=4.0, jitter=0.15, seed=13)
    o = oracle.from_problem(p)
    u = 0.02 * np.random.default_rng(7).standard_normal(p.n_dofs)
    fes, asm = problems.build_gpu(p, precision=1)
    asm.set_tangent_kernel(path)
    req = ikr.FERequirements(fes, u, 0.3)
    K = asm.matrix(req, dbc=ikr.DBCOption.Full).toarray()
    assert asm.tangent_kernel() == path
    assert rel_err(K, o.assemble_matrix_dense(u, 0.3)) <= 2e-6
    Kraw = asm.matrix(req, dbc=ikr.DBCOption.Raw).toarray()
    assert rel_err(Kraw, o.assemble_matrix_dense(u, 0.3, oracle.DBC_RAW)) <= 2e-6
    fes2, asm2 = problems.build_gpu(p, precision=1)
    K2 = asm2.matrix(ikr.FERequirements(fes2, u, 0.3), dbc=ikr.DBCOption.Full).toarray()
    assert asm2.tangent_kernel() in (1, 2, 3)
    assert rel_err(K2, K) <= 2e-6
