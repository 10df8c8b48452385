"""GPU parity of path following (pathfollowing.inl:25-73 with NewtonRaphsonWithSubsidiaryFunction,
newtonraphsonwithscalarsubsidiaryfunction.hh:207-316) against the oracle's restatement, which itself reproduces the
reference's testpathfollowing.cpp goldens (tests/test_oracle.py).

FP64 form: Newton iterations of every solve equal the oracle's, the load factor after every step within 1e-10
and the displacement within 1e-8 of the largest entry.  Mixed form (FP32 tangent and CG): every step converges to
an equilibrium on the arc-length sphere of its own psi, and psi (the initial prediction refined against the
FP64 tangent) and the path points agree with the FP64 oracle (psi 1e-7, lambda 1e-6, u 1e-5).
"""
import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu


def _problem(traction=(0.0, 0.0, -0.5), eas=0, n=0):
    return problems.cantilever(8, 2, 2, traction=traction, load_steps=4, eas=eas, n_eas=n)


def _step_size(p, lam_per_step=0.25):
    """Arc length s giving about lam_per_step per step: the first step has Dlambda = s / (sqrt(2) ||DD0||)."""
    o = oracle.from_problem(p)
    u0 = np.zeros(p.n_dofs)
    K = o.assemble_matrix_dense(u0, 1.0)
    dd0 = -np.linalg.solve(K, o.assemble_vector(u0, 1.0))
    return np.sqrt(2.0) * np.linalg.norm(dd0) * lam_per_step


def _device(ikr, p, steps, s, pft, precision=0, rate=None, adaptive=None, warm=True, multi=True):
    fes, asm = problems.build_gpu(p, precision=precision)
    if rate is not None:
        asm.set_dirichlet_values(rate)
    req = ikr.FERequirements(fes)
    if precision == 0:
        st = ikr.NRSettings(tol=1e-10, maxIter=30, linear_rtol=1e-13, linear_rtol_min=1e-13)
    else:
        st = ikr.NRSettings(tol=1e-10, maxIter=60, eisenstat_walker=True, linear_rtol=1e-2, linear_rtol_min=1e-7)
    ls = ikr.LinearSolver(rtol=1e-13)
    ls.set_multi_rhs(multi)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ls))
    pf = ikr.PathFollowing(nr, steps, s, pft, adaptive)
    pf.set_warm_start(warm)
    states = []

    def obs(msg, state):
        if msg == ikr.ControlMessages.SOLUTION_CHANGED:
            states.append((state["loadStep"], state["loadFactor"], req.globalSolution().copy()))

    pf.subscribe(obs)
    info = pf.run(req)
    return info, req, pf, states


def _check_fp64(info, states, ref):
    assert info.success
    assert [s.iterations for s in info.solverInfos] == list(ref["iterations"])
    lams = np.array([s[1] for s in states])
    np.testing.assert_allclose(lams, ref["lambdas"], rtol=0, atol=1e-10 * max(1.0, np.abs(ref["lambdas"]).max()))
    u = states[-1][2]
    assert np.abs(u - ref["u"]).max() <= 1e-8 * np.abs(ref["u"]).max()


@pytest.mark.parametrize("eas,n,warm", [(0, 0, True), (0, 0, False), (2, 9, True)])
def test_arc_length_matches_oracle(ikr, eas, n, warm):
    """warm: the load column's CG starts from the previous Newton iteration's solution (default) or from zero."""
    p = _problem(eas=eas, n=n)
    s = _step_size(p)
    ref = oracle.from_problem(p).path_following(4, s, tol=1e-10, max_iter=30)
    info, req, pf, states = _device(ikr, p, 4, s, ikr.ArcLength(), warm=warm)
    _check_fp64(info, states, ref)
    assert [st[0] for st in states] == [-1, 0, 1, 2, 3]
    assert abs(pf.subsidiary_args()["psi"] - ref["psi"]) <= 1e-10 * ref["psi"]


def test_load_control_subsidiary_matches_oracle(ikr):
    p = _problem()
    ref = oracle.from_problem(p).path_following(4, 0.25, kind=oracle.PF_LOAD_CONTROL, tol=1e-10, max_iter=30)
    info, req, pf, states = _device(ikr, p, 4, 0.25, ikr.LoadControlSubsidiaryFunction())
    _check_fp64(info, states, ref)
    np.testing.assert_allclose([st[1] for st in states], [0.0, 0.25, 0.5, 0.75, 1.0], atol=1e-14)


def test_displacement_control_matches_oracle(ikr):
    p = _problem(traction=(0.0, 0.0, 0.5))
    tip = np.nonzero(np.abs(p.mesh.coords[:, 0] - p.mesh.lengths[0]) < 1e-8)[0]
    ctrl = [3 * int(tip[0]) + 2]
    ref = oracle.from_problem(p).path_following(4, 0.3, kind=oracle.PF_DISPLACEMENT_CONTROL, controlled=ctrl,
                                                tol=1e-10, max_iter=30)
    info, req, pf, states = _device(ikr, p, 4, 0.3, ikr.DisplacementControl(ctrl))
    _check_fp64(info, states, ref)
    assert abs(req.globalSolution()[ctrl[0]] - 4 * 0.3) <= 1e-9


def test_arc_length_with_inhomogeneous_dirichlet_values_matches_oracle(ikr):
    """Prescribed tip displacement lambda * (-2) and no traction: the arc length measures the prescribed change
    too (idbcIncrement) and the second column of the bordered solve is Fext0 - K_raw rate."""
    p = _problem(traction=(0.0, 0.0, 0.0))
    tip = np.nonzero(np.abs(p.mesh.coords[:, 0] - p.mesh.lengths[0]) < 1e-8)[0]
    p.fixed = p.fixed.copy()
    p.fixed[3 * tip + 2] = 1
    rate = np.zeros(p.n_dofs)
    rate[3 * tip + 2] = -2.0
    o = oracle.from_problem(p)
    o.set_dirichlet_values(rate)
    ref = o.path_following(4, 1.0, tol=1e-10, max_iter=30)
    info, req, pf, states = _device(ikr, p, 4, 1.0, ikr.ArcLength(), rate=rate)
    _check_fp64(info, states, ref)
    u = req.globalSolution()
    np.testing.assert_array_equal(u[rate != 0], req.parameter() * rate[rate != 0])
    with pytest.raises(ikr.IkarusError):
        _device(ikr, p, 2, 0.25, ikr.LoadControlSubsidiaryFunction(), rate=rate)


def test_iteration_based_step_sizing_matches_oracle(ikr):
    p = _problem()
    s = _step_size(p, 0.3)
    ref = oracle.from_problem(p).path_following(4, s, target_iterations=2, tol=1e-10, max_iter=30)
    info, req, pf, states = _device(ikr, p, 4, s, ikr.ArcLength(), adaptive=ikr.AdaptiveStepSizing.IterationBased(2))
    _check_fp64(info, states, ref)
    assert pf.subsidiary_args()["stepSize"] < s
    with pytest.raises(ikr.IkarusError):
        ikr.AdaptiveStepSizing.IterationBased().setTargetIterations(0)


@pytest.mark.parametrize("multi", [True, False], ids=["two-rhs-launch", "sequential"])
def test_mixed_arc_length_is_on_the_path(ikr, multi):
    p = _problem()
    s = _step_size(p)
    ref = oracle.from_problem(p).path_following(4, s, tol=1e-10, max_iter=30)
    info, req, pf, states = _device(ikr, p, 4, s, ikr.ArcLength(), precision=1, multi=multi)
    assert info.success
    psi = pf.subsidiary_args()["psi"]
    o = oracle.from_problem(p)
    for k in range(1, len(states)):
        _, lam, u = states[k]
        assert np.linalg.norm(o.assemble_vector(u, lam)) <= 1e-9  # FP64 equilibrium
        du = u - states[k - 1][2]
        dl = lam - states[k - 1][1]
        assert abs(np.sqrt(du @ du + psi * psi * dl * dl) - s) <= 1e-8 * s
    # the initial prediction is refined against the FP64 tangent, so psi and the path points agree with the
    # FP64 oracle far below the FP32 solve's own accuracy
    assert abs(psi - ref["psi"]) <= 1e-7 * ref["psi"]
    lams = np.array([st[1] for st in states])
    np.testing.assert_allclose(lams, ref["lambdas"], rtol=1e-6, atol=1e-12)
    assert np.abs(states[-1][2] - ref["u"]).max() <= 1e-5 * np.abs(ref["u"]).max()


def test_path_following_argument_errors(ikr):
    """PathFollowing with steps <= 0 is an InvalidStateException (pathfollowing.hh:192-193); displacement control
    on a constrained or repeated dof is rejected before any solve."""
    p = _problem()
    fes, asm = problems.build_gpu(p)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(ikr.NRSettings(), ikr.LinearSolver()))
    with pytest.raises(ikr.IkarusError) as e:
        ikr.PathFollowing(nr, 0, 0.1)
    assert e.value.code == -3
    fixed = int(np.nonzero(p.fixed)[0][0])
    free = int(np.nonzero(p.fixed == 0)[0][0])
    with pytest.raises(ikr.IkarusError):
        ikr.PathFollowing(nr, 2, 0.1, ikr.DisplacementControl([fixed]))
    with pytest.raises(ikr.IkarusError):
        ikr.PathFollowing(nr, 2, 0.1, ikr.DisplacementControl([free, free]))
    pf = ikr.PathFollowing(nr, 2, 0.1, ikr.DisplacementControl([free]))
    assert pf.name() == "Path following with Displacement Control"


def test_cpp_facade_arc_length_matches_oracle(ikr, tmp_path):
    """PathFollowing through the C++ facade (tests/cpp/arclength.cpp) on the reference's 3D cantilever test mesh
    with H9 EAS and point loads: final load factor and max |d| of five arc-length steps as the oracle's."""
    import json
    import os
    import subprocess

    from ikarus_gb300 import build
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    gold = json.load(open(os.path.join(root, "tests", "golden", "reference_goldens.json")))["cantilever_3d"]
    p = problems.cantilever_golden(2, gold["eas_parameters"]["DisplacementGradient"])
    s = _step_size(p, 0.1)
    ref = oracle.from_problem(p).path_following(5, s, tol=1e-10, max_iter=30)
    exe = str(tmp_path / "arclength")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "arclength.cpp"), "-L" + build.OUT, "-likarus_gb300",
                    "-Wl,-rpath," + build.OUT, "-o", exe], check=True)
    args = [repr(float(v)) for v in (s, ref["lam"], np.abs(ref["u"]).max())]
    r = subprocess.run([exe, "2", "9", "5", *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
