"""The hyperelastic framework (materials/hyperelastic/: Hyperelastic<Deviatoric<DF>, Volumetric<VF>> with the
factories of hyperelastic/factory.hh) on the device against the oracle's restatement, whose deviatoric functions
are pinned by the reference's materialresultcollection.hh (tests/test_oracle_hyperelastic.py).

Tolerances: FP64 element vectors, matrices, energies and stresses within 1e-12 relative (max-norm, as the
closed-form laws; measured at most 3e-14); FP32 tangents within 2e-6; converged load paths within 1e-8 with equal
Newton iterations per step."""
import numpy as np
import pytest

import oracle
from ikarus_gb300 import problems

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def laws(ikr, mu=400.0, K=1200.0):
    """One law per deviatoric function of testMaterialResults (testhyperelasticity.hh:240-258), several with a
    volumetric part."""
    og_mu, og_al = [2 * mu / 3, mu / 6, mu / 6], [1.23, 0.59, 0.18]
    return {
        "BlatzKo": ikr.makeBlatzKo(mu),
        "OgdenTotal+VF5": ikr.makeOgden(og_mu, og_al, K, ikr.VF5()),
        "OgdenDeviatoric+VF4": ikr.makeOgden(og_mu, og_al, K, ikr.VF4(0.5), tag=ikr.PrincipalStretchTags.deviatoric),
        "MooneyRivlin+VF2": ikr.makeMooneyRivlin([mu / 2, mu / 2], K, ikr.VF2()),
        "Yeoh+VF9": ikr.makeYeoh([mu / 2, mu / 6, mu / 3], K, ikr.VF9()),
        "ArrudaBoyce+VF7": ikr.makeArrudaBoyce(mu, 0.85, K, ikr.VF7(0.5)),
        "Gent+VF10": ikr.makeGent(mu, 2.5, K, ikr.VF10(0.4)),
        "PureVolumetric VF11": ikr.makePureVolumetric(ikr.VF11(), K),
    }


LAWS = ["BlatzKo", "OgdenTotal+VF5", "OgdenDeviatoric+VF4", "MooneyRivlin+VF2", "Yeoh+VF9", "ArrudaBoyce+VF7",
        "Gent+VF10", "PureVolumetric VF11"]


def problem_with(ikr, law, eas=0, n=0, seed=5):
    p = problems.cantilever(3, 2, 2, L=3.0, jitter=0.15, seed=seed, eas=eas, n_eas=n)
    p.hyper = laws(ikr)[law]
    return p


@pytest.mark.parametrize("law", LAWS)
def test_element_vector_matrix_energy_match_oracle(ikr, law, parity_log):
    p = problem_with(ikr, law)
    fes, _ = problems.build_gpu(p)
    o = oracle.from_problem(p)
    u = 0.02 * np.random.default_rng(12).standard_normal(p.n_dofs)
    req = ikr.FERequirements(fes, u, 0.7)
    R, K, E = ikr.calculateVector(fes, req), ikr.calculateMatrix(fes, req), ikr.calculateScalar(fes, req)
    ne = p.mesh.n_elems
    eR = max(rel_err(R[e], o.element_vector(e, u, 0.7)) for e in range(ne))
    eK = max(rel_err(K[e], o.element_matrix(e, u, 0.7)) for e in range(ne))
    eE = rel_err(E, np.array([o.element_energy(e, u, 0.7) for e in range(ne)]))
    assert parity_log(f"hyperelastic {law}: element vectors", eR, RTOL)
    assert parity_log(f"hyperelastic {law}: element matrices", eK, RTOL)
    assert parity_log(f"hyperelastic {law}: element energies", eE, RTOL)


@pytest.mark.parametrize("law", ["OgdenDeviatoric+VF4", "ArrudaBoyce+VF7", "Gent+VF10"])
@pytest.mark.parametrize("eas,n", [(1, 9), (2, 9)])
def test_eas_elements_with_hyperelastic_laws_match_oracle(ikr, law, eas, n, parity_log):
    p = problem_with(ikr, law, eas, n)
    fes, _ = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(3)
    u = 0.02 * rng.standard_normal(p.n_dofs)
    alpha = (2e-4 if eas == 1 else 5e-3) * rng.standard_normal((p.mesh.n_elems, n))
    fes.alpha = alpha
    o.alpha = alpha
    req = ikr.FERequirements(fes, u, 0.4)
    R, K = ikr.calculateVector(fes, req), ikr.calculateMatrix(fes, req)
    eR = max(rel_err(R[e], o.element_vector(e, u, 0.4)) for e in range(p.mesh.n_elems))
    eK = max(rel_err(K[e], o.element_matrix(e, u, 0.4)) for e in range(p.mesh.n_elems))
    assert parity_log(f"hyperelastic {law} EAS({eas},{n}): element vectors", eR, RTOL)
    assert parity_log(f"hyperelastic {law} EAS({eas},{n}): element matrices", eK, RTOL)


@pytest.mark.parametrize("law", ["OgdenTotal+VF5", "Yeoh+VF9", "Gent+VF10"])
def test_assembled_system_and_fp32_tangent_match_oracle(ikr, law):
    p = problem_with(ikr, law)
    o = oracle.from_problem(p)
    u = 0.02 * np.random.default_rng(7).standard_normal(p.n_dofs)
    fes, asm = problems.build_gpu(p)
    req = ikr.FERequirements(fes, u, 0.3)
    assert rel_err(asm.vector(req, dbc=ikr.DBCOption.Full), o.assemble_vector(u, 0.3)) <= RTOL
    Kd = o.assemble_matrix_dense(u, 0.3)
    assert rel_err(asm.matrix(req, dbc=ikr.DBCOption.Full).toarray(), Kd) <= RTOL
    for path in (1, 3):  # coloured element kernel, element blocks + gather
        fes32, asm32 = problems.build_gpu(p, precision=1)
        asm32.set_tangent_kernel(path)
        K32 = asm32.matrix(ikr.FERequirements(fes32, u, 0.3), dbc=ikr.DBCOption.Full).toarray()
        assert rel_err(K32, Kd) <= 2e-6, path


def test_stresses_match_oracle(ikr):
    p = problem_with(ikr, "OgdenDeviatoric+VF4")
    fes, _ = problems.build_gpu(p)
    o = oracle.from_problem(p)
    rng = np.random.default_rng(4)
    u = 0.01 * rng.standard_normal(p.n_dofs)
    req = ikr.FERequirements(fes, u, 0.0)
    local = rng.uniform(0.0, 1.0, (p.mesh.n_elems, 3))
    for rt in ikr.ResultTypes:
        got = ikr.calculateAt(fes, req, rt, local)
        ref = np.array([o.calculate_at(e, u, int(rt), local[e]) for e in range(p.mesh.n_elems)])
        assert rel_err(got, ref) <= RTOL, rt


def test_neohooke_recovered_on_the_device(ikr):
    """makeOgden<1, total>({mu}, {2}, lambda, VF3) is NeoHooke (recoverNeoHookeTest, testhyperelasticity.hh:142-191):
    the device's element matrices of both laws agree to the FP64 bound."""
    p = problems.cantilever(3, 2, 2, L=3.0, jitter=0.15, seed=5)
    fes_nh, _ = problems.build_gpu(p)
    p.hyper = ikr.makeOgden([p.mu], [2.0], p.lam, ikr.VF3())
    fes_og, _ = problems.build_gpu(p)
    u = 0.02 * np.random.default_rng(1).standard_normal(p.n_dofs)
    K1 = ikr.calculateMatrix(fes_nh, ikr.FERequirements(fes_nh, u, 0.5))
    K2 = ikr.calculateMatrix(fes_og, ikr.FERequirements(fes_og, u, 0.5))
    assert rel_err(K2, K1) <= RTOL


@pytest.mark.parametrize("law", ["OgdenDeviatoric+VF4", "ArrudaBoyce+VF7"])
def test_load_path_matches_oracle(ikr, law, parity_log):
    p = problems.cantilever(8, 2, 2, traction=(0.0, 0.0, -0.3), load_steps=4, tol=1e-9, relative=True)
    p.hyper = laws(ikr)[law]
    o = oracle.from_problem(p)
    ref = o.load_control(p.load_steps, tol=p.tol, tol_mode=1, max_iter=30)
    fes, asm = problems.build_gpu(p)
    req = ikr.FERequirements(fes)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(
        ikr.NRSettings(tol=p.tol, maxIter=30, relative=True, linear_rtol=1e-13), ikr.LinearSolver(rtol=1e-13)))
    info = ikr.LoadControl(nr, p.load_steps).run(req)
    assert info.success
    assert [s.iterations for s in info.solverInfos] == list(ref["iterations"])
    assert parity_log(f"hyperelastic {law} load path: max|u - u_oracle| / max|u_oracle|",
                      rel_err(req.globalSolution(), ref["u"]), 1e-8)


def test_gent_outside_its_domain_is_an_invalid_state(ikr):
    """gent.hh checkJm throws InvalidStateException when Jm <= W1 - 3; the device reports INVALID_STATE."""
    p = problems.cantilever(3, 2, 2, L=3.0)
    p.hyper = ikr.makeGent(400.0, 0.01, 1000.0, ikr.VF5())
    fes, asm = problems.build_gpu(p)
    u = 0.1 * np.random.default_rng(2).standard_normal(p.n_dofs) * (1 - p.fixed)  # no element inverts
    with pytest.raises(ikr.IkarusError, match="INVALID_STATE"):
        asm.vector(ikr.FERequirements(fes, u, 0.0), dbc=ikr.DBCOption.Full)


def test_invalid_descriptions_are_rejected(ikr):
    p = problems.cantilever(2, 1, 1, L=2.0)
    p.hyper = ikr.makeInvariantBased([1.0], [0], [0])
    with pytest.raises(ikr.IkarusError, match="ARG"):
        problems.build_gpu(p)
