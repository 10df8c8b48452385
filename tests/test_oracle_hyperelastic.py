"""The oracle's hyperelastic framework (materials/hyperelastic/) pinned by the reference's own results:
the deviatoric functions' energies and derivatives at the five deformation states of
tests/src/materialresultcollection.hh (committed in tests/golden/reference_goldens.json), the recovery of
NeoHooke from Ogden (recoverNeoHookeTest, testhyperelasticity.hh:142-191), the volumetric functions'
derivatives (testVolumetricFunctions, testhyperelasticity.hh:92-140, here by central differences instead of
autodiff) and the consistency S = 2 dpsi/dC, moduli = 2 dS/dC of the assembled material point."""
import json
import os

import numpy as np
import pytest

import oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
HG = GOLD["hyperelastic_deviatoric"]
E, NU = HG["E"], HG["nu"]
MU = E / (2 * (1 + NU))
LAMBDA = E * NU / ((1 + NU) * (1 - 2 * NU))
STATES = ["Undeformed", "Uniaxial", "Biaxial", "PureShear", "Random"]


def deformation(state, s=HG["stretch"]):
    """Right Cauchy-Green tensor of a deformation state (testhyperelasticity.hh:42-88)."""
    if state == "Random":
        return np.array(HG["random_C"])
    F = {"Undeformed": np.eye(3), "Uniaxial": np.diag([s, 1 / np.sqrt(s), 1 / np.sqrt(s)]),
         "Biaxial": np.diag([s, s, 1 / (s * s)]), "PureShear": np.diag([s, 1.0, 1 / s])}[state]
    return F.T @ F


def deviatoric_functions():
    """The seven functions of testMaterialResults (testhyperelasticity.hh:240-258)."""
    og = dict(mu=[f * MU for f in HG["ogden_mu_fractions"]], alpha=HG["ogden_alpha"])
    return {
        "BlatzKo": oracle.hyper(oracle.DEV_BLATZKO, mu=[MU]),
        "OgdenTotal": oracle.hyper(oracle.DEV_OGDEN_TOTAL, **og),
        "OgdenDeviatoric": oracle.hyper(oracle.DEV_OGDEN_DEVIATORIC, **og),
        "MooneyRivlin": oracle.hyper(oracle.DEV_INVARIANT_BASED, mu=[f * MU for f in HG["mooney_rivlin_mu_fractions"]],
                                     p=[1, 0], q=[0, 1]),
        "Yeoh": oracle.hyper(oracle.DEV_INVARIANT_BASED, mu=[f * MU for f in HG["yeoh_mu_fractions"]], p=[1, 2, 3],
                             q=[0, 0, 0]),
        "ArrudaBoyce": oracle.hyper(oracle.DEV_ARRUDA_BOYCE, mu=[MU], param=HG["arruda_boyce_lambda_m"]),
        "Gent": oracle.hyper(oracle.DEV_GENT, mu=[MU], param=HG["gent_jm"]),
    }


@pytest.mark.parametrize("state", STATES)
@pytest.mark.parametrize("name", list(HG["results"]))
def test_deviatoric_function_results_match_reference(name, state):
    h = deviatoric_functions()[name]
    stretches = np.sqrt(np.linalg.eigvalsh(deformation(state)))  # ascending, as Eigen's solver returns them
    W, dW, ddW = oracle.hyper_deviatoric(h, stretches)
    ref = HG["results"][name][state]
    scale = max(1.0, np.abs(ref["second"]).max())
    assert W == pytest.approx(ref["energy"], rel=1e-12, abs=1e-12 * scale)
    np.testing.assert_allclose(dW, ref["first"], rtol=1e-12, atol=1e-12 * scale)
    np.testing.assert_allclose(ddW.ravel(), ref["second"], rtol=1e-12, atol=1e-12 * scale)


@pytest.mark.parametrize("state", STATES)
def test_neohooke_recovered_from_ogden_and_invariant_based(state):
    C = deformation(state)
    nh = oracle.material_point(oracle.MATERIAL_NEOHOOKE, C, lam=LAMBDA, mu=MU)
    og = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C,
                               h=oracle.hyper(oracle.DEV_OGDEN_TOTAL, mu=[MU], alpha=[2.0], volumetric=3, K=LAMBDA))
    for a, b in zip(nh, og):
        np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-12 * MU)
    ib = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C,
                               h=oracle.hyper(oracle.DEV_INVARIANT_BASED, mu=[MU / 2], p=[1], q=[0]))
    od = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C,
                               h=oracle.hyper(oracle.DEV_OGDEN_DEVIATORIC, mu=[MU], alpha=[2.0]))
    for a, b in zip(ib, od):
        np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-12 * MU)


@pytest.mark.parametrize("vf", range(1, 13))
def test_volumetric_function_derivatives(vf):
    beta = HG["volumetric_beta"].get(str(vf)) or 0.0
    J = np.sqrt(np.linalg.det(np.array(HG["random_C"])))
    h = 1e-5
    U = oracle.hyper_volumetric(vf, J, beta)
    Up, Um = oracle.hyper_volumetric(vf, J + h, beta), oracle.hyper_volumetric(vf, J - h, beta)
    assert U[1] == pytest.approx((Up[0] - Um[0]) / (2 * h), rel=1e-8, abs=1e-9)
    assert U[2] == pytest.approx((Up[1] - Um[1]) / (2 * h), rel=1e-8, abs=1e-9)


def voigt_sym(C):
    return [C[0, 0], C[1, 1], C[2, 2], C[1, 2], C[0, 2], C[0, 1]]


@pytest.mark.parametrize("vf", [0, 2, 5, 9])
@pytest.mark.parametrize("name", list(HG["results"]))
def test_material_point_is_consistent(name, vf):
    """S = 2 dpsi/dC and moduli = 2 dS/dC by central differences on a generic state (distinct stretches)."""
    h = deviatoric_functions()[name]
    h.volumetric, h.K, h.beta = vf, 2 * MU, 0.5
    rng = np.random.default_rng(7)
    F = np.eye(3) + 0.15 * rng.standard_normal((3, 3))
    C0 = F.T @ F
    psi, S, Cm = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C0, h=h)
    eps = 1e-6
    for v, (i, j) in enumerate([(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]):
        dC = np.zeros((3, 3))
        dC[i, j] = dC[j, i] = eps
        pp, Sp, _ = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C0 + dC, h=h)
        pm, Sm, _ = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C0 - dC, h=h)
        k = 1.0 if i == j else 0.5  # a symmetric perturbation moves both C_ij and C_ji
        assert S[v] == pytest.approx(2 * k * (pp - pm) / (2 * eps), rel=1e-6, abs=1e-6 * MU)
        np.testing.assert_allclose(Cm[:, v], 2 * k * (Sp - Sm) / (2 * eps), rtol=1e-5, atol=1e-5 * MU)


@pytest.mark.parametrize("state", ["Undeformed", "Uniaxial", "Biaxial"])
def test_equal_stretch_moduli_are_the_limit(state):
    """Repeated principal stretches take the (L_iiii - L_iikk) / 2 branch (deviatoric/interface.hh:108-116): its
    moduli equal the limit of the distinct-stretch formula (a state perturbed by 1e-5)."""
    h = deviatoric_functions()["OgdenDeviatoric"]
    h.volumetric, h.K = 5, 2 * MU
    C = deformation(state)
    _, _, M0 = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C, h=h)
    R = np.linalg.qr(np.random.default_rng(1).standard_normal((3, 3)))[0]
    Cp = C + np.diag([0.0, 1e-5, -1e-5])
    _, _, M1 = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, Cp, h=h)
    np.testing.assert_allclose(M0, M1, atol=1e-3 * np.abs(M0).max())
    # and it is objective: rotating C rotates the moduli (checked through the energy's invariance)
    p0 = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, C, h=h)[0]
    p1 = oracle.material_point(oracle.MATERIAL_HYPERELASTIC, R @ C @ R.T, h=h)[0]
    assert p1 == pytest.approx(p0, rel=1e-12, abs=1e-12)


def test_invalid_descriptions_are_rejected():
    with pytest.raises(oracle.OracleError):  # checkExponents: p = q = 0
        oracle.material_point(oracle.MATERIAL_HYPERELASTIC, np.eye(3),
                              h=oracle.hyper(oracle.DEV_INVARIANT_BASED, mu=[1.0], p=[0], q=[0]))
    with pytest.raises(oracle.OracleError):  # Gent: Jm must exceed W1 - 3
        oracle.hyper_deviatoric(oracle.hyper(oracle.DEV_GENT, mu=[MU], param=0.01), [0.5, 1.0, 2.0])
