"""Generates tests/golden/reference_goldens.json from the reference's own test sources (read as text).

Run with the path of a reference checkout as its only argument; the JSON it writes is committed so the tests
never read the reference at run time.

Sources:
  tests/src/testcantileverbeamEAS.cpp:60-96   3D cantilever (NR + LoadControl + SparseFlatAssembler + EAS):
                                               (total Newton iterations, max |d|) per enhanced strain & material
  tests/src/testcantileverbeamEAS.cpp:101-104 material parameters (E = 100, nu = 0.3; BlatzKo mu = 40)
  tests/src/testcantileverbeam.hh:42-53, 96-151  mesh 10x1x1 on (L, h, h) = (10, 2, 2), tol 1e-10, 20 steps
  tests/src/testcommon.hh:199-207             fixed corner distortion of the single-element tests
  tests/src/testpathfollowing.cpp:41-370      two-dof operator under PathFollowing (ArcLength, LoadControl
                                               subsidiary function, DisplacementControl, ArcLength with
                                               inhomogeneous Dirichlet values): iterations per solve, final
                                               (u, w) (per step for the load control), final lambda
  tests/src/teststresscomputation.cpp:29-47, 150-200, 245-250
                                               displacement-based "Q1" stresses (PK2, Kirchhoff, Cauchy) of
                                               the unit-square element under planeStrain(StVenantKirchhoff(E =
                                               1000, nu = 0.49)) at the displacement d and the local position
  tests/src/materialresultcollection.hh       deviatoric functions of the hyperelastic framework (BlatzKo, Ogden
                                               with total / deviatoric stretches, Mooney-Rivlin, Yeoh, Arruda-Boyce,
                                               Gent): energy, first and second derivative per deformation state
  tests/src/testhyperelasticity.hh:15-95, 240-275
                                               their parameters (E = 1000, nu = 0.25, Ogden mu / alpha, Arruda-Boyce
                                               lambdaM, Gent Jm), the deformation states (stretch 1.37; the random
                                               right Cauchy-Green tensor) and the volumetric functions' parameters
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python make_goldens.py <path of the reference checkout>")
REF = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")


def _numbers(text):
    return [float(x) for x in re.findall(r"-?[0-9]+\.?[0-9]*(?:e[-+]?[0-9]+)?", text)]


def hyperelastic_goldens():
    src = open(os.path.join(REF, "tests/src/materialresultcollection.hh")).read()
    hh = open(os.path.join(REF, "tests/src/testhyperelasticity.hh")).read()
    results = {}
    for name in ("BlatzKo", "OgdenTotal", "OgdenDeviatoric", "MooneyRivlin", "Yeoh", "ArrudaBoyce", "Gent"):
        body = src[src.index("auto " + name + "Results()"):]
        body = body[: body.index("return std::make_tuple")]
        states = {}
        for part in re.split(r"if constexpr \(def == DeformationState::", body)[1:]:
            state = part.split(")")[0]
            blk = part[: part.index("} else")] if "} else" in part else part
            states[state] = blk
        tail = body[body.rindex("} else {") + len("} else {"):]
        states["Undeformed"] = tail
        out = {}
        for state, blk in states.items():
            e = re.search(r"energy = ([-0-9.e+]+);", blk)
            fd = re.search(r"firstDerivatives <<([^;]*);", blk)
            sd = re.search(r"secondDerivatives <<([^;]*);", blk)
            sdd = re.search(r"secondDerivatives\.diagonal\(\) <<([^;]*);", blk)
            second = _numbers(sd.group(1)) if sd else [0.0] * 9
            if sdd:  # diagonal only
                d = _numbers(sdd.group(1))
                second = [d[0], 0.0, 0.0, 0.0, d[1], 0.0, 0.0, 0.0, d[2]]
            out[state] = {"energy": float(e.group(1)) if e else 0.0,
                          "first": _numbers(fd.group(1)) if fd else [0.0, 0.0, 0.0], "second": second}
        results[name] = out
    E = float(re.search(r"double Emod = ([0-9.]+);", hh).group(1))
    nu = float(re.search(r"double nu\s*= ([0-9.]+);", hh).group(1))
    tm = hh[hh.index("inline auto testMatrix()"):]
    tm = tm[: tm.index("};")]
    rnd = _numbers(tm.split("Matrix3d")[1])
    body = hh[hh.index("auto testMaterialResults()"):]
    body = body[: body.index("checkForDeformationType")]
    alpha = _numbers(re.search(r"alpha_og = \{([^}]*)\}", body).group(1))
    ab = _numbers(re.search(r"ArrudaBoyce\(\{mu, ([0-9.]+)\}\)", body).group(1))[0]
    gent = _numbers(re.search(r"Gent\(\{mu, ([0-9.]+)\}\)", body).group(1))[0]
    stretch = float(re.search(r"constexpr double lambda\s*= ([0-9.]+);", hh).group(1))
    vol = hh[hh.index("auto testVolumetricFunctions()"):]
    vol = vol[: vol.index("return t;")]
    vf_params = {m[0]: (float(m[1]) if m[1] else None)
                 for m in re.findall(r"checkVolumetricFunctionsByAD\(VF(\d+)\{([0-9.]*)\}\)", vol)}
    return {"source": "tests/src/materialresultcollection.hh, tests/src/testhyperelasticity.hh",
            "E": E, "nu": nu, "stretch": stretch, "random_C": [rnd[0:3], rnd[3:6], rnd[6:9]],
            "ogden_mu_fractions": [2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0], "ogden_alpha": alpha,
            "mooney_rivlin_mu_fractions": [0.5, 0.5], "yeoh_mu_fractions": [0.5, 1.0 / 6.0, 1.0 / 3.0],
            "arruda_boyce_lambda_m": ab, "gent_jm": gent, "volumetric_beta": vf_params, "results": results}


def main():
    src = open(os.path.join(REF, "tests/src/testcantileverbeamEAS.cpp")).read()
    body = src[src.index("cantileverBeamResults3D"):]
    body = body[: body.index("int main")]
    goldens = {}
    for es_block in re.split(r"std::same_as<ES, EAS::", body)[1:]:
        es = es_block.split(">")[0]
        for mat, it, md in re.findall(r"is_same_v<MAT, (.+?)>\)\s*\{\s*return std::make_pair\((\d+), ([0-9.e+-]+)\)", es_block):
            name = "BlatzKo" if "BlatzKo" in mat else mat.strip()
            goldens.setdefault(es, {})[name] = {"iterations": int(it), "max_disp": float(md)}
    blatzko_mu = float(re.search(r"makeBlatzKo\(([0-9.]+)\)", src).group(1))
    common = open(os.path.join(REF, "tests/src/testcommon.hh")).read()
    blk = common[common.index("if constexpr (gridDim == 3)", common.index("fixedDistorted")):]
    blk = blk[: blk.index("} else")]
    offsets = [[float(x) for x in m] for m in re.findall(r"push_back\(\{([-0-9.]+), ([-0-9.]+), ([-0-9.]+)\}\)", blk)]
    pf_src = open(os.path.join(REF, "tests/src/testpathfollowing.cpp")).read()
    pf = {}
    for name in ("simple2DOperatorArcLengthTest", "simple2DOperatorArcLengthTestWithIDBC",
                 "simple2DOperatorLoadControlTestPF", "simple2DOperatorDisplacementControlTest"):
        body = pf_src[pf_src.index("static auto " + name + "("):]
        body = body[: body.index("return t;")]
        its = [int(x) for x in re.search(r"expectedIterations = \{([^}]*)\}", body).group(1).split(",")]
        disp = [float(x) for x in re.search(r"expectedDisplacement <<([^;]*);", body).group(1).split(",")]
        lam = float(re.search(r"expectedLambda = ([0-9.e+-]+);", body).group(1))
        pf[name] = {"iterations": its, "displacement": disp, "lambda": lam}
    main_src = pf_src[pf_src.index("int main"):]
    step = float(re.search(r"stepSize = ([0-9.e+-]+);", main_src).group(1))
    steps = int(re.search(r"loadSteps\s*= (\d+);", main_src).group(1))
    st_src = open(os.path.join(REF, "tests/src/teststresscomputation.cpp")).read()
    blk = st_src[st_src.index('elementType == "Q1")'):]
    blk = blk[: blk.index("return std::make_tuple")]
    mats = re.findall(r"MatrixType\{\s*\{([^}]*)\},\s*\{([^}]*)\}\s*\}", blk)
    to_m = lambda m: [[float(x) for x in row.split(",")] for row in m]
    d_line = re.search(r"else\s*d << ([^;]*);", st_src).group(1)
    pos = [float(x) for x in re.search(r"FieldVector<double, 2> pos\{([^}]*)\}", st_src).group(1).split(",")]
    mp = re.search(r"emodul = ([0-9.]+), \.nu = ([0-9.]+)", st_src)
    stress = {"source": "tests/src/teststresscomputation.cpp", "element": "Q1 (2D, unit square, planeStrain SVK)",
              "E": float(mp.group(1)), "nu": float(mp.group(2)), "d": [float(x) for x in d_line.split(",")],
              "position": pos, "PK2": to_m(mats[0]), "kirchhoff": to_m(mats[1]), "cauchy": to_m(mats[2])}
    hyper = hyperelastic_goldens()
    data = {
        "hyperelastic_deviatoric": hyper,
        "source": "ikarus-project/ikarus tests/src/testcantileverbeamEAS.cpp:60-96, testcantileverbeam.hh:42-198, "
                  "testcommon.hh:199-207",
        "cantilever_3d": {"L": 10.0, "h": 2.0, "elements": [10, 1, 1], "E": 100.0, "nu": 0.3, "load_steps": 20,
                          "tol": 1e-10, "point_load_nodes": [[10.0, 2.0, 2.0], [10.0, 2.0, 0.0]],
                          "eas_parameters": {"GreenLagrangeStrain": 21, "DisplacementGradient": 9,
                                             "DisplacementGradientTransposed": 9},
                          "blatzko_mu": blatzko_mu, "results": goldens},
        "fixed_distortion_3d": offsets,
        "stress_q1_plane_strain_svk": stress,
        "path_following_2dof": {"source": "tests/src/testpathfollowing.cpp", "step_size": step, "load_steps": steps,
                                "tol": 1e-8, "max_iter": 20, "cases": pf},
    }
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
    print(OUT)


if __name__ == "__main__":
    main()
