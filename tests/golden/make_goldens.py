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
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python make_goldens.py <path of the reference checkout>")
REF = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")


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
    data = {
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
