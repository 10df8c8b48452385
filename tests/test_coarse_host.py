"""Host logic of the CG's coarse correction, without a GPU: the band Cholesky inverse of the coarse operator
(ikr_ls_s::band_spd_inverse in ikarus_gb300/csrc/host_internal.h), compiled from tests/cpp/band_inverse.cpp.
A random SPD block-tridiagonal matrix of 6x6 blocks with one aggregate without stiffness and one repeated mode:
the inverse is exact on the kept modes, zero on the seven dropped ones, and symmetric."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_band_inverse_of_the_coarse_operator(tmp_path):
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "band_inverse")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + inc, os.path.join(ROOT, "tests", "cpp", "band_inverse.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True, timeout=60).stdout.split()
    err, dropped_max, asym, dropped = float(out[0]), float(out[1]), float(out[2]), int(out[3])
    assert err <= 1e-12
    assert dropped_max == 0.0 and asym == 0.0
    assert dropped == 7
