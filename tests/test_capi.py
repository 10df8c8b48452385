"""CPU tests of the C ABI boundary: the library builds, loads and exports every declared entry point.

No compute call is made here (there is no GPU on the build host); GPU behaviour is covered by test_gpu_*.py.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ikarus_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|int64_t|void)\s+(ikr_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def built_lib():
    from ikarus_gb300 import build
    return build.build()


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ["ikr_fes_create", "ikr_fe_calculate_vector", "ikr_fe_calculate_matrix", "ikr_assembler_vector",
              "ikr_assembler_matrix", "ikr_linear_solver_solve", "ikr_newton_solve", "ikr_load_control_run"]:
        assert s in syms


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes

    L = ctypes.CDLL(built_lib)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_python_front_end_binds_every_symbol(built_lib):
    import ikarus_gb300

    assert set(declared_symbols()) == set(ikarus_gb300.SIGNATURES)
    assert ikarus_gb300.lib().ikr_version() >= 100  # pure host call, no device needed


def test_no_cpu_fallback_without_library(monkeypatch, tmp_path):
    import ikarus_gb300

    monkeypatch.setattr(ikarus_gb300, "_lib", None)
    monkeypatch.setattr(ikarus_gb300, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="CUDA library missing"):
        ikarus_gb300.lib()
