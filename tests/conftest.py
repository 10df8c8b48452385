import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def ikr():
    """The product library; GPU tests fail loudly if it is not built (no fallback)."""
    import ikarus_gb300
    ikarus_gb300.lib()
    return ikarus_gb300


@pytest.fixture
def parity_log(request):
    """record(output, error, bound): prints the measured error of an output beside its bound and, when the
    environment variable IKR_PARITY_LOG names a file, appends it there as one JSON line."""
    def record(output, error, bound, **extra):
        line = dict(test=request.node.nodeid, output=output, error=float(error), bound=float(bound), **extra)
        print(f"PARITY {output}: error {error:.3e} (bound {bound:.1e})")
        path = os.environ.get("IKR_PARITY_LOG")
        if path:
            with open(path, "a") as f:
                f.write(json.dumps(line) + "\n")
        return error <= bound
    return record
