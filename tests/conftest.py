"""pytest configuration: the ``gpu`` marker and shared fixtures.

``-m "not gpu"`` runs the oracle, golden-vector, host-table and ABI-export
checks (no GPU needed); ``-m gpu`` runs the parity tests through the C ABI on a
GB300.  The oracle is test infrastructure: it is only ever the checker.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    """Build (if needed) and load the native library."""
    from genpk_gb300 import build, native
    build.build()
    return native.load()


@pytest.fixture(scope="session")
def oracle_port():
    from oracle import oracle as O
    O.build()
    return O.port()


@pytest.fixture(scope="session")
def golden():
    out = {}
    for name in ("fieldize", "power", "counts"):
        with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
            out[name] = {k: z[k] for k in z.files}
    return out


def cases(store):
    """Group 'case/key' arrays of a fixture into {case: {key: array}}."""
    out = {}
    for k, v in store.items():
        case, key = k.split("/", 1)
        out.setdefault(case, {})[key] = v
    return out
