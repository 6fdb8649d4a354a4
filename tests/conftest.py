import gzip
import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def load_golden(name: str) -> dict:
    with gzip.open(os.path.join(GOLDEN, f"{name}.json.gz"), "rt") as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import build
    build.build()
    import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def sampo_lib():
    from sampo_gb300 import build
    build.build_library()
    from sampo_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu_ready(sampo_lib):
    """The CUDA library on a visible GPU; fails (does not skip) when the
    library cannot run, so a GPU test never passes without native code."""
    import ctypes
    import numpy as np
    x = np.linspace(0.1, 2.0, 64).astype(np.float32)
    out = np.zeros_like(x)
    rc = sampo_lib.sampo_eval_math(0, x.ctypes.data, None, out.ctypes.data, len(x), 0)
    assert rc == 0, "CUDA device not usable by libsampo_cuda.so"
    return sampo_lib
