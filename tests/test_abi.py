"""The C ABI: libsampo_cuda.so loads without a GPU and exports every function
include/sampo.h declares, with matching struct layouts. No compute calls."""
import ctypes
import os
import re

from tests.conftest import REPO


def _declared_functions():
    text = open(os.path.join(REPO, "include", "sampo.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(sampo_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported(sampo_lib):
    from sampo_gb300 import _lib
    names = _declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(sampo_lib, n), f"{n} declared in include/sampo.h but not exported"
        assert n in _lib.SIGNATURES, f"{n} missing from the ctypes binding"
    assert set(_lib.SIGNATURES) <= set(names)


def test_struct_layouts(sampo_lib):
    from sampo_gb300 import _lib
    assert ctypes.sizeof(_lib.Population) == 8 * 8 + 3 * 4          # struct Population, include/agent.h:109-123
    assert ctypes.sizeof(_lib.Environment) == 6 * 4                  # struct Environment, include/agent.h:22-35
    assert ctypes.sizeof(_lib.Seeds) == 16
    assert ctypes.sizeof(_lib.StatsRow) == 76 + 16
    assert sampo_lib.sampo_abi_version() == 1


def test_errors_without_handle(sampo_lib):
    assert sampo_lib.sampo_create(None, None) == -1
    assert sampo_lib.sampo_run(None, 1, None) == -1
    assert sampo_lib.sampo_run_async(None, 1, None) == -1
    assert sampo_lib.sampo_sync(None) == -1
    assert sampo_lib.sampo_destroy(None) == 0


def test_input_file_readers(sampo_lib, tmp_path):
    import numpy as np
    from sampo_gb300 import inputs
    w = inputs.seasonal_weather(3, 1)
    tp, ep = inputs.write_inputs(str(tmp_path), w, inputs.alternating_interventions(24))
    T = np.zeros(72, np.float32)
    assert sampo_lib.sampo_read_temperature_file(tp.encode(), T.ctypes.data, 72) == 0
    assert np.array_equal(T, inputs.read_temperature(tp, 72))
    env = np.zeros(72, dtype=inputs.ENV_DTYPE)
    assert sampo_lib.sampo_read_environment_file(ep.encode(), env.ctypes.data, 72, ctypes.c_float(5000.0)) == 0
    assert env.tobytes() == inputs.read_environment(ep, 72, 5000.0).tobytes()
    assert sampo_lib.sampo_read_temperature_file(tp.encode(), T.ctypes.data, 73) == -7
