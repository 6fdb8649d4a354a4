"""Deterministic transcendentals and the glibc-compatible seed stream."""
import ctypes
import ctypes.util

import numpy as np
import pytest

mpmath = pytest.importorskip("mpmath")


def _ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(1 << 31) - a, a)
    b = np.where(b < 0, -(1 << 31) - b, b)
    return np.abs(a - b)


def _eval(oracle_mod, fn, x, y=None):
    lib = oracle_mod.load()
    lib.orc_eval_math.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y if y is not None else np.zeros_like(x), np.float32)
    out = np.zeros_like(x)
    lib.orc_eval_math(fn, x.ctypes.data, y.ctypes.data, out.ctypes.data, len(x))
    return out


@pytest.mark.parametrize("fn,lo,hi,ref", [
    (0, -20.0, 20.0, lambda x, y: mpmath.exp(x)),
    (1, 2.0 ** -32, 1.0, lambda x, y: mpmath.log(x)),             # BoxMuller's u0
    (2, 0.0, 6.2831855, lambda x, y: mpmath.sin(x)),              # BoxMuller's theta
    (3, 0.2, 1.0, lambda x, y: mpmath.power(x, y)),               # pow(DSR, 1/24)
])
def test_math_correctly_rounded_on_model_domains(oracle_mod, fn, lo, hi, ref):
    rng = np.random.default_rng(fn)
    x = rng.uniform(lo, hi, 3000).astype(np.float32)
    y = np.full_like(x, np.float32(1.0) / np.float32(24.0))
    got = _eval(oracle_mod, fn, x, y)
    mpmath.mp.prec = 120
    want = np.array([np.float32(float(ref(mpmath.mpf(float(a)), mpmath.mpf(float(b))))) for a, b in zip(x, y)], np.float32)
    assert _ulps(got, want).max() == 0


def test_pow_integer_exponents(oracle_mod):
    """pow(.8f, numEggBatches) of generateEggs (include/properties.h:262)."""
    n = np.arange(0, 200, dtype=np.float32)
    x = np.full_like(n, np.float32(0.8))
    got = _eval(oracle_mod, 3, x, n)
    mpmath.mp.prec = 120
    want = np.array([np.float32(float(mpmath.power(mpmath.mpf(float(np.float32(0.8))), int(k)))) for k in n], np.float32)
    assert _ulps(got, want).max() <= 1
    assert got[0] == 1.0


def test_math_special_values(oracle_mod):
    inf, nan = np.float32(np.inf), np.float32(np.nan)
    assert _eval(oracle_mod, 0, [0.0])[0] == 1.0
    assert _eval(oracle_mod, 0, [inf])[0] == inf and _eval(oracle_mod, 0, [-inf])[0] == 0.0
    assert np.isnan(_eval(oracle_mod, 0, [nan])[0])
    assert _eval(oracle_mod, 1, [0.0])[0] == -inf and _eval(oracle_mod, 1, [1.0])[0] == 0.0
    assert np.isnan(_eval(oracle_mod, 1, [-1.0])[0])
    assert _eval(oracle_mod, 2, [0.0])[0] == 0.0
    assert _eval(oracle_mod, 3, [1.0], [nan])[0] == 1.0 and _eval(oracle_mod, 3, [nan], [0.0])[0] == 1.0
    assert _eval(oracle_mod, 3, [0.0], [0.5])[0] == 0.0


def _libc_rand(seed, n):
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srand(ctypes.c_uint(seed))
    return np.array([libc.rand() for _ in range(n)], dtype=np.uint32)


@pytest.mark.parametrize("seed", [0, 1, 7, 12345, 2**31 - 1, 2**31, 2**32 - 1, 3141592653])
def test_glibc_rand_streams(oracle_mod, sampo_lib, seed):
    """srand/rand as src/abms.c:611,146-149 call them: the oracle's and the
    library's restatements both reproduce the platform's glibc."""
    want = _libc_rand(seed, 1000)
    assert np.array_equal(oracle_mod.glibc_rand(seed, 1000), want)
    from sampo_gb300.sim import seed_stream
    init, steps = seed_stream(seed, 61)  # 16 + 61*16 = 992 draws
    got = np.concatenate([init.ravel(), steps.ravel()])
    assert np.array_equal(got, want[: got.size])
