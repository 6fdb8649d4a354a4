"""CPU oracle for the SAMPO per-step path - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
this package. It wraps oracle/_build/liboracle.so (the C restatement in
sampo_oracle.c, built by oracle/build.py) with the same call shapes as
sampo_gb300.sim.Simulation so that parity tests can drive both side by side.
The restatement is pinned to the reference through the golden fixtures in
tests/golden/ (produced by ref-as-C, see oracle/ref_build/).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
CLI = os.path.join(HERE, "_build", "sampo_oracle")

ROW_DTYPE = np.dtype([("ranges", "<u4", (8, 2)), ("L1de", "<u4"), ("numFemale", "<u4"), ("numPotInf", "<u4"),
                      ("numCycles", "<u4"), ("sumCycles", "<u4"), ("numBites", "<u4"), ("numInfectBites", "<u4")])
ENV_DTYPE = np.dtype([("bloodmealSuccess", "<f4"), ("ITNValue", "<f4"), ("IRSValue", "<f4"),
                      ("carryingCapacity", "<f4"), ("larvacideValue", "<f4"), ("oviTrapValue", "<f4")])
POOL_COLUMNS = (("ageInHours", np.float32), ("hoursInState", np.float32), ("delay", np.float32),
                ("cumulativeSporogonicDevelopment", np.float32), ("larvalDelayOrOviAttempts", np.uint32),
                ("availableEggs", np.uint32), ("cycleLength", np.uint32), ("humanBloodmealCount", np.uint32),
                ("numEggBatches", np.uint32), ("isFemale", np.uint8), ("state", np.uint8))


class _View(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("age", "his", "delay", "sporo", "uni", "avail", "cycle", "hbc", "batches",
                                         "female", "state")]


class _Pop(C.Structure):
    _fields_ = [("r", C.c_uint32 * 16), ("L1de", C.c_uint32), ("numFemale", C.c_uint32), ("numPotInf", C.c_uint32)]


class _Rand(C.Structure):
    _fields_ = [("r", C.c_uint32 * 31), ("i", C.c_uint32)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from . import build
            build.build()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        lib.orc_create.restype = P
        lib.orc_create.argtypes = [C.c_uint64, C.c_int]
        lib.orc_destroy.argtypes = [P]
        lib.orc_init_eggs.argtypes = [P, C.c_uint32, C.c_float, P, C.c_int, C.c_uint64]
        lib.orc_load_pool.argtypes = [P, C.POINTER(_Pop), C.POINTER(_View)]
        lib.orc_read_pool.argtypes = [P, C.POINTER(_Pop), C.POINTER(_View)]
        lib.orc_step.argtypes = [P, P, C.c_float, C.c_uint32, P, P]
        lib.orc_current_row.argtypes = [P, P]
        lib.orc_histogram.argtypes = [P, P]
        lib.orc_pool_hash.restype = C.c_uint64
        lib.orc_pool_hash.argtypes = [P]
        lib.orc_pool_end.restype = C.c_uint32
        lib.orc_pool_end.argtypes = [P]
        lib.orc_rand_seed.argtypes = [C.POINTER(_Rand), C.c_uint32]
        lib.orc_rand_next.restype = C.c_uint32
        lib.orc_rand_next.argtypes = [C.POINTER(_Rand)]
        _lib = lib
    return _lib


def glibc_rand(seed: int, n: int) -> np.ndarray:
    lib = load()
    st = _Rand()
    lib.orc_rand_seed(C.byref(st), seed & 0xFFFFFFFF)
    return np.array([lib.orc_rand_next(C.byref(st)) for _ in range(n)], dtype=np.uint32)


def _view(arrays) -> _View:
    v = _View()
    for (name, dt), f in zip(POOL_COLUMNS, _View._fields_):
        a = arrays[name]
        assert a.dtype == dt and a.flags["C_CONTIGUOUS"]
        setattr(v, f[0], a.ctypes.data)
    return v


class OracleSim:
    def __init__(self, capacity: int, threads: int = 0):
        self.lib = load()
        self.h = self.lib.orc_create(capacity, threads)
        if not self.h:
            raise MemoryError("oracle pool allocation failed")

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_eggs(self, n, T0, init_seeds, age_days_max=-1, age_seed=0):
        s = np.ascontiguousarray(init_seeds, dtype=np.uint32).reshape(4, 4)
        rc = self.lib.orc_init_eggs(self.h, n, float(np.float32(T0)), s.ctypes.data, age_days_max, age_seed)
        if rc:
            raise RuntimeError("oracle init failed")

    def load_pool(self, ranges, arrays):
        p = _Pop()
        for k in range(8):
            p.r[2 * k], p.r[2 * k + 1] = int(ranges[k][0]), int(ranges[k][1])
        if self.lib.orc_load_pool(self.h, C.byref(p), C.byref(_view(arrays))):
            raise RuntimeError("oracle load failed")

    def step(self, env_row, T, wt, seeds) -> np.ndarray:
        e = np.zeros(1, dtype=ENV_DTYPE)
        for n in ENV_DTYPE.names:
            e[n] = env_row[n]
        s = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(4, 4)
        row = np.zeros(1, dtype=ROW_DTYPE)
        rc = self.lib.orc_step(self.h, e.ctypes.data, float(np.float32(T)), int(wt), s.ctypes.data, row.ctypes.data)
        if rc:
            raise RuntimeError(f"oracle step failed ({rc})")
        return row[0]

    def run(self, T, env, seeds, first, n) -> np.ndarray:
        rows = np.zeros(n, dtype=ROW_DTYPE)
        for j in range(n):
            i = first + j
            rows[j] = self.step(env[i], T[i], i % 24, seeds[i])
        return rows

    def current_row(self):
        row = np.zeros(1, dtype=ROW_DTYPE)
        self.lib.orc_current_row(self.h, row.ctypes.data)
        return row[0]

    def read_pool(self):
        p = _Pop()
        self.lib.orc_read_pool(self.h, C.byref(p), None)
        n = p.r[15]
        arrays = {name: np.zeros(n, dtype=dt) for name, dt in POOL_COLUMNS}
        self.lib.orc_read_pool(self.h, C.byref(p), C.byref(_view(arrays)))
        ranges = np.array([[p.r[2 * k], p.r[2 * k + 1]] for k in range(8)], dtype=np.uint32)
        return ranges, arrays

    def histogram(self):
        h = np.zeros(100, dtype=np.uint32)
        self.lib.orc_histogram(self.h, h.ctypes.data)
        return h

    def pool_hash(self) -> int:
        return int(self.lib.orc_pool_hash(self.h))


# ---- the position-dependent pool hash, vectorised (same definition as
#      orc_pool_hash and the ref-as-C hook) ----
_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(z):
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def pool_hash(ranges, arrays) -> int:
    h = np.uint64(0)
    cols = [arrays["ageInHours"].view(np.uint32), arrays["hoursInState"].view(np.uint32), arrays["delay"].view(np.uint32),
            arrays["cumulativeSporogonicDevelopment"].view(np.uint32), arrays["larvalDelayOrOviAttempts"],
            arrays["availableEggs"], arrays["cycleLength"], arrays["humanBloodmealCount"], arrays["numEggBatches"]]
    with np.errstate(over="ignore"):
        for k in range(8):
            a, b = int(ranges[k][0]), int(ranges[k][1])
            h = h + _mix64(np.uint64((k << 40) ^ (a << 20) ^ b))
            if b <= a:
                continue
            i = np.arange(a, b, dtype=np.uint64)
            x = _mix64(i)
            x = _mix64(x ^ (arrays["state"][a:b].astype(np.uint64) | (arrays["isFemale"][a:b].astype(np.uint64) << np.uint64(8))))
            for c in cols:
                x = _mix64(x ^ c[a:b].astype(np.uint64))
            h = h + np.sum(x, dtype=np.uint64)
    return int(h)
