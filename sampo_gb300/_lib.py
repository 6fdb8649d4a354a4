"""ctypes binding of libsampo_cuda.so (include/sampo.h).

The library is built in-tree (sampo_gb300/_build/); importing this module
never falls back to anything else: if the shared object is missing or does
not load, load() raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsampo_cuda.so")

OK = 0
ERR_NAMES = {-1: "SAMPO_ERR_ARG", -2: "SAMPO_ERR_CUDA", -3: "SAMPO_ERR_CAPACITY", -4: "SAMPO_ERR_TEMPERATURE",
             -5: "SAMPO_ERR_STATE", -6: "SAMPO_ERR_INTERNAL", -7: "SAMPO_ERR_IO", -8: "SAMPO_ERR_SPECIES",
             -9: "SAMPO_ERR_UNSUPPORTED"}
DEV_ERR_CAPACITY, DEV_ERR_DEVRATES, DEV_ERR_TILECOUNT, DEV_ERR_LARVATABLE = 0x1, 0x2, 0x4, 0x8
DEV_ERR_TMA, DEV_ERR_BARRIER = 0x10, 0x20
DEV_WARN_REF_LAYOUT = 0x100
STATE_NAMES = ("EGG", "LARVA", "PUPA", "IMMATURE", "MATESEEKING", "BMS", "BMD", "GRAVID")


class Range(C.Structure):
    _fields_ = [("start", C.c_uint32), ("end", C.c_uint32)]


class Population(C.Structure):
    _fields_ = [("r", Range * 8), ("numLarvae1DayEquiv", C.c_uint32), ("numFemale", C.c_uint32),
                ("numPotentiallyInfective", C.c_uint32)]


class Environment(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("bloodmealSuccess", "ITNValue", "IRSValue", "carryingCapacity",
                                         "larvacideValue", "oviTrapValue")]


class Seeds(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("z1", "z2", "z3", "z4")]


class BitesCycles(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("numCyclesReported", "sumCyclesReported", "numBitesReported",
                                         "numInfectBitesReported")]


class StatsRow(C.Structure):
    _fields_ = [("pop", Population), ("bnc", BitesCycles)]


class PoolView(C.Structure):
    _fields_ = [("ageInHours", C.c_void_p), ("hoursInState", C.c_void_p), ("delay", C.c_void_p),
                ("cumulativeSporogonicDevelopment", C.c_void_p), ("larvalDelayOrOviAttempts", C.c_void_p),
                ("availableEggs", C.c_void_p), ("cycleLength", C.c_void_p), ("humanBloodmealCount", C.c_void_p),
                ("numEggBatches", C.c_void_p), ("isFemale", C.c_void_p), ("state", C.c_void_p)]


class Config(C.Structure):
    _fields_ = [("capacity", C.c_uint64), ("carrying_capacity", C.c_float), ("device", C.c_int),
                ("max_steps", C.c_uint32)]


class RandState(C.Structure):
    _fields_ = [("r", C.c_uint32 * 31), ("i", C.c_uint32)]


class DevicePool(C.Structure):
    """sampo_device_pool: device addresses of one caller-owned pool buffer."""
    _fields_ = [("ageInHours", C.c_void_p), ("hoursInState", C.c_void_p), ("delay", C.c_void_p),
                ("cumulativeSporogonicDevelopment", C.c_void_p), ("larvalDelayOrOviAttempts", C.c_void_p),
                ("availableEggs", C.c_void_p), ("cycleLength", C.c_void_p), ("humanBloodmealCount", C.c_void_p),
                ("numEggBatches", C.c_void_p), ("flags", C.c_void_p)]


# numpy views of the same layouts
ROW_DTYPE = np.dtype([("ranges", "<u4", (8, 2)), ("L1de", "<u4"), ("numFemale", "<u4"), ("numPotInf", "<u4"),
                      ("numCycles", "<u4"), ("sumCycles", "<u4"), ("numBites", "<u4"), ("numInfectBites", "<u4")])
assert ROW_DTYPE.itemsize == C.sizeof(StatsRow)
ENV_DTYPE = np.dtype([("bloodmealSuccess", "<f4"), ("ITNValue", "<f4"), ("IRSValue", "<f4"),
                      ("carryingCapacity", "<f4"), ("larvacideValue", "<f4"), ("oviTrapValue", "<f4")])
assert ENV_DTYPE.itemsize == C.sizeof(Environment)

# name, dtype of the pool columns, in PoolView order
POOL_COLUMNS = (("ageInHours", np.float32), ("hoursInState", np.float32), ("delay", np.float32),
                ("cumulativeSporogonicDevelopment", np.float32), ("larvalDelayOrOviAttempts", np.uint32),
                ("availableEggs", np.uint32), ("cycleLength", np.uint32), ("humanBloodmealCount", np.uint32),
                ("numEggBatches", np.uint32), ("isFemale", np.uint8), ("state", np.uint8))

# every function the header declares, with its ctypes signature
_P = C.c_void_p
class BatchConfig(C.Structure):
    _fields_ = [("max_replicates", C.c_uint32), ("ring_steps", C.c_uint32), ("device", C.c_int)]


class ReplicateConfig(C.Structure):
    _fields_ = [("capacity", C.c_uint64), ("carrying_capacity", C.c_float), ("stop_step", C.c_uint32)]


class SlotState(C.Structure):
    _fields_ = [("step", C.c_uint32), ("active", C.c_uint32), ("status", C.c_uint32), ("end", C.c_uint32),
                ("capacity", C.c_uint64)]


SIGNATURES = {
    "sampo_abi_version": (C.c_int, []),
    "sampo_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "sampo_destroy": (C.c_int, [_P]),
    "sampo_last_error": (C.c_char_p, [_P]),
    "sampo_set_inputs": (C.c_int, [_P, C.c_uint32, _P, _P, C.c_uint32]),
    "sampo_set_seeds": (C.c_int, [_P, C.c_uint32, _P, C.c_uint32]),
    "sampo_init_population": (C.c_int, [_P, C.c_uint32, _P, C.c_int, C.c_uint64]),
    "sampo_load_pool": (C.c_int, [_P, C.POINTER(Population), C.POINTER(PoolView)]),
    "sampo_step": (C.c_int, [_P, C.POINTER(Environment), C.c_float, C.c_uint32, _P, C.POINTER(StatsRow)]),
    "sampo_run": (C.c_int, [_P, C.c_uint32, _P]),
    "sampo_run_async": (C.c_int, [_P, C.c_uint32, _P]),
    "sampo_sync": (C.c_int, [_P]),
    "sampo_current_row": (C.c_int, [_P, C.POINTER(StatsRow)]),
    "sampo_get_step": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "sampo_histogram": (C.c_int, [_P, _P]),
    "sampo_read_pool": (C.c_int, [_P, C.POINTER(Population), C.POINTER(PoolView)]),
    "sampo_device_status": (C.c_int, [_P, C.POINTER(C.c_uint32), C.c_int]),
    "sampo_set_timing": (C.c_int, [_P, C.c_int]),
    "sampo_kernel_times": (C.c_int, [_P, C.POINTER(C.c_double * 3), C.POINTER(C.c_uint64)]),
    "sampo_rand_seed": (None, [C.POINTER(RandState), C.c_uint32]),
    "sampo_rand_next": (C.c_uint32, [C.POINTER(RandState)]),
    "sampo_rand_seeds": (None, [C.POINTER(RandState), _P, C.c_uint32]),
    "sampo_read_temperature_file": (C.c_int, [C.c_char_p, _P, C.c_uint32]),
    "sampo_read_environment_file": (C.c_int, [C.c_char_p, _P, C.c_uint32, C.c_float]),
    "sampo_eval_math": (C.c_int, [C.c_int, _P, _P, _P, C.c_uint32, C.c_int]),
    "sampo_last_run_ms": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "sampo_host_alloc": (_P, [C.c_size_t]),
    "sampo_host_free": (None, [_P]),
    "sampo_flush_l2": (C.c_int, [_P]),
    "sampo_step_noalloc": (C.c_int, [C.POINTER(DevicePool), C.c_uint32, C.POINTER(DevicePool), C.c_uint32,
                                     C.POINTER(Population), C.POINTER(Environment), C.c_float, C.c_uint32, _P,
                                     C.c_float, C.POINTER(StatsRow), C.POINTER(Population), C.POINTER(BitesCycles),
                                     C.c_int, _P]),
    "sampo_checkpoint_save": (C.c_int, [_P, C.c_char_p]),
    "sampo_autotune": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "sampo_set_grids": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "sampo_set_small_step": (C.c_int, [_P, C.c_uint32]),
    "sampo_set_small_step_items": (C.c_int, [_P, C.c_uint32]),
    "sampo_set_items_per_thread": (C.c_int, [_P, C.c_uint32]),
    "sampo_items_per_thread": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "sampo_batch_set_items_per_thread": (C.c_int, [_P, C.c_uint32]),
    "sampo_batch_items_per_thread": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "sampo_small_step_info": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_int),
                                         C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "sampo_species_compile": (C.c_int, [C.c_char_p, C.c_int, C.c_char_p, C.c_size_t, C.POINTER(_P)]),
    "sampo_species_compile_text": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_size_t, C.POINTER(_P)]),
    "sampo_species_check_text": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_size_t]),
    "sampo_species_free": (None, [_P]),
    "sampo_species_device": (C.c_int, [_P]),
    "sampo_set_species": (C.c_int, [_P, _P]),
    "sampo_batch_set_species": (C.c_int, [_P, _P]),
    "sampo_batch_autotune": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "sampo_checkpoint_load": (C.c_int, [_P, C.c_char_p]),
    "sampo_batch_create": (C.c_int, [C.POINTER(BatchConfig), C.POINTER(_P)]),
    "sampo_batch_destroy": (C.c_int, [_P]),
    "sampo_batch_last_error": (C.c_char_p, [_P]),
    "sampo_batch_replicate_bytes": (C.c_uint64, [C.c_uint64, C.c_uint32]),
    "sampo_batch_add": (C.c_int, [_P, C.POINTER(ReplicateConfig), C.POINTER(C.c_uint32)]),
    "sampo_batch_remove": (C.c_int, [_P, C.c_uint32]),
    "sampo_batch_set_inputs": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, _P, C.c_uint32]),
    "sampo_batch_set_seeds": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, C.c_uint32]),
    "sampo_batch_init_population": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, C.c_int, C.c_uint64]),
    "sampo_batch_set_grids": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "sampo_batch_checkpoint_save": (C.c_int, [_P, C.c_uint32, C.c_char_p]),
    "sampo_batch_checkpoint_load": (C.c_int, [_P, C.c_uint32, C.c_char_p]),
    "sampo_checkpoint_info": (C.c_int, [C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(Population), C.POINTER(Population),
                                        C.POINTER(C.c_int)]),
    "sampo_batch_seed_stream": (C.c_int, [_P, C.c_uint32, C.POINTER(RandState)]),
    "sampo_batch_seed_state": (C.c_int, [_P, C.c_uint32, C.POINTER(RandState), C.POINTER(C.c_uint32)]),
    "sampo_batch_run": (C.c_int, [_P, C.c_uint32, C.c_int]),
    "sampo_batch_sync": (C.c_int, [_P]),
    "sampo_batch_rows": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P]),
    "sampo_batch_state": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "sampo_batch_grow": (C.c_int, [_P, C.c_uint32, C.c_uint64]),
    "sampo_batch_states": (C.c_int, [_P, C.c_void_p, C.c_uint32]),
    "sampo_batch_histogram": (C.c_int, [_P, C.c_uint32, _P]),
    "sampo_batch_read_pool": (C.c_int, [_P, C.c_uint32, C.POINTER(Population), C.POINTER(PoolView)]),
    "sampo_batch_last_run_ms": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "sampo_batch_launches": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
}

_lib = None


def load(path: str | None = None):
    """Load libsampo_cuda.so (built by sampo_gb300.build). Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libsampo_cuda.so not built ({p}); run `python -m sampo_gb300.build`")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class SampoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data
