"""Batches of independent SAMPO simulations on one GPU (sampo_batch_* of the
C ABI), and the ensemble workload built on them.

A batch holds up to 1024 replicates, each with its own pool, carrying
capacity, glibc seed stream and inputs. ``Batch.run(n)`` advances every active
replicate by n hourly steps in one pass of the step kernels per hour; each
replicate's rows, pool and histogram are bit-identical to the same simulation
run alone through ``sim.Simulation``. Replicates can be added and removed
between runs (continuous batching)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib, inputs
from ._lib import ENV_DTYPE, ROW_DTYPE, BatchConfig, Population, RandState, ReplicateConfig, SampoError, ptr
from .sim import make_pool_arrays, pool_view, pop_to_numpy, rand_state, seed_stream

NEVER = 0xFFFFFFFF


class Batch:
    def __init__(self, max_replicates: int, ring_steps: int, device: int = 0):
        self.lib = _lib.load()
        cfg = BatchConfig(max_replicates=max_replicates, ring_steps=ring_steps, device=device)
        h = C.c_void_p()
        rc = self.lib.sampo_batch_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise SampoError(rc, "sampo_batch_create failed")
        self.h = h
        self.ring = ring_steps
        self.max_replicates = max_replicates

    def _check(self, rc: int):
        if rc != 0:
            raise SampoError(rc, self.lib.sampo_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.sampo_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def replicate_bytes(capacity: int, ring_steps: int) -> int:
        return int(_lib.load().sampo_batch_replicate_bytes(capacity, ring_steps))

    def add(self, capacity: int, carrying_capacity: float, stop_step: int = NEVER) -> int:
        rc = ReplicateConfig(capacity=capacity, carrying_capacity=carrying_capacity, stop_step=stop_step)
        slot = C.c_uint32()
        self._check(self.lib.sampo_batch_add(self.h, C.byref(rc), C.byref(slot)))
        return slot.value

    def remove(self, slot: int):
        self._check(self.lib.sampo_batch_remove(self.h, slot))

    def set_inputs(self, slot: int, T: np.ndarray, env: np.ndarray, first: int = 0):
        T = np.ascontiguousarray(T, dtype=np.float32)
        env = np.ascontiguousarray(env).view(ENV_DTYPE)
        assert len(T) == len(env)
        self._check(self.lib.sampo_batch_set_inputs(self.h, slot, first, ptr(T), ptr(env), len(T)))

    def set_seeds(self, slot: int, first: int, seeds: np.ndarray):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(-1, 4, 4)
        self._check(self.lib.sampo_batch_set_seeds(self.h, slot, first, ptr(seeds), len(seeds)))

    def init_population(self, slot: int, n: int, init_seeds: np.ndarray, age_days_max: int = -1, age_seed: int = 0):
        init_seeds = np.ascontiguousarray(init_seeds, dtype=np.uint32).reshape(4, 4)
        self._check(self.lib.sampo_batch_init_population(self.h, slot, n, ptr(init_seeds), age_days_max, age_seed))

    def checkpoint(self, slot: int, path: str):
        """sampo_batch_checkpoint_save: the slot at its step boundary (the file
        format of Simulation.checkpoint)."""
        self._check(self.lib.sampo_batch_checkpoint_save(self.h, slot, path.encode()))

    def resume(self, slot: int, path: str):
        """sampo_batch_checkpoint_load into a slot taken with add()."""
        self._check(self.lib.sampo_batch_checkpoint_load(self.h, slot, path.encode()))

    def seed_stream(self, slot: int, st: RandState):
        """sampo_batch_seed_stream: the slot draws each coming step's seeds
        from its own copy of the rand() stream `st` on the device."""
        self._check(self.lib.sampo_batch_seed_stream(self.h, slot, C.byref(st)))

    def seed_state(self, slot: int) -> tuple[RandState, int]:
        """(device stream state, first step whose seeds it has not drawn)."""
        st, nxt = RandState(), C.c_uint32()
        self._check(self.lib.sampo_batch_seed_state(self.h, slot, C.byref(st), C.byref(nxt)))
        return st, nxt.value

    def run(self, nsteps: int, wait: bool = True):
        self._check(self.lib.sampo_batch_run(self.h, nsteps, 1 if wait else 0))

    def sync(self):
        self._check(self.lib.sampo_batch_sync(self.h))

    def rows(self, slot: int, first: int, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=ROW_DTYPE)
        self._check(self.lib.sampo_batch_rows(self.h, slot, first, n, ptr(out)))
        return out

    def state(self, slot: int):
        step, active, bits = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._check(self.lib.sampo_batch_state(self.h, slot, C.byref(step), C.byref(active), C.byref(bits)))
        return step.value, bool(active.value), bits.value

    def grow(self, slot: int, capacity: int):
        """sampo_batch_grow: move the slot's pool into `capacity` slots per
        buffer (slot indices kept) and resume it if it paused for capacity."""
        self._check(self.lib.sampo_batch_grow(self.h, slot, capacity))

    def states(self) -> np.ndarray:
        """sampo_batch_states: step, active, status, end and capacity of every slot."""
        out = (_lib.SlotState * self.max_replicates)()
        self._check(self.lib.sampo_batch_states(self.h, C.addressof(out), self.max_replicates))
        a = np.zeros(self.max_replicates, dtype=[("step", "u4"), ("active", "u4"), ("status", "u4"), ("end", "u4"),
                                                 ("capacity", "u8")])
        for i, o in enumerate(out):
            a[i] = (o.step, o.active, o.status, o.end, o.capacity)
        return a

    def histogram(self, slot: int) -> np.ndarray:
        h = np.zeros(100, dtype=np.uint32)
        self._check(self.lib.sampo_batch_histogram(self.h, slot, ptr(h)))
        return h

    def read_pool(self, slot: int, ranges_only: bool = False):
        p = Population()
        self._check(self.lib.sampo_batch_read_pool(self.h, slot, C.byref(p), None))
        popd = pop_to_numpy(p)
        if ranges_only:
            return popd, None
        n = int(popd["ranges"][7][1])
        arrays = make_pool_arrays(n)
        v = pool_view(arrays)
        self._check(self.lib.sampo_batch_read_pool(self.h, slot, C.byref(p), C.byref(v)))
        return popd, arrays

    def autotune(self) -> tuple[int, int]:
        """sampo_batch_autotune: CTAs per SM of the count and update/scatter passes."""
        c, s = C.c_uint32(), C.c_uint32()
        self._check(self.lib.sampo_batch_autotune(self.h, C.byref(c), C.byref(s)))
        return c.value, s.value

    def set_species(self, species):
        """sampo_batch_set_species: every replicate uses this species (None: built in)."""
        self._check(self.lib.sampo_batch_set_species(self.h, species.h if species is not None else None))
        self._species = species

    def set_grids(self, count_ctas_per_sm: int, scatter_ctas_per_sm: int):
        """sampo_batch_set_grids: fix the grid sizes without tuning."""
        self._check(self.lib.sampo_batch_set_grids(self.h, count_ctas_per_sm, scatter_ctas_per_sm))

    def set_items_per_thread(self, items: int):
        """sampo_batch_set_items_per_thread: 2 or 4 slots per thread."""
        self._check(self.lib.sampo_batch_set_items_per_thread(self.h, items))

    def items_per_thread(self) -> int:
        v = C.c_uint32()
        self._check(self.lib.sampo_batch_items_per_thread(self.h, C.byref(v)))
        return v.value

    def last_run_ms(self) -> float:
        v = C.c_double()
        self._check(self.lib.sampo_batch_last_run_ms(self.h, C.byref(v)))
        return v.value

    def launches(self) -> int:
        """Kernels run() has launched since creation."""
        n = C.c_uint64()
        self._check(self.lib.sampo_batch_launches(self.h, C.byref(n)))
        return n.value


# ---------------------------------------------------------------------------
# Replicate descriptions (the ensemble and served workloads)
# ---------------------------------------------------------------------------
@dataclass
class ReplicateSpec:
    """One simulation: initial eggs (ages 24*U{0..3} h), its glibc seed, its
    seasonal weather and its horizon in days; carrying capacity 5 x initial
    agents (the default FACTOR of src/abms.c:18-19)."""
    initial: int
    seed: int
    mean_t: float
    amplitude: float
    rain_mean: float
    days: int
    capacity: int
    age_days_max: int = 3

    @property
    def cc(self) -> float:
        return float(np.float32(5.0 * self.initial))

    @property
    def steps(self) -> int:
        return self.days * 24

    def inputs(self):
        """(T per hourly step, environment rows) as the reference would read them."""
        w = inputs.seasonal_weather(self.days, self.seed, mean=self.mean_t, amplitude=self.amplitude,
                                    noise_sd=0.5, rain_mean=self.rain_mean)
        T = np.repeat(w.temperature_c.astype(np.float32), 24)
        env = np.zeros(len(T), dtype=ENV_DTYPE)
        env["bloodmealSuccess"] = 0.25
        env["carryingCapacity"] = self.cc
        return T, env


def ensemble_specs(n: int, seed: int, days: int, size_range=(1e3, 1e6), growth: float = 16.0) -> list[ReplicateSpec]:
    """The ensemble workload: n replicates with initial sizes log-uniform in
    size_range, each with its own seed and weather (mean temperature U[20,30] C,
    seasonal amplitude U[2,8] C, noise sd 0.5, rain mean U[2,8] mm).
    capacity = growth x initial + 65536 slots per pool buffer."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(size_range[0]), np.log(size_range[1])
    out = []
    for i in range(n):
        initial = int(round(float(np.exp(rng.uniform(lo, hi)))))
        out.append(ReplicateSpec(initial=initial, seed=int(rng.integers(1, 2**31 - 1)),
                                 mean_t=float(rng.uniform(20.0, 30.0)), amplitude=float(rng.uniform(2.0, 8.0)),
                                 rain_mean=float(rng.uniform(2.0, 8.0)), days=days,
                                 capacity=int(growth * initial) + 65536))
    return out


def admit(batch: Batch, spec: ReplicateSpec, steps: int | None = None, device_seeds: bool = False) -> int:
    """Add one replicate to the batch with all its inputs (the batch's ring
    must hold steps + 1 entries) and its seeds: uploaded for every step, or
    drawn on the device from its rand() stream (device_seeds); returns its slot."""
    steps = spec.steps if steps is None else steps
    slot = batch.add(spec.capacity, spec.cc, stop_step=steps)
    T, env = spec.inputs()
    batch.set_inputs(slot, T[:steps], env[:steps])
    if device_seeds:
        init, st = rand_state(spec.seed)
    else:
        init, seeds = seed_stream(spec.seed, steps)
        batch.set_seeds(slot, 0, seeds)
    batch.init_population(slot, spec.initial, init, age_days_max=spec.age_days_max, age_seed=spec.seed)
    if device_seeds:
        batch.seed_stream(slot, st)
    return slot
