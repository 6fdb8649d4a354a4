"""Host-side mirror of the reference's driver loop (src/abms.c) on top of
the C ABI: one Simulation per GPU-resident simulation.

Typical use, equivalent to `bin/abms temp.txt environment.txt`:

    sim = Simulation(capacity=6_000_000, carrying_capacity=160000.0, max_steps=8760)
    sim.set_inputs(T, env)                      # readSingleValFile / readEnvironment
    init, steps = seed_stream(seed, 8760)       # srand(seed); generateSeeds per step
    sim.set_seeds(0, steps)
    sim.init_population(32000, init)            # createInitialPopulation
    rows = sim.run(8760)                        # the step loop, rows = calcStats per step
    print("".join(stats_lines(rows, T, sim.initial_pop)))
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import (ENV_DTYPE, POOL_COLUMNS, ROW_DTYPE, Config, Environment, Population, PoolView, RandState,
                   SampoError, StatsRow, ptr)


def seed_stream(seed: int, nsteps: int):
    """glibc srand(seed) then 16 rand() per generateSeeds call
    (src/abms.c:611,671,511): returns (initial seeds (4,4), per-step seeds (nsteps,4,4))."""
    lib = _lib.load()
    st = RandState()
    lib.sampo_rand_seed(C.byref(st), seed & 0xFFFFFFFF)
    init = np.zeros((4, 4), dtype=np.uint32)
    lib.sampo_rand_seeds(C.byref(st), ptr(init), 1)
    steps = np.zeros((nsteps, 4, 4), dtype=np.uint32)
    if nsteps:
        lib.sampo_rand_seeds(C.byref(st), ptr(steps), nsteps)
    return init, steps


def rand_state(seed: int):
    """srand(seed) and the 16 initial draws (src/abms.c:611,671): returns
    (initial seeds (4,4), the stream positioned before step 0's draws)."""
    lib = _lib.load()
    st = RandState()
    lib.sampo_rand_seed(C.byref(st), seed & 0xFFFFFFFF)
    init = np.zeros((4, 4), dtype=np.uint32)
    lib.sampo_rand_seeds(C.byref(st), ptr(init), 1)
    return init, st


def make_pool_arrays(n: int) -> dict:
    return {name: np.zeros(n, dtype=dt) for name, dt in POOL_COLUMNS}


def pool_view(arrays: dict) -> PoolView:
    v = PoolView()
    for name, dt in POOL_COLUMNS:
        a = arrays[name]
        assert a.dtype == dt and a.flags["C_CONTIGUOUS"], name
        setattr(v, name, a.ctypes.data)
    return v


def pop_to_numpy(p: Population) -> dict:
    return {"ranges": np.array([[p.r[k].start, p.r[k].end] for k in range(8)], dtype=np.uint32),
            "L1de": p.numLarvae1DayEquiv, "numFemale": p.numFemale, "numPotInf": p.numPotentiallyInfective}


def pop_from_ranges(ranges) -> Population:
    p = Population()
    for k in range(8):
        p.r[k].start = int(ranges[k][0])
        p.r[k].end = int(ranges[k][1])
    return p


class Simulation:
    def __init__(self, capacity: int, carrying_capacity: float, max_steps: int = 8760, device: int = 0):
        self.lib = _lib.load()
        cfg = Config(capacity=capacity, carrying_capacity=carrying_capacity, device=device, max_steps=max_steps)
        h = C.c_void_p()
        rc = self.lib.sampo_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise SampoError(rc, "sampo_create failed (see stderr)")
        self.h = h
        self.capacity = capacity
        self.cc = np.float32(carrying_capacity)
        self.max_steps = max_steps
        self.initial_pop = None

    # -- plumbing --
    def _check(self, rc: int):
        if rc != 0:
            raise SampoError(rc, self.lib.sampo_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.sampo_destroy(self.h)
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

    # -- API --
    def set_inputs(self, T: np.ndarray, env: np.ndarray, first: int = 0):
        T = np.ascontiguousarray(T, dtype=np.float32)
        env = np.ascontiguousarray(env).view(ENV_DTYPE)
        assert len(T) == len(env)
        self._check(self.lib.sampo_set_inputs(self.h, first, ptr(T), ptr(env), len(T)))

    def set_seeds(self, first: int, seeds: np.ndarray):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(-1, 4, 4)
        self._check(self.lib.sampo_set_seeds(self.h, first, ptr(seeds), len(seeds)))

    def init_population(self, n: int, init_seeds: np.ndarray, age_days_max: int = -1, age_seed: int = 0):
        init_seeds = np.ascontiguousarray(init_seeds, dtype=np.uint32).reshape(4, 4)
        self._check(self.lib.sampo_init_population(self.h, n, ptr(init_seeds), age_days_max, age_seed))
        self.initial_pop = self.read_pool(ranges_only=True)[0]

    def load_pool(self, ranges, arrays: dict):
        p = pop_from_ranges(ranges)
        v = pool_view(arrays)
        self._check(self.lib.sampo_load_pool(self.h, C.byref(p), C.byref(v)))
        self.initial_pop = self.read_pool(ranges_only=True)[0]

    def run(self, nsteps: int, want_rows: bool = True) -> np.ndarray | None:
        rows = np.zeros(nsteps, dtype=ROW_DTYPE) if want_rows else None
        self._check(self.lib.sampo_run(self.h, nsteps, ptr(rows) if want_rows else None))
        return rows

    def step(self, env_row, T: float, world_time: int, seeds: np.ndarray) -> np.ndarray:
        e = Environment(*[float(env_row[n]) for n in ENV_DTYPE.names])
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(4, 4)
        row = StatsRow()
        self._check(self.lib.sampo_step(self.h, C.byref(e), float(np.float32(T)), world_time, ptr(seeds), C.byref(row)))
        return np.frombuffer(bytes(row), dtype=ROW_DTYPE)[0]

    def current_row(self) -> np.ndarray:
        row = StatsRow()
        self._check(self.lib.sampo_current_row(self.h, C.byref(row)))
        return np.frombuffer(bytes(row), dtype=ROW_DTYPE)[0]

    def histogram(self) -> np.ndarray:
        h = np.zeros(100, dtype=np.uint32)
        self._check(self.lib.sampo_histogram(self.h, ptr(h)))
        return h

    def read_pool(self, ranges_only: bool = False):
        p = Population()
        self._check(self.lib.sampo_read_pool(self.h, C.byref(p), None))
        popd = pop_to_numpy(p)
        if ranges_only:
            return popd, None
        n = int(popd["ranges"][7][1])
        arrays = make_pool_arrays(n)
        v = pool_view(arrays)
        self._check(self.lib.sampo_read_pool(self.h, C.byref(p), C.byref(v)))
        return popd, arrays

    def device_status(self, clear: bool = False) -> int:
        b = C.c_uint32()
        self._check(self.lib.sampo_device_status(self.h, C.byref(b), 1 if clear else 0))
        return b.value

    def set_timing(self, on: bool):
        self._check(self.lib.sampo_set_timing(self.h, 1 if on else 0))

    def kernel_times(self):
        t = (C.c_double * 3)()
        n = C.c_uint64()
        self._check(self.lib.sampo_kernel_times(self.h, C.byref(t), C.byref(n)))
        return list(t), n.value

    def last_run_ms(self) -> float:
        v = C.c_double()
        self._check(self.lib.sampo_last_run_ms(self.h, C.byref(v)))
        return v.value

    def flush_l2(self):
        self._check(self.lib.sampo_flush_l2(self.h))

    def autotune(self) -> tuple[int, int]:
        """Pick the step kernels' grid sizes on the coming step; returns the
        CTAs per SM of the count and update/scatter passes."""
        c, s = C.c_uint32(), C.c_uint32()
        self._check(self.lib.sampo_autotune(self.h, C.byref(c), C.byref(s)))
        return c.value, s.value

    def set_species(self, species):
        """Use a species header compiled at run time (sampo_gb300.species.Species),
        or the built-in species (None). Set it before init_population."""
        self._check(self.lib.sampo_set_species(self.h, species.h if species is not None else None))
        self._species = species  # the compiled kernels must outlive their use

    def set_grids(self, count_ctas_per_sm: int, scatter_ctas_per_sm: int):
        """Fix the grid sizes (CTAs per SM of the two passes) without tuning."""
        self._check(self.lib.sampo_set_grids(self.h, count_ctas_per_sm, scatter_ctas_per_sm))

    def set_items_per_thread(self, items: int):
        """Slots per thread of the count and update/scatter passes (2 or 4)."""
        self._check(self.lib.sampo_set_items_per_thread(self.h, items))

    def items_per_thread(self) -> int:
        v = C.c_uint32()
        self._check(self.lib.sampo_items_per_thread(self.h, C.byref(v)))
        return v.value

    def set_small_step(self, max_tiles: int | None = None):
        """Pools of at most max_tiles 1024-slot tiles take the one-launch
        step in day graphs (None: one tile per CTA of its largest grid; 0: never)."""
        self._check(self.lib.sampo_set_small_step(self.h, 0xFFFFFFFF if max_tiles is None else max_tiles))

    def set_small_step_items(self, items: int = 0):
        """Slots per thread of the one-launch step: 0 by pool size, 1, 2 or 4 fixed."""
        self._check(self.lib.sampo_set_small_step_items(self.h, items))

    def small_step_info(self) -> dict:
        """The one-launch step's largest grid, its current max_tiles, the
        kind of the last day launched (0 none, 1 three-kernel steps, 2
        one-launch steps launched cooperatively, 3 the same as plain launches)
        and the days run on each path."""
        g, m, k = C.c_uint32(), C.c_uint32(), C.c_int()
        d1, d3 = C.c_uint64(), C.c_uint64()
        self._check(self.lib.sampo_small_step_info(self.h, C.byref(g), C.byref(m), C.byref(k), C.byref(d1), C.byref(d3)))
        return {"grid": g.value, "max_tiles": m.value, "last_day": k.value, "days_one_launch": d1.value,
                "days_three_kernel": d3.value}

    def checkpoint(self, path: str):
        """Save the simulation at the current step boundary."""
        self._check(self.lib.sampo_checkpoint_save(self.h, os.fsencode(path)))

    def resume(self, path: str):
        """Continue from a checkpoint (the handle keeps its inputs and seeds)."""
        self._check(self.lib.sampo_checkpoint_load(self.h, os.fsencode(path)))

    def get_step(self) -> int:
        v = C.c_uint32()
        self._check(self.lib.sampo_get_step(self.h, C.byref(v)))
        return v.value

    def run_into(self, nsteps: int, rows_ptr: int):
        """sampo_run writing rows into caller memory (e.g. page-locked)."""
        self._check(self.lib.sampo_run(self.h, nsteps, rows_ptr))

    def run_async(self, nsteps: int, rows_ptr: int | None = None):
        """sampo_run_async: queues nsteps steps whose rows land in caller
        memory (page-locked for a copy that does not block); the memory must
        stay alive until sync()."""
        self._check(self.lib.sampo_run_async(self.h, nsteps, rows_ptr))

    def sync(self):
        """sampo_sync: waits for the queued steps and reports their status."""
        self._check(self.lib.sampo_sync(self.h))


class PinnedArray:
    """numpy array over page-locked host memory (sampo_host_alloc)."""

    def __init__(self, shape, dtype):
        self.lib = _lib.load()
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        self.p = self.lib.sampo_host_alloc(max(n, 1))
        if not self.p:
            raise MemoryError("cudaMallocHost failed")
        buf = (C.c_char * max(n, 1)).from_address(self.p)
        self.a = np.frombuffer(buf, dtype=np.uint8, count=n).view(dtype).reshape(shape)

    def free(self):
        if self.p:
            self.a = None
            self.lib.sampo_host_free(self.p)
            self.p = None


# ---------------------------------------------------------------------------
# printStats (src/abms.c:67-81) and calcStats's derived numbers (:287-302)
# ---------------------------------------------------------------------------
def stats_lines(rows: np.ndarray, T: np.ndarray, initial_ranges, first_step: int = 0,
                prev_ranges=None) -> list[str]:
    """The per-step lines abms.c prints. The adult-range test of calcStats
    (src/abms.c:235-236) uses the host copy of the population from the
    previous step (the initial ranges at step 0)."""
    out = []
    prev = np.asarray(initial_ranges if prev_ranges is None else prev_ranges, dtype=np.int64)
    for j, r in enumerate(rows):
        i = first_step + j
        rg = r["ranges"].astype(np.int64)
        num = (rg[:, 1] - rg[:, 0]) & 0xFFFFFFFF
        ub = max(prev[3][1], prev[5][1], prev[6][1], prev[7][1])
        adults_range = (ub - prev[3][0]) & 0xFFFFFFFF
        prev = rg
        adults = int(num[3] + num[4] + num[5] + num[6] + num[7]) & 0xFFFFFFFF
        l1 = int(r["L1de"]) if num[1] > 0 else 0
        fem = int(r["numFemale"]) if adults_range > 0 else 0
        inf = int(r["numPotInf"]) if adults_range > 0 else 0
        ncy = int(r["numCycles"])
        avg = int(r["sumCycles"]) // ncy if ncy > 0 else 0

        def d(x):
            x &= 0xFFFFFFFF
            return str(x - (1 << 32) if x >= 1 << 31 else x)
        hour = float(np.float32(1.0) * np.float32(i))
        line = "%0.1f, %0.1f" % (hour, float(np.float32(T[i])))
        line += ", " + ", ".join(d(x) for x in (adults, num[3], num[4], num[5], num[6], num[7], fem, inf, adults - fem))
        line += ", " + ", ".join(d(x) for x in (num[0], num[1], num[2], l1, l1 + num[0] + num[2])) + ", "
        line += "%s, %s, %s\r" % (d(avg), d(int(r["numBites"])), d(int(r["numInfectBites"])))
        out.append(line)
    return out


def population_lines(ranges) -> list[str]:
    """printPopulation (src/abms.c:83-92)."""
    names = ("Eggs \t\t", "Larvae \t\t", "Pupae \t\t", "Immatures \t", "MateSeeking \t", "BMS \t\t", "BMD \t\t",
             "Gravids \t")
    return ["%s[%d\t%d]\t%d\r" % (names[k], int(ranges[k][0]), int(ranges[k][1]), int(ranges[k][1]) - int(ranges[k][0]))
            for k in range(8)]


def histogram_text(hist) -> str:
    """histogram.txt (src/abms.c:176-180): "%d, " x 100, no newline."""
    return "".join("%d, " % int(x) for x in hist)
