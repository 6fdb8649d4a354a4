"""sampo_step_noalloc: one step for callers that cannot allocate device
memory (code inside another framework's memory arena, a service that must not
grow device memory after start-up, a memory-capped sandbox). The caller owns
both pool buffers; the step's scratch is the library's fixed device array.

Checked against the allocating entry point (sampo_step) on the same pool for
two steps in a row, ping-ponging the caller's two buffers: the stats row,
the next ranges and counters, and every field of every live slot must be
identical. This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COLS = [("ageInHours", np.float32), ("hoursInState", np.float32), ("delay", np.float32),
        ("cumulativeSporogonicDevelopment", np.float32), ("larvalDelayOrOviAttempts", np.uint32),
        ("availableEggs", np.uint32), ("cycleLength", np.uint32), ("humanBloodmealCount", np.uint32),
        ("numEggBatches", np.uint32)]


def _device_pool(torch, capacity):
    """Caller-owned buffers (torch allocates them, not the library): one column
    per field, 16 bytes of slack after `capacity` elements."""
    t = {name: torch.zeros(capacity + 4, dtype=torch.int32, device="cuda") for name, _ in COLS}
    t["flags"] = torch.zeros(capacity + 16, dtype=torch.uint8, device="cuda")
    from sampo_gb300._lib import DevicePool
    d = DevicePool(**{k: v.data_ptr() for k, v in t.items()})
    return t, d


def _upload(torch, t, ranges, arrays):
    n = int(ranges[7][1])
    for name, dt in COLS:
        t[name][:n].copy_(torch.from_numpy(arrays[name].view(np.int32).copy()))
    flags = (arrays["state"].astype(np.uint8) & 7) | (arrays["isFemale"].astype(np.uint8) << 3)
    t["flags"][:n].copy_(torch.from_numpy(flags))


def _download(t, n):
    out = {name: t[name][:n].cpu().numpy().view(dt) for name, dt in COLS}
    f = t["flags"][:n].cpu().numpy()
    out["state"] = f & 7
    out["isFemale"] = (f >> 3) & 1
    return out


def test_step_noalloc_matches_step(gpu_ready):
    torch = pytest.importorskip("torch")
    from sampo_gb300 import _lib, inputs
    from sampo_gb300.population import make_pool
    from sampo_gb300.sim import Simulation, pop_from_ranges, seed_stream
    lib = _lib.load()
    cap = 1 << 17
    cc = 4000.0
    ranges, arrays = make_pool((12000, 9000, 3000, 6000), 27.0, seed=11)
    n = 2
    T = np.array([27.0, 27.5], np.float32)
    env = np.zeros(n, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = cc
    env["ITNValue"] = 0.05
    _, seeds = seed_stream(21, n)

    # the allocating entry point
    sim = Simulation(capacity=cap, carrying_capacity=cc, max_steps=8)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.load_pool(ranges, arrays)
    ref_rows, ref_pools = [], []
    for i in range(n):
        ref_rows.append(sim.step(env[i], T[i], 18 + i, seeds[i]))
        ref_pools.append(sim.read_pool())
    ref_next = sim.current_row()
    sim.close()

    # the same two steps through sampo_step_noalloc on caller-owned buffers
    ta, da = _device_pool(torch, cap)
    tb, db = _device_pool(torch, cap)
    _upload(torch, ta, ranges, arrays)
    torch.cuda.synchronize()
    pop = pop_from_ranges(ranges)
    bufs = [(ta, da), (tb, db)]
    for i in range(n):
        (tin, din), (tout, dout) = bufs[i % 2], bufs[(i + 1) % 2]
        e = _lib.Environment(*[float(env[i][k]) for k in inputs.ENV_DTYPE.names])
        s = np.ascontiguousarray(seeds[i], dtype=np.uint32)
        row, pop_out, bnc = _lib.StatsRow(), _lib.Population(), _lib.BitesCycles()
        rc = lib.sampo_step_noalloc(C.byref(din), cap, C.byref(dout), cap, C.byref(pop), C.byref(e),
                                    float(T[i]), 18 + i, s.ctypes.data, cc, C.byref(row), C.byref(pop_out),
                                    C.byref(bnc), 0, None)
        assert rc == 0, f"step {i}: sampo_step_noalloc returned {rc}"
        got = np.frombuffer(bytes(row), dtype=_lib.ROW_DTYPE)[0]
        want = ref_rows[i]
        # the allocating path's row carries the previous step's counters; the
        # no-allocation call reports them separately (bnc_out)
        assert got["ranges"].tobytes() == want["ranges"].tobytes()
        assert (got["L1de"], got["numFemale"], got["numPotInf"]) == (want["L1de"], want["numFemale"], want["numPotInf"])
        ref_pop, ref_arrays = ref_pools[i]
        got_ranges = np.array([[pop_out.r[k].start, pop_out.r[k].end] for k in range(8)], dtype=np.uint32)
        assert np.array_equal(got_ranges, ref_pop["ranges"]), f"step {i}: next ranges differ"
        nxt = ref_next if i == n - 1 else ref_rows[i + 1]
        assert (bnc.numCyclesReported, bnc.sumCyclesReported, bnc.numBitesReported, bnc.numInfectBitesReported) == \
            (nxt["numCycles"], nxt["sumCycles"], nxt["numBites"], nxt["numInfectBites"])
        assert (pop_out.numLarvae1DayEquiv, pop_out.numFemale, pop_out.numPotentiallyInfective) == \
            (nxt["L1de"], nxt["numFemale"], nxt["numPotInf"])
        got_arrays = _download(tout, int(got_ranges[7][1]))
        for k in range(8):
            a, b = int(got_ranges[k][0]), int(got_ranges[k][1])
            for name in got_arrays:
                x, y = got_arrays[name][a:b], ref_arrays[name][a:b]
                if x.dtype == np.float32:
                    x, y = x.view(np.uint32), y.view(np.uint32)
                assert np.array_equal(x, y), f"step {i}: range {k} field {name} differs"
        pop = pop_out


def test_step_noalloc_rejects_oversized_pools(gpu_ready):
    from sampo_gb300 import _lib
    lib = _lib.load()
    d = _lib.DevicePool()
    pop = _lib.Population()
    e = _lib.Environment(0.25, 0, 0, 100.0, 0, 0)
    s = np.zeros(16, np.uint32)
    row, po, b = _lib.StatsRow(), _lib.Population(), _lib.BitesCycles()
    big = (1 << 24) + 1
    assert lib.sampo_step_noalloc(C.byref(d), big, C.byref(d), 1024, C.byref(pop), C.byref(e), 25.0, 0,
                                  s.ctypes.data, 100.0, C.byref(row), C.byref(po), C.byref(b), 0, None) == -1
    assert lib.sampo_step_noalloc(C.byref(d), 1024, C.byref(d), big, C.byref(pop), C.byref(e), 25.0, 0,
                                  s.ctypes.data, 100.0, C.byref(row), C.byref(po), C.byref(b), 0, None) == -1


def test_step_noalloc_rejects_overlapping_buffers(gpu_ready):
    """The step reads `in` while it writes `out`: the same buffers, or a
    column of one inside the other, are refused before anything runs."""
    torch = pytest.importorskip("torch")
    from sampo_gb300 import _lib
    lib = _lib.load()
    cap = 4096
    ta, da = _device_pool(torch, cap)
    tb, db = _device_pool(torch, cap)
    pop = _lib.Population()
    for k in range(8):
        pop.r[k].start = pop.r[k].end = 64 * (k + 1) if k else 0
    pop.r[0].end = 10
    e = _lib.Environment(0.25, 0, 0, 100.0, 0, 0)
    s = np.zeros(16, np.uint32)
    row, po, b = _lib.StatsRow(), _lib.Population(), _lib.BitesCycles()

    def call(din, dout):
        return lib.sampo_step_noalloc(C.byref(din), cap, C.byref(dout), cap, C.byref(pop), C.byref(e), 25.0, 0,
                                      s.ctypes.data, 100.0, C.byref(row), C.byref(po), C.byref(b), 0, None)
    assert call(da, da) == -1
    mixed = _lib.DevicePool(**{f: getattr(db, f) for f, _ in _lib.DevicePool._fields_})
    mixed.flags = da.flags
    assert call(da, mixed) == -1
    torch.cuda.synchronize()
