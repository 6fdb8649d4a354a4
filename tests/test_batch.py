"""Batches (sampo_batch_*): every replicate of a batch must equal the same
simulation run alone through the plain path - stats rows, final pool and age
histogram bit for bit - whatever else shares the batch, whenever it was
admitted and whichever slot it holds."""
import numpy as np
import pytest

from sampo_gb300.batch import ReplicateSpec

SPECS = [
    ReplicateSpec(initial=600, seed=11, mean_t=27.0, amplitude=3.0, rain_mean=4.0, days=3, capacity=40000),
    ReplicateSpec(initial=9000, seed=12, mean_t=24.0, amplitude=6.0, rain_mean=2.0, days=3, capacity=200000),
    ReplicateSpec(initial=40, seed=13, mean_t=29.5, amplitude=2.0, rain_mean=8.0, days=3, capacity=8192),
    ReplicateSpec(initial=2500, seed=14, mean_t=21.0, amplitude=8.0, rain_mean=5.0, days=3, capacity=60000,
                  age_days_max=-1),
    ReplicateSpec(initial=30000, seed=15, mean_t=28.0, amplitude=4.0, rain_mean=3.0, days=3, capacity=600000),
]


def plain_run(spec, steps):
    """The plain path alone: rows of steps 0..steps (row k = start of step k), pool, histogram."""
    from sampo_gb300.sim import Simulation, seed_stream
    T, env = spec.inputs()
    init, seeds = seed_stream(spec.seed, steps)
    with Simulation(capacity=spec.capacity, carrying_capacity=spec.cc, max_steps=steps + 1) as sim:
        sim.set_inputs(T[:steps], env[:steps])
        sim.set_seeds(0, seeds)
        sim.init_population(spec.initial, init, age_days_max=spec.age_days_max, age_seed=spec.seed)
        rows = sim.run(steps)
        rows = np.concatenate([rows, [sim.current_row()]])
        pop, arrays = sim.read_pool()
        return rows, pop, arrays, sim.histogram(), sim.device_status()


def compare(batch, slot, spec, steps, where):
    rows, pop, arrays, hist, status = plain_run(spec, steps)
    got = batch.rows(slot, 0, steps + 1)
    assert got.tobytes() == rows.tobytes(), f"{where}: stats rows differ from the plain run"
    bpop, barrays = batch.read_pool(slot)
    assert np.array_equal(bpop["ranges"], pop["ranges"]), f"{where}: ranges differ"
    for k in range(8):
        s, e = int(pop["ranges"][k][0]), int(pop["ranges"][k][1])
        for name in arrays:
            x, y = barrays[name][s:e], arrays[name][s:e]
            if x.dtype == np.float32:
                x, y = x.view(np.uint32), y.view(np.uint32)
            assert np.array_equal(x, y), f"{where}: range {k} field {name} differs"
    assert np.array_equal(batch.histogram(slot), hist), f"{where}: histogram differs"
    step, active, bits = batch.state(slot)
    assert step == steps and not active
    assert bits == status, f"{where}: status bits {bits:#x} vs plain {status:#x}"


@pytest.mark.gpu
def test_batch_replicates_equal_plain_runs(gpu_ready):
    from sampo_gb300.batch import Batch, admit
    steps = [72, 50, 72, 31, 72]
    with Batch(max_replicates=8, ring_steps=80) as b:
        slots = [admit(b, s, st) for s, st in zip(SPECS, steps)]
        b.run(48)          # two day graphs
        b.run(24, wait=False)
        b.sync()
        # a refresh per call, then count + update/scatter + publish per hour
        assert b.launches() == 2 + 3 * 72
        for s, spec, st in zip(slots, SPECS, steps):
            compare(b, s, spec, st, f"replicate {spec.seed}")


@pytest.mark.gpu
def test_continuous_batching_admits_and_retires(gpu_ready):
    """Replicates join a running batch at different batch steps and reuse the
    slots of finished ones; each still equals its plain run."""
    from sampo_gb300.batch import Batch, admit
    with Batch(max_replicates=3, ring_steps=80) as b:
        a = admit(b, SPECS[0], 30)
        c = admit(b, SPECS[4], 60)
        b.run(30)                      # a finishes, c is at step 30
        compare(b, a, SPECS[0], 30, "first occupant")
        b.remove(a)
        d = admit(b, SPECS[1], 40)     # takes a's slot, starts at its own step 0
        assert d == a
        e = admit(b, SPECS[3], 24)
        b.run(30)                      # c finishes at 60; e at 24; d at 30
        compare(b, c, SPECS[4], 60, "long-running")
        compare(b, e, SPECS[3], 24, "short joiner")
        b.run(15)                      # only d is left: it stops at 40
        compare(b, d, SPECS[1], 40, "slot reuser")


@pytest.mark.gpu
def test_capacity_error_stays_in_its_replicate(gpu_ready):
    """A replicate that outgrows its pool flags only itself; the others run on
    unchanged. (The oracle puts this one's layout end at 10820 slots at step
    336, past its 8000-slot pools.)"""
    from sampo_gb300.batch import Batch, admit
    from sampo_gb300._lib import SampoError
    tight = ReplicateSpec(initial=2000, seed=21, mean_t=29.0, amplitude=2.0, rain_mean=3.0, days=16, capacity=8000)
    with Batch(max_replicates=4, ring_steps=400) as b:
        t = admit(b, tight, 384)
        ok = admit(b, SPECS[0], 72)
        b.run(72)
        compare(b, ok, SPECS[0], 72, "neighbour of the overflowing replicate")
        b.run(312)
        _, _, bits = b.state(t)
        assert bits & 0x1, "the overflowing replicate carries SAMPO_DEV_ERR_CAPACITY"
    with pytest.raises(SampoError):
        from sampo_gb300.sim import Simulation
        with Simulation(capacity=tight.capacity, carrying_capacity=tight.cc, max_steps=385) as sim:
            from sampo_gb300.sim import seed_stream
            T, env = tight.inputs()
            init, seeds = seed_stream(tight.seed, 384)
            sim.set_inputs(T[:384], env[:384])
            sim.set_seeds(0, seeds)
            sim.init_population(tight.initial, init, age_days_max=3, age_seed=tight.seed)
            sim.run(384)


def test_replicate_bytes_without_gpu(sampo_lib):
    """The per-replicate footprint the admission policy budgets with is a host
    computation: two pool buffers of 37 B per slot (+ alignment and slack),
    the look-back tile arrays and the rings."""
    from sampo_gb300.batch import Batch
    b1 = Batch.replicate_bytes(1 << 20, 48)
    b2 = Batch.replicate_bytes(1 << 21, 48)
    assert 2 * 37 * (1 << 20) < b1 < 2 * 37 * (1 << 20) * 1.02
    assert abs((b2 - b1) - 2 * 37 * (1 << 20)) < 2 * 37 * (1 << 20) * 0.02
    assert sampo_lib.sampo_batch_destroy(None) == 0
    assert sampo_lib.sampo_batch_create(None, None) == -1


@pytest.mark.gpu
def test_grown_replicates_equal_plain_runs(gpu_ready):
    """Pools that start small and grow: a replicate whose next layout does not
    fit pauses at that step; sampo_batch_grow moves its pool (slot indices
    kept) into a larger allocation and the step runs again. Rows, pool and
    histogram still equal the plain run with room to spare, whether the slot
    was grown after a pause or ahead of need."""
    import dataclasses
    from sampo_gb300.batch import Batch, admit
    # the first two outgrow their pools on day 12 (the oracle's layout ends
    # pass 4096 at step 310 and 6000 at step 314, then reach 18714 slots)
    specs = [ReplicateSpec(initial=2000, seed=21, mean_t=29.0, amplitude=2.0, rain_mean=3.0, days=16, capacity=4096),
             ReplicateSpec(initial=2000, seed=21, mean_t=29.0, amplitude=2.0, rain_mean=3.0, days=16, capacity=6000),
             ReplicateSpec(initial=9000, seed=12, mean_t=24.0, amplitude=6.0, rain_mean=2.0, days=10, capacity=20000)]
    steps = [s.steps for s in specs]
    paused, grown_ahead = set(), False
    with Batch(max_replicates=4, ring_steps=max(steps) + 1) as b:
        slots = [admit(b, s, st, device_seeds=i == 0) for i, (s, st) in enumerate(zip(specs, steps))]
        for _ in range(max(steps) // 24 + 16):
            b.run(24)
            st = b.states()
            if all(st[s]["step"] == n for s, n in zip(slots, steps)):
                break
            for s, n in zip(slots, steps):
                o = st[s]
                if o["step"] < n and not o["active"]:
                    assert o["status"] & 0x1, o  # paused for capacity, nothing else
                    paused.add(s)
                    b.grow(s, 4 * int(o["end"]) + 1024)
                elif s == slots[2] and not grown_ahead and o["step"] >= 96:
                    b.grow(s, 3 * int(o["capacity"]))  # a running slot, ahead of need
                    grown_ahead = True
        assert len(paused) >= 2 and grown_ahead
        for s, spec, n in zip(slots, specs, steps):
            roomy = dataclasses.replace(spec, capacity=400_000)
            rows, pop, arrays, hist, status = plain_run(roomy, n)
            assert b.rows(s, 0, n + 1).tobytes() == rows.tobytes(), f"seed {spec.seed}: rows"
            bpop, barrays = b.read_pool(s)
            assert np.array_equal(bpop["ranges"], pop["ranges"])
            for name in arrays:
                x, y = barrays[name], arrays[name]
                if x.dtype == np.float32:
                    x, y = x.view(np.uint32), y.view(np.uint32)
                for k in range(8):
                    lo, hi = int(pop["ranges"][k][0]), int(pop["ranges"][k][1])
                    assert np.array_equal(x[lo:hi], y[lo:hi]), f"seed {spec.seed}: {name}"
            assert np.array_equal(b.histogram(s), hist)
            assert b.state(s)[2] == status == 0
