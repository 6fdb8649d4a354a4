"""The autotuner times the step kernels on the coming step and keeps the
fastest tile size (slots per thread) and grid sizes; a run tuned half-way must
equal the untuned run bit for bit (plain and batched), and so must runs with
either tile size."""
import numpy as np
import pytest

from tests.golden.cases import CASES, make_case_inputs


@pytest.mark.gpu
def test_autotune_leaves_the_run_unchanged(gpu_ready, tmp_path):
    from sampo_gb300 import inputs
    from sampo_gb300.sim import Simulation, seed_stream
    c = CASES["small_a"]
    n, k = c["steps"], 100
    tp, ep, _ = make_case_inputs("small_a", str(tmp_path))
    T = inputs.read_temperature(tp, n)
    env = inputs.read_environment(ep, n, c["cc"])
    init, seeds = seed_stream(c["seed"], n)
    out = []
    for tune in (False, True):
        with Simulation(capacity=1 << 20, carrying_capacity=c["cc"], max_steps=n + 1) as sim:
            sim.set_inputs(T, env)
            sim.set_seeds(0, seeds)
            sim.init_population(c["initial"], init, c["age_days"], c["age_seed"])
            rows = [sim.run(k)]
            if tune:
                cc_, cs = sim.autotune()
                assert 1 <= cc_ <= 8 and 1 <= cs <= 4
            rows.append(sim.run(n - k))
            pop, arrays = sim.read_pool()
            out.append((np.concatenate(rows), pop, arrays, sim.histogram(), sim.device_status()))
    (r0, p0, a0, h0, s0), (r1, p1, a1, h1, s1) = out
    assert r0.tobytes() == r1.tobytes()
    assert np.array_equal(p0["ranges"], p1["ranges"])
    for name in a0:
        assert a0[name].tobytes() == a1[name].tobytes(), name
    assert np.array_equal(h0, h1) and s0 == s1 == 0


@pytest.mark.gpu
def test_batch_autotune_leaves_replicates_unchanged(gpu_ready):
    from sampo_gb300.batch import Batch, admit
    from tests.test_batch import SPECS, compare
    with Batch(max_replicates=4, ring_steps=80) as b:
        slots = [admit(b, s, 72) for s in SPECS[:3]]
        b.run(24)
        cc_, cs = b.autotune()
        assert cc_ >= 1 and cs >= 1
        b.run(48)
        for slot, spec in zip(slots, SPECS[:3]):
            compare(b, slot, spec, 72, f"replicate {spec.seed} tuned half-way")


@pytest.mark.gpu
def test_set_grids_pins_the_choice(gpu_ready, tmp_path):
    """sampo_set_grids: any grid inside the occupancy limits gives the same run;
    values outside them are refused."""
    from sampo_gb300._lib import SampoError
    from sampo_gb300 import inputs
    from sampo_gb300.sim import Simulation, seed_stream
    c = CASES["small_a"]
    n = 96
    tp, ep, _ = make_case_inputs("small_a", str(tmp_path))
    T = inputs.read_temperature(tp, n)
    env = inputs.read_environment(ep, n, c["cc"])
    init, seeds = seed_stream(c["seed"], n)
    out = []
    for grids in (None, (1, 1), (3, 2)):
        with Simulation(capacity=1 << 20, carrying_capacity=c["cc"], max_steps=n + 1) as sim:
            sim.set_inputs(T, env)
            sim.set_seeds(0, seeds)
            sim.init_population(c["initial"], init, c["age_days"], c["age_seed"])
            if grids:
                sim.set_grids(*grids)
            out.append(sim.run(n).tobytes())
            with pytest.raises(SampoError):
                sim.set_grids(0, 1)
            with pytest.raises(SampoError):
                sim.set_grids(1, 64)
    assert out[1] == out[0] and out[2] == out[0]


@pytest.mark.gpu
def test_tile_size_does_not_change_results(gpu_ready, oracle_mod):
    """512- and 1024-slot tiles (2 or 4 slots per thread) through the
    three-kernel step: the same rows and pools; the autotuner's pick is one of
    them and keeps the run unchanged."""
    from sampo_gb300 import inputs
    from sampo_gb300.population import make_pool
    from sampo_gb300.sim import Simulation, seed_stream
    n = 144
    T = np.full(n, 27.5, np.float32)
    env = np.zeros(n, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = 40000.0
    ranges, arrays = make_pool((30000, 20000, 8000, 12000), T[0], seed=9)
    _, seeds = seed_stream(9, n)
    out = []
    for items in (4, 2, "tuned"):
        with Simulation(capacity=1 << 19, carrying_capacity=40000.0, max_steps=n + 1) as sim:
            sim.set_small_step(0)  # the three-kernel step every hour
            if items != "tuned":
                sim.set_items_per_thread(items)
                assert sim.items_per_thread() == items
            sim.set_inputs(T, env)
            sim.set_seeds(0, seeds)
            sim.load_pool(ranges, arrays)
            rows = [sim.run(48)]
            if items == "tuned":
                sim.autotune()
                assert sim.items_per_thread() in (2, 4)
            rows.append(sim.run(n - 48))
            pop, pool = sim.read_pool()
            assert sim.device_status() == 0
        out.append((np.concatenate(rows).tobytes(), oracle_mod.pool_hash(pop["ranges"], pool)))
    assert out[1] == out[0] and out[2] == out[0]


@pytest.mark.gpu
def test_batch_tile_size_does_not_change_replicates(gpu_ready):
    from sampo_gb300.batch import Batch, admit
    from tests.test_batch import SPECS, compare
    for items in (2, 4):
        with Batch(max_replicates=4, ring_steps=80) as b:
            b.set_items_per_thread(items)
            assert b.items_per_thread() == items
            slots = [admit(b, s, 72) for s in SPECS[:3]]
            b.run(72)
            for slot, spec in zip(slots, SPECS[:3]):
                compare(b, slot, spec, 72, f"replicate {spec.seed}, {items} slots per thread")


def test_items_per_thread_arguments(sampo_lib):
    """Only 2 and 4 slots per thread exist (checked without a device)."""
    assert sampo_lib.sampo_set_items_per_thread(None, 4) == -1
    assert sampo_lib.sampo_batch_set_items_per_thread(None, 2) == -1
