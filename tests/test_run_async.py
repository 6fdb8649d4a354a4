"""sampo_run_async / sampo_sync: queued runs give the rows and pools of
sampo_run, bit for bit, across ring chunks and back-to-back queues; device
errors of queued steps surface at sampo_sync; any other call waits for the
queue first."""
import numpy as np
import pytest

from tests.test_gpu_parity import _inputs

pytestmark = pytest.mark.gpu


def _sim(name, tmp_path, n, max_steps, capacity=1 << 21):
    from sampo_gb300.sim import Simulation, seed_stream
    c, T, env = _inputs(name, tmp_path, n)
    init, seeds = seed_stream(c["seed"], n)
    sim = Simulation(capacity=capacity, carrying_capacity=c["cc"], max_steps=max_steps)
    sim.set_inputs(T[:n], env[:n])
    sim.set_seeds(0, seeds[:n])
    sim.init_population(c["initial"], init, c["age_days"], c["age_seed"])
    return sim


def test_run_async_equals_run(gpu_ready, oracle_mod, tmp_path):
    from sampo_gb300.sim import ROW_DTYPE, PinnedArray
    n = 480
    ref = _sim("small_b", tmp_path, n, n + 1)
    rows_ref = ref.run(n)
    pop_ref, pool_ref = ref.read_pool()
    ref.close()
    # a ring of n slots: the second queue crosses a chunk boundary (ring - 1 steps)
    sim = _sim("small_b", tmp_path, n, n)
    rows = PinnedArray((n,), ROW_DTYPE)
    try:
        first = 130
        sim.run_async(first, rows.p)
        sim.run_async(n - first, rows.p + first * ROW_DTYPE.itemsize)
        assert sim.get_step() == n
        sim.sync()
        assert sim.last_run_ms() > 0.0
        assert rows.a.tobytes() == rows_ref.tobytes()
        pop, pool = sim.read_pool()
        assert oracle_mod.pool_hash(pop["ranges"], pool) == oracle_mod.pool_hash(pop_ref["ranges"], pool_ref)
    finally:
        sim.close()
        rows.free()


def test_calls_wait_for_the_queue(gpu_ready, oracle_mod, tmp_path):
    """read_pool and histogram straight after sampo_run_async (no sync) see
    the pool after the queued steps; rows may be NULL."""
    n = 240
    ref = _sim("small_a", tmp_path, n, n + 1)
    ref.run(n, want_rows=False)
    pop_ref, pool_ref = ref.read_pool()
    hist_ref = ref.histogram()
    ref.close()
    sim = _sim("small_a", tmp_path, n, n + 1)
    sim.run_async(n)
    pop, pool = sim.read_pool()
    assert oracle_mod.pool_hash(pop["ranges"], pool) == oracle_mod.pool_hash(pop_ref["ranges"], pool_ref)
    assert np.array_equal(sim.histogram(), hist_ref)
    sim.sync()  # nothing left to wait for
    sim.close()


def test_queued_capacity_error_surfaces_at_sync(gpu_ready, tmp_path):
    from sampo_gb300._lib import SampoError
    sim = _sim("small_a", tmp_path, 720, 721, capacity=1200)
    sim.run_async(720)
    with pytest.raises(SampoError) as e:
        sim.sync()
    assert e.value.code == -3
    sim.close()


def test_step_after_queue(gpu_ready, oracle_mod, tmp_path):
    """sampo_step with explicit inputs straight after a queued run (no sync)
    continues from the queued steps: its row and the pool equal sampo_run's
    over the same steps."""
    from sampo_gb300.sim import seed_stream
    n, k = 200, 150
    ref = _sim("small_b", tmp_path, n, n + 1)
    rows_ref = ref.run(n)
    pop_ref, pool_ref = ref.read_pool()
    ref.close()
    c, T, env = _inputs("small_b", tmp_path, n)
    _, seeds = seed_stream(c["seed"], n)
    sim = _sim("small_b", tmp_path, n, n + 1)
    sim.run_async(k)
    for i in range(k, n):
        row = sim.step(env[i], T[i], i % 24, seeds[i])
        assert row.tobytes() == rows_ref[i].tobytes(), f"step {i}"
    assert sim.get_step() == n
    pop, pool = sim.read_pool()
    assert oracle_mod.pool_hash(pop["ranges"], pool) == oracle_mod.pool_hash(pop_ref["ranges"], pool_ref)
    sim.close()
