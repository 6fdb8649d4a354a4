"""Checkpoint / resume: a simulation saved at a step boundary and resumed in
a new handle continues bit for bit like the uninterrupted run."""
import numpy as np
import pytest

from tests.conftest import load_golden
from tests.golden.cases import CASES, make_case_inputs


@pytest.mark.gpu
def test_resumed_run_equals_uninterrupted_run(gpu_ready, tmp_path):
    from sampo_gb300 import inputs
    from sampo_gb300.sim import Simulation, seed_stream, stats_lines
    name = "small_b"                      # interventions switching on and off
    c = CASES[name]
    n, k = c["steps"], 400
    tp, ep, _ = make_case_inputs(name, str(tmp_path))
    T = inputs.read_temperature(tp, n)
    env = inputs.read_environment(ep, n, c["cc"])
    init, seeds = seed_stream(c["seed"], n)

    def fresh():
        sim = Simulation(capacity=1 << 21, carrying_capacity=c["cc"], max_steps=n + 1)
        sim.set_inputs(T, env)
        sim.set_seeds(0, seeds)
        return sim

    sim = fresh()
    sim.init_population(c["initial"], init, c["age_days"], c["age_seed"])
    full = np.concatenate([sim.run(n), [sim.current_row()]])
    pool_full, arrays_full = sim.read_pool()
    hist_full = sim.histogram()
    sim.close()

    sim = fresh()
    sim.init_population(c["initial"], init, c["age_days"], c["age_seed"])
    first = sim.run(k)
    ck = str(tmp_path / "sim.ck")
    sim.checkpoint(ck)
    sim.close()

    sim = fresh()
    sim.resume(ck)
    assert sim.get_step() == k
    assert sim.current_row().tobytes() == full[k].tobytes()
    rest = np.concatenate([sim.run(n - k), [sim.current_row()]])
    assert np.concatenate([first, rest]).tobytes() == full.tobytes()
    pool, arrays = sim.read_pool()
    assert np.array_equal(pool["ranges"], pool_full["ranges"])
    for name_, col in arrays.items():
        a, b = col, arrays_full[name_]
        if a.dtype == np.float32:
            a, b = a.view(np.uint32), b.view(np.uint32)
        assert np.array_equal(a, b), name_
    assert np.array_equal(sim.histogram(), hist_full)
    # and the trace is the reference's own
    g = load_golden(name)
    assert stats_lines(full[:n], T, full[0]["ranges"]) [1:] == g["trace"][1:]
    sim.close()


def test_checkpoint_errors_without_gpu(sampo_lib, tmp_path):
    assert sampo_lib.sampo_checkpoint_save(None, b"x") == -1
    assert sampo_lib.sampo_checkpoint_load(None, b"x") == -1
