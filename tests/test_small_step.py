"""The one-launch day for small pools (k_step_small) against the three-kernel
step: day graphs picked per day on the host, at either tile size, give the
same rows and pools as the three-kernel step every hour, across the size
threshold and beyond the one-launch grid (more tiles than CTAs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(ranges, arrays, T, env, seeds, cc, n, max_tiles, capacity, items=0):
    from sampo_gb300.sim import Simulation
    sim = Simulation(capacity=capacity, carrying_capacity=cc, max_steps=n + 1)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.set_small_step(max_tiles)
    sim.set_small_step_items(items)
    sim.load_pool(ranges, arrays)
    rows = sim.run(n)
    info = sim.small_step_info()
    pop, pool = sim.read_pool()
    hist = sim.histogram()
    status = sim.device_status()
    launches = sim.kernel_times()[1]
    sim.close()
    return rows, pop, pool, hist, status, info, launches


def _workload(sizes, n, cc, seed):
    from sampo_gb300 import inputs
    from sampo_gb300.population import make_pool
    from sampo_gb300.sim import seed_stream
    w = inputs.seasonal_weather(n // 24 + 1, seed, 27.0, 3.0, 0.5)
    T = np.repeat(w.temperature_c.astype(np.float32), 24)[:n]
    env = np.zeros(n, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = cc
    env["ITNValue"][n // 2:n // 2 + 30] = 0.05
    ranges, arrays = make_pool(sizes, T[0], seed=seed)
    _, seeds = seed_stream(seed, n)
    return ranges, arrays, T, env, seeds


@pytest.mark.parametrize("sizes,n,cc", [((8000, 6000, 2000, 4000), 240, 50000.0),
                                        ((200000, 150000, 50000, 100000), 72, 2.0e6)])
def test_paths_agree(gpu_ready, oracle_mod, sizes, n, cc):
    """Never / always / default / a threshold inside the run's range of sizes:
    identical rows, pools, histograms. The second pool grows from 489 to
    about 2,500 tiles, more than the one-launch grid has CTAs, so 'always'
    takes the route that visits a CTA's extra tiles twice. The one-launch
    step's 256-, 512- and 1024-slot tiles are also forced on their own."""
    ranges, arrays, T, env, seeds = _workload(sizes, n, cc, seed=11)
    cap = 1 << 22
    ref = _run(ranges, arrays, T, env, seeds, cc, n, 0, cap)
    assert ref[4] == 0 and ref[5]["days_one_launch"] == 0 and ref[5]["days_three_kernel"] == n // 24
    tiles = (ref[0]["ranges"][:, 7, 1].astype(np.int64) + 1023) // 1024
    mid = int(np.median(tiles))
    # (max_tiles, slots per thread of the one-launch step: 0 by pool size)
    for max_tiles, items in ((1 << 30, 0), (None, 0), (mid, 0), (1 << 30, 1), (1 << 30, 2), (1 << 30, 4)):
        got = _run(ranges, arrays, T, env, seeds, cc, n, max_tiles, cap, items)
        assert got[4] == 0, f"max_tiles={max_tiles}, items={items}: device status {got[4]:#x}"
        info = got[5]
        assert info["days_one_launch"] + info["days_three_kernel"] == n // 24, info
        if max_tiles == 1 << 30 or (max_tiles is None and sizes[0] == 8000):  # every day small enough for the pick
            assert info["days_one_launch"] == n // 24, info
        if max_tiles == mid and sizes[0] == 8000:  # the pick changes during the ten days
            assert 0 < info["days_one_launch"] < n // 24, info
        for i in range(n):
            assert got[0][i].tobytes() == ref[0][i].tobytes(), f"max_tiles={max_tiles}, items={items}: row {i}"
        assert np.array_equal(got[1]["ranges"], ref[1]["ranges"])
        assert oracle_mod.pool_hash(got[1]["ranges"], got[2]) == oracle_mod.pool_hash(ref[1]["ranges"], ref[2])
        assert np.array_equal(got[3], ref[3])
    if sizes[0] == 8000:
        # a small pool takes one launch per simulated day (plus the constants
        # refresh at the start of the run)
        got = _run(ranges, arrays, T, env, seeds, cc, n, None, cap)
        assert got[6] == 1 + n // 24, got[6]


def test_small_step_matches_oracle(gpu_ready, oracle_mod):
    """A small mixed-stage pool under the one-launch step, row by row and
    slot by slot against the CPU oracle."""
    from oracle import OracleSim
    n = 192
    cc = 30000.0
    ranges, arrays, T, env, seeds = _workload((3000, 2500, 1000, 2000), n, cc, seed=4)
    rows, pop, pool, hist, status, info, _ = _run(ranges, arrays, T, env, seeds, cc, n, None, 1 << 20)
    assert status == 0 and info["days_one_launch"] == n // 24 and info["last_day"] in (2, 3)
    orc = OracleSim(1 << 20)
    orc.load_pool(ranges, arrays)
    for i in range(n):
        assert rows[i].tobytes() == orc.step(env[i], T[i], i % 24, seeds[i]).tobytes(), f"step {i}"
    ro, ao = orc.read_pool()
    assert np.array_equal(np.asarray(pop["ranges"], np.int64), np.asarray(ro, np.int64))
    for k in range(8):
        s, e = int(ro[k][0]), int(ro[k][1])
        for name in ao:
            x, y = pool[name][s:e], ao[name][s:e]
            if x.dtype == np.float32:
                x, y = x.view(np.uint32), y.view(np.uint32)
            assert np.array_equal(x, y), f"range {k} field {name}"
    assert np.array_equal(hist, orc.histogram())


@pytest.mark.parametrize("items", [1, 2, 4])
def test_pool_outgrowing_its_grid_matches_golden(gpu_ready, tmp_path, items):
    """The golden interventions case (a few thousand agents, 40 days): each
    day's grid is picked from the pool end seen two days earlier, so on some
    days the pool holds more tiles than the grid has CTAs and the statistics
    come from fewer CTAs than tiles. Every stats line equals the reference's."""
    from tests.conftest import load_golden
    from tests.golden.cases import CASES, make_case_inputs
    from sampo_gb300 import inputs
    from sampo_gb300.sim import Simulation, seed_stream, stats_lines
    name = "small_b"
    c = CASES[name]
    n = c["steps"]
    tp, ep, _ = make_case_inputs(name, str(tmp_path))
    T = inputs.read_temperature(tp, n)
    env = inputs.read_environment(ep, n, c["cc"])
    init, seeds = seed_stream(c["seed"], n)
    with Simulation(capacity=1 << 21, carrying_capacity=c["cc"], max_steps=n + 1) as sim:
        sim.set_inputs(T, env)
        sim.set_seeds(0, seeds)
        sim.set_small_step_items(items)
        sim.init_population(c["initial"], init, c["age_days"], c["age_seed"])
        rows = sim.run(n)
        assert sim.device_status() == 0
        assert sim.small_step_info()["days_one_launch"] == n // 24
    g = load_golden(name)
    assert stats_lines(rows, T, rows[0]["ranges"])[1:] == g["trace"][1:]
