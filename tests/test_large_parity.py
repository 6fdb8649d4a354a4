"""Bit-exactness at full size: the roofline workload (5e7 preloaded agents,
uniform over four stages, 50/50 gender, in a 1e8-slot pool, 28 C) stepped for
one simulated day on the GPU (a day graph) and by the oracle on the host
cores. Every stats row and, after the day, every slot of the pool must be
identical."""
import numpy as np
import pytest

from tests.test_gpu_parity import _compare_pools


@pytest.mark.gpu
def test_roofline_pool_5e7_bit_exact_against_oracle(gpu_ready, oracle_mod):
    from oracle import OracleSim
    from sampo_gb300 import inputs
    from sampo_gb300.population import make_pool
    from sampo_gb300.sim import Simulation, seed_stream
    steps, capacity, cc = 24, 100_000_000, 3_000_000.0
    weather = inputs.constant_weather(1, 28.0)
    T = np.repeat(weather.temperature_c.astype(np.float32), 24)[:steps]
    env = np.zeros(steps, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = np.float32(cc)
    ranges, arrays = make_pool((12_500_000,) * 4, T[0], seed=3)
    _, seeds = seed_stream(3, steps)
    with Simulation(capacity=capacity, carrying_capacity=cc, max_steps=steps + 1) as sim:
        sim.set_inputs(T, env)
        sim.set_seeds(0, seeds)
        sim.load_pool(ranges, arrays)
        rows = sim.run(steps)
        pg, ag = sim.read_pool()
        assert sim.device_status() == 0
    live = int(sum(int(e) - int(s) for s, e in pg["ranges"]))
    assert live > 25_000_000  # the preloaded mix loses about a third on its first day
    orc = OracleSim(capacity)
    orc.load_pool(ranges, arrays)
    del arrays
    for i in range(steps):
        ro = orc.step(env[i], T[i], i % 24, seeds[i])
        assert rows[i].tobytes() == ro.tobytes(), f"step {i}"
    ro_, ao = orc.read_pool()
    _compare_pools(pg["ranges"], ag, ro_, ao, "after one day")
    orc.close()


@pytest.mark.gpu
def test_plain_large_run_bit_exact_against_oracle(gpu_ready, oracle_mod):
    """The plain large run at its size (1e6 agents 40/30/10/20 in a 2^27-slot
    pool, seasonal weather seed 2, carrying capacity 5e6) over its first six
    simulated days: every stats row, and every slot after day 1 and after
    day 6 (the population passes 5e6 agents; days 5..6 are where the
    benchmark's timed window starts)."""
    from oracle import OracleSim
    from sampo_gb300.sim import Simulation
    from sampo_gb300.workloads import WORKLOADS, build_workload
    wl = WORKLOADS["plain-large"]
    days = 6
    steps = 24 * days
    T, env, init, seeds, (ranges, arrays) = build_workload(wl, days)
    with Simulation(capacity=wl["capacity"], carrying_capacity=wl["cc"], max_steps=steps + 1) as sim:
        sim.set_inputs(T, env)
        sim.set_seeds(0, seeds)
        sim.load_pool(ranges, arrays)
        rows = [sim.run(24)]
        pools = [sim.read_pool()]
        rows.append(sim.run(steps - 24))
        pools.append(sim.read_pool())
        assert sim.device_status() == 0
    rows = np.concatenate(rows)
    orc = OracleSim(wl["capacity"])
    orc.load_pool(ranges, arrays)
    del arrays
    for i in range(steps):
        ro = orc.step(env[i], T[i], i % 24, seeds[i])
        assert rows[i].tobytes() == ro.tobytes(), f"step {i}"
        if i + 1 in (24, steps):
            ro_, ao = orc.read_pool()
            pg, ag = pools[0 if i + 1 == 24 else 1]
            _compare_pools(pg["ranges"], ag, ro_, ao, f"after day {(i + 1) // 24}")
    live = int(sum(int(e) - int(s) for s, e in pools[1][0]["ranges"]))
    assert live > 4_000_000
    orc.close()
