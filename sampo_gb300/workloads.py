"""The synthetic workloads of the benchmark and the at-size parity tests, in
the reference's input formats (hourly temperature, environment rows, glibc
rand() seeds) and with mixed-stage initial pools (sampo_gb300.population).

  roofline      5e7 preloaded agents uniform over egg / larva / pupa / adult
                (50/50 gender), 1e8 slots, 28 C constant, 90 days, seed 3
  roofline-5m   the same mix at 5e6 agents and 1e7 slots (small captures)
  plain-large   1e6 agents 40/30/10/20, 2^27 slots, seasonal weather seed 2,
                730 days, carrying capacity 5 x 1e6
  plain-small   10,000 eggs aged U{0..3} days, 2^20 slots, 365 days, seed 1

Relative humidity and rainfall are drawn with the weather and have no
consumer in the reference (kernel/killAgents.cl:118 hard-codes the rainfall
coefficient), so they do not reach the step.
"""
from __future__ import annotations

import numpy as np

WORKLOADS = {
    # the large plain run
    "plain-large": dict(name="plain large run: 1e6 agents (egg/larva/pupa/adult 40/30/10/20), 2^27 slots, 730 days, seasonal weather seed 2",
                        counts=(400_000, 300_000, 100_000, 200_000), capacity=1 << 27, days=730, seed=2,
                        cc=5_000_000.0, weather=("seasonal", 2, 26.0, 4.0, 0.5)),
    # the bandwidth-roofline run
    "roofline": dict(name="roofline run: 5e7 preloaded agents (uniform over 4 stages, 50/50 gender), 1e8 slots, 28 C constant, 90 days, seed 3",
                     counts=(12_500_000,) * 4, capacity=100_000_000, days=90, seed=3, cc=3_000_000.0,
                     weather=("constant", 28.0)),
    # the roofline mix at a size whose ncu captures stay small (5e6 agents, 0.74 GB of pools)
    "roofline-5m": dict(name="roofline mix at 5e6 agents: preloaded uniform over 4 stages, 50/50 gender, 1e7 slots, 28 C constant, seed 3",
                        counts=(1_250_000,) * 4, capacity=10_000_000, days=90, seed=3, cc=300_000.0,
                        weather=("constant", 28.0)),
    # the CPU-runnable plain case: eggs only
    "plain-small": dict(name="plain single run: 10,000 eggs aged U{0..3} days, 2^20 slots, 365 days, seed 1",
                        eggs=10_000, capacity=1 << 20, days=365, seed=1, cc=50_000.0,
                        weather=("seasonal", 1, 26.0, 4.0, 0.5)),
}


def build_workload(wl: dict, days: int, seed_fn=None):
    """Hourly temperature and environment rows for `days` days, the initial
    seeds and the per-step seed stream, and the initial pool (None for the
    egg-only workload): (T, env, init, seeds, pool)."""
    from . import inputs
    from .population import make_pool
    if seed_fn is None:
        from .sim import seed_stream as seed_fn
    w = wl["weather"]
    if w[0] == "seasonal":
        weather = inputs.seasonal_weather(days, w[1], w[2], w[3], w[4])
    else:
        weather = inputs.constant_weather(days, w[1])
    T = np.repeat(weather.temperature_c.astype(np.float32), 24)
    n = days * 24
    env = np.zeros(n, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = np.float32(wl["cc"])
    init, seeds = seed_fn(wl["seed"], n)
    pool = None
    if "counts" in wl:
        pool = make_pool(wl["counts"], T[0], seed=wl["seed"])
    return T, env, init, seeds, pool
