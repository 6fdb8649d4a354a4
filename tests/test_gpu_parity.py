"""Parity of the CUDA path (libsampo_cuda.so through the C ABI) with the CPU
oracle and with the reference's own golden traces. Bit-exact: every stats
line, every field of every live slot, the pool hash, the histogram."""
import numpy as np
import pytest

from tests.conftest import load_golden
from tests.golden.cases import CASES, make_case_inputs

pytestmark = pytest.mark.gpu


def _inputs(name, tmp_path, n):
    from sampo_gb300 import inputs
    c = CASES[name]
    tp, ep, _ = make_case_inputs(name, str(tmp_path))
    T = inputs.read_temperature(tp, n)
    env = inputs.read_environment(ep, n, c["cc"])
    return c, T, env


def _sim_for_case(name, tmp_path, n, capacity=1 << 21):
    from sampo_gb300.sim import Simulation, seed_stream
    c, T, env = _inputs(name, tmp_path, n)
    init, seeds = seed_stream(c["seed"], n)
    sim = Simulation(capacity=capacity, carrying_capacity=c["cc"], max_steps=n + 1)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.init_population(c["initial"], init, c["age_days"], c["age_seed"])
    return sim, c, T, env, init, seeds


def test_device_math_matches_host(gpu_ready, oracle_mod):
    """sampo_math.h gives the same bits on sm_103a as on the host."""
    import ctypes
    lib = oracle_mod.load()
    lib.orc_eval_math.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
    rng = np.random.default_rng(0)
    doms = {0: (-30, 30), 1: (2.0 ** -32, 4.0), 2: (0, 6.2831855), 3: (0.0, 1.0)}
    for fn, (lo, hi) in doms.items():
        x = rng.uniform(lo, hi, 200000).astype(np.float32)
        y = np.where(rng.uniform(size=x.size) < 0.5, np.float32(1 / 24), rng.integers(0, 60, x.size)).astype(np.float32)
        host = np.zeros_like(x)
        dev = np.zeros_like(x)
        lib.orc_eval_math(fn, x.ctypes.data, y.ctypes.data, host.ctypes.data, x.size)
        assert gpu_ready.sampo_eval_math(fn, x.ctypes.data, y.ctypes.data, dev.ctypes.data, x.size, 0) == 0
        assert np.array_equal(host.view(np.uint32), dev.view(np.uint32)), f"fn {fn}"


def test_device_fast_paths_match_definitions(gpu_ready, oracle_mod):
    """The normal draw's binary32 log and sin (fn 4, 5) equal the binary64
    definitions (fn 1, 2) on the device for every input of their domains, and
    the host definitions on a sample."""
    import ctypes
    lib = oracle_mod.load()
    lib.orc_eval_math.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
    lo = int(np.float32(2.0 ** -32).view(np.uint32))
    hi = int(np.float32(1.0).view(np.uint32))
    u_all = np.arange(lo, hi + 1, dtype=np.uint32).view(np.float32)
    u_all = np.concatenate([np.zeros(1, np.float32), u_all])
    chunk = 1 << 26
    for fast, ref in ((4, 1), (5, 2)):
        for s in range(0, u_all.size, chunk):
            u = u_all[s:s + chunk]
            x = u if fast == 4 else (np.float32(6.2831855) * u).astype(np.float32)
            a = np.empty_like(x)
            b = np.empty_like(x)
            assert gpu_ready.sampo_eval_math(fast, x.ctypes.data, None, a.ctypes.data, x.size, 0) == 0
            assert gpu_ready.sampo_eval_math(ref, x.ctypes.data, None, b.ctypes.data, x.size, 0) == 0
            bad = np.nonzero(a.view(np.uint32) != b.view(np.uint32))[0]
            assert bad.size == 0, f"fn {fast}: x={x[bad[0]]!r} fast {a[bad[0]]!r} definition {b[bad[0]]!r}"
            if s == 0:
                xs = np.ascontiguousarray(x[::61])
                h = np.empty_like(xs)
                lib.orc_eval_math(ref, xs.ctypes.data, xs.ctypes.data, h.ctypes.data, xs.size)
                assert np.array_equal(h.view(np.uint32), a[::61].view(np.uint32)), f"fn {fast} vs host"


def _compare_pools(ra, aa, rb, ab, where):
    assert np.array_equal(np.asarray(ra, np.int64), np.asarray(rb, np.int64)), f"{where}: ranges differ"
    for k in range(8):
        s, e = int(ra[k][0]), int(ra[k][1])
        for name in aa:
            x, y = aa[name][s:e], ab[name][s:e]
            if x.dtype == np.float32:
                x, y = x.view(np.uint32), y.view(np.uint32)
            bad = np.nonzero(x != y)[0]
            assert bad.size == 0, f"{where}: state range {k} field {name} differs at slot {s + bad[0]}"


@pytest.mark.parametrize("name,n", [("small_a", 400), ("interventions", 500)])
def test_step_by_step_against_oracle(gpu_ready, oracle_mod, tmp_path, name, n):
    """sampo_step vs the oracle, comparing the full pool after every step."""
    from oracle import OracleSim
    sim, c, T, env, init, seeds = _sim_for_case(name, tmp_path, n)
    orc = OracleSim(1 << 21)
    orc.init_eggs(c["initial"], T[0], init, c["age_days"], c["age_seed"])
    for i in range(n):
        rg = sim.step(env[i], T[i], i % 24, seeds[i])
        ro = orc.step(env[i], T[i], i % 24, seeds[i])
        assert rg.tobytes() == ro.tobytes(), f"step {i}: stats row differs\n{rg}\n{ro}"
        if i % 7 == 0 or i == n - 1:
            pg, ag = sim.read_pool()
            rorc, ao = orc.read_pool()
            _compare_pools(pg["ranges"], ag, rorc, ao, f"after step {i}")
    assert np.array_equal(sim.histogram(), orc.histogram())
    sim.close()


@pytest.mark.parametrize("name", ["small_a", "small_b", "interventions", "reference_default", "eggs_1e4_year",
                                  "temperature_edges"])
def test_run_matches_reference_golden(gpu_ready, oracle_mod, tmp_path, name):
    """sampo_run (CUDA-graph days) against the reference's own trace: every
    printStats line, the pool hash at day boundaries, ranges, histogram.txt."""
    from sampo_gb300.sim import histogram_text, population_lines, stats_lines
    g = load_golden(name)
    n = CASES[name]["steps"]
    sim, c, T, env, init, seeds = _sim_for_case(name, tmp_path, n, capacity=6_000_000)
    initial = sim.initial_pop["ranges"]
    lines, done, chunk = [], 0, 24 * 10
    prev = None
    while done < n:
        m = min(chunk, n - done)
        rows = sim.run(m)
        lines += stats_lines(rows, T, initial, first_step=done, prev_ranges=prev)
        prev = rows[-1]["ranges"]
        done += m
        pop, arrays = sim.read_pool()
        assert format(oracle_mod.pool_hash(pop["ranges"], arrays), "016x") == g["pool_hash"][done - 1], f"pool after step {done - 1}"
    for i, (a, b) in enumerate(zip(lines, g["trace"])):
        assert a == b, f"step {i}: cuda {a!r} != reference {b!r}"
    assert len(lines) == len(g["trace"])
    pop, _ = sim.read_pool(ranges_only=True)
    assert population_lines(pop["ranges"]) == g["final_ranges"]
    assert histogram_text(sim.histogram()) == g["histogram_txt"]
    assert sim.device_status() == 0
    sim.close()


def test_mixed_stage_pool_matches_reference_golden(gpu_ready, oracle_mod, tmp_path):
    """The mixed-stage start of the reference's own code (ref-as-C from the
    same pool file): every printStats line, the pool hash after every day,
    the final ranges and histogram.txt, through sampo_run's day graphs."""
    from sampo_gb300.sim import Simulation, histogram_text, population_lines, seed_stream, stats_lines
    from tests.golden.cases import case_pool
    name = "mixed_pool"
    g = load_golden(name)
    n = CASES[name]["steps"]
    c, T, env = _inputs(name, tmp_path, n)
    ranges, arrays = case_pool(name, T[0])
    _, seeds = seed_stream(c["seed"], n)
    sim = Simulation(capacity=1 << 18, carrying_capacity=c["cc"], max_steps=n + 1)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.load_pool(ranges, arrays)
    lines, done, prev = [], 0, None
    while done < n:
        rows = sim.run(24)
        lines += stats_lines(rows, T, ranges, first_step=done, prev_ranges=prev)
        prev = rows[-1]["ranges"]
        done += 24
        pop, pool = sim.read_pool()
        assert format(oracle_mod.pool_hash(pop["ranges"], pool), "016x") == g["pool_hash"][done - 1], f"pool after step {done - 1}"
    for i, (a, b) in enumerate(zip(lines, g["trace"])):
        assert a == b, f"step {i}: cuda {a!r} != reference {b!r}"
    assert len(lines) == len(g["trace"])
    pop, _ = sim.read_pool(ranges_only=True)
    assert population_lines(pop["ranges"]) == g["final_ranges"]
    assert histogram_text(sim.histogram()) == g["histogram_txt"]
    assert sim.device_status() == 0
    sim.close()


def test_mixed_stage_pool_against_oracle(gpu_ready, oracle_mod):
    """A loaded mixed-stage pool (all eight states populated) stepped on both."""
    from oracle import OracleSim
    from sampo_gb300 import inputs
    from sampo_gb300.population import make_pool
    from sampo_gb300.sim import Simulation, seed_stream
    n = 480
    w = inputs.seasonal_weather(n // 24 + 1, 3, 27.0, 3.0, 0.5)
    T = np.repeat(w.temperature_c.astype(np.float32), 24)[:n]
    env = np.zeros(n, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = 50000.0
    env["ITNValue"][240:300] = 0.05
    ranges, arrays = make_pool((8000, 6000, 2000, 4000), T[0], seed=5)
    init, seeds = seed_stream(99, n)
    sim = Simulation(capacity=1 << 21, carrying_capacity=50000.0, max_steps=n + 1)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.load_pool(ranges, arrays)
    orc = OracleSim(1 << 21)
    orc.load_pool(ranges, arrays)
    rows = sim.run(n)
    for i in range(n):
        ro = orc.step(env[i], T[i], i % 24, seeds[i])
        assert rows[i].tobytes() == ro.tobytes(), f"step {i}"
    pg, ag = sim.read_pool()
    ro_, ao = orc.read_pool()
    _compare_pools(pg["ranges"], ag, ro_, ao, "end")
    assert np.array_equal(sim.histogram(), orc.histogram())
    sim.close()


def test_graph_replay_equals_single_launches(gpu_ready, oracle_mod, tmp_path):
    """Day graphs and per-kernel launches (timing mode) give identical pools."""
    hashes = []
    for timing in (False, True):
        sim, *_ = _sim_for_case("small_b", tmp_path, 480)
        sim.set_timing(timing)
        sim.run(480)
        pop, arrays = sim.read_pool()
        hashes.append(oracle_mod.pool_hash(pop["ranges"], arrays))
        if timing:
            t, launches = sim.kernel_times()
            # one constants refresh, then count + scatter + publish per step
            assert launches == 1 + 3 * 480 and t[0] > 0 and t[1] > 0
        sim.close()
    assert hashes[0] == hashes[1]


def test_reinitialised_handle_repeats_exactly(gpu_ready, oracle_mod):
    """Re-initialising one handle (new look-back epochs over tile flags left
    by the previous run) reproduces the first run bit for bit."""
    from sampo_gb300 import inputs
    from sampo_gb300.population import make_pool
    from sampo_gb300.sim import Simulation, seed_stream
    n = 240
    T = np.full(n, 28.0, np.float32)
    env = np.zeros(n, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = 12000.0
    ranges, arrays = make_pool((50000, 50000, 50000, 50000), 28.0, seed=3)
    init, seeds = seed_stream(3, n)
    sim = Simulation(capacity=1 << 20, carrying_capacity=12000.0, max_steps=n + 1)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    results = []
    for timing in (False, True, False):
        sim.load_pool(ranges, arrays)
        sim.set_timing(timing)
        rows = sim.run(n)
        pop, pool = sim.read_pool()
        results.append((rows.tobytes(), oracle_mod.pool_hash(pop["ranges"], pool)))
    assert results[0] == results[1] == results[2]
    sim.close()


def test_capacity_exhaustion_is_reported(gpu_ready, tmp_path):
    from sampo_gb300._lib import SampoError
    sim, *_ = _sim_for_case("small_a", tmp_path, 720, capacity=1200)
    with pytest.raises(SampoError) as e:
        sim.run(720)
    assert e.value.code == -3
    sim.close()


def test_temperature_outside_devrates_is_reported(gpu_ready, tmp_path):
    """T >= 44 C with larvae present: the reference reads past devRates."""
    from sampo_gb300._lib import SampoError
    from sampo_gb300.sim import Simulation, seed_stream
    n = 48
    T = np.full(n, 30.0, np.float32)
    T[40:] = 45.0
    env = np.zeros(n, dtype=__import__("sampo_gb300.inputs", fromlist=["x"]).ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = 5000.0
    init, seeds = seed_stream(3, n)
    sim = Simulation(capacity=1 << 16, carrying_capacity=5000.0, max_steps=n + 1)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.init_population(1000, init, 3, 1)
    with pytest.raises(SampoError) as e:
        sim.run(n)
    assert e.value.code == -4
    sim.close()


def test_reference_initial_layout_warning(gpu_ready):
    """Eggs hatching in the first step on the reference's shared empty ranges
    (only at absurd temperatures with age-0 eggs) raise the warning bit."""
    from sampo_gb300 import _lib
    from sampo_gb300.sim import Simulation, seed_stream
    T = np.full(4, 70.0, np.float32)
    env = np.zeros(4, dtype=_lib.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = 5000.0
    init, seeds = seed_stream(5, 4)
    sim = Simulation(capacity=1 << 16, carrying_capacity=5000.0, max_steps=8)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.init_population(2000, init)
    sim.run(1)
    assert sim.device_status() & _lib.DEV_WARN_REF_LAYOUT
    sim.close()


def test_extinction_keeps_running(gpu_ready, oracle_mod):
    """A population that dies out leaves empty ranges and zero counts; the
    library keeps stepping (the reference's driver asserts, src/abms.c:307)."""
    from oracle import OracleSim
    from sampo_gb300 import _lib
    from sampo_gb300.sim import Simulation, seed_stream
    n = 300
    T = np.full(n, 25.0, np.float32)
    env = np.zeros(n, dtype=_lib.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = 100.0
    env["larvacideValue"] = 1.0
    init, seeds = seed_stream(8, n)
    sim = Simulation(capacity=1 << 12, carrying_capacity=100.0, max_steps=n + 1)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.init_population(5, init, 3, 2)
    orc = OracleSim(1 << 12)
    orc.init_eggs(5, T[0], init, 3, 2)
    rows = sim.run(n)
    for i in range(n):
        assert rows[i].tobytes() == orc.step(env[i], T[i], i % 24, seeds[i]).tobytes()
    r = rows[-1]["ranges"]
    assert int((r[:, 1] - r[:, 0]).sum()) == 0
    sim.close()
