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


def test_checkpoint_info_without_gpu(sampo_lib, tmp_path):
    """sampo_checkpoint_info reads the header of a version-2 file (written
    here by hand: magic, version, step, cc, population, counters, n, flags,
    previous population) and refuses what is not a checkpoint."""
    import ctypes as C
    import struct
    from sampo_gb300._lib import Population
    pop = Population()
    for k in range(8):
        pop.r[k].start, pop.r[k].end = 0, 0
    prev = Population()
    prev.r[0].start, prev.r[0].end = 0, 7
    hdr = b"SAMPOCK1" + struct.pack("<IIf", 2, 123, 50.0) + bytes(pop) + bytes(16) + struct.pack("<II", 0, 1) + bytes(prev)
    hdr += bytes(4 + 31 * 4 + 4 + 64)   # seed stream (next, 31 words, i) and the coming seeds: unused
    p = tmp_path / "x.ck"
    p.write_bytes(hdr)
    step, has = C.c_uint32(), C.c_int()
    got = Population()
    assert sampo_lib.sampo_checkpoint_info(str(p).encode(), C.byref(step), None, C.byref(got), C.byref(has)) == 0
    assert step.value == 123 and has.value == 1 and got.r[0].end == 7
    (tmp_path / "y.ck").write_bytes(b"not a checkpoint at all" * 10)
    assert sampo_lib.sampo_checkpoint_info(str(tmp_path / "y.ck").encode(), None, None, None, None) == -7


@pytest.mark.gpu
@pytest.mark.parametrize("per_step", [False, True])
def test_cli_checkpoint_and_resume(gpu_ready, tmp_path, per_step):
    """sampo --checkpoint K F leaves the output unchanged; sampo --resume F
    prints the uninterrupted run's lines from step K on, its final ranges
    and histogram (the reference's, from the golden fixture)."""
    import subprocess
    from sampo_gb300 import build
    cli = build.build_cli()
    name = "small_a"
    c = CASES[name]
    g = load_golden(name)
    tp, ep, _ = make_case_inputs(name, str(tmp_path))
    n, k = c["steps"], 300
    base = [cli, "--seed", str(c["seed"]), "--initial", str(c["initial"]), "--cc", repr(c["cc"]),
            "--steps", str(n), "--age-days", str(c["age_days"]), "--age-seed", str(c["age_seed"])]
    if per_step:
        base.append("--per-step")
    ck = str(tmp_path / "run.ck")
    out = subprocess.run(base + ["--checkpoint", str(k), ck, tp, ep], capture_output=True, cwd=tmp_path, timeout=600)
    assert out.returncode == 0, out.stderr.decode()
    lines = out.stdout.decode().split("\n")
    assert lines[3:3 + n] == g["trace"] and lines[3 + n:3 + n + 8] == g["final_ranges"]
    (tmp_path / "histogram.txt").unlink()
    out = subprocess.run(base + ["--resume", ck, tp, ep], capture_output=True, cwd=tmp_path, timeout=600)
    assert out.returncode == 0, out.stderr.decode()
    lines = out.stdout.decode().split("\n")
    assert lines[3:3 + n - k] == g["trace"][k:]
    assert lines[3 + n - k:3 + n - k + 8] == g["final_ranges"]
    assert (tmp_path / "histogram.txt").read_text() == g["histogram_txt"]


@pytest.mark.gpu
def test_checkpoints_move_between_batches_and_simulations(gpu_ready, tmp_path):
    """A batch slot with a device seed stream, checkpointed mid-run, resumes
    in another batch and in a plain simulation (host seeds), and a plain
    simulation's checkpoint resumes in a batch slot: every continuation
    equals the uninterrupted batch run."""
    from sampo_gb300.batch import Batch, admit
    from sampo_gb300.sim import Simulation, seed_stream
    from tests.test_batch import SPECS
    spec, other = SPECS[1], SPECS[0]
    n, k = 72, 30
    with Batch(max_replicates=4, ring_steps=n + 1) as b:
        a = admit(b, spec, n, device_seeds=True)
        admit(b, other, n, device_seeds=True)
        b.run(k)
        ck_batch = str(tmp_path / "slot.ck")
        b.checkpoint(a, ck_batch)
        b.run(n - k)
        want = b.rows(a, 0, n + 1)
        pool_want, arrays_want = b.read_pool(a)
    T, env = spec.inputs()
    init, seeds = seed_stream(spec.seed, n)
    # batch -> batch (the seed stream travels with the slot)
    with Batch(max_replicates=2, ring_steps=n + 1) as b2:
        s = b2.add(spec.capacity, spec.cc, stop_step=n)
        b2.set_inputs(s, T[:n], env[:n])
        b2.resume(s, ck_batch)
        assert b2.state(s)[0] == k
        b2.run(n - k)
        assert b2.rows(s, k, n - k + 1).tobytes() == want[k:].tobytes()
        pool, arrays = b2.read_pool(s)
        assert np.array_equal(pool["ranges"], pool_want["ranges"])
        for name_ in arrays:
            x, y = arrays[name_], arrays_want[name_]
            if x.dtype == np.float32:
                x, y = x.view(np.uint32), y.view(np.uint32)
            assert np.array_equal(x, y), name_
    # batch -> plain simulation (host seeds from the same stream)
    with Simulation(capacity=spec.capacity, carrying_capacity=spec.cc, max_steps=n + 1) as sim:
        sim.set_inputs(T[:n], env[:n])
        sim.set_seeds(0, seeds)
        sim.resume(ck_batch)
        rest = np.concatenate([sim.run(n - k), [sim.current_row()]])
        assert rest.tobytes() == want[k:].tobytes()
        ck_plain = str(tmp_path / "plain.ck")
        sim2 = Simulation(capacity=spec.capacity, carrying_capacity=spec.cc, max_steps=n + 1)
        sim2.set_inputs(T[:n], env[:n])
        sim2.set_seeds(0, seeds)
        sim2.init_population(spec.initial, init, age_days_max=spec.age_days_max, age_seed=spec.seed)
        sim2.run(k)
        sim2.checkpoint(ck_plain)
        sim2.close()
    # plain -> batch slot (host seeds)
    with Batch(max_replicates=2, ring_steps=n + 1) as b3:
        s = b3.add(spec.capacity, spec.cc, stop_step=n)
        b3.set_inputs(s, T[:n], env[:n])
        b3.set_seeds(s, k, seeds[k:])
        b3.resume(s, ck_plain)
        b3.run(n - k)
        assert b3.rows(s, k, n - k + 1).tobytes() == want[k:].tobytes()


@pytest.mark.gpu
def test_checkpoint_with_broken_ranges_is_refused(gpu_ready, tmp_path):
    """A checkpoint whose ranges no step could have produced (here the egg
    range moved off slot 0, with the pool size left consistent) is refused
    before any column reaches the device."""
    import struct
    from sampo_gb300._lib import SampoError
    from sampo_gb300.sim import Simulation, seed_stream
    init, seeds = seed_stream(5, 48)
    T = np.full(48, 27.0, np.float32)
    from sampo_gb300 import inputs
    env = np.zeros(48, dtype=inputs.ENV_DTYPE)
    env["bloodmealSuccess"] = 0.25
    env["carryingCapacity"] = 5000.0
    sim = Simulation(capacity=1 << 16, carrying_capacity=5000.0, max_steps=49)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    sim.init_population(1000, init, 3, 5)
    sim.run(24)
    ck = str(tmp_path / "sim.ck")
    sim.checkpoint(ck)
    sim.close()
    raw = bytearray(open(ck, "rb").read())
    struct.pack_into("<I", raw, 20, 1)   # pop.r[0].start (after magic, version, step, cc)
    bad = str(tmp_path / "bad.ck")
    open(bad, "wb").write(bytes(raw))
    sim = Simulation(capacity=1 << 16, carrying_capacity=5000.0, max_steps=49)
    sim.set_inputs(T, env)
    sim.set_seeds(0, seeds)
    with pytest.raises(SampoError):
        sim.resume(bad)
    sim.resume(ck)             # the intact file still loads into the same handle
    assert sim.get_step() == 24
    sim.close()
