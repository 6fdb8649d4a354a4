"""Species headers compiled at run time (sampo_species_*, the `sampo`
command's third argument). The reference compiles its kernels with the
header named by argv[3] (src/abms.c:565-568); with the test header
tests/golden/species/hot_species.h, which changes every species hook, the
sampo command must print what the reference's own kernels compiled against
that header print (tests/golden/hot_species.json.gz, from ref-as-C)."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import load_golden
from tests.golden.cases import SPECIES_CASES, SPECIES_DIR, make_case_inputs

HOT = os.path.join(SPECIES_DIR, "hot_species.h")


def _hot_text():
    with open(HOT) as f:
        return f.read()


def test_species_header_compiles_without_gpu(sampo_lib):
    """The step kernels compile against the test header (NVRTC only, no device)."""
    from sampo_gb300.species import Species
    rc, log = Species.check(_hot_text())
    assert rc == 0, log


def test_species_errors_without_gpu(sampo_lib):
    """A header that does not compile, or lacks a function the kernels call,
    is refused with the compiler's message."""
    from sampo_gb300.species import Species
    rc, log = Species.check(_hot_text().replace("return 52.5f - 0.75f * temperature;", "return 52.5f - ;"))
    assert rc == -8 and "error" in log
    text = _hot_text()
    cut = text.index("INT layEggs(")
    rc, log = Species.check(text[:cut])
    assert rc == -8 and "layEggs" in log


def test_cli_species_errors_without_gpu(sampo_lib, tmp_path):
    from sampo_gb300 import build
    cli = build.build_cli()
    (tmp_path / "t.txt").write_text("25\n25\n")
    (tmp_path / "e.txt").write_text("0, 0, 0, 0, 0, 0, 0, 0, 0.25\n" * 2)
    out = subprocess.run([cli, "--steps", "2", "t.txt", "e.txt", "otherSpecies.h"], capture_output=True, text=True,
                         cwd=tmp_path)
    assert out.returncode == 2 and "did not build" in out.stderr and "cannot open otherSpecies.h" in out.stderr


@pytest.mark.gpu
def test_cli_species_matches_reference(gpu_ready, tmp_path):
    """The sampo command with the test header against the reference's kernels
    compiled with it: every stats line, the final ranges and histogram.txt."""
    from sampo_gb300 import build
    cli = build.build_cli()
    name = "hot_species"
    c = SPECIES_CASES[name]
    g = load_golden(name)
    tp, ep, _ = make_case_inputs(name, str(tmp_path))
    shutil.copy(HOT, tmp_path / c["species"])
    cmd = [cli, "--seed", str(c["seed"]), "--initial", str(c["initial"]), "--cc", repr(c["cc"]),
           "--steps", str(c["steps"]), "--age-days", str(c["age_days"]), "--age-seed", str(c["age_seed"]),
           tp, ep, c["species"]]
    out = subprocess.run(cmd, capture_output=True, cwd=tmp_path, timeout=900)
    assert out.returncode == 0, out.stderr.decode()
    lines = out.stdout.decode().split("\n")
    assert lines[:3] == [f"Temperature:\t{tp}", f"Environment:\t{ep}", f"Species:\t{c['species']}"]
    n = c["steps"]
    trace = lines[3:3 + n]
    for i, (a, b) in enumerate(zip(trace, g["trace"])):
        assert a == b, f"step {i}: sampo {a!r} != reference {b!r}"
    assert len(trace) == len(g["trace"])
    assert lines[3 + n:3 + n + 8] == g["final_ranges"]
    with open(tmp_path / "histogram.txt") as f:
        assert f.read() == g["histogram_txt"]


@pytest.mark.gpu
def test_species_batch_equals_plain_runs(gpu_ready):
    """A batch compiled with the test header: each replicate equals its plain
    run with the same header, and differs from the built-in species."""
    from sampo_gb300.batch import Batch, ReplicateSpec, admit
    from sampo_gb300.sim import Simulation, seed_stream
    from sampo_gb300.species import Species
    specs = [ReplicateSpec(initial=800, seed=31, mean_t=27.0, amplitude=3.0, rain_mean=4.0, days=4, capacity=60000),
             ReplicateSpec(initial=5000, seed=32, mean_t=24.0, amplitude=6.0, rain_mean=2.0, days=4, capacity=200000)]
    steps = 96
    with Species(HOT) as sp:
        assert sp.log is not None

        def plain(spec, species):
            T, env = spec.inputs()
            init, seeds = seed_stream(spec.seed, steps)
            with Simulation(capacity=spec.capacity, carrying_capacity=spec.cc, max_steps=steps + 1) as sim:
                sim.set_species(species)
                sim.set_inputs(T[:steps], env[:steps])
                sim.set_seeds(0, seeds)
                sim.init_population(spec.initial, init, age_days_max=spec.age_days_max, age_seed=spec.seed)
                return sim.run(steps)

        with Batch(max_replicates=4, ring_steps=steps + 1) as b:
            b.set_species(sp)
            slots = [admit(b, s, steps, device_seeds=True) for s in specs]
            b.run(steps)
            for slot, spec in zip(slots, specs):
                want = plain(spec, sp)
                got = b.rows(slot, 0, steps)
                assert got.tobytes() == want.tobytes(), f"replicate {spec.seed}"
                assert b.state(slot)[2] & 0xFF == 0
        builtin = plain(specs[0], None)
        assert builtin.tobytes() != plain(specs[0], sp).tobytes()
