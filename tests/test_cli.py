"""The sampo command (sampo_gb300/host/sampo_main.c): the reference's CLI and
output files on the GB300 library. Its stdout (stats line per step, final
ranges) and histogram.txt must equal the reference's own run for the same
inputs and seed, in both host-loop modes."""
import os
import subprocess

import pytest

from tests.conftest import load_golden
from tests.golden.cases import CASES, make_case_inputs


@pytest.fixture(scope="module")
def cli(sampo_lib):
    from sampo_gb300 import build
    path = build.build_cli()
    assert path and os.path.exists(path)
    return path


def test_cli_arguments_without_gpu(cli, tmp_path):
    out = subprocess.run([cli, "-h"], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("Usage: bin\\abms")
    out = subprocess.run([cli, str(tmp_path / "missing.txt")], capture_output=True, text=True, cwd=tmp_path)
    assert out.stdout.splitlines()[:4] == [f"Temperature:\t{tmp_path / 'missing.txt'}", "Environment:\tenvironment.txt",
                                           "Species:\tproperties.h",
                                           f"Cannot open {tmp_path / 'missing.txt'}. Check temperature file path"]
    out = subprocess.run([cli, "t.txt", "e.txt", "otherSpecies.h"], capture_output=True, text=True, cwd=tmp_path)
    assert out.stdout.splitlines()[3] == "Cannot open t.txt. Check temperature file path"


@pytest.mark.gpu
@pytest.mark.parametrize("name,per_step", [("eggs_1e4_year", False), ("interventions", True), ("reference_default", False)])
def test_cli_output_matches_reference(gpu_ready, cli, tmp_path, name, per_step):
    c = CASES[name]
    g = load_golden(name)
    tp, ep, _ = make_case_inputs(name, str(tmp_path))
    cmd = [cli, "--seed", str(c["seed"]), "--initial", str(c["initial"]), "--cc", repr(c["cc"]),
           "--steps", str(c["steps"]), "--age-days", str(c["age_days"]), "--age-seed", str(c["age_seed"])]
    if per_step:
        cmd.append("--per-step")
    # bytes: the reference's lines end in \r\n, which text mode would translate
    out = subprocess.run(cmd + [tp, ep], capture_output=True, cwd=tmp_path, timeout=600)
    assert out.returncode == 0, out.stderr.decode()
    lines = out.stdout.decode().split("\n")
    assert lines[:3] == [f"Temperature:\t{tp}", f"Environment:\t{ep}", "Species:\tproperties.h"]
    n = c["steps"]
    trace = lines[3:3 + n]
    for i, (a, b) in enumerate(zip(trace, g["trace"])):
        assert a == b, f"step {i}: sampo {a!r} != reference {b!r}"
    assert len(trace) == len(g["trace"])
    assert lines[3 + n:3 + n + 8] == g["final_ranges"]
    assert lines[3 + n + 8].startswith("Execution time: ")
    with open(tmp_path / "histogram.txt") as f:
        assert f.read() == g["histogram_txt"]
