"""The CPU oracle against the golden traces made by the reference's own code
(ref-as-C, tests/golden/make_golden.py): every stats line, the pool hash
after every step, the final ranges and histogram.txt must be identical."""
import subprocess

import numpy as np

import pytest

from tests.conftest import load_golden
from tests.golden.cases import CASES, make_case_inputs

# (case, steps): None = the whole case; a number = that prefix (CPU budget)
RUNS = [("small_a", None), ("small_b", None), ("interventions", None), ("reference_default", 600),
        ("eggs_1e4_year", 1000), ("temperature_edges", None)]


@pytest.mark.parametrize("name,steps", RUNS)
def test_oracle_matches_reference_trace(oracle_mod, tmp_path, name, steps):
    g = load_golden(name)
    c = CASES[name]
    n = steps or c["steps"]
    tp, ep, meta = make_case_inputs(name, str(tmp_path))
    assert meta == g["inputs"], "regenerated inputs differ from the ones the fixture was made from"
    hf = tmp_path / "hash.txt"
    cmd = [oracle_mod.CLI, "--seed", str(c["seed"]), "--initial", str(c["initial"]), "--cc", repr(c["cc"]),
           "--steps", str(n), "--hash-file", str(hf)]
    if c["age_days"] >= 0:
        cmd += ["--age-days", str(c["age_days"]), "--age-seed", str(c["age_seed"])]
    out = subprocess.run(cmd + [tp, ep], cwd=tmp_path, check=True, capture_output=True).stdout.decode()
    lines = out.split("\n")
    trace = [ln for ln in lines if ln.endswith("\r") and ln.count(",") == 18]
    assert len(trace) == n
    for i, (a, b) in enumerate(zip(trace, g["trace"][:n])):
        assert a == b, f"step {i}: oracle {a!r} != reference {b!r}"
    hashes = hf.read_text().split()
    assert hashes == g["pool_hash"][:n]
    if n == c["steps"]:
        ranges = [ln for ln in lines if ln.startswith(("Eggs", "Larvae", "Pupae", "Immatures", "MateSeeking", "BMS", "BMD", "Gravids"))]
        assert ranges == g["final_ranges"]
        assert (tmp_path / "histogram.txt").read_text() == g["histogram_txt"]


def test_oracle_thread_count_invariant(oracle_mod, tmp_path):
    """Integer reductions make the result independent of the thread count."""
    c = CASES["small_b"]
    tp, ep, _ = make_case_inputs("small_b", str(tmp_path))
    outs = []
    for t in (1, 3):
        hf = tmp_path / f"h{t}.txt"
        subprocess.run([oracle_mod.CLI, "--seed", str(c["seed"]), "--initial", str(c["initial"]), "--cc", repr(c["cc"]),
                        "--steps", "400", "--age-days", "2", "--age-seed", "4", "--threads", str(t),
                        "--hash-file", str(hf), tp, ep], cwd=tmp_path, check=True, capture_output=True)
        outs.append(hf.read_text())
    assert outs[0] == outs[1]


def test_golden_fixtures_are_complete():
    for name, c in CASES.items():
        g = load_golden(name)
        assert len(g["trace"]) == c["steps"] == len(g["pool_hash"])
        assert g["histogram_txt"].count(",") == 100
        assert len(g["final_ranges"]) == 8


def test_oracle_matches_reference_from_mixed_stage_pool(oracle_mod, tmp_path):
    """A mixed-stage start (all eight states populated) loaded into the
    oracle against the reference's own code started from the same pool
    (ref-as-C's --pool): every stats line and the pool hash after every step."""
    from oracle import OracleSim
    from sampo_gb300 import inputs
    from sampo_gb300.sim import seed_stream, stats_lines
    from tests.golden.cases import case_pool
    name = "mixed_pool"
    g = load_golden(name)
    c = CASES[name]
    n = c["steps"]
    tp, ep, meta = make_case_inputs(name, str(tmp_path))
    T = inputs.read_temperature(tp, n)
    env = inputs.read_environment(ep, n, c["cc"])
    ranges, arrays = case_pool(name, T[0])
    assert {k: v for k, v in g["inputs"].items() if k != "pool_slots"} == meta
    assert g["inputs"]["pool_slots"] == int(ranges[7][1])
    _, seeds = seed_stream(c["seed"], n)
    o = OracleSim(1 << 18)
    o.load_pool(ranges, arrays)
    rows = []
    for i in range(n):
        rows.append(o.step(env[i], T[i], i % 24, seeds[i]))
        assert format(o.pool_hash(), "016x") == g["pool_hash"][i], f"pool after step {i}"
    lines = stats_lines(np.array(rows), T, ranges)
    for i, (a, b) in enumerate(zip(lines, g["trace"])):
        assert a == b, f"step {i}: oracle {a!r} != reference {b!r}"
    o.close()
