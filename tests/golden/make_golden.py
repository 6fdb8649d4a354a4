"""Generate the golden fixtures in this directory from the reference itself.

Builds ref-as-C (the reference's own src/abms.c, src/boltScan.c and
kernel/*.cl compiled for the host over the lib_icl emulator in
oracle/ref_build) and runs it on synthetic inputs. For every case it stores
the per-step stats lines exactly as the reference prints them
(src/abms.c:67-81), a position-dependent hash of the pool after every step,
the final ranges and histogram.txt (src/abms.c:176-180).

Needs the reference checkout ($SAMPO_REFERENCE, else a checkout named
"reference" beside this repository)
and only runs where that exists; the fixtures it writes are committed.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import gzip
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from sampo_gb300 import inputs  # noqa: E402
from tests.golden.cases import CASES, SPECIES_CASES, SPECIES_DIR, case_pool, make_case_inputs, write_ref_pool  # noqa: E402

from oracle.build import reference_dir  # noqa: E402

REF = reference_dir()


def build_ref(species: str | None = None) -> str:
    """ref-as-C; with a species header, the build that compiles it in place of properties.h."""
    cmd = ["make", "-s", "-C", os.path.join(REPO, "oracle", "ref_build"), f"REF={REF}"]
    if species is None:
        subprocess.run(cmd, check=True)
        return os.path.join(REPO, "oracle", "_ref", "sampo_ref")
    subprocess.run(cmd + ["species", f"SPECIES_HDR={os.path.join(SPECIES_DIR, species)}"], check=True)
    return os.path.join(REPO, "oracle", "_ref", "species_" + os.path.splitext(species)[0], "sampo_ref")


def run_case(exe: str, name: str) -> dict:
    c = CASES[name] if name in CASES else SPECIES_CASES[name]
    with tempfile.TemporaryDirectory() as td:
        tp, ep, meta = make_case_inputs(name, td)
        hf = os.path.join(td, "hash.txt")
        cmd = [exe, "--seed", str(c["seed"]), "--initial", str(c["initial"]), "--cc", repr(c["cc"]),
               "--steps", str(c["steps"]), "--hash-file", hf]
        if c.get("age_days", -1) >= 0:
            cmd += ["--age-days", str(c["age_days"]), "--age-seed", str(c["age_seed"])]
        if c.get("pool"):
            ranges, arrays = case_pool(name, inputs.read_temperature(tp, 1)[0])
            pf = os.path.join(td, "pool.bin")
            write_ref_pool(pf, ranges, arrays)
            cmd += ["--pool", pf]
            meta["pool_slots"] = int(ranges[7][1])
        cmd += [tp, ep]
        if c.get("species"):
            cmd.append(c["species"])
            meta["species_sha256"] = inputs.file_sha256(os.path.join(SPECIES_DIR, c["species"]))
        out = subprocess.run(cmd, cwd=td, check=True, capture_output=True).stdout.decode()
        lines = out.split("\n")
        trace = [ln for ln in lines if ln.endswith("\r") and ln.count(",") == 18]
        ranges = [ln for ln in lines if ln.startswith(("Eggs", "Larvae", "Pupae", "Immatures", "MateSeeking", "BMS", "BMD", "Gravids"))]
        hist = open(os.path.join(td, "histogram.txt")).read()
        hashes = open(hf).read().split()
    assert len(trace) == c["steps"], (name, len(trace))
    assert len(hashes) == c["steps"], (name, len(hashes))
    return {"case": name, "params": c, "inputs": meta, "trace": trace, "pool_hash": hashes,
            "final_ranges": ranges, "histogram_txt": hist,
            "generator": "ref-as-C: reference src/abms.c + kernel/*.cl over oracle/ref_build"}


def main(argv):
    names = argv or list(CASES) + list(SPECIES_CASES)
    for name in names:
        c = CASES[name] if name in CASES else SPECIES_CASES[name]
        data = run_case(build_ref(c.get("species")), name)
        path = os.path.join(HERE, f"{name}.json.gz")
        with gzip.open(path, "wt") as f:
            json.dump(data, f, separators=(",", ":"))
        print(f"{name}: {data['params']['steps']} steps -> {os.path.relpath(path, REPO)} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main(sys.argv[1:])
