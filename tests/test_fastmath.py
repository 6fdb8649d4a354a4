"""The binary32 fast paths of sampo_math_fast.h (the normal draw's log and
sin, the sporogonic-development add) against the binary64 definitions of
sampo_math.h, on the host. fastmath_check.c enumerates the log and sin
domains the model produces (every 4th input here; the full enumeration is
the same program with stride 1) and bit-compares every result."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "sampo_gb300", "csrc")


def test_fast_paths_equal_binary64_definitions(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    exe = str(tmp_path / "fastmath_check")
    cmd = [gcc, "-O2", "-ffp-contract=off", "-fopenmp", "-I", CSRC, os.path.join(HERE, "fastmath_check.c"), "-o", exe, "-lm"]
    subprocess.run(cmd, check=True)
    out = subprocess.run([exe, "4", "200000"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = {l.split()[0]: l for l in out.stdout.splitlines() if l.strip()}
    for fn in ("log", "sin", "sporo"):
        assert "mismatches=0" in lines[fn], lines[fn]
    # the pair's measured error stays below its bound with the margin the bound assumes
    for fn, bound in (("log", -38), ("sin", -36)):
        e = float(re.search(r"maxrel=2\^(-?[\d.]+)", lines[fn]).group(1))
        assert e <= bound - 2 + 1e-9, lines[fn]
