"""Build the CPU oracle (TEST INFRASTRUCTURE ONLY).

  oracle/_build/liboracle.so   the C restatement, for ctypes (tests, bench)
  oracle/_build/sampo_oracle   its command-line driver (abms.c's I/O)
  oracle/_ref/sampo_ref        ref-as-C, only where the reference checkout
                               exists ($SAMPO_REFERENCE, else a checkout
                               named "reference" beside this repository);
                               built by ref_build/Makefile
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
CLI = os.path.join(OUT, "sampo_oracle")
REF_EXE = os.path.join(HERE, "_ref", "sampo_ref")
FLAGS = ["-O2", "-std=gnu11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-Wall", "-Wno-unused-result"]
DEPS = [os.path.join(HERE, f) for f in ("sampo_oracle.c", "sampo_oracle.h", "sampo_oracle_main.c")] + \
       [os.path.join(os.path.dirname(HERE), "sampo_gb300", "csrc", "sampo_math.h")]


def _stale(target):
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in DEPS)


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "sampo_oracle.c")
    if force or _stale(LIB):
        subprocess.run(["gcc"] + FLAGS + ["-shared", src, "-o", LIB, "-lm"], check=True)
    if force or _stale(CLI):
        subprocess.run(["gcc"] + FLAGS + [src, os.path.join(HERE, "sampo_oracle_main.c"), "-o", CLI, "-lm"], check=True)
    return LIB


def reference_dir() -> str:
    """The reference checkout: $SAMPO_REFERENCE, else a directory named
    "reference" beside this repository."""
    return os.environ.get("SAMPO_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build_ref() -> str | None:
    ref = reference_dir()
    if not os.path.isdir(os.path.join(ref, "kernel")):
        return None
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref_build"), f"REF={ref}"], check=True)
    return REF_EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_ref())
