"""Build the CUDA library (libsampo_cuda.so) and the drop-in CLI for sm_103a.

Everything is compiled in-tree into sampo_gb300/_build/ with nvcc directly:
one -gencode (arch=compute_103a, code=sm_103a), FP contraction off on both
the device (--fmad=false) and the host (-ffp-contract=off) so float
expressions round exactly as written, IEEE division and square root.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libsampo_cuda.so")
CLI = os.path.join(OUT, "sampo")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-lineinfo", "-std=c++17",
                  "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", f"-I{os.path.join(REPO, 'include')}"]
SOURCES = ["sampo_kernels.cu", "sampo_api.cu", "sampo_batch.cu", "sampo_host.cpp", "sampo_noalloc.cu", "sampo_species.cu"]
# the device sources a user species is compiled with at run time, under the
# names their #include lines use (embedded as text by jit_sources())
JIT_HEADERS = [("sampo_step_kernels.cuh", "sampo_step_kernels.cuh"), ("sampo_kernels.cuh", "sampo_kernels.cuh"),
               ("sampo_model.cuh", "sampo_model.cuh"), ("sampo_species.cuh", "sampo_species.cuh"),
               ("sampo_species_prelude.h", "sampo_species_prelude.h"), ("sampo_math.h", "sampo_math.h"),
               ("sampo_math_fast.h", "sampo_math_fast.h"), ("sampo_fast_tables.h", "sampo_fast_tables.h"),
               ("../../include/sampo.h", os.path.join("..", "..", "include", "sampo.h"))]
JIT_SRC = os.path.join(OUT, "sampo_jit_sources.cpp")


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def jit_sources(force: bool = False) -> str:
    """Write sampo_jit_sources.cpp: the JIT_HEADERS as C++ raw string literals."""
    files = [os.path.normpath(os.path.join(CSRC, rel)) for _, rel in JIT_HEADERS]
    if not force and not _stale(JIT_SRC, files + [os.path.abspath(__file__)]):
        return JIT_SRC
    delim = "sampo_jit"
    lines = ["// generated by sampo_gb300/build.py: the step kernel sources for run-time compilation", "",
             'extern "C" const char* const sampo_jit_names[] = {']
    lines += [f'    "{name}",' for name, _ in JIT_HEADERS]
    lines += ["};", 'extern "C" const char* const sampo_jit_texts[] = {']
    for f in files:
        text = open(f).read()
        assert f")" + delim + '"' not in text
        lines.append(f'    R"{delim}(' + text + f'){delim}",')
    lines += ["};", f'extern "C" const int sampo_jit_count = {len(JIT_HEADERS)};', ""]
    with open(JIT_SRC, "w") as fh:
        fh.write("\n".join(lines))
    return JIT_SRC


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    jit = jit_sources(force)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "sampo.h"))
    objs, jobs = [], []
    for s in [os.path.join(CSRC, src) for src in SOURCES] + [jit]:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc()] + NVFLAGS + ["-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(len(jobs)) as ex:
            for log in ex.map(_run, jobs):
                if verbose and log.strip():
                    print(log)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


def build_cli(force: bool = False) -> str:
    src = os.path.join(PKG, "host", "sampo_main.c")
    if not os.path.exists(src):
        return ""
    lib = build_library()
    if force or _stale(CLI, [src, lib, os.path.join(REPO, "include", "sampo.h")]):
        _run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", f"-I{os.path.join(REPO, 'include')}", src,
              "-o", CLI, f"-L{OUT}", "-lsampo_cuda", f"-Wl,-rpath,{OUT}", "-lm", "-pthread"])
    return CLI


def build(force: bool = False, verbose: bool = False) -> None:
    build_library(force, verbose)
    build_cli(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
