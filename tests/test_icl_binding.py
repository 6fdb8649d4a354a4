"""The reference's own host program, src/abms.c, unmodified, over this
library's lib_icl binding (sampo_gb300/host/icl_sampo.cpp): built from the
reference checkout where one exists (skipped elsewhere).

* With the C ABI implemented on the CPU oracle (oracle/ref_build target
  shim-oracle), its stdout and histogram.txt equal the reference's own
  golden runs byte for byte: the binding's protocol (which abms.c calls map
  to which steps, what the host reads back) is exact.
* Against libsampo_cuda.so (sampo_gb300/host/icl_sampo.mk) it compiles and
  links; that binary runs on the GPU (the same ABI calls the GPU tests check
  against the same oracle)."""
import os
import subprocess

import pytest

from tests.conftest import REPO, load_golden
from tests.golden.cases import CASES, make_case_inputs


@pytest.fixture(scope="module")
def reference():
    from oracle.build import reference_dir
    ref = reference_dir()
    if not os.path.exists(os.path.join(ref, "src", "abms.c")):
        pytest.skip("no reference checkout here")
    return ref


@pytest.fixture(scope="module")
def abms_on_oracle(reference):
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref_build"), f"REF={reference}", "shim-oracle"],
                   check=True)
    return os.path.join(REPO, "oracle", "_ref", "abms_icl_sampo_oracle")


@pytest.mark.parametrize("name", ["reference_default", "interventions", "small_b"])
def test_unmodified_abms_over_binding_matches_reference(abms_on_oracle, tmp_path, name):
    c = CASES[name]
    g = load_golden(name)
    tp, ep, _ = make_case_inputs(name, str(tmp_path))
    cmd = [abms_on_oracle, "--seed", str(c["seed"]), "--initial", str(c["initial"]), "--cc", repr(c["cc"]),
           "--steps", str(c["steps"])]
    if c["age_days"] >= 0:
        cmd += ["--age-days", str(c["age_days"]), "--age-seed", str(c["age_seed"])]
    out = subprocess.run(cmd + [tp, ep], capture_output=True, cwd=tmp_path, timeout=600)
    assert out.returncode == 0, out.stderr.decode()
    lines = out.stdout.decode().split("\n")
    assert lines[:3] == [f"Temperature:\t{tp}", f"Environment:\t{ep}", "Species:\tproperties.h"]
    assert lines[3].startswith("GPU: libsampo_cuda")  # the device line (icl_print_device_short_info)
    n = c["steps"]
    trace = lines[4:4 + n]
    for i, (a, b) in enumerate(zip(trace, g["trace"])):
        assert a == b, f"step {i}: {a!r} != reference {b!r}"
    assert len(trace) == len(g["trace"])
    assert lines[4 + n:4 + n + 8] == g["final_ranges"]
    assert lines[4 + n + 8].startswith("Execution time: ")
    with open(tmp_path / "histogram.txt") as f:
        assert f.read() == g["histogram_txt"]


def test_unmodified_abms_links_against_the_gpu_library(reference, sampo_lib, tmp_path):
    from sampo_gb300 import build
    build.build_library()
    out_dir = tmp_path / "icl"
    subprocess.run(["make", "-s", "-f", os.path.join(REPO, "sampo_gb300", "host", "icl_sampo.mk"),
                    f"SAMPO={reference}", f"OUT={out_dir}"], check=True)
    exe = out_dir / "abms_gb300"
    assert exe.exists()
    # abms.c answers -h before it touches a device (src/abms.c:558-562)
    out = subprocess.run([str(exe), "-h"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.startswith("Usage: bin\\abms")
