"""CPU test of the classic host call's bookkeeping (sfmm_hostbatch.cpp): the
parallel entry and slot construction against a sequential restatement, for
rising, sorted-with-runs and unordered target addresses, one and three
components, FP64 and FP32 shifts, 1, 3 and 8 threads, and the first-invalid-
translation report.  Built with the host compiler alone (no CUDA)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "solidfmm_gb300", "csrc")


def test_classic_bookkeeping_matches_sequential(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "hostbatch_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", CSRC,
                    os.path.join(ROOT, "tests", "cxx", "hostbatch_check.cpp"),
                    os.path.join(CSRC, "sfmm_hostbatch.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
