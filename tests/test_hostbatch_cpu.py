"""CPU tests of the library's host-only C++ (built with the host compiler
alone, no CUDA): the classic call's parallel bookkeeping
(sfmm_hostbatch.cpp) against a sequential restatement — rising,
sorted-with-runs and unordered target addresses, one and three components,
FP64 and FP32 shifts, 1, 3 and 8 threads, the first-invalid-translation
report — and the operator tables (sfmm_tables.cpp): orthogonal involutions,
the 8-row padded copy of contexts above order 32, table bounds.  Each also
runs under AddressSanitizer + UndefinedBehaviorSanitizer, and the threaded
bookkeeping under ThreadSanitizer, where the compiler provides them."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "solidfmm_gb300", "csrc")
CASES = {
    "hostbatch": (os.path.join(ROOT, "tests", "cxx", "hostbatch_check.cpp"), os.path.join(CSRC, "sfmm_hostbatch.cpp")),
    "tables": (os.path.join(ROOT, "tests", "cxx", "tables_check.cpp"), os.path.join(CSRC, "sfmm_tables.cpp")),
}
SANITIZERS = {"plain": [], "asan_ubsan": ["-fsanitize=address,undefined", "-fno-sanitize-recover=all"],
              "tsan": ["-fsanitize=thread"]}


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    return cxx


def _sanitizer_available(cxx, flags, tmp_path):
    if not flags:
        return True
    src = tmp_path / "probe.cpp"
    src.write_text("int main() { return 0; }\n")
    r = subprocess.run([cxx] + flags + [str(src), "-o", str(tmp_path / "probe")], capture_output=True)
    return r.returncode == 0 and subprocess.run([str(tmp_path / "probe")], capture_output=True).returncode == 0


@pytest.mark.parametrize("san", ["plain", "asan_ubsan", "tsan"])
@pytest.mark.parametrize("case", ["hostbatch", "tables"])
def test_host_code(tmp_path, case, san):
    if case == "tables" and san == "tsan":
        pytest.skip("the table builder is single-threaded")
    cxx = _cxx()
    flags = SANITIZERS[san]
    if not _sanitizer_available(cxx, flags, tmp_path):
        pytest.skip(f"{san} not available with {cxx}")
    exe = tmp_path / case
    opt = ["-O2"] if san == "plain" else ["-O1", "-g"]
    subprocess.run([cxx, "-std=c++17", "-pthread", "-I", CSRC] + opt + flags + list(CASES[case]) + ["-o", str(exe)],
                   check=True)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1",
               TSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-3000:] + r.stderr[-3000:]
