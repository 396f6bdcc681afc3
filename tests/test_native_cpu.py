"""CPU tests of the product library that need no GPU: it loads and exports
every function include/sfmm.h declares, argument checks that precede any
CUDA call, the operator tables, and the C++ drop-in API (the reference's own
test and benchmark programs compile and link against include/solidfmm/ and
libsfmm_gb300.so)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference's own sources (test programs), where this machine has them
REF = os.environ.get("SFMM_REF_SRC", "/root/reference")


def _declared():
    txt = open(os.path.join(ROOT, "include", "sfmm.h")).read()
    return sorted(set(re.findall(r"\b(sfmm_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(native):
    L = native.load()
    names = _declared()
    assert len(names) >= 15
    for nm in names:
        assert hasattr(L, nm), nm


def test_drop_in_cxx_symbols_exported(native):
    path = native._native.lib_path()
    out = subprocess.run(["nm", "-DC", path], capture_output=True, text=True).stdout
    for sym in ("solidfmm::m2l(", "solidfmm::m2m(", "solidfmm::l2l(", "solidfmm::m2l_unchecked(",
                "solidfmm::multithreaded_translator<double>::m2l(", "solidfmm::harmonics::R<double>",
                "solidfmm::operator_handle<float>::operator_handle(", "solidfmm::dot(", "solidfmm::fmadd("):
        assert sym in out, sym


def test_create_argument_errors_without_gpu(native):
    L = native.load()
    h = C.c_void_p()
    assert L.sfmm_create(C.byref(h), 1, 0, 0) == 1          # P == 0: invalid
    assert L.sfmm_create(C.byref(h), 1, 87, 0) == 3         # above the FP64 limit: overflow
    assert L.sfmm_create(C.byref(h), 0, 29, 0) == 3         # above the FP32 limit: overflow
    assert L.sfmm_create(C.byref(h), 7, 10, 0) == 1         # unknown dtype
    assert L.sfmm_create(None, 1, 10, 0) == 1


def test_swap_tables_orthogonal_symmetric(native):
    from solidfmm_gb300._native import host_table

    for P in (16, 40):
        for n in (0, 3, 8, min(P - 1, 20)):
            d = n + 1
            WR = host_table(P, 0, n).reshape(d, d)
            WI = host_table(P, 1, n).reshape(d, d)
            assert np.abs(WR @ WR.T - np.eye(d)).max() < 1e-13
            assert np.abs(WR - WR.T).max() < 1e-13
            assert np.abs(WR @ WR - np.eye(d)).max() < 1e-13
            if d > 1:
                S = WI[1:, 1:]
                assert np.abs(S @ S.T - np.eye(d - 1)).max() < 1e-13
            assert np.abs(WR).max() <= 1 + 1e-12


def test_swap_tables_match_reference_combinations(native, oracle):
    """W_R = E Rf E^-1 with Rf the reference's real swap matrix
    (operator_data.cpp:99-122) and E_m = sqrt((n-m)!(n+m)!)/(sqrt 2 if m = 0)."""
    from math import factorial, sqrt

    from solidfmm_gb300._native import host_table

    n = 7
    d = n + 1
    B = lambda m, l: oracle.swap_B(n, m, l)  # noqa: E731
    Rf = np.zeros((d, d))
    for i in range(d):
        for j in range(d):
            if (i + j + n) % 2:
                continue
            Rf[i, j] = B(0, i) if j == 0 else (B(j, i) - B(-j, i) if j % 2 else B(j, i) + B(-j, i))
    E = np.array([sqrt(factorial(n - m) * factorial(n + m)) / (sqrt(2) if m == 0 else 1) for m in range(d)])
    W = host_table(16, 0, n).reshape(d, d)
    assert np.allclose(W, Rf * E[:, None] / E[None, :], rtol=1e-13, atol=1e-15)


def test_z_tables(native):
    from math import factorial, sqrt

    from solidfmm_gb300._native import host_table

    P, m = 12, 2
    L = P - m
    H = host_table(P, 3, m).reshape(L, L)  # M2L
    D = lambda n: sqrt(factorial(n - m) * factorial(n + m))  # noqa: E731
    for a in range(L):
        for k in range(L):
            n, kk = a + m, k + m
            ref = (-1) ** (n + m) * factorial(n + kk) / (D(n) * D(kk))
            assert abs(H[a, k] - ref) <= 1e-13 * abs(ref)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "tests")), reason="reference sources not present")
@pytest.mark.parametrize("prog", ["test_m2l", "test_m2m", "test_l2l", "benchmark_m2l", "benchmark_m2m",
                                  "benchmark_l2l", "benchmark_multithreaded_translator"])
def test_reference_programs_compile_against_drop_in(native, prog, tmp_path):
    lib = os.path.dirname(native._native.lib_path())
    exe = tmp_path / prog
    r = subprocess.run(["g++", "-std=c++20", "-O0", "-I", os.path.join(ROOT, "include"),
                        os.path.join(REF, "tests", prog + ".cpp"), "-o", str(exe), "-L", lib, "-lsfmm_gb300",
                        f"-Wl,-rpath,{lib}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    assert exe.exists()


def test_drop_in_harmonics_match_reference_goldens(native, tmp_path):
    """solidfmm::harmonics::R/S/dR/dS of the drop-in library against the
    reference's own values at the golden points (solidfmm/harmonics.cpp:32-349,
    generated by tests/golden/make_golden.py)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "translations.npz"))
    pts = g["harmonics/points"]
    want = {k: g[f"harmonics/{k}"] for k in ("R", "S", "dR", "dS")}
    S = want["R"].shape[1]
    P = int(round((-1 + (1 + 4 * S) ** 0.5) / 2))
    assert P * (P + 1) == S
    lib = os.path.dirname(native._native.lib_path())
    exe = tmp_path / "harmonics_check"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cxx", "harmonics_check.cpp"), "-o", str(exe), "-L", lib,
                        "-lsfmm_gb300", f"-Wl,-rpath,{lib}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    args = [str(exe), str(P)] + [repr(float(v)) for v in pts.reshape(-1)]
    out = np.frombuffer(subprocess.run(args, capture_output=True, check=True).stdout, dtype=np.float64)
    per = 8 * S
    assert out.size == per * len(pts)
    for i in range(len(pts)):
        row = out[i * per:(i + 1) * per]
        got = {"R": row[:S], "S": row[S:2 * S], "dR": row[2 * S:5 * S], "dS": row[5 * S:]}
        for k in got:
            ref = want[k][i]
            err = np.abs(got[k] - ref).max() / np.abs(ref).max()
            assert err < 1e-13, (k, i, err)
