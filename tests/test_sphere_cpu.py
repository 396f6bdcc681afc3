"""Minimal bounding spheres (sfmm_bounding_sphere and the drop-in
solidfmm::bounding_sphere): against the reference's own implementation where
it was compiled here, against an independent convex solve, containment,
degenerate inputs and errors.  Host code only."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.fixture(scope="module")
def bs(native):
    from solidfmm_gb300._native import bounding_sphere

    return bounding_sphere


def _cases(seed, count):
    rng = np.random.default_rng(seed)
    for t in range(count):
        n = int(rng.integers(1, 120))
        p = rng.normal(size=(n, 3)) * 10 ** rng.uniform(-3, 3) + rng.normal(size=3) * 5
        r = rng.random(n) * np.abs(p).max() * 0.2 if t % 2 else None
        yield p, r


def _contained(s, p, r):
    d = np.linalg.norm(p - s[:3], axis=1) + (0 if r is None else r)
    return np.all(d <= s[3] * (1 + 1e-12) + 1e-300)


def test_matches_reference_implementation(bs, oracle):
    if not oracle.ref_available():
        pytest.skip("the reference library is built only where its sources are present")
    L = oracle.ref()
    for p, r in _cases(3, 200):
        ref = np.zeros(4)
        rr = None if r is None else np.ascontiguousarray(r)
        assert L.ref_bounding_sphere_d(len(p), p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy(),
                                       None if rr is None else rr.ctypes.data, ref) == 0
        got = bs(p[:, 0], p[:, 1], p[:, 2], r)
        scale = ref[3] + 1e-300
        assert abs(got[3] - ref[3]) <= 1e-10 * scale and np.linalg.norm(got[:3] - ref[:3]) <= 1e-10 * scale


def test_minimal_against_convex_solve(bs):
    opt = pytest.importorskip("scipy.optimize")
    for p, r in _cases(5, 40):
        if len(p) < 2:
            continue
        rr = np.zeros(len(p)) if r is None else r
        s = bs(p[:, 0], p[:, 1], p[:, 2], r)
        assert _contained(s, p, r)
        # minimise R subject to |c - c_i| + r_i <= R, from a perturbed start
        x0 = np.concatenate([s[:3] + 0.1 * s[3], [1.5 * s[3]]])
        cons = {"type": "ineq", "fun": lambda v: v[3] - np.linalg.norm(p - v[:3], axis=1) - rr}
        res = opt.minimize(lambda v: v[3], x0, constraints=[cons], method="SLSQP",
                           options={"ftol": 1e-14, "maxiter": 500})
        assert s[3] <= res.x[3] * (1 + 1e-7)


def test_small_and_degenerate_sets(bs):
    s = bs([1.0], [2.0], [3.0])
    assert np.allclose(s, [1, 2, 3, 0])
    s = bs([0.0, 2.0], [0.0, 0.0], [0.0, 0.0])
    assert np.allclose(s, [1, 0, 0, 1])
    # duplicates and collinear points
    x = np.array([0.0, 1.0, 1.0, 2.0, 2.0, 0.5])
    s = bs(x, 2 * x, -x)
    assert np.allclose(s[:3], [1, 2, -1]) and np.isclose(s[3], np.sqrt(6))
    # coplanar square: the circumscribed circle
    s = bs([1.0, -1.0, -1.0, 1.0], [1.0, 1.0, -1.0, -1.0], [0.0] * 4)
    assert np.allclose(s, [0, 0, 0, np.sqrt(2)])
    # nested balls: the big one is the answer
    s = bs([0.0, 0.5, -0.3], [0.0, 0.2, 0.1], [0.0, 0.0, 0.4], [3.0, 1.0, 0.5])
    assert np.allclose(s, [0, 0, 0, 3])


def test_errors(native):
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        native._native.bounding_sphere([], [], [])


def test_dropin_sphere_program(native, tmp_path):
    lib = os.path.dirname(native._native.lib_path())
    src = tmp_path / "sphere_check.cpp"
    src.write_text(r'''
#include <solidfmm/sphere.hpp>
#include <cmath>
#include <cstdio>
#include <stdexcept>
using namespace solidfmm;
int main()
{
    const double x[4] = {1, -1, 0, 0}, y[4] = {0, 0, 1, -1}, z[4] = {0, 0, 0, 0};
    sphere<double> s = bounding_sphere(4, x, y, z);
    if (std::fabs(s.r - 1) > 1e-12 || std::fabs(s.x) > 1e-12) return 1;
    const float xf[2] = {0, 2}, yf[2] = {0, 0}, zf[2] = {0, 0};
    sphere<float> f = bounding_sphere(2, xf, yf, zf);
    if (std::fabs(f.r - 1) > 1e-6f || std::fabs(f.x - 1) > 1e-6f) return 2;
    sphere<double> balls[2] = {{0, 0, 0, 1}, {3, 0, 0, 1}};
    sphere<double> b = bounding_sphere(balls, balls + 2);
    if (std::fabs(b.r - 2.5) > 1e-12 || std::fabs(b.x - 1.5) > 1e-12) return 3;
    try {
        bounding_sphere(balls, balls);
        return 4;
    } catch (const std::logic_error &) {
    }
    std::puts("ok");
    return 0;
}
''')
    exe = tmp_path / "sphere_check"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", lib, "-lsfmm_gb300", f"-Wl,-rpath,{lib}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "ok" in r.stdout, (r.returncode, r.stdout, r.stderr)
