"""CPU tests of the oracle (test infrastructure) against the reference's
golden vectors: Dehnen's swap matrices, the solid harmonics, and every
golden translation case (the naive O(P^4) formulas and the rotation-based
restatement)."""
import numpy as np
import pytest

from helpers import S_of, load_golden, rel_err

CASES = load_golden()


def _golden_raw():
    return np.load(__import__("helpers").GOLDEN)


def test_swap_matrix_known_answer(oracle):
    z = _golden_raw()
    for n in range(7):
        B = z[f"swapB/{n}"]
        ours = np.array([[oracle.swap_B(n, m, l) for l in range(-n, n + 1)] for m in range(-n, n + 1)])
        assert np.array_equal(ours, B), n
    # Dehnen's B_4 entries are integers over 2^4 (swap_matrix.cpp:149-171; tests/test_swap_matrix.cpp)
    B4 = z["swapB/4"] * 16
    assert np.array_equal(B4, np.round(B4))
    assert B4[0, 0] == 1 and B4[4, 4] == 6 and B4[0, 4] == 70


def test_swap_matrix_dyadic_and_orthogonal_scaled(oracle):
    # B_n 2^n is integral and D^-1 B D is orthogonal (D_m = sqrt((n-m)!(n+m)!))
    from math import factorial, sqrt

    for n in (5, 9, 14):
        B = np.array([[oracle.swap_B(n, m, l) for l in range(-n, n + 1)] for m in range(-n, n + 1)])
        assert np.allclose(B * 2 ** n, np.round(B * 2 ** n), atol=0, rtol=0)
        D = np.array([sqrt(factorial(n - abs(k)) * factorial(n + abs(k))) for k in range(-n, n + 1)])
        W = B * D[None, :] / D[:, None]
        assert np.abs(W @ W.T - np.eye(2 * n + 1)).max() < 1e-12


@pytest.mark.parametrize("which", ["R", "S"])
def test_harmonics_vs_golden(oracle, which):
    z = _golden_raw()
    pts = z["harmonics/points"]
    for row, (x, y, zz) in zip(z[f"harmonics/{which}"], pts):
        h = oracle.harmonic(which, 12, x, y, zz)
        assert np.allclose(h, row, rtol=1e-14, atol=1e-300), (which, x, y, zz)


def _cases(tag):
    return sorted(k for k in CASES if f"_{tag}_" in k)


@pytest.mark.parametrize("name", _cases("f64"))
def test_naive_oracle_vs_reference(oracle, name):
    c = CASES[name]
    got = c["dst0"].copy()
    oracle.naive(str(c["op"]), c["src"], c["Pin"], got, c["Pout"], c["xyz"], sidx=c["sidx"], tidx=c["tidx"])
    err = rel_err(got - c["dst0"], c["dst"] - c["dst0"])
    assert err < 1e-10, f"{name}: {err:.3e}"


@pytest.mark.parametrize("name", _cases("f64") + _cases("f32"))
def test_rotation_port_vs_reference(oracle, name):
    c = CASES[name]
    got = c["dst0"].copy()
    oracle.rot(str(c["op"]), c["src"], c["Pin"], got, c["Pout"], c["xyz"], sidx=c["sidx"], tidx=c["tidx"])
    tol = 1e-12 if got.dtype == np.float64 else 1e-5
    err = rel_err(got - c["dst0"], c["dst"] - c["dst0"])
    assert err < tol, f"{name}: {err:.3e}"


@pytest.mark.parametrize("op", ["m2m", "m2l", "l2l"])
def test_rotation_port_vs_formula_mixed_orders(oracle, op):
    """Both directions of mixed orders, including L2L with P_in > P_out,
    where the reference itself reads uncomputed rows (translations.cpp:412-419)."""
    import inputs

    rng = np.random.default_rng(5)
    b = inputs.make_batch(rng, op, (1, 14), (1, 14), 40, nq=12)
    a = b["dst"].copy()
    oracle.naive(op, b["src"], b["Pin"], a, b["Pout"], b["xyz"])
    r = b["dst"].copy()
    oracle.rot(op, b["src"], b["Pin"], r, b["Pout"], b["xyz"], nthreads=3)
    assert rel_err(r - b["dst"], a - b["dst"]) < 1e-10


@pytest.mark.parametrize("op", ["m2m", "m2l", "l2l"])
def test_translations_are_homogeneous_in_length(oracle, op):
    """Scaling every length by a power of two lambda scales multipole degree
    n by lambda^n and local degree n by lambda^-(n+1), exactly: translating
    the scaled sources by the scaled shift and scaling the result back gives
    the unit-scale result.  The FP32-range kernels run every translation at
    the length scale of its shift on this property."""
    import inputs

    rng = np.random.default_rng(7)
    P = 12
    b = inputs.make_batch(rng, op, P, P, 30, nq=8)
    deg = np.array([k for k in range(P) for _ in range(2 * k + 2)], dtype=np.float64)
    src_kind_m = op != "l2l"
    out_kind_m = op == "m2m"
    ref = np.zeros_like(b["dst"])
    oracle.naive(op, b["src"], b["Pin"], ref, b["Pout"], b["xyz"])
    for k in (-24, -3, 5, 24):  # the FP64 oracle's r^(n+k+1) stays in range
        lam = 2.0 ** k
        src = b["src"] * (lam ** deg if src_kind_m else lam ** -(deg + 1))
        got = np.zeros_like(ref)
        oracle.naive(op, src, b["Pin"], got, b["Pout"], b["xyz"] * lam)
        got = got * (lam ** -deg if out_kind_m else lam ** (deg + 1))
        assert rel_err(got, ref) < 1e-13, (op, k)


def test_threaded_port_equals_serial(oracle):
    import inputs

    rng = np.random.default_rng(6)
    b = inputs.make_batch(rng, "m2l", 8, 8, 60, nq=8, pattern="repeat")
    r1 = b["dst"].copy()
    r4 = b["dst"].copy()
    oracle.rot("m2l", b["src"], b["Pin"], r1, b["Pout"], b["xyz"], sidx=b["sidx"], tidx=b["tidx"], nthreads=1)
    oracle.rot("m2l", b["src"], b["Pin"], r4, b["Pout"], b["xyz"], sidx=b["sidx"], tidx=b["tidx"], nthreads=4)
    assert rel_err(r4, r1) < 1e-14


def test_p2m_then_evaluate_matches_coulomb(oracle):
    """fmadd(q, R(x-c)) then dot with S reproduces sum q/|x-y| (doc/solidfmm.tex:546-561)."""
    rng = np.random.default_rng(2)
    P = 16
    pos = rng.uniform(-0.4, 0.4, (1, 20, 3))
    q = rng.choice([-1.0, 1.0], (1, 20))
    M = oracle.p2m(P, q, pos, np.zeros((1, 3)))[0]
    x = np.array([2.0, -1.5, 1.0])
    Sx = oracle.harmonic("S", P, *x)
    phi = oracle.dot(M, P, Sx, P)
    exact = sum(qq / np.linalg.norm(x - p) for qq, p in zip(q[0], pos[0]))
    assert abs(phi - exact) / abs(exact) < 1e-8
