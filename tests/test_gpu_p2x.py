"""P2M / P2L on the GPU (sfmm_p2x_device, sfmm_p2x_ragged_device) against the
oracle's FP64 restatement of the reference's fmadd(q, harmonics::R/S(P, x - c))
(solid.cpp:70-104, harmonics.cpp:32-80 and :177-224).

Orders up to 32 run in float-float on the FP32 pipe over power-of-two scaled
coordinates (orders 25..32 in two launches, each accumulating half of the
harmonics); above, one FP64 thread per expansion.  Every coefficient's error
is measured against the sum of the absolute values of its terms' bounds
(p2x_abs_scale): float-float carries about 2^-48 per operation where FP64
carries 2^-53, and a sum of charges of both signs can cancel far below its
terms, so the sum itself is no scale for the error.  P2M is also checked
degree by degree in the Schmidt-normalised basis, where each degree carries its
share of the field, so that the small high-degree coefficients cannot hide
behind degree 0.
"""
import numpy as np
import pytest

from helpers import S_of, norm_weights, p2x_abs_scale, p2x_err, rel_err

pytestmark = pytest.mark.gpu

# float-float: error per coefficient over its absolute scale (measured
# <= 6.0e-14 at orders 1..32), and per degree of a P2M expansion (<= 2.9e-13)
TOL_ABS = 1e-13
TOL_DEG = 1e-12


def schmidt_degree_err(got, ref, P, kind):
    """max over expansions and degrees of the relative L2 error of one degree
    in the Schmidt-normalised basis (multipoles x sig, locals / sig)."""
    w = norm_weights(P, "M" if kind == 0 else "L")
    g = np.asarray(got, np.float64) * w
    r = np.asarray(ref, np.float64) * w
    worst = 0.0
    for n in range(P):
        idx = [n * (n + 1) + m for m in range(n + 1)] + [(n + 1) * (n + 1) + m for m in range(1, n + 1)]
        num = np.linalg.norm(g[:, idx] - r[:, idx], axis=1)
        den = np.linalg.norm(r[:, idx], axis=1)
        ok = den > 0
        if ok.any():
            worst = max(worst, float(np.max(num[ok] / den[ok])))
    return worst


def charges(rng, n, nq, kind, radius=0.5, offset=0.0):
    d = rng.normal(size=(n, nq, 3))
    d *= (radius * rng.random((n, nq, 1)) ** (1 / 3)) / np.linalg.norm(d, axis=2, keepdims=True)
    cen = rng.uniform(-0.1, 0.1, (n, 3)) * radius + offset
    pos = cen[:, None, :] + d
    if kind:  # P2L: charges outside a ball of radius 4 r around the centre
        pos = cen[:, None, :] + d + 4 * radius * np.array([1.0, 0.5, -0.25])
    q = rng.choice([-1.0, 1.0], (n, nq))
    return q, pos, cen


def run_p2x(native, P, kind, q, pos, cen, dtype="f64", init=None):
    import torch

    dev = torch.device("cuda", 0)
    n, nq = q.shape
    ctx = native.Context(P, dtype)
    tdt = torch.float64 if dtype == "f64" else torch.float32
    out = torch.zeros(n, S_of(P), dtype=tdt, device=dev) if init is None else torch.as_tensor(init, device=dev)
    ctx.p2x(kind, n, nq, torch.as_tensor(q, device=dev), torch.as_tensor(pos, device=dev),
            torch.as_tensor(cen, device=dev), out, S_of(P))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("P", list(range(1, 34)))
def test_every_order(native, oracle, P, kind):
    rng = np.random.default_rng(100 * P + kind)
    q, pos, cen = charges(rng, 37, 23, kind)
    ref = oracle.p2m(P, q, pos, cen, singular=bool(kind))
    got = run_p2x(native, P, kind, q, pos, cen)
    assert p2x_err(got, ref, P, kind, q, pos, cen) < TOL_ABS
    if kind == 0:
        assert schmidt_degree_err(got, ref, P, kind) < TOL_DEG


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("radius,offset", [(1e-6, 1e3), (1e4, 0.0), (3e-3, -7.0)])
def test_scales_and_offsets(native, oracle, kind, radius, offset):
    """Clusters far from the origin and of very different sizes: the power-of-two
    scaling keeps the float-float words in range."""
    P = 20
    rng = np.random.default_rng(7)
    q, pos, cen = charges(rng, 16, 40, kind, radius=radius, offset=offset)
    ref = oracle.p2m(P, q, pos, cen, singular=bool(kind))
    got = run_p2x(native, P, kind, q, pos, cen)
    assert p2x_err(got, ref, P, kind, q, pos, cen) < TOL_ABS
    if kind == 0:
        assert schmidt_degree_err(got, ref, P, kind) < TOL_DEG


@pytest.mark.parametrize("kind", [0, 1])
def test_accumulates_into_output(native, oracle, kind):
    P = 12
    rng = np.random.default_rng(3)
    q, pos, cen = charges(rng, 9, 17, kind)
    # existing contents of each coefficient's own magnitude, so that got - init
    # does not cancel the small high-degree coefficients away
    init = rng.normal(size=(9, S_of(P))) * p2x_abs_scale(P, kind, q, pos, cen)
    ref = oracle.p2m(P, q, pos, cen, singular=bool(kind))
    got = run_p2x(native, P, kind, q, pos, cen, init=init.copy())
    assert p2x_err(got - init, ref, P, kind, q, pos, cen) < TOL_ABS


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("P", [3, 12, 17, 24, 30])
def test_ragged_with_empty_leaves(native, oracle, P, kind):
    import torch

    rng = np.random.default_rng(P + 31 * kind)
    counts = np.array([0, 1, 5, 0, 33, 8, 0, 64, 2, 17, 0, 40])
    n = len(counts)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    q, pos, cen = charges(rng, n, int(counts.max()), kind)
    qs = np.concatenate([q[j, :c] for j, c in enumerate(counts)])
    ps = np.concatenate([pos[j, :c] for j, c in enumerate(counts)])
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    out = torch.zeros(n, S_of(P), dtype=torch.float64, device=dev)
    ctx.p2x_ragged(kind, n, torch.as_tensor(off.astype(np.int32), device=dev), torch.as_tensor(qs, device=dev),
                   torch.as_tensor(ps, device=dev), torch.as_tensor(cen, device=dev), out, S_of(P))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref = np.zeros_like(got)
    for j, c in enumerate(counts):
        if c:
            ref[j] = oracle.p2m(P, q[j:j + 1, :c], pos[j:j + 1, :c], cen[j:j + 1], singular=bool(kind))[0]
    assert np.all(got[counts == 0] == 0)
    qz = np.where(np.arange(q.shape[1])[None, :] < counts[:, None], q, 0.0)
    assert p2x_err(got, ref, P, kind, qz, pos, cen) < TOL_ABS
    if kind == 0:
        assert schmidt_degree_err(got[counts > 0], ref[counts > 0], P, kind) < TOL_DEG


@pytest.mark.parametrize("kind", [0, 1])
def test_fp32_context(native, oracle, kind):
    P = 16
    rng = np.random.default_rng(5)
    q, pos, cen = charges(rng, 20, 30, kind)
    ref = oracle.p2m(P, q, pos, cen, singular=bool(kind))
    got = run_p2x(native, P, kind, q, pos, cen, dtype="f32")
    assert got.dtype == np.float32
    assert p2x_err(got, ref, P, kind, q, pos, cen) < 1e-6


def test_many_expansions(native, oracle):
    """A leaf-level batch (4096 leaves x 32 charges at P=12) checked on a sample."""
    P = 12
    rng = np.random.default_rng(9)
    q, pos, cen = charges(rng, 4096, 32, 0, radius=1 / 64)
    got = run_p2x(native, P, 0, q, pos, cen)
    pick = rng.choice(4096, 64, replace=False)
    ref = oracle.p2m(P, q[pick], pos[pick], cen[pick])
    assert p2x_err(got[pick], ref, P, 0, q[pick], pos[pick], cen[pick]) < TOL_ABS
    assert rel_err(got[pick], ref) < TOL_ABS
    assert schmidt_degree_err(got[pick], ref, P, 0) < TOL_DEG


@pytest.mark.parametrize("P", [1, 5, 16, 30])
def test_p2m_charge_at_the_centre(native, oracle, P):
    """A charge exactly at the centre adds q to R_0^0 only; the expansion's
    scale then comes from the other charges (none in the first expansion)."""
    rng = np.random.default_rng(P)
    q = np.array([[2.5, 0.0, 0.0], [1.0, -1.0, 0.5]])
    cen = np.array([[0.3, -0.2, 0.1], [0.0, 0.0, 0.0]])
    pos = np.repeat(cen[:, None, :], 3, axis=1).copy()
    pos[1, 1:] += rng.normal(size=(2, 3)) * 0.3
    ref = oracle.p2m(P, q, pos, cen)
    got = run_p2x(native, P, 0, q, pos, cen)
    assert got[0, 0] == 2.5 and np.all(got[0, 1:] == 0)
    assert p2x_err(got, ref, P, 0, q, pos, cen) < TOL_ABS


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("radius", [1e-25, 1e20])
def test_scales_beyond_fp32_range(native, oracle, kind, radius):
    """|x - c|^2 outside the FP32 range: the scale comes from the doubles'
    exponents, so the float-float columns still see |x'| near 1."""
    P = 12
    rng = np.random.default_rng(31)
    q, pos, cen = charges(rng, 8, 24, kind, radius=radius)
    ref = oracle.p2m(P, q, pos, cen, singular=bool(kind))
    got = run_p2x(native, P, kind, q, pos, cen)
    assert p2x_err(got, ref, P, kind, q, pos, cen) < TOL_ABS
