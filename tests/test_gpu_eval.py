"""GPU evaluation of expansions (sfmm_eval_device): L2P and M2P potentials
against the oracle's dot(E, R/S(x - c)), L2P gradients against central
differences of the oracle potential, and the physics of P2M -> M2L -> L2P
against direct summation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# float-float evaluation: error per point over the sum of its terms' magnitudes
# (measured <= 2.9e-14 at orders 1..32, both kinds)
TOL_EVAL = 1e-13


def _pot(oracle, kind, E, P, pts, centre):
    h = "R" if kind == 0 else "S"
    return np.array([oracle.dot(E, P, oracle.harmonic(h, P, *(p - centre)), P) for p in pts])


def _pot_abs(oracle, kind, E, P, pts, centre):
    """Per point, the sum of the absolute values of the dot product's terms,
    sum w_m (|E_re H_re| + |E_im H_im|): the scale of the rounding errors of a
    sum whose terms may cancel."""
    h = "R" if kind == 0 else "S"
    w = np.ones(P * (P + 1))
    for n in range(P):
        w[n * (n + 1) + 1:n * (n + 1) + n + 1] = 2.0
        w[(n + 1) * (n + 1) + 1:(n + 1) * (n + 1) + n + 1] = 2.0
    return np.array([np.sum(w * np.abs(E * oracle.harmonic(h, P, *(p - centre)))) for p in pts])


# orders up to 32 in float-float over normalised expansions, 33 in FP64
@pytest.mark.parametrize("P", [1, 2, 6, 12, 20, 24, 32, 33])
@pytest.mark.parametrize("kind", [0, 1], ids=["l2p", "m2p"])
def test_eval_matches_oracle(native, oracle, kind, P):
    import torch

    rng = np.random.default_rng(P + 10 * kind)
    nexp, per = 5, 40
    q = rng.choice([-1.0, 1.0], size=(nexp, 16))
    d = rng.normal(size=(nexp, 16, 3))
    src = d / np.linalg.norm(d, axis=2, keepdims=True) * (0.4 * rng.random((nexp, 16, 1)))
    if kind == 0:  # local expansions of far clouds
        src = src + np.array([3.0, -1.0, 2.0])
    centres = rng.normal(size=(nexp, 3)) * 0.1
    E = oracle.p2m(P, q, src + centres[:, None, :], centres, singular=(kind == 0))
    # points: near the centre for locals, far away for multipoles
    u = rng.normal(size=(nexp * per, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    rad = 0.45 * rng.random((nexp * per, 1)) if kind == 0 else 2.5 + rng.random((nexp * per, 1))
    box = np.repeat(np.arange(nexp), per).astype(np.uint32)
    pts = u * rad + centres[box]
    ref = np.concatenate([_pot(oracle, kind, E[b], P, pts[box == b], centres[b]) for b in range(nexp)])
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    pot = torch.zeros(len(pts), dtype=torch.float64, device=dev)
    S = P * (P + 1)
    ctx.evaluate(kind, len(pts), torch.as_tensor(pts, device=dev), torch.as_tensor(E, device=dev), S, nexp,
                 torch.as_tensor(centres, device=dev), pot, box=torch.as_tensor(box.astype(np.int32), device=dev))
    torch.cuda.synchronize()
    got = pot.cpu().numpy()
    # float-float (orders up to 32): error against the terms' magnitudes
    scale = np.concatenate([_pot_abs(oracle, kind, E[b], P, pts[box == b], centres[b]) for b in range(nexp)])
    assert np.max(np.abs(got - ref) / scale) <= TOL_EVAL


@pytest.mark.parametrize("P", [12, 25])
def test_l2p_gradient_is_derivative(native, oracle, P):
    import torch

    rng = np.random.default_rng(3)
    q = rng.choice([-1.0, 1.0], size=(1, 24))
    d = rng.normal(size=(1, 24, 3))
    src = d / np.linalg.norm(d, axis=2, keepdims=True) * 0.4 + np.array([2.5, 1.0, -1.5])
    L = oracle.p2m(P, q, src, np.zeros((1, 3)), singular=True)
    pts = rng.normal(size=(50, 3)) * 0.2
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    pot = torch.zeros(50, dtype=torch.float64, device=dev)
    grad = torch.zeros(50, 3, dtype=torch.float64, device=dev)
    ctx.evaluate(0, 50, torch.as_tensor(pts, device=dev), torch.as_tensor(L, device=dev), P * (P + 1), 1,
                 torch.zeros(1, 3, dtype=torch.float64, device=dev), pot, gradient=grad,
                 box=torch.zeros(50, dtype=torch.int32, device=dev))
    torch.cuda.synchronize()
    g = grad.cpu().numpy()
    h = 1e-5
    fd = np.zeros_like(g)
    for a in range(3):
        e = np.zeros(3)
        e[a] = h
        fd[:, a] = (_pot(oracle, 0, L[0], P, pts + e, np.zeros(3)) - _pot(oracle, 0, L[0], P, pts - e, np.zeros(3))) / (2 * h)
    assert np.max(np.abs(g - fd)) <= 1e-8 * np.max(np.abs(fd))


def test_p2m_m2l_l2p_physics(native):
    """Charges in a ball of radius 0.5, targets near a centre at distance 4.1:
    P2M -> M2L -> L2P (split precision) reproduces the direct potential and
    field to the truncation error of order 16."""
    import torch

    rng = np.random.default_rng(11)
    P = 16
    dev = torch.device("cuda", 0)
    d = rng.normal(size=(64, 3))
    ys = d / np.linalg.norm(d, axis=1, keepdims=True) * (0.5 * rng.random((64, 1)) ** (1 / 3))
    qs = rng.choice([-1.0, 1.0], size=64)
    ctr = np.array([[2.0, -2.0, 3.0]])
    xs = ctr + rng.normal(size=(100, 3)) * 0.1
    ctx = native.Context(P, "f64")
    S = P * (P + 1)
    M = torch.zeros(1, S, dtype=torch.float64, device=dev)
    ctx.p2x(0, 1, 64, torch.as_tensor(qs[None, :], device=dev), torch.as_tensor(ys[None], device=dev),
            torch.zeros(1, 3, dtype=torch.float64, device=dev), M, S)
    L = torch.zeros(1, S, dtype=torch.float64, device=dev)
    one = torch.full((1,), P, dtype=torch.int32, device=dev)
    ctx.translate_device("m2l", 1, 1, M, S, 1, L, S, 1, one, one, torch.as_tensor(ctr, device=dev))
    pot = torch.zeros(100, dtype=torch.float64, device=dev)
    grad = torch.zeros(100, 3, dtype=torch.float64, device=dev)
    ctx.evaluate(0, 100, torch.as_tensor(xs, device=dev), L, S, 1, torch.as_tensor(ctr, device=dev), pot,
                 gradient=grad, box=torch.zeros(100, dtype=torch.int32, device=dev))
    torch.cuda.synchronize()
    diff = xs[:, None, :] - ys[None, :, :]
    r = np.linalg.norm(diff, axis=2)
    phi = (qs / r).sum(1)
    field = -(qs[None, :, None] * diff / r[..., None] ** 3).sum(1)  # grad of sum q/r
    assert np.max(np.abs(pot.cpu().numpy() - phi)) < 1e-7 * np.max(np.abs(phi))
    assert np.max(np.abs(grad.cpu().numpy() - field)) < 1e-6 * np.max(np.abs(field))


@pytest.mark.parametrize("kind", [0, 1], ids=["l2p", "m2p"])
def test_eval_fp32_context(native, oracle, kind):
    """FP32 expansions (an FP32 context) evaluated in float-float."""
    import torch

    P = 14
    rng = np.random.default_rng(40 + kind)
    q = rng.choice([-1.0, 1.0], size=(3, 16))
    d = rng.normal(size=(3, 16, 3))
    src = d / np.linalg.norm(d, axis=2, keepdims=True) * 0.4
    if kind == 0:
        src = src + np.array([3.0, -1.0, 2.0])
    centres = np.zeros((3, 3))
    E = oracle.p2m(P, q, src, centres, singular=(kind == 0)).astype(np.float32)
    u = rng.normal(size=(90, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pts = u * (0.4 if kind == 0 else 3.0)
    box = np.repeat(np.arange(3), 30).astype(np.uint32)
    ref = np.concatenate([_pot(oracle, kind, E[b].astype(np.float64), P, pts[box == b], centres[b])
                          for b in range(3)])
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f32")
    pot = torch.zeros(len(pts), dtype=torch.float64, device=dev)
    S = P * (P + 1)
    ctx.evaluate(kind, len(pts), torch.as_tensor(pts, device=dev), torch.as_tensor(E, device=dev), S, 3,
                 torch.as_tensor(centres, device=dev), pot, box=torch.as_tensor(box.astype(np.int32), device=dev))
    torch.cuda.synchronize()
    assert np.max(np.abs(pot.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))


def _grad_ref(oracle, L, P, pt):
    """grad of dot(L, R(x)) at x = pt: (d/dx - i d/dy) R_n^m = R_{n-1}^{m-1},
    (d/dx + i d/dy) R_n^m = -R_{n-1}^{m+1}, d/dz R_n^m = R_{n-1}^m, in FP64
    over the oracle's R."""
    R = oracle.harmonic("R", P, *pt)
    re = lambda n, m: L[n * (n + 1) + m]  # noqa: E731
    im = lambda n, m: L[(n + 1) * (n + 1) + m]  # noqa: E731
    g = np.zeros(3)
    for m in range(P):
        for n in range(m, P - 1):
            cr, ci = R[n * (n + 1) + m], R[(n + 1) * (n + 1) + m]
            k1, w = n + 1, (2.0 if m else 1.0)
            g[2] += w * (re(k1, m) * cr + im(k1, m) * ci)
            if m == 0:
                g[0] += cr * re(k1, 1)
                g[1] += cr * im(k1, 1)
            else:
                xr, xi = re(k1, m + 1) - re(k1, m - 1), im(k1, m + 1) - im(k1, m - 1)
                yr, yi = re(k1, m - 1) + re(k1, m + 1), im(k1, m - 1) + im(k1, m + 1)
                g[0] += cr * xr + ci * xi
                g[1] += cr * yi - ci * yr
    return g


@pytest.mark.parametrize("P", [3, 16, 32])
def test_l2p_gradient_matches_fp64_formula(native, oracle, P):
    import torch

    rng = np.random.default_rng(70 + P)
    q = rng.choice([-1.0, 1.0], size=(2, 20))
    d = rng.normal(size=(2, 20, 3))
    src = d / np.linalg.norm(d, axis=2, keepdims=True) * 0.4 + np.array([2.5, 1.0, -1.5])
    centres = np.array([[0.0, 0.0, 0.0], [0.1, -0.2, 0.05]])
    L = oracle.p2m(P, q, src + centres[:, None, :], centres, singular=True)
    box = np.repeat(np.arange(2), 40).astype(np.uint32)
    pts = rng.normal(size=(80, 3)) * 0.25 + centres[box]
    ref = np.array([_grad_ref(oracle, L[b], P, p - centres[b]) for p, b in zip(pts, box)])
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    pot = torch.zeros(80, dtype=torch.float64, device=dev)
    grad = torch.zeros(80, 3, dtype=torch.float64, device=dev)
    ctx.evaluate(0, 80, torch.as_tensor(pts, device=dev), torch.as_tensor(L, device=dev), P * (P + 1), 2,
                 torch.as_tensor(centres, device=dev), pot, gradient=grad,
                 box=torch.as_tensor(box.astype(np.int32), device=dev))
    torch.cuda.synchronize()
    assert np.max(np.abs(grad.cpu().numpy() - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("warm", [False, True], ids=["fresh-fp64", "scratch-float-float"])
def test_eval_inside_graph_capture(native, oracle, warm):
    """A captured evaluation allocates nothing: a fresh context runs the FP64
    kernel in the graph, one whose scratch exists runs the float-float path;
    either replay matches the oracle."""
    import torch

    P, n = 10, 64
    rng = np.random.default_rng(5)
    q = rng.choice([-1.0, 1.0], size=(1, 12))
    d = rng.normal(size=(1, 12, 3))
    src = d / np.linalg.norm(d, axis=2, keepdims=True) * 0.4 + np.array([2.5, 1.0, -1.5])
    L = oracle.p2m(P, q, src, np.zeros((1, 3)), singular=True)
    pts = rng.normal(size=(n, 3)) * 0.2
    ref = _pot(oracle, 0, L[0], P, pts, np.zeros(3))
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    tp, tL = torch.as_tensor(pts, device=dev), torch.as_tensor(L, device=dev)
    cen = torch.zeros(1, 3, dtype=torch.float64, device=dev)
    box = torch.zeros(n, dtype=torch.int32, device=dev)
    pot = torch.zeros(n, dtype=torch.float64, device=dev)
    if warm:  # sizes the scratch outside capture
        ctx.evaluate(0, n, tp, tL, P * (P + 1), 1, cen, pot, box=box)
        torch.cuda.synchronize()
    pot.zero_()
    s = torch.cuda.Stream(device=dev)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ctx.set_stream(s.cuda_stream)
        ctx.evaluate(0, n, tp, tL, P * (P + 1), 1, cen, pot, box=box)
    ctx.set_stream(torch.cuda.current_stream(dev).cuda_stream)
    pot.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert np.max(np.abs(pot.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_eval_few_points_many_expansions(native, oracle):
    """Fewer than one point per four expansions: no normalised copy of the
    whole array (the FP64 kernel), same results."""
    import torch

    P, nexp = 9, 400
    rng = np.random.default_rng(8)
    q = rng.choice([-1.0, 1.0], size=(nexp, 6))
    d = rng.normal(size=(nexp, 6, 3))
    src = d / np.linalg.norm(d, axis=2, keepdims=True) * 0.4 + np.array([2.5, 1.0, -1.5])
    L = oracle.p2m(P, q, src, np.zeros((nexp, 3)), singular=True)
    box = np.array([3, 77, 150, 399, 0, 201], dtype=np.uint32)
    pts = rng.normal(size=(len(box), 3)) * 0.2
    ref = np.array([_pot(oracle, 0, L[b], P, pts[i:i + 1], np.zeros(3))[0] for i, b in enumerate(box)])
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    pot = torch.zeros(len(box), dtype=torch.float64, device=dev)
    ctx.evaluate(0, len(box), torch.as_tensor(pts, device=dev), torch.as_tensor(L, device=dev), P * (P + 1), nexp,
                 torch.zeros(nexp, 3, dtype=torch.float64, device=dev), pot,
                 box=torch.as_tensor(box.astype(np.int32), device=dev))
    torch.cuda.synchronize()
    assert np.max(np.abs(pot.cpu().numpy() - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("P", [1, 2, 12])
def test_l2p_at_the_centre(native, oracle, P):
    """At the centre only R_0^0 = 1 is nonzero: the potential is L_0^0 and the
    gradient comes from the degree-1 coefficients alone."""
    import torch

    rng = np.random.default_rng(P)
    L = rng.normal(size=(1, P * (P + 1)))
    for n in range(P):
        L[0, (n + 1) * (n + 1)] = 0.0  # imaginary part of m = 0
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    pot = torch.zeros(1, dtype=torch.float64, device=dev)
    grad = torch.zeros(1, 3, dtype=torch.float64, device=dev)
    c = np.array([[0.25, -0.5, 1.0]])
    ctx.evaluate(0, 1, torch.as_tensor(c, device=dev), torch.as_tensor(L, device=dev), P * (P + 1), 1,
                 torch.as_tensor(c, device=dev), pot, gradient=grad)
    torch.cuda.synchronize()
    assert pot.item() == pytest.approx(L[0, 0], rel=1e-14, abs=0)
    ref = _grad_ref(oracle, L[0], P, np.zeros(3))
    assert np.max(np.abs(grad.cpu().numpy()[0] - ref)) <= 1e-14 * max(np.max(np.abs(ref)), 1e-300)


def test_eval_tiny_coefficients_with_zeros(native, oracle):
    """A local expansion scaled to ~1e-280 with exact zeros among its
    coefficients: the zeros stay zero and the potential scales exactly."""
    import torch

    P = 8
    rng = np.random.default_rng(12)
    L = rng.normal(size=(1, P * (P + 1)))
    L[0, ::3] = 0.0
    pts = rng.normal(size=(20, 3)) * 0.3
    ref = _pot(oracle, 0, L[0], P, pts, np.zeros(3))
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    pot = torch.zeros(20, dtype=torch.float64, device=dev)
    ctx.evaluate(0, 20, torch.as_tensor(pts, device=dev), torch.as_tensor(L * 1e-280, device=dev), P * (P + 1), 1,
                 torch.zeros(1, 3, dtype=torch.float64, device=dev), pot, box=torch.zeros(20, dtype=torch.int32, device=dev))
    torch.cuda.synchronize()
    got = pot.cpu().numpy() * 1e280
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("kind", [0, 1], ids=["l2p", "m2p"])
@pytest.mark.parametrize("scale", [1e-25, 1e20])
def test_eval_scales_beyond_fp32_range(native, oracle, kind, scale):
    """Geometry scaled so that |x - c|^2 leaves the FP32 range."""
    import torch

    P = 10
    rng = np.random.default_rng(77 + kind)
    q = rng.choice([-1.0, 1.0], size=(2, 12))
    d = rng.normal(size=(2, 12, 3))
    src = d / np.linalg.norm(d, axis=2, keepdims=True) * 0.4
    if kind == 0:
        src = src + np.array([3.0, -1.0, 2.0])
    centres = np.array([[0.0, 0.0, 0.0], [0.5, 0.2, -0.1]])
    E = oracle.p2m(P, q, (src + centres[:, None, :]) * scale, centres * scale, singular=(kind == 0))
    u = rng.normal(size=(40, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    box = np.repeat(np.arange(2), 20).astype(np.uint32)
    pts = (u * (0.3 if kind == 0 else 3.0) + centres[box]) * scale
    ref = np.concatenate([_pot(oracle, kind, E[b], P, pts[box == b], centres[b] * scale) for b in range(2)])
    scl = np.concatenate([_pot_abs(oracle, kind, E[b], P, pts[box == b], centres[b] * scale) for b in range(2)])
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    pot = torch.zeros(40, dtype=torch.float64, device=dev)
    ctx.evaluate(kind, 40, torch.as_tensor(pts, device=dev), torch.as_tensor(E, device=dev), P * (P + 1), 2,
                 torch.as_tensor(centres * scale, device=dev), pot,
                 box=torch.as_tensor(box.astype(np.int32), device=dev))
    torch.cuda.synchronize()
    assert np.max(np.abs(pot.cpu().numpy() - ref) / scl) <= TOL_EVAL
