"""Shared helpers for the tests: error metrics, golden-case loading, and a
runner that pushes a batch through the C ABI (device path) with torch
tensors as device memory."""
from __future__ import annotations

import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

GOLDEN = os.path.join(ROOT, "tests", "golden", "translations.npz")


def S_of(P: int) -> int:
    return P * (P + 1)


def norm_weights(P: int, kind: str) -> np.ndarray:
    """Weights turning solid coefficients of order P into the orthonormal
    (Schmidt) basis: L / sqrt((n-m)!(n+m)!) for locals, M * sqrt(...) for
    multipoles.  In that basis the squared L2 norm of an expansion is the
    squared L2 norm of its field over the unit sphere (up to a constant)."""
    w = np.ones(S_of(P))
    for n in range(P):
        for m in range(n + 1):
            d = math.sqrt(math.factorial(n - m) * math.factorial(n + m))
            f = d if kind == "M" else 1.0 / d
            w[n * (n + 1) + m] = f
            w[(n + 1) * (n + 1) + m] = f
    return w


def p2x_abs_scale(P, kind, q, pos, cen):
    """Per coefficient of a P2M (kind 0) or P2L (kind 1) sum, the sum of the
    absolute values of its terms' bounds: sum_k |q_k| |x_k|^n / sig(n,m) for R
    and sum_k |q_k| sig(n,m) / |x_k|^(n+1) for S, sig(n,m) = sqrt((n+m)!(n-m)!)
    (|R_n^m| and |S_n^m| never exceed those).  Rounding errors of the sum
    scale with it, not with the sum itself, which may cancel."""
    d = np.asarray(pos, np.float64) - np.asarray(cen, np.float64)[:, None, :]
    r = np.linalg.norm(d, axis=2)
    aq = np.abs(np.asarray(q, np.float64))
    out = np.zeros((aq.shape[0], S_of(P)))
    for n in range(P):
        s = (aq * (r ** n if kind == 0 else r ** (-(n + 1)))).sum(1)
        for m in range(n + 1):
            sg = math.sqrt(math.factorial(n + m) * math.factorial(n - m))
            out[:, n * (n + 1) + m] = out[:, (n + 1) * (n + 1) + m] = s / sg if kind == 0 else s * sg
    return out


def p2x_err(got, ref, P, kind, q, pos, cen):
    """max over coefficients of |got - ref| / p2x_abs_scale."""
    sc = p2x_abs_scale(P, kind, q, pos, cen)
    err = np.abs(np.asarray(got, np.float64) - np.asarray(ref, np.float64))
    return float(np.max(np.where(sc > 0, err / np.where(sc > 0, sc, 1.0), err)))


def rel_err(got, ref, weights=None):
    """max over rows of the relative L2 error (optionally weighted)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    if weights is not None:
        got = got * weights[: got.shape[-1]]
        ref = ref * weights[: ref.shape[-1]]
    num = np.linalg.norm(got - ref, axis=-1)
    den = np.linalg.norm(ref, axis=-1)
    ok = den > 0
    if not ok.any():
        return float(np.max(num))
    return float(np.max(num[ok] / den[ok]))


def per_degree_err(got, ref, P, weights=None):
    out = []
    for n in range(P):
        idx = list(range(n * (n + 1), n * (n + 1) + n + 1)) + list(range((n + 1) ** 2, (n + 1) ** 2 + n + 1))
        g = np.asarray(got)[..., idx]
        r = np.asarray(ref)[..., idx]
        if weights is not None:
            g = g * weights[idx]
            r = r * weights[idx]
        num = np.linalg.norm(g - r, axis=-1)
        den = np.linalg.norm(r, axis=-1)
        ok = den > 0
        out.append(float(np.max(num[ok] / den[ok])) if ok.any() else 0.0)
    return out


def load_golden():
    z = np.load(GOLDEN)
    cases = {}
    for k in z.files:
        name, field = k.split("/")
        cases.setdefault(name, {})[field] = z[k]
    return cases


def run_device(ctx, op, precision, src, dst0, Pin, Pout, xyz, sidx=None, tidx=None, repeat=False, order=None,
               order_bound=0):
    """dst0 + T(src) computed on the GPU through sfmm_translate_device."""
    import torch

    dev = torch.device("cuda", 0)
    dt = torch.float64 if src.dtype == np.float64 else torch.float32
    s = torch.as_tensor(np.ascontiguousarray(src), dtype=dt, device=dev)
    d = torch.as_tensor(np.ascontiguousarray(dst0), dtype=dt, device=dev)
    pi = torch.as_tensor(np.asarray(Pin, np.uint32).astype(np.int32), device=dev)
    po = torch.as_tensor(np.asarray(Pout, np.uint32).astype(np.int32), device=dev)
    sh = torch.as_tensor(np.ascontiguousarray(xyz, np.float64), device=dev)
    si = None if sidx is None else torch.as_tensor(np.asarray(sidx, np.uint32).astype(np.int32), device=dev)
    ti = None if tidx is None else torch.as_tensor(np.asarray(tidx, np.uint32).astype(np.int32), device=dev)
    od = None if order is None else torch.as_tensor(np.asarray(order, np.uint32).astype(np.int32), device=dev)
    ctx.translate_device(op, precision, len(Pin), s, s.shape[-1], s.shape[0], d, d.shape[-1], d.shape[0], pi, po, sh,
                         src_index=si, dst_index=ti, order=od, repeat=repeat, order_bound=order_bound)
    torch.cuda.synchronize()
    assert ctx.device_status() == 0
    return d.cpu().numpy()


def device_batch(ctx, op, P, N, nq, seed, dev):
    """Full-size inputs generated on the GPU (the benchmark's distribution):
    sources by P2M (P2L for L2L) of nq unit charges of random sign uniform in
    a ball of radius 0.5, the L2L clouds centred at distance U[2,4]; M2L
    shifts of uniform direction and length U[2,4], M2M/L2L shifts to a random
    octant corner (length 0.5 sqrt 3)."""
    import torch

    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    S = P * (P + 1)
    src = torch.zeros(N, S, dtype=torch.float64, device=dev)
    for b in range(0, N, 250_000):
        m = min(250_000, N - b)
        d = torch.randn(m, nq, 3, dtype=torch.float64, device=dev, generator=g)
        pos = d / d.norm(dim=2, keepdim=True) * 0.5 * torch.rand(m, nq, 1, dtype=torch.float64, device=dev,
                                                                 generator=g) ** (1.0 / 3.0)
        q = torch.randint(0, 2, (m, nq), device=dev, generator=g).to(torch.float64) * 2 - 1
        if op == "l2l":
            u = torch.randn(m, 3, dtype=torch.float64, device=dev, generator=g)
            pos = pos + (u / u.norm(dim=1, keepdim=True) *
                         (2 + 2 * torch.rand(m, 1, dtype=torch.float64, device=dev, generator=g)))[:, None, :]
        ctx.p2x(1 if op == "l2l" else 0, m, nq, q.contiguous(), pos.contiguous(),
                torch.zeros(m, 3, dtype=torch.float64, device=dev), src[b:b + m], S)
    if op == "m2l":
        u = torch.randn(N, 3, dtype=torch.float64, device=dev, generator=g)
        shift = u / u.norm(dim=1, keepdim=True) * (2 + 2 * torch.rand(N, 1, dtype=torch.float64, device=dev,
                                                                      generator=g))
    else:
        shift = 0.5 * (torch.randint(0, 2, (N, 3), device=dev, generator=g).to(torch.float64) * 2 - 1)
    return src, shift.contiguous()


def rel_err_dev(got, ref, weights=None):
    """rel_err on device tensors (max over rows of the relative L2 error),
    reduced on the GPU; rows with a zero reference are skipped."""
    import torch

    got = got.to(torch.float64)
    ref = ref.to(torch.float64)
    if weights is not None:
        w = torch.as_tensor(weights[: got.shape[-1]], dtype=torch.float64, device=got.device)
        got = got * w
        ref = ref * w
    num = (got - ref).norm(dim=-1)
    den = ref.norm(dim=-1)
    ok = den > 0
    return float((num[ok] / den[ok]).max()) if bool(ok.any()) else float(num.max())


# Fixed geometries of the reference's own physics checks (tests/test_m2l.cpp:
# 57-60, test_m2m.cpp:55-58, test_l2l.cpp:54-57): unit source s, expansion
# centres a (input) and b (output), evaluation point x.
PHYSICS = {
    "m2l": dict(s=(1.1, 0.2, 0.9), a=(1.0, 0.0, 1.0), b=(0.3, 0.1, 2.0), x=(0.1, 0.2, 2.5)),
    "m2m": dict(s=(1.1, 0.2, 0.9), a=(1.0, 0.0, 1.0), b=(0.0, 0.0, 0.0), x=(3.1, 0.1, 2.5)),
    "l2l": dict(s=(5.1, 0.2, 0.9), a=(1.0, 0.0, 1.0), b=(0.0, 0.0, 0.0), x=(0.1, 0.1, 0.2)),
}


def physics_inputs(op, P):
    """Input expansion (R of the source about a for M2M/M2L, S for L2L, by the
    oracle's harmonics) and the shift b - a of the reference's physics checks."""
    import pyoracle

    g = PHYSICS[op]
    s, a, b = (np.asarray(g[k]) for k in ("s", "a", "b"))
    d = s - a
    E = pyoracle.harmonic("S" if op == "l2l" else "R", P, *d)
    return E, b - a


def physics_errors(op, P, out):
    """Relative potential error r |phi - 1/r| and relative gradient error of
    the translated expansion `out` (centred at b) at the evaluation point, as
    the reference's tests print them; the gradient by central differences of
    the oracle's harmonics (step 1e-4 of |x - b|, error ~1e-9 relative)."""
    import pyoracle

    g = PHYSICS[op]
    s, b, x = (np.asarray(g[k]) for k in ("s", "b", "x"))
    kind = "S" if op == "m2m" else "R"
    r = float(np.linalg.norm(x - s))

    def phi(p):
        return pyoracle.dot(out, P, pyoracle.harmonic(kind, P, *(p - b)), P)

    pot = phi(x)
    h = 1e-4 * float(np.linalg.norm(x - b))
    grad = np.array([(phi(x + h * e) - phi(x - h * e)) / (2 * h) for e in np.eye(3)])
    exact = -(x - s) / r ** 3
    return r * abs(pot - 1.0 / r), float(np.linalg.norm(grad - exact) / np.linalg.norm(exact))


def physics_gpu(ctx, op, P, precision):
    """The reference's physics check through the C ABI: 32 identical
    translations into one target (accumulated with atomics), divided by 32."""
    E, shift = physics_inputs(op, P)
    S = P * (P + 1)
    src = E.reshape(1, S)
    dst = np.zeros((1, S))
    n = 32
    out = run_device(ctx, op, precision, src, dst, np.full(n, P, np.uint32), np.full(n, P, np.uint32),
                     np.tile(shift, (n, 1)), sidx=np.zeros(n, np.uint32), tidx=np.zeros(n, np.uint32), repeat=True,
                     order_bound=P)
    return physics_errors(op, P, out[0] / n)


def physics_reference(op, P, dtype=np.float64):
    """The same check through the reference library (its classic single-thread
    call, 32 translations into one target), or None where it was not built."""
    import pyoracle

    native = not pyoracle.ref_available()
    if not pyoracle.ref_available(native=native):
        return None
    E, shift = physics_inputs(op, P)
    S = P * (P + 1)
    n = 32
    src = E.reshape(1, S).astype(dtype)
    dst = np.zeros((1, S), dtype)
    pn = np.full(1, P, np.uint32)
    pyoracle.reference(op, P, src, pn, dst, pn, np.tile(shift, (n, 1)).astype(dtype), np.zeros(n, np.uint32),
                       np.zeros(n, np.uint32), mode=0, native=native)
    return physics_errors(op, P, dst[0].astype(np.float64) / n)
