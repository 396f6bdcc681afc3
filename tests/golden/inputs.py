"""Seeded synthetic translation batches built with the oracle's P2M/P2L.

Geometry follows the workload definitions of the translation benchmarks:
sources are unit charges of random sign, uniform in a ball of radius 0.5
around the expansion centre; M2L shifts have a uniform direction and length
U[2,4]; M2M/L2L shifts go to a random octant corner (+-0.5, +-0.5, +-0.5);
local (L2L) inputs are P2L expansions of a cloud centred at distance U[2,4].
Test infrastructure (uses the oracle).
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                "oracle"))
import pyoracle as O  # noqa: E402


def _orders(rng, spec, n):
    if isinstance(spec, tuple):
        return rng.integers(spec[0], spec[1] + 1, size=n).astype(np.uint32)
    return np.full(n, spec, np.uint32)


def _unit(rng, n):
    d = rng.normal(size=(n, 3))
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def cloud(rng, n, nq, far=False):
    pos = _unit(rng, n * nq).reshape(n, nq, 3) * (0.5 * rng.random((n, nq, 1)) ** (1 / 3))
    if far:
        pos = pos + _unit(rng, n)[:, None, :] * rng.uniform(2, 4, (n, 1, 1))
    q = rng.choice([-1.0, 1.0], size=(n, nq))
    return q, pos


def expansions(rng, kind, P, n, nq):
    """n expansions of order P: 'M' multipoles (P2M) or 'L' locals (P2L)."""
    q, pos = cloud(rng, n, nq, far=(kind == "L"))
    return O.p2m(P, q, pos, np.zeros((n, 3)), singular=(kind == "L"))


def shifts(rng, op, n):
    if op == "m2l":
        return _unit(rng, n) * rng.uniform(2, 4, (n, 1))
    return 0.5 * rng.choice([-1.0, 1.0], size=(n, 3))


def make_batch(rng, op, Pin, Pout, n, nq=24, pattern="distinct", zero_shift=False, in_le_out=False):
    Pi = _orders(rng, Pin, n)
    Po = _orders(rng, Pout, n)
    if in_le_out:
        Pi = np.minimum(Pi, Po)
    if pattern == "same32":
        Pi[:] = Pi[0]
        Po[:] = Po[0]
        nsrc, ntgt = 1, 1
        sidx = np.zeros(n, np.uint32)
        tidx = np.zeros(n, np.uint32)
    elif pattern == "repeat":
        nsrc, ntgt = n, max(n // 3, 1)
        sidx = np.arange(n, dtype=np.uint32)
        tidx = (np.arange(n) % ntgt).astype(np.uint32)
    else:
        nsrc, ntgt = n, n
        sidx = np.arange(n, dtype=np.uint32)
        tidx = np.arange(n, dtype=np.uint32)
    P = max(int(Pi.max()), int(Po.max()), 1)
    S = P * (P + 1)
    kin = "L" if op == "l2l" else "M"
    kout = "M" if op == "m2m" else "L"
    src = np.zeros((nsrc, S))
    Psrc = np.zeros(nsrc, np.uint32)
    Psrc[sidx] = Pi
    for j in range(nsrc):
        p = int(Psrc[j])
        if p:
            src[j, : p * (p + 1)] = expansions(rng, kin, p, 1, nq)[0]
    dst = np.zeros((ntgt, S))
    Ptgt = np.zeros(ntgt, np.uint32)
    Ptgt[tidx] = Po
    for j in range(ntgt):
        p = int(Ptgt[j])
        if p:
            dst[j, : p * (p + 1)] = 0.3 * expansions(rng, kout, p, 1, 4)[0]
    # per-translation orders must agree with the expansions they touch
    Pi = Psrc[sidx]
    Po = Ptgt[tidx]
    xyz = shifts(rng, op, n)
    if pattern == "same32":
        xyz[:] = xyz[0]
    if zero_shift:
        xyz[::2] = 0.0
    return dict(src=src, dst=dst, xyz=xyz, Pin=Pi.astype(np.uint32), Pout=Po.astype(np.uint32), sidx=sidx,
                tidx=tidx)
