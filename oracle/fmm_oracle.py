"""Test infrastructure: the FMM pass of a uniform octree restated on the CPU
with its own box indexing and interaction lists (numpy loops over offsets)
and the oracle's rotation-method translations in FP64 (pyoracle.rot), for
checking the GPU pass.  Box (i, j, k) of level l has index (i 2^l + j) 2^l + k
and centre ((i, j, k) + 1/2) 2^-l; interaction lists hold the children of
the parent's neighbours that are not neighbours (doc/solidfmm.tex:660-690
describes the level-wise use of the translations)."""
from __future__ import annotations

import itertools

import numpy as np

import pyoracle


def _centre(l, i, j, k):
    return (np.array([i, j, k], dtype=np.float64) + 0.5) / 2 ** l


def fmm_pass(depth: int, P: int, charges: np.ndarray, positions: np.ndarray, nthreads: int = 8):
    """Leaf local expansions of one pass (P2M, M2M up to level 2, M2L at
    levels 2..depth, L2L down): charges (leaves, q), positions (leaves, q, 3)."""
    S = P * (P + 1)
    M = {}
    L = {}
    n = 2 ** depth
    cen = np.array([_centre(depth, *ijk) for ijk in itertools.product(range(n), repeat=3)])
    M[depth] = pyoracle.p2m(P, charges, positions, cen)
    for l in range(depth, 2, -1):
        nc, npar = 2 ** l, 2 ** (l - 1)
        M[l - 1] = np.zeros((npar ** 3, S))
        src, tgt, sh = [], [], []
        for i, j, k in itertools.product(range(nc), repeat=3):
            c = (i * nc + j) * nc + k
            p = ((i // 2) * npar + j // 2) * npar + k // 2
            src.append(c)
            tgt.append(p)
            sh.append(_centre(l - 1, i // 2, j // 2, k // 2) - _centre(l, i, j, k))
        o = np.full(len(src), P, np.uint32)
        pyoracle.rot("m2m", M[l], o, M[l - 1], o, np.array(sh), sidx=np.array(src), tidx=np.array(tgt),
                     nthreads=nthreads)
    for l in range(2, depth + 1):
        nl = 2 ** l
        L[l] = np.zeros((nl ** 3, S))
        ijk = np.array(list(itertools.product(range(nl), repeat=3)))          # target coordinates
        offs = np.array([o for o in itertools.product(range(-3, 4), repeat=3) if max(map(abs, o)) >= 2])
        cand = ijk[:, None, :] + offs[None, :, :]
        ok = np.all((cand >= 0) & (cand < nl), axis=2)
        ok &= np.max(np.abs(cand // 2 - ijk[:, None, :] // 2), axis=2) <= 1
        t, k = np.nonzero(ok)
        sc = cand[t, k]
        src = (sc[:, 0] * nl + sc[:, 1]) * nl + sc[:, 2]
        tc = ijk[t]
        sh = (tc - sc).astype(np.float64) / 2 ** l
        o = np.full(len(src), P, np.uint32)
        pyoracle.rot("m2l", M[l], o, L[l], o, sh, sidx=src.astype(np.uint32), tidx=t.astype(np.uint32),
                     nthreads=nthreads)
    for l in range(2, depth):
        nc, npar = 2 ** (l + 1), 2 ** l
        src, tgt, sh = [], [], []
        for i, j, k in itertools.product(range(nc), repeat=3):
            src.append(((i // 2) * npar + j // 2) * npar + k // 2)
            tgt.append((i * nc + j) * nc + k)
            sh.append(_centre(l + 1, i, j, k) - _centre(l, i // 2, j // 2, k // 2))
        o = np.full(len(src), P, np.uint32)
        pyoracle.rot("l2l", L[l], o, L[l + 1], o, np.array(sh), sidx=np.array(src), tidx=np.array(tgt),
                     nthreads=nthreads)
    return L[depth]
