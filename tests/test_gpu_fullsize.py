"""GPU parity at the benchmark sizes, through properties that hold at any
size: agreement of the split and FP32 paths with plain FP64 over every
translation, bit-identical results whatever the batch is cut into,
linearity, the FP64 oracle on random samples drawn from the whole batch
(on all of it where the oracle is fast enough), plans against direct
launches, and a full FMM pass against the oracle's pass.

Sizes: M2L P=10 x 10^5 (64 charges per source); M2M, M2L, L2L P=20 x 10^6
(128 charges); M2L P=16 x 2*10^6 (64 charges); 1.5*10^6 mixed translations
(40% M2L, 30% M2M, 30% L2L, orders U{4..24}); a depth-5 octree at P=12
(32 768 leaves x 32 charges).  Inputs are generated on the GPU with fixed
seeds; tolerances are relative L2 errors per translation in the orthonormal
basis, maximum over the batch."""
import os
import sys

import numpy as np
import pytest

from helpers import device_batch, norm_weights, rel_err, rel_err_dev

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
THREADS = os.cpu_count() or 1


def _dev():
    import torch

    return torch.device("cuda", 0)


def _run(ctx, op, prec, src, shift, order, out=None, lo=0, hi=None):
    """T(src[lo:hi]) into out[lo:hi] (fresh zeros when out is None)."""
    import torch

    hi = len(src) if hi is None else hi
    S = src.shape[1]
    if out is None:
        out = torch.zeros(len(src), S, dtype=src.dtype, device=src.device)
    n = hi - lo
    ctx.translate_device(op, prec, n, src[lo:hi], S, n, out[lo:hi], S, n, order[lo:hi], order[lo:hi],
                         shift[lo:hi], order_bound=ctx.P)
    return out


def _rows(t, rows):
    """rows (a numpy index array) of a device tensor, on the host"""
    import torch

    return t[torch.as_tensor(rows, device=t.device)].cpu().numpy()


def _oracle_rows(oracle, op, src, shift, P, rows):
    S = P * (P + 1)
    ref = np.zeros((len(rows), S))
    o = np.full(len(rows), P, np.uint32)
    oracle.naive(op, _rows(src, rows), o, ref, o, _rows(shift, rows), nthreads=THREADS)
    return ref


def test_m2l_p10_1e5_all_against_oracle(native, oracle):
    """The whole 10^5 batch of M2L at P=10 against the FP64 oracle."""
    import torch

    P, N = 10, 100_000
    ctx = native.Context(P, "f64")
    src, shift = device_batch(ctx, "m2l", P, N, 64, 101, _dev())
    order = torch.full((N,), P, dtype=torch.int32, device=_dev())
    ref = _oracle_rows(oracle, "m2l", src, shift, P, np.arange(N))
    w = norm_weights(P, "L")
    for prec, tol in ((0, 1e-12), (1, 1e-7), (2, 1e-11)):
        got = _run(ctx, "m2l", prec, src, shift, order)
        torch.cuda.synchronize()
        assert rel_err(got.cpu().numpy(), ref, w) < tol, prec


@pytest.mark.parametrize("op", ["m2m", "m2l", "l2l"])
def test_p20_1e6_fp64_split_fp32(native, oracle, op):
    """10^6 translations at P=20: plain FP64 against the oracle on 500
    random rows; split and FP32 (above the reference's float limit of 18)
    against plain FP64 on every row."""
    import torch

    P, N = 20, 1_000_000
    dev = _dev()
    ctx = native.Context(P, "f64")
    src, shift = device_batch(ctx, op, P, N, 128, 200 + len(op), dev)
    order = torch.full((N,), P, dtype=torch.int32, device=dev)
    w = norm_weights(P, "M" if op == "m2m" else "L")
    plain = _run(ctx, op, 0, src, shift, order)
    rows = np.random.default_rng(7).choice(N, 500, replace=False)
    ref = _oracle_rows(oracle, op, src, shift, P, rows)
    torch.cuda.synchronize()
    assert rel_err(_rows(plain, rows), ref, w) < 1e-12
    split = _run(ctx, op, 1, src, shift, order)
    assert rel_err_dev(split, plain, w) < 1e-7
    del split
    c32 = native.Context(P, "f32")
    s32 = src.to(torch.float32)
    del src
    f32 = _run(c32, op, 0, s32, shift, order)
    torch.cuda.synchronize()
    assert rel_err_dev(f32, plain, w) < 2e-5


@pytest.fixture(scope="module")
def m2l16(native):
    import torch

    P, N = 16, 2_000_000
    ctx = native.Context(P, "f64")
    src, shift = device_batch(ctx, "m2l", P, N, 64, 1234, _dev())
    order = torch.full((N,), P, dtype=torch.int32, device=_dev())
    return ctx, src, shift, order


def test_m2l_p16_2e6_split_against_plain_and_oracle(native, oracle, m2l16):
    """The headline batch: split within 1e-7 of plain FP64 on all 2*10^6
    translations, both against the oracle on 1 000 rows drawn from the whole
    batch."""
    import torch

    ctx, src, shift, order = m2l16
    w = norm_weights(16, "L")
    plain = _run(ctx, "m2l", 0, src, shift, order)
    split = _run(ctx, "m2l", 1, src, shift, order)
    torch.cuda.synchronize()
    assert rel_err_dev(split, plain, w) < 1e-7
    rows = np.random.default_rng(8).choice(len(src), 1000, replace=False)
    ref = _oracle_rows(oracle, "m2l", src, shift, 16, rows)
    assert rel_err(_rows(plain, rows), ref, w) < 1e-12
    assert rel_err(_rows(split, rows), ref, w) < 1e-7


@pytest.mark.parametrize("prec", [0, 1], ids=["plain", "split"])
def test_m2l_p16_2e6_partition_invariance(native, m2l16, prec):
    """The same 2*10^6 translations launched as one batch and as uneven
    pieces (1, 333 332, 666 667, 999 999 and 1 translations) give
    bit-identical targets: no result depends on where a translation falls in
    the launch."""
    import torch

    ctx, src, shift, order = m2l16
    whole = _run(ctx, "m2l", prec, src, shift, order)
    cuts = [0, 1, 333_333, 1_000_000, 1_999_999, len(src)]
    pieces = torch.zeros_like(whole)
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        _run(ctx, "m2l", prec, src, shift, order, out=pieces, lo=lo, hi=hi)
    torch.cuda.synchronize()
    assert torch.equal(whole, pieces)


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-7)], ids=["plain", "split"])
def test_m2l_p16_linearity(native, m2l16, prec, tol):
    """T(A + 2B) = T(A) + 2 T(B) over 10^6 pairs of sources (the two halves
    of the batch, each half with its own shifts), relative to |T(A)| +
    2|T(B)| per translation."""
    import torch

    ctx, src, shift, order = m2l16
    h = len(src) // 2
    A, B = src[:h], src[h:2 * h]
    sh, o = shift[:h].contiguous(), order[:h]
    tA = _run(ctx, "m2l", prec, A, sh, o)
    tB = _run(ctx, "m2l", prec, B, sh, o)
    tAB = _run(ctx, "m2l", prec, (A + 2 * B).contiguous(), sh, o)
    torch.cuda.synchronize()
    w = torch.as_tensor(norm_weights(16, "L"), device=A.device)
    num = ((tAB - tA - 2 * tB) * w).norm(dim=1)
    den = (tA * w).norm(dim=1) + 2 * (tB * w).norm(dim=1)
    assert float((num / den).max()) < tol


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-7), (2, 1e-11)], ids=["plain", "split", "split_ff"])
def test_mixed_1_5e6_plan_against_direct_and_oracle(native, oracle, prec, tol):
    """1.5*10^6 mixed translations (40% M2L, 30% M2M, 30% L2L; P_in, P_out
    iid U{4..24}; sources drawn from 65 536 expansions per kind): one
    execution plan (order-sorted segments in a CUDA graph) against one
    unsorted launch per operator at order bound 24, and the plan against the
    oracle on 300 rows per operator."""
    import torch

    P, N, NS = 24, 1_500_000, 65_536
    S = P * (P + 1)
    dev = _dev()
    ctx = native.Context(P, "f64")
    srcM, _ = device_batch(ctx, "m2m", P, NS, 64, 500, dev)
    srcL, _ = device_batch(ctx, "l2l", P, NS, 64, 600, dev)
    g = torch.Generator(device=dev)
    g.manual_seed(700)
    counts = {"m2l": int(0.4 * N), "m2m": int(0.3 * N)}
    counts["l2l"] = N - counts["m2l"] - counts["m2m"]
    planned = torch.zeros(N, S, dtype=torch.float64, device=dev)
    direct = torch.zeros(N, S, dtype=torch.float64, device=dev)
    plan = native.Plan(ctx)
    batches = {}
    off = 0
    for op in ("m2l", "m2m", "l2l"):
        n = counts[op]
        pin = torch.randint(4, 25, (n,), device=dev, generator=g, dtype=torch.int32)
        pout = torch.randint(4, 25, (n,), device=dev, generator=g, dtype=torch.int32)
        sidx = torch.randint(0, NS, (n,), device=dev, generator=g, dtype=torch.int32)
        if op == "m2l":
            u = torch.randn(n, 3, dtype=torch.float64, device=dev, generator=g)
            sh = u / u.norm(dim=1, keepdim=True) * (2 + 2 * torch.rand(n, 1, dtype=torch.float64, device=dev,
                                                                          generator=g))
        else:
            sh = 0.5 * (torch.randint(0, 2, (n, 3), device=dev, generator=g).to(torch.float64) * 2 - 1)
        sh = sh.contiguous()
        src = srcL if op == "l2l" else srcM
        plan.add(op, prec, n, src, S, NS, planned[off:off + n], S, n, pin, pout, sh, src_index=sidx)
        ctx.translate_device(op, prec, n, src, S, NS, direct[off:off + n], S, n, pin, pout, sh, src_index=sidx,
                             order_bound=P)
        batches[op] = (off, n, pin, pout, sidx, sh, src)
        off += n
    plan.finalize()
    plan.run()
    torch.cuda.synchronize()
    rng = np.random.default_rng(9)
    for op, (o, n, pin, pout, sidx, sh, src) in batches.items():
        w = norm_weights(P, "M" if op == "m2m" else "L")
        assert rel_err_dev(planned[o:o + n], direct[o:o + n], w) < tol, op
        rows = rng.choice(n, 300, replace=False)
        ref = np.zeros((300, S))
        oracle.naive(op, src.cpu().numpy(), _rows(pin, rows).astype(np.uint32), ref,
                     _rows(pout, rows).astype(np.uint32), _rows(sh, rows),
                     sidx=_rows(sidx, rows).astype(np.uint32), nthreads=THREADS)
        got = _rows(planned[o:o + n], rows)
        assert rel_err(got, ref, w) < {0: 1e-12, 1: 1e-7, 2: 1e-11}[prec], op


def test_fmm_depth5_pass_against_oracle_pass(native, oracle):
    """The uniform depth-5 octree at P=12 (32 768 leaves x 32 charges,
    6 039 504 M2L): every leaf local of the split and plain passes against
    the oracle's CPU pass."""
    import torch
    from solidfmm_gb300 import fmm

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fmm_oracle

    depth, P, per = 5, 12, 32
    dev = _dev()
    ctx = native.Context(P, "f64")
    q, pos = fmm.random_particles(depth, per, 900, dev)
    ref = fmm_oracle.fmm_pass(depth, P, q.cpu().numpy(), pos.cpu().numpy(), nthreads=THREADS)
    w = norm_weights(P, "L")
    for prec, tol in ((0, 1e-12), (1, 1e-7)):
        f = fmm.UniformFMM(ctx, depth, prec, dev)
        f.run(q, pos)
        torch.cuda.synchronize()
        assert rel_err(f.leaf_locals().cpu().numpy(), ref, w) < tol, prec
