"""GPU FMM pass (solidfmm_gb300.fmm.UniformFMM): leaf local expansions of a
depth-3 octree against the oracle's independent CPU pass, and the
potential (far field by L2P + near field by direct sums) against direct
summation over all particles."""
import os
import sys

import numpy as np
import pytest

from helpers import norm_weights, rel_err

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fmm_case(native, oracle):
    import torch
    from solidfmm_gb300 import fmm

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fmm_oracle

    depth, P, per = 3, 8, 8
    dev = torch.device("cuda", 0)
    q, pos = fmm.random_particles(depth, per, 3, dev)
    ref = fmm_oracle.fmm_pass(depth, P, q.cpu().numpy(), pos.cpu().numpy())
    return depth, P, per, q, pos, ref


# tensor-core modes (FP32 accumulation in tensor memory): 3xTF32 / BF16x6 measured
# 1.2e-6 / 4.5e-7 and 3xBF16 6.3e-5 at depth 5, P=12
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-7), (2, 1e-11), (3, 5e-6), (4, 3e-4), (5, 2e-6)],
                         ids=["plain", "split", "split_ff", "tc_tf32", "tc_bf16", "tc_bf16x6"])
def test_fmm_pass_matches_oracle(native, fmm_case, prec, tol):
    import torch
    from solidfmm_gb300 import fmm

    depth, P, per, q, pos, ref = fmm_case
    ctx = native.Context(P, "f64")
    f = fmm.UniformFMM(ctx, depth, prec, q.device)
    f.run(q, pos)
    f.run(q, pos)  # a second pass starts from zeroed expansions
    torch.cuda.synchronize()
    got = f.leaf_locals().cpu().numpy()
    assert rel_err(got, ref, norm_weights(P, "L")) < tol


def test_fmm_potential_against_direct_sum(native, fmm_case):
    import torch
    from solidfmm_gb300 import fmm

    depth, P, per, q, pos, ref = fmm_case
    dev = q.device
    ctx = native.Context(P, "f64")
    f = fmm.UniformFMM(ctx, depth, 1, dev)
    f.run(q, pos)
    nleaf = 8 ** depth
    pts = pos.reshape(-1, 3).contiguous()
    box = torch.arange(nleaf, device=dev, dtype=torch.int32).repeat_interleave(per)
    pot = torch.zeros(len(pts), dtype=torch.float64, device=dev)
    ctx.evaluate(0, len(pts), pts, f.leaf_locals(), f.S, nleaf, f.leaf_centres, pot, box=box)
    torch.cuda.synchronize()
    far = pot.cpu().numpy()
    x = pts.cpu().numpy()
    qq = q.reshape(-1).cpu().numpy()
    ns, nt = fmm.neighbours(depth)
    near = np.zeros(len(x))
    leaf_of = np.repeat(np.arange(nleaf), per)
    nbr = [[] for _ in range(nleaf)]
    for a, b in zip(ns.tolist(), nt.tolist()):
        nbr[b].append(a)
    for b in range(nleaf):
        src = np.concatenate([np.arange(a * per, (a + 1) * per) for a in nbr[b]])
        tgt = np.arange(b * per, (b + 1) * per)
        r = np.linalg.norm(x[tgt][:, None, :] - x[src][None, :, :], axis=2)
        with np.errstate(divide="ignore"):
            inv = np.where(r > 0, 1.0 / r, 0.0)
        near[tgt] = (inv * qq[src][None, :]).sum(1)
    r = np.linalg.norm(x[:, None, :] - x[None, :, :], axis=2)
    with np.errstate(divide="ignore"):
        direct = (np.where(r > 0, 1.0 / r, 0.0) * qq[None, :]).sum(1)
    err = np.linalg.norm(far + near - direct) / np.linalg.norm(direct)
    assert leaf_of.shape == far.shape
    assert err < 1e-4, err


def test_fmm_arbitrary_particles(native, oracle):
    """Clustered particles in the unit cube (two blobs: leaves hold 0 to
    about 100 particles) binned on the GPU, P2M over each leaf's own range,
    one pass: the leaf locals match the oracle's pass over the same leaves
    (binned here with numpy, each leaf padded with zero charges), and the
    potential at every particle (far field by L2P at its leaf, near field by
    direct sums over the neighbour leaves) matches direct summation."""
    import torch
    from solidfmm_gb300 import fmm

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fmm_oracle

    depth, P = 3, 10
    n, nleaf = 2 ** depth, 8 ** depth
    rng = np.random.default_rng(21)
    x = np.concatenate([0.25 + 0.06 * rng.standard_normal((1500, 3)), 0.7 + 0.12 * rng.standard_normal((900, 3)),
                        rng.random((300, 3))])
    x = np.clip(x, 0.0, 1.0 - 1e-12)
    qq = rng.uniform(-1, 1, len(x))
    ijk = np.floor(x * n).astype(np.int64)
    leaf = (ijk[:, 0] * n + ijk[:, 1]) * n + ijk[:, 2]
    counts = np.bincount(leaf, minlength=nleaf)
    assert counts.min() == 0 and counts.max() > 40
    Q = np.zeros((nleaf, counts.max()))
    X = np.repeat(((np.stack(np.unravel_index(np.arange(nleaf), (n, n, n)), 1) + 0.5) / n)[:, None, :],
                  counts.max(), axis=1)
    fill = np.zeros(nleaf, np.int64)
    for k in np.argsort(leaf, kind="stable"):
        b = leaf[k]
        Q[b, fill[b]] = qq[k]
        X[b, fill[b]] = x[k]
        fill[b] += 1
    ref = fmm_oracle.fmm_pass(depth, P, Q, X)
    dev = torch.device("cuda", 0)
    ctx = native.Context(P, "f64")
    tq, tx = torch.as_tensor(qq, device=dev), torch.as_tensor(x, device=dev)
    w = norm_weights(P, "L")
    for prec, tol in ((0, 1e-12), (1, 1e-7)):
        f = fmm.UniformFMM(ctx, depth, prec, dev)
        sq, sx = f.run_particles(tq, tx)
        torch.cuda.synchronize()
        assert rel_err(f.leaf_locals().cpu().numpy(), ref, w) < tol, prec
    # potential of the split pass at every particle
    box = f.leaf_of_sorted()
    pot = torch.zeros(len(x), dtype=torch.float64, device=dev)
    ctx.evaluate(0, len(x), sx, f.leaf_locals(), f.S, nleaf, f.leaf_centres, pot, box=box)
    torch.cuda.synchronize()
    far = pot.cpu().numpy()
    xs, qs, lb = sx.cpu().numpy(), sq.cpu().numpy(), box.cpu().numpy().astype(np.int64)
    off = f.leaf_offsets.cpu().numpy().astype(np.int64)
    ns, nt = fmm.neighbours(depth)
    nbr = [[] for _ in range(nleaf)]
    for a, b in zip(ns.tolist(), nt.tolist()):
        nbr[b].append(a)
    near = np.zeros(len(xs))
    for b in range(nleaf):
        if off[b] == off[b + 1]:
            continue
        src = np.concatenate([np.arange(off[a], off[a + 1]) for a in nbr[b]])
        tgt = np.arange(off[b], off[b + 1])
        r = np.linalg.norm(xs[tgt][:, None, :] - xs[src][None, :, :], axis=2)
        with np.errstate(divide="ignore"):
            near[tgt] = (np.where(r > 0, 1.0 / r, 0.0) * qs[src][None, :]).sum(1)
    r = np.linalg.norm(xs[:, None, :] - xs[None, :, :], axis=2)
    with np.errstate(divide="ignore"):
        direct = (np.where(r > 0, 1.0 / r, 0.0) * qs[None, :]).sum(1)
    assert np.array_equal(lb, leaf[f.order.cpu().numpy()])
    assert np.linalg.norm(far + near - direct) / np.linalg.norm(direct) < 1e-4
