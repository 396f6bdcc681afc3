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


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-7), (2, 1e-11)], ids=["plain", "split", "split_ff"])
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
