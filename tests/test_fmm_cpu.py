"""CPU checks of the uniform-octree FMM driver's index arithmetic
(solidfmm_gb300.fmm): interaction lists are symmetric, well separated, at
most 189 per box, equal to the oracle's independent lists, and together
with the leaf neighbours they cover every pair of leaves exactly once."""
import itertools
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
torch = pytest.importorskip("torch")

from solidfmm_gb300 import fmm  # noqa: E402


@pytest.mark.parametrize("level", [2, 3, 4])
def test_interaction_lists(level):
    s, t = fmm.interaction_list(level)
    n = 2 ** level
    cnt = torch.bincount(t, minlength=n ** 3)
    assert int(cnt.max()) == (189 if level >= 3 else int(cnt.max()))
    c = fmm.box_coords(level)
    d = (c[s] - c[t]).abs().amax(1)
    assert bool((d >= 2).all()) and bool((d <= 3).all())
    pairs = set(zip(s.tolist(), t.tolist()))
    assert pairs == set((b, a) for a, b in pairs)
    pc = c // 2
    assert bool(((pc[s] - pc[t]).abs().amax(1) <= 1).all())


def test_lists_cover_every_leaf_pair_once():
    depth = 3
    nleaf = 8 ** depth
    cover = np.zeros((nleaf, nleaf), np.int32)
    ns, nt = fmm.neighbours(depth)
    np.add.at(cover, (nt.numpy(), ns.numpy()), 1)
    cl = fmm.box_coords(depth).numpy()
    for l in range(2, depth + 1):
        s, t = fmm.interaction_list(l)
        # every leaf under target box t receives from every leaf under s
        anc = ((cl[:, 0] >> (depth - l)) * 2 ** l + (cl[:, 1] >> (depth - l))) * 2 ** l + (cl[:, 2] >> (depth - l))
        members = [np.nonzero(anc == b)[0] for b in range(8 ** l)]
        for a, b in zip(s.tolist(), t.tolist()):
            cover[np.ix_(members[b], members[a])] += 1
    assert cover.min() == 1 and cover.max() == 1


def test_oracle_lists_agree_and_stage_counts():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    depth = 3
    st = fmm.pass_stages(depth)
    ops = [x.op for x in st]
    assert ops == ["m2m"] * (depth - 2) + ["m2l"] + ["l2l"] * (depth - 2)
    m2l = st[depth - 2]
    off = fmm.level_offsets(depth)
    got = set(zip(m2l.src_index.tolist(), m2l.dst_index.tolist()))
    want = set()
    for l in range(2, depth + 1):
        nl = 2 ** l
        for i, j, k in itertools.product(range(nl), repeat=3):
            for a, b, c in itertools.product(range(nl), repeat=3):
                if max(abs(a - i), abs(b - j), abs(c - k)) >= 2 and \
                        max(abs(a // 2 - i // 2), abs(b // 2 - j // 2), abs(c // 2 - k // 2)) <= 1:
                    want.add((off[l] + (a * nl + b) * nl + c, off[l] + (i * nl + j) * nl + k))
    assert got == want
    # shifts are target centre - source centre
    cen = np.concatenate([fmm.box_centres(l).numpy() for l in range(depth + 1)])
    assert np.allclose(m2l.shift.numpy(), cen[m2l.dst_index.numpy()] - cen[m2l.src_index.numpy()])
    for x in st:
        if x.op != "m2l":
            assert np.allclose(x.shift.numpy(), cen[x.dst_index.numpy()] - cen[x.src_index.numpy()])


def test_bin_particles_sorts_stably_by_leaf():
    """Every particle lands in the leaf floor(x 2^depth) (the face x = 1 in
    the last box), leaves come in index order, particles of one leaf keep
    their input order, the offsets count them, and empty leaves are empty
    ranges; positions outside the unit cube are refused."""
    depth = 3
    n = 2 ** depth
    g = torch.Generator().manual_seed(4)
    # clustered particles (two blobs) plus points on faces and corners
    blobs = torch.cat([0.2 + 0.05 * torch.randn(700, 3, generator=g, dtype=torch.float64),
                       0.7 + 0.1 * torch.randn(300, 3, generator=g, dtype=torch.float64)]).clamp(0, 1)
    faces = torch.tensor([[1.0, 1.0, 1.0], [0.0, 0.0, 0.0], [0.5, 1.0, 0.125], [0.125, 0.0, 1.0]],
                         dtype=torch.float64)
    pos = torch.cat([blobs, faces])
    order, off = fmm.bin_particles(pos, depth)
    assert off.dtype == torch.int32 and len(off) == n ** 3 + 1 and int(off[-1]) == len(pos)
    x = pos.numpy()
    ijk = np.minimum(np.floor(x * n).astype(np.int64), n - 1)
    leaf = (ijk[:, 0] * n + ijk[:, 1]) * n + ijk[:, 2]
    want = np.argsort(leaf, kind="stable")
    assert np.array_equal(order.numpy(), want)
    counts = np.bincount(leaf, minlength=n ** 3)
    assert np.array_equal(np.diff(off.numpy()), counts)
    assert (counts == 0).sum() > 0  # the clustered set leaves boxes empty
    assert int(leaf[len(blobs)]) == n ** 3 - 1 and int(leaf[len(blobs) + 1]) == 0
    with pytest.raises(ValueError):
        fmm.bin_particles(torch.tensor([[0.5, 0.5, 1.5]], dtype=torch.float64), depth)
    with pytest.raises(ValueError):
        fmm.bin_particles(torch.tensor([[-1e-9, 0.5, 0.5]], dtype=torch.float64), depth)
