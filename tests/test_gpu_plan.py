"""GPU tests of execution plans (sfmm_plan_*): order-sorted segments replayed
from a CUDA graph give the same targets as direct launches and as the FP64
oracle; stages run in order; replays accumulate; bad plans fail cleanly."""
import numpy as np
import pytest

from helpers import norm_weights, rel_err

pytestmark = pytest.mark.gpu


def _batch(op, Pin, Pout, n, seed, pattern="distinct"):
    import inputs

    rng = np.random.default_rng(seed)
    return inputs.make_batch(rng, op, Pin, Pout, n, nq=16, pattern=pattern)


def _dev(b):
    import torch

    dev = torch.device("cuda", 0)
    t = {k: torch.as_tensor(b[k], device=dev) for k in ("src", "dst", "xyz")}
    for k in ("Pin", "Pout", "sidx", "tidx"):
        t[k] = torch.as_tensor(b[k].astype(np.int32), device=dev)
    return t


def _oracle(oracle, op, b):
    ref = b["dst"].copy()
    oracle.naive(op, b["src"], b["Pin"], ref, b["Pout"], b["xyz"], sidx=b["sidx"], tidx=b["tidx"])
    return ref


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["plain", "split", "split_ff"])
@pytest.mark.parametrize("op", ["m2m", "m2l", "l2l"])
def test_plan_matches_direct_launch(native, op, prec):
    import torch

    ctx = native.Context(20, "f64")
    b = _batch(op, (1, 20), (1, 20), 400, 41)
    t = _dev(b)
    S = b["src"].shape[1]
    n = len(b["Pin"])
    direct = t["dst"].clone()
    ctx.translate_device(op, prec, n, t["src"], S, n, direct, S, n, t["Pin"], t["Pout"], t["xyz"], order_bound=20)
    planned = t["dst"].clone()
    plan = native.Plan(ctx)
    plan.add(op, prec, n, t["src"], S, n, planned, S, n, t["Pin"], t["Pout"], t["xyz"]).finalize()
    plan.run()
    torch.cuda.synchronize()
    segs = plan.segments()
    assert [s[0] for s in segs] == sorted(s[0] for s in segs)
    assert sum(s[1] for s in segs) == n and plan.launches == len(segs) > 1
    g = planned.cpu().numpy() - b["dst"]
    r = direct.cpu().numpy() - b["dst"]
    if prec == 1:
        # split M2M picks its arithmetic by order bound (fixed point up to 18,
        # float-float above): the plan's low-order segments and the direct
        # launch at bound 20 may differ within the 1e-7 contract
        assert rel_err(g, r, norm_weights(20, "M" if op == "m2m" else "L")) < 2e-7
    else:
        # segments of other order bounds may run another group size, whose
        # rotation factors round differently (powers e^{i q gamma} by other
        # products): equal to the arithmetic's rounding level
        assert rel_err(g, r) < (1e-13 if prec == 0 else 1e-11)


def test_plan_against_oracle_repeat_targets(native, oracle):
    import torch

    ctx = native.Context(14, "f64")
    b = _batch("m2l", (2, 14), (2, 14), 300, 43, pattern="repeat")
    ref = _oracle(oracle, "m2l", b)
    t = _dev(b)
    S = b["src"].shape[1]
    n = len(b["Pin"])
    for prec, tol in ((0, 1e-12), (1, 1e-7), (2, 1e-11)):
        d = t["dst"].clone()
        plan = native.Plan(ctx)
        plan.add("m2l", prec, n, t["src"], S, t["src"].shape[0], d, S, d.shape[0], t["Pin"], t["Pout"], t["xyz"],
                 src_index=t["sidx"], dst_index=t["tidx"], repeat=True).finalize()
        plan.run()
        torch.cuda.synchronize()
        assert rel_err(d.cpu().numpy() - b["dst"], ref - b["dst"], norm_weights(14, "L")) < tol, prec


def test_plan_stages_in_order_and_replay_accumulates(native, oracle):
    """Stage 2 (M2L) reads what stage 1 (M2M) wrote; a second run adds the
    whole pass again."""
    import torch

    P = 10
    ctx = native.Context(P, "f64")
    b = _batch("m2m", P, P, 64, 47)
    S = P * (P + 1)
    dev = torch.device("cuda", 0)
    leaves = torch.as_tensor(b["src"], device=dev)
    parents = torch.zeros(8, S, dtype=torch.float64, device=dev)
    locals_ = torch.zeros(8, S, dtype=torch.float64, device=dev)
    orders = torch.full((64,), P, dtype=torch.int32, device=dev)
    tidx = torch.arange(64, dtype=torch.int32, device=dev) // 8
    shift1 = torch.as_tensor(b["xyz"], device=dev)
    rng = np.random.default_rng(5)
    u = rng.normal(size=(8, 3))
    shift2 = torch.as_tensor(u / np.linalg.norm(u, axis=1, keepdims=True) * 3.0, device=dev)
    idx8 = torch.arange(8, dtype=torch.int32, device=dev)
    plan = native.Plan(ctx)
    plan.add("m2m", 0, 64, leaves, S, 64, parents, S, 8, orders, orders, shift1, dst_index=tidx, repeat=True)
    plan.add("m2l", 0, 8, parents, S, 8, locals_, S, 8, orders[:8], orders[:8], shift2, src_index=idx8,
             dst_index=idx8)
    plan.finalize()
    plan.run()
    torch.cuda.synchronize()
    # oracle: the same two steps
    par = np.zeros((8, S))
    oracle.naive("m2m", b["src"], b["Pin"], par, np.full(64, P, np.uint32), b["xyz"],
                 tidx=(np.arange(64) // 8).astype(np.uint32))
    loc = np.zeros((8, S))
    oracle.naive("m2l", par, np.full(8, P, np.uint32), loc, np.full(8, P, np.uint32), shift2.cpu().numpy())
    w = norm_weights(P, "L")
    assert rel_err(locals_.cpu().numpy(), loc, w) < 1e-12
    plan.run()
    torch.cuda.synchronize()
    # second run: parents doubled, locals = first + M2L(2 parents) = 3x
    assert rel_err(parents.cpu().numpy(), 2 * par, norm_weights(P, "M")) < 1e-12
    assert rel_err(locals_.cpu().numpy(), 3 * loc, w) < 1e-12


def test_plan_errors(native):
    import torch

    ctx = native.Context(8, "f64")
    dev = torch.device("cuda", 0)
    S = 72
    src = torch.zeros(4, S, dtype=torch.float64, device=dev)
    dst = torch.zeros(4, S, dtype=torch.float64, device=dev)
    sh = torch.ones(4, 3, dtype=torch.float64, device=dev)
    bad = torch.tensor([8, 9, 8, 8], dtype=torch.int32, device=dev)
    ok = torch.full((4,), 8, dtype=torch.int32, device=dev)
    plan = native.Plan(ctx)
    plan.add("m2l", 0, 4, src, S, 4, dst, S, 4, bad, ok, sh)
    with pytest.raises(native.SfmmError, match="ORDER_RANGE"):
        plan.finalize()
    plan = native.Plan(ctx)
    plan.add("m2l", 0, 4, src, S, 4, dst, S, 4, ok, ok, sh).finalize()
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        plan.add("m2l", 0, 4, src, S, 4, dst, S, 4, ok, ok, sh)
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        native.Plan(ctx).add("m2l", 0, 4, src, 20, 4, dst, S, 4, ok, ok, sh).finalize()


def test_plan_finalize_retried_after_fixing_orders(native, oracle):
    """A finalize that fails on an order above the context's leaves the plan
    unfinalized; after the stage's orders are corrected on the device, a
    second finalize records each translation once and the replay matches the
    oracle."""
    import torch

    P = 10
    ctx = native.Context(P, "f64")
    b = _batch("m2l", (1, P), (1, P), 200, 51)
    t = _dev(b)
    S = b["src"].shape[1]
    n = len(b["Pin"])
    good = t["Pin"].clone()
    t["Pin"][7] = P + 3
    d = t["dst"].clone()
    plan = native.Plan(ctx)
    plan.add("m2l", 0, n, t["src"], S, n, d, S, n, t["Pin"], t["Pout"], t["xyz"])
    with pytest.raises(native.SfmmError, match="ORDER_RANGE"):
        plan.finalize()
    t["Pin"].copy_(good)
    plan.finalize()
    assert sum(s[1] for s in plan.segments()) == n
    plan.run()
    torch.cuda.synchronize()
    ref = _oracle(oracle, "m2l", b)
    assert rel_err(d.cpu().numpy() - b["dst"], ref - b["dst"], norm_weights(P, "L")) < 1e-12


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["plain", "split", "split_ff"])
@pytest.mark.parametrize("op", ["m2m", "m2l", "l2l"])
def test_fused_plan_matches_segmented_plan(native, oracle, op, prec):
    """SFMM_PLAN_FUSED: one persistent launch per stage over a work list of
    order-sorted tiles gives the segmented plan's targets (and the oracle's),
    replay after replay (the work counter is reset inside the graph)."""
    import torch

    ctx = native.Context(24, "f64")
    b = _batch(op, (1, 24), (1, 24), 1500, 45)
    ref = _oracle(oracle, op, b)
    t = _dev(b)
    S = b["src"].shape[1]
    n = len(b["Pin"])
    outs = {}
    w = norm_weights(24, "M" if op == "m2m" else "L")
    for fused in (False, True):
        d = t["dst"].clone()
        plan = native.Plan(ctx).add(op, prec, n, t["src"], S, n, d, S, n, t["Pin"], t["Pout"], t["xyz"],
                                    src_index=t["sidx"], dst_index=t["tidx"]).options(fused=fused).finalize()
        plan.run()
        torch.cuda.synchronize()
        outs[fused] = d.cpu().numpy()
        if fused:
            assert plan.launches == 1
            plan.run()  # a second replay adds the same contribution again
            torch.cuda.synchronize()
            twice = d.cpu().numpy()
            # raw coefficients span ~1e20: compare in the orthonormal basis
            assert rel_err(twice - b["dst"], 2 * (outs[True] - b["dst"]), w) < 1e-12
    assert ctx.device_status() == 0
    tol = {0: 1e-12, 1: 1e-7, 2: 1e-11}[prec]
    assert rel_err(outs[True] - b["dst"], ref - b["dst"], w) < tol
    assert rel_err(outs[True] - b["dst"], outs[False] - b["dst"], w) < (2e-7 if prec == 1 else tol)


def test_fused_tuned_plan_two_stages_repeat_targets(native, oracle):
    """Fused and tuned together: two stages (M2M into shared parents with
    atomics, then M2L), one launch each, with the launch shapes the tuner
    measured at finalize."""
    import torch

    ctx = native.Context(12, "f64")
    b1 = _batch("m2m", (2, 12), (2, 12), 600, 46, pattern="repeat")
    b2 = _batch("m2l", (2, 12), (2, 12), 600, 47)
    t1, t2 = _dev(b1), _dev(b2)
    S = 12 * 13
    n = 600
    ref1 = _oracle(oracle, "m2m", b1)
    d1 = t1["dst"].clone()
    d2 = t2["dst"].clone()
    plan = native.Plan(ctx)
    plan.add("m2m", 0, n, t1["src"], S, n, d1, S, d1.shape[0], t1["Pin"], t1["Pout"], t1["xyz"],
             src_index=t1["sidx"], dst_index=t1["tidx"], repeat=True)
    plan.add("m2l", 0, n, t2["src"], S, n, d2, S, n, t2["Pin"], t2["Pout"], t2["xyz"],
             src_index=t2["sidx"], dst_index=t2["tidx"])
    plan.options(fused=True, tune=True).finalize()
    plan.run()
    torch.cuda.synchronize()
    assert plan.launches == 2 and ctx.device_status() == 0
    assert rel_err(d1.cpu().numpy() - b1["dst"], ref1 - b1["dst"]) < 1e-12
    ref2 = _oracle(oracle, "m2l", b2)
    assert rel_err(d2.cpu().numpy() - b2["dst"], ref2 - b2["dst"]) < 1e-12


def test_plan_options_after_finalize_rejected(native):
    import torch

    ctx = native.Context(6, "f64")
    b = _batch("m2l", 6, 6, 50, 48)
    t = _dev(b)
    plan = native.Plan(ctx).add("m2l", 0, 50, t["src"], 42, 50, t["dst"], 42, 50, t["Pin"], t["Pout"],
                                t["xyz"]).finalize()
    with pytest.raises(native.SfmmError):
        plan.options(fused=True)
    torch.cuda.synchronize()
