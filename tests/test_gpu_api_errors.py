"""Argument checking of the C ABI's newer entry points on a GPU context:
evaluation, tuning and plans report errors through their status codes and
leave their outputs untouched; empty plans run and launch nothing."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx8(native):
    return native.Context(8, "f64")


def test_eval_errors(native, ctx8):
    import torch

    dev = torch.device("cuda", 0)
    S = 72
    pts = torch.zeros(4, 3, dtype=torch.float64, device=dev)
    E = torch.zeros(4, S, dtype=torch.float64, device=dev)
    cen = torch.zeros(4, 3, dtype=torch.float64, device=dev)
    pot = torch.zeros(4, dtype=torch.float64, device=dev)
    grad = torch.zeros(4, 3, dtype=torch.float64, device=dev)
    with pytest.raises(native.SfmmError, match="UNSUPPORTED"):
        ctx8.evaluate(1, 4, pts, E, S, 4, cen, pot, gradient=grad)
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        ctx8.evaluate(0, 4, pts, E, S - 1, 4, cen, pot)
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        ctx8.evaluate(0, 4, pts, E, S, 3, cen, pot)          # fewer expansions than points, no box index
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        ctx8.evaluate(2, 4, pts, E, S, 4, cen, pot)
    ctx8.evaluate(0, 0, pts, E, S, 4, cen, pot)                # nothing to do
    torch.cuda.synchronize()
    assert float(pot.abs().sum()) == 0.0


def test_tune_and_group_errors(native, ctx8):
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        ctx8.tune("m2l", 0, n=0)
    with pytest.raises(native.SfmmError, match="ORDER_RANGE"):
        ctx8.tune("m2l", 0, n=1024, order_bound=9)
    with pytest.raises(native.SfmmError, match="INVALID_ARG"):
        ctx8.tune(7, 0, n=1024)
    with pytest.raises(native.SfmmError, match="ORDER_RANGE"):
        ctx8.set_group(0, 4, order_bound=9)
    f32 = native.Context(8, "f32")
    with pytest.raises(native.SfmmError, match="UNSUPPORTED"):
        f32.tune("m2l", 1, n=1024)
    g, rate = ctx8.tune("l2l", 0, n=4096)
    assert g in (4, 8) and rate > 0


def test_empty_plan_and_empty_stage(native, ctx8):
    import torch

    dev = torch.device("cuda", 0)
    plan = native.Plan(ctx8).finalize()
    plan.run()
    assert plan.launches == 0 and plan.segments() == []
    S = 72
    src = torch.ones(2, S, dtype=torch.float64, device=dev)
    dst = torch.zeros(2, S, dtype=torch.float64, device=dev)
    o = torch.full((2,), 8, dtype=torch.int32, device=dev)
    sh = torch.ones(2, 3, dtype=torch.float64, device=dev)
    plan = native.Plan(ctx8)
    plan.add("m2l", 0, 0, src, S, 2, dst, S, 2, o, o, sh)        # empty stage
    plan.add("m2l", 0, 2, src, S, 2, dst, S, 2, o, o, sh)
    plan.finalize()
    plan.run()
    torch.cuda.synchronize()
    assert plan.launches == 1
    assert float(dst.abs().sum()) > 0


def test_host_packed_zero_orders(native, ctx8):
    """Zero orders on the in-place host path: nothing is added to the target."""
    rng = np.random.default_rng(2)
    n, S = 64, 72
    src = rng.normal(size=(n, S))
    dst = rng.normal(size=(n, S))
    before = dst.copy()
    pin = np.zeros(n, np.uint32)
    pout = np.full(n, 8, np.uint32)
    xyz = rng.normal(size=(n, 3)) + 3
    ctx8.translate_host_packed("m2l", 0, src, dst, pin, pout, xyz)
    assert np.array_equal(dst, before)


def test_concurrent_device_calls_share_a_context(native):
    """Device calls from several host threads on one context, each at an
    order bound not used before (first use uploads tables and builds the
    launch shape): every thread's result equals a sequential run."""
    import threading

    import torch

    dev = torch.device("cuda", 0)
    P = 20
    ctx = native.Context(P, "f64")
    S = P * (P + 1)
    rng = np.random.default_rng(9)
    jobs = []
    for k, (bound, prec) in enumerate([(6, 0), (9, 1), (12, 2), (15, 1), (18, 0), (20, 2)]):
        n = 500
        src = torch.as_tensor(rng.normal(size=(n, S)) * 1e-2, device=dev)
        o = torch.full((n,), bound, dtype=torch.int32, device=dev)
        u = rng.normal(size=(n, 3))
        sh = torch.as_tensor(u / np.linalg.norm(u, axis=1, keepdims=True) * 3.0, device=dev)
        jobs.append((bound, prec, n, src, o, sh))
    out = [None] * len(jobs)

    def work(i):
        bound, prec, n, src, o, sh = jobs[i]
        st = torch.cuda.Stream(dev)
        with torch.cuda.stream(st):
            d = torch.zeros(n, S, dtype=torch.float64, device=dev)
            st.synchronize()
            ctx.translate_device("m2l", prec, n, src, S, n, d, S, n, o, o, sh, order_bound=bound)
            torch.cuda.synchronize()
            out[i] = d.cpu().numpy()

    th = [threading.Thread(target=work, args=(i,)) for i in range(len(jobs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, (bound, prec, n, src, o, sh) in enumerate(jobs):
        d = torch.zeros(n, S, dtype=torch.float64, device=dev)
        ctx.translate_device("m2l", prec, n, src, S, n, d, S, n, o, o, sh, order_bound=bound)
        torch.cuda.synchronize()
        assert np.array_equal(out[i], d.cpu().numpy()), bound


def test_device_allocation_failure_leaves_context_usable(native, oracle):
    """A device allocation that cannot succeed (a tuning sample of 2^24
    translations at P=86, about 1 TB) returns OOM; after each such failure
    the same context still launches its kernels (P2M, bucketing, a
    translation) and the result matches the oracle: the failed allocation's
    error is not reported by a later launch."""
    import torch

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import inputs
    from helpers import norm_weights, rel_err, run_device

    dev = torch.device("cuda", 0)
    ctx = native.Context(86, "f64")

    def oom():
        with pytest.raises(native.SfmmError, match="OOM"):
            ctx.tune("m2l", 0, n=1 << 24)

    oom()
    q = torch.ones(1, 4, dtype=torch.float64, device=dev)
    pos = torch.full((1, 4, 3), 0.1, dtype=torch.float64, device=dev)
    out = torch.zeros(1, 86 * 87, dtype=torch.float64, device=dev)
    ctx.p2x(0, 1, 4, q, pos, torch.zeros(1, 3, dtype=torch.float64, device=dev), out, 86 * 87)
    torch.cuda.synchronize()
    assert float(out[0, 0]) == 4.0  # R_0^0 = 1 per unit charge
    oom()
    o = torch.tensor([3, 1, 3, 2], dtype=torch.int32, device=dev)
    perm = torch.zeros(4, dtype=torch.int32, device=dev)
    ctx.bucket(4, o, o, perm)
    torch.cuda.synchronize()
    assert sorted(perm.cpu().tolist()) == [0, 1, 2, 3]
    oom()
    b = inputs.make_batch(np.random.default_rng(4), "m2l", 12, 12, 64, nq=16)
    ref = b["dst"].copy()
    oracle.naive("m2l", b["src"], b["Pin"], ref, b["Pout"], b["xyz"])
    got = run_device(ctx, "m2l", 0, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], order_bound=12)
    assert rel_err(got - b["dst"], ref - b["dst"], norm_weights(12, "L")) < 1e-12
