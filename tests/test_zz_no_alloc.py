"""The allocation-free bucketing entry point, sfmm_bucket_by_order_noalloc.

Some callers cannot allocate device memory: a code that has handed the whole
GPU to its own memory pool, a process under a hard device-memory cap, or a
hot loop where an allocation would stall.  Such callers cannot create a
context either, so this entry point takes only device arrays and a stream
and keeps its counters in a fixed device array inside the library.

The test calls it through the C ABI twice in a row (the shared counters must
be cleared by each call) and checks it against the context-based
sfmm_bucket_by_order: both must return a permutation with the same sequence
of (p_in, p_out) keys (the order inside a group of equal keys is unspecified).
This file sorts last so that a run stopping at the first failure has run
every other test already; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _keys(pin, pout, order):
    return pin[order].astype(np.int64) * 1000 + pout[order]


@pytest.mark.parametrize("max_order,n,seed", [(24, 5000, 1), (86, 777, 2)])
def test_noalloc_bucketing_matches_context_bucketing(native, max_order, n, seed):
    import torch

    L = native.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(seed)
    stream = torch.cuda.current_stream(dev)
    ctx = native.Context(max_order, "f64")
    for call in range(2):  # two calls in a row share the same device counters
        pin = rng.integers(0, max_order + 1, n).astype(np.uint32)
        pout = rng.integers(0, max_order + 1, n).astype(np.uint32)
        d_pin = torch.as_tensor(pin.astype(np.int32), device=dev)
        d_pout = torch.as_tensor(pout.astype(np.int32), device=dev)
        got = torch.full((n,), -1, dtype=torch.int32, device=dev)
        rc = L.sfmm_bucket_by_order_noalloc(n, d_pin.data_ptr(), d_pout.data_ptr(), got.data_ptr(), max_order,
                                            C.c_void_p(stream.cuda_stream))
        assert rc == 0
        want = torch.full((n,), -1, dtype=torch.int32, device=dev)
        ctx.set_stream(stream.cuda_stream)
        ctx.bucket(n, d_pin, d_pout, want)
        torch.cuda.synchronize()
        g = got.cpu().numpy()
        w = want.cpu().numpy()
        assert sorted(g.tolist()) == list(range(n)), f"call {call}: not a permutation"
        assert np.array_equal(_keys(pin, pout, g), _keys(pin, pout, w)), f"call {call}: key sequence differs"


def test_noalloc_bucketing_rejects_orders_above_limit(native):
    L = native.load()
    assert L.sfmm_bucket_by_order_noalloc(10, None, None, None, 87, None) == 2  # SFMM_ORDER_RANGE
