"""GPU tests of the tensor-core translation kernel (precision modes
SFMM_TC_TF32 = 3, SFMM_TC_BF16 = 4, SFMM_TC_BF16X6 = 5): the reference's golden outputs, the
FP64 naive oracle on mixed orders, repeated targets, permutations and index
arrays, malformed entries, zero shifts, the host-memory calls, plans, and
the routing of order bounds above 16 to the split kernel.

Tolerances (relative L2 per target expansion in the orthonormal basis, max
over the batch), from the operand precision of the split products:
  * 3xTF32 (two TF32 pieces, ~22 bits per operand, FP32 accumulation):
    4e-6 (measured up to 1.4e-6, L2L at P=16);
  * 3xBF16 (two BF16 pieces, ~16 bits per operand): 2e-4 (measured up to
    6e-5, M2M at P=16);
  * BF16x6 (three BF16 pieces, float-float edges): 1.5e-6 (measured up to
    5e-7 on 1 000 translations, 6.2e-7 over 2e6 M2L at P=16: the FP32
    accumulation in tensor memory rounds once per MMA stage).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_golden, norm_weights, per_degree_err, rel_err, rel_err_dev, run_device

pytestmark = pytest.mark.gpu

TC = {"tf32": 3, "bf16": 4, "bf16x6": 5}
TOL = {3: 4e-6, 4: 2e-4, 5: 1.5e-6}
CASES = load_golden()


def _batch(op, Pin, Pout, n, seed, pattern="distinct", in_le_out=False, zero_shift=False):
    import inputs

    rng = np.random.default_rng(seed)
    return inputs.make_batch(rng, op, Pin, Pout, n, nq=16, pattern=pattern, in_le_out=in_le_out,
                             zero_shift=zero_shift)


def _oracle(oracle, op, b):
    ref = b["dst"].copy()
    oracle.naive(op, b["src"], b["Pin"], ref, b["Pout"], b["xyz"], sidx=b["sidx"], tidx=b["tidx"])
    return ref


def _w(P, op):
    return norm_weights(P, "M" if op == "m2m" else "L")


@pytest.fixture(scope="module")
def ctx16(native):
    return native.Context(16, "f64")


def _golden_names():
    return sorted(k for k in CASES if "_f64_" in k and int(CASES[k]["Pop"]) <= 16)


@pytest.mark.parametrize("name", _golden_names())
@pytest.mark.parametrize("mode", sorted(TC), ids=sorted(TC))
def test_tc_golden_f64(ctx16, name, mode):
    c = CASES[name]
    op = str(c["op"])
    prec = TC[mode]
    repeat = len(np.unique(c["tidx"])) < len(c["tidx"])
    got = run_device(ctx16, op, prec, c["src"], c["dst0"], c["Pin"], c["Pout"], c["xyz"], c["sidx"], c["tidx"],
                     repeat=repeat, order_bound=int(c["Pop"]))
    err = rel_err(got - c["dst0"], c["dst"] - c["dst0"], _w(int(c["Pop"]), op))
    assert err < TOL[prec], f"{name}: {err:.3e}"


@pytest.mark.parametrize("op", ["m2m", "m2l", "l2l"])
@pytest.mark.parametrize("mode", sorted(TC), ids=sorted(TC))
def test_tc_mixed_orders_vs_oracle(native, ctx16, oracle, op, mode):
    b = _batch(op, (1, 16), (1, 16), 700, 41, in_le_out=(op == "l2l"))
    ref = _oracle(oracle, op, b)
    got = run_device(ctx16, op, TC[mode], b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"],
                     order_bound=16)
    err = rel_err(got - b["dst"], ref - b["dst"], _w(16, op))
    assert err < TOL[TC[mode]], err


@pytest.mark.parametrize("P", [1, 2, 5, 9, 16])
def test_tc_every_order_bound(native, oracle, P):
    """Uniform orders at several bounds (odd and even pairings of degrees and
    z-columns), on a context whose order is above the bound."""
    ctx = native.Context(20, "f64")
    for op in ("m2m", "m2l", "l2l"):
        b = _batch(op, P, P, 300, 50 + P)
        ref = _oracle(oracle, op, b)
        got = run_device(ctx, op, 3, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"],
                         order_bound=P)
        assert rel_err(got - b["dst"], ref - b["dst"], _w(P, op)) < TOL[3], (op, P)


@pytest.mark.parametrize("op", ["m2m", "m2l", "l2l"])
def test_tc_repeated_targets(native, ctx16, oracle, op):
    """Targets shared by many translations accumulate with FP64 atomics."""
    b = _batch(op, 12, 12, 900, 43, pattern="repeat")
    ref = _oracle(oracle, op, b)
    got = run_device(ctx16, op, 3, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"],
                     repeat=True, order_bound=12)
    assert rel_err(got - b["dst"], ref - b["dst"], _w(12, op)) < TOL[3]


def test_tc_permutation_is_bit_identical(native, ctx16):
    """A processing order (sfmm_translate_device's `order`) moves
    translations between tiles and threads without changing any result."""
    b = _batch("m2l", (1, 16), (1, 16), 1000, 44)
    a = run_device(ctx16, "m2l", 4, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"],
                   order_bound=16)
    perm = np.random.default_rng(5).permutation(len(b["Pin"])).astype(np.uint32)
    p = run_device(ctx16, "m2l", 4, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"],
                   order=perm, order_bound=16)
    assert np.array_equal(a, p)


@pytest.mark.parametrize("op", ["m2m", "l2l"])
def test_tc_zero_shift_is_prefix_add(native, ctx16, oracle, op):
    b = _batch(op, (1, 16), (1, 16), 200, 45, zero_shift=True)
    ref = _oracle(oracle, op, b)
    got = run_device(ctx16, op, 3, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"],
                     order_bound=16)
    zero = b["tidx"][::2]  # every other translation has a zero shift: an exact FP64 prefix add
    assert rel_err(got[zero] - b["dst"][zero], ref[zero] - b["dst"][zero]) < 1e-15
    assert rel_err(got - b["dst"], ref - b["dst"], _w(16, op)) < TOL[3]


def test_tc_malformed_entries_are_skipped_and_flagged(native, ctx16, oracle):
    import torch

    b = _batch("m2l", 8, 8, 300, 46)
    ref = _oracle(oracle, "m2l", b)
    tidx = b["tidx"].copy()
    pin = b["Pin"].copy()
    tidx[5] = 10 ** 6  # target out of range
    pin[9] = 12        # order above the bound
    dev = torch.device("cuda", 0)
    s = torch.as_tensor(b["src"], device=dev)
    d = torch.as_tensor(b["dst"].copy(), device=dev)
    i32 = lambda a: torch.as_tensor(np.asarray(a, np.uint32).astype(np.int32), device=dev)  # noqa: E731
    ctx16.translate_device("m2l", 3, len(pin), s, s.shape[1], s.shape[0], d, d.shape[1], d.shape[0], i32(pin),
                           i32(b["Pout"]), torch.as_tensor(b["xyz"], device=dev), src_index=i32(b["sidx"]),
                           dst_index=i32(tidx), order_bound=8)
    assert ctx16.device_status() & 1
    got = d.cpu().numpy()
    keep = np.ones(len(pin), bool)
    keep[[5, 9]] = False
    rows = b["tidx"][keep]
    w = _w(8, "m2l")
    assert rel_err(got[rows] - b["dst"][rows], ref[rows] - b["dst"][rows], w) < TOL[3]
    assert np.array_equal(got[b["tidx"][9]], b["dst"][b["tidx"][9]])  # the skipped entry touched nothing


def test_tc_order_bound_above_16_runs_split(native, oracle):
    """Order bounds above the tensor-core kernel's 16 run the split kernel
    (its 1e-7 contract holds)."""
    ctx = native.Context(24, "f64")
    b = _batch("m2l", (1, 24), (1, 24), 300, 47)
    ref = _oracle(oracle, "m2l", b)
    got = run_device(ctx, "m2l", 3, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"],
                     order_bound=24)
    assert rel_err(got - b["dst"], ref - b["dst"], _w(24, "m2l")) < 1e-7


def test_tc_per_degree_error(native, ctx16, oracle):
    """Per-degree error of both modes at M2L P=16 with the benchmark geometry
    (the FP32-class limit of the split products), and 3xTF32 at least 10x
    more accurate than 3xBF16 on the whole expansion."""
    b = _batch("m2l", 16, 16, 1000, 48)
    ref = _oracle(oracle, "m2l", b)
    w = _w(16, "m2l")
    errs = {}
    for mode, prec in TC.items():
        got = run_device(ctx16, "m2l", prec, b["src"], b["dst"], b["Pin"], b["Pout"], b["xyz"], b["sidx"], b["tidx"])
        pd = per_degree_err(got - b["dst"], ref - b["dst"], 16, w)
        assert max(pd) < 10 * TOL[prec], (mode, pd)
        errs[mode] = rel_err(got - b["dst"], ref - b["dst"], w)
    assert errs["tf32"] * 10 < errs["bf16"], errs


def test_tc_host_calls(native, oracle):
    """The host-memory calls with tensor-core precision: the packed call and
    the classic call over separate solids (the kernel reads and updates them
    in place)."""
    import torch

    ctx = native.Context(12, "f64")
    b = _batch("m2l", 12, 12, 1500, 49)
    ref = _oracle(oracle, "m2l", b)
    w = _w(12, "m2l")
    src = torch.as_tensor(b["src"]).pin_memory()
    dst = torch.as_tensor(b["dst"].copy()).pin_memory()
    ctx.translate_host_packed("m2l", 3, src, dst, b["Pin"], b["Pout"], b["xyz"], src_index=b["sidx"],
                              dst_index=b["tidx"])
    assert rel_err(dst.numpy() - b["dst"], ref - b["dst"], w) < TOL[3]
    L = native.load()
    n = len(b["Pin"])
    S = b["src"].shape[1]
    dst2 = b["dst"].copy()
    sa = (np.uint64(b["src"].ctypes.data) + b["sidx"].astype(np.uint64) * np.uint64(8 * S)).astype(np.uint64)
    da = (np.uint64(dst2.ctypes.data) + b["tidx"].astype(np.uint64) * np.uint64(8 * S)).astype(np.uint64)
    pi = b["Pin"].astype(np.uint64)
    po = b["Pout"].astype(np.uint64)
    xs, ys, zs = (np.ascontiguousarray(b["xyz"][:, k]) for k in range(3))
    L.sfmm_translate_host.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p]
    rc = L.sfmm_translate_host(ctx.h, 1, 3, n, sa.ctypes.data, pi.ctypes.data, da.ctypes.data, po.ctypes.data, 1,
                               xs.ctypes.data, ys.ctypes.data, zs.ctypes.data)
    assert rc == 0, L.sfmm_last_error(ctx.h)
    assert rel_err(dst2 - b["dst"], ref - b["dst"], w) < TOL[3]


def test_tc_plan_mixed_orders(native, oracle):
    """An execution plan in tensor-core precision over orders 1..20: segments
    up to 16 run the tensor-core kernel, the rest the split kernel."""
    import torch

    ctx = native.Context(20, "f64")
    dev = torch.device("cuda", 0)
    b = _batch("m2l", (1, 20), (1, 20), 1200, 51)
    ref = _oracle(oracle, "m2l", b)
    t = lambda a, dt=torch.float64: torch.as_tensor(a, dtype=dt, device=dev)  # noqa: E731
    i32 = lambda a: t(np.asarray(a, np.uint32).astype(np.int32), torch.int32)  # noqa: E731
    s, d = t(b["src"]), t(b["dst"].copy())
    plan = native.Plan(ctx).add("m2l", 3, len(b["Pin"]), s, s.shape[1], s.shape[0], d, d.shape[1], d.shape[0],
                                i32(b["Pin"]), i32(b["Pout"]), t(b["xyz"]), src_index=i32(b["sidx"]),
                                dst_index=i32(b["tidx"])).finalize()
    plan.run()
    torch.cuda.synchronize()
    assert ctx.device_status() == 0
    assert rel_err(d.cpu().numpy() - b["dst"], ref - b["dst"], _w(20, "m2l")) < TOL[3]


def test_tc_large_batch_against_plain(native, ctx16):
    """262 144 M2L translations at P=16 (the benchmark's geometry): every
    translation within the 3xTF32 tolerance of plain FP64."""
    import torch

    from helpers import device_batch

    dev = torch.device("cuda", 0)
    N, P = 262_144, 16
    S = P * (P + 1)
    src, shift = device_batch(ctx16, "m2l", P, N, 64, 52, dev)
    pin = torch.full((N,), P, dtype=torch.int32, device=dev)
    outs = {}
    for prec in (0, 3):
        d = torch.zeros(N, S, dtype=torch.float64, device=dev)
        ctx16.translate_device("m2l", prec, N, src, S, N, d, S, N, pin, pin, shift)
        torch.cuda.synchronize()
        outs[prec] = d
    assert ctx16.device_status() == 0
    assert rel_err_dev(outs[3], outs[0], _w(16, "m2l")) < TOL[3]
