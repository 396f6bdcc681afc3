"""GPU checks at the reference's own physics geometries (tests/test_m2l.cpp:
57-136, test_m2m.cpp:55-134, test_l2l.cpp:54-111): a unit source is
expanded, translated 32 times into one target through the C ABI, and the
target is evaluated against 1/r and its gradient.  The expansion's own
truncation error is what the oracle's exact (naive O(P^4)) translation gives;
each precision mode may add at most its arithmetic error to it:

  potential error |e_mode - e_exact| (relative potential, the r|phi - 1/r|
  units the reference prints):
    plain FP64 1e-13, split_ff 1e-11, split 2e-7, 3xTF32 5e-6,
    BF16x6 3e-6, 3xBF16 3e-4,
and the plain FP64 path reproduces the reference's double result where the
reference library was built (within 1e-9 relative of its printed error).
"""
import numpy as np
import pytest

from helpers import norm_weights, physics_errors, physics_gpu, physics_inputs, physics_reference, rel_err

pytestmark = pytest.mark.gpu

TOL = {0: 1e-13, 2: 1e-11, 1: 2e-7, 3: 5e-6, 5: 3e-6, 4: 3e-4}


@pytest.fixture(scope="module")
def ctx16(native):
    return native.Context(16, "f64")


def _exact(oracle, op, P):
    E, shift = physics_inputs(op, P)
    S = P * (P + 1)
    out = np.zeros((1, S))
    pn = np.full(1, P, np.uint32)
    oracle.naive(op, E.reshape(1, S), pn, out, pn, shift.reshape(1, 3))
    return physics_errors(op, P, out[0])


@pytest.mark.parametrize("P", [8, 16])
@pytest.mark.parametrize("op", ["m2l", "m2m", "l2l"])
def test_physics_every_mode(ctx16, oracle, op, P):
    ex_pot, ex_grad = _exact(oracle, op, P)
    for prec, tol in TOL.items():
        pot, grad = physics_gpu(ctx16, op, P, prec)
        assert abs(pot - ex_pot) <= tol, (prec, pot, ex_pot)
        assert abs(grad - ex_grad) <= max(10 * tol, 1e-8), (prec, grad, ex_grad)


@pytest.mark.parametrize("op", ["m2l", "m2m", "l2l"])
def test_physics_plain_matches_reference_double(ctx16, oracle, op):
    ref = physics_reference(op, 16)
    if ref is None:
        pytest.skip("reference library not built on this machine")
    pot, _ = physics_gpu(ctx16, op, 16, 0)
    assert abs(pot - ref[0]) <= 1e-9 * ref[0] + 1e-14, (pot, ref)


def norm_weights_for(op, P):
    return norm_weights(P, "M" if op == "m2m" else "L")


SCALE_TOL = {0: 1e-12, 1: 1e-7, 2: 1e-11, 3: 4e-6, 5: 1.5e-6, 4: 2e-4}


def _scaled_batch(oracle, op, P, n, scale):
    """Sources of the tree shape at one length scale, their shifts, the FP64
    oracle's translation and the per-coefficient factors back to unit scale
    (s^-n for multipole results, s^(n+1) for local results)."""
    rng = np.random.default_rng(5)
    q = rng.choice([-1.0, 1.0], size=(n, 12))
    d = rng.normal(size=(n, 12, 3))
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    if op == "l2l":  # locals of far charges
        src = oracle.p2m(P, q, (d * 0.4 + np.array([3.0, 0.5, -1.0])) * scale, np.zeros((n, 3)), singular=True)
    else:
        src = oracle.p2m(P, q, d * 0.4 * rng.random((n, 12, 1)) * scale, np.zeros((n, 3)))
    u = rng.normal(size=(n, 3))
    xyz = u / np.linalg.norm(u, axis=1, keepdims=True) * (3.0 if op == "m2l" else 0.5) * scale
    pin = np.full(n, P, np.uint32)
    ref = np.zeros((n, P * (P + 1)))
    oracle.naive(op, src, pin, ref, pin, xyz)
    deg = np.array([k for k in range(P) for _ in range(2 * k + 2)], dtype=np.float64)
    unit = np.exp(np.log(scale) * (-deg if op == "m2m" else deg + 1))
    return src, xyz, pin, ref, unit


@pytest.mark.parametrize("op", ["m2l", "m2m", "l2l"])
def test_fp32_context_at_length_scales_its_storage_holds(native, oracle, op):
    """The FP32 kernel (an SFMM_F32 context: FP32 expansions) runs every
    translation at the length scale of its shift too; at scales whose
    coefficients FP32 storage still holds (P=16: 1/8 ... 8) its error stays
    the unit-scale one."""
    import torch

    dev = torch.device("cuda", 0)
    P, n = 16, 48
    S = P * (P + 1)
    ctx = native.Context(P, "f32")
    w = norm_weights_for(op, P)
    for scale in (0.125, 0.5, 1.0, 2.0, 8.0):
        src, xyz, pin, ref, unit = _scaled_batch(oracle, op, P, n, scale)
        t_pin = torch.as_tensor(pin.astype(np.int32), device=dev)
        out = torch.zeros(n, S, dtype=torch.float32, device=dev)
        ctx.translate_device(op, 0, n, torch.as_tensor(src, dtype=torch.float32, device=dev), S, n, out, S, n,
                             t_pin, t_pin, torch.as_tensor(xyz, device=dev), order_bound=P)
        got = out.double().cpu().numpy()
        assert np.isfinite(got).all(), (op, scale)
        err = rel_err(got * unit, ref * unit, w)
        assert err <= 2e-6, (op, scale, err)


@pytest.mark.parametrize("op", ["m2l", "m2m", "l2l"])
def test_every_mode_at_every_length_scale(ctx16, oracle, native, op):
    """The same tree shape at length scales 1e-9 ... 1e9: translations are
    homogeneous (multipole degree n scales as s^n, local degree n as
    s^-(n+1)), so every precision mode keeps its accuracy at every scale,
    although the coefficients span far more than the FP32 range.  Errors are
    measured after bringing both results back to unit scale degree by degree
    (the norms stay finite) in the orthonormal basis."""
    import torch

    dev = torch.device("cuda", 0)
    P, n = 16, 48
    S = P * (P + 1)
    w = norm_weights_for(op, P)
    for scale in (1e-9, 1e-4, 1e-2, 1.0, 1e2, 1e4, 1e9):
        src, xyz, pin, ref, unit = _scaled_batch(oracle, op, P, n, scale)
        t_pin = torch.as_tensor(pin.astype(np.int32), device=dev)
        t_src = torch.as_tensor(src, device=dev)
        t_xyz = torch.as_tensor(xyz, device=dev)
        for prec, tol in SCALE_TOL.items():
            out = torch.zeros(n, S, dtype=torch.float64, device=dev)
            ctx16.translate_device(op, prec, n, t_src, S, n, out, S, n, t_pin, t_pin, t_xyz, order_bound=P)
            got = out.cpu().numpy()
            assert np.isfinite(got).all(), (op, scale, prec)
            err = rel_err(got * unit, ref * unit, w)
            assert err <= tol, (op, scale, prec, err)
