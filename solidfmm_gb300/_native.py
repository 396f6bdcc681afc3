"""ctypes binding of the C ABI (include/sfmm.h) in libsfmm_gb300.so.

The library is the product: there is no Python or CPU implementation of the
translations behind this module.  Loading fails loudly if the library has not
been built (python -m solidfmm_gb300.build).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

F32, F64 = 0, 1
M2M, M2L, L2L = 0, 1, 2
PLAIN, SPLIT, SPLIT_FF, TC_TF32, TC_BF16, TC_BF16X6 = 0, 1, 2, 3, 4, 5
TARGETS_UNIQUE, TARGETS_REPEAT, TARGETS_ON_DEVICE = 0, 1, 2
PLAN_FUSED, PLAN_TUNE = 1, 2
OPS = {"m2m": M2M, "m2l": M2L, "l2l": L2L}

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "ORDER_RANGE", 3: "OVERFLOW", 4: "DIM_MISMATCH", 5: "OOM",
          6: "CUDA_ERROR", 7: "UNSUPPORTED"}

EXPORTS = [
    "sfmm_create", "sfmm_destroy", "sfmm_order", "sfmm_data_type", "sfmm_last_error", "sfmm_status_string",
    "sfmm_set_stream", "sfmm_translate_device", "sfmm_device_status", "sfmm_translate_host_packed",
    "sfmm_translate_host", "sfmm_bucket_by_order", "sfmm_p2x_device", "sfmm_launch_count",
    "sfmm_host_table", "sfmm_measure_fma_peak", "sfmm_measure_imad_peak", "sfmm_bucket_by_order_noalloc",
    "sfmm_set_group", "sfmm_tune", "sfmm_plan_create", "sfmm_plan_add", "sfmm_plan_finalize", "sfmm_plan_run",
    "sfmm_plan_launches", "sfmm_plan_segments", "sfmm_plan_destroy", "sfmm_eval_device", "sfmm_bounding_sphere",
    "sfmm_p2x_ragged_device", "sfmm_plan_set_options",
]


class SfmmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def lib_path() -> str:
    return _build.LIB


def load():
    """Load libsfmm_gb300.so (must have been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"solidfmm_gb300 native library missing: {path} (run python -m solidfmm_gb300.build)")
    L = C.CDLL(path)
    vp, sz, u32p, dp = C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p
    L.sfmm_create.argtypes = [C.POINTER(vp), C.c_int, sz, C.c_int]
    L.sfmm_destroy.argtypes = [vp]
    L.sfmm_destroy.restype = None
    L.sfmm_order.argtypes = [vp]
    L.sfmm_order.restype = sz
    L.sfmm_data_type.argtypes = [vp]
    L.sfmm_last_error.argtypes = [vp]
    L.sfmm_last_error.restype = C.c_char_p
    L.sfmm_status_string.argtypes = [C.c_int]
    L.sfmm_status_string.restype = C.c_char_p
    L.sfmm_set_stream.argtypes = [vp, vp]
    L.sfmm_set_group.argtypes = [vp, C.c_int, sz, C.c_int]
    L.sfmm_tune.argtypes = [vp, C.c_int, C.c_int, sz, sz, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.sfmm_translate_device.argtypes = [vp, C.c_int, C.c_int, sz, vp, sz, sz, u32p, vp, sz, sz, u32p, u32p, u32p,
                                        dp, u32p, C.c_int, sz]
    L.sfmm_device_status.argtypes = [vp, C.POINTER(C.c_int)]
    L.sfmm_translate_host_packed.argtypes = [vp, C.c_int, C.c_int, sz, vp, sz, sz, u32p, vp, sz, sz, u32p, u32p,
                                             u32p, dp, C.c_int]
    L.sfmm_translate_host.argtypes = [vp, C.c_int, C.c_int, sz, vp, vp, vp, vp, sz, vp, vp, vp]
    L.sfmm_bucket_by_order.argtypes = [vp, sz, u32p, u32p, u32p]
    L.sfmm_p2x_device.argtypes = [vp, C.c_int, sz, sz, dp, dp, dp, vp, sz]
    L.sfmm_p2x_ragged_device.argtypes = [vp, C.c_int, sz, u32p, dp, dp, dp, vp, sz]
    L.sfmm_launch_count.argtypes = [vp]
    L.sfmm_launch_count.restype = C.c_uint64
    L.sfmm_host_table.argtypes = [sz, C.c_int, C.c_int, vp, sz, C.POINTER(C.c_size_t)]
    L.sfmm_measure_fma_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.sfmm_measure_imad_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.sfmm_bucket_by_order_noalloc.argtypes = [sz, u32p, u32p, u32p, sz, vp]
    L.sfmm_eval_device.argtypes = [vp, C.c_int, sz, dp, u32p, vp, sz, sz, dp, dp, dp]
    L.sfmm_bounding_sphere.argtypes = [sz, dp, dp, dp, dp, dp]
    L.sfmm_plan_create.argtypes = [vp, C.POINTER(vp)]
    L.sfmm_plan_add.argtypes = [vp, C.c_int, C.c_int, sz, vp, sz, sz, u32p, vp, sz, sz, u32p, u32p, u32p, dp,
                                C.c_int]
    L.sfmm_plan_finalize.argtypes = [vp]
    L.sfmm_plan_set_options.argtypes = [vp, C.c_int]
    L.sfmm_plan_run.argtypes = [vp]
    L.sfmm_plan_launches.argtypes = [vp]
    L.sfmm_plan_launches.restype = sz
    L.sfmm_plan_segments.argtypes = [vp, vp, vp, sz]
    L.sfmm_plan_segments.restype = sz
    L.sfmm_plan_destroy.argtypes = [vp]
    L.sfmm_plan_destroy.restype = None
    _lib = L
    return L


def host_table(P: int, which: int, n: int = 0) -> np.ndarray:
    """FP64 operator table (see sfmm_host_table in include/sfmm.h); host only."""
    L = load()
    cnt = C.c_size_t(0)
    rc = L.sfmm_host_table(P, which, n, None, 0, C.byref(cnt))
    if rc:
        raise SfmmError(rc, "sfmm_host_table")
    out = np.zeros(cnt.value)
    L.sfmm_host_table(P, which, n, out.ctypes.data, cnt.value, C.byref(cnt))
    return out


def bounding_sphere(x, y, z, r=None):
    """Smallest sphere containing the points (x, y, z), or the spheres of
    radii r: (cx, cy, cz, radius) (sfmm_bounding_sphere; host only)."""
    L = load()
    x, y, z = (np.ascontiguousarray(a, np.float64) for a in (x, y, z))
    rr = None if r is None else np.ascontiguousarray(r, np.float64)
    out = np.zeros(4)
    rc = L.sfmm_bounding_sphere(len(x), x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                None if rr is None else rr.ctypes.data, out.ctypes.data)
    if rc:
        raise SfmmError(rc, "bounding_sphere")
    return out


def measure_peak(kind: str, device: int = 0) -> float:
    """Measured pipe throughput: 'fp64' / 'fp32' (flop/s) or 'imad' (int64 MAC/s)."""
    L = load()
    v = C.c_double(0)
    if kind == "imad":
        rc = L.sfmm_measure_imad_peak(device, C.byref(v))
    else:
        rc = L.sfmm_measure_fma_peak(1 if kind == "fp64" else 0, device, C.byref(v))
    if rc:
        raise SfmmError(rc, "peak probe")
    return v.value


def _ptr(x):
    """device/host address of a torch tensor or numpy array (None -> NULL)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


class Context:
    """An operator context (the reference's operator_data / operator_handle)."""

    def __init__(self, P: int, dtype: str = "f64", device: int = 0):
        L = load()
        self.dtype = F64 if dtype in ("f64", "double", np.float64) else F32
        h = C.c_void_p()
        rc = L.sfmm_create(C.byref(h), self.dtype, P, device)
        if rc:
            raise SfmmError(rc, L.sfmm_status_string(rc).decode())
        self.h = h
        self.P = P
        self.L = L

    def close(self):
        if getattr(self, "h", None):
            self.L.sfmm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise SfmmError(rc, self.L.sfmm_last_error(self.h).decode())

    @property
    def launches(self) -> int:
        return self.L.sfmm_launch_count(self.h)

    def set_stream(self, stream_ptr: int | None):
        self._check(self.L.sfmm_set_stream(self.h, stream_ptr))

    def set_group(self, precision: int, group: int, order_bound: int = 0):
        """Pin the threads per translation for (precision, order bound)."""
        self._check(self.L.sfmm_set_group(self.h, precision, order_bound, group))

    def tune(self, op, precision: int, n: int = 65536, order_bound: int = 0):
        """Time every supported group size on n synthetic translations and
        keep the fastest; returns (group, translations per second)."""
        g = C.c_int(0)
        r = C.c_double(0)
        self._check(self.L.sfmm_tune(self.h, OPS.get(op, op), precision, order_bound, n, C.byref(g), C.byref(r)))
        return g.value, r.value

    def translate_device(self, op, precision, n, src, src_stride, src_count, dst, dst_stride, dst_count, p_in, p_out,
                         shift, src_index=None, dst_index=None, order=None, repeat=False, order_bound=0):
        op = OPS.get(op, op)
        self._check(self.L.sfmm_translate_device(
            self.h, op, precision, n, _ptr(src), src_stride, src_count, _ptr(src_index), _ptr(dst), dst_stride,
            dst_count, _ptr(dst_index), _ptr(p_in), _ptr(p_out), _ptr(shift), _ptr(order),
            TARGETS_REPEAT if repeat else TARGETS_UNIQUE, order_bound))

    def device_status(self) -> int:
        v = C.c_int(0)
        self._check(self.L.sfmm_device_status(self.h, C.byref(v)))
        return v.value

    def translate_host_packed(self, op, precision, src, dst, p_in, p_out, shift, src_index=None, dst_index=None,
                              repeat=False, targets_on_device=False):
        """sfmm_translate_host_packed: host sources and metadata; host targets
        updated in place, or (targets_on_device) a device tensor of targets
        that keeps the results across calls."""
        op = OPS.get(op, op)
        n = len(p_in)
        p_in = np.ascontiguousarray(p_in, np.uint32)
        p_out = np.ascontiguousarray(p_out, np.uint32)
        shift = np.ascontiguousarray(shift, np.float64)
        si = None if src_index is None else np.ascontiguousarray(src_index, np.uint32)
        ti = None if dst_index is None else np.ascontiguousarray(dst_index, np.uint32)
        self._check(self.L.sfmm_translate_host_packed(
            self.h, op, precision, n, _ptr(src), src.shape[-1], src.shape[0], _ptr(si), _ptr(dst), dst.shape[-1],
            dst.shape[0], _ptr(ti), _ptr(p_in), _ptr(p_out), _ptr(shift),
            (TARGETS_REPEAT if repeat else TARGETS_UNIQUE) | (TARGETS_ON_DEVICE if targets_on_device else 0)))

    def bucket(self, n, p_in, p_out, order):
        self._check(self.L.sfmm_bucket_by_order(self.h, n, _ptr(p_in), _ptr(p_out), _ptr(order)))

    def evaluate(self, kind, npts, pos, E, stride, nexp, centre, potential, gradient=None, box=None):
        """L2P (kind 0) / M2P (kind 1): potential[j] (+ gradient) += the
        expansion's field at pos[j] (sfmm_eval_device)."""
        self._check(self.L.sfmm_eval_device(self.h, kind, npts, _ptr(pos), _ptr(box), _ptr(E), stride, nexp,
                                            _ptr(centre), _ptr(potential), _ptr(gradient)))

    def p2x(self, kind, nexp, nq, charge, pos, centre, out, out_stride):
        self._check(self.L.sfmm_p2x_device(self.h, kind, nexp, nq, _ptr(charge), _ptr(pos), _ptr(centre),
                                           _ptr(out), out_stride))

    def p2x_ragged(self, kind, nexp, offset, charge, pos, centre, out, out_stride):
        """P2M (kind 0) / P2L (kind 1) with expansion j taking particles
        offset[j] .. offset[j+1]-1 (offset: nexp + 1 device int32 values)."""
        self._check(self.L.sfmm_p2x_ragged_device(self.h, kind, nexp, _ptr(offset), _ptr(charge), _ptr(pos),
                                                  _ptr(centre), _ptr(out), out_stride))


class Plan:
    """An execution plan (sfmm_plan_*): stages of device batches recorded
    once into a CUDA graph, sorted and segmented by order, replayed by run().
    Tensors passed to add() are kept alive by the plan."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.L = ctx.L
        h = C.c_void_p()
        ctx._check(self.L.sfmm_plan_create(ctx.h, C.byref(h)))
        self.h = h
        self._keep = []

    def add(self, op, precision, n, src, src_stride, src_count, dst, dst_stride, dst_count, p_in, p_out, shift,
            src_index=None, dst_index=None, repeat=False):
        self._keep += [src, dst, p_in, p_out, shift, src_index, dst_index]
        self.ctx._check(self.L.sfmm_plan_add(
            self.h, OPS.get(op, op), precision, n, _ptr(src), src_stride, src_count, _ptr(src_index), _ptr(dst),
            dst_stride, dst_count, _ptr(dst_index), _ptr(p_in), _ptr(p_out), _ptr(shift),
            TARGETS_REPEAT if repeat else TARGETS_UNIQUE))
        return self

    def options(self, fused=False, tune=False):
        """SFMM_PLAN_FUSED (one persistent launch per stage over a work list)
        and SFMM_PLAN_TUNE (measured launch shapes), before finalize()."""
        self.ctx._check(self.L.sfmm_plan_set_options(self.h, (PLAN_FUSED if fused else 0) |
                                                     (PLAN_TUNE if tune else 0)))
        return self

    def finalize(self):
        self.ctx._check(self.L.sfmm_plan_finalize(self.h))
        return self

    def run(self):
        self.ctx._check(self.L.sfmm_plan_run(self.h))

    @property
    def launches(self) -> int:
        return self.L.sfmm_plan_launches(self.h)

    def segments(self):
        k = self.L.sfmm_plan_segments(self.h, None, None, 0)
        b = (C.c_int * max(k, 1))()
        n = (C.c_size_t * max(k, 1))()
        self.L.sfmm_plan_segments(self.h, b, n, k)
        return [(b[i], n[i]) for i in range(k)]

    def close(self):
        if getattr(self, "h", None):
            self.L.sfmm_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
