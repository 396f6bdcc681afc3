"""ctypes access to the CPU oracle (oracle/_build/liboracle.so) and, where it
was compiled, to the reference library (oracle/_ref/libsolidfmm_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py as the checker, never by the product package.

Batches use the uniform-stride layout of oracle.h: expansion j at
base[j*stride:], orders per translation, op 0 = M2M, 1 = M2L, 2 = L2L.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
# generic-microkernel build: the correctness checker (bit-identical to the
# portable C++ kernels); native build: the reference's own SIMD dispatch, used
# for timing (its AVX-512F double kernel mishandles lanes 12-15 of a batch).
REF_LIB = os.path.join(HERE, "_ref", "libsolidfmm_ref_generic.so")
REF_LIB_NATIVE = os.path.join(HERE, "_ref", "libsolidfmm_ref.so")
# The reference's sources: the copy `make -C oracle stage` leaves under
# _ref/src (on a machine without a reference checkout), else SFMM_REF_SRC.
STAGED_SRC = os.path.join(HERE, "_ref", "src")
REF_SRC = (STAGED_SRC if os.path.isdir(os.path.join(STAGED_SRC, "solidfmm"))
           else os.environ.get("SFMM_REF_SRC", "/root/reference"))

OPS = {"m2m": 0, "m2l": 1, "l2l": 2}

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C")


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (and the reference library when its sources exist:
    both dispatch builds on x86-64, where the generic one is the golden
    generator, only the native build elsewhere)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_ref is None:
        with_ref = os.path.isdir(os.path.join(REF_SRC, "solidfmm"))
    if with_ref:
        if REF_SRC != STAGED_SRC:  # keep a copy that travels to machines without the checkout
            subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF={REF_SRC}"], check=True)
        target = "ref" if platform.machine() in ("x86_64", "AMD64") else "ref-native"
        jobs = str(min(16, os.cpu_count() or 1))
        subprocess.run(["make", "-s", f"-j{jobs}", "-C", HERE, target, f"REF={REF_SRC}"], check=True)


def stage_reference() -> str:
    """Copy the reference's library sources to _ref/src so that they travel to
    a machine without a reference checkout (git-ignored, never committed)."""
    subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF={REF_SRC}"], check=True)
    return STAGED_SRC


_lib = None
_ref = {}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_ref=False)
        L = C.CDLL(LIB)
        L.orc_R_d.argtypes = [C.c_size_t, C.c_double, C.c_double, C.c_double, _f64p]
        L.orc_S_d.argtypes = [C.c_size_t, C.c_double, C.c_double, C.c_double, _f64p]
        L.orc_swap_B.argtypes = [C.c_int, C.c_int, C.c_int]
        L.orc_swap_B.restype = C.c_double
        for f in (L.orc_p2m_d, L.orc_p2l_d):
            f.argtypes = [C.c_size_t, C.c_size_t, C.c_size_t, _f64p, _f64p, _f64p, _f64p, C.c_size_t]
        L.orc_dot_d.argtypes = [C.c_size_t, _f64p, C.c_size_t, _f64p]
        L.orc_dot_d.restype = C.c_double
        L.orc_naive_d.argtypes = [C.c_int, C.c_size_t, _f64p, C.c_size_t, _u32p, _f64p, C.c_size_t, _u32p,
                                  C.c_void_p, C.c_void_p, _f64p, C.c_int]
        for f, fp in ((L.orc_rot_d, _f64p), (L.orc_rot_f, _f32p)):
            f.argtypes = [C.c_int, C.c_size_t, fp, C.c_size_t, _u32p, fp, C.c_size_t, _u32p,
                          C.c_void_p, C.c_void_p, fp, C.c_int, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def ref_available(native: bool = False) -> bool:
    return os.path.exists(REF_LIB_NATIVE if native else REF_LIB)


def ref(native=False):
    path = REF_LIB_NATIVE if native else REF_LIB
    if path not in _ref:
        L = C.CDLL(path)
        for f, fp in ((L.ref_translate_d, _f64p), (L.ref_translate_f, _f32p)):
            f.argtypes = [C.c_int, C.c_size_t, C.c_size_t, C.c_size_t, fp, _u32p, C.c_size_t, C.c_size_t, fp,
                          _u32p, C.c_size_t, _u32p, _u32p, fp, C.c_size_t, C.c_int, C.POINTER(C.c_double)]
            f.restype = C.c_int
        L.ref_last_error.restype = C.c_char_p
        L.ref_harmonic_d.argtypes = [C.c_int, C.c_size_t, C.c_double, C.c_double, C.c_double, _f64p]
        L.ref_swap_B.argtypes = [C.c_int, C.c_int, C.c_int]
        L.ref_swap_B.restype = C.c_double
        L.ref_dot_d.argtypes = [C.c_size_t, C.c_size_t, _f64p, C.c_size_t, C.c_size_t, _f64p, _f64p]
        L.ref_hw_threads.restype = C.c_uint
        L.ref_bounding_sphere_d.argtypes = [C.c_size_t, _f64p, _f64p, _f64p, C.c_void_p, _f64p]
        L.ref_mt_batch_create_d.argtypes = [C.c_int, C.c_size_t, C.c_size_t, _f64p]
        L.ref_mt_batch_create_d.restype = C.c_void_p
        L.ref_mt_batch_run_d.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.ref_mt_batch_destroy_d.argtypes = [C.c_void_p]
        _ref[path] = L
    return _ref[path]


def S_of(P: int) -> int:
    return P * (P + 1)


def harmonic(which: str, P: int, x: float, y: float, z: float) -> np.ndarray:
    out = np.zeros(max(S_of(P), 1))
    getattr(lib(), "orc_R_d" if which == "R" else "orc_S_d")(P, x, y, z, out)
    return out[: S_of(P)]


def swap_B(n: int, m: int, l: int) -> float:
    return lib().orc_swap_B(n, m, l)


def _ptr(a):
    return None if a is None else a.ctypes.data


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def naive(op, src, Pin, dst, Pout, xyz, sidx=None, tidx=None, nthreads=None):
    """dst += T(src) by the O(P^4) formulas, FP64."""
    op = OPS.get(op, op)
    n = len(Pin)
    sidx = None if sidx is None else _u32(sidx)
    tidx = None if tidx is None else _u32(tidx)
    nthreads = nthreads or min(os.cpu_count() or 1, 64)
    rc = lib().orc_naive_d(op, n, src.reshape(-1), src.shape[-1], _u32(Pin), dst.reshape(-1), dst.shape[-1],
                           _u32(Pout), _ptr(sidx), _ptr(tidx), np.ascontiguousarray(xyz, np.float64).reshape(-1),
                           nthreads)
    assert rc == 0
    return dst


def rot(op, src, Pin, dst, Pout, xyz, sidx=None, tidx=None, nthreads=1):
    """dst += T(src) by the lane-batched rotation-based restatement; returns seconds."""
    op = OPS.get(op, op)
    n = len(Pin)
    sidx = None if sidx is None else _u32(sidx)
    tidx = None if tidx is None else _u32(tidx)
    sec = C.c_double(0)
    f = lib().orc_rot_d if src.dtype == np.float64 else lib().orc_rot_f
    rc = f(op, n, src.reshape(-1), src.shape[-1], _u32(Pin), dst.reshape(-1), dst.shape[-1], _u32(Pout),
           _ptr(sidx), _ptr(tidx), np.ascontiguousarray(xyz, src.dtype).reshape(-1), nthreads, C.byref(sec))
    assert rc == 0
    return sec.value


class RefError(Exception):
    def __init__(self, code, msg):
        super().__init__(f"reference error {code}: {msg}")
        self.code = code


def reference(op, Pop, src, Psrc, dst, Ptgt, xyz, sidx, tidx, dim=1, mode=0, native=False):
    """dst += T(src) through the reference library's own API; returns seconds."""
    op = OPS.get(op, op)
    R = ref(native)
    f = R.ref_translate_d if src.dtype == np.float64 else R.ref_translate_f
    sec = C.c_double(0)
    rc = f(op, Pop, len(sidx), src.shape[0], src.reshape(-1), _u32(Psrc), src.shape[-1], dst.shape[0],
           dst.reshape(-1), _u32(Ptgt), dst.shape[-1], _u32(sidx), _u32(tidx),
           np.ascontiguousarray(xyz, src.dtype).reshape(-1), dim, mode, C.byref(sec))
    if rc:
        raise RefError(rc, R.ref_last_error().decode())
    return sec.value


def p2m(P, charges, pos, centres, singular=False):
    """expansions[j] = sum_q charges[j,q] * R(pos[j,q]-centres[j]) (S for singular)."""
    nexp, nq = charges.shape
    out = np.zeros((nexp, S_of(P)))
    f = lib().orc_p2l_d if singular else lib().orc_p2m_d
    f(P, nexp, nq, np.ascontiguousarray(charges, np.float64).reshape(-1),
      np.ascontiguousarray(pos, np.float64).reshape(-1), np.ascontiguousarray(centres, np.float64).reshape(-1),
      out.reshape(-1), S_of(P))
    return out


def dot(A, PA, B, PB):
    return lib().orc_dot_d(PA, np.ascontiguousarray(A, np.float64), PB, np.ascontiguousarray(B, np.float64))


class MtBatch:
    """n translations between separately allocated solids of order P, timed
    through the reference's multithreaded_translator<double>::*_unchecked
    (its own SIMD kernels, one worker per core), set up once."""

    def __init__(self, op, P, xyz, native=True):
        self.R = ref(native)
        xyz = np.ascontiguousarray(xyz, np.float64)
        self.h = self.R.ref_mt_batch_create_d(OPS.get(op, op), P, len(xyz), xyz.reshape(-1))
        if not self.h:
            raise RefError(9, self.R.ref_last_error().decode())

    def run(self) -> float:
        sec = C.c_double(0)
        assert self.R.ref_mt_batch_run_d(self.h, C.byref(sec)) == 0
        return sec.value

    def close(self):
        if self.h:
            self.R.ref_mt_batch_destroy_d(self.h)
            self.h = None

    def __del__(self):
        self.close()
