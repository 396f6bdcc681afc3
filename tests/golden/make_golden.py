"""Generate golden vectors for the translation path from the reference itself.

Runs the reference library compiled from its own sources (oracle/Makefile,
target `ref`, the build whose get_microkernel() returns the portable generic
microkernels) on small seeded inputs and writes tests/golden/*.npz.  Needs the
reference sources (only present in the development container); the fixtures
it writes are committed so the GPU tests never need the reference.

    python tests/golden/make_golden.py

Cases (op, P_in, P_out, dtype):
  * uniform orders 1..16 (double) and 1..14 (float), mixed orders both ways,
  * 32 identical translations into one target (the accumulation pattern of
    the reference's tests/test_m2l.cpp),
  * zero shift for M2M/L2L (prefix add, solidfmm/translations.cpp:540-547),
  * repeated targets with distinct sources,
  * Dehnen's swap matrix B_n^{m,l} for n <= 6 (swap_matrix.cpp:149-171).
L2L with P_in > P_out is excluded: the reference reads uncomputed euler rows
there (translations.cpp:412-419); those cases are pinned to the formula by
the oracle tests instead.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as O  # noqa: E402

from inputs import make_batch  # noqa: E402


def run_case(name, op, Pin, Pout, n, dtype, seed, pattern="distinct", zero_shift=False, nq=24):
    rng = np.random.default_rng(seed)
    b = make_batch(rng, op, Pin, Pout, n, nq=nq, pattern=pattern, zero_shift=zero_shift,
                   in_le_out=(op == "l2l"))
    P = max(int(b["Pin"].max()), int(b["Pout"].max()), 1)
    src = b["src"].astype(dtype)
    dst0 = b["dst"].astype(dtype)
    dst = dst0.copy()
    xyz = b["xyz"].astype(dtype)
    Psrc = np.zeros(src.shape[0], np.uint32)
    Psrc[b["sidx"]] = b["Pin"]
    Ptgt = np.zeros(dst.shape[0], np.uint32)
    Ptgt[b["tidx"]] = b["Pout"]
    O.reference(op, P, src, Psrc, dst, Ptgt, xyz, b["sidx"], b["tidx"], mode=0)
    return dict(op=np.array(op), src=src, dst0=dst0, dst=dst, xyz=xyz, Pin=b["Pin"], Pout=b["Pout"],
                sidx=b["sidx"], tidx=b["tidx"], Pop=np.array(P))


def main():
    if not O.ref_available():
        O.build(with_ref=True)
    cases = {}
    seed = 100
    for dtype, tag, Pmax in ((np.float64, "f64", 16), (np.float32, "f32", 14)):
        for op in ("m2l", "m2m", "l2l"):
            for P in list(range(1, 9)) + [10, 12, Pmax]:
                seed += 1
                cases[f"{op}_{tag}_P{P}"] = run_case(op, op, P, P, 12, dtype, seed)
            for Pin, Pout in ((4, 9), (9, 4), (1, 6), (6, 1), (11, 7), (7, 11)):
                if op == "l2l" and Pin > Pout:
                    continue
                seed += 1
                cases[f"{op}_{tag}_mix{Pin}_{Pout}"] = run_case(op, op, Pin, Pout, 12, dtype, seed)
            seed += 1
            cases[f"{op}_{tag}_ragged"] = run_case(op, op, (2, 10), (2, 10), 24, dtype, seed)
            seed += 1
            cases[f"{op}_{tag}_same32"] = run_case(op, op, 8, 8, 32, dtype, seed, pattern="same32")
            seed += 1
            cases[f"{op}_{tag}_repeat"] = run_case(op, op, 6, 6, 30, dtype, seed, pattern="repeat")
            if op != "m2l":
                seed += 1
                cases[f"{op}_{tag}_zero"] = run_case(op, op, 5, 7, 10, dtype, seed, zero_shift=True)
    out = {}
    for k, v in cases.items():
        for f, a in v.items():
            out[f"{k}/{f}"] = a
    # harmonics R, S, dR, dS of order 12 at a few points (harmonics.cpp:32-349)
    pts = [(0.3, -0.2, 0.5), (1.1, 0.2, -0.9), (-0.7, 0.4, 0.1), (0.0, 0.0, 1.5)]
    for wi, which in enumerate(("R", "S", "dR", "dS")):
        rows = []
        for (px, py, pz) in pts:
            dim = 3 if which.startswith("d") else 1
            buf = np.zeros(12 * 13 * dim)
            O.ref().ref_harmonic_d(wi, 12, px, py, pz, buf)
            rows.append(buf)
        out[f"harmonics/{which}"] = np.array(rows)
    out["harmonics/points"] = np.array(pts)
    B = {}
    for n in range(7):
        B[n] = np.array([[O.ref().ref_swap_B(n, m, l) for l in range(-n, n + 1)] for m in range(-n, n + 1)])
        out[f"swapB/{n}"] = B[n]
    path = os.path.join(HERE, "translations.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(cases)} cases, {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
