"""CPU checks of bench.py's roofline arithmetic: the algorithmic flops and
bytes per translation match the closed forms the roofline is stated in
(rotations sum_{d<=P} (4d^2 + 16d) per direction; M2L z-translation
sum_m 4 (P-m)^2, M2M/L2L triangular sum_m 2 (P-m)(P-m+1); bytes = 8 (S_in + 2
S_out) + 24), and the JSON contract's helper values stay consistent."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_flops_closed_forms():
    for P in (1, 2, 10, 12, 16, 20, 24):
        m2l = 2 * P * (P + 1) * (2 * P + 1) + 16 * P * (P + 1)
        tri = (4 * P * (P + 1) * (2 * P + 1)) // 3 + 16 * P * (P + 1) + (2 * P * (P + 1) * (P + 2)) // 3
        assert bench.useful_flops("m2l", P) == m2l
        assert bench.useful_flops("m2m", P) == tri == bench.useful_flops("l2l", P)
    assert bench.useful_flops("m2l", 16) == 22304
    assert bench.useful_flops("m2l", 10) == 6380
    assert bench.useful_flops("m2m", 20) == 35840


def test_bytes_per_translation():
    assert bench.algorithmic_bytes(16) == 6552
    assert bench.algorithmic_bytes(20, esize=4) == 4 * 3 * 420 + 24


def test_measured_constants_are_per_translation_and_plausible():
    # ncu-derived DRAM traffic per translation stays at or below the
    # algorithmic bytes (targets still dirty in L2 are not written back),
    # and the instruction count is a per-translation figure of the split kernel
    for (op, P), t in bench.TRAFFIC.items():
        assert 0.5 * bench.algorithmic_bytes(P) < t <= bench.algorithmic_bytes(P)
    for (op, P), ipt in bench.INSTRUCTIONS.items():
        assert 1000 < ipt < 50000
