"""Benchmark: M2L translations/s at P=16 (2,000,000 translations), the
split-precision ("chosen") path against the plain FP64 GPU path, with
relative error against the FP64 naive oracle and roofline fractions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload m2l16|m2l10|m2m20|l2l20|m2l20]

One step = one pass of the translation kernel over the whole batch.  Inputs
are synthetic with the benchmark's geometry: each source multipole comes from
64 unit charges of random sign uniform in a ball of radius 0.5 (P2M on the
GPU), each target centre lies at distance U[2,4] in a uniform direction.
The batch (src + dst = 8.7 GB in FP64) is far larger than L2 (129 MB), so no
flush is needed between steps.  With --gpus N > 1 every rank runs an
independent replica of the batch (translations are independent; no
collective), reported as weak scaling.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (op, P, N, charges per source)
    "m2l16": ("m2l", 16, 2_000_000, 64),
    # the same kernel on 65 536 translations (1 GB of expansions, still far
    # above L2): the case that ncu --set full captures
    "m2l16_small": ("m2l", 16, 65_536, 64),
    "m2l10": ("m2l", 10, 100_000, 64),
    "m2l20": ("m2l", 20, 1_000_000, 128),
    "m2m20": ("m2m", 20, 1_000_000, 128),
    "l2l20": ("l2l", 20, 1_000_000, 128),
    # 1.5e6 translations, 40% M2L / 30% M2M / 30% L2L, orders U{4..24}
    "mixed": ("mixed", 24, 1_500_000, 64),
    # one FMM pass: uniform octree of depth 5 (32 768 leaves) on the unit cube,
    # 32 charges U[-1, 1] per leaf, P=12
    "fmm": ("fmm", 12, 32768, 32),
    # M2M, M2L, L2L at P=20, FP64 (plain, split, split_ff) and FP32, 1e6 each;
    # plus M2L at P=16 and P=17 (the other reading of "order")
    "ops20": ("ops20", 20, 1_000_000, 128),
}

METRIC = "M2L translations/s at P=16, chosen vs plain FP64 GPU at equal rel. error; %roofline"

# HBM traffic per translation of the split kernel from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum over the launch / 65 536
# translations, workload m2l16_small); see profiles/
TRAFFIC = {("m2l", 16): 5641.0}
# warp instructions per translation of the split kernel from the same capture
# (smsp__inst_executed.sum / 65 536): the kernel is issue bound, so its
# instruction rate against one warp instruction per cycle per SM sub-partition
# is the roofline that bounds it
INSTRUCTIONS = {("m2l", 16): 8275.0}


def useful_flops(op, P):
    """Algorithmic flops of one translation (rotations + z-translation), equal orders."""
    rot = 2 * sum(4 * d * d + 16 * d for d in range(1, P + 1))
    if op == "m2l":
        z = sum(4 * (P - m) * (P - m) for m in range(P))
    else:
        z = sum(2 * (P - m) * (P - m + 1) for m in range(P))
    return rot + z


def algorithmic_bytes(P, esize=8):
    """HBM bytes of one translation: read source, read+write target, FP64 shift."""
    S = P * (P + 1)
    return esize * 3 * S + 24


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = []
        mx = 0.0
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = max(mx, float(s[2]))
                for nm, v in zip(names, s[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl != "reference" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, v, device):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_inputs(ctx, op, P, N, nq, seed, dev):
    """Sources by P2M/P2L on the GPU (float-float), shifts, orders."""
    import torch

    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    S = P * (P + 1)
    src = torch.zeros(N, S, dtype=torch.float64, device=dev)
    chunk = 250_000
    for b in range(0, N, chunk):
        m = min(chunk, N - b)
        d = torch.randn(m, nq, 3, dtype=torch.float64, device=dev, generator=g)
        d = d / d.norm(dim=2, keepdim=True)
        rr = 0.5 * torch.rand(m, nq, 1, dtype=torch.float64, device=dev, generator=g) ** (1.0 / 3.0)
        pos = d * rr
        q = torch.randint(0, 2, (m, nq), device=dev, generator=g).to(torch.float64) * 2 - 1
        cen = torch.zeros(m, 3, dtype=torch.float64, device=dev)
        if op == "l2l":  # local inputs: P2L of a cloud at distance U[2,4]
            u = torch.randn(m, 3, dtype=torch.float64, device=dev, generator=g)
            u = u / u.norm(dim=1, keepdim=True)
            pos = pos + (u * (2 + 2 * torch.rand(m, 1, dtype=torch.float64, device=dev, generator=g)))[:, None, :]
        ctx.p2x(1 if op == "l2l" else 0, m, nq, q.contiguous(), pos.contiguous(), cen, src[b:b + m], S)
    if op == "m2l":
        u = torch.randn(N, 3, dtype=torch.float64, device=dev, generator=g)
        u = u / u.norm(dim=1, keepdim=True)
        shift = u * (2 + 2 * torch.rand(N, 1, dtype=torch.float64, device=dev, generator=g))
    else:
        shift = 0.5 * (torch.randint(0, 2, (N, 3), device=dev, generator=g).to(torch.float64) * 2 - 1)
    pin = torch.full((N,), P, dtype=torch.int32, device=dev)
    return src, shift.contiguous(), pin


def accuracy(ctx, op, P, src, shift, pin, nsub, dev):
    """Relative errors of the plain FP64 and split paths against the naive
    FP64 oracle on the first nsub translations (orthonormal basis and raw)."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import pyoracle
    from helpers import norm_weights, per_degree_err, rel_err

    S = P * (P + 1)
    s = src[:nsub].contiguous()
    sh = shift[:nsub].contiguous()
    pi = pin[:nsub].contiguous()
    s_h = s.cpu().numpy()
    ref = np.zeros((nsub, S))
    pyoracle.naive(op, s_h, pi.cpu().numpy().astype(np.uint32), ref, pi.cpu().numpy().astype(np.uint32),
                   sh.cpu().numpy())
    w = norm_weights(P, "M" if op == "m2m" else "L")
    out = {}
    for name, prec in (("plain_fp64", 0), ("split", 1), ("split_ff", 2), ("tc_tf32x3", 3), ("tc_bf16x3", 4), ("tc_bf16x6", 5)):
        d = torch.zeros(nsub, S, dtype=torch.float64, device=dev)
        ctx.translate_device(op, prec, nsub, s, S, nsub, d, S, nsub, pi, pi, sh)
        torch.cuda.synchronize()
        got = d.cpu().numpy()
        out[name] = {"rel_l2_orthonormal_max": rel_err(got, ref, w), "rel_l2_raw_max": rel_err(got, ref),
                     "rel_l2_orthonormal_per_degree_max": per_degree_err(got, ref, P, w),
                     "rel_l2_raw_per_degree_max": per_degree_err(got, ref, P)}
    return out


def physics_table(ctx, P):
    """The reference's own physics checks (tests/test_m2l.cpp:57-136,
    test_m2m.cpp, test_l2l.cpp: a unit source expanded, translated 32 times
    into one target, evaluated against 1/r and its gradient) for every
    precision mode at order P, beside the same check with the oracle's exact
    (naive O(P^4)) translation and with the reference's double and float."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import pyoracle
    from helpers import physics_errors, physics_gpu, physics_inputs, physics_reference

    out = {}
    for op in ("m2l", "m2m", "l2l"):
        row = {}
        E, shift = physics_inputs(op, P)
        S = P * (P + 1)
        exact = np.zeros((1, S))
        pn = np.full(1, P, np.uint32)
        pyoracle.naive(op, E.reshape(1, S), pn, exact, pn, shift.reshape(1, 3))
        pe = physics_errors(op, P, exact[0])
        row["oracle_exact_translation"] = {"potential": pe[0], "gradient": pe[1]}
        for name, prec in (("plain_fp64", 0), ("split", 1), ("split_ff", 2), ("tc_tf32x3", 3), ("tc_bf16x3", 4),
                           ("tc_bf16x6", 5)):
            e = physics_gpu(ctx, op, P, prec)
            row[name] = {"potential": e[0], "gradient": e[1]}
        for nm, dt in (("reference_double", np.float64), ("reference_float", np.float32)):
            if dt == np.float32 and P > 18:
                continue
            e = physics_reference(op, P, dt)
            if e is not None:
                row[nm] = {"potential": e[0], "gradient": e[1]}
        out[op] = row
    return out


def workload_shifts(op, n, seed):
    """Shifts with the workload's geometry (numpy, seeded): M2L at distance
    U[2,4] in a uniform direction, M2M/L2L to a random octant corner."""
    rng = np.random.default_rng(seed)
    if op == "m2l":
        u = rng.standard_normal((n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        return u * rng.uniform(2, 4, (n, 1))
    return 0.5 * (rng.integers(0, 2, (n, 3)) * 2 - 1).astype(np.float64)


def reference_batch(op, P, n, seed):
    """The reference's own multithreaded_translator<double> (its SIMD
    microkernels, one pinned worker per core) over n translations between
    separately allocated solids, or None where the reference library was not
    built (no reference sources on this machine)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    try:
        pyoracle.build()
    except Exception:  # noqa: BLE001 - a failed reference build leaves the port
        return None
    if not pyoracle.ref_available(native=True):
        return None
    return pyoracle.MtBatch(op, P, workload_shifts(op, n, seed))


def cpu_leg_port(op, P, seconds_target, seed):
    """The oracle's C port of the rotation-based driver (2-wide SIMD, one
    pthread per core) on passes of 20 000 translations for about
    seconds_target seconds: translations/s, threads, pass size, total."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    rng = np.random.default_rng(seed)
    ns = 20_000 if P >= 16 else 50_000
    S = P * (P + 1)
    src = rng.standard_normal((ns, S)) * 1e-3
    dst = np.zeros((ns, S))
    shift = workload_shifts(op, ns, seed)
    pin = np.full(ns, P, np.uint32)
    threads = os.cpu_count() or 1
    total = 0.0
    done = 0
    while total < seconds_target:
        total += pyoracle.rot(op, src, pin, dst, pin, shift, nthreads=threads)
        done += ns
    return done / total, threads, ns, done


def cpu_leg(op, P, seconds_target, seed):
    """CPU baseline on a bounded sample: the reference's own
    multithreaded_translator over 200 000 translations per pass where it was
    built, else the port; repeated for about seconds_target seconds."""
    threads = os.cpu_count() or 1
    ns = 200_000
    b = reference_batch(op, P, ns, seed)
    if b is None:
        v, threads, ns, done = cpu_leg_port(op, P, seconds_target, seed)
        return {"value": v, "unit": "translations/s", "cores": threads, "kind": "port",
                "sample": f"{done} {op.upper()} translations at P={P} in passes of {ns}, FP64, oracle port of the "
                          f"rotation-based driver, one pthread per core (reference library not built here)"}
    total, done = 0.0, 0
    while total < seconds_target:
        total += b.run()
        done += ns
    b.close()
    return {"value": done / total, "unit": "translations/s", "cores": threads, "kind": "reference",
            "sample": f"{done} {op.upper()} translations at P={P} in passes of {ns} separately allocated FP64 "
                      f"solids, reference multithreaded_translator<double>::{op}_unchecked (its own SIMD "
                      f"microkernels, {platform.machine()}, one worker per core)"}


def run_c0(local, steps):
    """M2L at P=10 over 100 000 translations (64 unit charges per source), plain
    FP64 on the GPU, against the reference's own CPU translations on the same
    inputs (its multithreaded_translator where the reference library was
    built) and the FP64 naive oracle on the whole batch."""
    import torch
    import solidfmm_gb300 as sf

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import pyoracle
    from helpers import norm_weights, rel_err

    dev = torch.device("cuda", local)
    P, N = 10, 100_000
    S = P * (P + 1)
    ctx = sf.Context(P, "f64", device=local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    src, shift, pin = make_inputs(ctx, "m2l", P, N, 64, 77, dev)
    dst = torch.zeros(N, S, dtype=torch.float64, device=dev)
    ctx.translate_device("m2l", 0, N, src, S, N, dst, S, N, pin, pin, shift)
    torch.cuda.synchronize()
    got = dst.cpu().numpy()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ctx.translate_device("m2l", 0, N, src, S, N, dst, S, N, pin, pin, shift)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    src_h, sh_h = src.cpu().numpy(), shift.cpu().numpy()
    pin_h = np.full(N, P, np.uint32)
    idx = np.arange(N, dtype=np.uint32)
    ref = np.zeros((N, S))
    pyoracle.naive("m2l", src_h, pin_h, ref, pin_h, sh_h)
    w = norm_weights(P, "L")
    row = {"workload": "M2L P=10, 100 000 translations, 64 unit charges per source, FP64",
           "plain_fp64": {"value": N / (ms * 1e-3), "unit": "translations/s", "ms_per_step": ms},
           "rel_err_vs_fp64_oracle": {"raw": rel_err(got, ref), "orthonormal": rel_err(got, ref, w)}}
    native = not pyoracle.ref_available()  # the generic-dispatch checker where it was built, else native
    if pyoracle.ref_available(native=native):
        rd = np.zeros((N, S))
        sec = pyoracle.reference("m2l", P, src_h, pin_h, rd, pin_h, sh_h, idx, idx, mode=3, native=native)
        row["reference_cpu"] = {"value": N / sec, "unit": "translations/s", "cores": os.cpu_count(),
                                "build": "native SIMD" if native else "generic microkernels"}
        row["rel_err_vs_reference_double"] = {"raw": rel_err(got, rd), "orthonormal": rel_err(got, rd, w)}
        row["reference_double_vs_oracle"] = {"raw": rel_err(rd, ref), "orthonormal": rel_err(rd, ref, w)}
    return row


def extras(args, local):
    """Configurations beside the headline, in bounded time (tens of seconds):
    config 0 (M2L P=10), config 1 (P=20 M2M/M2L/L2L, FP64 and FP32), config 3
    (mixed orders, execution plan) and config 4 (FMM pass)."""
    import torch

    out = {}
    t0 = time.perf_counter()
    out["c0_m2l_p10"] = run_c0(local, max(3, args.steps // 4))
    torch.cuda.empty_cache()
    sub = argparse.Namespace(**vars(args))
    sub.steps = max(3, args.steps // 4)
    sub.warmup = 2
    r = run_ops20(sub, nested=True)
    out["c1_p20"] = r["rows"] if r else None
    torch.cuda.empty_cache()
    r = run_mixed(sub, nested=True)
    keys = ("value", "unit", "ms_per_step", "value_from", "plan_fused", "plan_segmented", "plan_segmented_tuned",
            "unsorted_one_launch_per_op",
            "per_order_pair_launches", "config")
    out["c3_mixed"] = {k: r[k] for k in keys} if r else None
    torch.cuda.empty_cache()
    r = run_fmm(sub, nested=True)
    out["c4_fmm"] = {k: r[k] for k in ("value", "unit", "plain_fp64_ms_per_pass", "translations_per_s",
                                       "leaf_local_rel_err_vs_oracle_pass",
                                       "potential_rel_err_vs_direct_2000_particles", "tensor_core_passes",
                                       "l2p_gradient_all_particles",
                                       "cpu_baseline", "config")} if r else None
    torch.cuda.empty_cache()
    out["seconds"] = time.perf_counter() - t0
    return out


MIXED_METRIC = "mixed M2L/M2M/L2L translations/s, orders U{4..24}, 1.5e6 per GPU"


def run_mixed(args, nested=False):
    """Mixed-order batch: 40% M2L, 30% M2M, 30% L2L with P_in, P_out iid
    U{4..24}, sources gathered from 65 536 P2M/P2L expansions per kind,
    distinct targets.  One execution plan (three stages, order-sorted
    segments, CUDA graph) against one unsorted launch per operator at order
    bound 24 and against one launch per (operator, P_in, P_out) group."""
    import torch
    import solidfmm_gb300 as sf
    from solidfmm_gb300 import build as _b

    world, rank, local = (1, 0, 0) if nested else dist_init(args)
    if not nested:
        _b.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    P, N = 24, WORKLOADS["mixed"][2]
    S = P * (P + 1)
    NS = 65536
    ctx = sf.Context(P, "f64", device=local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    srcM, _, _ = make_inputs(ctx, "m2m", P, NS, 64, 500 + rank, dev)
    srcL, _, _ = make_inputs(ctx, "l2l", P, NS, 64, 600 + rank, dev)
    g = torch.Generator(device=dev)
    g.manual_seed(700 + rank)
    counts = {"m2l": int(0.4 * N), "m2m": int(0.3 * N)}
    counts["l2l"] = N - counts["m2l"] - counts["m2m"]
    dst = torch.zeros(N, S, dtype=torch.float64, device=dev)
    batches = {}
    off = 0
    for op in ("m2l", "m2m", "l2l"):
        n = counts[op]
        pin = torch.randint(4, 25, (n,), device=dev, generator=g, dtype=torch.int32)
        pout = torch.randint(4, 25, (n,), device=dev, generator=g, dtype=torch.int32)
        sidx = torch.randint(0, NS, (n,), device=dev, generator=g, dtype=torch.int32)
        if op == "m2l":
            u = torch.randn(n, 3, dtype=torch.float64, device=dev, generator=g)
            sh = u / u.norm(dim=1, keepdim=True) * (2 + 2 * torch.rand(n, 1, dtype=torch.float64, device=dev,
                                                                          generator=g))
        else:
            sh = 0.5 * (torch.randint(0, 2, (n, 3), device=dev, generator=g).to(torch.float64) * 2 - 1)
        batches[op] = dict(n=n, pin=pin, pout=pout, sidx=sidx, shift=sh.contiguous(), dst=dst[off:off + n],
                           src=srcL if op == "l2l" else srcM)
        off += n

    def plan_for(prec, fused=False, tune=False):
        pl = sf.Plan(ctx)
        for op, b in batches.items():
            pl.add(op, prec, b["n"], b["src"], S, NS, b["dst"], S, b["n"], b["pin"], b["pout"], b["shift"],
                   src_index=b["sidx"])
        return pl.options(fused=fused, tune=tune).finalize()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        barrier(world)
        l0 = ctx.launches
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return allmax(world, e0.elapsed_time(e1) / steps, dev), (ctx.launches - l0) // max(steps, 1)

    clocks = Clocks(local)
    # the configuration's own form: one persistent fused launch per operator,
    # launch shapes measured by the tuner, captured in a CUDA graph
    plan_ft = plan_for(1, fused=True, tune=True)
    plan_split = plan_for(1)  # one launch per order segment, segments on four concurrent graph branches
    plan_st = plan_for(1, tune=True)  # the same, every segment's shape measured on the segment itself
    clocks.start()
    ms_ft, launches = timed(plan_ft.run, args.steps, args.warmup)
    ms_plan, seg_launches = timed(plan_split.run, args.steps, args.warmup)
    ms_st, _ = timed(plan_st.run, args.steps, args.warmup)
    clk = clocks.stop()
    plan_fused_plain = plan_for(0, fused=True, tune=True)
    ms_ft_plain, _ = timed(plan_fused_plain.run, max(2, args.steps // 2), 1)
    plan_plain = plan_for(0)
    ms_plan_plain, _ = timed(plan_plain.run, max(2, args.steps // 2), 1)

    def unsorted(prec):
        def f():
            for op, b in batches.items():
                ctx.translate_device(op, prec, b["n"], b["src"], S, NS, b["dst"], S, b["n"], b["pin"], b["pout"],
                                     b["shift"], src_index=b["sidx"], order_bound=P)
        return f

    ms_unsorted, _ = timed(unsorted(1), max(2, args.steps // 2), 1)
    ms_unsorted_plain, _ = timed(unsorted(0), max(2, args.steps // 2), 1)

    # one launch per (operator, P_in, P_out) group
    groups = []
    for op, b in batches.items():
        key = (b["pin"].long() * 32 + b["pout"].long())
        order = torch.argsort(key)
        ks = key[order]
        bounds = torch.nonzero(ks[1:] != ks[:-1]).flatten().cpu().tolist()
        starts = [0] + [x + 1 for x in bounds]
        ends = starts[1:] + [b["n"]]
        kl = ks.cpu().tolist()
        for s0, s1 in zip(starts, ends):
            pi, po = divmod(kl[s0], 32)
            idx = order[s0:s1]
            groups.append((op, s1 - s0, max(pi, po), b["src"], b["sidx"][idx].contiguous(), b["dst"],
                           idx.to(torch.int32).contiguous(), b["pin"][idx].contiguous(), b["pout"][idx].contiguous(),
                           b["shift"][idx].contiguous(), b["n"]))

    def per_pair(prec):
        def f():
            for op, n, bnd, src, si, d, ti, pi, po, sh, nd in groups:
                ctx.translate_device(op, prec, n, src, S, NS, d, S, nd, pi, po, sh, src_index=si, dst_index=ti,
                                     order_bound=bnd)
        return f

    ms_pairs, _ = timed(per_pair(1), 2, 1)
    ms_pairs_plain, _ = timed(per_pair(0), 2, 1)
    if rank != 0:
        return
    segs = plan_split.segments()
    rate = lambda ms: world * N / (ms * 1e-3)  # noqa: E731
    # the value is the fastest plan form; all are reported
    forms = {"plan_fused": ms_ft, "plan_segmented": ms_plan, "plan_segmented_tuned": ms_st}
    value_from = min(forms, key=forms.get)
    fused_wins = value_from == "plan_fused"
    ms_best = forms[value_from]
    line = {"metric": MIXED_METRIC, "value": rate(ms_best), "unit": "translations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_best, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "split (int32 block fixed point rotations, float-float z-translation, f64 accumulation)",
            "data": "synthetic (seeded P2M/P2L sources, random orders and shifts)",
            "config": {"workload": "mixed: 600k M2L + 450k M2M + 450k L2L, P_in, P_out iid U{4..24}, sources "
                                   "gathered from 65 536 expansions per kind, distinct targets, FP64 storage at "
                                   "stride 600", "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas x{world}"},
            "value_from": value_from,
            "plan_fused": {"form": "one persistent launch per operator over a device work list of order-sorted "
                                   "tiles, launch shapes measured by sfmm_tune at finalize (SFMM_PLAN_FUSED | "
                                   "SFMM_PLAN_TUNE)", "split": rate(ms_ft), "plain_fp64": rate(ms_ft_plain),
                           "launches_per_step": launches, "cuda_graph": True},
            "plan_segmented": {"form": "one launch per order-bound segment at that order's own launch shape, the "
                                       "segments of an operator on four concurrent graph branches (the default)",
                               "split": rate(ms_plan), "plain_fp64": rate(ms_plan_plain), "segments": len(segs),
                               "launches_per_step": seg_launches, "cuda_graph": True},
            "plan_segmented_tuned": {"form": "the segmented plan with SFMM_PLAN_TUNE: every segment's launch shape "
                                             "measured at finalize on the segment's own data (targets in scratch)",
                                     "split": rate(ms_st)},
            "unsorted_one_launch_per_op": {"split": rate(ms_unsorted), "plain_fp64": rate(ms_unsorted_plain)},
            "per_order_pair_launches": {"split": rate(ms_pairs), "plain_fp64": rate(ms_pairs_plain),
                                        "launches_per_step": len(groups)},
            "clocks": clk, "gpu_launches": launches if fused_wins else seg_launches}
    if not nested:
        print(json.dumps(line))
    return line


OPS_METRIC = "translations/s per operator and arithmetic, P=20, 1e6 translations"


def run_ops20(args, nested=False):
    """Every operator at P=20 in every arithmetic (1e6 translations, 128
    charges per source), with the relative error against the FP64 naive
    oracle on 500 translations; M2L at P=16 and P=17 beside it.  FP32 at
    P=20 is above the reference's float limit (18) and is checked against the
    FP64 oracle."""
    import torch
    import solidfmm_gb300 as sf
    from solidfmm_gb300 import build as _b

    world, rank, local = (1, 0, 0) if nested else dist_init(args)
    if not nested:
        _b.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import pyoracle
    from helpers import norm_weights, rel_err

    pyoracle.build(with_ref=False)
    rows = []
    cases = [("m2m", 20, 1_000_000), ("m2l", 20, 1_000_000), ("l2l", 20, 1_000_000)]
    if not nested:  # the other reading of "order P" beside the headline's
        cases += [("m2l", 16, 1_000_000), ("m2l", 17, 1_000_000)]
    for op, P, N in cases:
        S = P * (P + 1)
        ctx = sf.Context(P, "f64", device=local)
        ctx32 = sf.Context(P, "f32", device=local)
        stream = torch.cuda.current_stream(dev)
        ctx.set_stream(stream.cuda_stream)
        ctx32.set_stream(stream.cuda_stream)
        src, shift, pin = make_inputs(ctx, op, P, N, 128 if P == 20 else 64, 321 + rank, dev)
        src32 = src.to(torch.float32)
        dst = torch.zeros(N, S, dtype=torch.float64, device=dev)
        dst32 = torch.zeros(N, S, dtype=torch.float32, device=dev)
        nsub = 500
        ref = np.zeros((nsub, S))
        pinh = pin[:nsub].cpu().numpy().astype(np.uint32)
        pyoracle.naive(op, src[:nsub].cpu().numpy(), pinh, ref, pinh, shift[:nsub].cpu().numpy())
        w = norm_weights(P, "M" if op == "m2m" else "L")
        for name, c, prec, sb, db in (("plain_fp64", ctx, 0, src, dst), ("split", ctx, 1, src, dst),
                                      ("split_ff", ctx, 2, src, dst), ("plain_fp32", ctx32, 0, src32, dst32)):
            def f():
                c.translate_device(op, prec, N, sb, S, N, db, S, N, pin, pin, shift)
            for _ in range(args.warmup):
                f()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(max(2, args.steps // 4)):
                f()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = allmax(world, e0.elapsed_time(e1) / max(2, args.steps // 4), dev)
            d = torch.zeros(nsub, S, dtype=db.dtype, device=dev)
            c.translate_device(op, prec, nsub, sb[:nsub].contiguous(), S, nsub, d, S, nsub, pin[:nsub].contiguous(),
                               pin[:nsub].contiguous(), shift[:nsub].contiguous())
            got = d.double().cpu().numpy()
            rows.append({"op": op, "P": P, "arith": name, "translations_per_s": world * N / (ms * 1e-3),
                         "rel_err_orthonormal_max": rel_err(got, ref, w), "rel_err_raw_max": rel_err(got, ref)})
        del src, src32, dst, dst32, ctx, ctx32
        torch.cuda.empty_cache()
    if rank != 0:
        return
    head = next(r for r in rows if r["op"] == "m2l" and r["P"] == 20 and r["arith"] == "split")
    line = {"metric": OPS_METRIC, "value": head["translations_per_s"], "unit": "translations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "per row", "data": "synthetic (seeded P2M/P2L of random charges)",
            "config": {"workload": "M2M/M2L/L2L at P=20 (1e6 each, 128 charges per source), M2L at P=16 and 17",
                       "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
            "rows": rows}
    if not nested:
        print(json.dumps(line))
    return line


FMM_METRIC = "FMM pass time (P2M + M2M + M2L + L2L), uniform octree depth 5, P=12, 32 charges per leaf"


def run_fmm(args, nested=False):
    """One FMM pass on a depth-5 uniform octree at P=12 (solidfmm_gb300.fmm):
    P2M at the leaves, M2M to level 2, M2L over the interaction lists of
    levels 2..5, L2L to the leaves, in one execution plan.  The leaf locals
    are checked against the oracle's CPU pass (FP64 rotation method), whose
    time is the CPU baseline, and the potential (L2P + near-field direct
    sums) against direct summation at 2 000 sampled particles."""
    import torch
    import solidfmm_gb300 as sf
    from solidfmm_gb300 import build as _b
    from solidfmm_gb300 import fmm

    world, rank, local = (1, 0, 0) if nested else dist_init(args)
    if not nested:
        _b.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    depth, P, per = 5, 12, 32
    ctx = sf.Context(P, "f64", device=local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    q, pos = fmm.random_particles(depth, per, 900 + rank, dev)
    f = fmm.UniformFMM(ctx, depth, sf.SPLIT, dev)
    fp = fmm.UniformFMM(ctx, depth, sf.PLAIN, dev)
    # the same pass with every translation on the tensor-core kernel
    ftc = {name: fmm.UniformFMM(ctx, depth, mode, dev)
           for name, mode in (("tc_bf16x6", sf.TC_BF16X6), ("tc_tf32x3", sf.TC_TF32), ("tc_bf16x3", sf.TC_BF16))}
    counts = f.translations
    ntr = sum(counts.values())

    def timed(obj, steps, warmup):
        for _ in range(warmup):
            obj.run(q, pos)
        torch.cuda.synchronize()
        barrier(world)
        l0 = ctx.launches
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            obj.run(q, pos)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return allmax(world, e0.elapsed_time(e1) / steps, dev), (ctx.launches - l0) // max(steps, 1)

    clocks = Clocks(local)
    clocks.start()
    ms, launches = timed(f, args.steps, args.warmup)
    clk = clocks.stop()
    ms_plain, _ = timed(fp, max(2, args.steps // 2), 1)
    ms_tc = {name: timed(obj, max(2, args.steps // 2), 1)[0] for name, obj in ftc.items()}
    # L2P with gradients at every particle from the leaf locals (the step after the pass)
    nleaf_all = 8 ** depth
    pts_all = pos.reshape(-1, 3).contiguous()
    box_all = torch.arange(nleaf_all, device=dev, dtype=torch.int32).repeat_interleave(per)
    pot_all = torch.zeros(len(pts_all), dtype=torch.float64, device=dev)
    grad_all = torch.zeros(len(pts_all), 3, dtype=torch.float64, device=dev)

    class _L2P:
        @staticmethod
        def run(_q, _pos):
            ctx.evaluate(0, len(pts_all), pts_all, f.leaf_locals(), f.S, nleaf_all, f.leaf_centres, pot_all,
                         gradient=grad_all, box=box_all)

    f.run(q, pos)
    ms_l2p, _ = timed(_L2P, max(2, args.steps), 2)
    if rank != 0:
        return
    # physics: potential at sampled particles, far field (L2P) + near field vs direct sum
    nleaf = 8 ** depth
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    samp = torch.randint(0, nleaf * per, (2000,), device=dev, generator=g)
    pts = pos.reshape(-1, 3)[samp].contiguous()
    box = (samp // per).to(torch.int32)
    allp = pos.reshape(-1, 3)
    allq = q.reshape(-1)
    direct = torch.zeros(len(samp), dtype=torch.float64, device=dev)
    for c0 in range(0, len(allp), 1 << 18):
        r = torch.cdist(pts, allp[c0:c0 + (1 << 18)], compute_mode="donot_use_mm_for_euclid_dist")
        direct += torch.where(r > 0, allq[c0:c0 + (1 << 18)][None, :] / r.clamp_min(1e-300),
                              torch.zeros_like(r)).sum(1)
    ns, nt = fmm.neighbours(depth, dev)
    near = torch.zeros(len(samp), dtype=torch.float64, device=dev)
    for i in range(len(samp)):
        b = int(box[i])
        srcb = ns[nt == b]
        idx = (srcb[:, None] * per + torch.arange(per, device=dev)[None, :]).reshape(-1)
        r = torch.linalg.norm(allp[idx] - pts[i], dim=1)
        near[i] = torch.where(r > 0, allq[idx] / r.clamp_min(1e-300), torch.zeros_like(r)).sum()
    def potential_err(obj):
        obj.run(q, pos)
        pot = torch.zeros(len(samp), dtype=torch.float64, device=dev)
        ctx.evaluate(0, len(samp), pts, obj.leaf_locals(), obj.S, nleaf, obj.leaf_centres, pot, box=box)
        return float(torch.linalg.norm(pot + near - direct) / torch.linalg.norm(direct))

    phys_tc = {name: potential_err(obj) for name, obj in ftc.items()}
    phys_plain = potential_err(fp)
    phys = potential_err(f)
    # leaf locals against the oracle's CPU pass
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fmm_oracle
    import pyoracle

    pyoracle.build(with_ref=False)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import norm_weights, rel_err

    qh, ph = q.cpu().numpy(), pos.cpu().numpy()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = fmm_oracle.fmm_pass(depth, P, qh, ph, nthreads=threads)
    cpu_s = time.perf_counter() - t0
    w = norm_weights(P, "L")
    err_split = rel_err(f.leaf_locals().cpu().numpy(), ref, w)
    fp.run(q, pos)
    torch.cuda.synchronize()
    err_plain = rel_err(fp.leaf_locals().cpu().numpy(), ref, w)
    tc_rows = {}
    for name, obj in ftc.items():
        obj.run(q, pos)
        torch.cuda.synchronize()
        tc_rows[name] = {"ms_per_pass": ms_tc[name],
                         "leaf_local_rel_err_vs_oracle_pass": rel_err(obj.leaf_locals().cpu().numpy(), ref, w),
                         "potential_rel_err_vs_direct_2000_particles": phys_tc[name]}
    line = {"metric": FMM_METRIC, "value": ms, "unit": "ms per pass", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "split (int32 block fixed point rotations, float-float z-translation, "
                                          "f64 accumulation)",
            "data": "synthetic (seeded uniform charges in every leaf)",
            "config": {"workload": "uniform octree depth 5 on [0,1]^3, 32 768 leaves x 32 charges U[-1,1], P=12",
                       "translations_per_pass": counts, "l2": "expansions of all levels (93 MB) fit in L2",
                       "parallelism": f"replicas x{world}"},
            "translations_per_s": ntr / (ms * 1e-3), "plain_fp64_ms_per_pass": ms_plain,
            "leaf_local_rel_err_vs_oracle_pass": {"split": err_split, "plain_fp64": err_plain,
                                                   "metric": "max over leaves, relative L2, orthonormal basis"},
            "potential_rel_err_vs_direct_2000_particles": phys,
            "potential_rel_err_vs_direct_plain_fp64": phys_plain,
            "l2p_gradient_all_particles": {"ms": ms_l2p, "points": nleaf_all * per,
                                           "points_per_s": nleaf_all * per / (ms_l2p * 1e-3),
                                           "what": "sfmm_eval_device: potential and gradient of the leaf "
                                                   "locals at every particle (float-float, after the pass)"},
            "tensor_core_passes": tc_rows,
            "tensor_core_note": "the same pass with every translation (M2M, M2L, L2L) on the tcgen05 kernel; "
                                "at P=12 the expansion's own truncation error sets the potential error",
            "cpu_baseline": {"value": cpu_s * 1e3, "unit": "ms per pass", "cores": threads, "kind": "port",
                             "sample": "the same pass (P2M + all translations) by the oracle's FP64 rotation-method "
                                       "port, one pthread per core"},
            "clocks": clk, "gpu_launches": launches}
    if not nested:
        print(json.dumps(line))
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="m2l16", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the other configurations")
    args = ap.parse_args()
    if args.workload == "mixed":
        return run_mixed(args)
    if args.workload == "fmm":
        return run_fmm(args)
    if args.workload == "ops20":
        return run_ops20(args)
    op, P, N, nq = WORKLOADS[args.workload]
    world, rank, local = dist_init(args)
    config = {"workload": f"{op.upper()} P={P} (reference order: degrees 0..{P - 1}), {N} translations per GPU, "
                          f"{nq} charges per source, FP64 expansions",
              "op": op, "P": P, "translations": N, "charges_per_source": nq,
              "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        b = reference_batch(op, P, N, 4321)
        if b is not None:  # the full workload per step, as the reference's own benchmark does
            for _ in range(args.warmup):
                b.run()
            times = [b.run() for _ in range(args.steps)]
            b.close()
            value = N * len(times) / sum(times)
            kind = "reference"
            sample = (f"{N} {op.upper()} translations at P={P} per step (the whole workload) between separately "
                      f"allocated FP64 solids, reference multithreaded_translator<double>::{op}_unchecked with its "
                      f"own SIMD microkernels ({platform.machine()}), one worker per core")
            ms = 1e3 * sum(times) / len(times)
        else:  # no reference build on this machine: the port, on passes of 20 000
            vals = []
            for i in range(args.warmup + args.steps):
                v, threads, ns, done = cpu_leg_port(op, P, 2.0, 1000 + i)
                if i >= args.warmup:
                    vals.append(v)
            value = statistics.median(vals)
            kind = "port"
            sample = (f"passes of {ns} {op.upper()} translations at P={P} repeated >= 2 s per step, oracle port "
                      f"of the rotation-based driver, one pthread per core (reference library not built here)")
            ms = 1e3 * N / value
        line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "translations/s", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": config,
                "cpu_baseline": {"value": value, "unit": "translations/s", "cores": threads, "kind": kind,
                                 "sample": sample},
                "e2e": {"value": value, "unit": "translations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    import solidfmm_gb300 as sf
    from solidfmm_gb300 import build as _b

    _b.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = sf.Context(P, "f64", device=local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    src, shift, pin = make_inputs(ctx, op, P, N, nq, 1234 + rank, dev)
    S = P * (P + 1)
    dst = torch.zeros(N, S, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    L = sf.load()
    L.sfmm_measure_fma_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    peaks = {}
    for fp64, nm in ((1, "fp64"), (0, "fp32")):
        v = C.c_double(0)
        L.sfmm_measure_fma_peak(fp64, local, C.byref(v))
        peaks[nm] = v.value

    def run(prec):
        ctx.translate_device(op, prec, N, src, S, N, dst, S, N, pin, pin, shift)

    def timed(prec, steps, warmup, clocks=None):
        for _ in range(warmup):
            run(prec)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        l0 = ctx.launches
        if clocks:
            clocks.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            run(prec)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        clk = clocks.stop() if clocks else None
        ms = e0.elapsed_time(e1) / steps
        return allmax(world, ms, dev), ctx.launches - l0, clk

    clocks = Clocks(local)
    ms_split, launches, clk = timed(1, args.steps, args.warmup, clocks)
    ms_plain, _, _ = timed(0, max(2, args.steps // 2), 1)
    ms_ff, _, _ = timed(2, max(2, args.steps // 2), 1)
    tc_ms = {}
    tc_clk = {}
    if P <= 16:  # the tensor-core kernel's order range
        for name, prec in (("tc_tf32x3", 3), ("tc_bf16x3", 4), ("tc_bf16x6", 5)):
            tc_ms[name], _, tc_clk[name] = timed(prec, max(3, args.steps // 2), 2, Clocks(local))
    value = world * N / (ms_split * 1e-3)
    plain_value = world * N / (ms_plain * 1e-3)
    ff_value = world * N / (ms_ff * 1e-3)

    # end to end through the C ABI with pinned host buffers
    h_src = torch.empty(N, S, dtype=torch.float64, pin_memory=True)
    h_src.copy_(src)
    h_dst = torch.zeros(N, S, dtype=torch.float64, pin_memory=True)
    h_pin = pin.cpu().numpy().astype(np.uint32)
    h_shift = shift.cpu().numpy()
    e2e_steps = max(2, args.steps // 2)
    ctx.translate_host_packed(op, 1, h_src, h_dst, h_pin, h_pin, h_shift)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.translate_host_packed(op, 1, h_src, h_dst, h_pin, h_pin, h_shift)
    t1 = time.perf_counter()
    e2e_s = allmax(world, (t1 - t0) / e2e_steps, dev)
    h2d = N * S * 8 * 2 + N * 8 + N * 24
    d2h = N * S * 8

    # the classic call (sfmm_translate_host, what the drop-in
    # multithreaded_translator and m2l(op, buf, howmany, M**, L**, ...) use):
    # arrays of solid addresses, here the rows of the same pinned buffers
    Lb = sf.load()
    Lb.sfmm_translate_host.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p]
    addr_s = np.uint64(h_src.data_ptr()) + np.arange(N, dtype=np.uint64) * np.uint64(S * 8)
    addr_d = np.uint64(h_dst.data_ptr()) + np.arange(N, dtype=np.uint64) * np.uint64(S * 8)
    ord64 = h_pin.astype(np.uint64)
    sx, sy, sz = (np.ascontiguousarray(h_shift[:, k]) for k in range(3))
    opc = {"m2m": 0, "m2l": 1, "l2l": 2}[op]

    def classic():
        rc = Lb.sfmm_translate_host(ctx.h, opc, 1, N, addr_s.ctypes.data, ord64.ctypes.data, addr_d.ctypes.data,
                                    ord64.ctypes.data, 1, sx.ctypes.data, sy.ctypes.data, sz.ctypes.data)
        assert rc == 0, Lb.sfmm_last_error(ctx.h)

    classic()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        classic()
    classic_s = allmax(world, (time.perf_counter() - t0) / e2e_steps, dev)

    acc = accuracy(ctx, op, P, src, shift, pin, 1000, dev) if rank == 0 else None
    physics = physics_table(ctx, P) if rank == 0 else None

    if rank != 0:
        return
    F = useful_flops(op, P)
    B = algorithmic_bytes(P)
    t_kernel = ms_split * 1e-3 / N  # seconds per translation (one launch per step)
    achieved_gbs = B / t_kernel / 1e9
    hbm_peak = 6747.3
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak_src = "fallback"
    if os.path.exists(mp):
        with open(mp) as f:
            hbm_peak = json.load(f).get("hbm_gbs", hbm_peak)
        peak_src = "measured"
    tb = TRAFFIC.get((op, P))
    # t_roof = max over the bounds of the work the kernel must do: HBM bytes,
    # useful flops on the FP64 pipe (none in split), on the FP32/INT pipes
    # (all of split's), on the tensor pipe (none in split)
    t_hbm = B / (hbm_peak * 1e9)
    t_fp32 = F / peaks["fp32"]
    t_roof = max(t_hbm, t_fp32)
    roof = {"bound": "hbm" if t_hbm >= t_fp32 else "fp32", "achieved": achieved_gbs, "peak": hbm_peak,
            "unit": "GB/s", "frac": t_roof / t_kernel, "traffic": tb * N if tb else None,
            "traffic_source": (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of the split kernel, "
                               f"{tb:.0f} B per translation on 65 536 translations, scaled to {N}") if tb else None,
            "peak_source": peak_src, "kernel": "k_translate<ff, G, ACC, fixed, in HBM> (split)",
            "bytes_per_translation": B, "useful_flops_per_translation": F,
            "t_roof_ns_per_translation": {"hbm": t_hbm * 1e9, "fp32_pipe": t_fp32 * 1e9, "fp64_pipe": 0.0,
                                          "tensor_pipe": 0.0},
            "frac_definition": "t_roof / t_measured, t_roof = max(bytes / HBM peak, useful FP32-pipe flops / "
                               "measured FFMA peak) per translation"}
    issue_util = None
    ipt = INSTRUCTIONS.get((op, P))
    if ipt and clk and clk.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        peak_issue = sms * 4 * clk["sm_mhz"] * 1e6
        issue_util = {"what": "issue-slot utilisation of the split kernel (a diagnostic, not a roofline: the "
                              "instructions counted include the emulation around the useful work)",
                      "instructions_per_translation": ipt, "achieved": ipt / t_kernel, "peak": peak_issue,
                      "frac": ipt / t_kernel / peak_issue,
                      "peak_source": f"{sms} SMs x 4 schedulers x 1 instruction/cycle at the sampled {clk['sm_mhz']} MHz",
                      "instructions_source": "ncu smsp__inst_executed.sum of the split kernel / 65 536 translations"}
    tc_rows = {}
    for name, ms in tc_ms.items():
        tk = ms * 1e-3 / N
        row = {"value": world * N / (ms * 1e-3), "unit": "translations/s", "ms_per_step": ms,
               "over_plain_fp64": (world * N / (ms * 1e-3)) / plain_value,
               "over_split": (world * N / (ms * 1e-3)) / value,
               "roofline": {"bound": "hbm", "frac": t_hbm / tk, "achieved_gbs": B / tk / 1e9,
                            "peak": hbm_peak, "note": "t_roof = bytes / HBM peak (the tensor and FP32 pipes need "
                                                      "far less time for the useful work)"},
               "clocks": tc_clk.get(name)}
        if acc and name in acc:
            row["accuracy_vs_fp64_oracle_1000"] = acc[name]
        tc_rows[name] = row
    # the split path does FP64-class work on the FP32 and integer pipes: its
    # useful flop rate set against the FP64 pipe's measured peak (a ratio
    # above 1 is beyond any FP64 kernel's reach)
    roof_compute = {
        "basis": "useful flops of the rotation method per translation (2 per multiply-add)",
        "useful_flops_per_translation": F,
        "achieved_tflops": F / t_kernel / 1e12,
        "fp64_peak_tflops": peaks["fp64"] / 1e12, "frac_of_fp64_peak": F / t_kernel / peaks["fp64"],
        "fp32_peak_tflops": peaks["fp32"] / 1e12, "peak_source": "measured DFMA / FFMA loops in this run"}
    roof_fp64 = {"kernel": "k_translate<double,4> (plain FP64)", "pipe": "fp64",
                 "achieved_tflops": F * plain_value / world / 1e12, "peak_tflops": peaks["fp64"] / 1e12,
                 "frac": F * plain_value / world / peaks["fp64"], "peak_source": "measured DFMA loop in this run"}
    cpu = cpu_port = None
    if not args.no_cpu:
        cpu = cpu_leg(op, P, args.cpu_seconds, 99)
        if cpu["kind"] == "reference":  # the port beside it, for continuity
            v, threads, ns, done = cpu_leg_port(op, P, min(5.0, args.cpu_seconds), 98)
            cpu_port = {"value": v, "unit": "translations/s", "cores": threads, "kind": "port",
                        "sample": f"{done} translations in passes of {ns}, oracle port, one pthread per core"}
    line = {"metric": METRIC, "value": value, "unit": "translations/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_split, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "split: int32 block fixed point (swaps, polar rotations), f32x2 float-float (z-translation, "
                     "azimuthal rotations, scaling, geometry), f64 accumulation",
            "data": "synthetic (seeded P2M of random charges)",
            "config": config,
            "plain_fp64": {"value": plain_value, "ms_per_step": ms_plain},
            "split_over_plain_fp64": value / plain_value,
            "split_ff": {"value": ff_value, "ms_per_step": ms_ff,
                         "note": "float-float throughout (relative error ~1e-13)"},
            "accuracy_vs_fp64_oracle_1000": acc,
            "physics_checks": {"what": "relative potential error r|phi - 1/r| and relative gradient error at the "
                                       "reference's own test geometries (tests/test_{m2l,m2m,l2l}.cpp), order "
                                       f"{P}, 32 translations into one target; the expansion's truncation error "
                                       "is the oracle_exact_translation row",
                               "rows": physics},
            "e2e": {"value": world * N / e2e_s, "unit": "translations/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "api": "sfmm_translate_host_packed on pinned host buffers: the kernel reads the sources and "
                           "updates the targets in place over the host link (bytes counted are those crossing it)"},
            "e2e_classic_call": {"value": world * N / classic_s, "unit": "translations/s",
                                 "api": "sfmm_translate_host: arrays of N source and target solid addresses (the "
                                        "drop-in classic and multithreaded_translator calls), in place over the "
                                        "host link"},
            "tensor_core": tc_rows or None,
            "tensor_core_note": "tcgen05 kernel, one thread per translation, 128 translations per MMA tile: swaps "
                                "and z-translations as M=128 N=K=16 MMAs with operands split in two (3xTF32, "
                                "3xBF16) or three (BF16x6) pieces, FP32 accumulation in tensor memory; the "
                                "accumulator's rounding per MMA stage keeps every mode above the 1e-7 contract, so "
                                "the headline value stays the split kernel",
            "split_m2m_note": "split M2M batches with an order bound above 18 run float-float",
            "roofline": roof, "issue_utilisation": issue_util, "roofline_compute": roof_compute,
            "roofline_plain_fp64": roof_fp64,
            "cpu_baseline": cpu, "cpu_baseline_port": cpu_port, "clocks": clk, "gpu_launches": launches}
    if world == 1 and not args.no_extras and args.workload == "m2l16":
        del src, dst, h_src, h_dst
        torch.cuda.empty_cache()
        line["configs"] = extras(args, local)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
