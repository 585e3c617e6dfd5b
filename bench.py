"""Benchmark of the Galerkin hot path on the 25k-triangle lifting wing, and of the free wake.

Workload: rectangular wing of aspect ratio 8, NACA 0012 section, 112 full-cosine chordwise x 56 full-cosine spanwise
panels per side (25,088 surface + 444 cap triangles, 12.9k unknowns), rigid wake 2.5 spans (20 chords) long along +x
with tip filaments, alpha = 5 deg. One step = assemble (all tiers) + factorize (bordered LU) + solve + loads (CL by
pressure, CDi by Trefftz) + the adjoint gradients of CL and CDi with respect to every node and alpha, through the
library, in mixed precision (FP32 far/near tiers and LU, FP64 touching tiers and refinement). The plain FP64 GPU path
is timed on the same workload for the comparison, with |dCL| and |dCDi|. The free wake line runs 500 steps of the
6,556-triangle wing at alpha 8 deg (dt 0.02, core 0.05) on the GPU and times step! at the end.

The reference arm (--impl reference) runs the reference's path on the host cores: the oracle (C++ restatement of the
assembly) and LAPACK through scipy, whole unsampled steps (no adjoint: the reference has none).

Every N > 1 rank runs an independent replica (the solve of one wing does not shard in this build).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "vortexpanel.jl_gb300"))

METRIC = "assemble+factor+solve+adjoint s at 25k tris: mixed vs FP64 GPU, |ΔCL|<1e-6"
# algorithmic flops per quadrature point: forward (kernel evaluation ~230 + contraction into the hat block 18) and
# adjoint (value and reverse-mode derivatives of the kernel ~620, once per point, + the sums of the test and source
# sides ~110 per adjoint vector; the CL and CDi vectors share one pass of every adjoint kernel)
FLOP_FWD_POINT = 248
FLOP_ADJ_EVAL = 620
FLOP_ADJ_SUMS = 110
# DRAM bytes per touching/contact point of the pair-parallel kernels, from ncu captures on the 28 x 14 per side wing
# (115.3M such points): adj_pairs_kernel 0.091 GB read + 1.308 GB written, near_kernel_pairs 0.024 + 0.390 GB. It is
# stack traffic of the walkers' frames and spills, which grows with the points; the algorithmic bytes are a few MB.
DRAM_PER_TOUCH_POINT = {"adj_pairs": 12.13, "near_pairs": 3.59}
NCHORD, NSPAN, ASPECT, ALPHA = 112, 56, 8.0, 5.0
SIZES = {"wing25k": (112, 56), "medium": (56, 28), "small": (28, 14)}  # panels per side: chordwise, spanwise


def workload(name="wing25k"):
    from vortexpanel_gpu import meshes

    global NCHORD, NSPAN
    NCHORD, NSPAN = SIZES[name]
    w = meshes.wing(NCHORD, NSPAN, aspect=ASPECT)
    wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.5)
    W = meshes.wake_rows(w.dm, wake.te)
    a = math.radians(ALPHA)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    return w, wake, W, V


def step(vp, w, wake, W, precision, ctx):
    """one pass of the hot path: assemble + factorize + solve + loads (CL by pressure, CDi by Trefftz) + the adjoint
    gradients of both with respect to every node and alpha; returns the result dict of wing_gradients"""
    from vortexpanel_gpu.adjoint import wing_gradients

    return wing_gradients(w, wake, W, math.radians(ALPHA), precision=precision, ctx=ctx)


class Clocks:
    """nvidia-smi samples of the SM clock and throttle reasons while the timed region runs"""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def nbody(vp, ctx, n=400_000, reps=3):
    """The free wake's blob N-body kernel on a synthetic cloud of n blobs at their own n positions (positions uniform
    in [0,8] x [-4,4] x [-1,1], strengths N(0,1)^3 1e-3, core 0.05, seed 1), mixed precision: interactions per second
    and its roofline (28 FP32 flops per interaction) from the kernel's device time"""
    from vortexpanel_gpu import freewake

    rng = np.random.default_rng(1)
    x = rng.uniform([0, -4, -1], [8, 4, 1], (n, 3))
    blobs = np.hstack([x, 1e-3 * rng.standard_normal((n, 3)), np.full((n, 1), 0.05)])
    freewake.blob_velocities(blobs[:1000], x[:1000], precision="mixed", ctx=ctx)
    ctx.phase_times(reset=True)
    for _ in range(reps):
        freewake.blob_velocities(blobs, x, precision="mixed", ctx=ctx)
    ph, _ = ctx.phase_times(reset=True)
    t = ph["wake"] / 1e3 / reps
    pk, _ = peaks()
    peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    ach = 28 * n * n / t / 1e12
    return {"blobs": n, "points": n, "ms": t * 1e3, "interactions_per_s": n * n / t,
            "roofline": {"kernel": "blob_kernel<float>", "bound": "fp32", "achieved": ach, "peak": peak,
                         "unit": "TFLOP/s", "frac": ach / peak, "peak_source": "nominal"}}


def cpu_step(w, wake, W, V):
    """One step of the reference's path on all host cores, unsampled: the oracle (the C++ restatement of the
    reference's assembly, OpenMP over test triangles as assemble.jl:395) assembles every row of A and b, then the
    bordered matrix, the reference's LAPACK dgetrf and dgecon through scipy, the solve, and the loads (CL by the pressure
    route, CDi by Trefftz). The reference has no adjoint (it differentiates with ForwardDiff), so the CPU step has
    none."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    sig = oracle.source_strengths(w.g, V)
    A, b, _ = oracle.assemble(w.g, w.dm, sig, V, wake=wake, nthreads=cores)
    t1 = time.perf_counter()
    sol = oracle.solve_galerkin(w.dm, A, b, W=W)
    del A
    t2 = time.perf_counter()
    els = oracle.elements(w.g)
    cp = oracle.pressure_coefficient(oracle.gradient_velocity(w.g, w.dm, sol["mu"], V, els=els), V)
    a = math.radians(ALPHA)
    S = w.span * w.chord
    CL = float(oracle.pressure_force(els, cp)[0] @ np.array([-math.sin(a), 0.0, math.cos(a)]) / S)
    CDi = float(oracle.trefftz_drag(w.dm.wake_te, w.dm.K @ sol["q"], V) / S)
    t3 = time.perf_counter()
    return {"value": t3 - t0, "unit": "s", "cores": cores, "kind": "port", "assembly_s": t1 - t0,
            "factor_solve_s": t2 - t1, "loads_s": t3 - t2, "CL": CL, "CDi": CDi}


CPU_SAMPLE = ("the whole step, unsampled: oracle assembly of all {ntri} test-triangle rows ({asm:.1f} s), bordered matrix "
              "+ scipy/LAPACK dgetrf + dgecon + solve ({fs:.1f} s), loads ({ld:.2f} s); no adjoint (the reference "
              "differentiates with ForwardDiff and has no adjoint)")


def freewake_bench(vp, ctx, steps=500):
    """The free wake of the wing of 40 x 40 panels per side (6,556 triangles), alpha = 8 deg, |V∞| = 1, dt = 0.02
    chord, particle core 0.05 chord, mixed precision, `steps` steps of the device-resident FreeWakeSim from an
    impulsive start: the time per step! at the end of the run (the last 50 steps: wall time per call and device time
    from CUDA events) at its particle count, beside the reference's published 1.8 s per step at 32,684 particles
    (its README, 16 threads)"""
    from vortexpanel_gpu import freewake as fwk

    w = vp.meshes.wing(40, 40, aspect=8.0)
    a = math.radians(8.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    eL = np.array([-math.sin(a), 0.0, math.cos(a)])
    t0 = time.perf_counter()
    sim = fwk.FreeWakeSim(w.g, w.dm, V, fwk.FreeWakeOptions(dt=0.02, core=0.05),
                          assembly=vp.AssemblyOptions(precision="mixed"), ctx=ctx, capacity=50_000)
    t_setup = time.perf_counter() - t0
    last = min(50, steps)
    t0 = time.perf_counter()
    for _ in range(steps - last):
        sim.step()
    ctx.phase_times(reset=True)
    t1 = time.perf_counter()
    for _ in range(last):
        rec = sim.step()
    t2 = time.perf_counter()
    ph, launches = ctx.phase_times(reset=True)
    S = w.span * w.chord
    return {"workload": f"wing AR8 NACA0012 40x40/side ({w.g.ntri} tris), alpha 8 deg, dt 0.02, core 0.05, mixed",
            "steps": steps, "particles": rec["particles"], "rows": rec["rows"], "setup_s": t_setup,
            "run_s": t2 - t0, "ms_per_step_wall": (t2 - t1) / last * 1e3,
            "ms_per_step_device": (ph["wake"] + ph["solve"] + ph["wake_rhs"] + ph["wake_vel"]) / last,
            "phases_ms_per_step": {k: ph[k] / last for k in ("wake_rhs", "wake_vel", "solve", "wake")},
            "launches_per_step": launches / last,
            "CL_pressure_last": float(rec["F_pressure"] @ eL / S), "CL_kj_last": float(rec["F_kj"] @ eL / S),
            "reference_published": {"ms_per_step": 1800.0, "particles": 32684,
                                    "source": "VortexPanel.jl README, free wake L2, 16 threads, author's CPU"}}


BATCH_WINGS = ((28, 18, 4.0), (36, 22, 5.0), (44, 28, 6.0), (56, 32, 7.0), (64, 40, 8.0), (80, 44, 9.0),
               (96, 50, 10.0), (112, 56, 12.0))


def batch_bench(vp, ctx, reps=2):
    """The uneven batch: 8 wings of 2,124 to 25,532 triangles, aspect ratios 4 to 12, each with its rigid wake, alpha
    5 deg, mixed precision. One vp_assemble_batch call (far tier per colour over all wings, the touching and contact
    pairs of all wings in one persistent launch) against the 8 wings assembled one after another; wall time of the
    call (host classification included) and device time (CUDA events of the library's phases), the best of reps
    after one warm-up. Throughput: pair integrals (test x source triangle pairs, wakes included) per second."""
    a = math.radians(ALPHA)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    cases = []
    for nc, ns, ar in BATCH_WINGS:
        w = vp.meshes.wing(nc, ns, aspect=ar)
        wake = vp.meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.5)
        els = vp.build_elements(w.g)
        cases.append((w.g, w.dm, vp.source_strengths(els, V), V, wake))
    opts = vp.AssemblyOptions(precision="mixed")
    pairs = sum(g.ntri * (g.ntri + len(wk.tris) + len(wk.filaments)) for g, _, _, _, wk in cases)

    def run_batch():
        out = vp.assemble_batch(cases, opts=opts, ctx=ctx)
        del out

    def run_single():
        for g, dm, sig, VV, wk in cases:
            A, b, _ = vp.assemble(g, dm, vp.build_elements(g), sig, VV, opts=opts, wake=wk, ctx=ctx)
            del A

    res = {}
    for name, fn in (("batch", run_batch), ("one_by_one", run_single)):
        fn()
        best = None
        for _ in range(reps):
            ctx.phase_times(reset=True)
            t0 = time.perf_counter()
            fn()
            wall = time.perf_counter() - t0
            ph, launches = ctx.phase_times(reset=True)
            dev = sum(ph.values()) / 1e3
            if best is None or wall < best[0]:
                best = (wall, dev, launches)
        res[name] = {"wall_s": best[0], "device_s": best[1], "launches": best[2],
                     "pairs_per_s_wall": pairs / best[0], "pairs_per_s_device": pairs / best[1]}
    return {"workload": "8 wings AR 4-12, " + ", ".join(str(c[0].ntri) for c in cases) + " tris, rigid wakes, "
                        "alpha 5 deg, mixed", "wings": len(cases), "tris": int(sum(c[0].ntri for c in cases)),
            "pair_integrals": int(pairs), **res,
            "speedup_wall": res["one_by_one"]["wall_s"] / res["batch"]["wall_s"],
            "speedup_device": res["one_by_one"]["device_s"] / res["batch"]["device_s"]}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def rooflines(per, points, adjoint_points, n, pk_src):
    """The achieved FLOP/s of every pair kernel and of the LU (n: the bordered system's order), each over its own
    CUDA-event phase (per: ms per step), and the roofline object of the dominant one"""
    # roofline of every pair kernel and of the LU (algorithmic flops per evaluated point from the device's per-tier
    # point counts, over the kernel's CUDA-event time on the library's stream); the dominant one is the headline
    pk, src = pk_src
    sm_max = pk.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s, nominal FP32 FMA rate at the max SM clock
    pts, apts = points, adjoint_points
    touch = lambda p: sum(v for k, v in p.items() if k not in ("far", "near"))  # noqa: E731  self/edge/vertex/contact
    kern = {  # phase: (kernels, bound, flops, points)
        "far": ("far_kernel<float,TT> (TT the autotuner's tile)", "fp32", pts["far"] * FLOP_FWD_POINT, pts["far"]),
        "near": ("near_kernel_lanes (+ near_kernel_rest)", "fp32", pts["near"] * FLOP_FWD_POINT, pts["near"]),
        "near_pairs": ("near_kernel_pairs", "fp32", touch(pts) * FLOP_FWD_POINT, touch(pts)),
        "adj_far": ("adj_far_kernel<float,8,2>", "fp32", apts["far"] * (FLOP_ADJ_EVAL + 2 * FLOP_ADJ_SUMS), apts["far"]),
        "adj_near": ("adj_lanes_kernel, both vectors (+ adj_near_kernel)", "fp32",
                     apts["near"] * (FLOP_ADJ_EVAL + 2 * FLOP_ADJ_SUMS), apts["near"]),
        "adj_pairs": ("adj_pairs_kernel<AdjAccW>", "fp32", touch(apts) * (FLOP_ADJ_EVAL + 2 * FLOP_ADJ_SUMS), touch(apts)),
        "lu": ("lu (cluster leaf panels + tcgen05 bf16x3 trailing updates)", "fp32", 2 / 3 * n ** 3, None),
    }
    kernels = {}
    for ph, (name, bound, flops, npts) in kern.items():
        if per.get(ph, 0.0) <= 0:
            continue
        peak = fp32_peak if bound == "fp32" else pk.get("bf16_tflops", 1900.0)
        ach = flops / (per[ph] / 1e3) / 1e12
        kernels[ph] = {"kernel": name, "ms": per[ph], "achieved": ach, "frac": ach / peak}
    dom = max(kernels, key=lambda k: per[k])
    name, bound, flops, npts = kern[dom]
    roof = {"kernel": name, "bound": bound, "achieved": kernels[dom]["achieved"],
            "peak": fp32_peak if bound == "fp32" else pk.get("bf16_tflops", 1900.0), "unit": "TFLOP/s"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["peak_source"] = "nominal (152 SMs x 128 FP32 lanes x 2 x max SM clock)" if bound == "fp32" else src
    traffic = DRAM_PER_TOUCH_POINT.get(dom)
    roof["traffic"] = traffic * npts if traffic is not None and npts else None
    roof["traffic_unit"] = "B per launch (ncu, small wing, scaled by points)" if roof["traffic"] else None
    return kernels, roof


def max_over_ranks(vals, dist):
    """each value's largest over the ranks (the slowest replica sets the step time); the values themselves on one rank"""
    if not dist:
        return [float(v) for v in vals]
    import torch

    t = torch.tensor([float(v) for v in vals], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--freewake-steps", type=int, default=500)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--workload", default="wing25k", choices=list(SIZES),
                    help="wing25k (the measured configuration); medium (56x28 per side) and small (28x14) for profiler captures")
    args = ap.parse_args()
    rank, world, local, dist = dist_setup(args.gpus)
    w, wake, W, V = workload(args.workload)
    config = {"workload": f"wing AR{ASPECT:g} NACA0012 {NCHORD}x{NSPAN}/side ({w.g.ntri} tris, {w.dm.nq} unknowns), "
                          f"rigid wake {len(wake.tris)} tris + {len(wake.filaments)} filaments, alpha {ALPHA:g} deg",
              "ntri": w.g.ntri, "nq": w.dm.nq, "nwake_nodes": wake.nwake, "precision": "mixed",
              "l2": ("inputs larger than L2" if 8 * w.dm.nslot * (w.dm.nslot + wake.nwake) > 129e6 else "inputs within L2") +
                    f" (A is {8 * w.dm.nslot * (w.dm.nslot + wake.nwake) / 1e9:.2f} GB FP64)",
              "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        # the reference's path on the host cores, whole steps of about half a minute each: at most one untimed and
        # three timed, so that the run ends in a few minutes whatever --steps and --warmup ask for
        nw, nt = min(1, args.warmup), min(3, max(1, args.steps))
        for _ in range(nw):
            cpu_step(w, wake, W, V)
        runs = [cpu_step(w, wake, W, V) for _ in range(nt)]
        cb = dict(runs[-1], value=statistics.mean(r["value"] for r in runs))
        sample = CPU_SAMPLE.format(ntri=w.g.ntri, asm=cb["assembly_s"], fs=cb["factor_solve_s"], ld=cb["loads_s"])
        sample += f"; {nt} timed steps after {nw} untimed (asked for {args.steps} and {args.warmup})"
        line = {"metric": METRIC, "value": cb["value"], "unit": "s", "n_gpus": world, "steps": nt,
                "warmup": nw, "requested_steps": args.steps, "requested_warmup": args.warmup,
                "ms_per_step": cb["value"] * 1e3, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": config, "impl": "reference",
                "cpu_baseline": {"value": cb["value"], "unit": "s", "cores": cb["cores"], "kind": "port",
                                 "sample": sample},
                "CL": cb["CL"], "CDi": cb["CDi"],
                "e2e": {"value": cb["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import vortexpanel_gpu as vp

    ctx = vp.Context(local)
    for _ in range(args.warmup):
        step(vp, w, wake, W, "mixed", ctx)
    ctx.phase_times(reset=True)
    ctx.transfer_bytes(reset=True)
    if dist:
        dist.barrier()
    walls = []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            out = step(vp, w, wake, W, "mixed", ctx)
            walls.append(time.perf_counter() - t0)
    if dist:
        dist.barrier()
    phases, launches = ctx.phase_times(reset=True)
    h2d, d2h = ctx.transfer_bytes(reset=True)
    dev_s = sum(phases.values()) / 1e3 / args.steps
    e2e_s = sum(walls) / args.steps
    dev_s, e2e_s = max_over_ranks([dev_s, e2e_s], dist)
    CL, CDi, stats, cond = out["CL"], out["CDi"], out["stats"], out["cond"]
    # the plain FP64 GPU path on the same workload
    fp = {}
    if args.fp64_steps > 0:
        step(vp, w, wake, W, "fp64", ctx)
        ctx.phase_times(reset=True)
        fw = []
        for _ in range(args.fp64_steps):
            t0 = time.perf_counter()
            o64 = step(vp, w, wake, W, "fp64", ctx)
            fw.append(time.perf_counter() - t0)
        ph64, _ = ctx.phase_times(reset=True)
        grel = {n: float(np.abs(out[f"d{n}_dx"] - o64[f"d{n}_dx"]).max() / np.abs(o64[f"d{n}_dx"]).max())
                for n in ("CL", "CDi")}
        fp = {"fp64_s": sum(ph64.values()) / 1e3 / args.fp64_steps, "fp64_e2e_s": sum(fw) / len(fw),
              "fp64_phases_ms": {k: v / args.fp64_steps for k, v in ph64.items()},
              "CL_fp64": o64["CL"], "CDi_fp64": o64["CDi"], "dCL": abs(CL - o64["CL"]), "dCDi": abs(CDi - o64["CDi"]),
              "grad_rel_diff_vs_fp64": grel,
              "dalpha_rel_diff_vs_fp64": {n: abs(out[f"d{n}_dalpha"] - o64[f"d{n}_dalpha"]) / abs(o64[f"d{n}_dalpha"])
                                          for n in ("CL", "CDi")}}
        fp["speedup_vs_fp64"] = fp["fp64_s"] / dev_s
        fp["e2e_speedup_vs_fp64"] = fp["fp64_e2e_s"] / e2e_s
    if rank != 0:
        return
    per = {k: v / args.steps for k, v in phases.items()}
    kernels, roof = rooflines(per, stats["points"], out["adjoint_points"], w.dm.nq + 1, peaks())
    line = {"metric": METRIC, "value": dev_s, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_s * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "config": config,
            "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps},
            "gpu_launches": launches // args.steps * args.steps, "phases_ms": per,
            "CL": CL, "CDi": CDi, "cond": cond, "tiers": stats, "roofline": roof, "clocks": clk.summary(),
            "fp64_point_share": stats["points_fp64"] / max(1, sum(stats["points"].values())),
            "adjoint_points": out["adjoint_points"],
            "adjoint_fp64_point_share": out["adjoint_points_fp64"] / max(1, sum(out["adjoint_points"].values())),
            "kernels": kernels}
    line.update(fp)
    line["nbody"] = nbody(vp, ctx)
    if args.freewake_steps > 0:
        line["freewake"] = freewake_bench(vp, ctx, args.freewake_steps)
    if not args.no_batch:
        line["batch"] = batch_bench(vp, ctx)
    if not args.no_cpu_baseline:
        cb = cpu_step(w, wake, W, V)
        line["cpu_baseline"] = {"value": cb["value"], "unit": "s", "cores": cb["cores"], "kind": "port",
                                "sample": CPU_SAMPLE.format(ntri=w.g.ntri, asm=cb["assembly_s"],
                                                            fs=cb["factor_solve_s"], ld=cb["loads_s"]) +
                                "; one step"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
