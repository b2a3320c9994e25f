#!/usr/bin/env python
"""Benchmark of the GB300 subjective-surfaces segmentation solver.

Metric: time-steps/s of the semi-implicit segmentation at 256x256x128x20
(the multi-object drifting scene), every step solved by red-black SOR to the
FP64 residual tolerance sum r^2 h^4 <= 1e-6.  A "step" is one time step:
coefficient assembly, the SOR solve, the per-step rescale.  Inputs (about
25 GB of working set) are far larger than the 129 MB L2, so no flush is
needed between steps.

Prints ONE JSON line on rank 0.  `--impl reference` times the reference's
CPU algorithm instead (the compiled reference where it runs, else the C
oracle that restates it), on all host cores.

Multi-GPU: N ranks run N independent volumes ("replicas", weak scaling);
`value` is the steps of all ranks over the slowest rank's time.  Splitting
one volume across ranks by frames (the library's t-slab entry points,
ss4d_slab_*) is not what this benchmark times.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "4d-image-segmentation-algorithm_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "time-steps/s @256²×128×20 to FP64 res 1e-6: mixed+learned vs plain FP64; HBM %"
WORKLOAD = ("segmentation time steps, 256x256x128x20 multi-object drifting scene (3 ellipsoids, noise 30, 10% "
            "boundary erasure), K=1000, eps2=1e-3, tau=0.5, omega=1.8, gsTol=1e-6")
# algorithmic bytes per interior voxel (each reference array touched once)
BYTES_FP64_ITER = 88.0  # read u, prev, 8 coefficients; write u
# FP32 correction sweep: the 20-byte record (8 16-bit fractions + FP32 scale),
# right-hand side, correction read and written (44 B with 8 FP32 coefficients)
BYTES_FP32_ITER = 32.0
# DRAM bytes per target voxel of one half-sweep launch (dram__bytes_read.sum +
# dram__bytes_write.sum from ncu), scaled by the targets of a launch at the
# benchmarked size: k_sweep32 from two launches at 256x256x128x20
# (83,886,080 targets; a one-pass capture), k_sweep64 from one launch at
# 128x128x64x8 (4,194,304 targets)
EXTRAP_ORDER = 3  # the extrap form's order (ss4d_solver_set_extrapolation)
# one step's coefficient assembly (_gs_coefficients_ with the prev_u copy):
# read u and the 8 g faces, write the 8 coefficients, copy u to prev
BYTES_ASSEMBLY = 152.0
# DRAM bytes per interior voxel of the mixed form's three assembly kernels
# (first differences with the pack, faces, coefficient records with the first
# refinement pass's residual), one ncu capture at 128x128x64x8: 82.7 + 142.9
# + 190.5 (the first-difference kernel's 62.2 B per padded voxel counted per
# interior voxel)
TRAFFIC_ASSEMBLY = 416.1
TRAFFIC_PER_TARGET = {"k_sweep32": 39.8, "k_sweep64": 118.6}
FP64_INSTR_PER_TARGET = 11.4  # k_sweep64, ncu at 128x128x64x8
TRAFFIC_SOURCE = {"k_sweep32": "ncu capture of two launches at 256x256x128x20",
                  "k_sweep64": "ncu capture of one launch at 128x128x64x8"}
# the forms the metric names: FP32 sweeps with FP64 refinement started from
# the learned warm start (from u^n, or at the extrapolated start)
NAMED_FORMS = ("learned", "learned_x")
FORM_LABEL = {"fp64": "plain FP64 sweeps", "mixed": "mixed (FP32 sweeps, FP64 residual/refinement)",
              "extrap": "mixed + cubic extrapolated start (no network)",
              "proj": "mixed + cubic extrapolated start, first round projected onto the earlier changes (no network)",
              "learned": "mixed + learned warm start (the metric's named form)",
              "learned_x": "mixed + learned warm start at the extrapolated start (the metric's named form)",
              "extrap_w": "mixed + extrapolated start, FP32 sweeps relaxed by --inner-omega (reported only)"}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, nargs=4, default=[256, 256, 128, 20], metavar=("NX", "NY", "NZ", "NT"))
    ap.add_argument("--forms", default="fp64,mixed,extrap,proj,learned,learned_x,extrap_w",
                    help="fp64: plain FP64 sweeps; mixed: FP32 sweeps + FP64 refinement; extrap: mixed started "
                         "from the cubic extrapolation u^n + 3 d_(n-1) - 3 d_(n-2) + d_(n-3) of the earlier "
                         "changes; proj: extrap whose first FP32 round starts from the least-residual combination "
                         "of the last changes and the extrapolation; learned: mixed started from the warm-start network (weights/wsnet_seg.npy); "
                         "learned_x: the learned warm start at the extrapolated start (the network predicts the "
                         "correction the extrapolation leaves), run while it pays (--ws-gate); "
                         "extrap_w: extrap with --inner-omega")
    ap.add_argument("--ws-gate", type=int, default=0,
                    help="learned_x: run the network in a step only when the previous step took at least this many "
                         "FP32 sweeps (0: every step)")
    ap.add_argument("--inner-omega", type=float, default=1.2,
                    help="relaxation factor of the extra form 'extrap_w' (extrap with its FP32 sweeps relaxed by "
                         "this instead of the configured omega 1.8; reported, never the headline)")
    ap.add_argument("--assembly-order", type=int, default=None, metavar="PLANES",
                    help="block order of the mixed form's assembly kernels (0 frame by frame, n >= 1 in blocks of "
                         "n k planes across the frames; default: the library's)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="leave out the short batched-workload measurement (16 uneven volumes, FP64 and mixed + "
                         "extrapolation, 10 steps after 3) that the default line carries as `batch`")
    ap.add_argument("--no-frontend", action="store_true",
                    help="skip the timing of the work around the time loop (thresholding, edge detector, ...)")
    ap.add_argument("--no-graph", action="store_true",
                    help="run the sweep loop host-driven instead of as one CUDA graph (same kernels)")
    ap.add_argument("--workload", choices=["single", "batch", "conv"], default="single",
                    help="batch: 16 uneven volumes, the SOR loop of all of them in one launch (reports "
                         "voxel-updates/s; not the headline metric); conv: the warm-start network's forward "
                         "(four tensor-core convolutions) on random features of --size (reports TFLOP/s; for "
                         "profiling)")
    ap.add_argument("--batch-config", choices=["16x_64-192", "48x_24-48"], default="16x_64-192",
                    help="batch workload: the configuration's 16 volumes, or 48 small ones")
    ap.add_argument("--batch-sequential", action="store_true",
                    help="batch workload: also time the same volumes solved one after another")
    ap.add_argument("--batch-loop", choices=["persistent", "graph"], default="persistent",
                    help="batch workload: the SOR loop of all volumes as one persistent launch (default) or as a "
                         "CUDA graph's while loop of per-phase kernels")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--steps100", type=int, default=100,
                    help="every form also runs on from the timed window to this many time steps from u0 (the "
                         "headline configuration's 100 steps) and reports their average rate (0: skip)")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.tmp,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as fh:
            for ln in fh:
                f = [x.strip() for x in ln.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        # samples while the GPU is busy (the upper half of the observed clocks)
        busy = sorted(sm)[len(sm) // 2:] if sm else []
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max([num(r[3]) for r in rows if num(r[3])] or [0])}


# --------------------------------------------------------------------------
# our arm

def fp64_peak_flops(device) -> float | None:
    """FP64 FLOP/s of a cuBLAS DGEMM (4096^3, best of 3) on this GPU: the
    measured ceiling of the FP64 pipe, beside the copy bandwidth"""
    try:
        import torch
        a = torch.randn((4096, 4096), dtype=torch.float64, device=device)
        b = torch.randn_like(a)
        torch.matmul(a, b)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = None
        for _ in range(3):
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize(device)
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        del a, b
        return 2.0 * 4096 ** 3 / (best / 1e3)
    except Exception:
        return None


def slowest_rank_ms(ms: float, dist, device) -> float:
    """The timed region's duration of the slowest rank (ranks = independent
    replicas); every rank returns the same value."""
    if not dist:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def replica_steps_per_s(steps: int, world: int, ms: float) -> float:
    """Whole-job throughput: every rank steps its own volume `steps` times."""
    return steps * world / (ms / 1e3)


def run_ours(args, rank, world, dist):
    import numpy as np
    import torch

    import ss4d

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    nx, ny, nz, nt = args.size
    p = ss4d.scene_params(maxNoOfTimeSteps=args.steps + args.warmup)
    i0h, u0h = ss4d.scene(3, nx, ny, nz, nt, seed=args.seed + rank, threads=os.cpu_count() or 1)
    shape = i0h.shape
    n_pad = int(np.prod(shape))
    n_int = nx * ny * nz * nt
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    i0 = torch.from_numpy(i0h).to(dev)
    g = [torch.empty(shape, dtype=torch.float64, device=dev) for _ in range(8)]
    S = ss4d.Solver(*shape[::-1], arith="fp64", stream=sh)
    S.set_graph(not args.no_graph)
    S.edge_detector(p, i0, None, g)  # i0 is now the presmoothed image
    S.synchronize()
    u0 = torch.from_numpy(u0h).to(dev)

    forms = [f for f in args.forms.split(",") if f]
    net = None
    if "learned" in forms or "learned_x" in forms:
        net = ss4d.Wsnet(stream=sh, seed=None)
        net.set_params(np.load(os.path.join(PKG, "weights", "wsnet_seg.npy")))

    def use_form(form):
        S.set_arith("mixed" if form in ("learned", "learned_x", "extrap", "proj", "extrap_w") else form)
        S.set_warm_start(net if form in ("learned", "learned_x") else None, i0)
        S.set_warm_start_gate(args.ws_gate if form == "learned_x" else 0)
        S.set_extrapolation(EXTRAP_ORDER if form in ("extrap", "proj", "extrap_w", "learned_x") else 0)
        S.set_projection(form == "proj")
        S.set_inner_omega(args.inner_omega if form == "extrap_w" else 0.0)
        if args.assembly_order is not None:
            S.set_assembly_order(args.assembly_order)

    results = {}
    finals = {}
    first_fp64 = None  # u after the plain FP64 form's first step (parity against the oracle's step)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def timed_step(u):
        """one time step, its device time (CUDA events on the stream)"""
        ev[0].record(stream)
        st = S.seg_time_step(p, u, None, g)
        ev[1].record(stream)
        ev[1].synchronize()
        return st, ev[0].elapsed_time(ev[1])

    for form in forms:
        use_form(form)
        u = u0.clone()
        its = []
        per_step = []  # (ms, iterations) of every step from u0
        for n in range(args.warmup):
            st, ms1 = timed_step(u)
            per_step.append((ms1, st["iterations"]))
            its.append(st["iterations"])
            if form == "fp64" and n == 0 and rank == 0:
                first_fp64 = (u.cpu().numpy(), st)
        launches0 = S.launch_count()
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        clk = Clocks(dev.index)
        clk.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        steps = []
        for _ in range(args.steps):
            st = S.seg_time_step(p, u, None, g)
            steps.append(st)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        clocks = clk.stop()
        ms = slowest_rank_ms(ms, dist, dev)
        launches = S.launch_count() - launches0
        # the timed steps' own times are not taken apart: their mean stands in
        per_step += [(ms / args.steps, s["iterations"]) for s in steps]
        while len(per_step) < args.steps100:
            st, ms1 = timed_step(u)
            per_step.append((ms1, st["iterations"]))
            if not (st["residual"] <= p.gsTol or st["iterations"] >= p.maxNoGSIteration):
                steps.append(st)  # counted against `converged`
        ok = all(s["residual"] <= p.gsTol or s["iterations"] >= p.maxNoGSIteration for s in steps)
        results[form] = {
            "steps_per_s": replica_steps_per_s(args.steps, world, ms),
            "ms_per_step": ms / args.steps,
            "iterations_per_step": statistics.mean(s["iterations"] for s in steps),
            "iterations": [s["iterations"] for s in steps],
            "refinements_per_step": statistics.mean(s["refinements"] for s in steps),
            "warm_started_steps": sum(s["warm_started"] for s in steps),
            "projected_steps": sum(s["projected"] for s in steps),
            "max_residual": max(s["residual"] for s in steps),
            "converged": ok,
            "launches": launches,
            "clocks": clocks,
        }
        if args.steps100 > 0:
            head = per_step[:args.steps100]
            tot = sum(m for m, _ in head)
            ok100 = all(s["residual"] <= p.gsTol or s["iterations"] >= p.maxNoGSIteration for s in steps)
            results[form]["steps100"] = {
                "steps": len(head), "steps_per_s": len(head) / (tot / 1e3), "ms_per_step": tot / len(head),
                "iterations_mean": statistics.mean(z for _, z in head),
                "iterations_first_last": [head[0][1], head[-1][1]], "converged": ok100,
                "how": f"steps 1..{len(head)} from u0: per-step CUDA events outside the timed window, the timed "
                       f"window's mean inside it"}
        finals[form] = u

    # per-kernel device time (CUDA events on the launching stream), one more
    # step per form with timing on: the roofline of the dominant kernel
    roof = {}
    for form in forms:
        use_form(form)
        u = finals[form].clone()
        if form in ("extrap", "proj", "extrap_w", "learned_x"):  # untimed steps rebuild the history
            for _ in range(EXTRAP_ORDER):
                S.seg_time_step(p, u, None, g)
        S.set_timing(True)
        S.reset_timing()
        S.seg_time_step(p, u, None, g)
        kt = S.kernel_times()
        S.set_timing(False)
        roof[form] = kt
    hbm, how = peaks()
    fp64_peak = fp64_peak_flops(dev)

    def roofline(form):
        kt = roof[form]
        if form == "mixed":
            ms, n = kt["sweep32"]
            per_unit = BYTES_FP32_ITER
        elif form in ("learned", "learned_x", "extrap", "proj", "extrap_w"):
            ms, n = kt["sweep32"]
            per_unit = BYTES_FP32_ITER
        else:
            ms, n = kt["sweep64"]
            per_unit = BYTES_FP64_ITER
        if n == 0:
            return None
        per_launch = per_unit * (n_int / 2.0)  # a launch updates one colour: half the voxels
        avg = ms / n
        ach = per_launch / (avg / 1e3) / 1e9
        tot = sum(v[0] for v in kt.values())
        kern = "k_sweep64" if form == "fp64" else "k_sweep32"
        fp64 = None
        if kern == "k_sweep64" and fp64_peak:
            # the FP64 pipe: instructions per target from ncu against the
            # DGEMM rate (one fused multiply-add = two flops)
            rate = FP64_INSTR_PER_TARGET * (n_int / 2.0) / (avg / 1e3)
            fp64 = {"instr_per_target": FP64_INSTR_PER_TARGET, "achieved_instr_per_s": rate,
                    "peak_fma_per_s": fp64_peak / 2.0, "frac": rate / (fp64_peak / 2.0),
                    "peak_source": "torch float64 matmul 4096^3 on this GPU (cuBLAS DGEMM), best of 3",
                    "instr_source": "ncu smsp FP64 instructions of one launch at 128x128x64x8 / targets: 8 stencil "
                                    "FMAs, 2 for the update, 1 for the residual, 0.4 for the black residual scale"}
        return {"bound": "hbm", "kernel": kern, "achieved": ach,
                "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_source": how,
                "traffic": TRAFFIC_PER_TARGET[kern] * (n_int / 2.0),
                "traffic_source": f"{TRAFFIC_SOURCE[kern]}: {TRAFFIC_PER_TARGET[kern]} DRAM B/target x targets per "
                                  f"launch",
                "avg_launch_ms": avg, "launches": n, "bytes_per_launch": per_launch,
                "share_of_step_kernel_time": (ms / tot) if tot else None,
                "kernel_ms": {k: v[0] for k, v in kt.items()}, "fp64_pipe": fp64}

    def roofline_assembly(form):
        """the mixed form's coefficient assembly of one step (three kernels,
        timed together) against the copy bandwidth, with its algorithmic bytes"""
        ms, n = roof[form]["assemble"]
        if n == 0:
            return None
        avg = ms / n
        ach = BYTES_ASSEMBLY * n_int / (avg / 1e3) / 1e9
        return {"bound": "hbm", "kernels": "k_fdiff<2> + k_faces_ff + k_voxel_coef_ff<1>", "achieved": ach,
                "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_source": how,
                "bytes_per_voxel": BYTES_ASSEMBLY, "traffic": TRAFFIC_ASSEMBLY * n_int,
                "traffic_source": f"ncu capture of the three kernels at 128x128x64x8: {TRAFFIC_ASSEMBLY} DRAM "
                                  f"B/voxel x voxels",
                "avg_ms_per_step": avg,
                "note": "float-float arithmetic on the FP32 pipe; beyond the algorithmic bytes the kernels move "
                        "their intermediates (first differences, face quantities), the FP32 sweep records, the "
                        "split copies of u and the first refinement pass's residual; the coefficient kernel is "
                        "bound by the FP64 pipe (18 FP64 instructions per voxel), the faces kernel by issue"}

    # error of the mixed forms against the plain FP64 form after the same steps
    err = {}
    for form in ("mixed", "extrap", "proj", "extrap_w", "learned", "learned_x"):
        if "fp64" not in finals or form not in finals:
            continue
        a = finals[form][1:-1, 1:-1, 1:-1, 1:-1]
        b = finals["fp64"][1:-1, 1:-1, 1:-1, 1:-1]
        d = (a - b)
        lev = 0.5 * (b.min() + b.max())
        ma, mb = a >= lev, b >= lev
        inter = (ma & mb).sum().item()
        dice = 2.0 * inter / max(1, ma.sum().item() + mb.sum().item())
        err[form] = {"max_abs": d.abs().max().item(), "max_rel": (d.abs().max() / b.abs().max()).item(),
                     "rel_l2": (d.norm() / b.norm()).item(), "mask_dice": dice,
                     "mask_level": "(min+max)/2 of fp64 u"}
    S.close()
    if net is not None:
        net.close()
    return results, roofline, roofline_assembly, err, (shape, n_pad, n_int, p, i0h, u0h, first_fp64)


def frontend_balls(nx, ny, nz, nt, seed, per_frame=5, radius=8.0):
    """Seeded ball centres for the front-end measurement: `per_frame` per
    frame, integral coordinates, every ball box inside the array (the reference
    main's radius 8 and 4 to 7 centres per frame, segmentation4D.c:1337-1348)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    lo = int(radius) + 2
    return [(l, float(rng.integers(lo, nx - lo + 1)), float(rng.integers(lo, ny - lo + 1)),
             float(rng.integers(lo, nz - lo + 1))) for l in range(1, nt + 1) for _ in range(per_frame)]


def run_frontend(args, ctx, arith="fp64"):
    """The reference main's work around the time loop (segmentation4D.c:
    1380-1393: local thresholding, edge detector on both images, initial
    function, rescale; frame conversion for reading and writing; the explicit
    smoother) on the benchmarked volume with the reference main's front-end
    parameters (radius-8 balls, alpha 0.85, beta 0.15, theta_img = rho_thr =
    0.5).  Each component: one untimed call, then the median of 3 calls timed
    with CUDA events on the launching stream (inputs restored between calls,
    outside the timed region); algorithmic bytes per call and the fraction of
    the measured copy bandwidth, in the arithmetic form `arith` (fp64: the
    reference's FP64 rounding; mixed: the edge detector in float-float).  The
    C oracle times the same sequence on a two-frame sample of the volume on
    all host cores (with arith == "fp64" only)."""
    import numpy as np
    import torch

    import oracle
    import ss4d

    shape, n_pad, n_int, p0, i0h, u0h, _ = ctx
    nx, ny, nz, nt = args.size
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    stream = torch.cuda.current_stream(dev)
    hbm, how = peaks()
    R = 8.0
    p = ss4d.scene_params(ballRadius=R, theta_img=0.5, rho_thr=0.5)
    balls = frontend_balls(nx, ny, nz, nt, args.seed)
    box = (2 * int(R) + 2) ** 3  # voxels of one ball's box (R = 8: 18^3)
    fb = torch.from_numpy(np.rint(i0h[1:-1, 1:-1, 1:-1, 1:-1] * 255.0).astype(np.uint8)).to(dev)
    i0 = torch.from_numpy(i0h).to(dev)
    u0 = torch.from_numpy(u0h).to(dev)
    img, thr, u, mm = (torch.empty_like(i0) for _ in range(4))
    g = [torch.empty_like(i0) for _ in range(8)]
    scratch = torch.empty_like(i0)
    out = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ss4d.Solver(*shape[::-1], arith=arith, stream=stream.cuda_stream) as S:

        def measure(name, setup, fn, bytes_per_call, note):
            """bytes_per_call: a number, or a function of fn's last result"""
            setup()
            fn()
            ts = []
            for _ in range(3):
                setup()
                torch.cuda.synchronize(dev)
                e0.record(stream)
                r = fn()
                e1.record(stream)
                torch.cuda.synchronize(dev)
                ts.append(e0.elapsed_time(e1))
            ms = statistics.median(ts)
            nb = bytes_per_call(r) if callable(bytes_per_call) else bytes_per_call
            gbs = nb / (ms / 1e3) / 1e9
            out[name] = {"ms": ms, "bytes": nb, "GB/s": gbs, "frac": gbs / hbm, "bytes_counted": note}
            return r

        def restore(*pairs):
            def f():
                for dst, src in pairs:
                    dst.copy_(src)
            return f

        measure("frames_from_bytes", lambda: None,
                lambda: [S.frame_from_bytes(img, l, fb[l - 1]) for l in range(1, nt + 1)],
                9.0 * n_int, "1 B read + 8 B written per interior voxel")
        z = measure("presmooth_implicit", restore((img, i0)),
                    lambda: S.presmooth_step(p, img, scratch)["iterations"], lambda z: (16.0 + 40.0 * z) * n_int,
                    "copy 16 B + per iteration 24 B (two half-sweeps: read u, prev, write u) + 16 B (residual: "
                    "read u, prev) per voxel")
        out["presmooth_implicit"]["iterations"] = z
        measure("presmooth_explicit", restore((img, i0)), lambda: S.presmooth_explicit(p, 1, img, scratch),
                32.0 * n_int, "copy 16 B + read prev 8 B + write u 8 B per voxel")
        measure("gaussian_sigma1_xyz", restore((img, i0)), lambda: S.gaussian_smooth((1.0, 1.0, 1.0, 0.0), img, scratch),
                64.0 * n_int, "3 axis passes (read 8 B + write 8 B per voxel each) + copy back 16 B per voxel")
        measure("max4d", lambda: None, lambda: S.max4d(i0), 8.0 * n_pad, "8 B read per voxel")
        measure("local_threshold", restore((thr, u0)), lambda: S.local_threshold(0.85, 0.15, R, i0, thr, balls),
                8.0 * n_pad + 24.0 * box * len(balls), "max4d pass + per ball box: min/max read, threshold read "
                                                      "and write")
        measure("edge_detector", restore((img, i0), (thr, u0)), lambda: S.edge_detector(p, img, thr, g, scratch),
                (2 * (16.0 + 40.0 * z) + 80.0) * n_int, "two presmoothings as above + g faces: read 2 images, "
                                                      "write 8 faces")
        measure("initial_function", restore((u, u0), (mm, torch.zeros_like(u0))),
                lambda: S.generate_segm_function(R, u, mm, balls), 24.0 * box * len(balls),
                "per ball box: read u, write u and Mmask")
        measure("rescale", restore((u, u0)), lambda: S.rescale_to_zero_one(p, u, mm, balls),
                24.0 * box * len(balls) + 24.0 * n_int, "per ball box: min/max read, rescale read and write; "
                                                       "Mmask pass: read u, Mmask, write u")
        measure("frames_to_bytes", lambda: None,
                lambda: [S.frame_to_bytes(u, l, fb[l - 1], 1) for l in range(1, nt + 1)],
                9.0 * n_int, "8 B read + 1 B written per interior voxel")
    del img, thr, u, mm, g, scratch, i0, u0, fb
    torch.cuda.empty_cache()
    total = sum(v["ms"] for k, v in out.items() if k in ("local_threshold", "edge_detector", "initial_function",
                                                          "rescale"))
    res = {"workload": f"{nx}x{ny}x{nz}x{nt}, {len(balls)} balls of radius {R:g} (5 per frame)", "arith": arith,
           "peak": hbm, "peak_source": how, "components": out, "main_front_end_ms": total,
           "gpu_ms_per_frame": total / nt}
    if arith != "fp64":
        return res

    # the oracle on a two-frame sample: the same front-end sequence
    ntc = 2
    ci0, cu0 = ss4d.scene(3, nx, ny, nz, ntc, seed=args.seed, threads=os.cpu_count() or 1)
    cb = frontend_balls(nx, ny, nz, ntc, args.seed)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    cthr = cu0.copy()
    oracle.local_threshold(0.85, 0.15, R, ci0, cthr, cb)
    oracle.edge_detector(p, ci0, cthr)
    cmm = np.zeros_like(cu0)
    oracle.generate_segm(R, cu0, cmm, cb)
    oracle.rescale(R, cu0, cmm, cb)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    res["cpu"] = {"ms": cpu_ms, "frames": ntc, "ms_per_frame": cpu_ms / ntc, "cores": threads, "kind": "port",
                  "sequence": "local threshold, edge detector, initial function, rescale"}
    return res


def run_e2e(args, form, ctx):
    """The same steps through the reference-named layer (libss4d_seg.so) with
    host arrays, as a reference driver calls it: every _segTimeStep_() uploads
    u and Mmask and downloads u (page-locked host memory; Mmask beside the
    solve, prev_u <- u copied on the host meanwhile)."""
    import ctypes as C

    import numpy as np

    import ss4d

    shape, n_pad, n_int, p, i0h, u0h, _ = ctx
    os.environ["SS4D_ARITH"] = "mixed" if form in ("extrap", "proj") else form
    os.environ["SS4D_EXTRAPOLATE"] = str(EXTRAP_ORDER) if form in ("extrap", "proj") else "0"
    os.environ["SS4D_PROJECT"] = "1" if form == "proj" else "0"
    L = C.CDLL(ss4d.SEG_PATH, mode=os.RTLD_LOCAL)
    lM, kM, jM, iM = shape
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM), ("maxNoGSIteration", p.maxNoGSIteration),
                  ("maxNoOfTimeSteps", p.maxNoOfTimeSteps)):
        C.c_int.in_dll(L, nm).value = int(v)
    for nm in ("K", "eps2", "tau", "h", "omega_c", "gsTol", "segTol", "sigma", "omega_sigma",
               "maxNoGSIteration_sigma", "theta_img", "rho_thr", "ballRadius"):
        C.c_double.in_dll(L, nm).value = float(getattr(p, nm))
    noc = (C.c_int * lM)()
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    L._allocateMem_.restype = C.c_bool
    L._segTimeStep_.restype = C.c_bool
    L._gf_inputImage_plus_thresholdedImage_.restype = C.c_bool
    assert L._allocateMem_()

    def arr(name):
        addr = C.c_void_p.in_dll(L, name).value
        return np.ctypeslib.as_array((C.c_double * n_pad).from_address(addr)).reshape(shape)

    i0, u, mm = arr("i0"), arr("u"), arr("Mmask")
    i0[...] = i0h
    mm[...] = 1.0
    assert L._gf_inputImage_plus_thresholdedImage_(C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
    u[...] = u0h
    for _ in range(args.warmup):
        assert L._segTimeStep_()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert L._segTimeStep_()
    dt = time.perf_counter() - t0
    L._deallocateMem_()
    nbytes = 8 * n_pad
    return {"value": args.steps / dt, "unit": "time-steps/s", "h2d_bytes_per_step": 2 * nbytes,
            "d2h_bytes_per_step": nbytes, "path": "libss4d_seg.so _segTimeStep_() on host arrays (u, Mmask up, "
                                                  "Mmask beside the solve; u down; prev_u <- u on the host)",
            "form": form}


# --------------------------------------------------------------------------
# CPU: the reference's algorithm on the host cores

def cpu_kind():
    """'reference' when the reference compiled from its own sources loads
    on this host, else 'port' (the C oracle restating it)."""
    import ctypes as C
    ref = os.path.join(ROOT, "oracle", "_ref", "libref_seg.so")
    if os.path.exists(ref):
        try:
            C.CDLL(ref, mode=os.RTLD_LOCAL)
            return "reference"
        except OSError:
            pass
    return "port"


def cpu_model() -> str:
    """the host CPU's model name (lscpu, else /proc/cpuinfo)"""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as fh:
            for ln in fh:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_steps(size, seed, warmup, steps, threads, keep_u=False):
    """Time `steps` segmentation time steps of the oracle (after `warmup`)
    on `threads` cores (the edge detector before them on every core,
    untimed); returns (seconds per step, iterations, u or None)."""
    import numpy as np

    import oracle
    import ss4d

    nx, ny, nz, nt = size
    p = ss4d.scene_params()
    i0, u = ss4d.scene(3, nx, ny, nz, nt, seed=seed, threads=os.cpu_count() or 1)
    oracle.set_threads(os.cpu_count() or 1)
    g, _, _ = oracle.edge_detector(p, i0, np.zeros_like(i0))
    del i0
    oracle.set_threads(threads)
    prev = np.zeros_like(u)
    mm = np.ones_like(u)
    coef = oracle.new_like(u, 8)
    for _ in range(warmup):
        oracle.seg_time_step(p, u, prev, g, coef=coef, mmask=mm)
    its = []
    t0 = time.perf_counter()
    for _ in range(steps):
        z, _ = oracle.seg_time_step(p, u, prev, g, coef=coef, mmask=mm)
        its.append(z)
    sec = (time.perf_counter() - t0) / max(1, steps)
    return sec, its, (u if keep_u else None)


def cpu_baseline(args, first_fp64=None):
    """The oracle on the host cores: one full time step of the benchmarked
    volume on every core (compared with the GPU's plain FP64 first step from
    the same u0), and the reference's serial path (one core) on a two-frame
    sample of the same scene."""
    import numpy as np

    threads = os.cpu_count() or 1
    sec, its, u = cpu_steps(args.size, args.seed, 0, 1, threads, keep_u=first_fp64 is not None)
    nx, ny, nz, nt = args.size
    n_int = nx * ny * nz * nt
    out = {"value": 1.0 / sec, "unit": "time-steps/s", "cores": threads, "kind": "port",
           "cpu_model": cpu_model(),
           "sample": f"1 time step of the same {nx}x{ny}x{nz}x{nt} workload ({its[0]} SOR iterations), C oracle "
                     f"restating segmentation4D.c with OpenMP over frames as mcf_4D_openmp.c does, {threads} threads",
           "ns_per_voxel_iteration": sec / (n_int * its[0]) * 1e9}
    if first_fp64 is not None:
        got, st = first_fp64
        inner = (slice(1, -1),) * 4
        same = st["iterations"] == its[0]
        err = float(np.abs(got[inner] - u[inner]).max() / np.abs(u[inner]).max()) if same else None
        out["parity_config3"] = {
            "what": "u after the first time step from u0: GPU plain FP64 form vs the oracle (its red-black SOR "
                    "restates segmentation4D.c:228-309)",
            "iterations_gpu": st["iterations"], "iterations_oracle": its[0], "max_rel_diff_u": err,
            "near_tolerance": bool(st["near_tolerance"]), "bar": 1e-10,
            "pass": bool(same and err is not None and err <= 1e-10)}
    del u
    # serial: the reference's segmentation is single-threaded
    ns = 2
    sec1, its1, _ = cpu_steps((nx, ny, nz, ns), args.seed, 0, 1, 1)
    ns_vi = sec1 / (nx * ny * nz * ns * its1[0]) * 1e9
    out["serial"] = {"value": 1.0 / (ns_vi * 1e-9 * n_int * its[0]), "unit": "time-steps/s", "cores": 1,
                     "kind": "port", "ns_per_voxel_iteration": ns_vi,
                     "sample": f"1 time step of a {nx}x{ny}x{nz}x{ns} volume of the same generator ({its1[0]} SOR "
                               f"iterations, {sec1:.1f} s) on one core; value = its time per voxel-iteration x the "
                               f"full volume's voxels x its {its[0]} iterations"}
    return out


def run_mcf(args):
    """The MCF known-answer step (mcf_4D.c:102-205; OpenMP variant
    mcf_4D_openmp.c:102-205) at the reference's OpenMP size, 80^4 interior
    voxels: the oracle on every host core (OpenMP over frames) against the
    GPU's plain FP64 form, the same steps from the exact solution at t = 0."""
    import numpy as np
    import torch

    import oracle
    import ss4d

    n, steps = 80, 2
    p = ss4d.mcf_params(n, steps)
    shape = (n + 2,) * 4
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    u = oracle.mcf_exact(p.h, 0.0, shape)
    prev = np.zeros_like(u)
    coef = oracle.new_like(u, 8)
    t0 = time.perf_counter()
    its = [oracle.mcf_time_step(p, k, u, prev, coef=coef)[0] for k in range(1, steps + 1)]
    sec = (time.perf_counter() - t0) / steps
    want = u
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ss4d.Solver(*shape, arith="fp64", stream=stream.cuda_stream) as S:
        ug = torch.zeros(shape, dtype=torch.float64, device=dev)
        pg = torch.zeros_like(ug)
        S.mcf_exact_solution(p.h, 0.0, ug)
        S.mcf_time_step(p, 1, ug.clone(), pg)  # untimed: graph set-up
        S.mcf_exact_solution(p.h, 0.0, ug)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        gits = [S.mcf_time_step(p, k, ug, pg)["iterations"] for k in range(1, steps + 1)]
        e1.record(stream)
        torch.cuda.synchronize(dev)
        gms = e0.elapsed_time(e1) / steps
        err = float((ug.cpu() - torch.from_numpy(want)).abs().max() / np.abs(want).max())
    vox = n ** 4
    return {"workload": f"MCF known-answer steps at {n}^4 interior voxels (tau = eps2 = h^2), {steps} steps from "
                        f"the exact solution",
            "cpu": {"steps_per_s": 1.0 / sec, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                    "iterations": its, "ns_per_voxel_iteration": sec / (vox * statistics.mean(its)) * 1e9,
                    "what": "C oracle restating mcf_4D.c's step, OpenMP over frames as mcf_4D_openmp.c"},
            "gpu_fp64": {"steps_per_s": 1e3 / gms, "ms_per_step": gms, "iterations": gits,
                         "max_rel_diff_u_vs_oracle": err}}


def run_reference(args):
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    sec, its, _ = cpu_steps(args.size, args.seed, args.warmup, args.steps, threads)
    v = 1.0 / sec
    kind = "port"  # the compiled reference needs its sources, which only the build host has
    return {"metric": METRIC, "value": v, "unit": "time-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "nx": args.size[0], "ny": args.size[1], "nz": args.size[2],
                       "nt": args.size[3], "parallelism": "host cores", "l2": "working set >> L2"},
            "cpu_baseline": {"value": v, "unit": "time-steps/s", "cores": threads, "kind": kind,
                             "cpu_model": cpu_model(),
                             "sample": f"{args.steps} full time steps after {args.warmup} warm-up steps, "
                                       f"SOR iterations {its}"},
            "e2e": {"value": v, "unit": "time-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_batch(args):
    print(json.dumps(batch_line(args, args.steps, args.warmup, args.forms, config=args.batch_config,
                                sequential=args.batch_sequential)))


BATCH_CONFIGS = {
    # the configuration's batch: volumes that each fill the GPU on their own
    "16x_64-192": (16, (64, 193), (64, 193), (48, 97), (8, 25)),
    # many small volumes, where one volume alone leaves the GPU idle
    "48x_24-48": (48, (24, 49), (24, 49), (24, 49), (4, 9)),
}


def batch_line(args, steps, warmup, forms_arg, config="16x_64-192", sequential=False):
    """Independent volumes (BATCH_CONFIGS: 16 of U[64..192] x U[64..192] x
    U[48..96] x U[8..24] per axis by default), single-ellipsoid scenes with
    per-volume K in [500, 2000] and tau in [0.25, 1], stepped together (the
    SOR loop of all volumes in one persistent launch, per-volume convergence,
    autotuned tile shapes), in the forms of --forms among fp64, mixed, extrap
    (mixed with the cubic extrapolated start) and proj (extrap with the
    projected start of each first round), each from the same
    start; `value` is the FP64 form's (or the first form's) aggregate
    voxel-updates/s, every form's numbers are in `forms`.  With sequential,
    each form is also timed with the same volumes solved one after another
    by single-volume handles (same steps, same stream)."""
    import numpy as np
    import torch

    import ss4d

    rng = np.random.default_rng(args.seed)
    nvol, rx, ry, rz, rt = BATCH_CONFIGS[config]
    sizes = [(int(rng.integers(*rx)), int(rng.integers(*ry)), int(rng.integers(*rz)), int(rng.integers(*rt)))
             for _ in range(nvol)]
    dev = torch.device("cuda", 0)
    params, u0s, gs = [], [], []
    for v, (nx, ny, nz, nt) in enumerate(sizes):
        p = ss4d.scene_params(K=float(rng.uniform(500, 2000)), tau=float(rng.uniform(0.25, 1.0)))
        i0h, u0h = ss4d.scene(1, nx, ny, nz, nt, seed=args.seed + 100 + v, threads=os.cpu_count() or 1)
        i0 = torch.from_numpy(i0h).to(dev)
        g = [torch.zeros_like(i0) for _ in range(8)]
        with ss4d.Solver(nx + 2, ny + 2, nz + 2, nt + 2) as S:
            S.edge_detector(p, i0, None, g)
            S.synchronize()
        params.append(p)
        u0s.append(torch.from_numpy(u0h).to(dev))
        gs.append(g)
    dims = [(nx + 2, ny + 2, nz + 2, nt + 2) for nx, ny, nz, nt in sizes]
    vox = [nx * ny * nz * nt for nx, ny, nz, nt in sizes]
    forms = [f for f in forms_arg.split(",") if f in ("fp64", "mixed", "extrap", "proj")] or ["fp64"]
    stream = torch.cuda.current_stream(dev)
    shapes = None
    results = {}
    for form in forms:
        us = [u.clone() for u in u0s]
        B = ss4d.Batch(dims, stream=stream.cuda_stream)
        B.set_graph(not args.no_graph)
        B.set_persistent(args.batch_loop == "persistent")
        if form != "fp64":
            B.set_arith("mixed")
        if form in ("extrap", "proj"):
            B.set_extrapolation(EXTRAP_ORDER)
        B.set_projection(form == "proj")
        if shapes is None:
            shapes = B.autotune(params, us, gs)
        else:
            for v, (xt, kb) in enumerate(shapes):
                B.set_shape(v, xt, kb)
        for _ in range(warmup):
            B.seg_time_step(params, us, gs)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stats = [B.seg_time_step(params, us, gs) for _ in range(steps)]
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        B.close()
        its = [[s["iterations"] for s in step] for step in stats]
        updates = sum(vv * z for step in its for vv, z in zip(vox, step))
        results[form] = {"ms_per_step": ms / steps, "voxel_updates_per_s": updates / (ms / 1e3),
                         "volume_steps_per_s": len(sizes) * steps / (ms / 1e3),
                         "iterations_per_volume": its,
                         "refinements_per_volume": [[s["refinements"] for s in step] for step in stats],
                         "max_residual": max(s["residual"] for step in stats for s in step),
                         "tolerance_met": all(s["residual"] <= p.gsTol or s["iterations"] >= p.maxNoGSIteration
                                              for step in stats for s, p in zip(step, params))}
        if sequential:
            us = [u.clone() for u in u0s]
            handles = [ss4d.Solver(*d, arith="fp64" if form == "fp64" else "mixed", stream=stream.cuda_stream)
                       for d in dims]
            for S in handles:
                S.set_extrapolation(EXTRAP_ORDER if form in ("extrap", "proj") else 0)
                S.set_projection(form == "proj")
            for _ in range(warmup):
                for v, S in enumerate(handles):
                    S.seg_time_step(params[v], us[v], None, gs[v])
            torch.cuda.synchronize(dev)
            e0.record(stream)
            seq = [[S.seg_time_step(params[v], us[v], None, gs[v])["iterations"] for v, S in enumerate(handles)]
                   for _ in range(steps)]
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms_seq = e0.elapsed_time(e1) / steps
            for S in handles:
                S.close()
            results[form]["sequential"] = {
                "ms_per_step": ms_seq, "batch_speedup": ms_seq / results[form]["ms_per_step"],
                "same_iterations": seq == its,
                "how": "the same volumes from the same start, one single-volume handle each, solved one after "
                       "another on the same stream"}
    head = "fp64" if "fp64" in results else forms[0]
    r = results[head]
    line = {"metric": f"aggregate voxel-updates/s, {nvol} uneven volumes (batched, one launch per solve)",
            "value": r["voxel_updates_per_s"], "unit": "voxel-updates/s", "n_gpus": 1, "steps": steps,
            "warmup": warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "dtype": "f64", "data": "synthetic", "impl": "ours",
            "config": {"workload": f"{nvol} volumes U[{rx[0]}..{rx[1] - 1}]x U[{ry[0]}..{ry[1] - 1}]x "
                                   f"U[{rz[0]}..{rz[1] - 1}]x U[{rt[0]}..{rt[1] - 1}], kind-1 scenes, K~U[500,2000], "
                                   "tau~U[0.25,1], gsTol 1e-6", "form": head,
                       "loop": args.batch_loop,
                       "sizes": sizes, "voxels": sum(vox)},
            "autotuned_shapes": shapes, "iterations_per_volume": r["iterations_per_volume"],
            "forms": results}
    if "fp64" in results:
        for f in results:
            if f != "fp64":
                line[f"{f}_step_speedup_over_fp64"] = results["fp64"]["ms_per_step"] / results[f]["ms_per_step"]
    del us, u0s, gs
    torch.cuda.empty_cache()
    return line


def run_conv(args):
    """The warm-start network's forward on random BF16 features of --size
    (nx ny nz frames): W untimed calls, then K timed with CUDA events; FLOP
    counted at the network's real widths (16 -> 24 -> 24 -> 24 -> 1)."""
    import numpy as np
    import torch

    import ss4d

    nx, ny, nz, nf = args.size
    net = ss4d.Wsnet(seed=3)
    x = torch.randn((nf, 2, nz, ny, nx, 8), device="cuda").to(torch.bfloat16)
    out = torch.empty((nf, nz, ny, nx), device="cuda", dtype=torch.float32)
    for _ in range(args.warmup):
        net.forward(x, nx, ny, nz, nf, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        net.forward(x, nx, ny, nz, nf, out)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    vox = nx * ny * nz * nf
    flop = vox * 2 * 27 * (16 * 24 + 24 * 24 + 24 * 24 + 24)
    net.close()
    print(json.dumps({"metric": "warm-start network forward", "value": flop / (ms / 1e3) / 1e12, "unit": "TFLOP/s",
                      "ms_per_forward": ms, "ns_per_voxel": ms / vox * 1e6, "finite": bool(torch.isfinite(out).all()),
                      "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                      "config": {"workload": f"random features {nx}x{ny}x{nz}x{nf}", "flop_per_voxel": flop // vox}}))


def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "conv":
        run_conv(args)
        return
    if args.impl == "reference":
        line = run_reference(args)
        if line:
            print(json.dumps(line))
        return
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    results, roofline, roofline_assembly, err, ctx = run_ours(args, rank, world, dist)
    forms = list(results)
    # headline: the faster of the mixed forms (with and without the learned
    # warm start) among those that converged every step, else plain FP64
    fast = [f for f in ("mixed", "extrap", "proj", "learned", "learned_x") if f in results and results[f]["converged"]]
    head = max(fast, key=lambda f: results[f]["steps_per_s"]) if fast else forms[0]
    r = results[head]
    line = {"metric": METRIC, "value": r["steps_per_s"], "unit": "time-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "mixed": "f32 sweeps + f64 residual/refinement",
                      "extrap": "f32 sweeps + f64 residual/refinement",
                      "proj": "f32 sweeps + f64 residual/refinement",
                      "learned": "f32 sweeps + f64 residual/refinement, bf16 warm-start network",
                      "learned_x": "f32 sweeps + f64 residual/refinement, bf16 warm-start network"}[head],
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": head, "form_label": FORM_LABEL.get(head, head),
                       "is_named_form": head in NAMED_FORMS, "nx": args.size[0], "ny": args.size[1],
                       "nz": args.size[2], "nt": args.size[3], "parallelism": f"replicas x{world}",
                       "l2": "inputs >> L2 (about 25 GB working set), no flush"},
            "roofline": roofline(head), "gpu_launches": r["launches"], "clocks": r["clocks"],
            "forms": {f: {k: v for k, v in results[f].items() if k != "clocks"} for f in forms}}
    named = [f for f in NAMED_FORMS if f in results and results[f]["converged"]]
    if named:
        nn = max(named, key=lambda f: results[f]["steps_per_s"])  # the faster of the named forms
        nf = results[nn]
        line["named_form"] = {"form": nn, "label": FORM_LABEL[nn], "steps_per_s": nf["steps_per_s"],
                              "over_fp64": (nf["steps_per_s"] / results["fp64"]["steps_per_s"]
                                            if "fp64" in results else None),
                              "steps100_per_s": nf.get("steps100", {}).get("steps_per_s")}
    if "fp64" in results:
        for f in ("mixed", "extrap", "proj", "extrap_w", "learned", "learned_x"):
            if f in results:
                line[f"{f}_over_fp64"] = results[f]["steps_per_s"] / results["fp64"]["steps_per_s"]
        if args.steps100 > 0:
            line["steps100_over_fp64"] = {f: results[f]["steps100"]["steps_per_s"] /
                                          results["fp64"]["steps100"]["steps_per_s"] for f in forms}
        line["roofline_fp64"] = roofline("fp64")
        line["error_vs_fp64"] = err
    for f in ("mixed", "extrap", "proj", "learned", "learned_x"):
        if f in results and f != head:
            line[f"roofline_{f}"] = roofline(f)
    if head != "fp64":
        line["roofline_assembly"] = roofline_assembly(head)
    if rank == 0 and world == 1 and not args.no_e2e:
        try:
            # the reference-named layer runs the mixed form without the network
            ef = {"learned": "mixed", "learned_x": "extrap"}.get(head, head)
            line["e2e"] = run_e2e(args, ef, ctx)
            line["e2e"]["form"] = ef
        except Exception as ex:  # reported, not hidden
            line["e2e"] = {"value": None, "unit": "time-steps/s", "error": repr(ex)}
    if rank == 0 and world == 1 and not args.no_frontend:
        line["frontend"] = run_frontend(args, ctx, "fp64")
        line["frontend_mixed"] = run_frontend(args, ctx, "mixed")
    if rank == 0 and world == 1 and not args.no_batch:
        # the batched workload, short: per-volume iteration counts of the last
        # step only (the full record is `--workload batch`)
        b = batch_line(args, 10, 3, "fp64,extrap,proj", sequential=True)
        small = batch_line(args, 10, 3, "fp64,extrap,proj", config="48x_24-48", sequential=True)
        for bl in (b, small):
            for f in bl["forms"].values():
                f["iterations_last_step"] = f.pop("iterations_per_volume")[-1]
                f.pop("refinements_per_volume", None)
            bl.pop("iterations_per_volume", None)
        b["small_volumes"] = small
        line["batch"] = b
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args, ctx[6])
        if "parity_config3" in line["cpu_baseline"]:
            line["parity_config3"] = line["cpu_baseline"]["parity_config3"]
        line["mcf_openmp"] = run_mcf(args)
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
