#!/usr/bin/env python
"""Training and evaluation of the learned warm start (ss4d_wsnet) of the
mixed-precision segmentation step.

Data: synthetic multi-object scenes (ss4d_scene_generate kind 3, the
256x256x128x20 workload's generator) at 128x128x64x12, stepped by the plain
FP64 solver to a tight tolerance.  For every time step n the features of
u^n (ss4d_ws_features: residual, coefficients, g, u, image) and the exact
first correction (u^{n+1} - u^n) / s, s the RMS of the step's initial
residual, are cut into crops.  Training: Adam on the mean squared error of
the crops' inner voxels (a border of 4 voxels, the network's reach, is
excluded), all on the GPU through the library's own kernels.  Evaluation:
SOR iterations and time per step of the mixed form with and without the
network on scenes it has not seen (other seeds, and the 256x256x128x20 size).

    python train_wsnet.py --out weights/wsnet_seg.npy
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import ss4d  # noqa: E402

MARGIN = 4  # receptive-field radius of four 3x3x3 layers


def prepare_scene(torch, kind, dims, seed, p):
    """(presmoothed image i0, g faces, u0) on the device"""
    nx, ny, nz, nt = dims
    i0h, u0h = ss4d.scene(kind, nx, ny, nz, nt, seed=seed, threads=os.cpu_count() or 1)
    i0 = torch.from_numpy(i0h).cuda()
    g = [torch.empty_like(i0) for _ in range(8)]
    with ss4d.Solver(*i0h.shape[::-1], arith="fp64") as S:
        S.edge_detector(p, i0, None, g)
        S.synchronize()
    return i0, g, torch.from_numpy(u0h).cuda()


def make_dataset(torch, scenes, dims, steps, crops_per_step, crop, gs_tol, rng, log=print):
    """Crops of features [N, 2, cz, cy, cx, 8] (BF16, the network's planar
    layout: a crop is one frame of the training batch) and targets
    [N, cz, cy, cx]."""
    nx, ny, nz, nt = dims
    cx, cy, cz = crop
    n = len(scenes) * steps * crops_per_step
    X = torch.empty((n, 2, cz, cy, cx, 8), dtype=torch.bfloat16, device="cuda")
    T = torch.empty((n, cz, cy, cx), dtype=torch.float32, device="cuda")
    x0 = torch.empty((nt, 2, nz, ny, nx, 8), dtype=torch.bfloat16, device="cuda")
    q = 0
    for kind, seed in scenes:
        p = ss4d.scene_params(gsTol=gs_tol)
        i0, g, u = prepare_scene(torch, kind, dims, seed, p)
        shape = tuple(u.shape)
        with ss4d.Solver(*shape[::-1], arith="fp64") as S, ss4d.Solver(*shape[::-1], arith="mixed") as F:
            its = []
            for _ in range(steps):
                sigma = F.ws_features(p, u, g, i0, x0)
                un = u.clone()
                st = S.seg_time_step(p, u, None, g)
                its.append(st["iterations"])
                d = ((u - un)[1:-1, 1:-1, 1:-1, 1:-1] / sigma).float()
                for _ in range(crops_per_step):
                    f = int(rng.integers(nt))
                    z0 = int(rng.integers(nz - cz + 1))
                    y0 = int(rng.integers(ny - cy + 1))
                    xs = int(rng.integers(nx - cx + 1))
                    X[q] = x0[f, :, z0:z0 + cz, y0:y0 + cy, xs:xs + cx]
                    T[q] = d[f, z0:z0 + cz, y0:y0 + cy, xs:xs + cx]
                    q += 1
        log(f"scene kind {kind} seed {seed}: iterations/step {its}")
    return X, T


def train(torch, net, X, T, iters, batch, lr, rng, val_frac=0.1, log=print):
    n = X.shape[0]
    perm = rng.permutation(n)
    nval = max(1, int(n * val_frac))
    val, tr = perm[:nval], perm[nval:]
    cz, cy, cx = X.shape[2:5]
    hist = []

    def val_loss():
        tot = 0.0
        for i in range(0, nval, batch):
            idx = torch.from_numpy(val[i:i + batch]).cuda()
            b = idx.numel()
            tot += net.train_step(X[idx].contiguous(), T[idx].contiguous(), cx, cy, cz, b, MARGIN, 0.0) * b
        return tot / nval

    t0 = time.time()
    v0 = val_loss()
    log(f"initial validation loss {v0:.5f}")
    for it in range(iters):
        a = lr * (0.05 + 0.95 * 0.5 * (1 + math.cos(math.pi * it / iters)))  # cosine to lr/20
        idx = torch.from_numpy(rng.choice(tr, size=batch, replace=False)).cuda()
        loss = net.train_step(X[idx].contiguous(), T[idx].contiguous(), cx, cy, cz, batch, MARGIN, a)
        if (it + 1) % max(1, iters // 10) == 0:
            v = val_loss()
            hist.append((it + 1, loss, v))
            log(f"iter {it + 1}: train {loss:.5f} validation {v:.5f} ({time.time() - t0:.0f} s)")
    return {"initial_val": v0, "history": hist, "seconds": time.time() - t0}


def evaluate(torch, net, kind, dims, seed, steps, gs_tol=1e-6):
    """per-step iterations and device time of the mixed form, cold and warm
    started, from the same u0; and the two final states' agreement"""
    p = ss4d.scene_params(gsTol=gs_tol)
    i0, g, u0 = prepare_scene(torch, kind, dims, seed, p)
    shape = tuple(u0.shape)
    out = {}
    finals = {}
    for form in ("cold", "warm"):
        u = u0.clone()
        with ss4d.Solver(*shape[::-1], arith="mixed") as S:
            if form == "warm":
                S.set_warm_start(net, i0)
            stats = [S.seg_time_step(p, u, None, g) for _ in range(steps)]
            S.synchronize()
        out[form] = {"iterations": [s["iterations"] for s in stats], "ms": [round(s["ms"], 3) for s in stats],
                     "warm_started": [s["warm_started"] for s in stats],
                     "max_residual": max(s["residual"] for s in stats)}
        finals[form] = u
    a, b = finals["warm"], finals["cold"]
    out["max_rel_diff"] = float((a - b).abs().max() / b.abs().max())
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "weights", "wsnet_seg.npy"))
    ap.add_argument("--dims", type=int, nargs=4, default=[128, 128, 64, 12])
    ap.add_argument("--kinds", type=int, nargs="+", default=[3], help="scene generator kinds, used in turn")
    ap.add_argument("--scenes", type=int, default=12)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--crops", type=int, default=84, help="crops per time step (12 x 20 x 84 = 20160)")
    ap.add_argument("--crop", type=int, nargs=3, default=[40, 40, 20], metavar=("CX", "CY", "CZ"))
    ap.add_argument("--iters", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--gs-tol", type=float, default=1e-9)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eval-dims", type=int, nargs=4, default=[256, 256, 128, 20])
    ap.add_argument("--eval-steps", type=int, default=6)
    ap.add_argument("--eval-kinds", type=int, nargs="+", default=[3])
    ap.add_argument("--init", default=None, help="start from these parameters (.npy)")
    args = ap.parse_args()

    import torch

    rng = np.random.default_rng(args.seed)
    scenes = [(args.kinds[i % len(args.kinds)], 1000 + i) for i in range(args.scenes)]
    t0 = time.time()
    X, T = make_dataset(torch, scenes, args.dims, args.steps, args.crops, args.crop, args.gs_tol, rng)
    print(f"dataset: {X.shape[0]} crops in {time.time() - t0:.0f} s; target rms {T.float().pow(2).mean().sqrt():.4f}")
    net = ss4d.Wsnet(seed=args.seed + 1)
    if args.init:
        net.set_params(np.load(args.init))
    summary = train(torch, net, X, T, args.iters, args.batch, args.lr, rng)
    params = net.get_params()
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.save(args.out, params)
    del X, T
    torch.cuda.empty_cache()
    ev = {}
    for kind in args.eval_kinds:
        ev[f"kind{kind}"] = evaluate(torch, net, kind, args.eval_dims, 5000 + kind, args.eval_steps)
        e = ev[f"kind{kind}"]
        print(f"eval kind {kind}: cold its {e['cold']['iterations']} warm its {e['warm']['iterations']} "
              f"kept {e['warm']['warm_started']} max rel diff {e['max_rel_diff']:.2e}")
    rec = dict(vars(args))
    rec["out"] = os.path.basename(args.out)  # the record names the file, not where it was written
    meta = {"args": rec, "train": summary, "eval": ev, "param_count": int(params.size)}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(meta, fh, indent=1)


if __name__ == "__main__":
    main()
