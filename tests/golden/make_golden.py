"""Generate the golden fixtures of tests/golden/ by running the REFERENCE itself.

The reference's segmentation4D.c and mcf_4D.c are compiled from their own,
unmodified sources into oracle/_ref/ (``make -C oracle ref``; needs the
reference checkout, named by the environment variable SS4D_REFERENCE_DIR, so
this script runs only where it is present).  This
script drives them through their global variables and functions exactly as
their main() does, captures what they print (iteration counts, residuals),
and stores inputs and outputs as .npz files:

  seg_small.npz   scene kind 1 at 10x8x6x4: edge detector (presmoothing + 8
                  face g), 5 segmentation time steps (u, prev_u after each,
                  the coefficients of step 1, iteration counts, residuals,
                  ||u - prev_u||), masks of the last step
  seg_balls.npz   the reference main's own parameters (h = tau = 0.01, K = 1,
                  eps2 = 1, theta = rho = 0.5) with rescale balls: local
                  thresholding, edge detector with a thresholded image,
                  initial function in the balls, Mmask, 3 time steps
  mcf_small.npz   MCF known-answer problem at n = 8 (3 steps) and the
                  error history at n = 16 (4 steps)
  seg_32x32x32x8.npz the 32^3 x 8 scene, 20 steps: per-step iteration counts,
                  residuals, ||u - prev_u||, u at 4096 fixed probe voxels,
                  checksums, and the final masks (bit-packed)
  pipeline.npz    the reference main's whole sequence on frame and centre
                  files at 24x22x20x4, ending in _writeData_
  vtk_io.npz      the reference's frame and centre files: _readData_ on a
                  directory of frame/centre files, _writeData_ of a volume
  seg_init.npz    initial segmentation at 36x34x32x3 with ball radius 13:
                  global maximum, per-ball minimum/maximum, local
                  thresholding into a non-zero image, initial function on a
                  non-zero u with overlapping balls, Mmask

Usage:  SS4D_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py [fixture ...]
        (from the repository root;
        names are the functions below, all of them by default)
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, os.path.join(ROOT, "4d-image-segmentation-algorithm_gb300"))
import ss4d  # noqa: E402  (scene generator and parameter sets only)

libc = C.CDLL(None)


class Captured:
    """Redirect fd 1 while the reference prints, then return its text."""

    def __enter__(self):
        libc.fflush(None)
        self.tmp = tempfile.TemporaryFile(mode="w+b")
        self.saved = os.dup(1)
        os.dup2(self.tmp.fileno(), 1)
        return self

    def __exit__(self, *a):
        libc.fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)
        self.tmp.seek(0)
        self.text = self.tmp.read().decode()
        self.tmp.close()


class Ref:
    """One compiled reference program, driven through its globals."""

    def __init__(self, so: str):
        self.L = C.CDLL(so, mode=os.RTLD_LOCAL)
        self.keep = []

    def i(self, name, v=None):
        x = C.c_int.in_dll(self.L, name)
        if v is not None:
            x.value = int(v)
        return x.value

    def d(self, name, v=None):
        x = C.c_double.in_dll(self.L, name)
        if v is not None:
            x.value = float(v)
        return x.value

    def arr(self, name, shape):
        addr = C.c_void_p.in_dll(self.L, name).value
        n = int(np.prod(shape))
        return np.ctypeslib.as_array((C.c_double * n).from_address(addr)).reshape(shape)

    def call(self, fn, *args, restype=C.c_bool):
        f = getattr(self.L, fn)
        f.restype = restype
        with Captured() as cap:
            r = f(*args)
        return r, cap.text


def build_ref():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)


def parse_steps(text):
    its = [int(m) for m in re.findall(r"total number of RBSOR is (\d+)", text)]
    res = [float(m) for m in re.findall(r"Mean square residue is (\S+)", text)]
    return its, res


def seg_setup(R: Ref, shape, p, centers=None):
    lM, kM, jM, iM = shape
    R.i("iMax", iM), R.i("jMax", jM), R.i("kMax", kM), R.i("lMax", lM)
    noc = (C.c_int * lM)(*([0] * lM))
    if centers:
        for l, c in centers.items():
            noc[l] = len(c)
    R.keep.append(noc)
    C.c_void_p.in_dll(R.L, "no_of_centers").value = C.addressof(noc)
    for name in ("K", "eps2", "tau", "h", "omega_c", "gsTol", "segTol", "sigma", "omega_sigma",
                 "maxNoGSIteration_sigma", "theta_img", "rho_thr", "ballRadius"):
        R.d(name, getattr(p, name))
    R.i("maxNoGSIteration", p.maxNoGSIteration)
    R.i("maxNoOfTimeSteps", p.maxNoOfTimeSteps)
    ok, _ = R.call("_allocateMem_")
    assert ok
    if centers:
        pp = C.POINTER(C.POINTER(C.c_double))
        cx, cy, cz = (pp.in_dll(R.L, n) for n in ("center_x", "center_y", "center_z"))
        for l, cs in centers.items():
            for c, (x, y, z) in enumerate(cs):
                cx[l][c], cy[l][c], cz[l][c] = x, y, z


def seg_small():
    R = Ref(os.path.join(REF_DIR, "libref_seg.so"))
    nx, ny, nz, nt = 10, 8, 6, 4
    p = ss4d.scene_params(maxNoOfTimeSteps=5)
    i0_in, u0 = ss4d.scene(1, nx, ny, nz, nt, seed=7)
    shape = i0_in.shape
    seg_setup(R, shape, p)
    i0 = R.arr("i0", shape)
    u = R.arr("u", shape)
    prev = R.arr("prev_u", shape)
    i0[...] = i0_in
    R.arr("Mmask", shape)[...] = 1.0  # no centres: the per-step rescale is the identity
    thr_in = u.copy()  # the thresholded-image buffer (u, all zeros here)
    _, t_gf = R.call("_gf_inputImage_plus_thresholdedImage_", C.c_void_p(i0.ctypes.data),
                     C.c_void_p(u.ctypes.data))
    ps = [int(m) for m in re.findall(r"total number of RBSOR is (\d+)", t_gf)]
    out = {"i0_in": i0_in, "thr_in": thr_in, "u0": u0, "i0_smooth": i0.copy(), "thr_smooth": u.copy(),
           "presmooth_its": np.array(ps)}
    for f, nm in enumerate(("g_e", "g_w", "g_n", "g_s", "g_t", "g_b", "g_fw", "g_bw")):
        out[f"g{f}"] = R.arr(nm, shape).copy()
    u[...] = u0
    its, res, l2 = [], [], []
    us = []
    for step in range(1, 6):
        R.i("numberOfTimeStep", step)
        _, txt = R.call("_segTimeStep_")
        a, b = parse_steps(txt)
        its += a
        res += b
        d, _ = R.call("_l2norm_", C.c_void_p(prev.ctypes.data), C.c_void_p(u.ctypes.data), restype=C.c_double)
        l2.append(d)
        us.append(u.copy())
        if step == 1:
            out["prev1"] = prev.copy()
            for f, nm in enumerate(("e", "w", "n", "s", "t", "b", "fw", "bw")):
                out[f"coef{f}"] = R.arr(nm, shape).copy()
    out["u_steps"] = np.stack(us)
    out["its"] = np.array(its)
    out["res"] = np.array(res)
    out["l2"] = np.array(l2)
    mass, _ = R.call("_mass4D_", C.c_void_p(u.ctypes.data), restype=C.c_double)
    out["mass"] = np.array(mass)
    out["params"] = np.array([p.as_dict()[k] for k in sorted(p.as_dict())])
    out["param_names"] = np.array(sorted(p.as_dict()))
    np.savez_compressed(os.path.join(OUT, "seg_small.npz"), **out)
    print("seg_small:", its, ["%.3e" % r for r in res])


def seg_balls():
    """The reference main's parameter set with balls (segmentation4D.c:1338-1371)."""
    R = Ref(os.path.join(REF_DIR, "libref_seg.so"))
    nx, ny, nz, nt = 12, 12, 10, 3
    p = ss4d.Params(K=1.0, eps2=1.0, tau=0.01, h=0.01, omega_c=1.8, gsTol=1e-12, maxNoGSIteration=5,
                    maxNoOfTimeSteps=3, segTol=1e-12, sigma=0.01 * 0.01 / 8, omega_sigma=1.3,
                    maxNoGSIteration_sigma=10.0, theta_img=0.5, rho_thr=0.5, ballRadius=3.0)
    i0_in, _ = ss4d.scene(1, nx, ny, nz, nt, seed=11)
    shape = i0_in.shape
    centers = {1: [(6.0, 6.0, 5.0), (8.0, 7.0, 6.0)], 2: [(6.0, 7.0, 5.0)], 3: [(7.0, 6.0, 5.0), (5.0, 5.0, 4.0)]}
    seg_setup(R, shape, p, centers)
    R.d("alpha", 0.85), R.d("beta", 0.15)
    i0 = R.arr("i0", shape)
    u = R.arr("u", shape)
    prev = R.arr("prev_u", shape)
    mm = R.arr("Mmask", shape)
    i0[...] = i0_in
    out = {"i0_in": i0_in}
    R.call("_locallyThreshold4Ddata_", C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
    out["thr_in"] = u.copy()
    R.call("_gf_inputImage_plus_thresholdedImage_", C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
    out["i0_smooth"] = i0.copy()
    out["thr_smooth"] = u.copy()
    for f, nm in enumerate(("g_e", "g_w", "g_n", "g_s", "g_t", "g_b", "g_fw", "g_bw")):
        out[f"g{f}"] = R.arr(nm, shape).copy()
    R.call("_generate4DsegmFunct_", C.c_void_p(u.ctypes.data))
    out["u_gen"] = u.copy()
    out["mmask"] = mm.copy()
    R.call("_rescale4DdataToZeroOne_", C.c_void_p(u.ctypes.data))
    out["u0"] = u.copy()
    its, res, us = [], [], []
    for step in range(1, 4):
        R.i("numberOfTimeStep", step)
        _, txt = R.call("_segTimeStep_")
        a, b = parse_steps(txt)
        its += a
        res += b
        us.append(u.copy())
    out["u_steps"] = np.stack(us)
    out["its"] = np.array(its)
    out["res"] = np.array(res)
    balls = [(l, x, y, z) for l in sorted(centers) for (x, y, z) in centers[l]]
    out["balls"] = np.array(balls, dtype=np.float64)
    out["params"] = np.array([p.as_dict()[k] for k in sorted(p.as_dict())])
    out["param_names"] = np.array(sorted(p.as_dict()))
    np.savez_compressed(os.path.join(OUT, "seg_balls.npz"), **out)
    print("seg_balls:", its)


def mcf_run(n: int, steps: int):
    R = Ref(os.path.join(REF_DIR, "libref_mcf.so"))
    M = n + 2
    for nm in ("iMax", "jMax", "kMax", "lMax"):
        R.i(nm, M)
    p = ss4d.mcf_params(n, steps)
    for nm in ("eps2", "tau", "h", "omega_c", "gsTol"):
        R.d(nm, getattr(p, nm))
    R.i("maxNoGSIteration", p.maxNoGSIteration)
    R.i("maxNoOfTimeSteps", steps)
    R.d("mcfTol", 1e-12)
    R.call("_allocateMem_mcf")
    shape = (M, M, M, M)
    u = R.arr("u", shape)
    ex = R.arr("exact_u", shape)
    R.call("_exactSolution_mcf", C.c_double(0.0), restype=None)
    u[...] = ex
    errs, its, us = [], [], []
    for step in range(1, steps + 1):
        R.i("numberOfTimeStep", step)
        _, txt = R.call("_mcfTimeStep")
        its += [1 for _ in re.findall(r"Residuum is", txt)]
        R.call("_exactSolution_mcf", C.c_double(step * p.tau), restype=None)
        e, _ = R.call("_l2norm_mcf", C.c_void_p(ex.ctypes.data), C.c_void_p(u.ctypes.data), restype=C.c_double)
        errs.append(e)
        us.append(u.copy())
    return np.stack(us), np.array(errs)


def mcf_small():
    u8, e8 = mcf_run(8, 3)
    _, e16 = mcf_run(16, 4)
    np.savez_compressed(os.path.join(OUT, "mcf_small.npz"), u8=u8, err8=e8, err16=e16)
    print("mcf: err8", e8, "err16", e16)


def seg_32x32x32x8():
    R = Ref(os.path.join(REF_DIR, "libref_seg.so"))
    nx, ny, nz, nt = 32, 32, 32, 8
    p = ss4d.scene_params(maxNoOfTimeSteps=20)
    i0_in, u0 = ss4d.scene(1, nx, ny, nz, nt, seed=1)
    shape = i0_in.shape
    seg_setup(R, shape, p)
    i0 = R.arr("i0", shape)
    u = R.arr("u", shape)
    prev = R.arr("prev_u", shape)
    i0[...] = i0_in
    R.arr("Mmask", shape)[...] = 1.0  # no centres: the per-step rescale is the identity
    R.call("_gf_inputImage_plus_thresholdedImage_", C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
    u[...] = u0
    rng = np.random.default_rng(1234)
    probes = rng.integers(0, u.size, 4096)
    its, res, l2, probe_vals, sums = [], [], [], [], []
    for step in range(1, 21):
        R.i("numberOfTimeStep", step)
        _, txt = R.call("_segTimeStep_")
        a, b = parse_steps(txt)
        its += a
        res += b
        d, _ = R.call("_l2norm_", C.c_void_p(prev.ctypes.data), C.c_void_p(u.ctypes.data), restype=C.c_double)
        l2.append(d)
        probe_vals.append(u.reshape(-1)[probes].copy())
        sums.append((u.sum(), (u * u).sum()))
    inner = u[1:-1, 1:-1, 1:-1, 1:-1]
    m05 = (inner >= 0.5).astype(np.uint8).reshape(-1)
    lo, hi = inner.min(), inner.max()
    mnorm = (inner >= lo + 0.5 * (hi - lo)).astype(np.uint8).reshape(-1)
    np.savez_compressed(os.path.join(OUT, "seg_32x32x32x8.npz"), its=np.array(its), res=np.array(res),
                        l2=np.array(l2), probes=probes, probe_vals=np.stack(probe_vals), sums=np.array(sums),
                        mask05=np.packbits(m05), masknorm=np.packbits(mnorm), seed=1,
                        dims=np.array([nx, ny, nz, nt]))
    print("seg_32x32x32x8: its", its)


def seg_init():
    """Initial segmentation with a ball radius above the initial function's
    fixed radius 12 (segmentation4D.c:1110): the reference's _get4DMax_,
    _get3DMinWithinR_/_get3DMaxWithinR_ per ball, _locallyThreshold4Ddata_
    into a non-zero thresholded image, _generate4DsegmFunct_ on a non-zero u
    with overlapping balls."""
    R = Ref(os.path.join(REF_DIR, "libref_seg.so"))
    nx, ny, nz, nt = 36, 34, 32, 3
    p = ss4d.scene_params(ballRadius=13.0)
    i0_in, u_in = ss4d.scene(1, nx, ny, nz, nt, seed=21)
    shape = i0_in.shape
    centers = {1: [(18.0, 17.0, 16.5), (20.5, 18.0, 17.0)], 2: [(17.0, 18.5, 16.0)],
               3: [(18.5, 17.5, 17.5), (16.0, 16.0, 15.0), (19.0, 19.0, 16.0)]}
    seg_setup(R, shape, p, centers)
    R.d("alpha", 0.7), R.d("beta", 0.3)
    i0 = R.arr("i0", shape)
    u = R.arr("u", shape)
    mm = R.arr("Mmask", shape)
    i0[...] = i0_in
    out = {"i0_in": i0_in}
    gmax, _ = R.call("_get4DMax_", C.c_void_p(i0.ctypes.data), restype=C.c_double)
    out["gmax"] = np.array(gmax)
    mins, maxs = [], []
    for l in sorted(centers):
        for (x, y, z) in centers[l]:
            args = (C.c_void_p(i0.ctypes.data), C.c_int(l), C.c_double(x), C.c_double(y), C.c_double(z),
                    C.c_double(p.ballRadius))
            mn, _ = R.call("_get3DMinWithinR_", *args, restype=C.c_double)
            mx, _ = R.call("_get3DMaxWithinR_", *args, restype=C.c_double)
            mins.append(mn)
            maxs.append(mx)
    out["ball_min"] = np.array(mins)
    out["ball_max"] = np.array(maxs)
    thr0 = 0.25 * u_in  # a non-zero thresholded-image buffer: only some voxels are overwritten
    u[...] = thr0
    out["thr_before"] = thr0
    R.call("_locallyThreshold4Ddata_", C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
    out["thr_after"] = u.copy()
    u[...] = u_in
    mm[...] = 0.0
    out["u_before"] = u_in
    R.call("_generate4DsegmFunct_", C.c_void_p(u.ctypes.data))
    out["u_gen"] = u.copy()
    out["mmask"] = mm.copy()
    balls = [(l, x, y, z) for l in sorted(centers) for (x, y, z) in centers[l]]
    out["balls"] = np.array(balls, dtype=np.float64)
    out["alpha_beta_R"] = np.array([0.7, 0.3, p.ballRadius])
    np.savez_compressed(os.path.join(OUT, "seg_init.npz"), **out)
    print("seg_init: gmax", gmax, "changed thr", int((out["thr_after"] != thr0).sum()),
          "changed u", int((out["u_gen"] != u_in).sum()))


def presmooth_exp():
    """The reference's explicit smoother _presmoothStepEXP_ (declared, never
    called by its main) on a ragged volume with random ghosts, h != 1, for
    timeStepsNum 0, 1 and 3: u and prev_u after the call."""
    R = Ref(os.path.join(REF_DIR, "libref_seg.so"))
    nx, ny, nz, nt = 13, 10, 9, 4
    p = ss4d.scene_params(sigma=0.07, h=0.9)
    shape = (nt + 2, nz + 2, ny + 2, nx + 2)
    seg_setup(R, shape, p)
    rng = np.random.default_rng(33)
    v0 = rng.random(shape)
    u, prev = R.arr("u", shape), R.arr("prev_u", shape)
    out = {"v_in": v0, "sigma_h": np.array([p.sigma, p.h])}
    for steps in (0, 1, 3):
        R.i("timeStepsNum", steps)
        u[...] = v0
        prev[...] = 0.0
        R.call("_presmoothStepEXP_", C.c_void_p(u.ctypes.data), restype=None)
        out["u_%d" % steps] = u.copy()
        out["prev_%d" % steps] = prev.copy()
    np.savez_compressed(os.path.join(OUT, "presmooth_exp.npz"), **out)
    print("presmooth_exp: changed", int((out["u_1"] != v0).sum()), "of", v0.size,
          "3 == 1:", bool(np.array_equal(out["u_3"], out["u_1"])))


VTK_HEADER = ("# vtk DataFile Version 3.0\nmovingBalls test frame\nBINARY\nDATASET STRUCTURED_POINTS\n"
              "DIMENSIONS {nx} {ny} {nz}\nORIGIN 0 0 0\nSPACING 0.5 0.25 1\nPOINT_DATA {n}\n"
              "SCALARS scalars unsigned_char\nLOOKUP_TABLE default\n")


def vtk_io():
    """The reference's file formats: _readData_ on a directory of frame files
    (random bytes, including newline bytes in the payload) and centre files
    (two comment lines, a POINTS line with a type word, non-integral
    coordinates at spacing 0.5 / 0.25 / 1), and _writeData_ of a volume in
    [0, 1] with values on the rounding boundaries."""
    R = Ref(os.path.join(REF_DIR, "libref_seg.so"))
    nx, ny, nz, nt = 9, 7, 5, 3
    shape = (nt + 2, nz + 2, ny + 2, nx + 2)
    p = ss4d.scene_params(ballRadius=1.0)
    rng = np.random.default_rng(31)
    pts = {1: [(2.1, 1.3, 2.9), (3.3, 0.8, 1.1)], 2: [(1.74, 1.12, 2.5)],
           3: [(2.6, 1.0, 3.0), (1.2, 0.9, 2.0), (3.9, 1.62, 1.7)]}
    seg_setup(R, shape, p, {l: [(0.0, 0.0, 0.0)] * len(c) for l, c in pts.items()})
    for nm, v in (("spacing_x", 0.5), ("spacing_y", 0.25), ("spacing_z", 1.0), ("origin_x", 0.5),
                  ("origin_y", -1.25), ("origin_z", 2.0)):
        R.d(nm, v)
    out = {"dims": np.array([nx, ny, nz, nt])}
    with tempfile.TemporaryDirectory() as td:
        payloads, ctexts = [], []
        for l in range(1, nt + 1):
            pay = rng.integers(0, 256, nx * ny * nz, dtype=np.uint8)
            pay[::37] = 10  # newline bytes inside the payload
            payloads.append(pay)
            with open(os.path.join(td, "movingBalls_457_at_time_%03d.vtk" % l), "wb") as fh:
                fh.write(VTK_HEADER.format(nx=nx, ny=ny, nz=nz, n=nx * ny * nz).encode() + pay.tobytes())
            txt = ("# vtk DataFile Version 3.0\n# centres of frame %d\ncentres\nASCII\nDATASET POLYDATA\n"
                   "POINTS %d float\n" % (l, len(pts[l])) + "".join("%g %g %g\n" % q for q in pts[l]))
            ctexts.append(txt)
            with open(os.path.join(td, "movingBalls_457_centers_at_timestep_%03d.vtk" % l), "w") as fh:
                fh.write(txt)
        i0 = R.arr("i0", shape)
        i0[...] = -1.0  # ghosts and untouched voxels keep this value
        R.call("_readData_", C.c_void_p(i0.ctypes.data), C.c_char_p(td.encode()), restype=None)
        out["payloads"] = np.stack(payloads)
        out["centre_texts"] = np.array(ctexts)
        out["i0_read"] = i0.copy()
        pp = C.POINTER(C.POINTER(C.c_double))
        cx, cy, cz = (pp.in_dll(R.L, n) for n in ("center_x", "center_y", "center_z"))
        out["centres"] = np.array([(l, cx[l][c], cy[l][c], cz[l][c]) for l in sorted(pts)
                                   for c in range(len(pts[l]))])
        u = R.arr("u", shape)
        v = rng.random(shape)
        v.reshape(-1)[::11] = (np.arange(v.size)[::11] % 255 + 0.5) / 255.0  # rounding boundaries
        v.reshape(-1)[::13] = 0.0
        v.reshape(-1)[::17] = 1.0
        u[...] = v
        out["u_written"] = v
        R.call("_writeData_", C.c_void_p(u.ctypes.data), C.c_char_p(os.path.join(td, "out").encode()))
        files = []
        for l in range(1, nt + 1):
            with open(os.path.join(td, "out_at_time_%03d.vtk" % l), "rb") as fh:
                files.append(np.frombuffer(fh.read(), dtype=np.uint8))
        out["written"] = np.stack(files).astype(np.uint8)  # equal lengths: same header and size per frame
    out["origin_spacing"] = np.array([0.5, -1.25, 2.0, 0.5, 0.25, 1.0])
    np.savez_compressed(os.path.join(OUT, "vtk_io.npz"), **out)
    print("vtk_io: centres", out["centres"].tolist())


def pipeline():
    """The reference main's whole sequence (segmentation4D.c:1325-1420) on
    files: _readData_ of frame and centre files, _locallyThreshold4Ddata_,
    _gf_inputImage_plus_thresholdedImage_, _generate4DsegmFunct_,
    _rescale4DdataToZeroOne_, time steps with _l2norm_ until segTol or
    maxNoOfTimeSteps, _writeData_.  Its parameters (h = tau = 0.01, K = 1,
    eps2 = 1, theta = rho = 0.5, alpha 0.85, beta 0.15, 5 SOR iterations);
    ball radius 6 at 24x22x20x4."""
    R = Ref(os.path.join(REF_DIR, "libref_seg.so"))
    nx, ny, nz, nt = 24, 22, 20, 4
    shape = (nt + 2, nz + 2, ny + 2, nx + 2)
    p = ss4d.Params(K=1.0, eps2=1.0, tau=0.01, h=0.01, omega_c=1.8, gsTol=1e-12, maxNoGSIteration=5,
                    maxNoOfTimeSteps=4, segTol=1e-12, sigma=0.01 * 0.01 / 8, omega_sigma=1.3,
                    maxNoGSIteration_sigma=10.0, theta_img=0.5, rho_thr=0.5, ballRadius=6.0)
    img, _ = ss4d.scene(1, nx, ny, nz, nt, seed=41)
    pay = [np.clip(np.rint(img[l, 1:-1, 1:-1, 1:-1] * 255.0), 0, 255).astype(np.uint8).reshape(-1)
           for l in range(1, nt + 1)]
    sp = (0.5, 0.5, 0.5)
    pts = {1: [(6.1, 5.4, 5.0), (7.2, 6.1, 4.7)], 2: [(6.4, 5.6, 5.2)], 3: [(5.8, 5.3, 4.9), (6.9, 6.4, 5.6)],
           4: [(6.2, 5.9, 5.1)]}
    seg_setup(R, shape, p, {l: [(0.0, 0.0, 0.0)] * len(c) for l, c in pts.items()})
    for nm, v in (("spacing_x", sp[0]), ("spacing_y", sp[1]), ("spacing_z", sp[2]), ("origin_x", 0.0),
                  ("origin_y", 0.0), ("origin_z", 0.0), ("alpha", 0.85), ("beta", 0.15)):
        R.d(nm, v)
    i0, u, prev = R.arr("i0", shape), R.arr("u", shape), R.arr("prev_u", shape)
    out = {"dims": np.array([nx, ny, nz, nt]), "payloads": np.stack(pay)}
    with tempfile.TemporaryDirectory() as td:
        texts = []
        for l in range(1, nt + 1):
            with open(os.path.join(td, "movingBalls_457_at_time_%03d.vtk" % l), "wb") as fh:
                fh.write(VTK_HEADER.format(nx=nx, ny=ny, nz=nz, n=nx * ny * nz).encode() + pay[l - 1].tobytes())
            txt = ("# vtk DataFile Version 3.0\ncentres\nASCII\nDATASET POLYDATA\nPOINTS %d float\n" % len(pts[l])
                   + "".join("%g %g %g\n" % q for q in pts[l]))
            texts.append(txt)
            with open(os.path.join(td, "movingBalls_457_centers_at_timestep_%03d.vtk" % l), "w") as fh:
                fh.write(txt)
        out["centre_texts"] = np.array(texts)
        with Captured() as cap:
            R.L._readData_.restype = None
            R.L._readData_(C.c_void_p(i0.ctypes.data), C.c_char_p(td.encode()))
            R.L._locallyThreshold4Ddata_(C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
            R.L._gf_inputImage_plus_thresholdedImage_(C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
            R.L._generate4DsegmFunct_(C.c_void_p(u.ctypes.data))
            R.L._rescale4DdataToZeroOne_(C.c_void_p(u.ctypes.data))
            R.L._l2norm_.restype = C.c_double
            l2s = []
            t = 1
            while True:
                R.i("numberOfTimeStep", t)
                R.L._segTimeStep_()
                l2s.append(R.L._l2norm_(C.c_void_p(prev.ctypes.data), C.c_void_p(u.ctypes.data)))
                t += 1
                if not (t <= p.maxNoOfTimeSteps and l2s[-1] > p.segTol):
                    break
            R.L._writeData_(C.c_void_p(u.ctypes.data), C.c_char_p(os.path.join(td, "result").encode()))
        its, res = parse_steps(cap.text)
        files = []
        for l in range(1, nt + 1):
            with open(os.path.join(td, "result_at_time_%03d.vtk" % l), "rb") as fh:
                files.append(np.frombuffer(fh.read(), dtype=np.uint8))
    out["written"] = np.stack(files).astype(np.uint8)
    out["u_final"] = u.copy()
    out["its"] = np.array(its)
    out["l2"] = np.array(l2s)
    out["params"] = np.array([p.as_dict()[k] for k in sorted(p.as_dict())])
    out["param_names"] = np.array(sorted(p.as_dict()))
    out["spacing"] = np.array(sp)
    np.savez_compressed(os.path.join(OUT, "pipeline.npz"), **out)
    print("pipeline: its", its, "l2", ["%.3e" % v for v in l2s])


if __name__ == "__main__":
    build_ref()
    if len(sys.argv) > 1:  # only the named fixtures
        for name in sys.argv[1:]:
            globals()[name]()
        sys.exit(0)
    seg_small()
    seg_balls()
    mcf_small()
    seg_32x32x32x8()
    seg_init()
    presmooth_exp()
    vtk_io()
    pipeline()
