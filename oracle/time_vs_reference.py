"""Speed of the C oracle against the compiled reference on this host (TEST
INFRASTRUCTURE: it needs the reference's own build in oracle/_ref/, made by
``make -C oracle ref`` with SS4D_REFERENCE_DIR naming the reference checkout, so it runs only on
the build host; the GPU machine has no reference sources).

The benchmark's CPU baseline on the GPU machine is the oracle (a restatement of
segmentation4D.c's time step that keeps its evaluation order), run with
OpenMP over frames on all host cores.  This script shows what that stands
for: on the same inputs it runs one segmentation time step
(``_segTimeStep_``, segmentation4D.c:215-315) with the compiled reference
(serial, as the reference has no parallel segmentation) and with the oracle
on 1 and on all threads, checks that u agrees bit for bit, and prints the
time per voxel-iteration of each (the oracle's iteration count).

Usage:  python oracle/time_vs_reference.py [nx ny nz nt]   (default 96 96 64 8)
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "4d-image-segmentation-algorithm_gb300"))
import oracle  # noqa: E402
import ss4d  # noqa: E402  (scene generator and parameter sets only)

GLOBAL_D = ("K", "eps2", "tau", "h", "omega_c", "gsTol", "segTol", "sigma", "omega_sigma", "maxNoGSIteration_sigma",
            "theta_img", "rho_thr", "ballRadius")
FACES = ("g_e", "g_w", "g_n", "g_s", "g_t", "g_b", "g_fw", "g_bw")


def reference_step(so, p, g, u0):
    """One _segTimeStep_ of the compiled reference; returns (u, seconds)."""
    L = C.CDLL(so, mode=os.RTLD_LOCAL)
    shape = u0.shape
    lM, kM, jM, iM = shape
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM), ("maxNoGSIteration", p.maxNoGSIteration),
                  ("maxNoOfTimeSteps", 1), ("numberOfTimeStep", 1)):
        C.c_int.in_dll(L, nm).value = int(v)
    for nm in GLOBAL_D:
        C.c_double.in_dll(L, nm).value = float(getattr(p, nm))
    noc = (C.c_int * lM)()
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    L._allocateMem_.restype = C.c_bool
    L._segTimeStep_.restype = C.c_bool
    assert L._allocateMem_()
    n = int(np.prod(shape))

    def arr(name):
        addr = C.c_void_p.in_dll(L, name).value
        return np.ctypeslib.as_array((C.c_double * n).from_address(addr)).reshape(shape)

    for nm, a in zip(FACES, g):
        arr(nm)[...] = a
    arr("Mmask")[...] = 1.0
    u = arr("u")
    u[...] = u0
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    sys.stdout.flush()
    os.dup2(devnull, 1)  # the reference prints its residuals
    try:
        t0 = time.perf_counter()
        assert L._segTimeStep_()
        sec = time.perf_counter() - t0
        C.CDLL(None).fflush(None)  # the reference's buffered text, still into the null device
    finally:
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)
    return u.copy(), sec


def main():
    nx, ny, nz, nt = (int(a) for a in sys.argv[1:5]) if len(sys.argv) >= 5 else (96, 96, 64, 8)
    so = os.path.join(HERE, "_ref", "libref_seg.so")
    if not os.path.exists(so):
        sys.exit("oracle/_ref/libref_seg.so is missing: run `make -C oracle ref` where the reference exists")
    p = ss4d.scene_params()
    i0, u0 = ss4d.scene(3, nx, ny, nz, nt, seed=1, threads=os.cpu_count() or 1)
    g = oracle.gfaces(p, i0, np.zeros_like(i0))
    u_ref, t_ref = reference_step(so, p, g, u0)
    out = {}
    for threads in (1, os.cpu_count() or 1):
        oracle.set_threads(threads)
        u = u0.copy()
        t0 = time.perf_counter()
        z, _ = oracle.seg_time_step(p, u, np.zeros_like(u), g, mmask=np.ones_like(u))
        out[threads] = (time.perf_counter() - t0, z)
        assert np.array_equal(u, u_ref), "oracle and reference differ"
    z = out[1][1]
    work = nx * ny * nz * nt * z
    print(f"{nx}x{ny}x{nz}x{nt}, {z} SOR iterations, u bit-identical")
    print(f"reference (serial)      {t_ref:8.3f} s  {t_ref / work * 1e9:6.2f} ns/voxel-iteration")
    for threads, (sec, _) in out.items():
        print(f"oracle, {threads:2d} thread(s)     {sec:8.3f} s  {sec / work * 1e9:6.2f} ns/voxel-iteration")


if __name__ == "__main__":
    main()
