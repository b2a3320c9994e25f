"""Python view of the GB300 solver's C ABI (include/ss4d.h).

The reference is a set of C programs whose "interface" is the functions and
globals of segmentation4D.c / mcf_4D.c.  This module mirrors that interface
for Python callers (tests, benchmarks): the reference's parameter names in
`Params`, its step functions as `Solver` methods, the same padded x-fastest
FP64 layout.  The reference-named C layer (libss4d_seg.so / libss4d_mcf.so,
include/ss4d_compat.h) sits at `SEG_PATH` / `MCF_PATH`.  Device arrays are passed as integer device pointers
or as objects with a ``data_ptr()`` method (e.g. torch tensors).

Every call goes to libss4d.so; there is no Python or CPU implementation of
the solver here.  A missing or unloadable library raises `SS4DError`.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libss4d.so")
SEG_PATH = os.path.join(HERE, "libss4d_seg.so")
MCF_PATH = os.path.join(HERE, "libss4d_mcf.so")

ARITH = {"reference": 0, "fp64": 1, "mixed": 2}
STATUS = {0: "OK", 1: "INVALID", 2: "ALLOC", 3: "CUDA", 4: "NONFINITE", 5: "TIMEOUT", 6: "UNSUPPORTED",
          7: "NO_DEVICE"}


class SS4DError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)} {detail}".strip())


class Dims(C.Structure):
    _fields_ = [("iMax", C.c_int), ("jMax", C.c_int), ("kMax", C.c_int), ("lMax", C.c_int)]


class Params(C.Structure):
    """ss4d_params: the reference's tunables under their own names."""
    _fields_ = [("K", C.c_double), ("eps2", C.c_double), ("tau", C.c_double), ("h", C.c_double),
                ("omega_c", C.c_double), ("gsTol", C.c_double), ("maxNoGSIteration", C.c_int),
                ("maxNoOfTimeSteps", C.c_int), ("segTol", C.c_double), ("sigma", C.c_double),
                ("omega_sigma", C.c_double), ("maxNoGSIteration_sigma", C.c_double), ("theta_img", C.c_double),
                ("rho_thr", C.c_double), ("ballRadius", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class StepStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("status", C.c_int), ("residual", C.c_double),
                ("first_residual", C.c_double), ("refinements", C.c_int), ("warm_started", C.c_int),
                ("ms", C.c_float), ("near_tolerance", C.c_int), ("projected", C.c_int)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class Balls(C.Structure):
    _fields_ = [("n", C.c_int), ("l", C.POINTER(C.c_int)), ("cx", C.POINTER(C.c_double)),
                ("cy", C.POINTER(C.c_double)), ("cz", C.POINTER(C.c_double))]


def scene_params(**over) -> Params:
    """Parameters of the synthetic-scene workloads: K = 1000, eps2 = 1e-3,
    h = 1, tau = 0.5, omega_c = 1.8, gsTol = 1e-6, 1000 SOR iterations; the
    edge detector's presmoothing matches a Gaussian of sigma = 1 voxel in its
    second moment (sigma = 0.5 h^2), with the reference main's omega_sigma = 1.3
    and 10 iterations (segmentation4D.c:1353-1363); theta_img = 1, rho_thr = 0."""
    p = Params(K=1000.0, eps2=1e-3, tau=0.5, h=1.0, omega_c=1.8, gsTol=1e-6, maxNoGSIteration=1000,
               maxNoOfTimeSteps=20, segTol=0.0, sigma=0.5, omega_sigma=1.3, maxNoGSIteration_sigma=10.0,
               theta_img=1.0, rho_thr=0.0, ballRadius=8.0)
    for k, v in over.items():
        setattr(p, k, v)
    return p


def mcf_params(n: int, steps: int = 4, **over) -> Params:
    """The MCF known-answer configuration of mcf_4D.c:478-490 for interior n:
    h = 2.5/n, tau = eps2 = h^2, omega_c = 1.8, gsTol = 1e-12, 1000 iterations."""
    h = 2.5 / n
    p = Params(K=0.0, eps2=h * h, tau=h * h, h=h, omega_c=1.8, gsTol=1e-12, maxNoGSIteration=1000,
               maxNoOfTimeSteps=steps, segTol=0.0, sigma=0.0, omega_sigma=1.0, maxNoGSIteration_sigma=0.0,
               theta_img=0.0, rho_thr=0.0, ballRadius=0.0)
    for k, v in over.items():
        setattr(p, k, v)
    return p


_lib = None
ABI_VERSION = 3  # include/ss4d.h SS4D_ABI_VERSION: the structures above mirror it


# t-slab callbacks (include/ss4d.h: ss4d_slab_comm, ss4d_slab_ops)
EXCHANGE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p)
ALLREDUCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double))
HALF_SWEEP_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int)
RESIDUAL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double))


class SlabComm(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("exchange", EXCHANGE_FN), ("allreduce_sum", ALLREDUCE_FN)]


class SlabOps(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("half_sweep", HALF_SWEEP_FN), ("residual", RESIDUAL_FN), ("u", C.c_void_p),
                ("frame_elems", C.c_longlong), ("lMax", C.c_int), ("stream", C.c_void_p)]


def _guarded(fn):
    """a callback that reports a Python exception as a non-zero status"""
    def call(*a):
        try:
            r = fn(*a)
            return 0 if r is None else int(r)
        except Exception as ex:  # noqa: BLE001  (surfaced through the library's status)
            import traceback
            traceback.print_exc()
            call.error = ex
            return 1
    call.error = None
    return call


def slab_comm(exchange, allreduce_sum):
    """An ss4d_slab_comm from Python callables:
    exchange(u_ptr: int, frame_elems: int, lMax: int, stream: int | None) and
    allreduce_sum(value: float) -> float.  Keep the returned object alive
    while the library may call it."""
    def ex(ctx, u, fe, lM, stream):
        exchange(u, fe, lM, stream)

    def ar(ctx, v):
        v[0] = float(allreduce_sum(v[0]))

    keep = (EXCHANGE_FN(_guarded(ex)), ALLREDUCE_FN(_guarded(ar)))
    c = SlabComm(None, keep[0], keep[1])
    c._keep = keep
    return c


def slab_ops(half_sweep, residual, u_ptr: int, frame_elems: int, lMax: int):
    """An ss4d_slab_ops from Python callables (host work): half_sweep(colour)
    and residual() -> float, over the slab array at u_ptr."""
    def hs(ctx, colour):
        half_sweep(colour)

    def rs(ctx, out):
        out[0] = float(residual())

    keep = (HALF_SWEEP_FN(_guarded(hs)), RESIDUAL_FN(_guarded(rs)))
    o = SlabOps(None, keep[0], keep[1], u_ptr, frame_elems, lMax, None)
    o._keep = keep
    return o


def slab_partition(nt: int, nranks: int):
    """[(first, count)] per rank: global interior frames first..first+count-1"""
    first = (C.c_int * nranks)()
    count = (C.c_int * nranks)()
    _check(lib().ss4d_slab_partition(nt, nranks, first, count), "slab_partition")
    return [(first[r], count[r]) for r in range(nranks)]


def slab_sor_loop(ops: SlabOps, comm: SlabComm, p: Params, nint_global: int) -> dict:
    """ss4d_slab_sor_loop: the slab SOR loop over the given callbacks"""
    st = StepStats()
    _check(lib().ss4d_slab_sor_loop(C.byref(ops), C.byref(comm), C.byref(p), nint_global, C.byref(st)),
           "slab_sor_loop")
    return st.as_dict()


def lib() -> C.CDLL:
    """Load libss4d.so (built by build.py) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SS4DError(6, "libss4d.so is not built", f"(expected at {LIB_PATH}; run build.py)")
    L = C.CDLL(LIB_PATH)
    vp, dp, st = C.c_void_p, C.POINTER(C.c_double), C.c_int
    P8 = C.c_void_p * 8
    sig = {
        "ss4d_abi_version": ([], C.c_int),
        "ss4d_last_error": ([], C.c_char_p),
        "ss4d_device_count": ([C.POINTER(C.c_int)], st),
        "ss4d_solver_create": ([C.POINTER(Dims), C.c_int, vp, C.POINTER(vp)], st),
        "ss4d_solver_destroy": ([vp], st),
        "ss4d_solver_set_stream": ([vp, vp], st),
        "ss4d_solver_set_arith": ([vp, C.c_int], st),
        "ss4d_solver_set_graph": ([vp, C.c_int], st),
        "ss4d_solver_workspace_bytes": ([vp, C.POINTER(C.c_size_t)], st),
        "ss4d_solver_set_timing": ([vp, C.c_int], st),
        "ss4d_solver_set_tiling": ([vp, C.c_int, C.c_int], st),
        "ss4d_solver_set_assembly_order": ([vp, C.c_int], st),
        "ss4d_solver_kernel_time": ([vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong)], st),
        "ss4d_solver_reset_timing": ([vp], st),
        "ss4d_solver_launch_count": ([vp, C.POINTER(C.c_longlong)], st),
        "ss4d_reflect": ([vp, vp], st),
        "ss4d_presmooth_step": ([vp, C.POINTER(Params), vp, vp, C.POINTER(StepStats)], st),
        "ss4d_edge_detector": ([vp, C.POINTER(Params), vp, vp, vp, P8], st),
        "ss4d_gs_coefficients": ([vp, C.POINTER(Params), vp, vp, P8], st),
        "ss4d_sor_solve": ([vp, C.POINTER(Params), vp, vp, P8, C.POINTER(StepStats)], st),
        "ss4d_seg_time_step": ([vp, C.POINTER(Params), vp, vp, P8, vp, C.POINTER(Balls), C.POINTER(StepStats)], st),
        "ss4d_mcf_time_step": ([vp, C.POINTER(Params), C.c_int, vp, vp, C.POINTER(StepStats)], st),
        "ss4d_rescale_to_zero_one": ([vp, C.POINTER(Params), vp, vp, C.POINTER(Balls)], st),
        "ss4d_rescale_to_zero_one_noalloc": ([C.POINTER(Dims), C.POINTER(Params), vp, vp, C.POINTER(Balls), vp], st),
        "ss4d_threshold_mask": ([vp, vp, C.c_double, C.c_int, vp], st),
        "ss4d_max4d": ([vp, vp, dp], st),
        "ss4d_vtk_write_frame": ([C.c_char_p, C.c_int, C.c_int, C.c_int, dp, dp, vp], st),
        "ss4d_vtk_read_frame": ([C.c_char_p, C.c_int, C.c_int, C.c_int, vp], st),
        "ss4d_vtk_read_centers": ([C.c_char_p, dp, C.c_int, dp, dp, dp, C.POINTER(C.c_int)], st),
        "ss4d_frame_from_bytes": ([vp, vp, C.c_int, vp], st),
        "ss4d_frame_to_bytes": ([vp, vp, C.c_int, C.c_int, vp], st),
        "ss4d_ball_min_max": ([vp, vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, dp, dp], st),
        "ss4d_local_threshold": ([vp, C.c_double, C.c_double, C.c_double, vp, vp, C.POINTER(Balls)], st),
        "ss4d_generate_segm_function": ([vp, C.c_double, vp, vp, C.POINTER(Balls)], st),
        "ss4d_l2norm": ([vp, C.c_double, vp, vp, dp], st),
        "ss4d_mass": ([vp, C.c_double, vp, dp], st),
        "ss4d_mcf_set_boundary_exact": ([vp, C.c_double, C.c_double, vp], st),
        "ss4d_mcf_exact_solution": ([vp, C.c_double, C.c_double, vp], st),
        "ss4d_dev_alloc": ([C.c_size_t, C.POINTER(vp)], st),
        "ss4d_dev_free": ([vp], st),
        "ss4d_host_alloc": ([C.c_size_t, C.POINTER(vp)], st),
        "ss4d_host_free": ([vp], st),
        "ss4d_copy_to_device": ([vp, vp, vp, C.c_size_t], st),
        "ss4d_copy_to_host": ([vp, vp, vp, C.c_size_t], st),
        "ss4d_copy_to_device_side": ([vp, vp, vp, C.c_size_t], st),
        "ss4d_presmooth_explicit": ([vp, C.POINTER(Params), C.c_int, vp, vp], st),
        "ss4d_gaussian_smooth": ([vp, dp, vp, vp], st),
        "ss4d_seg_time_step_host": ([vp, C.POINTER(Params), vp, vp, vp, vp, vp, P8, C.POINTER(Balls),
                                     C.POINTER(StepStats)], st),
        "ss4d_gfaces": ([vp, C.POINTER(Params), vp, vp, P8], st),
        "ss4d_join_side": ([vp], st),
        "ss4d_copy_device": ([vp, vp, vp, C.c_size_t], st),
        "ss4d_synchronize": ([vp], st),
        "ss4d_scene_generate": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, vp, vp, C.c_int], st),
        "ss4d_batch_create": ([C.c_int, C.POINTER(Dims), vp, C.POINTER(vp)], st),
        "ss4d_batch_destroy": ([vp], st),
        "ss4d_batch_set_graph": ([vp, C.c_int], st),
        "ss4d_batch_set_persistent": ([vp, C.c_int], st),
        "ss4d_batch_set_test_withhold_barrier": ([vp, C.c_int], st),
        "ss4d_batch_set_arith": ([vp, C.c_int], st),
        "ss4d_batch_set_extrapolation": ([vp, C.c_int], st),
        "ss4d_batch_set_projection": ([vp, C.c_int], st),
        "ss4d_batch_set_shape": ([vp, C.c_int, C.c_int, C.c_int], st),
        "ss4d_batch_autotune": ([vp, C.POINTER(Params), C.POINTER(vp), C.POINTER(vp), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int)], st),
        "ss4d_batch_seg_time_step": ([vp, C.POINTER(Params), C.POINTER(vp), C.POINTER(vp), C.POINTER(StepStats)], st),
        "ss4d_wsnet_param_count": ([], C.c_size_t),
        "ss4d_wsnet_create": ([vp, C.POINTER(vp)], st),
        "ss4d_wsnet_destroy": ([vp], st),
        "ss4d_wsnet_set_stream": ([vp, vp], st),
        "ss4d_wsnet_init": ([vp, C.c_uint64], st),
        "ss4d_wsnet_set_params": ([vp, vp], st),
        "ss4d_wsnet_get_params": ([vp, vp], st),
        "ss4d_wsnet_forward": ([vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp], st),
        "ss4d_wsnet_check": ([vp], st),
        "ss4d_wsnet_set_test_withhold_loads": ([vp, C.c_int], st),
        "ss4d_wsnet_train_step": ([vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                   C.POINTER(C.c_float), vp], st),
        "ss4d_ws_features": ([vp, C.POINTER(Params), vp, P8, vp, vp, dp], st),
        "ss4d_solver_set_warm_start": ([vp, vp, vp], st),
        "ss4d_solver_set_extrapolation": ([vp, C.c_int], st),
        "ss4d_solver_set_projection": ([vp, C.c_int], st),
        "ss4d_solver_set_inner_omega": ([vp, C.c_double], st),
        "ss4d_solver_set_warm_start_gate": ([vp, C.c_int], st),
        "ss4d_slab_partition": ([C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)], st),
        "ss4d_slab_sor_loop": ([C.POINTER(SlabOps), C.POINTER(SlabComm), C.POINTER(Params), C.c_longlong,
                                C.POINTER(StepStats)], st),
        "ss4d_slab_sor_solve": ([vp, C.POINTER(Params), vp, vp, P8, C.POINTER(SlabComm), C.c_longlong,
                                 C.POINTER(StepStats)], st),
        "ss4d_slab_seg_time_step": ([vp, C.POINTER(Params), vp, vp, P8, vp, C.POINTER(Balls), C.POINTER(SlabComm),
                                     C.c_longlong, C.POINTER(StepStats)], st),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    if L.ss4d_abi_version() != ABI_VERSION:
        raise SS4DError(6, "libss4d.so has another ABI version",
                        f"({L.ss4d_abi_version()}, this binding expects {ABI_VERSION}; rebuild)")
    _lib = L
    return L


def declared_symbols() -> list[str]:
    """Names of the functions include/ss4d.h declares."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "ss4d.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"\b(ss4d_[a-z0-9_]+)\s*\(", text)))


def _ptr(x) -> int | None:
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if hasattr(x, "ctypes"):  # numpy array (host memory)
        return int(x.ctypes.data)
    return int(x)


def _check(status: int, what: str):
    if status != 0:
        raise SS4DError(status, what, lib().ss4d_last_error().decode(errors="replace"))


def device_count() -> int:
    n = C.c_int(0)
    s = lib().ss4d_device_count(C.byref(n))
    return n.value if s == 0 else 0


def scene(kind: int, nx: int, ny: int, nz: int, nt: int, seed: int, threads: int = 0):
    """Synthetic scene (host numpy arrays i0, u0 in the padded layout)."""
    import numpy as np
    shape = (nt + 2, nz + 2, ny + 2, nx + 2)
    i0 = np.empty(shape, dtype=np.float64)
    u0 = np.empty(shape, dtype=np.float64)
    _check(lib().ss4d_scene_generate(kind, nx, ny, nz, nt, seed, i0.ctypes.data, u0.ctypes.data, threads),
           "scene_generate")
    return i0, u0


def vtk_write_frame(path: str, bytes_xyz, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0)):
    """One frame file (the reference's header, then the bytes); bytes_xyz is a
    uint8 array [nz][ny][nx]."""
    import numpy as np
    b = np.ascontiguousarray(bytes_xyz, dtype=np.uint8)
    nz, ny, nx = b.shape
    o, sp = (C.c_double * 3)(*origin), (C.c_double * 3)(*spacing)
    _check(lib().ss4d_vtk_write_frame(path.encode(), nx, ny, nz, o, sp, b.ctypes.data), "vtk_write_frame")


def vtk_read_frame(path: str, nx: int, ny: int, nz: int):
    import numpy as np
    out = np.empty((nz, ny, nx), dtype=np.uint8)
    _check(lib().ss4d_vtk_read_frame(path.encode(), nx, ny, nz, out.ctypes.data), "vtk_read_frame")
    return out


def vtk_read_centers(path: str, spacing=(1.0, 1.0, 1.0), max_points: int = 4096):
    """[(x, y, z)] in voxel units, as the reference's _readData_ converts them"""
    cx, cy, cz = ((C.c_double * max_points)() for _ in range(3))
    n = C.c_int(0)
    sp = (C.c_double * 3)(*spacing)
    _check(lib().ss4d_vtk_read_centers(path.encode(), sp, max_points, cx, cy, cz, C.byref(n)), "vtk_read_centers")
    return [(cx[i], cy[i], cz[i]) for i in range(n.value)]


def _p8(arrs):
    if arrs is None:
        return None
    P8 = C.c_void_p * 8
    return P8(*[_ptr(a) for a in arrs])


def _balls(balls):
    """balls: None or a list of (l, cx, cy, cz) in frame order."""
    if not balls:
        return None, None
    n = len(balls)
    keep = ((C.c_int * n)(*[b[0] for b in balls]), (C.c_double * n)(*[b[1] for b in balls]),
            (C.c_double * n)(*[b[2] for b in balls]), (C.c_double * n)(*[b[3] for b in balls]))
    B = Balls(n, C.cast(keep[0], C.POINTER(C.c_int)), C.cast(keep[1], C.POINTER(C.c_double)),
              C.cast(keep[2], C.POINTER(C.c_double)), C.cast(keep[3], C.POINTER(C.c_double)))
    return B, keep


def rescale_to_zero_one_noalloc(dims: tuple, p: Params, img, mmask=None, balls=None, stream: int | None = None):
    """ss4d_rescale_to_zero_one_noalloc: the per-step rescale for callers that
    cannot allocate device memory (no handle; fixed internal table of at most
    SS4D_NOALLOC_MAX_BALLS centres and frames).  dims = (iMax, jMax, kMax, lMax).

    No handle checks the arrays against dims here, so this wrapper does:
    img (and mmask, if given) must be contiguous float64 CUDA tensors of shape
    (lMax, kMax, jMax, iMax); anything else raises ValueError before the call."""
    want = tuple(int(x) for x in dims)[::-1]
    for name, a in (("img", img), ("mmask", mmask)):
        if a is None and name == "mmask":
            continue
        if not (hasattr(a, "is_cuda") and a.is_cuda):
            raise ValueError(f"{name} must be a CUDA tensor (device memory)")
        if str(a.dtype) != "torch.float64":
            raise ValueError(f"{name} must be float64, not {a.dtype}")
        if not a.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
        if tuple(a.shape) != want:
            raise ValueError(f"{name} has shape {tuple(a.shape)}; dims {tuple(dims)} need {want}")
    B, keep = _balls(balls)
    d = Dims(*dims)
    _check(lib().ss4d_rescale_to_zero_one_noalloc(C.byref(d), C.byref(p), _ptr(img), _ptr(mmask),
                                                   C.byref(B) if B is not None else None, stream),
           "rescale_to_zero_one_noalloc")
    del keep


class Solver:
    """A solver handle bound to one volume size (padded extents)."""

    def __init__(self, iMax: int, jMax: int, kMax: int, lMax: int, arith: str = "fp64", stream: int | None = None):
        self.L = lib()
        self.dims = Dims(iMax, jMax, kMax, lMax)
        h = C.c_void_p()
        _check(self.L.ss4d_solver_create(C.byref(self.dims), ARITH[arith], stream, C.byref(h)), "solver_create")
        self.h = h

    @classmethod
    def for_interior(cls, nx, ny, nz, nt, **kw):
        return cls(nx + 2, ny + 2, nz + 2, nt + 2, **kw)

    def close(self):
        if getattr(self, "h", None):
            self.L.ss4d_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # settings
    def set_arith(self, arith: str):
        _check(self.L.ss4d_solver_set_arith(self.h, ARITH[arith]), "set_arith")

    def set_graph(self, on: bool):
        _check(self.L.ss4d_solver_set_graph(self.h, 1 if on else 0), "set_graph")

    def set_inner_omega(self, omega: float):
        """mixed form: relaxation factor of the FP32 sweeps (0: the step's omega_c)"""
        _check(self.L.ss4d_solver_set_inner_omega(self.h, float(omega)), "set_inner_omega")

    def set_extrapolation(self, order: int):
        """mixed form: start each segmentation step from an extrapolation in
        time of the earlier steps' changes (0 off, order 1, 2 or 3)"""
        _check(self.L.ss4d_solver_set_extrapolation(self.h, int(order)), "set_extrapolation")

    def set_projection(self, enable: bool):
        """mixed form with extrapolation of order 3: start each step's first
        FP32 round from the least-residual combination of the earlier changes"""
        _check(self.L.ss4d_solver_set_projection(self.h, 1 if enable else 0), "set_projection")

    def set_stream(self, stream: int | None):
        _check(self.L.ss4d_solver_set_stream(self.h, stream), "set_stream")

    def set_tiling(self, k_block: int, max_grid: int = 0):
        _check(self.L.ss4d_solver_set_tiling(self.h, k_block, max_grid), "set_tiling")

    def set_assembly_order(self, planes: int):
        """block order of the mixed form's assembly: 0 frame by frame, n >= 1
        in blocks of n k planes across the frames"""
        _check(self.L.ss4d_solver_set_assembly_order(self.h, planes), "set_assembly_order")

    KERNELS = ("sweep64", "sweep32", "refine", "assemble", "pack", "warm", "project")

    def set_timing(self, on: bool):
        _check(self.L.ss4d_solver_set_timing(self.h, 1 if on else 0), "set_timing")

    def reset_timing(self):
        _check(self.L.ss4d_solver_reset_timing(self.h), "reset_timing")

    def kernel_times(self) -> dict:
        """{kernel: (total ms, launches)} accumulated while timing was on."""
        out = {}
        for k, name in enumerate(self.KERNELS):
            ms, n = C.c_double(0), C.c_longlong(0)
            _check(self.L.ss4d_solver_kernel_time(self.h, k, C.byref(ms), C.byref(n)), "kernel_time")
            out[name] = (ms.value, n.value)
        return out

    def workspace_bytes(self) -> int:
        v = C.c_size_t(0)
        _check(self.L.ss4d_solver_workspace_bytes(self.h, C.byref(v)), "workspace_bytes")
        return v.value

    def launch_count(self) -> int:
        v = C.c_longlong(0)
        _check(self.L.ss4d_solver_launch_count(self.h, C.byref(v)), "launch_count")
        return v.value

    # hot path
    def reflect(self, img):
        _check(self.L.ss4d_reflect(self.h, _ptr(img)), "reflect")

    def presmooth_step(self, p: Params, img, scratch=None) -> dict:
        st = StepStats()
        _check(self.L.ss4d_presmooth_step(self.h, C.byref(p), _ptr(img), _ptr(scratch), C.byref(st)), "presmooth")
        return st.as_dict()

    def presmooth_explicit(self, p: Params, steps: int, img, scratch=None):
        """_presmoothStepEXP_ on img; scratch (optional) receives the reference's prev_u"""
        _check(self.L.ss4d_presmooth_explicit(self.h, C.byref(p), int(steps), _ptr(img), _ptr(scratch)),
               "presmooth_explicit")

    def seg_time_step_host(self, p: Params, h_u, d_u, g8, h_prev=None, h_mmask=None, d_mmask=None,
                           balls=None) -> dict:
        """ss4d_seg_time_step_host: h_u, h_prev, h_mmask are page-locked host
        buffers (numpy views of ss4d_host_alloc memory), d_u / d_mmask their
        device mirrors"""
        B, keep = _balls(balls)
        st = StepStats()
        _check(self.L.ss4d_seg_time_step_host(self.h, C.byref(p), h_u.ctypes.data, _ptr(d_u),
                                              h_prev.ctypes.data if h_prev is not None else None,
                                              h_mmask.ctypes.data if h_mmask is not None else None, _ptr(d_mmask),
                                              _p8(g8), C.byref(B) if B is not None else None, C.byref(st)),
               "seg_time_step_host")
        del keep
        return st.as_dict()

    def gaussian_smooth(self, sigma, img, scratch=None):
        """separable Gaussian, sigma per axis (x, y, z, t), in place on img"""
        s = (C.c_double * 4)(*[float(x) for x in sigma])
        _check(self.L.ss4d_gaussian_smooth(self.h, s, _ptr(img), _ptr(scratch)), "gaussian_smooth")

    def gfaces(self, p: Params, i0, i0_thr, g8):
        """the 8 face g values from images already smoothed"""
        _check(self.L.ss4d_gfaces(self.h, C.byref(p), _ptr(i0), _ptr(i0_thr), _p8(g8)), "gfaces")

    def edge_detector(self, p: Params, i0, i0_thr, g8, scratch=None):
        _check(self.L.ss4d_edge_detector(self.h, C.byref(p), _ptr(i0), _ptr(i0_thr), _ptr(scratch), _p8(g8)),
               "edge_detector")

    def gs_coefficients(self, p: Params, u, g8, coef8):
        _check(self.L.ss4d_gs_coefficients(self.h, C.byref(p), _ptr(u), _p8(g8), _p8(coef8)), "gs_coefficients")

    def sor_solve(self, p: Params, u, prev, coef8) -> dict:
        st = StepStats()
        _check(self.L.ss4d_sor_solve(self.h, C.byref(p), _ptr(u), _ptr(prev), _p8(coef8), C.byref(st)), "sor_solve")
        return st.as_dict()

    def seg_time_step(self, p: Params, u, prev, g8, mmask=None, balls=None) -> dict:
        st = StepStats()
        B, keep = _balls(balls)
        _check(self.L.ss4d_seg_time_step(self.h, C.byref(p), _ptr(u), _ptr(prev), _p8(g8), _ptr(mmask),
                                         C.byref(B) if B is not None else None, C.byref(st)), "seg_time_step")
        del keep
        return st.as_dict()

    def ws_features(self, p: Params, u, g8, i0, x0) -> float:
        """Warm-start features of the step from u (BF16, planar [nt][2][nz][ny][nx][8]
        into x0); returns the RMS s of the step's initial residual."""
        sig = C.c_double(0)
        _check(self.L.ss4d_ws_features(self.h, C.byref(p), _ptr(u), _p8(g8), _ptr(i0), _ptr(x0), C.byref(sig)),
               "ws_features")
        return sig.value

    def set_warm_start_gate(self, min_iterations: int):
        """run the network only after a mixed step of >= min_iterations FP32 sweeps (0: always)"""
        _check(self.L.ss4d_solver_set_warm_start_gate(self.h, int(min_iterations)), "set_warm_start_gate")

    def slab_sor_solve(self, p: Params, u, prev, coef8, comm: SlabComm, nint_global: int) -> dict:
        """ss4d_slab_sor_solve: this handle's volume is one slab of a volume
        split by frames; comm exchanges ghost frames and sums the residual"""
        st = StepStats()
        _check(self.L.ss4d_slab_sor_solve(self.h, C.byref(p), _ptr(u), _ptr(prev), _p8(coef8), C.byref(comm),
                                          nint_global, C.byref(st)), "slab_sor_solve")
        return st.as_dict()

    def slab_seg_time_step(self, p: Params, u, prev, g8, comm: SlabComm, nint_global: int, mmask=None,
                           balls=None) -> dict:
        """ss4d_slab_seg_time_step: one time step of this slab"""
        st = StepStats()
        B, keep = _balls(balls)
        _check(self.L.ss4d_slab_seg_time_step(self.h, C.byref(p), _ptr(u), _ptr(prev), _p8(g8), _ptr(mmask),
                                              C.byref(B) if B is not None else None, C.byref(comm), nint_global,
                                              C.byref(st)), "slab_seg_time_step")
        del keep
        return st.as_dict()

    def set_warm_start(self, net, i0):
        """Attach a `Wsnet` (None detaches); i0 is the presmoothed image.  The
        mixed-form segmentation steps then start from its prediction."""
        self._ws_keep = (net, i0)
        _check(self.L.ss4d_solver_set_warm_start(self.h, net.h if net is not None else None,
                                                 _ptr(i0) if net is not None else None), "set_warm_start")

    def mcf_time_step(self, p: Params, step: int, u, prev=None) -> dict:
        st = StepStats()
        _check(self.L.ss4d_mcf_time_step(self.h, C.byref(p), step, _ptr(u), _ptr(prev), C.byref(st)), "mcf_time_step")
        return st.as_dict()

    def rescale_to_zero_one(self, p: Params, img, mmask=None, balls=None):
        B, keep = _balls(balls)
        _check(self.L.ss4d_rescale_to_zero_one(self.h, C.byref(p), _ptr(img), _ptr(mmask),
                                               C.byref(B) if B is not None else None), "rescale")
        del keep

    # frame files (segmentation4D.c:1149-1324)
    def frame_from_bytes(self, img, l: int, dbytes):
        _check(self.L.ss4d_frame_from_bytes(self.h, _ptr(img), l, _ptr(dbytes)), "frame_from_bytes")

    def frame_to_bytes(self, img, l: int, dbytes, mode: int = 0):
        _check(self.L.ss4d_frame_to_bytes(self.h, _ptr(img), l, mode, _ptr(dbytes)), "frame_to_bytes")

    # initial segmentation (segmentation4D.c:876-1018, 1106-1147)
    def max4d(self, img) -> float:
        v = C.c_double(0)
        _check(self.L.ss4d_max4d(self.h, _ptr(img), C.byref(v)), "max4d")
        return v.value

    def ball_min_max(self, img, l: int, cx: float, cy: float, cz: float, R: float):
        mn, mx = C.c_double(0), C.c_double(0)
        _check(self.L.ss4d_ball_min_max(self.h, _ptr(img), l, cx, cy, cz, R, C.byref(mn), C.byref(mx)),
               "ball_min_max")
        return mn.value, mx.value

    def local_threshold(self, alpha: float, beta: float, ball_radius: float, img, thr, balls):
        B, keep = _balls(balls)
        _check(self.L.ss4d_local_threshold(self.h, alpha, beta, ball_radius, _ptr(img), _ptr(thr),
                                           C.byref(B) if B is not None else None), "local_threshold")
        del keep

    def generate_segm_function(self, ball_radius: float, u, mmask, balls):
        B, keep = _balls(balls)
        _check(self.L.ss4d_generate_segm_function(self.h, ball_radius, _ptr(u), _ptr(mmask),
                                                  C.byref(B) if B is not None else None), "generate_segm_function")
        del keep

    def threshold_mask(self, u, mask, level: float = 0.5, normalise: bool = False):
        _check(self.L.ss4d_threshold_mask(self.h, _ptr(u), level, 1 if normalise else 0, _ptr(mask)), "threshold_mask")

    def l2norm(self, h: float, a, b) -> float:
        v = C.c_double(0)
        _check(self.L.ss4d_l2norm(self.h, h, _ptr(a), _ptr(b), C.byref(v)), "l2norm")
        return v.value

    def mass(self, h: float, a) -> float:
        v = C.c_double(0)
        _check(self.L.ss4d_mass(self.h, h, _ptr(a), C.byref(v)), "mass")
        return v.value

    def mcf_set_boundary_exact(self, h: float, t: float, u):
        _check(self.L.ss4d_mcf_set_boundary_exact(self.h, h, t, _ptr(u)), "mcf_set_boundary_exact")

    def mcf_exact_solution(self, h: float, t: float, out):
        _check(self.L.ss4d_mcf_exact_solution(self.h, h, t, _ptr(out)), "mcf_exact_solution")

    def synchronize(self):
        _check(self.L.ss4d_synchronize(self.h), "synchronize")

    def copy_to_device_side(self, dst, src):
        """Host -> device copy on the handle's side stream (after the work queued
        so far); ``join_side`` orders it before the calls that follow.  ``src``
        must stay alive until then."""
        import numpy as np
        src = np.ascontiguousarray(src)
        _check(self.L.ss4d_copy_to_device_side(self.h, _ptr(dst), src.ctypes.data, src.nbytes), "copy_to_device_side")
        return src

    def join_side(self):
        _check(self.L.ss4d_join_side(self.h), "join_side")


class Batch:
    """ss4d_batch: many volumes (uneven sizes, own parameters) stepped together
    in the plain FP64 form (or the mixed form, set_arith), one persistent launch
    per loop kernel for all."""

    def __init__(self, dims_list, stream: int | None = None):
        self.L = lib()
        n = len(dims_list)
        arr = (Dims * n)(*[Dims(*d) for d in dims_list])
        h = C.c_void_p()
        _check(self.L.ss4d_batch_create(n, arr, stream, C.byref(h)), "batch_create")
        self.h, self.n = h, n

    def close(self):
        if getattr(self, "h", None):
            self.L.ss4d_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_graph(self, on: bool):
        _check(self.L.ss4d_batch_set_graph(self.h, 1 if on else 0), "batch_set_graph")

    def set_persistent(self, on: bool):
        """the SOR loop as one persistent launch (default) or as the graph's while loop"""
        _check(self.L.ss4d_batch_set_persistent(self.h, 1 if on else 0), "batch_set_persistent")

    def set_test_withhold_barrier(self, on: bool):
        """test of the timeout path: the persistent loop's grid barrier can
        never complete, so the next step returns SS4D_ERR_TIMEOUT"""
        _check(self.L.ss4d_batch_set_test_withhold_barrier(self.h, 1 if on else 0), "batch_set_test_withhold_barrier")

    def set_shape(self, v: int, xt: int, k_block: int):
        _check(self.L.ss4d_batch_set_shape(self.h, v, xt, k_block), "batch_set_shape")

    def set_arith(self, arith: str):
        _check(self.L.ss4d_batch_set_arith(self.h, ARITH[arith]), "batch_set_arith")

    def set_extrapolation(self, order: int):
        _check(self.L.ss4d_batch_set_extrapolation(self.h, order), "batch_set_extrapolation")

    def set_projection(self, enable: bool):
        """every volume's first FP32 round from its projected start (with order 3)"""
        _check(self.L.ss4d_batch_set_projection(self.h, 1 if enable else 0), "batch_set_projection")

    @staticmethod
    def _args(params, us, gs):
        n = len(us)
        P = (Params * n)(*params)
        U = (C.c_void_p * n)(*[_ptr(u) for u in us])
        G = (C.c_void_p * (8 * n))(*[_ptr(g) for g8 in gs for g in g8])
        return P, U, G

    def autotune(self, params, us, gs):
        P, U, G = self._args(params, us, gs)
        xt = (C.c_int * self.n)()
        kb = (C.c_int * self.n)()
        _check(self.L.ss4d_batch_autotune(self.h, P, U, G, xt, kb), "batch_autotune")
        return list(zip(list(xt), list(kb)))

    def seg_time_step(self, params, us, gs) -> list:
        P, U, G = self._args(params, us, gs)
        S = (StepStats * self.n)()
        _check(self.L.ss4d_batch_seg_time_step(self.h, P, U, G, S), "batch_seg_time_step")
        return [s.as_dict() for s in S]


def features_to_planar(x):
    """[F][nz][ny][nx][C] -> the network's channel-group planar layout
    [F][C/8][nz][ny][nx][8] (torch tensor or numpy array; a contiguous copy)"""
    F, nz, ny, nx, C = x.shape
    y = x.reshape(F, nz, ny, nx, C // 8, 8)
    y = y.permute(0, 4, 1, 2, 3, 5) if hasattr(y, "permute") else y.transpose(0, 4, 1, 2, 3, 5)
    return y.contiguous() if hasattr(y, "contiguous") else y.copy()


def features_from_planar(x):
    """[F][G][nz][ny][nx][8] -> [F][nz][ny][nx][8 G]"""
    F, G, nz, ny, nx, e = x.shape
    y = x.permute(0, 2, 3, 4, 1, 5) if hasattr(x, "permute") else x.transpose(0, 2, 3, 4, 1, 5)
    return y.reshape(F, nz, ny, nx, G * e)


class Wsnet:
    """ss4d_wsnet: the learned warm start's convolutional network (BF16
    weights/activations, FP32 master parameters and Adam state on the device).
    Parameter vector layout: per layer L = 0..3, weights [27][cout][cin]
    (tap = 9 dz + 3 dy + dx, offsets -1..1, x fastest) then bias [cout];
    channels 16 -> 24 -> 24 -> 24 -> 1.  Features are channel-group planar,
    [F][2][nz][ny][nx][8] BF16 (features_to_planar)."""

    LAYERS = ((16, 24), (24, 24), (24, 24), (24, 1))

    def __init__(self, stream: int | None = None, seed: int | None = 0):
        self.L = lib()
        h = C.c_void_p()
        _check(self.L.ss4d_wsnet_create(stream, C.byref(h)), "wsnet_create")
        self.h = h
        self.nparam = int(self.L.ss4d_wsnet_param_count())
        if seed is not None:
            self.init(seed)

    def close(self):
        if getattr(self, "h", None):
            self.L.ss4d_wsnet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream: int | None):
        _check(self.L.ss4d_wsnet_set_stream(self.h, stream), "wsnet_set_stream")

    def init(self, seed: int):
        _check(self.L.ss4d_wsnet_init(self.h, seed), "wsnet_init")

    def get_params(self):
        import numpy as np
        out = np.empty(self.nparam, dtype=np.float32)
        _check(self.L.ss4d_wsnet_get_params(self.h, out.ctypes.data), "wsnet_get_params")
        return out

    def set_params(self, params):
        import numpy as np
        a = np.ascontiguousarray(params, dtype=np.float32)
        if a.size != self.nparam:
            raise SS4DError(1, "wsnet_set_params", f"expected {self.nparam} values, got {a.size}")
        _check(self.L.ss4d_wsnet_set_params(self.h, a.ctypes.data), "wsnet_set_params")

    def forward(self, x0, nx: int, ny: int, nz: int, nf: int, out):
        _check(self.L.ss4d_wsnet_forward(self.h, _ptr(x0), nx, ny, nz, nf, _ptr(out)), "wsnet_forward")

    def check(self):
        """synchronise; SS4DError (SS4D_ERR_TIMEOUT) if a convolution of the
        last forward gave up a bounded wait"""
        _check(self.L.ss4d_wsnet_check(self.h), "wsnet_check")

    def set_test_withhold_loads(self, on: bool):
        """test of the timeout path: the convolutions issue no loads, so their
        waits run out and the prediction is NaN"""
        _check(self.L.ss4d_wsnet_set_test_withhold_loads(self.h, 1 if on else 0), "wsnet_set_test_withhold_loads")

    def train_step(self, x0, target, nx: int, ny: int, nz: int, nf: int, margin: int = 0, lr: float = 1e-3,
                   grad=None) -> float:
        loss = C.c_float(0)
        _check(self.L.ss4d_wsnet_train_step(self.h, _ptr(x0), _ptr(target), nx, ny, nz, nf, margin, lr,
                                            C.byref(loss), _ptr(grad)), "wsnet_train_step")
        return loss.value

    @classmethod
    def split(cls, params):
        """[(W [27][cout][cin], b [cout]) per layer] views of a parameter vector."""
        out, off = [], 0
        for cin, cout in cls.LAYERS:
            nw = 27 * cout * cin
            out.append((params[off:off + nw].reshape(27, cout, cin), params[off + nw:off + nw + cout]))
            off += nw + cout
        return out
