"""ctypes wrapper of the CPU oracle (oracle/ss4d_oracle.c) — TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
the checker of the CUDA path; the product never imports it.  Arrays are
numpy float64 in the reference's padded layout, shape (lMax, kMax, jMax, iMax).
Parameters are an ``ss4d_params``-layout ctypes structure (include/ss4d.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libss4d_oracle.so")


class _Dims(C.Structure):
    _fields_ = [("iMax", C.c_int), ("jMax", C.c_int), ("kMax", C.c_int), ("lMax", C.c_int)]


_L = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib() -> C.CDLL:
    global _L
    if _L is None:
        if not os.path.exists(LIB):
            build()
        _L = C.CDLL(LIB)
        vp = C.c_void_p
        _L.or_presmooth.restype = C.c_int
        _L.or_sor.restype = C.c_int
        _L.or_seg_time_step.restype = C.c_int
        _L.or_mcf_time_step.restype = C.c_int
        _L.or_rescale.restype = C.c_int
        _L.or_l2norm.restype = C.c_double
        _L.or_mass.restype = C.c_double
        _L.or_max_threads.restype = C.c_int
        _L.or_l2norm.argtypes = [vp, C.c_double, vp, vp]
        _L.or_mass.argtypes = [vp, C.c_double, vp]
        _L.or_mcf_exact_solution.argtypes = [vp, C.c_double, C.c_double, vp]
        _L.or_mcf_set_boundary.argtypes = [vp, C.c_double, C.c_double, vp]
        _L.or_threshold_mask.argtypes = [vp, vp, C.c_double, C.c_int, vp]
        _L.or_rescale.argtypes = [vp, C.c_double, vp, vp, C.c_int, vp, vp, vp, vp]
        _L.or_max4d.restype = C.c_double
        _L.or_max4d.argtypes = [vp, vp]
        _L.or_ball_min_max.restype = C.c_int
        _L.or_ball_min_max.argtypes = [vp, vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _L.or_local_threshold.restype = C.c_int
        _L.or_local_threshold.argtypes = [vp, C.c_double, C.c_double, C.c_double, vp, vp, C.c_int, vp, vp, vp, vp]
        _L.or_generate_segm.restype = C.c_int
        _L.or_generate_segm.argtypes = [vp, C.c_double, vp, vp, C.c_int, vp, vp, vp, vp]
    return _L


def set_threads(n: int):
    lib().or_set_threads(int(n))


def max_threads() -> int:
    return int(lib().or_max_threads())


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def _dims(shape) -> _Dims:
    lM, kM, jM, iM = shape
    return _Dims(iM, jM, kM, lM)


def _p8(arrs):
    return (C.c_void_p * 8)(*[_d(a) for a in arrs])


def new_like(a: np.ndarray, n: int = 1):
    return [np.zeros_like(a) for _ in range(n)]


def reflect(v: np.ndarray):
    d = _dims(v.shape)
    lib().or_reflect(C.byref(d), C.c_void_p(_d(v)))


def presmooth(p, v: np.ndarray, scratch: np.ndarray | None = None):
    d = _dims(v.shape)
    scratch = np.zeros_like(v) if scratch is None else scratch
    R = C.c_double(0)
    z = lib().or_presmooth(C.byref(d), C.byref(p), C.c_void_p(_d(v)), C.c_void_p(_d(scratch)), C.byref(R))
    return z, R.value


def presmooth_explicit(p, steps: int, v: np.ndarray, scratch: np.ndarray | None = None):
    """_presmoothStepEXP_ in place on v; scratch receives the reference's prev_u"""
    d = _dims(v.shape)
    scratch = np.zeros_like(v) if scratch is None else scratch
    lib().or_presmooth_explicit(C.byref(d), C.byref(p), C.c_int(steps), C.c_void_p(_d(v)), C.c_void_p(_d(scratch)))
    return scratch


def gaussian(sigma, v: np.ndarray, scratch: np.ndarray | None = None) -> int:
    """separable Gaussian with sigma per axis (x, y, z, t) in place on v"""
    d = _dims(v.shape)
    scratch = np.zeros_like(v) if scratch is None else scratch
    s = (C.c_double * 4)(*[float(x) for x in sigma])
    return lib().or_gaussian(C.byref(d), s, C.c_void_p(_d(v)), C.c_void_p(_d(scratch)))


def gfaces(p, i0: np.ndarray, ithr: np.ndarray):
    d = _dims(i0.shape)
    g = new_like(i0, 8)
    lib().or_gfaces(C.byref(d), C.byref(p), C.c_void_p(_d(i0)), C.c_void_p(_d(ithr)), _p8(g))
    return g


def edge_detector(p, i0: np.ndarray, ithr: np.ndarray):
    """presmooth i0 and ithr in place, then the 8 face g arrays"""
    d = _dims(i0.shape)
    g = new_like(i0, 8)
    scratch = np.zeros_like(i0)
    z0, z1 = C.c_int(0), C.c_int(0)
    lib().or_edge_detector(C.byref(d), C.byref(p), C.c_void_p(_d(i0)), C.c_void_p(_d(ithr)),
                           C.c_void_p(_d(scratch)), _p8(g), C.byref(z0), C.byref(z1))
    return g, (z0.value, z1.value), scratch


def coefficients(p, u: np.ndarray, g=None):
    d = _dims(u.shape)
    coef = new_like(u, 8)
    lib().or_coefficients(C.byref(d), C.byref(p), C.c_void_p(_d(u)), _p8(g) if g is not None else None, _p8(coef))
    return coef


def sor(p, u: np.ndarray, prev: np.ndarray, coef):
    d = _dims(u.shape)
    R = C.c_double(0)
    z = lib().or_sor(C.byref(d), C.byref(p), C.c_void_p(_d(u)), C.c_void_p(_d(prev)), _p8(coef), C.byref(R))
    return z, R.value


def sor_half(p, u: np.ndarray, prev: np.ndarray, coef, colour: int):
    """one red (0) or black (1) half-sweep of the SOR loop over u's interior"""
    lib().or_sor_half(C.byref(_dims(u.shape)), C.byref(p), C.c_void_p(_d(u)), C.c_void_p(_d(prev)), _p8(coef),
                      C.c_int(colour))


def sor_residual(p, u: np.ndarray, prev: np.ndarray, coef) -> float:
    """the SOR loop's residual sum r^2 h^4 over u's interior"""
    f = lib().or_sor_residual
    f.restype = C.c_double
    return f(C.byref(_dims(u.shape)), C.byref(p), C.c_void_p(_d(u)), C.c_void_p(_d(prev)), _p8(coef))


def _balls(balls):
    if not balls:
        return 0, None, None, None, None
    bl = np.ascontiguousarray([b[0] for b in balls], dtype=np.int32)
    bx = np.ascontiguousarray([b[1] for b in balls], dtype=np.float64)
    by = np.ascontiguousarray([b[2] for b in balls], dtype=np.float64)
    bz = np.ascontiguousarray([b[3] for b in balls], dtype=np.float64)
    return len(balls), bl, bx, by, bz


def seg_time_step(p, u, prev, g, coef=None, mmask=None, balls=None):
    d = _dims(u.shape)
    coef = new_like(u, 8) if coef is None else coef
    nb, bl, bx, by, bz = _balls(balls)
    R = C.c_double(0)
    z = lib().or_seg_time_step(C.byref(d), C.byref(p), C.c_void_p(_d(u)), C.c_void_p(_d(prev)), _p8(g), _p8(coef),
                               C.c_void_p(_d(mmask)) if mmask is not None else None, C.c_int(nb),
                               C.c_void_p(bl.ctypes.data) if nb else None, C.c_void_p(bx.ctypes.data) if nb else None,
                               C.c_void_p(by.ctypes.data) if nb else None, C.c_void_p(bz.ctypes.data) if nb else None,
                               C.byref(R))
    return z, R.value


def mcf_time_step(p, step: int, u, prev, coef=None):
    d = _dims(u.shape)
    coef = new_like(u, 8) if coef is None else coef
    R = C.c_double(0)
    z = lib().or_mcf_time_step(C.byref(d), C.byref(p), C.c_int(step), C.c_void_p(_d(u)), C.c_void_p(_d(prev)),
                               _p8(coef), C.byref(R))
    return z, R.value


def rescale(R: float, v, mmask=None, balls=None) -> int:
    d = _dims(v.shape)
    nb, bl, bx, by, bz = _balls(balls)
    return lib().or_rescale(C.byref(d), R, _d(v), _d(mmask) if mmask is not None else None, nb,
                            bl.ctypes.data if nb else None, bx.ctypes.data if nb else None,
                            by.ctypes.data if nb else None, bz.ctypes.data if nb else None)


def max4d(v) -> float:
    """_get4DMax_ (segmentation4D.c:876-895)"""
    return lib().or_max4d(C.byref(_dims(v.shape)), _d(v))


def ball_min_max(v, l: int, cx: float, cy: float, cz: float, R: float):
    """_get3DMinWithinR_ / _get3DMaxWithinR_ (segmentation4D.c:897-969)"""
    mn, mx = C.c_double(0), C.c_double(0)
    rc = lib().or_ball_min_max(C.byref(_dims(v.shape)), _d(v), l, cx, cy, cz, R, C.byref(mn), C.byref(mx))
    if rc != 0:
        raise ValueError("ball box leaves the array")
    return mn.value, mx.value


def local_threshold(alpha: float, beta: float, R: float, img, thr, balls) -> int:
    """_locallyThreshold4Ddata_ (segmentation4D.c:971-1018): thr updated in place"""
    nb, bl, bx, by, bz = _balls(balls)
    return lib().or_local_threshold(C.byref(_dims(img.shape)), alpha, beta, R, _d(img), _d(thr), nb,
                                    bl.ctypes.data if nb else None, bx.ctypes.data if nb else None,
                                    by.ctypes.data if nb else None, bz.ctypes.data if nb else None)


def generate_segm(R: float, u, mmask, balls) -> int:
    """_generate4DsegmFunct_ (segmentation4D.c:1106-1147): u and mmask updated in place"""
    nb, bl, bx, by, bz = _balls(balls)
    return lib().or_generate_segm(C.byref(_dims(u.shape)), R, _d(u), _d(mmask), nb,
                                  bl.ctypes.data if nb else None, bx.ctypes.data if nb else None,
                                  by.ctypes.data if nb else None, bz.ctypes.data if nb else None)


def threshold_mask(u, level=0.5, normalise=False) -> np.ndarray:
    d = _dims(u.shape)
    lM, kM, jM, iM = u.shape
    m = np.zeros((lM - 2) * (kM - 2) * (jM - 2) * (iM - 2), dtype=np.uint8)
    lib().or_threshold_mask(C.byref(d), _d(u), level, 1 if normalise else 0, m.ctypes.data)
    return m


def l2norm(h, a, b) -> float:
    return lib().or_l2norm(C.byref(_dims(a.shape)), h, _d(a), _d(b))


def mass(h, a) -> float:
    return lib().or_mass(C.byref(_dims(a.shape)), h, _d(a))


def mcf_exact(h, t, shape) -> np.ndarray:
    out = np.zeros(shape, dtype=np.float64)
    lib().or_mcf_exact_solution(C.byref(_dims(shape)), h, t, _d(out))
    return out


def mcf_boundary(h, t, u):
    lib().or_mcf_set_boundary(C.byref(_dims(u.shape)), h, t, _d(u))
