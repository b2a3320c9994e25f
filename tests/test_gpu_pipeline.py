"""The reference main's whole sequence (segmentation4D.c:1325-1420) through
the reference-named layer, on files: _readData_, _locallyThreshold4Ddata_,
_gf_inputImage_plus_thresholdedImage_, _generate4DsegmFunct_,
_rescale4DdataToZeroOne_, time steps with _l2norm_ until segTol or
maxNoOfTimeSteps, _writeData_ -- against the reference's own run of the
same sequence (tests/golden/pipeline.npz)."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import load_golden, rel_err
from test_vtk_io import VTK_HEADER

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("arith", ["reference", "fp64"])
def test_reference_main_sequence_on_files(ss4d, cuda, tmp_path, arith):
    d = load_golden("pipeline.npz")
    nx, ny, nz, nt = (int(v) for v in d["dims"])
    shape = (nt + 2, nz + 2, ny + 2, nx + 2)
    lM, kM, jM, iM = shape
    for l in range(1, nt + 1):
        with open(tmp_path / ("movingBalls_457_at_time_%03d.vtk" % l), "wb") as fh:
            fh.write(VTK_HEADER.format(nx=nx, ny=ny, nz=nz, n=nx * ny * nz).encode() + d["payloads"][l - 1].tobytes())
        with open(tmp_path / ("movingBalls_457_centers_at_timestep_%03d.vtk" % l), "w") as fh:
            fh.write(str(d["centre_texts"][l - 1]))
    os.environ["SS4D_ARITH"] = arith
    os.environ["SS4D_EXTRAPOLATE"] = "0"
    L = C.CDLL(ss4d.SEG_PATH, mode=os.RTLD_LOCAL)
    params = dict(zip((str(n) for n in d["param_names"]), d["params"]))
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM),
                  ("maxNoGSIteration", params["maxNoGSIteration"]), ("maxNoOfTimeSteps", params["maxNoOfTimeSteps"])):
        C.c_int.in_dll(L, nm).value = int(v)
    for nm in ("K", "eps2", "tau", "h", "omega_c", "gsTol", "segTol", "sigma", "omega_sigma",
               "maxNoGSIteration_sigma", "theta_img", "rho_thr", "ballRadius"):
        C.c_double.in_dll(L, nm).value = float(params[nm])
    for nm, v in zip(("spacing_x", "spacing_y", "spacing_z"), d["spacing"]):
        C.c_double.in_dll(L, nm).value = float(v)
    for nm, v in (("origin_x", 0.0), ("origin_y", 0.0), ("origin_z", 0.0), ("alpha", 0.85), ("beta", 0.15)):
        C.c_double.in_dll(L, nm).value = v
    noc = (C.c_int * lM)()
    for l, txt in enumerate(d["centre_texts"], start=1):
        noc[l] = int(str(txt).split("POINTS ")[1].split()[0])
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    for fn in ("_allocateMem_", "_deallocateMem_", "_locallyThreshold4Ddata_", "_gf_inputImage_plus_thresholdedImage_",
               "_generate4DsegmFunct_", "_rescale4DdataToZeroOne_", "_segTimeStep_", "_writeData_"):
        getattr(L, fn).restype = C.c_bool
    L._readData_.restype = None
    L._l2norm_.restype = C.c_double
    assert L._allocateMem_()
    try:
        n = int(np.prod(shape))

        def arr(name):
            addr = C.c_void_p.in_dll(L, name).value
            return np.ctypeslib.as_array((C.c_double * n).from_address(addr)).reshape(shape)

        i0, u, prev = arr("i0"), arr("u"), arr("prev_u")
        p = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
        L._readData_(p(i0), C.c_char_p(str(tmp_path).encode()))
        assert L._locallyThreshold4Ddata_(p(i0), p(u))
        assert L._gf_inputImage_plus_thresholdedImage_(p(i0), p(u))
        assert L._generate4DsegmFunct_(p(u))
        assert L._rescale4DdataToZeroOne_(p(u))
        l2s, t = [], 1
        while True:
            C.c_int.in_dll(L, "numberOfTimeStep").value = t
            assert L._segTimeStep_()
            l2s.append(L._l2norm_(p(prev), p(u)))
            t += 1
            if not (t <= params["maxNoOfTimeSteps"] and l2s[-1] > params["segTol"]):
                break
        assert L._writeData_(p(u), C.c_char_p(str(tmp_path / "result").encode()))
        tol = 1e-13 if arith == "reference" else 1e-10
        assert len(l2s) == len(d["l2"])
        assert rel_err(l2s, d["l2"]) <= tol
        assert rel_err(u, d["u_final"]) <= tol
        for l in range(1, nt + 1):
            with open(tmp_path / ("result_at_time_%03d.vtk" % l), "rb") as fh:
                got = np.frombuffer(fh.read(), dtype=np.uint8)
            assert np.array_equal(got, d["written"][l - 1]), f"frame {l}"
    finally:
        L._deallocateMem_()
        os.environ.pop("SS4D_ARITH", None)
        os.environ.pop("SS4D_EXTRAPOLATE", None)


def test_reference_named_layer_mixed_extrapolated_steps_equal_native(ss4d, cuda):
    """The path of the end-to-end measurement: _segTimeStep_() of the
    reference-named layer with SS4D_ARITH=mixed and SS4D_EXTRAPOLATE=3 on host
    arrays (Mmask uploaded beside the solve, prev_u copied on the host) gives,
    step after step, the u, prev_u and iteration counts of the native mixed
    solver with the cubic extrapolated start on the same g."""
    torch = cuda
    nx, ny, nz, nt = 40, 36, 24, 6
    p = ss4d.scene_params(maxNoOfTimeSteps=6)
    i0h, u0h = ss4d.scene(3, nx, ny, nz, nt, seed=5)
    shape = i0h.shape
    lM, kM, jM, iM = shape
    n = int(np.prod(shape))
    os.environ["SS4D_ARITH"] = "mixed"
    os.environ["SS4D_EXTRAPOLATE"] = "3"
    L = C.CDLL(ss4d.SEG_PATH, mode=os.RTLD_LOCAL)
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM), ("maxNoGSIteration", p.maxNoGSIteration),
                  ("maxNoOfTimeSteps", p.maxNoOfTimeSteps)):
        C.c_int.in_dll(L, nm).value = int(v)
    for nm in ("K", "eps2", "tau", "h", "omega_c", "gsTol", "segTol", "sigma", "omega_sigma",
               "maxNoGSIteration_sigma", "theta_img", "rho_thr", "ballRadius"):
        C.c_double.in_dll(L, nm).value = float(getattr(p, nm))
    noc = (C.c_int * lM)()
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    for fn in ("_allocateMem_", "_deallocateMem_", "_segTimeStep_", "_gf_inputImage_plus_thresholdedImage_",
               "ss4d_compat_sync_host", "ss4d_compat_last_stats"):
        getattr(L, fn).restype = C.c_bool
    assert L._allocateMem_()
    try:
        def arr(name):
            addr = C.c_void_p.in_dll(L, name).value
            return np.ctypeslib.as_array((C.c_double * n).from_address(addr)).reshape(shape)

        i0, u, prev, mm = arr("i0"), arr("u"), arr("prev_u"), arr("Mmask")
        i0[...] = i0h
        mm[...] = 1.0
        assert L._gf_inputImage_plus_thresholdedImage_(C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
        assert L.ss4d_compat_sync_host()
        g_host = [arr(nm).copy() for nm in ("g_e", "g_w", "g_n", "g_s", "g_t", "g_b", "g_fw", "g_bw")]
        u[...] = u0h
        got = []
        for _ in range(5):
            before = u.copy()
            assert L._segTimeStep_()
            st = ss4d.StepStats()
            assert L.ss4d_compat_last_stats(C.byref(st))
            assert np.array_equal(prev, before)
            got.append((st.iterations, u.copy()))
    finally:
        L._deallocateMem_()
        os.environ.pop("SS4D_ARITH", None)
        os.environ.pop("SS4D_EXTRAPOLATE", None)
    g = [torch.from_numpy(a).cuda() for a in g_host]
    ud = torch.from_numpy(u0h).cuda()
    with ss4d.Solver(*shape[::-1], arith="mixed") as S:
        S.set_extrapolation(3)
        for its, u_got in got:
            st = S.seg_time_step(p, ud, None, g)
            assert st["iterations"] == its
            assert np.array_equal(ud.cpu().numpy(), u_got)


@pytest.mark.parametrize("arith", ["reference", "fp64"])
def test_strict_layer_refreshes_g_and_coefficients(ss4d, cuda, arith):
    """SS4D_COMPAT_STRICT=1: the host copies of the edge detector's g faces
    and of the step's coefficients e..bw are those of the reference after
    _gf_inputImage_plus_thresholdedImage_ and after _segTimeStep_."""
    d = load_golden("seg_small.npz")
    params = dict(zip((str(n) for n in d["param_names"]), d["params"]))
    shape = d["u0"].shape
    lM, kM, jM, iM = shape
    n = int(np.prod(shape))
    os.environ["SS4D_ARITH"] = arith
    os.environ["SS4D_COMPAT_STRICT"] = "1"
    L = C.CDLL(ss4d.SEG_PATH, mode=os.RTLD_LOCAL)
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM),
                  ("maxNoGSIteration", params["maxNoGSIteration"]), ("maxNoOfTimeSteps", params["maxNoOfTimeSteps"])):
        C.c_int.in_dll(L, nm).value = int(v)
    for nm in ("K", "eps2", "tau", "h", "omega_c", "gsTol", "segTol", "sigma", "omega_sigma",
               "maxNoGSIteration_sigma", "theta_img", "rho_thr", "ballRadius"):
        C.c_double.in_dll(L, nm).value = float(params[nm])
    noc = (C.c_int * lM)()
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    for fn in ("_allocateMem_", "_deallocateMem_", "_segTimeStep_", "_gf_inputImage_plus_thresholdedImage_"):
        getattr(L, fn).restype = C.c_bool
    assert L._allocateMem_()
    try:
        def arr(name):
            addr = C.c_void_p.in_dll(L, name).value
            return np.ctypeslib.as_array((C.c_double * n).from_address(addr)).reshape(shape)

        i0, u, mm = arr("i0"), arr("u"), arr("Mmask")
        i0[...] = d["i0_in"]
        u[...] = d["thr_in"]
        mm[...] = 1.0
        assert L._gf_inputImage_plus_thresholdedImage_(C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
        for f, nm in enumerate(("g_e", "g_w", "g_n", "g_s", "g_t", "g_b", "g_fw", "g_bw")):
            assert np.array_equal(arr(nm), d[f"g{f}"]), nm
        u[...] = d["u0"]
        C.c_int.in_dll(L, "numberOfTimeStep").value = 1
        assert L._segTimeStep_()
        for f, nm in enumerate(("e", "w", "n", "s", "t", "b", "fw", "bw")):
            inner = (slice(1, -1),) * 4
            assert rel_err(arr(nm)[inner], d[f"coef{f}"][inner]) <= 4e-16, nm
        assert rel_err(u, d["u_steps"][0]) <= (1e-13 if arith == "reference" else 1e-10)
    finally:
        L._deallocateMem_()
        os.environ.pop("SS4D_ARITH", None)
        os.environ.pop("SS4D_COMPAT_STRICT", None)
