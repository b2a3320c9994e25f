"""The reference main's pipeline before the time steps (segmentation4D.c:
1383-1393) on the GPU: global maximum, per-ball minimum/maximum, local
thresholding and the initial segmentation function, bit-exact against the
reference's own outputs (tests/golden/seg_balls.npz, seg_init.npz), through
the native C ABI and through the reference-named layer."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def host(t):
    return t.detach().cpu().numpy()


def _balls(d):
    return [(int(b[0]), float(b[1]), float(b[2]), float(b[3])) for b in d["balls"]]


@pytest.mark.parametrize("fixture", ["seg_balls.npz", "seg_init.npz"])
def test_initial_segmentation_matches_reference(ss4d, cuda, fixture):
    torch = cuda
    d = load_golden(fixture)
    balls = _balls(d)
    if fixture == "seg_init.npz":
        alpha, beta, R = (float(v) for v in d["alpha_beta_R"])
        thr0, u0 = d["thr_before"], d["u_before"]
        thr_want = d["thr_after"]
    else:
        alpha, beta, R = 0.85, 0.15, 3.0
        thr0, u0 = np.zeros_like(d["i0_in"]), d["thr_smooth"]
        thr_want = d["thr_in"]
    shape = d["i0_in"].shape
    i0 = dev(torch, d["i0_in"])
    with ss4d.Solver(*shape[::-1], arith="fp64") as S:
        if fixture == "seg_init.npz":
            assert S.max4d(i0) == float(d["gmax"])
            for b, (l, x, y, z) in enumerate(balls):
                assert S.ball_min_max(i0, l, x, y, z, R) == (d["ball_min"][b], d["ball_max"][b])
        thr = dev(torch, thr0)
        S.local_threshold(alpha, beta, R, i0, thr, balls)
        u = dev(torch, u0)
        mm = torch.zeros_like(u)
        S.generate_segm_function(R, u, mm, balls)
        S.synchronize()
    assert np.array_equal(host(thr), thr_want)
    assert np.array_equal(host(u), d["u_gen"])
    assert np.array_equal(host(mm), d["mmask"])
    assert np.array_equal(host(i0), d["i0_in"])  # the input image is left alone


def test_ball_outside_the_array_is_refused(ss4d, cuda):
    torch = cuda
    d = load_golden("seg_init.npz")
    i0 = dev(torch, d["i0_in"])
    with ss4d.Solver(*d["i0_in"].shape[::-1]) as S:
        with pytest.raises(ss4d.SS4DError) as ei:
            S.local_threshold(0.7, 0.3, 13.0, i0, torch.zeros_like(i0), [(1, 3.0, 17.0, 16.0)])
        assert ei.value.status == 1  # SS4D_ERR_INVALID
        with pytest.raises(ss4d.SS4DError):
            S.ball_min_max(i0, 1, 3.0, 17.0, 16.0, 13.0)


def test_reference_named_layer_runs_the_initial_segmentation(ss4d, cuda):
    """A reference-style driver: globals, _allocateMem_, centres, then
    _get4DMax_, _get3DMin/MaxWithinR_, _locallyThreshold4Ddata_ and
    _generate4DsegmFunct_ on host arrays."""
    d = load_golden("seg_init.npz")
    alpha, beta, R = (float(v) for v in d["alpha_beta_R"])
    balls = _balls(d)
    shape = d["i0_in"].shape
    lM, kM, jM, iM = shape
    L = C.CDLL(ss4d.SEG_PATH, mode=os.RTLD_LOCAL)
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM)):
        C.c_int.in_dll(L, nm).value = v
    for nm, v in (("alpha", alpha), ("beta", beta), ("ballRadius", R)):
        C.c_double.in_dll(L, nm).value = v
    noc = (C.c_int * lM)()
    for l, *_ in balls:
        noc[l] += 1
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    for fn in ("_allocateMem_", "_deallocateMem_", "_locallyThreshold4Ddata_", "_generate4DsegmFunct_"):
        getattr(L, fn).restype = C.c_bool
    for fn in ("_get4DMax_", "_get3DMinWithinR_", "_get3DMaxWithinR_"):
        getattr(L, fn).restype = C.c_double
    L._get3DMinWithinR_.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 4
    L._get3DMaxWithinR_.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 4
    assert L._allocateMem_()
    try:
        pp = C.POINTER(C.POINTER(C.c_double))
        cx, cy, cz = (pp.in_dll(L, n) for n in ("center_x", "center_y", "center_z"))
        seen = [0] * lM
        for l, x, y, z in balls:
            c = seen[l]
            cx[l][c], cy[l][c], cz[l][c] = x, y, z
            seen[l] += 1
        n = int(np.prod(shape))

        def arr(name):
            addr = C.c_void_p.in_dll(L, name).value
            return np.ctypeslib.as_array((C.c_double * n).from_address(addr)).reshape(shape)

        i0, u, mm = arr("i0"), arr("u"), arr("Mmask")
        i0[...] = d["i0_in"]
        assert L._get4DMax_(C.c_void_p(i0.ctypes.data)) == float(d["gmax"])
        for b, (l, x, y, z) in enumerate(balls):
            assert L._get3DMinWithinR_(C.c_void_p(i0.ctypes.data), l, x, y, z, R) == d["ball_min"][b]
            assert L._get3DMaxWithinR_(C.c_void_p(i0.ctypes.data), l, x, y, z, R) == d["ball_max"][b]
        u[...] = d["thr_before"]
        assert L._locallyThreshold4Ddata_(C.c_void_p(i0.ctypes.data), C.c_void_p(u.ctypes.data))
        assert np.array_equal(u, d["thr_after"])
        u[...] = d["u_before"]
        mm[...] = 0.0
        assert L._generate4DsegmFunct_(C.c_void_p(u.ctypes.data))
        assert np.array_equal(u, d["u_gen"])
        assert np.array_equal(mm, d["mmask"])
    finally:
        L._deallocateMem_()
