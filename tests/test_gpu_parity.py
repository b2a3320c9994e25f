"""CUDA path vs the reference (golden fixtures) and the oracle, through the C ABI.

Bars: the plain FP64 forms match the reference's red-black SOR
to <= 1e-10 relative in u per time step with the same iteration counts, and
masks are bit-exact.  The reference-order kernels (SS4D_ARITH_REFERENCE) are
held to 1e-13 (they differ from the reference only where it calls pow()).
The mixed form must reach the same FP64 residual tolerance every step.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import load_golden, params_from_golden, rel_err

pytestmark = pytest.mark.gpu

TOL = {"reference": 1e-13, "fp64": 1e-10}


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def host(t):
    return t.detach().cpu().numpy()


def zeros8(torch, shape):
    return [torch.zeros(shape, dtype=torch.float64, device="cuda") for _ in range(8)]


@pytest.mark.parametrize("fixture", ["seg_small.npz", "seg_balls.npz"])
def test_edge_detector_matches_reference(ss4d, cuda, fixture):
    torch = cuda
    d = load_golden(fixture)
    p = params_from_golden(ss4d, d)
    shape = d["i0_in"].shape
    i0 = dev(torch, d["i0_in"])
    thr = dev(torch, d["thr_in"])
    g = zeros8(torch, shape)
    with ss4d.Solver(*shape[::-1], arith="reference") as S:
        S.edge_detector(p, i0, thr, g)
        S.synchronize()
    assert np.array_equal(host(i0), d["i0_smooth"])
    assert np.array_equal(host(thr), d["thr_smooth"])
    for f in range(8):
        assert np.array_equal(host(g[f]), d[f"g{f}"]), f"g face {f}"


def test_coefficients_match_reference(ss4d, cuda):
    torch = cuda
    d = load_golden("seg_small.npz")
    p = params_from_golden(ss4d, d)
    shape = d["u0"].shape
    u = dev(torch, d["u0"])
    g = [dev(torch, d[f"g{f}"]) for f in range(8)]
    coef = zeros8(torch, shape)
    with ss4d.Solver(*shape[::-1], arith="reference") as S:
        S.gs_coefficients(p, u, g, coef)
        S.synchronize()
    for f in range(8):
        assert rel_err(host(coef[f]), d[f"coef{f}"]) <= 4e-16, f"coefficient {f}"


@pytest.mark.parametrize("arith", ["reference", "fp64"])
@pytest.mark.parametrize("graph", [True, False])
def test_seg_time_steps_match_reference(ss4d, cuda, arith, graph):
    if arith == "reference" and not graph:
        pytest.skip("the reference form has no graph")
    torch = cuda
    d = load_golden("seg_small.npz")
    p = params_from_golden(ss4d, d)
    shape = d["u0"].shape
    u = dev(torch, d["u0"])
    prev = torch.zeros_like(u)
    mm = torch.ones_like(u)
    g = [dev(torch, d[f"g{f}"]) for f in range(8)]
    with ss4d.Solver(*shape[::-1], arith=arith) as S:
        S.set_graph(graph)
        for step in range(5):
            st = S.seg_time_step(p, u, prev, g, mmask=mm)
            assert st["iterations"] == d["its"][step], f"step {step + 1}"
            assert rel_err(st["residual"], d["res"][step]) < 1e-5  # printed with 7 digits
            assert rel_err(host(u), d["u_steps"][step]) <= TOL[arith], f"u after step {step + 1}"
            assert abs(S.l2norm(p.h, prev, u) - d["l2"][step]) <= 1e-10 * d["l2"][step]


@pytest.mark.parametrize("arith", ["reference", "fp64", "mixed"])
def test_seg_balls_rescale_path(ss4d, cuda, arith):
    torch = cuda
    d = load_golden("seg_balls.npz")
    p = params_from_golden(ss4d, d)
    balls = [(int(b[0]), b[1], b[2], b[3]) for b in d["balls"]]
    shape = d["u0"].shape
    g = [dev(torch, d[f"g{f}"]) for f in range(8)]
    mm = dev(torch, d["mmask"])
    u = dev(torch, d["u_gen"])
    prev = torch.zeros_like(u)
    with ss4d.Solver(*shape[::-1], arith=arith) as S:
        S.rescale_to_zero_one(p, u, mm, balls)
        S.synchronize()
        assert rel_err(host(u), d["u0"]) <= 1e-15
        for step in range(3):
            st = S.seg_time_step(p, u, prev, g, mmask=mm, balls=balls)
            if arith == "mixed":
                # five iterations are the cap here: both stop at the cap, before
                # the tolerance, so the mixed iterate differs from the reference's
                # by what five sweeps on its own inner operator make of it (its
                # FP32 sweeps' coefficients are 16-bit fractions of the row sum)
                assert st["iterations"] <= p.maxNoGSIteration
                assert rel_err(host(u), d["u_steps"][step]) <= 1e-4
            else:
                assert st["iterations"] == d["its"][step]
                assert rel_err(host(u), d["u_steps"][step]) <= TOL[arith]


def test_rescale_rejects_ball_outside_array(ss4d, cuda):
    torch = cuda
    p = ss4d.scene_params(ballRadius=3.0)
    u = torch.zeros((5, 8, 8, 8), dtype=torch.float64, device="cuda")
    with ss4d.Solver(8, 8, 8, 5) as S:
        with pytest.raises(ss4d.SS4DError) as ei:
            S.rescale_to_zero_one(p, u, None, [(1, 1.0, 4.0, 4.0)])
        assert ei.value.status == 1


@pytest.mark.parametrize("arith", ["reference", "fp64"])
def test_mcf_known_answer(ss4d, cuda, arith):
    torch = cuda
    d = load_golden("mcf_small.npz")
    for n, steps, key in ((8, 3, "err8"), (16, 4, "err16")):
        p = ss4d.mcf_params(n, steps)
        shape = (n + 2,) * 4
        u = torch.zeros(shape, dtype=torch.float64, device="cuda")
        ex = torch.zeros_like(u)
        prev = torch.zeros_like(u)
        with ss4d.Solver(*shape, arith=arith) as S:
            S.mcf_exact_solution(p.h, 0.0, u)
            for step in range(1, steps + 1):
                S.mcf_time_step(p, step, u, prev)
                S.mcf_exact_solution(p.h, step * p.tau, ex)
                err = S.l2norm(p.h, ex, u)
                assert abs(err - d[key][step - 1]) <= 1e-10 * d[key][step - 1]
                if n == 8:
                    assert rel_err(host(u), d["u8"][step - 1]) <= TOL[arith]


def test_mcf_boundary_matches_oracle(ss4d, oracle, cuda):
    torch = cuda
    shape = (6, 5, 7, 8)  # lMax, kMax, jMax, iMax: unequal extents
    h, t = 0.3125, 0.77
    u0 = np.random.default_rng(0).standard_normal(shape)
    want = u0.copy()
    oracle.mcf_boundary(h, t, want)
    u = dev(torch, u0)
    with ss4d.Solver(*shape[::-1]) as S:
        S.mcf_set_boundary_exact(h, t, u)
        S.synchronize()
    assert np.array_equal(host(u), want)


@pytest.mark.parametrize("arith", ["reference", "fp64"])
def test_32x32x32x8_twenty_steps_match_reference(ss4d, oracle, cuda, arith):
    """32^3 x 8, 20 steps: iteration counts, step differences, probes and
    both masks against the reference's run."""
    torch = cuda
    d = load_golden("seg_32x32x32x8.npz")
    nx, ny, nz, nt = (int(v) for v in d["dims"])
    p = ss4d.scene_params(maxNoOfTimeSteps=20)
    i0h, u0h = ss4d.scene(1, nx, ny, nz, nt, seed=int(d["seed"]))
    shape = i0h.shape
    i0 = dev(torch, i0h)
    thr = torch.zeros_like(i0)
    g = zeros8(torch, shape)
    u = dev(torch, u0h)
    prev = torch.zeros_like(u)
    mm = torch.ones_like(u)
    nint = nx * ny * nz * nt
    m05 = torch.zeros(nint, dtype=torch.uint8, device="cuda")
    mn = torch.zeros_like(m05)
    with ss4d.Solver(*shape[::-1], arith=arith) as S:
        S.edge_detector(p, i0, thr, g)
        for step in range(20):
            st = S.seg_time_step(p, u, prev, g, mmask=mm)
            assert st["iterations"] == d["its"][step], f"step {step + 1}"
            assert abs(S.l2norm(p.h, prev, u) - d["l2"][step]) <= 1e-10 * d["l2"][step]
            got = host(u).reshape(-1)[d["probes"]]
            assert rel_err(got, d["probe_vals"][step]) <= TOL[arith]
        S.threshold_mask(u, m05, 0.5, False)
        S.threshold_mask(u, mn, 0.5, True)
        S.synchronize()
    assert np.array_equal(np.packbits(host(m05)), d["mask05"])
    assert np.array_equal(np.packbits(host(mn)), d["masknorm"])


def test_sor_solve_with_injected_coefficients(ss4d, cuda):
    """The SOR loop alone on the reference's own step-1 coefficients."""
    torch = cuda
    d = load_golden("seg_small.npz")
    p = params_from_golden(ss4d, d)
    coef = [dev(torch, d[f"coef{f}"]) for f in range(8)]
    for arith, tol in (("reference", 1e-13), ("fp64", 1e-10)):
        u = dev(torch, d["u0"])
        prev = dev(torch, d["prev1"])
        with ss4d.Solver(*d["u0"].shape[::-1], arith=arith) as S:
            st = S.sor_solve(p, u, prev, coef)
        assert st["iterations"] == d["its"][0]
        assert rel_err(host(u), d["u_steps"][0]) <= tol


@pytest.mark.parametrize("dims", [(9, 7, 5, 3), (1, 1, 1, 1), (33, 6, 4, 2), (2, 3, 2, 5)])
@pytest.mark.parametrize("arith", ["reference", "fp64", "mixed"])
def test_ragged_and_minimal_sizes_match_oracle(ss4d, oracle, cuda, dims, arith):
    torch = cuda
    nx, ny, nz, nt = dims
    p = ss4d.scene_params(gsTol=1e-14)
    i0h, u0h = ss4d.scene(1, nx, ny, nz, nt, seed=9)
    g = oracle.gfaces(p, i0h, np.zeros_like(i0h))
    want = u0h.copy()
    oprev = np.zeros_like(want)
    zs = []
    for _ in range(2):
        z, _ = oracle.seg_time_step(p, want, oprev, g, mmask=np.ones_like(want))
        zs.append(z)
    u = dev(torch, u0h)
    prev = torch.zeros_like(u)
    gd = [dev(torch, a) for a in g]
    with ss4d.Solver(*u0h.shape[::-1], arith=arith) as S:
        for step in range(2):
            st = S.seg_time_step(p, u, prev, gd)
            if arith != "mixed":
                assert st["iterations"] == zs[step]
            else:
                assert st["residual"] <= p.gsTol
    tol = {"reference": 1e-13, "fp64": 1e-10, "mixed": 1e-6}[arith]
    assert rel_err(host(u), want) <= tol


def test_nonfinite_input_is_reported(ss4d, cuda):
    torch = cuda
    p = ss4d.scene_params()
    i0h, u0h = ss4d.scene(1, 8, 8, 8, 3, seed=2)
    u0h[2, 4, 4, 4] = np.nan
    u = dev(torch, u0h)
    g = [torch.ones_like(u) for _ in range(8)]
    for arith in ("reference", "fp64", "mixed"):
        with ss4d.Solver(*u0h.shape[::-1], arith=arith) as S:
            with pytest.raises(ss4d.SS4DError) as ei:
                S.seg_time_step(p, u.clone(), None, g)
            assert ei.value.status == 4  # SS4D_ERR_NONFINITE


def test_side_copy_lands_before_the_calls_after_the_join(ss4d, cuda):
    """A mask uploaded on the side stream, joined before the rescale, gives the
    rescale of a mask uploaded in order (the overlap the reference-named time
    step uses)."""
    torch = cuda
    rng = np.random.default_rng(9)
    shape = (3, 10, 9, 12)
    img = rng.random(shape)
    mask = (rng.random(shape) > 0.3).astype(np.float64)
    p = ss4d.scene_params()
    with ss4d.Solver(*shape[::-1]) as S:
        want = dev(torch, img)
        S.rescale_to_zero_one(p, want, dev(torch, mask), None)
        got = dev(torch, img)
        d_mask = torch.zeros(shape, dtype=torch.float64, device="cuda")
        keep = S.copy_to_device_side(d_mask, mask)
        S.join_side()
        S.rescale_to_zero_one(p, got, d_mask, None)
        S.synchronize()
        del keep
    assert np.array_equal(host(got), host(want))
    assert np.array_equal(host(d_mask), mask)


def test_norms_match_oracle(ss4d, oracle, cuda):
    torch = cuda
    rng = np.random.default_rng(5)
    a = rng.standard_normal((5, 6, 7, 9))
    b = rng.standard_normal((5, 6, 7, 9))
    with ss4d.Solver(9, 7, 6, 5) as S:
        l2 = S.l2norm(0.5, dev(torch, a), dev(torch, b))
        m = S.mass(0.5, dev(torch, a))
    assert abs(l2 - oracle.l2norm(0.5, a, b)) <= 1e-13 * abs(l2)
    assert abs(m - oracle.mass(0.5, a)) <= 1e-12 * max(1.0, abs(m))


@pytest.mark.parametrize("arith", ["fp64", "mixed"])
def test_sweeps_do_not_depend_on_block_order(ss4d, oracle, cuda, arith):
    """Red-black colour independence: each half-sweep reads only the other
    colour, so the tile order and grid size (k-block depth, persistent grid)
    must not change u.  The residual's per-block partial sums are grouped
    differently, so the iteration counts are compared, and u bit for bit."""
    torch = cuda
    dims = nx, ny, nz, nt = (37, 21, 13, 5)
    p = ss4d.scene_params(gsTol=1e-10)
    i0h, u0h = ss4d.scene(3, nx, ny, nz, nt, seed=81)
    g = [dev(torch, a) for a in oracle.gfaces(p, i0h, np.zeros_like(i0h))]
    runs = []
    for k_block, max_grid in ((4, 0), (1, 7), (8, 300), (2, 1)):
        u = dev(torch, u0h)
        with ss4d.Solver.for_interior(*dims, arith=arith) as S:
            S.set_tiling(k_block, max_grid)
            its = [S.seg_time_step(p, u, None, g)["iterations"] for _ in range(2)]
        runs.append((its, host(u)))
    for its, u in runs[1:]:
        assert its == runs[0][0]
        assert np.array_equal(u, runs[0][1])


@pytest.mark.parametrize("steps", [0, 1, 3])
def test_explicit_presmoothing_matches_reference(ss4d, cuda, steps):
    """_presmoothStepEXP_ on a ragged volume with random ghosts: u and prev_u
    bit-exact with the reference, through the native ABI."""
    torch = cuda
    d = load_golden("presmooth_exp.npz")
    sigma, h = (float(v) for v in d["sigma_h"])
    p = ss4d.scene_params(sigma=sigma, h=h)
    shape = d["v_in"].shape
    with ss4d.Solver(*shape[::-1]) as S:
        v = dev(torch, d["v_in"])
        prev = torch.zeros_like(v)
        S.presmooth_explicit(p, steps, v, prev)
        S.synchronize()
    assert np.array_equal(host(v), d[f"u_{steps}"])
    assert np.array_equal(host(prev), d[f"prev_{steps}"])


def test_explicit_presmoothing_through_reference_named_layer(ss4d, cuda):
    """_presmoothStepEXP_(u) of libss4d_seg.so on its host arrays, driven
    through the reference's globals (timeStepsNum, sigma, h)."""
    d = load_golden("presmooth_exp.npz")
    sigma, h = (float(v) for v in d["sigma_h"])
    shape = d["v_in"].shape
    lM, kM, jM, iM = shape
    L = C.CDLL(ss4d.SEG_PATH, mode=os.RTLD_LOCAL)
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM), ("timeStepsNum", 3)):
        C.c_int.in_dll(L, nm).value = v
    for nm, v in (("sigma", sigma), ("h", h)):
        C.c_double.in_dll(L, nm).value = v
    noc = (C.c_int * lM)()
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    L._allocateMem_.restype = C.c_bool
    L._presmoothStepEXP_.restype = None
    assert L._allocateMem_()
    try:
        n = int(np.prod(shape))

        def arr(name):
            addr = C.c_void_p.in_dll(L, name).value
            return np.ctypeslib.as_array((C.c_double * n).from_address(addr)).reshape(shape)

        u, prev = arr("u"), arr("prev_u")
        u[...] = d["v_in"]
        L._presmoothStepEXP_(C.c_void_p(u.ctypes.data))
        assert np.array_equal(u, d["u_3"])
        assert np.array_equal(prev, d["prev_3"])
    finally:
        L._deallocateMem_()


@pytest.mark.parametrize("arith", ["reference", "fp64"])
def test_stop_test_at_the_tolerance_is_reported(ss4d, cuda, arith):
    """A stop test whose residual lies within the summation-order band of
    gsTol sets near_tolerance (the reference's serial sum could have decided
    it the other way); one 0.1 % away does not.  The solve is repeated with
    gsTol set to the residual it ended on, which the same device reproduces
    exactly."""
    torch = cuda
    d = load_golden("seg_small.npz")
    p = params_from_golden(ss4d, d)
    g = [dev(torch, d[f"g{f}"]) for f in range(8)]
    shape = d["u0"].shape
    with ss4d.Solver(*shape[::-1], arith=arith) as S:
        u = dev(torch, d["u0"])
        st = S.seg_time_step(p, u, None, g)
        assert st["near_tolerance"] == 0
        z, R = st["iterations"], st["residual"]
        for tol, near in ((R, 1), (R * 1.001, 0)):
            q = params_from_golden(ss4d, d)
            q.gsTol = tol
            u = dev(torch, d["u0"])
            st = S.seg_time_step(q, u, None, g)
            assert st["iterations"] == z
            assert st["residual"] == R
            assert st["near_tolerance"] == near


def test_allocation_failure_is_reported_and_the_context_survives(ss4d, cuda):
    """An allocation the device or host cannot serve returns SS4D_ERR_ALLOC
    (the reference's _allocateMem_ returns false) and leaves the context
    usable for the next solve."""
    import ctypes as C

    torch = cuda
    L = ss4d.lib()
    ptr = C.c_void_p()
    assert L.ss4d_dev_alloc(1 << 60, C.byref(ptr)) == 2  # SS4D_ERR_ALLOC
    assert L.ss4d_host_alloc(1 << 60, C.byref(ptr)) == 2
    assert b"failed" in L.ss4d_last_error()
    d = load_golden("seg_small.npz")
    p = params_from_golden(ss4d, d)
    g = [dev(torch, d[f"g{f}"]) for f in range(8)]
    with ss4d.Solver(*d["u0"].shape[::-1], arith="fp64") as S:
        u = dev(torch, d["u0"])
        st = S.seg_time_step(p, u, None, g)
    assert st["iterations"] == d["its"][0]


@pytest.mark.parametrize("fixture", ["seg_small.npz", "seg_balls.npz"])
def test_mixed_edge_detector_is_close_to_reference(ss4d, cuda, fixture):
    """The mixed form runs the edge detector in float-float arithmetic
    (about 48 significant bits on the FP32 pipe): the smoothed images within
    1e-13 and the g faces within 1e-12 of the reference's FP64 values, the
    same presmoothing iteration counts, and the reference's prev_u copy."""
    torch = cuda
    d = load_golden(fixture)
    p = params_from_golden(ss4d, d)
    shape = d["i0_in"].shape
    i0 = dev(torch, d["i0_in"])
    thr = dev(torch, d["thr_in"])
    g = zeros8(torch, shape)
    with ss4d.Solver(*shape[::-1], arith="mixed") as S:
        S.edge_detector(p, i0, thr, g)
        one = dev(torch, d["i0_in"])
        prev = torch.zeros_like(one)
        st = S.presmooth_step(p, one, prev)
        S.synchronize()
    assert rel_err(host(i0), d["i0_smooth"]) <= 1e-13
    assert rel_err(host(thr), d["thr_smooth"]) <= 1e-13
    for f in range(8):
        assert rel_err(host(g[f]), d[f"g{f}"]) <= 1e-12, f"g face {f}"
    if "presmooth_its" in d:  # the fixtures that recorded the reference's counts
        assert st["iterations"] == d["presmooth_its"][0]
    assert np.array_equal(host(prev), d["i0_in"])
    assert rel_err(host(one), d["i0_smooth"]) <= 1e-13


@pytest.mark.parametrize("sigma", [(1.0, 0.7, 1.3, 0.0), (0.4, 0.0, 2.5, 1.0)])
def test_gaussian_smooth_and_gfaces_match_oracle(ss4d, oracle, cuda, sigma):
    """The separable Gaussian bit for bit against the oracle (two and three
    axes: the result ends in the scratch and is copied back), and the g faces
    of the smoothed images: bit-exact in the FP64 form, within 1e-12 in the
    mixed form's float-float arithmetic."""
    torch = cuda
    rng = np.random.default_rng(4)
    shape = (6, 9, 10, 12)
    a = rng.random(shape)
    b = rng.random(shape)
    p = ss4d.scene_params(theta_img=0.5, rho_thr=0.5, h=0.5)
    wa, wb = a.copy(), b.copy()
    assert oracle.gaussian(sigma, wa) == 0 and oracle.gaussian(sigma, wb) == 0
    g_want = oracle.gfaces(p, wa, wb)
    for arith, tol in (("fp64", 0.0), ("mixed", 1e-12)):
        with ss4d.Solver(*shape[::-1], arith=arith) as S:
            da, db = dev(torch, a), dev(torch, b)
            S.gaussian_smooth(sigma, da)
            S.gaussian_smooth(sigma, db)
            g = zeros8(torch, shape)
            S.gfaces(p, da, db, g)
            S.synchronize()
        assert np.array_equal(host(da), wa) and np.array_equal(host(db), wb)
        inner = (slice(1, -1),) * 4
        for f in range(8):
            assert rel_err(host(g[f])[inner], g_want[f][inner]) <= tol, (arith, f)


def test_gaussian_smooth_refuses_wide_taps(ss4d, cuda):
    torch = cuda
    with ss4d.Solver(8, 8, 8, 5) as S:
        with pytest.raises(ss4d.SS4DError) as ei:
            S.gaussian_smooth((11.0, 0.0, 0.0, 0.0), torch.zeros((5, 8, 8, 8), dtype=torch.float64, device="cuda"))
        assert ei.value.status == 1


def test_gaussian_smooth_with_taps_wider_than_the_volume(ss4d, oracle, cuda):
    """A radius of 3 taps on extents of 1, 2 and 3 voxels: the mirrored
    coordinates fold more than once, bit for bit as the oracle folds them."""
    torch = cuda
    rng = np.random.default_rng(6)
    shape = (5, 3, 4, 3)  # interior t 3, z 1, y 2, x 1
    a = rng.random(shape)
    sigma = (1.0, 1.0, 1.0, 1.0)
    want = a.copy()
    assert oracle.gaussian(sigma, want) == 0
    with ss4d.Solver(*shape[::-1]) as S:
        da = dev(torch, a)
        S.gaussian_smooth(sigma, da)
        S.synchronize()
    assert np.array_equal(host(da), want)


def _pinned(ss4d, shape):
    """a page-locked host array (ss4d_host_alloc) and its release"""
    import ctypes as Cm

    L = ss4d.lib()
    n = int(np.prod(shape))
    ptr = Cm.c_void_p()
    assert L.ss4d_host_alloc(8 * n, Cm.byref(ptr)) == 0
    a = np.ctypeslib.as_array((Cm.c_double * n).from_address(ptr.value)).reshape(shape)
    return a, (lambda: L.ss4d_host_free(ptr))


@pytest.mark.parametrize("form", ["fp64", "mixed", "extrap", "tight", "proj", "capped"])
@pytest.mark.parametrize("nt", [1, 3, 6])
def test_host_array_step_equals_device_step(ss4d, oracle, cuda, form, nt):
    """ss4d_seg_time_step_host (u up and down in frame chunks overlapped with
    the step's first and last kernels, Mmask beside the solve, prev_u copied
    on the host; in the mixed form u formed from a round goes down while that
    round's refinement pass decides) gives, step after step, the u of
    ss4d_seg_time_step on device arrays with the same Mmask and balls, and
    prev_u = the step's input.  "tight": the mixed form with extrapolation at
    gsTol 1e-13, where rounds fall short of the tolerance and the loop goes
    on after the download that a refinement pass rejected; "proj": with the
    projected start (the third step); "capped": gsTol 1e-13 with at most 3
    iterations, so every step ends at the cap inside a round."""
    torch = cuda
    nx, ny, nz = 20, 18, 14
    tight = form in ("tight", "capped")
    p = ss4d.scene_params(ballRadius=3.0, gsTol=1e-13 if tight else 1e-6,
                          **({"maxNoGSIteration": 3} if form == "capped" else {}))
    i0h, u0h = ss4d.scene(1, nx, ny, nz, nt, seed=8)
    shape = i0h.shape
    g = [dev(torch, a) for a in oracle.gfaces(p, i0h, np.zeros_like(i0h))]
    rng = np.random.default_rng(2)
    mask = (rng.random(shape) > 0.1).astype(np.float64)
    balls = [(l, 10.0, 9.0, 7.0) for l in range(1, nt + 1)] + [(l, 6.0, 12.0, 8.0) for l in range(1, nt + 1, 2)]
    balls.sort(key=lambda b: b[0])
    arith = "fp64" if form == "fp64" else "mixed"
    hu, free_u = _pinned(ss4d, shape)
    hp, free_p = _pinned(ss4d, shape)
    hm, free_m = _pinned(ss4d, shape)
    try:
        hu[...] = u0h
        hm[...] = mask
        du, dm = torch.zeros_like(g[0]), torch.zeros_like(g[0])
        ref_u, ref_m = dev(torch, u0h), dev(torch, mask)
        with ss4d.Solver(*shape[::-1], arith=arith) as A, ss4d.Solver(*shape[::-1], arith=arith) as B:
            for S in (A, B):
                S.set_extrapolation(3 if form in ("extrap", "tight", "proj", "capped") else 0)
                S.set_projection(form == "proj")
            rounds = []
            for _ in range(3):
                before = hu.copy()
                sa = A.seg_time_step_host(p, hu, du, g, h_prev=hp, h_mmask=hm, d_mmask=dm, balls=balls)
                sb = B.seg_time_step(p, ref_u, None, g, ref_m, balls)
                B.synchronize()
                assert sa["iterations"] == sb["iterations"] and sa["status"] == 0
                assert sa["refinements"] == sb["refinements"]
                assert np.array_equal(hu, host(ref_u))
                assert np.array_equal(hp, before)
                assert sa["projected"] == sb["projected"]
                if form == "capped":
                    assert sa["iterations"] == p.maxNoGSIteration
                rounds.append(sa["refinements"])
            if form == "tight":  # some step needed more than one round
                assert max(rounds) > 2, rounds
    finally:
        free_u(), free_p(), free_m()
