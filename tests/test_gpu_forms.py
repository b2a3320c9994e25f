"""Error of the mixed-precision forms against the plain FP64 form (which
itself matches the reference to 1e-10 per step) on the plain-vs-mixed
workloads: 32^3 x 8 for 20 steps (the CPU-runnable configuration) and
128^3 x 16 for 50 steps (two erased sectors, noise 25).  Every step of every
form meets the FP64 residual tolerance; the masks (level (min+max)/2 of the
FP64 state) agree with Dice >= 0.999."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dice(a, b):
    return 2.0 * float((a & b).sum()) / max(1.0, float(a.sum() + b.sum()))


@pytest.mark.parametrize("kind,dims,steps", [(1, (32, 32, 32, 8), 20), (2, (128, 128, 128, 16), 50)])
def test_mixed_forms_against_fp64(ss4d, cuda, kind, dims, steps):
    torch = cuda
    nx, ny, nz, nt = dims
    p = ss4d.scene_params(maxNoOfTimeSteps=steps)
    i0h, u0h = ss4d.scene(kind, nx, ny, nz, nt, seed=7, threads=0)
    shape = i0h.shape
    i0 = torch.from_numpy(i0h).cuda()
    g = [torch.empty_like(i0) for _ in range(8)]
    finals, its = {}, {}
    with ss4d.Solver(*shape[::-1], arith="fp64") as S:
        S.edge_detector(p, i0, None, g)
        for form in ("fp64", "mixed", "extrap", "proj"):
            S.set_arith("fp64" if form == "fp64" else "mixed")
            S.set_extrapolation(3 if form in ("extrap", "proj") else 0)
            S.set_projection(form == "proj")
            u = torch.from_numpy(u0h).cuda()
            st = [S.seg_time_step(p, u, None, g) for _ in range(steps)]
            assert all(s["status"] == 0 and s["residual"] <= p.gsTol for s in st), form
            finals[form] = u[1:-1, 1:-1, 1:-1, 1:-1].cpu().numpy()
            its[form] = sum(s["iterations"] for s in st)
            # the projected start from the third step on (two earlier changes)
            assert [s["projected"] for s in st[:2]] == [0, 0]
            assert all(s["projected"] == (form == "proj") for s in st[2:]), form
    ref = finals["fp64"]
    lev = 0.5 * (ref.min() + ref.max())
    for form in ("mixed", "extrap", "proj"):
        d = finals[form] - ref
        max_rel = float(np.abs(d).max() / np.abs(ref).max())
        rel_l2 = float(np.linalg.norm(d) / np.linalg.norm(ref))
        dice = _dice(finals[form] >= lev, ref >= lev)
        print(f"config kind {kind} {dims} x {steps} steps, {form}: max rel {max_rel:.2e}, rel L2 {rel_l2:.2e}, "
              f"Dice {dice:.6f}, SOR iterations {its[form]} (fp64 {its['fp64']})")
        # both states meet the same residual tolerance every step; their
        # distance is that of two such iterates (no parity bar), the masks agree
        assert max_rel <= 2e-3 and dice >= 0.999
    assert its["proj"] < its["extrap"] < its["mixed"]


@pytest.mark.parametrize("arith", ["fp64", "mixed"])
def test_true_fp64_residual_meets_the_tolerance(ss4d, oracle, cuda, arith):
    """The mixed form assembles its coefficients in float-float arithmetic
    (48-bit significands) and measures its FP64 residual against them.  The
    residual of its result against the oracle's FP64 coefficients (the
    reference's arithmetic) must meet the same tight tolerance: coefficient
    errors of FP32 size (1e-7) would leave it near 1e-12 here."""
    torch = cuda
    dims = nx, ny, nz, nt = (24, 20, 12, 5)
    p = ss4d.scene_params(gsTol=1e-14)
    i0h, u0h = ss4d.scene(3, nx, ny, nz, nt, seed=61)
    g = oracle.gfaces(p, i0h, np.zeros_like(i0h))
    u = torch.from_numpy(u0h).cuda()
    with ss4d.Solver.for_interior(*dims, arith=arith) as S:
        st = S.seg_time_step(p, u, None, [torch.from_numpy(a).cuda() for a in g])
    assert st["residual"] <= p.gsTol
    u1 = u.cpu().numpy()
    coef = oracle.coefficients(p, u0h, g)
    c = p.tau / (p.h * p.h)
    inner = (slice(1, -1),) * 4
    offs = [(0, 0, 0, 1), (0, 0, 0, -1), (0, 0, 1, 0), (0, 0, -1, 0), (0, 1, 0, 0), (0, -1, 0, 0), (1, 0, 0, 0),
            (-1, 0, 0, 0)]
    r = u1[inner] - u0h[inner]
    for f, o in enumerate(offs):
        nb = tuple(slice(1 + d, u1.shape[a] - 1 + d) for a, d in enumerate(o))
        r += c * coef[f][inner] * (u1[inner] - u1[nb])
    R = float(np.sum(r * r) * p.h ** 4)
    assert R <= p.gsTol * (1 + 1e-6), R


def test_inner_omega_changes_only_the_iteration_count(ss4d, oracle, cuda):
    """The mixed form's FP32 sweeps relaxed by another factor than omega_c:
    the same FP64 tolerance every step, the same states to within it; for this
    operator (c = tau/h^2 = 0.5) 1.2 needs far fewer sweeps than 1.8."""
    torch = cuda
    dims = nx, ny, nz, nt = (40, 36, 24, 6)
    p = ss4d.scene_params(gsTol=1e-10)
    i0h, u0h = ss4d.scene(3, nx, ny, nz, nt, seed=71)
    g = [torch.from_numpy(a).cuda() for a in oracle.gfaces(p, i0h, np.zeros_like(i0h))]
    out = {}
    for w in (0.0, 1.2):
        u = torch.from_numpy(u0h).cuda()
        with ss4d.Solver.for_interior(*dims, arith="mixed") as S:
            S.set_inner_omega(w)
            st = [S.seg_time_step(p, u, None, g) for _ in range(4)]
        assert all(s["status"] == 0 and s["residual"] <= p.gsTol for s in st)
        out[w] = (u.cpu().numpy(), sum(s["iterations"] for s in st))
    (a, za), (b, zb) = out[0.0], out[1.2]
    assert zb < za
    assert float(np.abs(a - b).max() / np.abs(a).max()) <= 1e-4
    with pytest.raises(ss4d.SS4DError):
        with ss4d.Solver.for_interior(*dims, arith="mixed") as S:
            S.set_inner_omega(2.5)



@pytest.mark.parametrize("host_arrays", [False, True])
def test_assembly_order_changes_no_bit(ss4d, cuda, host_arrays):
    """The mixed form's faces and coefficient kernels may visit the planes
    frame by frame or in blocks of k planes across the frames: every voxel's
    arithmetic is the same, so steps must agree bit for bit (with the
    extrapolated start and the first refinement pass formed by the assembly;
    on device arrays and through the host-array step, which assembles frame
    ranges as chunks arrive)."""
    from test_gpu_parity import _pinned

    torch = cuda
    nx, ny, nz, nt = 37, 21, 13, 7  # ragged against the 32 x 8 face tiles and every block depth below
    p = ss4d.scene_params()
    i0h, u0h = ss4d.scene(1, nx, ny, nz, nt, seed=61)
    shape = i0h.shape
    i0 = torch.from_numpy(i0h).cuda()
    g = [torch.zeros_like(i0) for _ in range(8)]
    with ss4d.Solver(*shape[::-1], arith="fp64") as S:
        S.edge_detector(p, i0, None, g)
    hu, free_u = _pinned(ss4d, shape)
    hp, free_p = _pinned(ss4d, shape)
    results = {}
    try:
        for order in (0, 1, 3, 5, 14, 100):
            with ss4d.Solver(*shape[::-1], arith="mixed") as S:  # a fresh extrapolation history each
                S.set_extrapolation(3)
                S.set_assembly_order(order)
                if host_arrays:
                    hu[...] = u0h
                    du = torch.zeros_like(i0)
                    its = [S.seg_time_step_host(p, hu, du, g, h_prev=hp)["iterations"] for _ in range(4)]
                    results[order] = (hu.copy(), its)
                else:
                    u = torch.from_numpy(u0h).cuda()
                    its = [S.seg_time_step(p, u, None, g)["iterations"] for _ in range(4)]
                    results[order] = (u.cpu().numpy(), its)
    finally:
        free_u(), free_p()
    want_u, want_its = results[0]
    for order, (u, its) in results.items():
        assert its == want_its, (order, its, want_its)
        assert np.array_equal(u, want_u), order


def test_projected_start_same_on_host_arrays(ss4d, cuda):
    """The projected start (the first FP32 round from the least-residual
    combination of the earlier changes) through the host-array step equals the
    device-array step bit for bit, steps and iteration counts alike; a solver
    without extrapolation of order 3 ignores it."""
    from test_gpu_parity import _pinned

    torch = cuda
    nx, ny, nz, nt = 33, 26, 17, 9
    p = ss4d.scene_params()
    i0h, u0h = ss4d.scene(3, nx, ny, nz, nt, seed=83)
    shape = i0h.shape
    i0 = torch.from_numpy(i0h).cuda()
    g = [torch.zeros_like(i0) for _ in range(8)]
    with ss4d.Solver(*shape[::-1], arith="fp64") as S:
        S.edge_detector(p, i0, None, g)
    with ss4d.Solver(*shape[::-1], arith="mixed") as S:
        S.set_extrapolation(3)
        S.set_projection(True)
        u = torch.from_numpy(u0h).cuda()
        dev = [S.seg_time_step(p, u, None, g) for _ in range(6)]
        want = u.cpu().numpy()
    hu, free_u = _pinned(ss4d, shape)
    hp, free_p = _pinned(ss4d, shape)
    try:
        with ss4d.Solver(*shape[::-1], arith="mixed") as S:
            S.set_extrapolation(3)
            S.set_projection(True)
            hu[...] = u0h
            du = torch.zeros_like(i0)
            host = [S.seg_time_step_host(p, hu, du, g, h_prev=hp) for _ in range(6)]
            got = hu.copy()
    finally:
        free_u(), free_p()
    assert [s["projected"] for s in dev] == [0, 0, 1, 1, 1, 1]
    assert [(s["iterations"], s["projected"]) for s in host] == [(s["iterations"], s["projected"]) for s in dev]
    assert np.array_equal(got, want)
    with ss4d.Solver(*shape[::-1], arith="mixed") as S:
        S.set_extrapolation(2)
        S.set_projection(True)
        u = torch.from_numpy(u0h).cuda()
        assert not any(S.seg_time_step(p, u, None, g)["projected"] for _ in range(4))


@pytest.mark.parametrize("dims", [(1, 1, 1, 1), (2, 3, 2, 5), (9, 7, 5, 3), (33, 6, 4, 2), (17, 9, 5, 1)])
def test_projected_start_on_ragged_and_minimal_sizes_matches_oracle(ss4d, oracle, cuda, dims):
    """Six steps of the projected form (the projection from the third step on)
    on odd, one-voxel and one-frame shapes, where the earlier changes can be
    linearly dependent and the normal equations singular: every step meets the
    FP64 tolerance and u stays within the mixed form's bar of the oracle's
    FP64 steps, as the extrapolated form without the projection does."""
    from conftest import rel_err

    torch = cuda
    nx, ny, nz, nt = dims
    steps = 6
    p = ss4d.scene_params(gsTol=1e-14)
    i0h, u0h = ss4d.scene(1, nx, ny, nz, nt, seed=19)
    g = oracle.gfaces(p, i0h, np.zeros_like(i0h))
    want = u0h.copy()
    oprev = np.zeros_like(want)
    for _ in range(steps):
        oracle.seg_time_step(p, want, oprev, g, mmask=np.ones_like(want))
    gd = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in g]
    for proj in (False, True):
        u = torch.from_numpy(u0h.copy()).cuda()
        with ss4d.Solver(*u0h.shape[::-1], arith="mixed") as S:
            S.set_extrapolation(3)
            S.set_projection(proj)
            st = [S.seg_time_step(p, u, None, gd) for _ in range(steps)]
        assert all(s["status"] == 0 and s["residual"] <= p.gsTol for s in st), (proj, st)
        assert not any(s["projected"] for s in st[:2])
        if not proj:
            assert not any(s["projected"] for s in st)
        assert rel_err(u.cpu().numpy(), want) <= 1e-6, proj
