"""Batched volumes: one persistent launch per half-sweep over volumes of
different sizes and parameters must give every volume exactly what the
single-volume FP64 form gives it (same per-voxel arithmetic; only the
residual summation is organised differently)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _volumes(ss4d, oracle, sizes, seed=5):
    rng = np.random.default_rng(seed)
    vols = []
    for n, dims in enumerate(sizes):
        p = ss4d.scene_params(K=float(rng.uniform(500, 2000)), tau=float(rng.uniform(0.25, 1.0)))
        i0, u0 = ss4d.scene(1, *dims, seed=seed + n)
        g = oracle.gfaces(p, i0, np.zeros_like(i0))
        vols.append((p, u0, g))
    return vols


@pytest.mark.parametrize("loop", ["persistent", "graph", "host"])
def test_batch_matches_single_volume_solves(ss4d, oracle, cuda, loop):
    torch = cuda
    sizes = [(20, 16, 12, 5), (33, 9, 14, 7), (12, 24, 10, 3)]
    vols = _volumes(ss4d, oracle, sizes)
    want, its = [], []
    for (p, u0, g), dims in zip(vols, sizes):
        u = _dev(torch, u0)
        gd = [_dev(torch, a) for a in g]
        with ss4d.Solver.for_interior(*dims, arith="fp64") as S:
            z = [S.seg_time_step(p, u, None, gd)["iterations"] for _ in range(2)]
        want.append(u.cpu().numpy())
        its.append(z)
    us = [_dev(torch, u0) for _, u0, _ in vols]
    gs = [[_dev(torch, a) for a in g] for _, _, g in vols]
    params = [p for p, _, _ in vols]
    with ss4d.Batch([(d[0] + 2, d[1] + 2, d[2] + 2, d[3] + 2) for d in sizes]) as B:
        B.set_persistent(loop == "persistent")
        B.set_graph(loop == "graph")
        got_its = [[s["iterations"] for s in B.seg_time_step(params, us, gs)] for _ in range(2)]
    for v in range(len(sizes)):
        assert [got_its[0][v], got_its[1][v]] == its[v], v
        assert np.array_equal(us[v].cpu().numpy(), want[v]), v


def test_batch_autotuned_shapes_do_not_change_results(ss4d, oracle, cuda):
    torch = cuda
    sizes = [(40, 20, 12, 4), (17, 30, 9, 6)]
    vols = _volumes(ss4d, oracle, sizes, seed=9)
    params = [p for p, _, _ in vols]
    gs = [[_dev(torch, a) for a in g] for _, _, g in vols]
    dims = [(d[0] + 2, d[1] + 2, d[2] + 2, d[3] + 2) for d in sizes]
    out = []
    for tune in (False, True):
        us = [_dev(torch, u0) for _, u0, _ in vols]
        with ss4d.Batch(dims) as B:
            if tune:
                shapes = B.autotune(params, us, gs)
                assert all(xt >= 8 and (xt & (xt - 1)) == 0 and kb >= 1 for xt, kb in shapes)
                # the autotuner only reads u
                assert all(np.array_equal(u.cpu().numpy(), v[1]) for u, v in zip(us, vols))
            else:
                B.set_shape(0, 8, 1)
                B.set_shape(1, 64, 8)
            stats = B.seg_time_step(params, us, gs)
        out.append(([u.cpu().numpy() for u in us], [s["iterations"] for s in stats]))
    assert out[0][1] == out[1][1]
    for a, b in zip(out[0][0], out[1][0]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("loop", ["persistent", "graph"])
@pytest.mark.parametrize("extrap", [0, 3, "proj"])
def test_mixed_batch_matches_single_volume_mixed_solves(ss4d, oracle, cuda, extrap, loop):
    """The mixed form batched (refinement passes and FP32 sweeps of all volumes
    in one persistent launch, or as kernels of a graph's while loop, every
    volume in its own phase) gives each volume what its own mixed-form solver
    gives it, step after step, with and without the extrapolated start, and
    with the projected start ("proj": extrapolation of order 3 whose first
    round starts from the projection onto the earlier changes): the same
    counts, the same u, the FP64 tolerance met.  Both have the assembly form
    each step's first refinement pass (start correction and FP64 residual)."""
    proj = extrap == "proj"
    extrap = 3 if proj else extrap
    torch = cuda
    sizes = [(20, 16, 12, 5), (33, 9, 14, 7), (12, 24, 10, 3)]
    vols = _volumes(ss4d, oracle, sizes, seed=11)
    steps = 5
    want = []
    for (p, u0, g), dims in zip(vols, sizes):
        u = _dev(torch, u0)
        gd = [_dev(torch, a) for a in g]
        with ss4d.Solver.for_interior(*dims, arith="mixed") as S:
            S.set_extrapolation(extrap)
            S.set_projection(proj)
            rec = []
            for _ in range(steps):
                st = S.seg_time_step(p, u, None, gd)
                rec.append((st["iterations"], st["refinements"], st["projected"], u.cpu().numpy()))
        want.append(rec)
    us = [_dev(torch, u0) for _, u0, _ in vols]
    gs = [[_dev(torch, a) for a in g] for _, _, g in vols]
    params = [p for p, _, _ in vols]
    with ss4d.Batch([(d[0] + 2, d[1] + 2, d[2] + 2, d[3] + 2) for d in sizes]) as B:
        B.set_arith("mixed")
        B.set_extrapolation(extrap)
        B.set_projection(proj)
        B.set_persistent(loop == "persistent")
        for step in range(steps):
            stats = B.seg_time_step(params, us, gs)
            for v, st in enumerate(stats):
                its, refs, prj, u_want = want[v][step]
                assert st["residual"] <= params[v].gsTol, (v, step)
                assert (st["iterations"], st["refinements"], st["projected"]) == (its, refs, prj), (v, step)
                assert prj == (proj and step >= 2), (v, step)
                assert np.array_equal(us[v].cpu().numpy(), u_want), (v, step)


def test_batch_switches_forms(ss4d, oracle, cuda):
    """One batch run in the FP64 form, then the mixed form, then FP64 again:
    each form's graph and buffers stay valid, and FP64 steps after the mixed
    ones equal FP64 steps from the same u."""
    torch = cuda
    sizes = [(16, 12, 10, 4), (10, 18, 8, 5)]
    vols = _volumes(ss4d, oracle, sizes, seed=13)
    params = [p for p, _, _ in vols]
    gs = [[_dev(torch, a) for a in g] for _, _, g in vols]
    dims = [(d[0] + 2, d[1] + 2, d[2] + 2, d[3] + 2) for d in sizes]
    us = [_dev(torch, u0) for _, u0, _ in vols]
    with ss4d.Batch(dims) as B:
        B.seg_time_step(params, us, gs)
        B.set_arith("mixed")
        st = B.seg_time_step(params, us, gs)
        assert all(s["residual"] <= p.gsTol and s["refinements"] >= 1 for s, p in zip(st, params))
        mid = [u.clone() for u in us]
        B.set_arith("fp64")
        B.seg_time_step(params, us, gs)
    with ss4d.Batch(dims) as B2:
        B2.seg_time_step(params, mid, gs)
    for a, b in zip(us, mid):
        assert np.array_equal(a.cpu().numpy(), b.cpu().numpy())


@pytest.mark.parametrize("arith", ["fp64", "mixed"])
def test_batch_with_minimal_and_ragged_volumes(ss4d, oracle, cuda, arith):
    """Volumes with a single interior voxel, odd and one-voxel extents next to
    an ordinary one, batched: each gets what its own solver gives it."""
    torch = cuda
    sizes = [(1, 1, 1, 1), (3, 2, 5, 2), (17, 4, 3, 6), (2, 9, 1, 3)]
    vols = _volumes(ss4d, oracle, sizes, seed=17)
    want = []
    for (p, u0, g), dims in zip(vols, sizes):
        u = _dev(torch, u0)
        gd = [_dev(torch, a) for a in g]
        with ss4d.Solver.for_interior(*dims, arith=arith) as S:
            z = [S.seg_time_step(p, u, None, gd)["iterations"] for _ in range(2)]
        want.append((z, u.cpu().numpy()))
    us = [_dev(torch, u0) for _, u0, _ in vols]
    gs = [[_dev(torch, a) for a in g] for _, _, g in vols]
    params = [p for p, _, _ in vols]
    with ss4d.Batch([(d[0] + 2, d[1] + 2, d[2] + 2, d[3] + 2) for d in sizes]) as B:
        B.set_arith(arith)
        got = [[s["iterations"] for s in B.seg_time_step(params, us, gs)] for _ in range(2)]
    for v in range(len(sizes)):
        assert [got[0][v], got[1][v]] == want[v][0], v
        assert np.array_equal(us[v].cpu().numpy(), want[v][1]), v


@pytest.mark.parametrize("arith", ["fp64", "mixed"])
def test_grid_barrier_timeout_is_reported(ss4d, oracle, cuda, arith):
    """Failure detection without a fault: a grid barrier that no arrival can
    complete (its arrival count starts beyond the grid) makes every block of
    the persistent loop give up its wait after about a second; the step
    returns SS4D_ERR_TIMEOUT, the context stays usable, and the same handle's
    next step from fresh inputs equals a fresh handle's step bit for bit."""
    torch = cuda
    sizes = [(20, 16, 12, 5), (12, 24, 10, 3)]
    vols = _volumes(ss4d, oracle, sizes, seed=9)
    params = [p for p, _, _ in vols]
    gs = [[_dev(torch, a) for a in g] for _, _, g in vols]
    dims = [(d[0] + 2, d[1] + 2, d[2] + 2, d[3] + 2) for d in sizes]
    with ss4d.Batch(dims) as B:
        if arith == "mixed":
            B.set_arith("mixed")
        B.set_test_withhold_barrier(True)
        us = [_dev(torch, u0) for _, u0, _ in vols]
        with pytest.raises(ss4d.SS4DError) as ei:
            B.seg_time_step(params, us, gs)
        assert ei.value.status == 5  # SS4D_ERR_TIMEOUT
        B.set_test_withhold_barrier(False)
        us = [_dev(torch, u0) for _, u0, _ in vols]
        got = [s["iterations"] for s in B.seg_time_step(params, us, gs)]
    with ss4d.Batch(dims) as F:
        if arith == "mixed":
            F.set_arith("mixed")
        ref = [_dev(torch, u0) for _, u0, _ in vols]
        want = [s["iterations"] for s in F.seg_time_step(params, ref, gs)]
    assert got == want
    for v in range(len(sizes)):
        assert np.array_equal(us[v].cpu().numpy(), ref[v].cpu().numpy()), v
