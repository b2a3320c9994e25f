"""One volume split across ranks by frames (t-slabs; the reference's MPI
program, segmentation4D_mpi.c:282-397 and :485-526).

The library's slab loop (ss4d_slab_sor_loop) runs here on the CPU: each of
two gloo ranks holds its slab of an oracle volume as a padded volume with
one ghost frame per side, the oracle does the half-sweeps and the residual
of its slab, gloo exchanges the ghost frames after every half-sweep and sums
the residual every iteration.  Time steps of the slabs must reproduce the
single-volume oracle's iterates bit for bit, with the same iteration counts.
"""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import PKG, ROOT

DIMS = (12, 10, 8, 7)  # nt = 7: slabs of 4 and 3 frames, the second starting on an even offset
STEPS = 3


def _single_volume(ss4d, oracle):
    """the oracle's steps on the whole volume: u after each, iteration counts"""
    p = ss4d.scene_params(gsTol=1e-10)
    i0, u0 = ss4d.scene(1, *DIMS, seed=17)
    g = oracle.gfaces(p, i0, np.zeros_like(i0))
    u = u0.copy()
    prev = np.zeros_like(u)
    out = []
    for _ in range(STEPS):
        z, R = oracle.seg_time_step(p, u, prev, g, mmask=np.ones_like(u))
        out.append((z, u.copy()))
    return p, u0, g, out


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    for pth in (PKG, os.path.join(ROOT, "oracle"), ROOT):
        sys.path.insert(0, pth)
    import torch
    import torch.distributed as dist

    import oracle
    import ss4d

    oracle.set_threads(1)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p, u0, g, _ = _single_volume(ss4d, oracle)
        nx, ny, nz, nt = DIMS
        first, count = ss4d.slab_partition(nt, world)[rank]
        lo, hi = first - 1, first + count + 1  # global frames of the slab, ghosts included
        u = np.ascontiguousarray(u0[lo:hi])
        gs = [np.ascontiguousarray(a[lo:hi]) for a in g]
        lM = u.shape[0]
        fe = u[0].size

        def exchange(u_ptr, frame_elems, lMax, stream):
            assert u_ptr == u.ctypes.data and frame_elems == fe and lMax == lM and stream is None
            reqs = []
            down = torch.empty(fe, dtype=torch.float64)
            up = torch.empty(fe, dtype=torch.float64)
            first_f = torch.from_numpy(u[1].reshape(-1).copy())
            last_f = torch.from_numpy(u[lM - 2].reshape(-1).copy())
            if rank > 0:
                reqs.append(dist.isend(first_f, rank - 1))
                reqs.append(dist.irecv(down, rank - 1))
            if rank < world - 1:
                reqs.append(dist.isend(last_f, rank + 1))
                reqs.append(dist.irecv(up, rank + 1))
            for r in reqs:
                r.wait()
            if rank > 0:
                u[0] = down.numpy().reshape(u[0].shape)
            if rank < world - 1:
                u[lM - 1] = up.numpy().reshape(u[lM - 1].shape)

        def allreduce_sum(v):
            t = torch.tensor([v], dtype=torch.float64)
            dist.all_reduce(t)
            return float(t.item())

        comm = ss4d.slab_comm(exchange, allreduce_sum)
        results = []
        prev = np.zeros_like(u)
        for _ in range(STEPS):
            # the step of _segTimeStep_mpi_: ghosts current, prev <- u,
            # coefficients of the slab, the slab loop; rescale is the identity
            exchange(u.ctypes.data, fe, lM, None)
            prev[...] = u
            coef = oracle.coefficients(p, u, gs)
            ops = ss4d.slab_ops(lambda colour: oracle.sor_half(p, u, prev, coef, colour),
                                lambda: oracle.sor_residual(p, u, prev, coef), u.ctypes.data, fe, lM)
            st = ss4d.slab_sor_loop(ops, comm, p, nx * ny * nz * nt)
            results.append((st["iterations"], st["near_tolerance"], u[1:lM - 1].copy()))
        q.put((rank, first, count, results))
    finally:
        dist.destroy_process_group()


def _port():
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        return sck.getsockname()[1]


def test_two_slabs_reproduce_the_single_volume_steps(ss4d, oracle):
    mp = pytest.importorskip("torch.multiprocessing")
    p, u0, g, want = _single_volume(ss4d, oracle)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = sorted(q.get(timeout=300) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert [(f, c) for _, f, c, _ in got] == [(1, 4), (5, 3)]
    for step in range(STEPS):
        z_want, u_want = want[step]
        for rank, first, count, res in got:
            z, near, u_slab = res[step]
            assert z == z_want or near, (step, rank, z, z_want)
            assert np.array_equal(u_slab, u_want[first:first + count]), (step, rank)


@pytest.mark.parametrize("nt,nranks", [(20, 2), (7, 2), (7, 4), (9, 3), (2, 1), (1, 1), (40, 8)])
def test_partition_gives_even_slabs_but_the_last(ss4d, nt, nranks):
    parts = ss4d.slab_partition(nt, nranks)
    assert parts[0][0] == 1 and sum(c for _, c in parts) == nt
    for (f, c), (f2, _) in zip(parts, parts[1:]):
        assert f2 == f + c and c % 2 == 0 and c >= 2
    assert all((f - 1) % 2 == 0 for f, _ in parts)  # every slab starts on an even offset
    assert max(c for _, c in parts) - min(c for _, c in parts) <= 3


def test_partition_refuses_too_few_frames(ss4d):
    with pytest.raises(ss4d.SS4DError):
        ss4d.slab_partition(6, 4)  # some rank would need an odd start or no frame


def test_slab_loop_reports_callback_failures(ss4d):
    p = ss4d.scene_params()
    u = np.zeros((5, 4, 4, 4))
    ops = ss4d.slab_ops(lambda c: 1 / 0, lambda: 0.0, u.ctypes.data, 64, 5)
    comm = ss4d.slab_comm(lambda *a: None, lambda v: v)
    with pytest.raises(ss4d.SS4DError) as ei:
        ss4d.slab_sor_loop(ops, comm, p, 2 * 2 * 2 * 3)
    assert "half-sweep" in str(ei.value)
