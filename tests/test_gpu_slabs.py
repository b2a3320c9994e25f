"""The GPU slab path (ss4d_slab_seg_time_step) on one GPU: two slabs of one
volume, each on its own solver handle and stream in its own host thread,
stand in for two ranks.  The host orders everything: an exchange waits for
the device, meets the other thread at a barrier, copies the neighbour's
boundary frame into the ghost frame and meets it again; the residual sum is
a host-side sum at a barrier.  No kernel waits on another.  The slabs' time
steps must equal the single-volume steps of the same (reference-order)
arithmetic bit for bit, with the same iteration counts."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS = (20, 14, 10, 9)  # nt = 9: slabs of 4 and 5 frames
STEPS = 3


def test_two_slabs_on_one_gpu_equal_the_single_volume(ss4d, oracle, cuda):
    torch = cuda
    nx, ny, nz, nt = DIMS
    p = ss4d.scene_params(gsTol=1e-9)
    i0, u0 = ss4d.scene(1, *DIMS, seed=29)
    g = oracle.gfaces(p, i0, np.zeros_like(i0))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731

    # the whole volume
    u = dev(u0)
    gd = [dev(a) for a in g]
    want_its = []
    with ss4d.Solver(*u0.shape[::-1], arith="reference") as S:
        for _ in range(STEPS):
            want_its.append(S.seg_time_step(p, u, None, gd)["iterations"])
    want = u.cpu().numpy()

    parts = ss4d.slab_partition(nt, 2)
    assert parts == [(1, 4), (5, 5)]
    slabs = []
    for first, count in parts:
        lo, hi = first - 1, first + count + 1
        slabs.append({"u": dev(u0[lo:hi]), "g": [dev(a[lo:hi]) for a in g], "first": first, "count": count})
    bar = threading.Barrier(2)
    sums = [0.0, 0.0]
    got_its = [[], []]
    errors = []

    def rank(r):
        me = slabs[r]
        lM = me["u"].shape[0]

        def exchange(u_ptr, fe, lMax, stream):
            assert u_ptr == me["u"].data_ptr() and lMax == lM
            torch.cuda.synchronize()
            bar.wait(timeout=60)
            if r == 1:  # ghost 0 <- the lower slab's last interior frame
                lower = slabs[0]["u"]
                me["u"][0].copy_(lower[lower.shape[0] - 2])
            else:  # ghost lM-1 <- the upper slab's first interior frame
                me["u"][lM - 1].copy_(slabs[1]["u"][1])
            torch.cuda.synchronize()
            bar.wait(timeout=60)

        def allreduce_sum(v):
            sums[r] = v
            bar.wait(timeout=60)
            total = sums[0] + sums[1]
            bar.wait(timeout=60)
            return total

        comm = ss4d.slab_comm(exchange, allreduce_sum)
        stream = torch.cuda.Stream()
        try:
            with ss4d.Solver(*me["u"].shape[::-1], arith="reference", stream=stream.cuda_stream) as S:
                for _ in range(STEPS):
                    st = S.slab_seg_time_step(p, me["u"], None, me["g"], comm, nx * ny * nz * nt)
                    got_its[r].append(st["iterations"])
        except Exception as ex:  # reported below
            errors.append((r, ex))
            bar.abort()

    th = [threading.Thread(target=rank, args=(r,)) for r in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=300)
    assert not errors, errors
    assert got_its[0] == got_its[1] == want_its, (got_its, want_its)
    for sl in slabs:
        f, c = sl["first"], sl["count"]
        assert np.array_equal(sl["u"][1:c + 1].cpu().numpy(), want[f:f + c])
        # the ghosts hold the neighbours' final frames (or the volume's boundary)
        assert np.array_equal(sl["u"][0].cpu().numpy(), want[f - 1])
        assert np.array_equal(sl["u"][c + 1].cpu().numpy(), want[f + c])
