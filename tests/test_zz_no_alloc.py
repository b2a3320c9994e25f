"""The allocation-free rescale, ss4d_rescale_to_zero_one_noalloc.

It serves callers that cannot allocate device memory — a host application
whose GPU memory is owned by its own fixed pool, or a per-frame loop that must
not pay cudaMalloc's implicit synchronisation — so it takes no solver handle
and stages its centre table in a fixed array inside the library.  Here it is
called through the C ABI and checked against the handle-based entry point
(ss4d_rescale_to_zero_one) on two calls in a row with different centre
tables: the second call must not see the first call's table, which the shared
array still holds.  Both paths run the same kernels on the same data, so the
results must agree exactly (the tolerance of the rescale parity tests).

This file is named so that pytest collects it last.
"""
import numpy as np
import pytest

from conftest import load_golden, params_from_golden

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def test_noalloc_rescale_matches_handle_path_on_two_calls(ss4d, cuda):
    torch = cuda
    d = load_golden("seg_balls.npz")
    p = params_from_golden(ss4d, d)
    shape = d["u_gen"].shape
    dims = shape[::-1]
    mm = _dev(torch, d["mmask"])
    all_balls = [(int(b[0]), b[1], b[2], b[3]) for b in d["balls"]]
    calls = [
        (d["u_gen"], all_balls),
        # second call: fewer centres, in one frame only, on another field
        (d["u_steps"][0] + 0.25 * d["u_gen"], [b for b in all_balls if b[0] == 2]),
    ]
    with ss4d.Solver(*dims) as S:
        for u_in, balls in calls:
            want = _dev(torch, u_in)
            S.rescale_to_zero_one(p, want, mm, balls)
            got = _dev(torch, u_in)
            ss4d.rescale_to_zero_one_noalloc(dims, p, got, mm, balls)
            torch.cuda.synchronize()
            assert not torch.equal(got, _dev(torch, u_in))  # the call did work
            assert torch.equal(got, want)


def test_noalloc_rescale_rejects_inputs_beyond_its_table(ss4d, cuda):
    torch = cuda
    p = ss4d.scene_params(ballRadius=2.0)
    lM = 8
    u = torch.zeros((lM, 10, 10, 10), dtype=torch.float64, device="cuda")
    too_many = [(1, 5.0, 5.0, 5.0)] * 1025  # SS4D_NOALLOC_MAX_BALLS + 1
    with pytest.raises(ss4d.SS4DError) as ei:
        ss4d.rescale_to_zero_one_noalloc((10, 10, 10, lM), p, u, None, too_many)
    assert ei.value.status == 1 and "exceed" in str(ei.value)
    long = torch.zeros((1026, 3, 3, 3), dtype=torch.float64, device="cuda")  # lMax beyond 1024 frames
    with pytest.raises(ss4d.SS4DError) as ei:
        ss4d.rescale_to_zero_one_noalloc((3, 3, 3, 1026), p, long, None, [(1, 1.0, 1.0, 1.0)])
    assert ei.value.status == 1 and "exceeds" in str(ei.value)
