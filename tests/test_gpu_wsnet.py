"""The learned warm start of the mixed form: the network's CUDA kernels
(forward, gradients, Adam) against a plain PyTorch FP32 reference on the CPU,
its features against the oracle's coefficients, and the solver path with a
network attached (the FP64 tolerance is still met; a prediction that does not
lower the correction residual is discarded and the step is then bit-identical
to a cold start)."""
import numpy as np
import pytest

import wsnet_ref
from conftest import rel_err

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def host(t):
    return t.detach().cpu().numpy()


def random_features(torch, rng, nf, nz, ny, nx):
    """device features in the network's planar layout, and the same values
    channels-last on the host for the reference"""
    import ss4d
    x = rng.standard_normal((nf, nz, ny, nx, 16)).astype(np.float32)
    xb = torch.from_numpy(x).to(torch.bfloat16)
    return ss4d.features_to_planar(xb).to("cuda"), host(xb.float())


def l2rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture
def net(ss4d, cuda):
    with ss4d.Wsnet(seed=3) as n:
        p = n.get_params()
        rng = np.random.default_rng(5)
        off = 0
        for cin, cout in n.LAYERS:  # non-zero biases so that their paths are tested too
            off += 27 * cin * cout
            p[off:off + cout] = 0.05 * rng.standard_normal(cout)
            off += cout
        n.set_params(p)
        yield n


@pytest.mark.parametrize("shape", [(2, 5, 11, 13), (1, 4, 8, 8), (3, 1, 2, 3),
                                   # partial tiles along every axis (tiles are 8 x 16 x 4 voxels)
                                   (2, 7, 35, 21),
                                   # 512 tiles: several per CTA, so the halo stages and the two
                                   # accumulator buffers each go round more than once
                                   (4, 16, 64, 64)])
def test_forward_matches_torch_reference(ss4d, cuda, net, shape):
    torch = cuda
    nf, nz, ny, nx = shape
    rng = np.random.default_rng(11)
    xd, xh = random_features(torch, rng, nf, nz, ny, nx)
    out = torch.full((nf, nz, ny, nx), float("nan"), dtype=torch.float32, device="cuda")
    net.forward(xd, nx, ny, nz, nf, out)
    torch.cuda.synchronize()
    want = wsnet_ref.predict(net.get_params(), xh)
    assert np.isfinite(host(out)).all()
    # BF16 activations: per-element differences come from one-ulp rounding
    # flips where the FP32 sums are accumulated in another order
    assert l2rel(host(out), want) <= 1e-2


def test_gradient_matches_autograd(ss4d, cuda, net):
    torch = cuda
    nf, nz, ny, nx, margin = 2, 6, 10, 12, 1
    rng = np.random.default_rng(12)
    xd, xh = random_features(torch, rng, nf, nz, ny, nx)
    target = rng.standard_normal((nf, nz, ny, nx)).astype(np.float32)
    params = net.get_params()
    grad = torch.zeros(net.nparam, dtype=torch.float32, device="cuda")
    loss = net.train_step(xd, dev(torch, target), nx, ny, nz, nf, margin=margin, lr=0.0, grad=grad)
    torch.cuda.synchronize()
    assert np.array_equal(net.get_params(), params)  # lr == 0 leaves the parameters alone
    want_loss, want_grad = wsnet_ref.loss_and_grad(params, xh, target, margin)
    assert abs(loss - want_loss) <= 1e-3 * want_loss
    g = host(grad)
    off = 0
    for L, (cin, cout) in enumerate(net.LAYERS):
        nw = 27 * cin * cout
        # BF16-rounded propagated gradients: a few 1e-3 relative at most
        assert l2rel(g[off:off + nw], want_grad[off:off + nw]) <= 2e-2, f"layer {L} weights"
        assert l2rel(g[off + nw:off + nw + cout], want_grad[off + nw:off + nw + cout]) <= 2e-2, f"layer {L} bias"
        off += nw + cout


def test_adam_steps_follow_the_reference(ss4d, cuda, net):
    """30 Adam steps on the GPU track the same steps taken with the reference
    gradient (torch autograd, FP32) from the same parameters."""
    torch = cuda
    nf, nz, ny, nx, steps, lr = 2, 8, 16, 16, 30, 3e-3
    rng = np.random.default_rng(13)
    xd, xh = random_features(torch, rng, nf, nz, ny, nx)
    k = np.array([0.25, 0.5, 0.25], np.float32)
    t = xh[..., 0]
    for ax in (1, 2, 3):  # a smoothed copy of channel 0 as the target
        t = sum(w * np.roll(t, s, axis=ax) for w, s in zip(k, (-1, 0, 1)))
    t = t.astype(np.float32)
    td = dev(torch, t)
    p0 = net.get_params()
    gpu = [net.train_step(xd, td, nx, ny, nz, nf, margin=1, lr=lr) for _ in range(steps)]
    q, m, v, cpu = p0.astype(np.float64), 0.0, 0.0, []
    for s in range(1, steps + 1):
        loss, g = wsnet_ref.loss_and_grad(q.astype(np.float32), xh, t, 1)
        cpu.append(loss)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        q = q - lr * (m / (1 - 0.9 ** s)) / (np.sqrt(v / (1 - 0.999 ** s)) + 1e-8)
    assert np.all(np.abs(np.array(gpu) - cpu) <= 3e-2 * np.array(cpu))
    assert gpu[-1] < 0.9 * gpu[0]
    change = net.get_params() - p0
    assert l2rel(change, q - p0) <= 0.1


def _scene(ss4d, oracle, dims, seed, kind=1):
    nx, ny, nz, nt = dims
    p = ss4d.scene_params(gsTol=1e-10)
    i0h, u0h = ss4d.scene(kind, nx, ny, nz, nt, seed=seed)
    g = oracle.gfaces(p, i0h, np.zeros_like(i0h))
    return p, i0h, u0h, g


def test_features_match_oracle(ss4d, oracle, cuda):
    torch = cuda
    dims = nx, ny, nz, nt = (13, 10, 7, 4)
    p, i0h, u0h, g = _scene(ss4d, oracle, dims, seed=21)
    coef = oracle.coefficients(p, u0h, g)
    c = p.tau / (p.h * p.h)
    # r0 = b - A u at u = prev: c * sum_f a_f (u_nb - u); faces e w n s t b fw bw
    offs = [(0, 0, 0, 1), (0, 0, 0, -1), (0, 0, 1, 0), (0, 0, -1, 0), (0, 1, 0, 0), (0, -1, 0, 0), (1, 0, 0, 0),
            (-1, 0, 0, 0)]
    inner = (slice(1, -1),) * 4
    ca = [c * coef[f][inner] for f in range(8)]
    r = np.zeros(ca[0].shape)
    for f, o in enumerate(offs):
        nb = tuple(slice(1 + d, u0h.shape[a] - 1 + d) for a, d in enumerate(o))
        r += ca[f] * (u0h[nb] - u0h[inner])
    sigma_want = float(np.sqrt(np.mean(r * r)))
    rs = r / sigma_want
    idiag = 1.0 / (1.0 + sum(ca))
    want = np.zeros((nt, nz, ny, nx, 16))
    want[..., 0] = rs
    want[1:, ..., 1] = rs[:-1]
    want[:-1, ..., 2] = rs[1:]
    want[..., 3] = rs * idiag
    for f in range(8):
        want[..., 4 + f] = ca[f] * idiag
    want[..., 12] = idiag
    want[..., 13] = sum(g[f][inner] for f in range(8)) / 8
    want[..., 14] = u0h[inner]
    want[..., 15] = i0h[inner]

    x0 = torch.zeros((nt, 2, nz, ny, nx, 8), dtype=torch.bfloat16, device="cuda")  # planar
    u = dev(torch, u0h)
    with ss4d.Solver.for_interior(*dims, arith="mixed") as S:
        sigma = S.ws_features(p, u, [dev(torch, a) for a in g], dev(torch, i0h), x0)
    torch.cuda.synchronize()
    assert np.array_equal(host(u), u0h)  # features leave u alone
    assert abs(sigma - sigma_want) <= 1e-12 * sigma_want
    x = host(ss4d.features_from_planar(x0).float())
    assert not x[0, ..., 1].any() and not x[-1, ..., 2].any()  # frames outside 1..nt
    # BF16 storage: at most one unit in the last place (2^-8 relative) apart
    for ch in range(16):
        err = np.abs(x[..., ch] - want[..., ch])
        assert np.all(err <= np.abs(want[..., ch]) / 128 + 1e-6), f"channel {ch}: max err {err.max()}"


def _run_steps(ss4d, torch, dims, p, u0h, g, i0h, steps, net=None, graph=True):
    u = dev(torch, u0h)
    gd = [dev(torch, a) for a in g]
    i0 = dev(torch, i0h)
    stats = []
    with ss4d.Solver.for_interior(*dims, arith="mixed") as S:
        S.set_graph(graph)
        if net is not None:
            S.set_warm_start(net, i0)
        for _ in range(steps):
            stats.append(S.seg_time_step(p, u, None, gd))
    torch.cuda.synchronize()
    return host(u), stats


@pytest.mark.parametrize("graph", [True, False])
def test_warm_started_steps_meet_the_fp64_tolerance(ss4d, oracle, cuda, net, graph):
    torch = cuda
    dims = (24, 20, 12, 5)
    p, i0h, u0h, g = _scene(ss4d, oracle, dims, seed=31)
    cold, cs = _run_steps(ss4d, torch, dims, p, u0h, g, i0h, 3)
    warm, ws = _run_steps(ss4d, torch, dims, p, u0h, g, i0h, 3, net=net, graph=graph)
    for st in cs + ws:
        assert st["status"] == 0 and st["residual"] <= p.gsTol
    assert all(st["warm_started"] in (0, 1) for st in ws)
    assert rel_err(warm, cold) <= 1e-4


@pytest.mark.parametrize("graph", [True, False])
def test_bad_prediction_is_discarded(ss4d, oracle, cuda, net, graph):
    torch = cuda
    dims = (20, 16, 10, 4)
    p, i0h, u0h, g = _scene(ss4d, oracle, dims, seed=41)
    params = net.get_params()
    params[-1] = 1e3  # the output bias: a prediction of 1000 s everywhere
    net.set_params(params)
    cold, cs = _run_steps(ss4d, torch, dims, p, u0h, g, i0h, 2)
    warm, ws = _run_steps(ss4d, torch, dims, p, u0h, g, i0h, 2, net=net, graph=graph)
    assert [st["warm_started"] for st in ws] == [0, 0]
    assert [st["iterations"] for st in ws] == [st["iterations"] for st in cs]
    assert [st["refinements"] for st in ws] == [st["refinements"] for st in cs]
    assert np.array_equal(warm, cold)


def test_trained_network_cuts_iterations_on_unseen_scenes(ss4d, oracle, cuda):
    """The committed parameters (weights/wsnet_seg.npy, trained by
    train_wsnet.py on 128x128x64x12 multi-object scenes) on scenes of other
    seeds and sizes: every step keeps the prediction, needs fewer FP32
    iterations (at 256x256x128x20, 6 steps: 209 -> 152), meets the same FP64
    tolerance, and ends where the cold start ends (masks differ in at most
    0.1 % of their voxels)."""
    import os

    torch = cuda
    params = np.load(os.path.join(os.path.dirname(ss4d.__file__), "weights", "wsnet_seg.npy"))
    with ss4d.Wsnet(seed=None) as net:
        net.set_params(params)
        for kind, seed, dims in ((3, 777, (128, 112, 56, 10)), (3, 778, (96, 80, 40, 8))):
            nx, ny, nz, nt = dims
            p = ss4d.scene_params()
            i0h, u0h = ss4d.scene(kind, nx, ny, nz, nt, seed=seed)
            # the edge detector as in training: presmoothed image, its g faces
            i0d = dev(torch, i0h)
            gd = [torch.empty_like(i0d) for _ in range(8)]
            with ss4d.Solver.for_interior(*dims, arith="fp64") as S:
                S.edge_detector(p, i0d, None, gd)
                S.synchronize()
            i0h, g = host(i0d), [host(a) for a in gd]
            cold, cs = _run_steps(ss4d, torch, dims, p, u0h, g, i0h, 6)
            warm, ws = _run_steps(ss4d, torch, dims, p, u0h, g, i0h, 6, net=net)
            assert all(st["warm_started"] == 1 for st in ws)
            assert all(st["residual"] <= p.gsTol for st in cs + ws)
            ci, wi = sum(st["iterations"] for st in cs), sum(st["iterations"] for st in ws)
            assert wi <= 0.9 * ci, (ci, wi)
            assert rel_err(warm, cold) <= 1e-3
            lev = 0.5 * (cold.min() + cold.max())
            a, b = warm[1:-1, 1:-1, 1:-1, 1:-1] >= lev, cold[1:-1, 1:-1, 1:-1, 1:-1] >= lev
            assert (a ^ b).sum() <= max(2, 1e-3 * (a.sum() + b.sum()))


@pytest.mark.parametrize("graph", [True, False])
def test_extrapolated_start_meets_the_fp64_tolerance(ss4d, oracle, cuda, graph):
    """Mixed steps started from the extrapolation of order 1, 2 or 3 of the
    earlier steps' changes: the first step (no history)
    is bit-identical to a plain mixed step, every step meets the FP64
    tolerance, fewer iterations are needed, and the states agree with the
    plain mixed steps."""
    torch = cuda
    dims = (40, 32, 24, 6)
    p, i0h, u0h, g = _scene(ss4d, oracle, dims, seed=51)
    gd = [dev(torch, a) for a in g]
    runs = {}
    for order in (0, 1, 2, 3):
        u = dev(torch, u0h)
        with ss4d.Solver.for_interior(*dims, arith="mixed") as S:
            S.set_graph(graph)
            S.set_extrapolation(order)
            stats, states = [], []
            for _ in range(6):
                stats.append(S.seg_time_step(p, u, None, gd))
                states.append(host(u))
        runs[order] = (stats, states)
    cs, cu = runs[0]
    for order in (1, 2, 3):
        xs, xu = runs[order]
        assert np.array_equal(xu[0], cu[0]) and xs[0]["iterations"] == cs[0]["iterations"]
        assert all(st["status"] == 0 and st["residual"] <= p.gsTol for st in cs + xs)
        assert sum(st["iterations"] for st in xs[1:]) < sum(st["iterations"] for st in cs[1:])
        assert rel_err(xu[-1], cu[-1]) <= 1e-4


def test_convolution_wait_timeout_is_reported(ss4d, cuda, net):
    """Failure detection without a fault: with its halo loads withheld, every
    tensor-core convolution's waits run out after about a second; the
    prediction is NaN (which the warm start's check discards), the network
    reports SS4D_ERR_TIMEOUT, and the next forward is exact again."""
    torch = cuda
    nf, nz, ny, nx = 1, 4, 16, 16
    rng = np.random.default_rng(13)
    xd, _ = random_features(torch, rng, nf, nz, ny, nx)
    good = torch.full((nf, nz, ny, nx), float("nan"), dtype=torch.float32, device="cuda")
    net.forward(xd, nx, ny, nz, nf, good)
    net.check()
    out = torch.zeros_like(good)
    net.set_test_withhold_loads(True)
    try:
        net.forward(xd, nx, ny, nz, nf, out)
        with pytest.raises(ss4d.SS4DError) as ei:
            net.check()
        assert ei.value.status == 5  # SS4D_ERR_TIMEOUT
        assert torch.isnan(out).all()
    finally:
        net.set_test_withhold_loads(False)
    net.forward(xd, nx, ny, nz, nf, out)
    net.check()
    assert torch.equal(out, good)
