"""Pin the CPU oracle against fixtures produced by the reference itself
(tests/golden/make_golden.py runs the reference compiled from its own
sources).  The oracle keeps the reference's evaluation order and calls pow()
where the reference does, so on the same host every comparison is exact."""
import numpy as np
import pytest

from conftest import load_golden, params_from_golden


def test_seg_small_edge_detector_bit_exact(ss4d, oracle):
    d = load_golden("seg_small.npz")
    p = params_from_golden(ss4d, d)
    i0 = d["i0_in"].copy()
    thr = d["thr_in"].copy()
    g, zs, _ = oracle.edge_detector(p, i0, thr)
    assert list(zs) == list(d["presmooth_its"])
    assert np.array_equal(i0, d["i0_smooth"])
    assert np.array_equal(thr, d["thr_smooth"])
    for f in range(8):
        assert np.array_equal(g[f], d[f"g{f}"]), f"g face {f}"


def test_seg_small_time_steps_bit_exact(ss4d, oracle):
    d = load_golden("seg_small.npz")
    p = params_from_golden(ss4d, d)
    g = [d[f"g{f}"] for f in range(8)]
    u = d["u0"].copy()
    prev = np.zeros_like(u)
    mm = np.ones_like(u)
    for step in range(5):
        coef = oracle.new_like(u, 8)
        z, R = oracle.seg_time_step(p, u, prev, g, coef=coef, mmask=mm)
        assert z == d["its"][step]
        assert float("%.6e" % R) == d["res"][step]
        assert np.array_equal(u, d["u_steps"][step]), f"u after step {step + 1}"
        assert oracle.l2norm(p.h, prev, u) == d["l2"][step]
        if step == 0:
            assert np.array_equal(prev, d["prev1"])
            for f in range(8):
                assert np.array_equal(coef[f], d[f"coef{f}"]), f"coefficient {f}"
    assert oracle.mass(p.h, u) == float(d["mass"])


def test_seg_balls_rescale_and_threshold_path(ss4d, oracle):
    d = load_golden("seg_balls.npz")
    p = params_from_golden(ss4d, d)
    balls = [(int(b[0]), b[1], b[2], b[3]) for b in d["balls"]]
    i0 = d["i0_in"].copy()
    thr = d["thr_in"].copy()
    g, _, _ = oracle.edge_detector(p, i0, thr)
    assert np.array_equal(i0, d["i0_smooth"])
    assert np.array_equal(thr, d["thr_smooth"])
    for f in range(8):
        assert np.array_equal(g[f], d[f"g{f}"])
    u = d["u_gen"].copy()
    assert oracle.rescale(p.ballRadius, u, d["mmask"], balls) == 0
    assert np.array_equal(u, d["u0"])
    prev = np.zeros_like(u)
    for step in range(3):
        z, R = oracle.seg_time_step(p, u, prev, g, mmask=d["mmask"], balls=balls)
        assert z == d["its"][step]
        assert np.array_equal(u, d["u_steps"][step])


def test_rescale_refuses_ball_outside_array(ss4d, oracle):
    u = np.zeros((5, 8, 8, 8))
    assert oracle.rescale(3.0, u, None, [(1, 1.0, 4.0, 4.0)]) == -1


def test_mcf_known_answer_bit_exact(ss4d, oracle):
    d = load_golden("mcf_small.npz")
    for n, steps, key in ((8, 3, "err8"), (16, 4, "err16")):
        p = ss4d.mcf_params(n, steps)
        shape = (n + 2,) * 4
        u = oracle.mcf_exact(p.h, 0.0, shape)
        prev = np.zeros_like(u)
        errs = []
        for step in range(1, steps + 1):
            oracle.mcf_time_step(p, step, u, prev)
            ex = oracle.mcf_exact(p.h, step * p.tau, shape)
            errs.append(oracle.l2norm(p.h, ex, u))
            if n == 8:
                assert np.array_equal(u, d["u8"][step - 1])
        assert np.array_equal(np.array(errs), d[key])
    # first-order convergence in h of the known-answer error (mcf_4D.c:512-515)
    assert d["err16"][0] < d["err8"][0] / 4


def test_32x32x32x8_twenty_steps(ss4d, oracle):
    """The 32^3 x 8 workload: the oracle reproduces the reference's
    iteration counts, residual print-outs, step differences, probes and
    masks over 20 steps."""
    d = load_golden("seg_32x32x32x8.npz")
    nx, ny, nz, nt = (int(v) for v in d["dims"])
    p = ss4d.scene_params(maxNoOfTimeSteps=20)
    i0, u = ss4d.scene(1, nx, ny, nz, nt, seed=int(d["seed"]))
    thr = np.zeros_like(u)
    oracle.set_threads(4)
    try:
        g, _, _ = oracle.edge_detector(p, i0, thr)
    finally:
        oracle.set_threads(1)
    prev = np.zeros_like(u)
    mm = np.ones_like(u)
    coef = oracle.new_like(u, 8)
    for step in range(20):
        z, R = oracle.seg_time_step(p, u, prev, g, coef=coef, mmask=mm)
        assert z == d["its"][step], f"step {step + 1}"
        assert float("%.6e" % R) == d["res"][step]
        assert oracle.l2norm(p.h, prev, u) == d["l2"][step]
        assert np.array_equal(u.reshape(-1)[d["probes"]], d["probe_vals"][step])
    m05 = oracle.threshold_mask(u, 0.5, False)
    mn = oracle.threshold_mask(u, 0.5, True)
    assert np.array_equal(np.packbits(m05), d["mask05"])
    assert np.array_equal(np.packbits(mn), d["masknorm"])


def _balls(d):
    return [(int(b[0]), float(b[1]), float(b[2]), float(b[3])) for b in d["balls"]]


def test_initial_segmentation_small_balls(oracle):
    """Local thresholding and the initial function of the reference main's
    pipeline (ball radius 3, alpha 0.85, beta 0.15), bit-exact."""
    d = load_golden("seg_balls.npz")
    balls = _balls(d)
    thr = np.zeros_like(d["i0_in"])
    assert oracle.local_threshold(0.85, 0.15, 3.0, d["i0_in"].copy(), thr, balls) == 0
    assert np.array_equal(thr, d["thr_in"])
    u = d["thr_smooth"].copy()
    mm = np.zeros_like(u)
    assert oracle.generate_segm(3.0, u, mm, balls) == 0
    assert np.array_equal(u, d["u_gen"])
    assert np.array_equal(mm, d["mmask"])


def test_initial_segmentation_large_balls(oracle):
    """Ball radius 13 (above the initial function's fixed radius 12), a
    non-zero thresholded image, overlapping balls: global maximum, per-ball
    minimum/maximum, local thresholding, initial function and Mmask."""
    d = load_golden("seg_init.npz")
    alpha, beta, R = (float(v) for v in d["alpha_beta_R"])
    balls = _balls(d)
    i0 = d["i0_in"]
    assert oracle.max4d(i0) == float(d["gmax"])
    for b, (l, x, y, z) in enumerate(balls):
        assert oracle.ball_min_max(i0, l, x, y, z, R) == (d["ball_min"][b], d["ball_max"][b])
    thr = d["thr_before"].copy()
    assert oracle.local_threshold(alpha, beta, R, i0.copy(), thr, balls) == 0
    assert np.array_equal(thr, d["thr_after"])
    u = d["u_before"].copy()
    mm = np.zeros_like(u)
    assert oracle.generate_segm(R, u, mm, balls) == 0
    assert np.array_equal(u, d["u_gen"])
    assert np.array_equal(mm, d["mmask"])
    # a ball whose box leaves the array is refused (the reference would read outside it)
    assert oracle.local_threshold(alpha, beta, R, i0.copy(), thr, [(1, 3.0, 17.0, 16.0)]) == -1


@pytest.mark.parametrize("steps", [0, 1, 3])
def test_explicit_presmoothing_bit_exact(ss4d, oracle, steps):
    d = load_golden("presmooth_exp.npz")
    sigma, h = (float(v) for v in d["sigma_h"])
    p = ss4d.scene_params(sigma=sigma, h=h)
    v = d["v_in"].copy()
    prev = oracle.presmooth_explicit(p, steps, v)
    assert np.array_equal(v, d[f"u_{steps}"])
    assert np.array_equal(prev, d[f"prev_{steps}"])
