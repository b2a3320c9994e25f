"""The separable Gaussian G_sigma offered beside the reference's implicit
presmoothing (an option the reference does not have): the C oracle against
scipy's Gaussian filter with the same taps and the same mirrored boundary
(scipy's 'reflect': ghost 0 = voxel 1, as the reference's reflection)."""
import math

import numpy as np
import pytest

from conftest import rel_err


def _inner(a):
    return a[1:-1, 1:-1, 1:-1, 1:-1]


@pytest.mark.parametrize("sigma", [(1.0, 0.7, 1.3, 0.0), (0.4, 0.0, 2.5, 1.0), (3.0, 3.0, 3.0, 3.0)])
def test_oracle_gaussian_matches_scipy(oracle, sigma):
    nd = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(21)
    v = rng.random((7, 9, 11, 13))  # padded (l, k, j, i): interior 5 x 7 x 9 x 11
    want = _inner(v).copy()
    for a, s in enumerate(sigma):  # x, y, z, t = array axes 3, 2, 1, 0
        if s > 0:
            want = nd.gaussian_filter1d(want, s, axis=3 - a, mode="reflect", radius=math.ceil(3 * s))
    got = v.copy()
    assert oracle.gaussian(sigma, got) == 0
    assert rel_err(_inner(got), want) <= 1e-13
    # the ghost layer by reflection
    assert np.array_equal(got[1:-1, 1:-1, 1:-1, 0], got[1:-1, 1:-1, 1:-1, 1])
    assert np.array_equal(got[0], got[1])
    assert np.array_equal(got[-1], got[-2])


def test_oracle_gaussian_keeps_constants_and_refuses_wide_taps(oracle):
    v = np.full((6, 8, 7, 9), 0.375)
    assert oracle.gaussian((1.2, 0.9, 2.0, 0.5), v) == 0
    assert np.abs(v - 0.375).max() <= 1e-15
    assert oracle.gaussian((11.0, 0.0, 0.0, 0.0), v) == -1  # ceil(33) > 32 taps
