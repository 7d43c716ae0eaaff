"""The oracle's restatement of four_run's Lanczos filter (oracle/filter.py)
against closed forms: a delta's response is the reference's kernel table
normalised to sum 1, centred for odd extents and moved by the index maps for
even ones (one sample in 2D/3D, two in 1D, worked out by hand from the map
formulas of lib_f90/map_1dtofield.f90); a constant stays constant; extents
below the kernel table are refused."""
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import filter as FO  # noqa: E402


def f1(d, m=4, damp=0.5, one_d=False):
    if abs(d) >= m:
        return 0.0
    w = FO.sinc(math.pi * d * damp)
    return (w * w if one_d else w) * FO.sinc(math.pi * d / m)


@pytest.mark.parametrize("n,shift", [(21, 0), (20, -2), (23, 0), (26, -2)])
def test_delta_1d(n, shift):
    x = np.zeros(n)
    i = n // 2
    x[i] = 3.0
    y = FO.lanczos(x, 0.5, 4)
    want = np.array([f1((o - i - shift), one_d=True) for o in range(n)])
    want *= 3.0 / want.sum()
    np.testing.assert_allclose(y, want, atol=1e-13)


@pytest.mark.parametrize("shape,shift", [((21, 17), 0), ((20, 18), -1), ((21, 18), None)])
def test_delta_2d(shape, shift):
    x = np.zeros(shape)
    i, j = shape[0] // 2, shape[1] // 2
    x[i, j] = 1.0
    y = FO.lanczos(x, 0.5, 4)
    s = [0 if n % 2 else -1 for n in shape] if shift is None else [shift, shift]
    want = np.array([[f1(a - i - s[0]) * f1(b - j - s[1]) for b in range(shape[1])] for a in range(shape[0])])
    want /= want.sum()
    np.testing.assert_allclose(y, want, atol=1e-13)


def test_delta_3d_and_constant():
    shape = (13, 12, 11)
    x = np.zeros(shape)
    c = (5, 6, 5)
    x[c] = 1.0
    y = FO.lanczos(x, 0.3, 3)
    s = [0 if n % 2 else -1 for n in shape]
    want = np.zeros(shape)
    for a in range(shape[0]):
        for b in range(shape[1]):
            for l in range(shape[2]):
                want[a, b, l] = (f1(a - c[0] - s[0], 3, 0.3) * f1(b - c[1] - s[1], 3, 0.3)
                                 * f1(l - c[2] - s[2], 3, 0.3))
    want /= want.sum()
    np.testing.assert_allclose(y, want, atol=1e-13)
    np.testing.assert_allclose(FO.lanczos(np.full(shape, 2.5), 0.3, 3), 2.5, rtol=1e-12)


def test_wraps_around_the_edges():
    x = np.zeros(21)
    x[0] = 1.0
    y = FO.lanczos(x, 0.5, 4)
    assert y[-1] > 0 and y[-3] > 0 and abs(y.sum() - 1.0) < 1e-13


def test_extents_below_the_table_are_refused():
    for n in (9, 10):                              # the smallest extents are 2 m + 3 = 11 (odd), 2 m + 4 = 12
        with pytest.raises(ValueError):
            FO.lanczos(np.ones(n), 0.5, 4)
    for n in (11, 12):
        np.testing.assert_allclose(FO.lanczos(np.ones(n), 0.5, 4), 1.0, rtol=1e-12)


def test_four_filter_dispatch():
    rng = np.random.default_rng(3)
    d = rng.uniform(0.0, 5.0, (21, 17, 5))        # 3D with a short third axis: (i, j) slices
    y = FO.four_filter(d, 0.5, 4)
    for k in range(5):
        np.testing.assert_allclose(y[:, :, k], FO.lanczos(d[:, :, k], 0.5, 4), rtol=1e-14)
    p = rng.uniform(0.0, 5.0, (21, 17, 1))
    np.testing.assert_allclose(FO.four_filter(p, 0.5, 4)[:, :, 0], FO.lanczos(p[:, :, 0], 0.5, 4), rtol=1e-14)
