"""four_run's Lanczos filter on the device (k_filter.cu) against the oracle's
FFT restatement (oracle/filter.py): the standalone entry on 1D, 2D, 3D and
sliced 3D fields of odd and even extents, four_run with opts.filter (dsi
filtered before the statistics), and the refusals."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S
from oracle import filter as FO

pytestmark = pytest.mark.gpu


def opts(width=4, damp=0.5, scale=1.0):
    return K.opts(filter=_abi.FILTER_LANCZOS, filter_width=width, filter_damp=damp, filter_scale=scale)


@pytest.mark.parametrize("shape", [(31, 1, 1), (30, 1, 1), (25, 21, 1), (24, 22, 1), (15, 13, 11), (16, 14, 12),
                                   (21, 17, 5), (21, 5, 17), (5, 21, 17), (20, 6, 16)])
def test_filter_vs_oracle(ctx, shape):
    rng = np.random.default_rng(sum(shape))
    d = np.asfortranarray(rng.uniform(0.0, 50.0, shape) * (1 + 100 * (rng.uniform(size=shape) < 0.02)))
    got = FR.four_filter(d, opts(), ctx=ctx)
    want = FO.four_filter(d, 0.5, 4)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def test_filter_width_and_damp(ctx):
    rng = np.random.default_rng(5)
    d = np.asfortranarray(rng.uniform(0.0, 1.0, (19, 23, 1)))
    got = FR.four_filter(d, opts(width=3, damp=0.8), ctx=ctx)
    np.testing.assert_allclose(got, FO.four_filter(d, 0.8, 3), rtol=1e-12, atol=1e-13)


def test_four_run_filters_dsi_before_the_statistics(ctx):
    cr, _ = S.small_lots_anis(anis=False)
    g = S.GridData.from_corners((-2.0, -2.0, 0.5), (2.0, -2.0, 0.5), (-2.0, 2.0, 0.5), inc=(25, 21, 1))
    base = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64), ctx=ctx)
    r = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64, filter=_abi.FILTER_LANCZOS), ctx=ctx)
    want = FO.four_filter(base.dsi, 0.5, 4)
    np.testing.assert_allclose(r.dsi, want, rtol=1e-11, atol=1e-11 * want.max())
    np.testing.assert_array_equal(r.csf, base.csf)
    # four_qinfo's maximum and minimum over the grid are taken from the filtered dsi
    assert np.isclose(max(r.info.res[2], r.info.res[6]), r.dsi.max(), rtol=1e-12)


@pytest.mark.parametrize("shape,kw", [((9, 1, 1), {}), ((10, 1, 1), {}), ((1, 25, 21), {}), ((25, 1, 21), {}),
                                      ((25, 21, 1), {"scale": 2.0})])
def test_filter_refusals(ctx, shape, kw):
    with pytest.raises(Exception) as e:
        FR.four_filter(np.ones(shape), opts(**kw), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_UNSUPPORTED


def test_gradient_refuses_a_filtered_intensity(ctx):
    from diffusecode_gb300.autograd import chi2_grad
    cr, _ = S.small_lots_anis(anis=False)
    g = S.GridData.from_corners((-2.0, -2.0, 0.5), (2.0, -2.0, 0.5), (-2.0, 2.0, 0.5), inc=(25, 21, 1))
    it = np.ones(g.inc)
    with pytest.raises(Exception) as e:
        chi2_grad(cr, g, K.opts(phase=_abi.PHASE_EXACT64, filter=_abi.FILTER_LANCZOS), it, None, ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_UNSUPPORTED
