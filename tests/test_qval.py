"""qval (discus/prog/qval.f90:65-290): the oracle against closed forms (CPU)
and the device against the oracle on the same csf/acsf/dsi (GPU)."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import structures as S
from oracle import oracle as O

VALUES = [_abi.VAL_INTEN, _abi.VAL_AMPLI, _abi.VAL_PHASE, _abi.VAL_REAL, _abi.VAL_IMAG, _abi.VAL_RANPH,
          _abi.VAL_SQ, _abi.VAL_F2AVER, _abi.VAL_FAVER2, _abi.VAL_FAVER, _abi.VAL_IQ, _abi.VAL_F2AVERB,
          _abi.VAL_FAVER2B, _abi.VAL_FAVERB]


def _case():
    cr, g = S.small_lots_anis(anis=False, inc=(13, 11, 3))
    op = K.opts(phase=_abi.PHASE_EXACT64, fave=1.0)
    rc, csf, acsf, dsi, info = O.four_run(cr, g, op)
    assert rc == 0
    rnd = np.random.default_rng(5).random(g.inc)
    return cr, g, op, csf, acsf, dsi, rnd


def test_oracle_qval_closed_forms():
    cr, g, op, csf, acsf, dsi, rnd = _case()
    q = lambda v, **kw: O.qval(cr, g, op, v, csf, acsf, dsi, rand=rnd, **kw)[1]
    np.testing.assert_array_equal(q(_abi.VAL_INTEN), dsi)
    np.testing.assert_allclose(q(_abi.VAL_INTEN, laver=True), np.abs(acsf) ** 2, rtol=1e-14)
    np.testing.assert_allclose(q(_abi.VAL_AMPLI), np.abs(csf), rtol=1e-14)
    np.testing.assert_allclose(q(_abi.VAL_PHASE), np.degrees(np.angle(csf)), rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(q(_abi.VAL_REAL), csf.real)
    np.testing.assert_array_equal(q(_abi.VAL_IMAG, laver=True), acsf.imag)
    n_real = np.count_nonzero(cr.iscat > 0)
    np.testing.assert_allclose(q(_abi.VAL_IQ), dsi / n_real, rtol=1e-14)
    # neutron scattering lengths: <f^2>, <f>^2, <f> are constants of the composition
    op_n = K.opts(phase=_abi.PHASE_EXACT64, lxray=0)
    amount = np.array([np.count_nonzero(cr.iscat == t) for t in range(1, cr.nscat + 1)])
    c = cr.scat[1:, 0]
    f2 = O.qval(cr, g, op_n, _abi.VAL_F2AVER, csf, acsf, dsi)[1]
    np.testing.assert_allclose(f2, np.sum(c ** 2 * amount) / n_real, rtol=1e-14)
    fa = O.qval(cr, g, op_n, _abi.VAL_FAVER, csf, acsf, dsi)[1]
    np.testing.assert_allclose(fa, np.sum(np.abs(c) * amount) / n_real, rtol=1e-14)
    # random phases: the caller's draw away from integer hkl
    rp = q(_abi.VAL_RANPH)
    hkl = g.hkl()
    off = ~np.all(np.abs(hkl[:, :, :, :] - np.rint(hkl)) < 1e-6, axis=0)
    np.testing.assert_allclose(rp[off], (rnd[off] - 0.5) * 360.0, rtol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("laver", [0, 1])
def test_qval_device_vs_oracle(ctx, laver):
    from diffusecode_gb300 import fourier as FR
    cr, g, op, csf, acsf, dsi, rnd = _case()
    r = FR.four_run(cr, g, op, ctx=ctx)
    for v in VALUES:
        rc, ref = O.qval(cr, g, op, v, r.csf, r.acsf, r.dsi, laver=bool(laver), rand=rnd)
        assert rc == 0
        out = FR.qval(cr, g, op, v, r, laver=bool(laver), rand=rnd, ctx=ctx)
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(ref).max()), err_msg=str(v))


@pytest.mark.gpu
def test_qval_pdf_values_rejected(ctx):
    from diffusecode_gb300 import fourier as FR
    cr, g, op, csf, acsf, dsi, rnd = _case()
    r = FR.four_run(cr, g, op, ctx=ctx)
    with pytest.raises(Exception) as e:
        FR.qval(cr, g, op, 15, r, ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_UNSUPPORTED
