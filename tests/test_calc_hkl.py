"""calc_hkl core (fourier_sup.f90:3230-3549): the oracle against closed forms
(CPU) and the device against the oracle (GPU)."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import structures as S
from oracle import oracle as O


def _single_atom():
    scat = np.zeros((2, 11))
    scat[1, 0] = 2.5                                   # neutron scattering length
    cr = S.CrystalData(pos=np.zeros((1, 3)), iscat=np.array([1], np.int32), nscat=1, ncatoms=1, icc=(1, 1, 1),
                       rten=S.reciprocal_metric(4.0, 4.0, 4.0, 90, 90, 90), scat=scat, occ=np.ones(2),
                       dw=np.zeros(2))
    return cr


def test_oracle_calc_hkl_single_atom():
    cr = _single_atom()
    hkl = np.array([[1, 0, 0], [0, 2, -1], [-3, 1, 2], [0, 0, 0], [2, 2, 2]])
    op = K.opts(lxray=0, phase=_abi.PHASE_EXACT64, ldbw=0)
    rc, ic, sg, ph = O.calc_hkl(cr, op, hkl, scale=1.7)
    assert rc == 0
    want = np.where(np.all(hkl == 0, axis=1), 0.0, 2.5 ** 2 * 1.7)
    np.testing.assert_allclose(ic, want, rtol=1e-13)
    np.testing.assert_allclose(sg, np.sqrt(want), rtol=1e-13)
    np.testing.assert_allclose(ph, 0.0, atol=1e-9)
    # extinction: (1/(1 + 0.001 x F^2 lambda^3 / sin 2theta))^(1/4), F = 2.5
    lam, x = 0.71, 50.0
    rc, ic2, _, _ = O.calc_hkl(cr, op, hkl, scale=1.0, exti=x, rlambda=lam)
    ds = np.sqrt(np.einsum("ri,ij,rj->r", hkl.astype(float), cr.rten, hkl.astype(float)))
    tth = 2 * np.arcsin(0.5 * lam * ds)
    ext = np.where(ds > 0, (1 / (1 + 0.001 * x * 2.5 ** 2 * lam ** 3 / np.sin(np.where(ds > 0, tth, 1.0)))) ** 0.25, 0)
    np.testing.assert_allclose(ic2, (2.5 * ext) ** 2, rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_calc_hkl_vs_oracle(ctx, engine):
    from diffusecode_gb300 import fourier as FR
    cr, _ = S.small_lots_anis(anis=False)
    rng = np.random.default_rng(9)
    hkl = rng.integers(-4, 5, size=(60, 3))
    hkl[0] = 0
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine)
    rc, ic, sg, ph = O.calc_hkl(cr, op, hkl, scale=0.3, exti=20.0, rlambda=0.5)
    assert rc == 0
    gic, gsg, gph = FR.calc_hkl(cr, op, hkl, scale=0.3, exti=20.0, rlambda=0.5, ctx=ctx)
    np.testing.assert_allclose(gic, ic, rtol=2e-5, atol=2e-5 * ic.max())
    np.testing.assert_allclose(gsg, sg, rtol=1e-5, atol=1e-5 * sg.max())
    big = ic > 1e-3 * ic.max()                          # phases of the non-vanishing reflections
    d = np.abs(((gph - ph) + 180) % 360 - 180)
    assert np.all(d[big] < 1e-2)
