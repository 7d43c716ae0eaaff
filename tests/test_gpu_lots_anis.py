"""Anisotropic ADPs and lots on the GPU against the oracle.

Cases: (type, ADP type) groups with the anisotropic Debye-Waller term
(four_dbwtab, tcsf_form_aniso), box and ellipsoid lots with periodic wrap,
interstitial atoms, lot_all over a non-periodic csize and <F> with the lot
lattice (fourier_sup.f90:136-277, 1194-1357, 1806-2140).  Intensities are
compared as max |I - I_ref| / (I_ref + N<|f|^2>) <= 1e-5 (both engines),
csf within 3e-5 of max |csf| + max |acsf| (its size before the <F>
subtraction), acsf within 3e-5 of its maximum.
"""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S

pytestmark = pytest.mark.gpu
TOL = 1e-5

CASES = {
    "anis": dict(anis=True, opts=dict(ldbw=1)),
    "anis-nodbw": dict(anis=True, opts=dict(ldbw=0, fave=1.0)),
    "anis-box-aver": dict(anis=True, opts=dict(ldbw=1, ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), fave=1.0),
                          origins=[(1, 1, 1), (4, 3, 2), (5, 4, 3)]),
    "iso-eli-all-nonperiodic": dict(anis=False, opts=dict(ilots=_abi.LOT_ELI, ls_xyz=(3, 3, 2), lot_all=1,
                                                          lperiod=0, fave=0.5)),
    "anis-eli-origins": dict(anis=True, opts=dict(ldbw=1, ilots=_abi.LOT_ELI, ls_xyz=(4, 3, 3), diff_scale=2.5),
                             origins=[(2, 1, 1), (5, 4, 1)]),
    "iso-box-all": dict(anis=False, opts=dict(ilots=_abi.LOT_BOX, ls_xyz=(2, 2, 1), lot_all=1, fave=1.0)),
}


def _cells(cr, op, seed=3):
    if not 0 < op.fave < 1:
        return None
    cs = [cr.icc[k] if op.lperiod else max(1, cr.icc[k] - op.ls_xyz[k] + 1) for k in range(3)]
    return (np.random.default_rng(seed).random(cs) < op.fave).astype(np.uint8)


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC], ids=["direct", "tc"])
@pytest.mark.parametrize("form", [_abi.FORM_TABLE, _abi.FORM_ANALYTIC], ids=["table", "analytic"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_lots_anis_vs_oracle(oracle, ctx, name, form, engine):
    case = CASES[name]
    cr, g = S.small_lots_anis(anis=case["anis"])
    op = K.opts(phase=_abi.PHASE_EXACT64, form=form, engine=engine, **case["opts"])
    cells = _cells(cr, op)
    origins = case.get("origins")
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op, aver_cells=cells, lot_origins=origins)
    r = FR.four_run(cr, g, op, ctx=ctx, aver_cells=cells, lot_origins=origins)
    assert rc == 0 and r.status == 0
    assert r.info.engine_used == engine
    assert r.info.friedel_dim == info.friedel_dim == 1
    floor = K.incoherent_floor(cr, g, K.opts(ldbw=0))
    assert K.rel_err(r.dsi, dsi, floor) <= TOL
    # csf = F - <F>: the error scales with |F| before the subtraction
    assert np.abs(r.csf - csf).max() <= 3e-5 * (np.abs(csf).max() + np.abs(acsf).max())
    if op.fave:
        assert np.abs(r.acsf - acsf).max() <= 3e-5 * np.abs(acsf).max()
        assert r.info.ncell == info.ncell
    assert r.info.pairs == info.pairs


@pytest.mark.parametrize("name", ["anis", "anis-box-aver", "iso-eli-all-nonperiodic"])
def test_lots_anis_ref22(oracle, ctx, name):
    """The reference's integer phases (CUDA-core engine) on the same cases."""
    case = CASES[name]
    cr, g = S.small_lots_anis(anis=case["anis"])
    op = K.opts(phase=_abi.PHASE_REF22, engine=_abi.ENGINE_DIRECT, **case["opts"])
    cells = _cells(cr, op)
    origins = case.get("origins")
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op, aver_cells=cells, lot_origins=origins)
    r = FR.four_run(cr, g, op, ctx=ctx, aver_cells=cells, lot_origins=origins)
    assert rc == 0 and r.status == 0
    assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, K.opts(ldbw=0))) <= TOL


def test_many_lots_chunked(oracle, ctx, monkeypatch):
    """More (lot, group) pairs than one engine launch takes (63): 40 lots of
    3 groups run in two chunks, counted together in one batch, or (a batch
    limit of one slot) as one batch each, with the same result."""
    cr, g = S.small_lots_anis(anis=True, icc=(6, 5, 4), inc=(9, 9, 5))
    rng = np.random.default_rng(11)
    origins = np.stack([rng.integers(1, cr.icc[k] + 1, size=40) for k in range(3)], axis=1)
    for engine in (_abi.ENGINE_DIRECT, _abi.ENGINE_TC):
        op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine, ilots=_abi.LOT_BOX, ls_xyz=(3, 3, 2), fave=1.0)
        rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op, lot_origins=origins)
        r = FR.four_run(cr, g, op, ctx=ctx, lot_origins=origins)
        assert rc == 0 and r.status == 0
        assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, K.opts(ldbw=0))) <= TOL
        assert np.abs(r.csf - csf).max() <= 3e-5 * (np.abs(csf).max() + np.abs(acsf).max())
        monkeypatch.setenv("DGPU_LOT_BATCH_SLOTS", "1")
        r1 = FR.four_run(cr, g, op, ctx=ctx, lot_origins=origins)
        monkeypatch.delenv("DGPU_LOT_BATCH_SLOTS")
        assert r1.status == 0 and r1.info.pairs == r.info.pairs
        assert np.array_equal(r1.dsi, r.dsi) and np.array_equal(r1.csf, r.csf)


def _status(fn):
    try:
        return fn().status
    except Exception as e:          # the host wrapper raises on errors
        return getattr(e, "code", None)


def test_lot_and_adp_argument_errors(ctx):
    cr, g = S.small_lots_anis(anis=True)
    op = K.opts(ilots=_abi.LOT_BOX, ls_xyz=(9, 1, 1))
    assert _status(lambda: FR.four_run(cr, g, op, ctx=ctx, lot_origins=[(1, 1, 1)])) == _abi.DGPU_ERR_ARG
    op = K.opts(ilots=_abi.LOT_BOX, ls_xyz=(2, 2, 2))
    assert _status(lambda: FR.four_run(cr, g, op, ctx=ctx, lot_origins=[(0, 1, 1)])) == _abi.DGPU_ERR_ARG
    bad = cr.ianis.copy()
    k = int(np.flatnonzero(cr.iscat > 0)[0])
    bad[k] = 9
    cr.ianis = bad
    assert _status(lambda: FR.four_run(cr, g, K.opts(), ctx=ctx)) == _abi.DGPU_ERR_ARG


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC], ids=["direct", "tc"])
def test_gradient_anisotropic(oracle, ctx, engine):
    """chi^2 gradient of an anisotropic crystal: the adjoint weights carry
    each group's Debye-Waller term."""
    from diffusecode_gb300.autograd import chi2_grad
    cr, g = S.small_lots_anis(anis=True, inc=(11, 9, 5))
    cr.atom_occ = np.linspace(0.9, 1.1, cr.natoms).astype(np.float32)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine, ldbw=1)
    tgt = S.perturbed_copy(cr, 3, 0.05, 4.5, 0.1)
    tgt.ianis, tgt.anis_full, tgt.ar = cr.ianis, cr.anis_full, cr.ar
    it = FR.four_run(tgt, g, K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT, ldbw=1), ctx=ctx).dsi
    wt = 1.0 / (it + 1.0)
    c2, gp, go, _ = chi2_grad(cr, g, op, it, wt, ctx=ctx)
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, op, it, wt)
    assert abs(c2 - oc2) <= 1e-4 * oc2
    assert np.max(np.abs(gp - ogp)) <= 2e-4 * np.abs(ogp).max()
    assert np.max(np.abs(go - ogo)) <= 2e-4 * np.abs(ogo).max()


def test_batch_member_path_for_lots_and_average(ctx):
    """Options outside the population graph (lots, <F>) run member by member
    through dgpu_four_run / dgpu_chi2_grad: the same intensities and chi^2
    as those single-crystal calls, the same gradients to FP64 rounding, and
    no graph."""
    from diffusecode_gb300.autograd import chi2_grad
    pop = [S.small_lots_anis(anis=a, icc=icc, inc=(9, 9, 3)) for a, icc in ((True, (6, 5, 4)), (False, (5, 5, 5)))]
    crs, grids = [p[0] for p in pop], [p[1] for p in pop]
    for op in (K.opts(phase=_abi.PHASE_EXACT64, ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), lot_all=1, ldbw=1),
               K.opts(phase=_abi.PHASE_EXACT64, fave=1.0, ldbw=1)):
        targets = [FR.four_run(c, g, K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT), ctx=ctx).dsi
                   for c, g in zip(crs, grids)]
        weights = [1.0 / (t + 1.0) for t in targets]
        dsi, c2, gp, go, ms = FR.batch_run(crs, grids, op, targets=targets, weights=weights, ctx=ctx)
        assert ms > 0 and FR.batch_graph_nodes(ctx=ctx) == (0, 0)
        for k, (c, g) in enumerate(zip(crs, grids)):
            one = FR.four_run(c, g, op, ctx=ctx).dsi
            np.testing.assert_array_equal(dsi[k], one)
            oc2, ogp, ogo, _ = chi2_grad(c, g, op, targets[k], weights[k], ctx=ctx)
            assert c2[k] == oc2
            # the lot gradient adds per-atom sums atomically: same values to FP64 rounding
            np.testing.assert_allclose(gp[k], ogp, rtol=1e-12, atol=1e-12 * np.abs(ogp).max())
            np.testing.assert_allclose(go[k], ogo, rtol=1e-12, atol=1e-12 * np.abs(ogo).max())


def test_lots_tc_several_slices(oracle, ctx):
    """Lots on the tensor-core engine with several K slices per (lot, group)
    pair (tc_kslice = 64 atoms; 2 groups x 3 slices = 6 partials per lot,
    the lot combine specialised for up to 8): its slices of a group are added
    before the group product, as the generic combine does; against the
    oracle and the CUDA-core engine."""
    cr, g = S.small_lots_anis(anis=False, icc=(10, 8, 6), inc=(9, 9, 5))
    origins = [(1, 1, 1), (4, 3, 2), (9, 7, 5)]
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC, ilots=_abi.LOT_BOX, ls_xyz=(8, 6, 4), nlots=3,
                tc_kslice=64)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op, lot_origins=origins)
    r = FR.four_run(cr, g, op, ctx=ctx, lot_origins=origins)
    assert rc == 0 and r.status == 0 and r.info.engine_used == _abi.ENGINE_TC
    floor = K.incoherent_floor(cr, g, K.opts(ldbw=0))
    assert K.rel_err(r.dsi, dsi, floor) <= TOL
    d = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT, ilots=_abi.LOT_BOX,
                                  ls_xyz=(8, 6, 4), nlots=3), ctx=ctx, lot_origins=origins)
    assert K.rel_err(r.dsi, d.dsi, floor) <= TOL
