"""The oracle's FP64 chi^2 gradient with <F> subtracted (four_aver), on CPU.

With fave > 0 every atom of a selected cell also enters A(h) = L(h)/ncell
sum_t c_t(h) S_t^fold(h) at its position moved into one cell, so it carries
a second gradient term.  The restatement is pinned two ways: its chi^2
equals sum wt (dsi - it)^2 of the oracle's own four_run (the forward
restatement, checked against the reference's golden vectors elsewhere),
and its gradient equals central finite differences of that chi^2 (step
1e-6 lattice units; the truncation error is ~1e-12 relative).
"""
import copy

import numpy as np
import pytest

from diffusecode_gb300 import _abi
from diffusecode_gb300 import structures as S
from oracle import oracle as O


def _case(fave):
    cr0, g = S.rocksalt_volume(cells=(3, 3, 3), inc=7, step=0.37)
    cr = S.perturbed_copy(cr0, 5, 0.04, 5.64, 0.1)
    tgt = S.perturbed_copy(cr0, 3, 0.05, 5.64, 0.1)
    cells = None
    if fave < 1.0:
        cells = (np.random.default_rng(1).random(27) < 0.5).astype(np.uint8).reshape((3, 3, 3), order="F")
    op = _abi.default_opts(ldbw=1, phase=_abi.PHASE_EXACT64, fave=fave)
    rc, csf, acsf, it, info = O.four_run(tgt, g, op, aver_cells=cells)
    assert rc == 0 and info.ncell == (27 if cells is None else int(cells.sum()))
    return cr, g, it, 1.0 / (it + 1.0), cells


def _chi2(cr, g, fave, it, wt, cells):
    op = _abi.default_opts(ldbw=1, phase=_abi.PHASE_EXACT64, fave=fave)
    return O.chi2_grad(cr, g, op, it, wt, aver_cells=cells)


@pytest.mark.parametrize("fave", [1.0, 0.5])
def test_average_gradient_matches_forward_and_differences(fave):
    cr, g, it, wt, cells = _case(fave)
    c2, gp, go = _chi2(cr, g, fave, it, wt, cells)
    op = _abi.default_opts(ldbw=1, phase=_abi.PHASE_EXACT64, fave=fave)
    rc, csf, acsf, dsi, info = O.four_run(cr, g, op, aver_cells=cells)
    assert np.abs(acsf).max() > 0.1 * np.abs(csf + acsf).max()      # <F> is a large part of F
    assert abs(c2 - np.sum(wt * (dsi - it) ** 2)) <= 1e-12 * c2
    eps = 1e-6
    sel = np.repeat(np.ones(27, bool) if cells is None else cells.reshape(-1, order="F").astype(bool), 8)
    atoms = [0, 101, 190] + ([int(np.flatnonzero(~sel)[0])] if not sel.all() else [])
    for a in atoms:
        for k in range(3):
            vals = []
            for sgn in (1, -1):
                c = copy.deepcopy(cr)
                c.pos[a, k] += sgn * eps
                vals.append(_chi2(c, g, fave, it, wt, cells)[0])
            fd = (vals[0] - vals[1]) / (2 * eps)
            assert abs(fd - gp[a, k]) <= 1e-8 * np.abs(gp).max()
        vals = []
        for sgn in (1, -1):
            c = copy.deepcopy(cr)
            c.atom_occ = np.asarray(c.atom_occ, np.float32).copy()
            c.atom_occ[a] += np.float32(sgn * 2.0 ** -10)       # exact in float32
            vals.append(_chi2(c, g, fave, it, wt, cells)[0])
        fd = (vals[0] - vals[1]) / (2 * 2.0 ** -10)
        # chi2 is quartic in the occupancy: the central difference is exact up to h^2 |d3 chi2|
        assert abs(fd - go[a]) <= 1e-6 * np.abs(go).max()


def test_average_term_changes_the_gradient():
    """The <F> term is not negligible: the gradient with fave = 1 differs
    from the one without subtraction by more than 10 % of its scale."""
    cr, g, it, wt, _ = _case(1.0)
    _, gp1, _ = _chi2(cr, g, 1.0, it, wt, None)
    _, gp0, _ = _chi2(cr, g, 0.0, it, wt, None)
    assert np.abs(gp1 - gp0).max() > 0.1 * np.abs(gp1).max()


LOT_CASES = {
    "box": dict(anis=False, opts=dict(ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), nlots=3), origins=[(1, 1, 1), (4, 3, 2), (5, 4, 3)]),
    "box-aver-anis": dict(anis=True, opts=dict(ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), nlots=3, fave=1.0),
                          origins=[(1, 1, 1), (4, 3, 2), (5, 4, 3)]),
    "eli-all": dict(anis=False, opts=dict(ilots=_abi.LOT_ELI, ls_xyz=(3, 3, 2), lot_all=1, lperiod=0)),
}


@pytest.mark.parametrize("name", sorted(LOT_CASES))
def test_lots_gradient_matches_forward_and_differences(name):
    """With lots: the oracle's chi^2 equals that of its own four_run with the
    same lots, and its gradient equals central differences (atoms in several
    lots, wrapped lots, interstitial atoms, <F> of the lot lattice)."""
    case = LOT_CASES[name]
    cr, g = S.small_lots_anis(anis=case["anis"], icc=(5, 4, 3), inc=(7, 7, 3))
    origins = case.get("origins")

    def opts():
        return _abi.default_opts(ldbw=1, phase=_abi.PHASE_EXACT64, **case["opts"])

    def with_origins(op):
        keep = None
        if origins is not None:
            keep = np.ascontiguousarray(np.asarray(origins, np.int32).reshape(-1, 3))
            op.lot_origins = _abi.iptr(keep)
        return op, keep

    tgt = cr.with_positions(cr.pos + np.random.default_rng(2).normal(0, 0.01, cr.pos.shape))
    rc, _, _, it, info = O.four_run(tgt, g, opts(), lot_origins=origins)
    assert rc == 0
    wt = 1.0 / (it + 1.0)
    op, keep = with_origins(opts())
    c2, gp, go = O.chi2_grad(cr, g, op, it, wt)
    rc, _, _, dsi, _ = O.four_run(cr, g, opts(), lot_origins=origins)
    assert abs(c2 - np.sum(wt * (dsi - it) ** 2)) <= 1e-11 * c2
    eps = 1e-6
    for a in [0, 7, cr.natoms - 2]:
        if cr.iscat[a] == 0:
            continue
        for k in range(3):
            vals = []
            for sgn in (1, -1):
                c = copy.deepcopy(cr)
                c.pos[a, k] += sgn * eps
                op, keep = with_origins(opts())
                vals.append(O.chi2_grad(c, g, op, it, wt)[0])
            fd = (vals[0] - vals[1]) / (2 * eps)
            assert abs(fd - gp[a, k]) <= 1e-7 * np.abs(gp).max()
