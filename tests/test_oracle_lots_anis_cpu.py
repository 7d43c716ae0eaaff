"""The oracle's lots and anisotropic ADPs against an independent numpy
restatement (CPU only).

four_run's lot loop (discus/prog/fourier_sup.f90:136-277), four_getatm_anis
(:1975-2140), four_nanis (:4294-4326), four_dbwtab (:2747-2855),
tcsf_form_aniso (fourier_form.f90:106-143), four_aver over csize with the
lot lattice of four_getav (:1194-1357, 2440-2510) are restated here with
plain loops and numpy exp(2 pi i h.x) sums over the full grid (no Friedel
halving), and compared with the C oracle, which halves and mirrors as the
reference does.  Neutron scattering lengths (lxray = 0) keep cfact free of
the sin(theta)/lambda table, so the comparison isolates the atom gathering,
the group factors and the normalisation.
"""
import math

import numpy as np
import pytest

from diffusecode_gb300 import _abi
from diffusecode_gb300.structures import small_lots_anis
from oracle import oracle as O


def _hkl(grid):
    i, j, k = np.meshgrid(*(np.arange(n) for n in grid.inc), indexing="ij")
    return (grid.eck[:, 0][None, None, None, :] + i[..., None] * grid.vi[:, 0] + j[..., None] * grid.vi[:, 1]
            + k[..., None] * grid.vi[:, 2])


def _csize(cr, op):
    ls = list(op.ls_xyz)
    return [cr.icc[k] if op.lperiod else max(1, cr.icc[k] - ls[k] + 1) for k in range(3)]


def _in_lot(op, d):
    if op.ilots != _abi.LOT_ELI:
        return True
    s = 0.0
    for k in range(3):
        x0 = op.ls_xyz[k] / 2.0
        s += (d[k] - x0 + 0.5) ** 2 / x0 ** 2
    return s <= 1.0


def _lot_atoms(cr, op, lbeg, t, a):
    """four_getatm_anis for one (type, ADP) and one lot, as plain loops."""
    icc, nc = cr.icc, cr.ncatoms
    cr_end = nc * icc[0] * icc[1] * icc[2]
    sel = lambda i: cr.iscat[i] == t and (a == 0 or cr.ianis[i] == a)
    out, ncell = [], 0
    if op.ilots not in (_abi.LOT_BOX, _abi.LOT_ELI):
        return [cr.pos[i] for i in range(cr.natoms) if sel(i)], icc[0] * icc[1] * icc[2]
    for kk in range(op.ls_xyz[2]):
        for jj in range(op.ls_xyz[1]):
            for ii in range(op.ls_xyz[0]):
                d = (ii, jj, kk)
                icell, off = [0] * 3, [0.0] * 3
                for k in range(3):
                    icell[k] = d[k] + lbeg[k]
                    off[k] = cr.dim0[k] + lbeg[k] - 1
                    if icell[k] > icc[k]:
                        icell[k] -= icc[k]
                        off[k] -= icc[k]
                if not _in_lot(op, d):
                    continue
                ncell += 1
                for s in range(nc):
                    ia = ((icell[2] - 1) * icc[0] * icc[1] + (icell[1] - 1) * icc[0] + icell[0] - 1) * nc + s
                    if ia < cr.natoms and sel(ia):
                        out.append(cr.pos[ia] - np.asarray(off))
                jc = [icell[k] + int(round(cr.dim_lo[k])) - 1 for k in range(3)]
                for ir in range(cr_end, cr.natoms):
                    if all(math.trunc(cr.pos[ir][k]) == jc[k] for k in range(3)) and sel(ir):
                        out.append(cr.pos[ir] - np.asarray(off))
    return out, ncell


def _strucf(h, x):
    if len(x) == 0:
        return np.zeros(h.shape[:-1], complex)
    x = np.asarray(x)
    return np.exp(2j * np.pi * np.tensordot(h, x.T, axes=([3], [0]))).sum(-1)


def _numpy_four_run(cr, grid, op, origins=None, aver_cells=None):
    h = _hkl(grid)
    cf = {t: cr.occ[t] * cr.scat[t, 0] for t in range(1, cr.nscat + 1)}       # lxray = 0

    def dbw(a):
        u, ar = cr.anis_full[a - 1], cr.ar
        arg = (h[..., 0] ** 2 * ar[0] ** 2 * u[0] + h[..., 1] ** 2 * ar[1] ** 2 * u[1]
               + h[..., 2] ** 2 * ar[2] ** 2 * u[2] + 2 * h[..., 1] * h[..., 2] * ar[1] * ar[2] * u[3]
               + 2 * h[..., 0] * h[..., 2] * ar[0] * ar[2] * u[4] + 2 * h[..., 0] * h[..., 1] * ar[0] * ar[1] * u[5])
        return np.exp(-2 * np.pi ** 2 * arg) if op.ldbw else 1.0

    lots = op.ilots in (_abi.LOT_BOX, _abi.LOT_ELI)
    cs = _csize(cr, op)
    acsf = np.zeros(h.shape[:-1], complex)
    if op.fave:
        ncell = 0
        for t in range(1, cr.nscat + 1):
            xs = []
            for ii in range(cs[0]):
                for jj in range(cs[1]):
                    for kk in range(cs[2]):
                        if op.fave < 1 and not aver_cells[ii, jj, kk]:
                            continue
                        ncell += 1
                        c = ii + cr.icc[0] * (jj + cr.icc[1] * kk)
                        for s in range(cr.ncatoms):
                            ia = c * cr.ncatoms + s
                            if ia < cr.natoms and cr.iscat[ia] == t:
                                xs.append(cr.pos[ia] - np.array([ii, jj, kk]) - np.asarray(cr.dim0))
            acsf += cf[t] * _strucf(h, xs)
        ncell //= cr.nscat
        if not lots:
            lat = [np.array([i, j, k]) + np.asarray(cr.dim0) for i in range(cr.icc[0]) for j in range(cr.icc[1])
                   for k in range(cr.icc[2])]
        else:
            lat = [np.array([i, j, k], float) for k in range(op.ls_xyz[2]) for j in range(op.ls_xyz[1])
                   for i in range(op.ls_xyz[0]) if _in_lot(op, (i, j, k))]
        acsf = acsf * _strucf(h, lat) / ncell
    if not lots:
        origins = [(1, 1, 1)]
    elif op.lot_all:
        origins = [(i + 1, j + 1, k + 1) for k in range(cs[2]) for j in range(cs[1]) for i in range(cs[0])]
    dsi = np.zeros(h.shape[:-1])
    lcell = 0
    for lbeg in origins:
        F = np.zeros(h.shape[:-1], complex)
        for t in range(1, cr.nscat + 1):
            alist = [0]
            if cr.is_anis:
                alist = list(dict.fromkeys(int(a) for a, s in zip(cr.ianis, cr.iscat) if s == t))
            for a in alist:
                xs, lcell = _lot_atoms(cr, op, lbeg, t, a)
                if xs:
                    F += cf[t] * (dbw(a) if a else 1.0) * _strucf(h, xs)
        F -= acsf
        dsi += np.abs(F) ** 2
    if len(origins) != 1:
        dsi *= cr.icc[0] * cr.icc[1] * cr.icc[2] / (lcell * len(origins))
    return F * math.sqrt(op.diff_scale), acsf, dsi * op.diff_scale


CASES = {
    "anis-nolots": dict(anis=True, opts=dict(ldbw=1)),
    "anis-box-aver": dict(anis=True, opts=dict(ldbw=1, ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), fave=1.0),
                          origins=[(1, 1, 1), (4, 3, 2), (5, 4, 3)]),
    "iso-eli-all-nonperiodic": dict(anis=False, opts=dict(ilots=_abi.LOT_ELI, ls_xyz=(3, 3, 2), lot_all=1,
                                                          lperiod=0, fave=0.5)),
    "anis-eli-origins": dict(anis=True, opts=dict(ldbw=1, ilots=_abi.LOT_ELI, ls_xyz=(4, 3, 3), diff_scale=2.5),
                             origins=[(2, 1, 1), (5, 4, 1)]),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_lots_anis_vs_numpy(name):
    case = CASES[name]
    cr, grid = small_lots_anis(anis=case["anis"], lxray=False)
    op = _abi.default_opts(lxray=0, phase=_abi.PHASE_EXACT64, **case["opts"])
    rng = np.random.default_rng(3)
    cells = None
    if 0 < op.fave < 1:
        cells = (rng.random(_csize(cr, op)) < op.fave).astype(np.uint8)
    origins = case.get("origins")
    rc, csf, acsf, dsi, info = O.four_run(cr, grid, op, aver_cells=cells, lot_origins=origins)
    assert rc == 0
    assert info.friedel_dim == 1
    ref_csf, ref_acsf, ref_dsi = _numpy_four_run(cr, grid, op, origins, cells)
    scale = np.abs(ref_dsi).max()
    assert np.abs(dsi - ref_dsi).max() <= 1e-10 * scale
    assert np.abs(acsf - ref_acsf).max() <= 1e-10 * max(1.0, np.abs(ref_acsf).max())
    assert np.abs(csf - ref_csf).max() <= 1e-10 * max(1.0, np.abs(ref_csf).max())


def test_oracle_isotropic_adp_equals_iso_path():
    """U_ij = U delta_ij on an orthogonal cell is the isotropic B = 8 pi^2 U:
    the anisotropic group factor equals cfact's exp(-B s^2) at the exact
    sin(theta)/lambda (ANALYTIC form)."""
    cr, grid = small_lots_anis(anis=True)
    U = 0.012
    cr.anis_full = np.tile([U, U, U, 0.0, 0.0, 0.0], (3, 1))
    cr_iso, _ = small_lots_anis(anis=False)
    cr_iso.dw[1:] = 8 * np.pi ** 2 * U
    op = _abi.default_opts(ldbw=1, form=_abi.FORM_ANALYTIC, phase=_abi.PHASE_EXACT64, fave=1.0)
    rc, csf_a, acsf_a, dsi_a, _ = O.four_run(cr, grid, op)
    op2 = _abi.default_opts(ldbw=1, form=_abi.FORM_ANALYTIC, phase=_abi.PHASE_EXACT64)
    rc2, csf_i, _, dsi_i, _ = O.four_run(cr_iso, grid, op2)
    assert rc == 0 and rc2 == 0
    # <F> of an anisotropic crystal carries no Debye-Waller term (four_aver
    # calls four_strucf with the isotropic form and cfact has sb = occ)
    op3 = _abi.default_opts(ldbw=0, form=_abi.FORM_ANALYTIC, phase=_abi.PHASE_EXACT64, fave=1.0)
    _, _, acsf_nodw, _, _ = O.four_run(cr_iso, grid, op3)
    assert np.abs(acsf_a - acsf_nodw).max() <= 1e-12 * np.abs(acsf_nodw).max()
    # without <F>: the same intensities
    op4 = _abi.default_opts(ldbw=1, form=_abi.FORM_ANALYTIC, phase=_abi.PHASE_EXACT64)
    _, _, _, dsi_a0, _ = O.four_run(cr, grid, op4)
    assert np.abs(dsi_a0 - dsi_i).max() <= 1e-12 * dsi_i.max()


def test_oracle_single_lot_whole_crystal_equals_lot_off():
    """One box lot of the whole periodic crystal (lbeg = 1) is the crystal
    shifted by dim0: the same |F|^2 (no interstitials, nlots = 1)."""
    cr, grid = small_lots_anis(anis=False, nextra=0)
    op = _abi.default_opts(phase=_abi.PHASE_EXACT64)
    rc, _, _, dsi0, _ = O.four_run(cr, grid, op)
    op2 = _abi.default_opts(phase=_abi.PHASE_EXACT64, ilots=_abi.LOT_BOX, ls_xyz=cr.icc)
    rc2, _, _, dsi1, _ = O.four_run(cr, grid, op2, lot_origins=[(1, 1, 1)])
    assert rc == 0 and rc2 == 0
    assert np.abs(dsi1 - dsi0).max() <= 1e-11 * dsi0.max()


def test_oracle_lot_argument_checks():
    cr, grid = small_lots_anis(anis=False)
    bad = [dict(ilots=_abi.LOT_BOX, ls_xyz=(6, 1, 1)), dict(ilots=_abi.LOT_BOX, ls_xyz=(0, 1, 1)),
           dict(ilots=7)]
    for kw in bad:
        op = _abi.default_opts(**kw)
        rc, *_ = O.four_run(cr, grid, op, lot_origins=[(1, 1, 1)])
        assert rc == _abi.DGPU_ERR_ARG, kw
    op = _abi.default_opts(ilots=_abi.LOT_BOX, ls_xyz=(2, 2, 2))
    rc, *_ = O.four_run(cr, grid, op, lot_origins=[(5, 4, 4)])
    assert rc == _abi.DGPU_ERR_ARG
