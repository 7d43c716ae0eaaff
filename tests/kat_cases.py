"""Crystals and grids of the known-answer fixtures in tests/golden/."""
import json
import os

import numpy as np

from diffusecode_gb300 import _abi
from diffusecode_gb300.structures import CrystalData, GridData

HERE = os.path.dirname(os.path.abspath(__file__))
KAT = np.load(os.path.join(HERE, "golden", "kat.npz"))
with open(os.path.join(HERE, "golden", "lmn.json")) as f:
    LMN_CASES = json.load(f)


def _grid(eck, vi, inc):
    e = np.zeros((3, 4))
    e[:, 0] = eck
    return GridData(eck=e, vi=np.asarray(vi, dtype=np.float64).T, inc=tuple(int(x) for x in inc))


def _crystal(pos, iscat, nscat, icc=(1, 1, 1), ncatoms=1):
    scat = KAT["scat"][: nscat + 1].copy()
    occ = np.ones(nscat + 1)
    dw = np.full(nscat + 1, 0.5)
    return CrystalData(pos=np.asarray(pos, dtype=np.float64).reshape(-1, 3), iscat=np.asarray(iscat, np.int32),
                       nscat=nscat, ncatoms=ncatoms, icc=icc, rten=KAT["rten_cubic4"], scat=scat, occ=occ, dw=dw)


def single_atom():
    cr = _crystal([[0.0, 0.0, 0.0]], [1], 1)
    g = _grid(KAT["single_atom_eck"], KAT["single_atom_vi"], KAT["single_atom_inc"])
    return cr, g, KAT["single_atom_csf"], KAT["single_atom_istl"]


def laue():
    pos = KAT["laue_pos"]
    icc = tuple(int(x) for x in KAT["laue_icc"])
    cr = _crystal(pos, np.ones(pos.shape[0], np.int32), 1, icc=icc, ncatoms=1)
    g = _grid(KAT["laue_eck"], KAT["laue_vi"], KAT["laue_inc"])
    return cr, g, KAT["laue_csf"]


def two_atoms():
    cr = _crystal(KAT["two_pos"], [1, 2], 2)
    g = _grid(KAT["two_eck"], KAT["two_vi"], KAT["two_inc"])
    return cr, g, KAT["two_csf"]


def opts(**kw):
    base = dict(ldbw=1)
    base.update(kw)
    return _abi.default_opts(**base)


def rel_err(i_test, i_ref, floor):
    """max |I - I_ref| / (I_ref + floor): intensity error normalised by the
    point's intensity plus the incoherent level N<|f|^2>."""
    return float(np.max(np.abs(i_test - i_ref) / (i_ref + floor)))


def incoherent_floor(cr, grid, opts_):
    """N <|f|^2> at each grid point from the analytic form factor (EXACT)."""
    h = grid.hkl()
    s2 = np.einsum("a...,ab,b...->...", h, cr.rten, h) / 4.0
    tot = np.zeros(grid.inc)
    for t in range(1, cr.nscat + 1):
        n_t = np.count_nonzero(cr.iscat == t)
        if n_t == 0:
            continue
        sc = cr.scat[t]
        f = sc[0] + sum(sc[2 * i - 1] * np.exp(-sc[2 * i] * s2) for i in range(1, opts_.power + 1))
        sb = np.exp(-cr.dw[t] * s2) * cr.occ[t] if opts_.ldbw else cr.occ[t]
        tot += n_t * (sb * f) ** 2
    return tot
