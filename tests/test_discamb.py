"""DISCAMB aspherical form factors (four_run with diff_table RAD_DISC).

The reference sums the atoms per (type, symmetry operation, ADP type)
group (discus/prog/fourier_sup.f90:166-193, four_getatm_discamb :2259-2436)
and multiplies each group's sum at grid point h by its type's table for
that symmetry at nint(h) and by four_dbw (tcsf_form_discamb,
fourier_form.f90:63-102).  The tables come from the caller (read from a
DISCAMB .tsc file by discamb_read in the reference), here seeded random
complex values.

CPU: the oracle's restatement against known answers -- unit tables equal
the independent atom model with a unit form factor; a single atom at the
origin returns the table itself at nint(h), half-integers rounded away
from zero; its errors.  GPU: both engines and both phase modes against
the oracle with anisotropic Debye-Waller terms, box lots, the argument
checks, and the chi^2 gradient against central differences.  Intensity
tolerance as everywhere: max |I - I_ref| / (I_ref + N<|f|^2>) <= 1e-5,
with <|f|^2> the mean squared table magnitude.
"""
import ctypes as C

import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S

TOL = 1e-5
SYMS = [[1, 4], [1, 2, 5]]          # symmetry operation numbers per type
MAXHKL = (4, 3, 2)


def _grid(inc=(23, 19, 9)):
    return S.GridData.from_corners((-3.3, -2.7, -1.6), (3.3, -2.7, -1.6), (-3.3, 2.7, -1.6),
                                   (-3.3, -2.7, 1.6), inc=inc)


def _tables(seed=11, syms=SYMS, maxhkl=MAXHKL, const=None):
    rng = np.random.default_rng(seed)
    shape = tuple(2 * m + 1 for m in maxhkl)
    tabs = []
    for ys in syms:
        ts = []
        for _ in ys:
            if const is not None:
                ts.append(np.full(shape, const, np.complex128))
            else:
                ts.append(rng.uniform(0.5, 3.0, shape) * np.exp(2j * np.pi * rng.random(shape)))
        tabs.append(ts)
    return FR.DiscambTables(maxhkl, syms, tabs)


def _crystal(seed=5, anis=True, icc=(5, 4, 3)):
    cr, _ = S.small_lots_anis(seed=seed, icc=icc, anis=anis)
    rng = np.random.default_rng(seed + 100)
    isym = np.zeros(cr.natoms, np.int32)
    for t, ys in enumerate(SYMS, start=1):
        m = cr.iscat == t
        isym[m] = rng.choice(ys, size=int(m.sum()))
    cr.isym = isym
    if not anis:
        cr.ianis = None
    return cr


def _opts(tabs, **kw):
    op = K.opts(**kw)
    tabs.attach(op)
    return op


def _floor(cr, tabs):
    mean_f2 = np.mean([np.mean(np.abs(t) ** 2) for ts in tabs.tables for t in ts])
    return cr.n_scattering() * mean_f2


# ---------------------------------------------------------------------------- CPU (oracle)

def test_oracle_unit_tables_equal_unit_form_factor(oracle):
    cr = _crystal(anis=False)
    g = _grid()
    tabs = _tables(const=1.0)
    rc, csf_d, _, dsi_d, _ = oracle.four_run(cr, g, _opts(tabs, lxray=0, ldbw=0, phase=_abi.PHASE_EXACT64))
    assert rc == 0
    cr1 = cr.with_positions(cr.pos)
    cr1.scat = np.zeros_like(cr.scat)
    cr1.scat[:, 0] = 1.0
    cr1.occ = np.ones_like(cr.occ)
    rc, csf_i, _, dsi_i, _ = oracle.four_run(cr1, g, K.opts(lxray=0, ldbw=0, phase=_abi.PHASE_EXACT64))
    assert rc == 0
    np.testing.assert_allclose(csf_d, csf_i, rtol=0, atol=1e-12 * np.abs(csf_i).max())


def test_oracle_single_atom_returns_the_table(oracle):
    """One atom at the origin: S = 1, so csf(h) = table(nint(h)); the grid
    steps by 0.5, so half-integers are met and round away from zero."""
    cr = S.CrystalData(pos=np.zeros((1, 3)), iscat=np.array([1], np.int32), nscat=1, ncatoms=1, icc=(1, 1, 1),
                       rten=np.eye(3), scat=np.zeros((2, 11)), occ=np.ones(2), dw=np.zeros(2),
                       isym=np.array([3], np.int32))
    g = S.GridData.from_corners((-2.5, -1.5, 1.0), (2.5, -1.5, 1.0), (-2.5, 1.5, 1.0), inc=(11, 7, 1))
    tabs = _tables(syms=[[3]])
    rc, csf, _, _, _ = oracle.four_run(cr, g, _opts(tabs, ldbw=0, friedel=0, phase=_abi.PHASE_EXACT64))
    assert rc == 0
    h = g.hkl()
    want = np.empty(g.inc, np.complex128)
    for idx in np.ndindex(*g.inc):
        want[idx] = tabs.value(1, 0, h[(slice(None),) + idx])
    assert np.max(np.abs(csf - want)) <= 1e-13 * np.abs(want).max()
    assert tabs.value(1, 0, (-2.5, 0.5, 1.0)) == tabs.tables[0][0][-3 + 4, 1 + 3, 1 + 2]


def test_oracle_discamb_errors(oracle):
    cr = _crystal()
    tabs = _tables(maxhkl=(2, 3, 2))
    rc, *_ = oracle.four_run(cr, _grid(), _opts(tabs, ldbw=1))             # h = +-3.3 beyond +-2
    assert rc == _abi.DGPU_ERR_ARG
    rc, *_ = oracle.four_run(cr, _grid(), _opts(_tables(), ldbw=1, fave=1.0))
    assert rc == _abi.DGPU_ERR_UNSUPPORTED


# ---------------------------------------------------------------------------- GPU

CASES = {
    "direct-ref22": dict(engine=_abi.ENGINE_DIRECT, phase=_abi.PHASE_REF22, ldbw=1),
    "direct-exact": dict(engine=_abi.ENGINE_DIRECT, phase=_abi.PHASE_EXACT64, ldbw=1),
    "tc-exact": dict(engine=_abi.ENGINE_TC, phase=_abi.PHASE_EXACT64, ldbw=1),
    "tc-nodbw-iso": dict(engine=_abi.ENGINE_TC, phase=_abi.PHASE_EXACT64, ldbw=0, iso=True),
    "direct-box-lots": dict(engine=_abi.ENGINE_DIRECT, phase=_abi.PHASE_EXACT64, ldbw=1, ilots=_abi.LOT_BOX,
                            ls_xyz=(3, 2, 2), origins=[(1, 1, 1), (4, 3, 2)]),
    "tc-box-lots": dict(engine=_abi.ENGINE_TC, phase=_abi.PHASE_EXACT64, ldbw=1, ilots=_abi.LOT_BOX,
                        ls_xyz=(3, 2, 2), origins=[(1, 1, 1), (4, 3, 2)]),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_discamb_against_oracle(oracle, ctx, name):
    case = dict(CASES[name])
    iso = case.pop("iso", False)
    origins = case.pop("origins", None)
    if origins is not None:
        case["nlots"] = len(origins)
    cr = _crystal(anis=not iso)
    g = _grid()
    tabs = _tables()
    got = FR.four_run(cr, g, _opts(tabs, **case), ctx=ctx, lot_origins=origins)
    rc, csf, _, dsi, info = oracle.four_run(cr, g, _opts(tabs, **case), lot_origins=origins)
    assert rc == 0
    assert got.info.friedel_dim == info.friedel_dim
    rel = np.abs(got.dsi - dsi) / (dsi + _floor(cr, tabs))
    assert rel.max() <= TOL, rel.max()
    assert np.max(np.abs(got.csf - csf)) <= 3e-5 * np.abs(csf).max()


@pytest.mark.gpu
def test_discamb_argument_checks(ctx):
    cr = _crystal()
    g = _grid()
    with pytest.raises(Exception) as e:                 # grid beyond the tables
        FR.four_run(cr, g, _opts(_tables(maxhkl=(2, 3, 2)), ldbw=1), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_ARG
    bad = cr.with_positions(cr.pos)
    bad.isym = cr.isym.copy()
    bad.isym[np.flatnonzero(cr.iscat == 1)[0]] = 2      # type 1 has no table for symmetry 2
    with pytest.raises(Exception) as e:
        FR.four_run(bad, g, _opts(_tables(), ldbw=1), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_ARG
    with pytest.raises(Exception) as e:
        FR.four_run(cr, g, _opts(_tables(), ldbw=1, fave=1.0), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_UNSUPPORTED


@pytest.mark.gpu
def test_discamb_gradient_central_differences(ctx):
    """The adjoint multiplies by the same group factor as the forward pass, so
    the DISCAMB gradient follows; central differences (1e-4 A) of the GPU's
    own chi^2 on seeded atoms, CUDA-core engine."""
    from diffusecode_gb300.autograd import chi2_grad
    cr = _crystal()
    g = _grid()
    tabs = _tables()
    tgt = S.perturbed_copy(cr, 3, 0.05, 4.5, 0.1)
    tgt.isym = cr.isym
    op = _opts(tabs, ldbw=1, phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT)
    it = FR.four_run(tgt, g, op, ctx=ctx).dsi
    wt = 1.0 / (it + 1.0)
    c2, gp, go, _ = chi2_grad(cr, g, op, it, wt, ctx=ctx)
    h = 1e-4 / 4.5
    scale = np.abs(gp).max()
    rng = np.random.default_rng(2)
    for atom in rng.choice(np.flatnonzero(cr.iscat > 0), 5, replace=False):
        for k in range(3):
            vals = []
            for sgn in (1, -1):
                p = cr.pos.copy()
                p[atom, k] += sgn * h
                vals.append(chi2_grad(cr.with_positions(p), g, op, it, wt, ctx=ctx)[0])
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - gp[atom, k]) <= 1e-3 * scale + 1e-3 * abs(gp[atom, k])
