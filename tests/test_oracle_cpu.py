"""The CPU oracle against the closed-form known answers (parity unpinned by
the reference itself; see oracle/discus_oracle.h)."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import structures as S


@pytest.mark.parametrize("case", K.LMN_CASES, ids=[c["name"] for c in K.LMN_CASES])
def test_lmn_known_decompositions(oracle, case):
    eck = np.zeros((3, 4))
    eck[:, 0] = case["eck"]
    vi = np.asarray(case["vi"], dtype=np.float64).T
    rc, lmn, off = oracle.fourier_lmn(eck, vi, case["inc"])
    assert rc == case["rc"]
    if rc == 0:
        assert list(lmn) == case["lmn"]
        np.testing.assert_allclose(off.T, np.asarray(case["off"]), atol=1e-15)


def test_lmn_reconstructs_corner(oracle):
    """eck(:,1) = sum lmn(1:3) vi + sum lmn(4:6) off for generic 2D/3D grids."""
    rng = np.random.Generator(np.random.PCG64(7))
    for inc in [(11, 13, 1), (9, 7, 5)]:
        for _ in range(20):
            vi = np.zeros((3, 3))
            vi[:, 0] = np.round(rng.uniform(-0.3, 0.3, 3), 3)
            vi[:, 1] = np.round(rng.uniform(-0.3, 0.3, 3), 3)
            if inc[2] > 1:
                vi[:, 2] = np.round(rng.uniform(-0.3, 0.3, 3), 3)
            eck = np.zeros((3, 4))
            eck[:, 0] = np.round(rng.uniform(-5, 5, 3), 3)
            rc, lmn, off = oracle.fourier_lmn(eck, vi, inc)
            assert rc == 0
            rec = vi @ lmn[:3] + off @ lmn[3:]
            if inc[2] > 1:     # full 3D: corner must be reproduced exactly
                np.testing.assert_allclose(rec, eck[:, 0], atol=1e-9)


def test_cexpt_table(oracle):
    cex = oracle.cexpt()
    k = np.arange(65536)
    np.testing.assert_allclose(cex, np.exp(2j * np.pi * k / 65536), atol=1e-15)


def test_single_atom_ref22_is_cfact(oracle):
    cr, g, csf_ref, istl_ref = K.single_atom()
    rc, istl = oracle.stltab(g, cr.rten)
    assert rc == 0
    np.testing.assert_array_equal(istl, istl_ref)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, K.opts(phase=_abi.PHASE_REF22))
    assert rc == 0 and info.friedel_dim == 1
    np.testing.assert_allclose(csf, csf_ref, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(dsi, np.abs(csf_ref) ** 2, rtol=1e-12)


def test_laue_exact(oracle):
    cr, g, F = K.laue()
    op = K.opts(phase=_abi.PHASE_EXACT64, form=_abi.FORM_ANALYTIC)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    assert rc == 0
    np.testing.assert_allclose(csf, F, atol=1e-10 * np.abs(F).max())


def test_laue_ref22_within_table_floor(oracle):
    """REF22 differs from the exact Laue function only by the 2^-16-turn
    truncated phase and the 0.001/A form-factor grid."""
    cr, g, F = K.laue()
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, K.opts(phase=_abi.PHASE_REF22, form=_abi.FORM_ANALYTIC))
    assert rc == 0
    n = cr.natoms
    fmax = np.abs(F).max() / n
    # 2 pi 2^-16 rad per term, coherent worst case
    assert np.max(np.abs(csf - F)) <= n * fmax * (2 * np.pi / 65536) * 1.5


def test_table_floor_tolerance_covers_ref22(oracle):
    """The oracle's REF22 (the reference's table arithmetic) against its
    EXACT64 on the 5000-site perovskite plane: the difference is the table's
    floor, and oracle.lut_floor_tol, the tolerance the GPU comparisons with
    REF22 use, must cover it (with the same form-factor table in both)."""
    cr, g = S.perovskite_plane()
    rc, _, _, a, info = oracle.four_run(cr, g, K.opts(phase=_abi.PHASE_REF22))
    rc2, _, _, b, _ = oracle.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64))
    assert rc == rc2 == 0
    err = K.rel_err(a, b, K.incoherent_floor(cr, g, K.opts()))
    tol = oracle.lut_floor_tol(g, list(info.lmn))
    assert 1e-6 < err <= tol / 2


def test_two_atoms_exact(oracle):
    cr, g, F = K.two_atoms()
    op = K.opts(phase=_abi.PHASE_EXACT64, form=_abi.FORM_ANALYTIC, friedel=0)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    assert rc == 0
    np.testing.assert_allclose(csf, F, atol=1e-12 * np.abs(F).max())


def test_increments_match_definition(oracle):
    """NINT(2^22 * (x.v - INT(x.v))) (four_strucf_OMP_mod.f90:143-148)."""
    rng = np.random.Generator(np.random.PCG64(3))
    x = rng.uniform(-40, 40, size=(500, 3))
    u, v, w = np.array([0.05, 0.0, 0.01]), np.array([0.0, 0.05, 0.0]), np.array([0.013, -0.02, 0.08])
    off = np.zeros((3, 3))
    off[:, 2] = [0, 0, 0.001]
    inc = oracle.increments(x, u, v, w, off)
    for k, vec in enumerate([u, v, w, off[:, 0], off[:, 1], off[:, 2]]):
        d = (x[:, 0] * vec[0] + x[:, 1] * vec[1]) + x[:, 2] * vec[2]
        fr = d - np.trunc(d)
        y = 4194304.0 * fr
        exp = np.where(y >= 0, np.floor(y + 0.5), -np.floor(-y + 0.5)).astype(np.int64)
        np.testing.assert_array_equal(inc[k], exp)


def test_friedel_symmetry_and_reduction(oracle):
    cr, g = S.perovskite_plane(cells=3)
    op = K.opts(phase=_abi.PHASE_EXACT64)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    assert rc == 0 and list(info.fnum) == [101, 201, 1] and info.friedel_dim == 1
    op2 = K.opts(phase=_abi.PHASE_EXACT64, friedel=0)
    rc, csf2, acsf2, dsi2, info2 = oracle.four_run(cr, g, op2)
    assert info2.friedel_dim == 0
    np.testing.assert_allclose(dsi, dsi2, rtol=1e-9, atol=1e-9 * dsi2.max())
    np.testing.assert_allclose(dsi, dsi[::-1, ::-1, ::-1], rtol=1e-12)


def test_average_subtraction_perfect_crystal(oracle):
    """A perfect crystal minus <F> (fave = 1) leaves ~0 everywhere."""
    rng = np.random.Generator(np.random.PCG64(11))
    sites = [[0, 0, 0], [0.5, 0.5, 0.5]]
    pos, iscat = S.build_periodic(sites, [1, 2], (4, 4, 3), 4.0, rng, 0.0)
    scat, occ, dw = S.random_form_factors(rng, 2)
    cr = S.CrystalData(pos=pos, iscat=iscat, nscat=2, ncatoms=2, icc=(4, 4, 3), rten=K.KAT["rten_cubic4"],
                       scat=scat, occ=occ, dw=dw)
    g = S.GridData.from_corners((-1.5, -1.5, 0.25), (1.5, -1.5, 0.25), (-1.5, 1.5, 0.25), inc=(31, 31, 1))
    for phase in (_abi.PHASE_EXACT64, _abi.PHASE_REF22):
        rc, csf, acsf, dsi, info = oracle.four_run(cr, g, K.opts(phase=phase, fave=1.0))
        assert rc == 0 and info.ncell == 48
        tot = np.abs(acsf).max()
        assert np.abs(csf).max() <= 1e-9 * tot + (1e-3 * tot if phase == _abi.PHASE_REF22 else 0)


def test_translation_invariance(oracle):
    """Shifting all atoms by a lattice vector leaves dsi unchanged (EXACT64)."""
    cr, g = S.small_random(seed=5, natoms=40, inc=(7, 9, 3))
    op = K.opts(phase=_abi.PHASE_EXACT64, friedel=0)
    _, _, _, d1, _ = oracle.four_run(cr, g, op)
    cr2 = cr.with_positions(cr.pos + np.array([3.0, -2.0, 7.0]))
    _, _, _, d2, _ = oracle.four_run(cr2, g, op)
    # h is not integer, so a lattice translation changes F only by a global phase
    np.testing.assert_allclose(d1, d2, rtol=1e-9)


def test_qinfo_statistics(oracle):
    cr, g = S.perovskite_plane(cells=3)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64))
    h = g.hkl()
    bragg = np.all(h == np.round(h), axis=0)
    res = list(info.res)
    assert res[0] == 6
    np.testing.assert_allclose(res[6], dsi[bragg].max())
    np.testing.assert_allclose(res[2], dsi[~bragg].max())
    np.testing.assert_allclose(res[3], dsi[~bragg].mean(), rtol=1e-12)


def test_stl_range_error(oracle):
    cr, g, _, _ = K.single_atom()
    big = S.GridData.from_corners((-60, -60, 0), (60, -60, 0), (-60, 60, 0), inc=(5, 5, 1))
    rc, istl = oracle.stltab(big, cr.rten)
    assert rc == _abi.DGPU_ERR_STL_RANGE


def test_oracle_gradient_matches_finite_differences(oracle):
    """The FP64 reference gradient (oc_chi2_grad) against central differences."""
    cr, g = S.small_random(seed=8, natoms=30, nscat=2, inc=(5, 5, 3))
    cr.atom_occ = np.linspace(0.9, 1.1, cr.natoms).astype(np.float32)
    tgt = S.perturbed_copy(cr, 3, 0.05, 4.0, 0.1)
    op = K.opts(phase=_abi.PHASE_EXACT64, friedel=0)
    rc, csf, acsf, it, info = oracle.four_run(tgt, g, op)
    wt = 1.0 / (it + 1.0)
    c2, gp, go = oracle.chi2_grad(cr, g, op, it, wt)
    h = 1e-6
    for a in (1, 7):
        for k in range(3):
            p = cr.pos.copy()
            p[a, k] += h
            cp, _, _ = oracle.chi2_grad(cr.with_positions(p), g, op, it, wt)
            p[a, k] -= 2 * h
            cm, _, _ = oracle.chi2_grad(cr.with_positions(p), g, op, it, wt)
            assert abs((cp - cm) / (2 * h) - gp[a, k]) <= 1e-6 * np.abs(gp).max()


def test_timing_build_computes_the_same_sums(oracle):
    """The release-flag build (-O3 -ffast-math) timed as the CPU baseline runs
    the same REF22 loop: its four_run agrees with the exact build to FP64
    reassociation, and its timed row sample counts the same pairs."""
    import ctypes as C
    cr, g = S.small_random(seed=9, natoms=400, nscat=2, inc=(11, 9, 5))
    op = K.opts(phase=_abi.PHASE_REF22)
    out = []
    for L in (oracle.lib(), oracle.timing_lib()):
        np_ = g.npoints
        csf, acsf, dsi = np.zeros(2 * np_), np.zeros(2 * np_), np.zeros(np_)
        info = _abi.Info()
        c, gg = cr.to_c(), g.to_c()
        rc = L.oc_four_run(C.byref(c), C.byref(gg), C.byref(op), oracle._d(csf), oracle._d(acsf), oracle._d(dsi),
                           C.byref(info), 2)
        assert rc == 0
        pairs = C.c_int64(0)
        L.oc_time_ref_rows(C.byref(c), C.byref(gg), 0, 3, 2, C.byref(pairs))
        out.append((dsi, pairs.value))
    (d0, p0), (d1, p1) = out
    assert p0 == p1 > 0
    np.testing.assert_allclose(d1, d0, rtol=1e-9, atol=1e-9 * d0.max())
