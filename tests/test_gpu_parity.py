"""GPU path against the oracle and the closed-form known answers.

Tolerances: integer work (increments, istl, lmn) is bit-exact; tables are
FP64 (1e-14); type sums use FP32 phasors with FP64 reduction, so
intensities are compared as max |I - I_ref| / (I_ref + N<|f|^2>) <= 1e-5
(the headline metric's accuracy bound) -- REF22 against the oracle's REF22 (same
2^-16-turn phase table), EXACT64 against the oracle's exact FP64 sums.
"""
import ctypes as C

import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S

pytestmark = pytest.mark.gpu
TOL = 1e-5


def run_both(oracle, ctx, cr, g, op, **kw):
    og = oracle.four_run(cr, g, op)
    gg = FR.four_run(cr, g, op, ctx=ctx, **kw)
    return og, gg


def test_stltab_bitexact(oracle, ctx):
    for cr, g in (S.perovskite_plane(cells=2), S.small_random(seed=3, inc=(11, 9, 5))):
        rc_o, istl_o = oracle.stltab(g, cr.rten)
        rc_g, istl_g = FR.four_stltab(g, cr.rten, ctx=ctx)
        assert rc_o == rc_g == 0
        np.testing.assert_array_equal(istl_g, istl_o)


def test_stltab_range_error(ctx):
    cr, _, _, _ = K.single_atom()
    big = S.GridData.from_corners((-60, -60, 0), (60, -60, 0), (-60, 60, 0), inc=(5, 5, 1))
    rc, _ = FR.four_stltab(big, cr.rten, ctx=ctx)
    assert rc == _abi.DGPU_ERR_STL_RANGE


def test_formtab(oracle, ctx):
    cr, _ = S.perovskite_plane(cells=2)
    for ldbw in (0, 1):
        op = K.opts(ldbw=ldbw)
        a = oracle.formtab(cr, op)
        b = FR.four_formtab(cr, op, ctx=ctx)
        np.testing.assert_allclose(b, a, rtol=1e-14, atol=1e-14 * np.abs(a).max())


def test_increments_bitexact(oracle, ctx):
    rng = np.random.Generator(np.random.PCG64(9))
    x = rng.uniform(-60, 60, size=(4096, 3))
    u, v, w = np.array([0.05, 0.0, 0.013]), np.array([-0.007, 0.05, 0.0]), np.array([0.013, -0.02, 0.08])
    off = rng.uniform(-0.01, 0.01, size=(3, 3))
    np.testing.assert_array_equal(FR.four_increments(x, u, v, w, off, ctx=ctx),
                                  oracle.increments(x, u, v, w, off))


def test_lmn_device_library_matches_cases(ctx):
    for case in K.LMN_CASES:
        eck = np.zeros((3, 4))
        eck[:, 0] = case["eck"]
        rc, lmn, off = FR.fourier_lmn(eck, np.asarray(case["vi"]).T, case["inc"], ctx=ctx)
        assert rc == case["rc"]
        if rc == 0:
            assert list(lmn) == case["lmn"]


def test_single_atom_known_answer(ctx):
    cr, g, csf_ref, _ = K.single_atom()
    for eng in (_abi.ENGINE_DIRECT,):
        r = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_REF22, engine=eng), ctx=ctx)
        np.testing.assert_allclose(r.csf, csf_ref, rtol=1e-12, atol=1e-12)


def test_laue_known_answer(ctx):
    cr, g, F = K.laue()
    r = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64, form=_abi.FORM_ANALYTIC, engine=_abi.ENGINE_DIRECT),
                    ctx=ctx)
    assert np.max(np.abs(r.csf - F)) <= 1e-5 * np.abs(F).max()


def test_two_atoms_known_answer(ctx):
    cr, g, F = K.two_atoms()
    r = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64, form=_abi.FORM_ANALYTIC, friedel=0,
                                  engine=_abi.ENGINE_DIRECT), ctx=ctx)
    assert np.max(np.abs(r.csf - F)) <= 1e-6 * np.abs(F).max()


@pytest.mark.parametrize("phase", [_abi.PHASE_REF22, _abi.PHASE_EXACT64])
def test_perovskite_plane_parity(oracle, ctx, phase):
    """The CPU-runnable workload (5000 sites, 201x201 hk0) end to end."""
    cr, g = S.perovskite_plane()
    op = K.opts(phase=phase, engine=_abi.ENGINE_DIRECT)
    (rc, csf, acsf, dsi, info), r = run_both(oracle, ctx, cr, g, op)
    assert rc == 0 and r.status == 0
    assert list(r.info.fnum) == list(info.fnum) and r.info.friedel_dim == info.friedel_dim == 1
    assert list(r.info.lmn) == list(info.lmn)
    floor = K.incoherent_floor(cr, g, op)
    assert K.rel_err(r.dsi, dsi, floor) <= TOL
    # four_qinfo statistics; minima sit at near-cancellations, so the
    # tolerance scales with the mean diffuse intensity
    ref = np.array(list(info.res)[1:])
    assert np.all(np.abs(np.array(r.res[1:]) - ref) <= 1e-4 * np.abs(ref) + 1e-5 * ref[2])
    assert r.info.pairs == cr.n_scattering() * g.npoints


def test_random_3d_parity(oracle, ctx):
    cr, g = S.small_random(seed=21, natoms=300, nscat=3, inc=(13, 11, 7))
    for phase in (_abi.PHASE_REF22, _abi.PHASE_EXACT64):
        for form in (_abi.FORM_TABLE, _abi.FORM_ANALYTIC):
            op = K.opts(phase=phase, form=form, engine=_abi.ENGINE_DIRECT)
            (rc, csf, acsf, dsi, info), r = run_both(oracle, ctx, cr, g, op)
            assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op)) <= TOL


def test_stacking_fault_plane_full_grid(oracle, ctx):
    """Layered crystal with stacking faults on an h0l plane and no
    displacements: atoms at equivalent positions have identical phases, so
    any error that is a function of the phase alone adds up coherently over a
    layer, and the in-plane sums are coherent along the rods.  Full-grid
    maximum against the oracle's EXACT64 intensities over all 40 401 points,
    within the metric's 1e-5 for both engines and both tensor-core operand
    paths (the CUDA-core engine within 5e-6)."""
    cr, g = S.hex_layers_plane(na=40, nc=8, inc=201, hmax=10.0)
    op = K.opts(phase=_abi.PHASE_EXACT64)
    rc, csf, acsf, ref, info = oracle.four_run(cr, g, op)
    fl = K.incoherent_floor(cr, g, op)
    d = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT), ctx=ctx).dsi
    assert K.rel_err(d, ref, fl) <= 5e-6
    for vimg in (1, -1):
        t = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC, tc_vimg=vimg), ctx=ctx).dsi
        assert K.rel_err(t, ref, fl) <= TOL


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_stacking_fault_plane_average_full_grid(oracle, ctx, engine):
    """The same plane with <F> subtracted (fave = 1): on the rods of the
    average lattice F and <F> are both hundreds of times the incoherent level
    and cancel; the tensor-core engine recomputes those points exactly
    (info.refined > 0).  Full grid within 1e-5 of the oracle."""
    cr, g = S.hex_layers_plane(na=40, nc=8, inc=201, hmax=10.0)
    op = K.opts(phase=_abi.PHASE_EXACT64, fave=1.0, engine=engine)
    (rc, csf, acsf, ref, info), r = run_both(oracle, ctx, cr, g, op)
    fl = K.incoherent_floor(cr, g, op)
    assert K.rel_err(r.dsi, ref, fl) <= TOL
    assert np.max(np.abs(r.acsf - acsf)) <= 1e-6 * np.abs(acsf).max()
    if engine == _abi.ENGINE_TC:
        assert r.info.engine_used == _abi.ENGINE_TC and r.info.refined > 0
    else:
        assert r.info.refined == 0


def test_friedel_on_off_agree(ctx):
    cr, g = S.perovskite_plane(cells=4)
    a = FR.four_run(cr, g, K.opts(engine=_abi.ENGINE_DIRECT), ctx=ctx)
    b = FR.four_run(cr, g, K.opts(engine=_abi.ENGINE_DIRECT, friedel=0), ctx=ctx)
    assert a.info.friedel_dim == 1 and b.info.friedel_dim == 0
    assert K.rel_err(a.dsi, b.dsi, K.incoherent_floor(cr, g, K.opts())) <= TOL
    np.testing.assert_array_equal(a.dsi, a.dsi[::-1, ::-1, ::-1])


@pytest.mark.parametrize("phase", [_abi.PHASE_REF22, _abi.PHASE_EXACT64])
def test_average_structure_parity(oracle, ctx, phase):
    cr, g = S.perovskite_plane(cells=4, vacancy=0.3)
    op = K.opts(phase=phase, fave=1.0, engine=_abi.ENGINE_DIRECT)
    (rc, csf, acsf, dsi, info), r = run_both(oracle, ctx, cr, g, op)
    assert r.info.ncell == info.ncell == 64
    scale = np.abs(acsf).max()
    assert np.max(np.abs(r.acsf - acsf)) <= 1e-5 * scale
    assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op)) <= TOL


def test_partial_average_with_cell_mask(oracle, ctx):
    cr, g = S.perovskite_plane(cells=4)
    rng = np.random.Generator(np.random.PCG64(5))
    cells = (rng.random(cr.icc) < 0.5).astype(np.uint8)
    op = K.opts(phase=_abi.PHASE_EXACT64, fave=0.5, engine=_abi.ENGINE_DIRECT)
    keep = np.ascontiguousarray(cells.reshape(-1, order="F"))
    op.aver_cells = keep.ctypes.data_as(C.POINTER(C.c_uint8))
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx, aver_cells=cells)
    assert r.info.ncell == info.ncell == int(cells.sum())
    assert np.max(np.abs(r.acsf - acsf)) <= 1e-5 * np.abs(acsf).max()


def test_per_type_dropin_matches_oracle(oracle, ctx):
    cr, g = S.perovskite_plane(cells=3)
    rc, lmn, off = oracle.fourier_lmn(g.eck, g.vi, g.inc)
    xat = cr.pos[cr.iscat == 3]
    num = g.inc
    fnum = (101, 201, 1)
    rc, istl = oracle.stltab(g, cr.rten)
    cf = oracle.formtab(cr, K.opts())[2]
    a = oracle.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, num, fnum, cf, istl)
    b = FR.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, num, fnum, cf, istl, ctx=ctx)
    assert np.all(b[101:] == 0)
    assert np.max(np.abs(b - a)) <= 1e-5 * np.abs(a).max()


def test_device_resident_api(ctx):
    import torch
    cr, g = S.perovskite_plane(cells=4)
    op = K.opts(engine=_abi.ENGINE_DIRECT)
    host = FR.four_run(cr, g, op, ctx=ctx)
    dev = torch.device("cuda:0")
    pos = torch.from_numpy(cr.pos).to(dev)
    isc = torch.from_numpy(cr.iscat).to(dev)
    csf = torch.zeros(2 * g.npoints, dtype=torch.float64, device=dev)
    acsf = torch.zeros_like(csf)
    dsi = torch.zeros(g.npoints, dtype=torch.float64, device=dev)
    c = cr.to_c(pos_ptr=C.cast(pos.data_ptr(), C.POINTER(C.c_double)),
                iscat_ptr=C.cast(isc.data_ptr(), C.POINTER(C.c_int32)))
    info = _abi.Info()
    torch.cuda.synchronize()
    rc = ctx.check(ctx.lib.dgpu_four_run_device(ctx.h, C.byref(c), C.byref(g.to_c()), C.byref(op),
                                                C.c_void_p(csf.data_ptr()), C.c_void_p(acsf.data_ptr()),
                                                C.c_void_p(dsi.data_ptr()), C.byref(info)))
    assert rc == 0
    d = dsi.cpu().numpy().reshape(g.inc, order="F")
    np.testing.assert_array_equal(d, host.dsi)


def test_cancel_flag(ctx):
    cr, g = S.perovskite_plane(cells=2)
    op = K.opts(engine=_abi.ENGINE_DIRECT)
    flag = C.c_int32(1)
    op.cancel = C.pointer(flag)
    with pytest.raises(Exception) as e:
        FR.four_run(cr, g, op, ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_CANCELLED


def test_argument_errors(ctx):
    cr, g = S.perovskite_plane(cells=2)
    bad = S.GridData(eck=g.eck, vi=np.zeros((3, 3)), inc=(11, 11, 1))
    with pytest.raises(Exception) as e:
        FR.four_run(cr, bad, K.opts(), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_ZERO_INC
    empty = cr.with_positions(cr.pos)
    empty.pos = np.zeros((0, 3))
    empty.iscat = np.zeros(0, np.int32)
    with pytest.raises(Exception) as e:
        FR.four_run(empty, g, K.opts(), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_NO_ATOMS


@pytest.mark.parametrize("phase", [_abi.PHASE_REF22, _abi.PHASE_EXACT64], ids=["ref22", "exact64"])
@pytest.mark.parametrize("rhkl", [(0.0, 0.0, 0.0), (1.0, -2.0, 3.0), (0.5, 0.25, -1.5)])
def test_calc_000_single_point(oracle, ctx, phase, rhkl):
    """calc_000: four_run on one point with zero increments (a single spot
    for fourier_lmn: identity offsets); res_para against the oracle's
    four_run on the same grid, and F(000) = sum_t N_t cfact_t(0)."""
    cr, _ = S.small_random(seed=5, natoms=300, nscat=2)
    op = K.opts(phase=phase)
    res = FR.calc_000(cr, op, rhkl, ctx=ctx)
    g = S.GridData(eck=np.repeat(np.asarray(rhkl)[:, None], 4, axis=1), vi=np.zeros((3, 3)), inc=(1, 1, 1))
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    assert rc == 0 and res[0] == 4.0
    f = complex(csf.reshape(-1)[0])
    scale = np.sqrt(abs(f) ** 2 + float(K.incoherent_floor(cr, g, op).reshape(-1)[0]))
    assert abs(complex(res[1], res[2]) - f) <= 1e-5 * scale
    ncell = float(np.prod(cr.icc))
    assert res[3] == res[1] / ncell and res[4] == res[2] / ncell
    if rhkl == (0.0, 0.0, 0.0):
        cfact = oracle.formtab(cr, op)
        f000 = sum(np.count_nonzero(cr.iscat == t) * cfact[t - 1, 0] for t in range(1, cr.nscat + 1))
        assert abs(complex(res[1], res[2]) - f000) <= 1e-6 * abs(f000)


def test_all_void_crystal_gives_zero(ctx):
    cr, g = S.perovskite_plane(cells=2)
    cr.iscat[:] = 0
    r = FR.four_run(cr, g, K.opts(engine=_abi.ENGINE_DIRECT), ctx=ctx)
    assert np.all(r.dsi == 0) and r.info.pairs == 0


def test_cached_tables_follow_the_grid_and_form_factors(oracle, ctx):
    """istl and cfact are kept between calls while the grid, metric and form
    factors stay (as four_layer does): a second grid of the same size, other
    form-factor coefficients, and a per-type call that loads the caller's
    tables in between all give the oracle's result."""
    cr, g = S.small_random(seed=5, natoms=200, nscat=2, inc=(9, 7, 5))
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT)
    floor = K.incoherent_floor(cr, g, op)
    g2 = S.GridData(eck=g.eck + 0.37, vi=g.vi * 1.1, inc=g.inc)
    for grid in (g, g, g2, g):
        r = FR.four_run(cr, grid, op, ctx=ctx)
        rc, _, _, ref, _ = oracle.four_run(cr, grid, op)
        assert K.rel_err(r.dsi, ref, K.incoherent_floor(cr, grid, op)) <= 1e-5
    cr2 = cr.with_positions(cr.pos)
    cr2.scat = cr.scat * 1.3
    r = FR.four_run(cr2, g, op, ctx=ctx)
    rc, _, _, ref, _ = oracle.four_run(cr2, g, op)
    assert K.rel_err(r.dsi, ref, K.incoherent_floor(cr2, g, op)) <= 1e-5
    # a per-type call with the caller's tables, then the run again
    rc, lmn, off = FR.fourier_lmn(g.eck, g.vi, g.inc, ctx=ctx)
    xat = cr.pos[cr.iscat == 1]
    fnum = g.inc
    FR.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, g.inc, fnum, None, None, ctx=ctx)
    r = FR.four_run(cr, g, op, ctx=ctx)
    rc, _, _, ref, _ = oracle.four_run(cr, g, op)
    assert K.rel_err(r.dsi, ref, floor) <= 1e-5
