"""Tensor-core engine (tcgen05 split-precision GEMM) against the oracle's
exact FP64 sums: max |I - I_64| / (I_64 + N<|f|^2>) <= 1e-5 with the fp16
hi/lo split.  Shapes exercise padding of rows (M = 128) and columns
(N multiple of 16), several K slices per type and several work items per CTA."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S

pytestmark = pytest.mark.gpu
TOL = 1e-5


def tc_opts(**kw):
    base = dict(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC)
    base.update(kw)
    return K.opts(**base)


@pytest.mark.parametrize("vimg", [1, -1], ids=["v-images", "v-in-kernel"])
@pytest.mark.parametrize("inc,natoms", [((13, 11, 7), 300), ((37, 5, 3), 1000), ((3, 129, 2), 77),
                                        ((201, 1, 1), 40)])
def test_tc_random_vs_oracle(oracle, ctx, inc, natoms, vimg):
    """Both V operand paths: images streamed by the copy warp (independent
    stmatrix producers) and V generated in the kernel (producer barrier)."""
    cr, g = S.small_random(seed=31, natoms=natoms, nscat=3, inc=inc)
    for form in (_abi.FORM_TABLE, _abi.FORM_ANALYTIC):
        op = tc_opts(form=form, tc_vimg=vimg)
        rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
        r = FR.four_run(cr, g, op, ctx=ctx)
        assert r.info.engine_used == _abi.ENGINE_TC
        assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op)) <= TOL


@pytest.mark.parametrize("engine", [_abi.ENGINE_TC, _abi.ENGINE_DIRECT], ids=["tc", "direct"])
@pytest.mark.parametrize("inc", [(1, 1, 1), (1, 1, 9), (1, 7, 1), (2, 2, 2), (4, 1, 3)])
def test_degenerate_grids_and_absent_types(oracle, ctx, engine, inc):
    """One point, rods along the second and third axes, 2 x 2 x 2 and a
    plane across axes 1 and 3; of three types the second is absent and the
    third holds a single atom (an empty type range beside a one-atom one)."""
    cr, g = S.small_random(seed=41, natoms=150, nscat=3, inc=inc)
    cr.iscat[cr.iscat == 2] = 1
    cr.iscat[cr.iscat == 3] = 0
    cr.iscat[17] = 3
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx)
    assert r.info.engine_used == engine
    assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op)) <= TOL
    np.testing.assert_allclose(r.csf, csf, rtol=0, atol=3e-3 * np.sqrt(np.abs(dsi).max() + 1.0))


@pytest.mark.parametrize("vimg", [1, -1], ids=["v-images", "v-in-kernel"])
@pytest.mark.parametrize("tile_n,kslice", [(16, 1024), (64, 2048), (112, 0), (128, 96), (80, 4096)])
def test_tc_tiles_and_slices(oracle, ctx, tile_n, kslice, vimg):
    cr, g = S.perovskite_plane(cells=6)
    op = tc_opts(tc_tile_n=tile_n, tc_kslice=kslice, tc_vimg=vimg)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx)
    assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op)) <= TOL


def test_tc_perovskite_plane(oracle, ctx):
    cr, g = S.perovskite_plane()
    op = tc_opts()
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx)
    err = K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op))
    print(f"perovskite TC rel err {err:.2e}")
    assert err <= TOL


def test_tc_average_structure(oracle, ctx):
    cr, g = S.perovskite_plane(cells=5)
    op = tc_opts(fave=1.0)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx)
    assert np.max(np.abs(r.acsf - acsf)) <= 1e-5 * np.abs(acsf).max()
    assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op)) <= TOL


def test_tc_known_answers(ctx):
    cr, g, F = K.laue()
    r = FR.four_run(cr, g, tc_opts(form=_abi.FORM_ANALYTIC), ctx=ctx)
    assert np.max(np.abs(r.csf - F)) <= 1e-5 * np.abs(F).max()
    cr, g, F = K.two_atoms()
    r = FR.four_run(cr, g, tc_opts(form=_abi.FORM_ANALYTIC, friedel=0), ctx=ctx)
    assert np.max(np.abs(r.csf - F)) <= 1e-5 * np.abs(F).max()


def test_tc_bf16_split_error_is_reported(oracle, ctx):
    """bf16 hi/lo keeps ~16 significant bits; it runs, with a larger error."""
    cr, g = S.perovskite_plane(cells=4)
    op = tc_opts(split=_abi.SPLIT_BF16)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx)
    err = K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op))
    print(f"bf16 split rel err {err:.2e}")
    assert err <= 1e-3


@pytest.mark.parametrize("case", ["perovskite", "fcc-alloy"])
def test_tc_against_reference_arithmetic(oracle, ctx, case):
    """The tensor-core engine (exact 64-bit phases) against the oracle's
    REF22 four_run, the reference's own arithmetic (2^-22-turn increments,
    2^-16-turn cos/sin table): the 5000-site perovskite plane (201 x 201
    hk0) and a 12^3-cell fcc alloy on the 101^3 grid.  Every point within the
    table's floor (oracle.lut_floor_tol: six sigma of the table truncation and
    increment rounding, in units of I + N<|f|^2>)."""
    cr, g = S.perovskite_plane() if case == "perovskite" else S.fcc_alloy_volume(cells=12)
    r = FR.four_run(cr, g, tc_opts(), ctx=ctx)
    rc, csf, acsf, ref, info = oracle.four_run(cr, g, K.opts(phase=_abi.PHASE_REF22))
    tol = oracle.lut_floor_tol(g, list(info.lmn))
    err = K.rel_err(r.dsi, ref, K.incoherent_floor(cr, g, tc_opts()))
    print(f"{case}: TC vs REF22 {err:.2e} (table floor {tol:.2e})")
    assert r.info.engine_used == _abi.ENGINE_TC
    assert err <= tol


@pytest.mark.parametrize("vimg", [1, -1], ids=["v-images", "v-in-kernel"])
def test_tc_wait_limit_runs_out_and_context_recovers(oracle, ctx, vimg):
    """Failure detection on the device without a fault: with a 1 us limit on
    every wait of one warp for another's progress, the drain warps' first
    wait for the MMAs cannot be met; the kernel stops, waits for its own MMAs
    and copies, frees its tensor memory, and the call returns
    DGPU_ERR_TIMEOUT.  The next call on the same context, with the default
    limit, gives the oracle's result."""
    cr, g = S.perovskite_plane(cells=6)
    with pytest.raises(Exception) as e:
        FR.four_run(cr, g, tc_opts(tc_vimg=vimg, tc_wait_us=1), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_TIMEOUT
    op = tc_opts(tc_vimg=vimg)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx)
    assert r.info.engine_used == _abi.ENGINE_TC
    assert K.rel_err(r.dsi, dsi, K.incoherent_floor(cr, g, op)) <= TOL


def test_tc_ref22_rejected(ctx):
    cr, g = S.perovskite_plane(cells=2)
    with pytest.raises(Exception) as e:
        FR.four_run(cr, g, tc_opts(phase=_abi.PHASE_REF22), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_UNSUPPORTED
