"""four_weight and four_accumulate on the GPU against the oracle."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S
from test_oracle_weight_cpu import _crystal, _grid

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", range(4))
def test_four_weight_vs_oracle(oracle, ctx, case):
    rt = S.reciprocal_metric(4.1, 4.6, 5.3, 90, 103, 90)
    cr = _crystal((5, 4, 3), rt)
    vi, inc, op = [
        (np.array([[0.1, 0.02, 0.0], [0.0, 0.2, 0.01], [0.03, 0.0, 0.25]]), (9, 7, 5), _abi.default_opts()),
        (np.array([[0.05, 0.0, 0.0], [0.0, 0.05, 0.0], [0.0, 0.0, 0.0]]), (21, 21, 1), _abi.default_opts()),
        (np.diag([0.1, 0.1, 0.1]), (11, 11, 11),
         _abi.default_opts(ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), nlots=7)),
        (np.diag([0.1, 0.1, 0.1]), (11, 11, 11), _abi.default_opts(fave=0.5)),
    ][case]
    g = _grid(vi, inc)
    dsi = np.random.default_rng(case).random(g.inc) + 0.5
    ref, _ = oracle.four_weight(cr, g, dsi, op)
    out = FR.four_weight(cr, g, dsi, op, ctx=ctx)
    np.testing.assert_allclose(out, ref, rtol=1e-12)


def test_four_weight_after_run(oracle, ctx):
    """four_run then four_weight on the run's own dsi (the reference's order)."""
    cr, g = S.small_lots_anis(anis=False, inc=(13, 11, 5))
    op = K.opts(phase=_abi.PHASE_EXACT64)
    r = FR.four_run(cr, g, op, ctx=ctx)
    d3 = FR.four_weight(cr, g, r.dsi, op, ctx=ctx)
    ref, scalef = oracle.four_weight(cr, g, r.dsi, op)
    assert scalef != 1.0
    np.testing.assert_allclose(d3, ref, rtol=1e-12)


def test_four_accumulate(oracle, ctx):
    g = _grid(np.diag([0.25, 0.25, 0.0]), (9, 9, 1))
    rng = np.random.default_rng(4)
    runs = [(rng.random(g.inc) + 1j * rng.random(g.inc), rng.random(g.inc)) for _ in range(3)]
    FR.four_accumulate(_abi.ACCUM_INIT, g, ctx=ctx)
    for c, d in runs:
        FR.four_accumulate(_abi.ACCUM_ACCUM, g, c, d, ctx=ctx)
    csum = sum(c for c, _ in runs)
    dsum = sum(d for _, d in runs)
    c_out, d_out = FR.four_accumulate(_abi.ACCUM_FINISHED, g, runs[0][0], runs[0][1], ctx=ctx)
    np.testing.assert_allclose(c_out, csum, rtol=1e-14)
    np.testing.assert_allclose(d_out, dsum, rtol=1e-14)
    # fave < 0: Bragg points filled from their neighbours
    for c, d in runs:
        FR.four_accumulate(_abi.ACCUM_ACCUM, g, c, d, ctx=ctx)
    c_out, d_out = FR.four_accumulate(_abi.ACCUM_FINISHED, g, runs[0][0], runs[0][1], fave=-1.0, ctx=ctx)
    np.testing.assert_allclose(c_out, oracle.fill_bragg(g, csum), rtol=1e-14)
    np.testing.assert_allclose(d_out, oracle.fill_bragg(g, dsum), rtol=1e-14)
    # finished without sums; symmetry averaging with no operations set
    FR.set_symmetry(np.zeros((0, 3, 3)), ctx=ctx)
    for mode, kw, code in ((_abi.ACCUM_FINISHED, {}, _abi.DGPU_ERR_NO_ACCUM),
                           (_abi.ACCUM_SINGLE, {"symm": 1}, _abi.DGPU_ERR_ARG)):
        with pytest.raises(Exception) as e:
            FR.four_accumulate(mode, g, runs[0][0], runs[0][1], ctx=ctx, **kw)
        assert getattr(e.value, "code", None) == code


def test_negative_fave_is_no_cell(oracle, ctx):
    """fave < 0: four_aver draws no cell (<F> = 0, warning +1), as the
    reference does; the Bragg fill of four_accumulate keys on it."""
    cr, g = S.small_lots_anis(anis=False)
    op = K.opts(phase=_abi.PHASE_EXACT64, fave=-1.0)
    rc, csf, acsf, dsi, info = oracle.four_run(cr, g, op)
    r = FR.four_run(cr, g, op, ctx=ctx)
    assert rc == r.status == _abi.DGPU_WARN_NO_CELL
    assert not np.any(r.acsf) and not np.any(acsf)
    r0 = FR.four_run(cr, g, K.opts(phase=_abi.PHASE_EXACT64), ctx=ctx)
    np.testing.assert_allclose(r.dsi, r0.dsi, rtol=1e-12)


def _mmm():
    return np.array([np.diag([sx, sy, sz]).astype(float) for sx in (1, -1) for sy in (1, -1) for sz in (1, -1)])


def _four_fold():
    r = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    return np.array([np.linalg.matrix_power(r, k) for k in range(4)])


@pytest.mark.parametrize("ops", ["mmm", "4"])
def test_four_symm_single_vs_oracle(oracle, ctx, ops):
    """four_symm on one pattern (SINGLE with symm): the point-group average of
    csf and dsi on a 3D grid off-centre along x (images falling outside keep
    their own weight), the same arithmetic in the same order as the oracle's
    sequential restatement of four_symm_csf / four_symm_dsi."""
    mats = _mmm() if ops == "mmm" else _four_fold()
    g = _grid(np.diag([0.25, 0.25, 0.5]), (13, 13, 5), lo=(-1.25, -1.5, -1.0))
    rng = np.random.default_rng(3)
    d = rng.random(g.inc)
    z = d * np.exp(2j * np.pi * rng.random(g.inc))
    FR.set_symmetry(mats, ctx=ctx)
    c, di = FR.four_accumulate(_abi.ACCUM_SINGLE, g, z, d, fave=0.0, symm=1, ctx=ctx)
    np.testing.assert_array_equal(di, oracle.four_symm(g, d, mats))
    np.testing.assert_array_equal(c, oracle.four_symm(g, z, mats))


def test_four_symm_finished_with_bragg_fill(oracle, ctx):
    """Two accumulated patterns finished with symm and fave < 0: the point-
    group average of the sums, then the Bragg fill (four_fill_csf /
    four_fill_dsi, fourier_sup.f90:3844-4044)."""
    mats = _mmm()
    g = _grid(np.diag([0.25, 0.25, 0.5]), (13, 13, 5), lo=(-1.5, -1.5, -1.0))
    rng = np.random.default_rng(5)
    FR.set_symmetry(mats, ctx=ctx)
    FR.four_accumulate(_abi.ACCUM_INIT, g, ctx=ctx)
    tot_d, tot_z = 0.0, 0.0
    for _ in range(2):
        d = rng.random(g.inc)
        z = d * np.exp(2j * np.pi * rng.random(g.inc))
        FR.four_accumulate(_abi.ACCUM_ACCUM, g, z, d, ctx=ctx)
        tot_d, tot_z = tot_d + d, tot_z + z
    c, di = FR.four_accumulate(_abi.ACCUM_FINISHED, g, fave=-1.0, symm=1, ctx=ctx)
    np.testing.assert_allclose(di, oracle.fill_bragg(g, oracle.four_symm(g, tot_d, mats)), rtol=1e-14)
    np.testing.assert_allclose(c, oracle.fill_bragg(g, oracle.four_symm(g, tot_z, mats)), rtol=1e-14, atol=1e-14)


def test_four_symm_rejects_non_integer_operations(ctx):
    with pytest.raises(Exception) as e:
        FR.set_symmetry([np.eye(3), np.diag([0.5, 2.0, 1.0])], ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_ARG
