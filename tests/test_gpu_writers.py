"""The output path end to end on the device: four_run, qval of the values
the writers need, the file through dgpu_output_write, against the oracle's
writer fed with the same arrays (the writer's bytes; qval and four_run are
checked against the oracle in their own tests; HDF5 read back with the
oracle's reader) -- and calc_hkl with its
files (HKLF4 and CIF in, calcfile and .fcf out), against the oracle's
calc_hkl values and file restatement."""
import math

import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import output as OUT
from diffusecode_gb300 import structures as S
from oracle import hdf5 as H5
from oracle import writers as W

pytestmark = pytest.mark.gpu


def flat(a):
    return np.asfortranarray(a).reshape(-1, order="F")


@pytest.fixture(scope="module")
def run(ctx):
    cr, _ = S.small_lots_anis(anis=False)
    g = S.GridData.from_corners((-3.0, -2.0, -1.0), (3.0, -2.0, -1.0), (-3.0, 2.0, -1.0), (-3.0, -2.0, 1.0),
                                inc=(13, 9, 3))
    op = K.opts(phase=_abi.PHASE_EXACT64)
    r = FR.four_run(cr, g, op, ctx=ctx)
    vals = {v: FR.qval(cr, g, op, v, r, ctx=ctx) for v in (1, 2, 3)}
    return cr, g, op, r, vals


def spec_pair(fmt, code, cr, g, **kw):
    ours = OUT.output_spec(fmt, g, cr=cr, **kw)
    kw2 = {k: v for k, v in kw.items() if k != "value"}
    theirs = W.Spec(code, kw.get("value", 1), g.inc, g.eck.reshape(-1, order="F"), g.vi.reshape(-1, order="F"),
                    rten=np.asarray(cr.rten).reshape(-1, order="F"), icc=cr.icc, **kw2)
    return ours, theirs


@pytest.mark.parametrize("fmt,code", [("hklf4", 6), ("list5", 7), ("list9", 8)])
def test_shelx_files_from_device_values(run, tmp_path, fmt, code):
    cr, g, op, r, vals = run
    f000 = float(vals[2][0, 0, 0])
    for valmax in (0.0, -1.0, -2.0):
        ours, theirs = spec_pair(fmt, code, cr, g, value=2, valmax=valmax, f000=f000, exti=0.3, rlambda=0.71)
        p = str(tmp_path / f"{fmt}{valmax}")
        fac = OUT.write(p, ours, vals[2], vals[2], vals[3])
        want, wfac = W.other(theirs, flat(vals[2]), flat(vals[2]), flat(vals[3]))
        assert open(p, "rb").read() == want
        assert fac == wfac


@pytest.mark.parametrize("fmt,code", [("standard", 0), ("gnuplot", 3), ("3d", 9), ("mrc", 12), ("xplor", 14)])
def test_grid_files_from_device_values(run, tmp_path, fmt, code):
    cr, g, op, r, vals = run
    nipl = OUT.nipl_info(cr, g, lambda_name="CUA1") if code == 0 else None
    ours, theirs = spec_pair(fmt, code, cr, g, value=1, nipl=nipl, name="lots crystal")
    p = str(tmp_path / fmt)
    OUT.write(p, ours, vals[1])
    v = flat(vals[1])
    if code == 0:
        for suf, b in W.standard(theirs, v).items():
            assert open(p + suf, "rb").read() == b
    elif code in (3, 9):
        assert open(p, "rb").read() == W.other(theirs, v)[0]
    elif code == 12:
        assert open(p, "rb").read() == W.mrc(theirs, v)
    else:
        assert open(W.xplor_name(p), "rb").read() == W.xplor(theirs, v)


def test_standard_2d_plane_with_fourier_header(ctx, tmp_path):
    """A 2D Fourier (four_last = 2) writes the FOURIER section with the
    angles of its axes in the crystal's metric."""
    cr, _ = S.small_lots_anis(anis=False)
    g = S.GridData.from_corners((-2.0, -2.0, 0.5), (2.0, -2.0, 0.5), (-2.0, 2.0, 0.5), inc=(17, 11, 1))
    op = K.opts(phase=_abi.PHASE_EXACT64)
    r = FR.four_run(cr, g, op, ctx=ctx)
    v = FR.qval(cr, g, op, 1, r, ctx=ctx)
    nipl = OUT.nipl_info(cr, g, radiation=2, ldbw=True)
    ours, theirs = spec_pair("standard", 0, cr, g, value=1, nipl=nipl)
    p = str(tmp_path / "plane")
    OUT.write(p, ours, v)
    got = open(p, "rb").read()
    assert got == W.standard(theirs, flat(v))[""]
    assert b"# FOURIER : type        ;1C:: 2D Fourier complete crystal" in got
    assert b"# FOURIER : radiation   ;1C:: neutron" in got


@pytest.mark.parametrize("valmax,scale", [(0.0, 1.0), (10000.0, 1.0), (-1.0, 0.25)])
def test_hdf5_from_device_values(run, tmp_path, valmax, scale):
    cr, g, op, r, vals = run
    p = str(tmp_path / "yell.h5")
    a0, win = (3.9, 3.9, 3.9), (90.0, 90.0, 90.0)
    OUT.write(p, OUT.output_spec("hdf5", g, cr=cr, valmax=valmax, scale=scale, a0=a0, win=win), vals[1])
    got = H5.read(open(p, "rb").read())
    want = H5.yell(g.inc, g.eck, g.vi, (1, 2, 3), a0, win, 1, flat(vals[1]), valmax=valmax, scale=scale)
    for name, w in want.items():
        if isinstance(w, np.ndarray):
            np.testing.assert_array_equal(got[name][0], w, err_msg=name)
        else:
            assert got[name][0] == w, name


def test_vtk_from_device_dsi(run, tmp_path):
    cr, g, op, r, vals = run
    ours, theirs = spec_pair("vtk", 11, cr, g)
    p = str(tmp_path / "d.vtk")
    OUT.write(p, ours, r.dsi)
    assert open(p, "rb").read() == W.vtk(theirs, flat(r.dsi))


def _hklf4_text(hkl, iobs):
    lines = [W.I(4, h) + W.I(4, k) + W.I(4, l) + W.F(8, 2, i) + W.F(8, 2, math.sqrt(abs(i)))
             for (h, k, l), i in zip(hkl, iobs)]
    return "\n".join(lines) + "\n"


def _cif_text(hkl, iobs):
    head = ["data_test", "loop_", "_refln_index_h", "_refln_index_k", "_refln_index_l", "_refln_F_squared_calc",
            "_refln_F_squared_meas", "_refln_F_squared_sigma", "_refln_observed_status"]
    rows = [f"{h} {k} {l} 0.0 {i:.2f} {math.sqrt(abs(i)):.2f} o" for (h, k, l), i in zip(hkl, iobs)]
    return "\n".join(head + rows) + "\n"


@pytest.mark.parametrize("style", ["hklf4", "cif"])
def test_calc_hkl_files(ctx, tmp_path, style):
    cr, _ = S.small_lots_anis(anis=False)
    rng = np.random.default_rng(21)
    hkl = rng.integers(-4, 5, size=(40, 3))
    hkl[7] = 0                                         # 0 0 0 inside the list
    hkl = np.vstack([hkl, [[0, 0, 0]]])                # and as the HKLF4 terminator
    iobs = rng.uniform(0.0, 300.0, size=hkl.shape[0])
    op = K.opts(phase=_abi.PHASE_EXACT64)
    text = _hklf4_text(hkl, iobs) if style == "hklf4" else _cif_text(hkl, iobs)
    inp = tmp_path / ("in.hkl" if style == "hklf4" else "in.cif")
    inp.write_text(text)
    calc = str(tmp_path / "calc.hkl")
    OUT.calc_hkl_files(cr, op, str(inp), calc, style=style, scale=0.4, exti=10.0, rlambda=0.6, ctx=ctx)
    ic, sg, ph = FR.calc_hkl(cr, op, hkl, scale=0.4, exti=10.0, rlambda=0.6, ctx=ctx)
    want_c, want_l = W.calc_hkl_files(4 if style == "hklf4" else 1, text, ic, sg, ph)
    assert open(calc, "rb").read() == want_c
    assert open(str(tmp_path / "calc.fcf"), "rb").read() == want_l
    # the oracle's calc_hkl agrees with the device values to the written precision
    from oracle import oracle as O
    rc, oic, osg, oph = O.calc_hkl(cr, op, hkl, scale=0.4, exti=10.0, rlambda=0.6)
    assert rc == 0
    np.testing.assert_allclose(ic, oic, rtol=2e-5, atol=2e-5 * oic.max())
    # a name without "hkl" gets ".fcf" appended
    calc2 = str(tmp_path / "calc.out")
    OUT.calc_hkl_files(cr, op, str(inp), calc2, style=style, scale=0.4, exti=10.0, rlambda=0.6, ctx=ctx)
    assert open(calc2 + ".fcf", "rb").read() == want_l


def test_calc_hkl_files_rejects_comment_lines(ctx, tmp_path):
    cr, _ = S.small_lots_anis(anis=False)
    inp = tmp_path / "bad.hkl"
    inp.write_text("# a comment\n   1   0   0   10.00    1.00\n")
    with pytest.raises(Exception):
        OUT.calc_hkl_files(cr, K.opts(), str(inp), str(tmp_path / "o.hkl"), ctx=ctx)
