"""Output-menu and calc_hkl file writers (host code of the C-ABI library)
against the oracle's restatement (oracle/writers.py), byte for byte.

The edit descriptors of the oracle are pinned first by known answers
derived by hand from the Fortran rules (Ew.d with scale factor 0, the
optional leading zero, exponent forms, asterisks on overflow, gfortran's
list-directed layout); the writers are then compared on seeded values over
1D, 2D and 3D grids, every format, scaling mode and range option.  No GPU:
the writers are host functions of the library.
"""
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import writers as W  # noqa: E402

from diffusecode_gb300 import _abi  # noqa: E402
from diffusecode_gb300 import output as OUT  # noqa: E402
from diffusecode_gb300.structures import GridData, reciprocal_metric  # noqa: E402


@pytest.fixture(scope="module")
def lib():
    from diffusecode_gb300 import _lib
    try:
        return _lib.load()
    except ImportError as e:
        pytest.skip(str(e))


# ------------------------------------------------------------- oracle pins

@pytest.mark.parametrize("args,want", [
    ((12, 5, 1.0), " 0.10000E+01"),
    ((12, 5, -0.000123456), "-0.12346E-03"),
    ((12, 5, 0.0), " 0.00000E+00"),
    ((12, 5, 1.0e100), " 0.10000+101"),
    ((12, 5, -9.999996), "-0.10000E+02"),
    ((11, 5, -1.0), "-.10000E+01"),
    ((10, 5, -1.0), "**********"),
    ((12, 4, 1.0), "  0.1000E+01"),
])
def test_oracle_e_edit(args, want):
    assert W.E(*args) == want


def test_oracle_e_edit_with_exponent_digits():
    assert W.E(13, 6, 1234.5678, 2) == " 0.123457E+04"
    assert W.E(13, 6, 1.0e100, 2) == "*" * 13
    assert W.E(13, 6, 2.5e-7, 2) == " 0.250000E-06"


@pytest.mark.parametrize("args,want", [
    ((8, 2, 0.0), "    0.00"),
    ((8, 2, -0.001), "   -0.00"),
    ((8, 2, 123.456), "  123.46"),
    ((8, 2, 123456.0), "********"),
    ((3, 2, 0.5), ".50"),
    ((10, 6, -1.5), " -1.500000"),
    ((7, 2, 359.999), " 360.00"),
])
def test_oracle_f_edit(args, want):
    assert W.F(*args) == want


def test_oracle_other_edits():
    assert W.I(4, 12345) == "****"
    assert W.I(4, -12) == " -12"
    assert W.F0(4, 0.5) == "0.5000"
    assert W.F0(4, -12.345678) == "-12.3457"
    assert W.A(5, "O   ") == " O   "
    assert W.A(3, "ABCDE") == "ABC"


def test_oracle_list_directed():
    assert W.ld_int(5) == "           5"
    assert W.ld_int(-123) == "        -123"
    assert W.ld_real(1.0) == "   1.0000000000000000     "
    assert W.ld_real(0.1) == "  0.10000000000000001     "
    assert W.ld_real(-2.5) == "  -2.5000000000000000     "
    assert W.ld_real(0.0) == "   0.0000000000000000     "
    assert W.ld_real(1.0e-3) == "   1.0000000000000000E-003"
    assert W.ld_real(-123.456) == "  -123.45600000000000     "


def test_oracle_format_reversion():
    assert W.groups(["a", "b", "c"], 2) == ["ab", "c"]
    assert W.groups([], 5) == [""]


# ------------------------------------------------------------- cases

RTEN = reciprocal_metric(4.1, 4.3, 5.2, 88, 92, 95)


class Cr:
    """the crystal fields the writers read"""

    def __init__(self, icc=(3, 4, 2)):
        self.icc = icc
        self.rten = RTEN
        self.nscat = 2
        self.ncatoms = 2
        self.iscat = np.array([1, 2, 1, 0, 2, 2], dtype=np.int32)
        self.dw = np.array([0.0, 0.5, 1.25])


def grid(inc, ll=(-2.0, -1.5, 0.25), step=(0.5, 0.25, 0.75)):
    ll = np.asarray(ll)
    lr = ll + np.array([step[0] * (inc[0] - 1), 0.1 * (inc[0] - 1), 0.0])
    ul = ll + np.array([0.0, step[1] * (inc[1] - 1), 0.0])
    tl = ll + np.array([0.0, 0.0, step[2] * (inc[2] - 1)])
    return GridData.from_corners(ll, lr, ul, tl, inc=inc)


def values(g, seed, lo=-5.0, hi=50.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    v = rng.uniform(lo, hi, size=g.inc).astype(np.float64)
    v.reshape(-1)[::7] *= 1e-4
    return v


def oracle_spec(fmt, g, **kw):
    return W.Spec(fmt, kw.pop("value", 1), g.inc, g.eck.reshape(-1, order="F"), g.vi.reshape(-1, order="F"),
                  **kw)


def ours(tmp_path, fname, fmt, g, vals=None, ampl=None, phase=None, **kw):
    p = str(tmp_path / fname)
    spec = OUT.output_spec(fmt, g, **kw)
    fac = OUT.write(p, spec, vals, ampl, phase)
    return p, fac


def flat(a):
    return np.asfortranarray(a).reshape(-1, order="F")


NIPL = {"natoms": 6, "nscat": 2, "ncatoms": 2, "at_lis": ["VOID", "O", "ZN"], "amount": [1, 2, 3],
        "dw": [0.0, 0.5, 1.25], "four_last": 2, "radiation": 1, "rlambda": 0.70932, "lambda": "MOA1",
        "ldbw": 1, "ano": 0}


def nipl_for(g, **kw):
    n = dict(NIPL)
    n.update({"inc": list(g.inc), "eck": list(g.eck.reshape(-1, order="F")),
              "vi": list(g.vi.reshape(-1, order="F"))})
    n.update(kw)
    return n


# ------------------------------------------------------------- writers

@pytest.mark.parametrize("inc", [(7, 1, 1), (1, 6, 1), (1, 1, 5)])
def test_standard_1d(lib, tmp_path, inc):
    g = grid(inc)
    v = values(g, 1)
    p, _ = ours(tmp_path, "s1", "standard", g, v, extr=(2, 1, 3))
    want = W.standard(oracle_spec(0, g, extr=(2, 1, 3)), flat(v))[""]
    assert open(p, "rb").read() == want


@pytest.mark.parametrize("with_header", [False, True])
def test_standard_2d(lib, tmp_path, with_header):
    g = grid((11, 7, 1))
    v = values(g, 2)
    n = nipl_for(g) if with_header else None
    p, _ = ours(tmp_path, "s2", "standard", g, v, cr=Cr(), nipl=n)
    want = W.standard(oracle_spec(0, g, rten=RTEN.reshape(-1, order="F"), nipl=n), flat(v))[""]
    got = open(p, "rb").read()
    assert got == want
    if with_header:
        lines = got.decode().splitlines()
        assert lines[0].startswith("# HEADER  : lines, sec  ;2I::") and lines[0].endswith("2")
        assert "# FOURIER : wave name   ;1C::MOA1" in lines
        assert "# CRYSTAL : type atom   ;1C 2I 1R::  ZN  ,            2,            3,  1.25000" in lines


def test_standard_3d_parts_and_header_variants(lib, tmp_path):
    g = grid((6, 5, 3))
    v = values(g, 3)
    n = nipl_for(g, four_last=-3, lambda_="", radiation=2)
    n["lambda"] = ""
    p, _ = ours(tmp_path, "s3", "standard", g, v, cr=Cr(), nipl=n, extr=(1, 2, 3))
    want = W.standard(oracle_spec(0, g, rten=RTEN.reshape(-1, order="F"), nipl=n), flat(v))
    assert sorted(want) == [".PART_0001", ".PART_0002", ".PART_0003"]
    for suf, b in want.items():
        assert open(p + suf, "rb").read() == b
    assert not os.path.exists(p)
    # four_last = -3: no FOURIER section
    assert b"FOURIER" not in want[".PART_0001"]
    n2 = nipl_for(g)
    p2, _ = ours(tmp_path, "s3b", "standard", g, v, cr=Cr(), nipl=n2)
    want2 = W.standard(oracle_spec(0, g, rten=RTEN.reshape(-1, order="F"), nipl=n2), flat(v))
    for suf, b in want2.items():
        got = open(p2 + suf, "rb").read()
        assert got == b
        assert b"# FOURIER : current top ;1I::            %d" % int(suf[-1]) in got


@pytest.mark.parametrize("inc", [(9, 6, 1), (8, 1, 1), (1, 5, 1)])
def test_gnuplot(lib, tmp_path, inc):
    g = grid(inc)
    v = values(g, 4)
    p, _ = ours(tmp_path, "g", "gnuplot", g, v, extr=(1, 2, 3))
    want, _ = W.other(oracle_spec(3, g), flat(v))
    assert open(p, "rb").read() == want
    if inc[0] == 1 or inc[1] == 1:
        assert want == b""                      # the reference writes no 1D gnuplot rows


def test_nipl3d_first_layer_only(lib, tmp_path):
    g = grid((5, 4, 3))
    v = values(g, 5)
    p, _ = ours(tmp_path, "n3", "3d", g, v, extr=(2, 1, 3))
    want, _ = W.other(oracle_spec(9, g, extr=(2, 1, 3)), flat(v))
    got = open(p, "rb").read()
    assert got == want
    assert got.decode().splitlines()[0] == "           5           4           3"


def shelx_grid(inc):
    # integer-stepped reflections around the origin, one row through 0 0 0
    ll = (-2.0, -1.0, -1.0)
    lr = (2.0, -1.0, -1.0)
    ul = (-2.0, 2.0, -1.0)
    tl = (-2.0, -1.0, 1.0)
    return GridData.from_corners(ll, lr if inc[0] > 1 else ll, ul if inc[1] > 1 else ll,
                                 tl if inc[2] > 1 else ll, inc=inc)


@pytest.mark.parametrize("fmt,code", [("hklf4", 6), ("list5", 7), ("list9", 8)])
@pytest.mark.parametrize("valmax", [0.0, -1.0, -2.0, 0.37])
@pytest.mark.parametrize("exti", [0.0, 0.4])
def test_shelx_3d(lib, tmp_path, fmt, code, valmax, exti):
    g = shelx_grid((5, 4, 3))
    cr = Cr()
    amp = np.abs(values(g, 6, 0.0, 400.0)) * 24 + 1.0
    ph = values(g, 7, -180.0, 180.0)
    kw = dict(valmax=valmax, f000=5000.0, exti=exti, rlambda=0.70932)
    p, fac = ours(tmp_path, "sh", fmt, g, amp, amp, ph, cr=cr, value=2, **kw)
    want, wfac = W.other(oracle_spec(code, g, value=2, rten=RTEN.reshape(-1, order="F"), icc=cr.icc, **kw),
                         flat(amp), flat(amp), flat(ph))
    assert open(p, "rb").read() == want
    assert fac == wfac
    # every reflection but 0 0 0
    assert len(want.splitlines()) == 5 * 4 * 3 - 1


@pytest.mark.parametrize("fmt,code", [("hklf4", 6), ("list5", 7), ("list9", 8)])
@pytest.mark.parametrize("inc", [(1, 4, 1), (5, 1, 1)])
@pytest.mark.parametrize("valmax", [0.0, -1.0])
def test_shelx_1d_rows(lib, tmp_path, fmt, code, inc, valmax):
    g = shelx_grid(inc)
    cr = Cr()
    v = np.abs(values(g, 8, 1.0, 900.0)) * 24
    amp = np.sqrt(v)
    ph = values(g, 9, -180.0, 180.0)
    kw = dict(valmax=valmax, f000=4000.0)
    p, fac = ours(tmp_path, "r", fmt, g, v, amp, ph, cr=cr, value=1, **kw)
    want, wfac = W.other(oracle_spec(code, g, value=1, rten=RTEN.reshape(-1, order="F"), icc=cr.icc, **kw),
                         flat(v), flat(amp), flat(ph))
    assert open(p, "rb").read() == want
    assert fac == wfac


def test_vtk_writes_the_dsi_array(lib, tmp_path):
    g = grid((4, 3, 2))
    dsi = values(g, 10)
    p, _ = ours(tmp_path, "v.vtk", "vtk", g, dsi)
    got = open(p, "rb").read()
    assert got == W.vtk(oracle_spec(11, g), flat(dsi))
    assert got.decode().splitlines()[4] == "DIMENSIONS 4 3 2"


def test_mrc_bytes(lib, tmp_path):
    g = grid((5, 4, 3))
    v = values(g, 11)
    p, _ = ours(tmp_path, "m.mrc", "mrc", g, v, ar=(0.25, 0.3, 0.2), wrez=(90.0, 91.0, 119.5), extr=(2, 3, 1))
    got = open(p, "rb").read()
    want = W.mrc(oracle_spec(12, g, ar=(0.25, 0.3, 0.2), wrez=(90.0, 91.0, 119.5), extr=(2, 3, 1)), flat(v))
    assert got == want
    assert len(got) == 4096 + 4 * 60
    assert np.frombuffer(got[:12], "<i4").tolist() == [5, 4, 3]
    assert got[208:212] == b"MAP\0"


@pytest.mark.parametrize("rng_kw", [
    {},
    {"lrange": 1, "lcenter": 1, "center": (3, 2, 2), "lpixel": 1, "pixel": (3, 2, 2)},
    {"lrange": 1},
    {"lrange": 2, "quad": "lr "},
    {"lrange": 2, "quad": "rl ", "lcenter": 1, "center": (2, 2, 2)},
])
def test_xplor(lib, tmp_path, rng_kw):
    g = grid((7, 6, 4))
    v = values(g, 12)
    p, _ = ours(tmp_path, "x", "xplor", g, v, value=1, name="my crystal", ar=(0.2, 0.25, 0.3), **rng_kw)
    want = W.xplor(oracle_spec(14, g, value=1, name="my crystal", ar=(0.2, 0.25, 0.3), **rng_kw), flat(v))
    assert open(p + ".xplor", "rb").read() == want
    p2, _ = ours(tmp_path, "y.XPLOR", "xplor", g, v, value=14)
    assert os.path.exists(p2) and not os.path.exists(p2 + ".xplor")
    assert W.xplor(oracle_spec(14, g, value=14), flat(v)) == open(p2, "rb").read()


def test_writer_argument_errors(lib, tmp_path):
    g = grid((4, 3, 1))
    v = values(g, 13)
    spec = OUT.output_spec("standard", g)
    with pytest.raises(OSError):
        OUT.write(str(tmp_path / "a"), spec, v[:2, :2])              # wrong count
    spec = OUT.output_spec("list5", g)
    with pytest.raises(OSError):
        OUT.write(str(tmp_path / "b"), spec, v, v, None)             # LIST5 needs the phase
    spec = OUT.output_spec(2, g)                                       # PGM: disabled in the reference
    with pytest.raises(OSError):
        OUT.write(str(tmp_path / "c"), spec, v)
    spec = OUT.output_spec("standard", g)
    with pytest.raises(OSError):
        OUT.write(str(tmp_path / "no_such_dir" / "d"), spec, v)     # DGPU_ERR_IO


def test_oracle_header_angles_closed_form():
    """four_angles on a cubic metric: a* x b* at 90 degrees, aver = ratio of
    the steps along the axes."""
    g = GridData.from_corners((0, 0, 0), (2, 0, 0), (0, 1, 0), inc=(5, 3, 1))
    spec = W.Spec(0, 1, g.inc, g.eck.reshape(-1, order="F"), g.vi.reshape(-1, order="F"),
                  rten=(np.eye(3) * 0.0625).reshape(-1))
    ang, avr = W.four_angles(nipl_for(g), spec)
    # do_bang divides by rad converted to default REAL: 90.0000007, printed 90.00000
    assert math.isclose(ang[0], (math.pi / 2) / float(np.float32(math.pi / 180)), rel_tol=1e-15)
    assert W.F(12, 5, ang[0]) == "    90.00000" and ang[1:] == (90.0, 90.0)
    assert math.isclose(avr[0], 1.0)


def test_shelx_overflow_and_scaling_bring_values_into_the_field(lib, tmp_path):
    """HKLF4's F8.2 overflows to asterisks for large intensities, as the
    reference's records do; scaling by the largest reflection (valmax -2)
    brings them back into the field."""
    g = shelx_grid((5, 4, 3))
    cr = Cr(icc=(1, 1, 1))
    amp = np.full(g.inc, 2000.0)                 # |F|^2 = 4e6 per cell: beyond F8.2
    ph = np.zeros(g.inc)
    p, fac = ours(tmp_path, "big", "hklf4", g, amp, amp, ph, cr=cr, value=2)
    got = open(p, "rb").read()
    assert b"********" in got
    assert got == W.other(oracle_spec(6, g, value=2, rten=RTEN.reshape(-1, order="F"), icc=cr.icc),
                          flat(amp), flat(amp), flat(ph))[0]
    p2, fac2 = ours(tmp_path, "scaled", "hklf4", g, amp, amp, ph, cr=cr, value=2, valmax=-2.0)
    assert fac2 == 10.0 ** -3 and b"*" not in open(p2, "rb").read()
