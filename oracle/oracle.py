"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU legs as the
reference for comparisons / timed CPU baseline; never by the product package.
Parity unpinned (see discus_oracle.h).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from diffusecode_gb300 import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
# the same source built with the reference's release flags (-O3 -ffast-math,
# OpenMP): only for timing the reference's loops (bench CPU legs)
_TLIB = os.path.join(_HERE, "_build", "liboracle_timing.so")
_lib = None
_tlib = None


def build():
    subprocess.check_call(["sh", os.path.join(_HERE, "build_oracle.sh")])


def lib():
    global _lib
    if _lib is None:
        _lib = _load(_LIB)
    return _lib


def timing_lib():
    """The oracle built with the reference's release flags; its results are
    not checked, only its time is used."""
    global _tlib
    if _tlib is None:
        _tlib = _load(_TLIB)
    return _tlib


def _load(path):
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    dp, ip, fp = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_float)
    L.oc_fourier_lmn.argtypes = [dp, dp, ip, ip, dp]
    L.oc_cexpt.argtypes = [dp]
    L.oc_stltab.argtypes = [dp, dp, ip, dp, ip]
    L.oc_formtab.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Opts), dp]
    L.oc_increments.argtypes = [dp, C.c_int64, dp, dp, dp, dp, C.POINTER(C.c_int64)]
    L.oc_four_strucf.argtypes = [dp, C.c_int64, dp, dp, dp, dp, ip, ip, ip, dp, ip, dp]
    L.oc_four_run.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Grid), C.POINTER(_abi.Opts),
                              dp, dp, dp, C.POINTER(_abi.Info), C.c_int]
    L.oc_chi2_grad.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Grid), C.POINTER(_abi.Opts),
                               dp, dp, dp, dp, dp, C.c_int]
    L.oc_time_ref_rows.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Grid), C.c_int32,
                                   C.c_int32, C.c_int, C.POINTER(C.c_int64)]
    L.oc_time_ref_rows.restype = C.c_double
    L.oc_four_weight.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Grid), C.POINTER(_abi.Opts),
                                 dp, dp, dp]
    L.oc_fill_bragg.argtypes = [C.POINTER(_abi.Grid), dp, C.c_int]
    L.oc_fill_bragg.restype = None
    L.oc_four_symm.argtypes = [C.POINTER(_abi.Grid), C.c_int32, dp, dp, C.c_int]
    L.oc_four_symm.restype = None
    L.oc_calc_hkl.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Opts), C.POINTER(C.c_int32), C.c_int64,
                              C.c_double, C.c_double, C.c_double, dp, dp, dp, C.c_int]
    L.oc_qval.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Grid), C.POINTER(_abi.Opts), C.c_int,
                          C.c_int, dp, dp, dp, dp, dp]
    L.oc_powder_npkt.argtypes = [C.POINTER(_abi.Powder)]
    L.oc_powder_complete.argtypes = [C.POINTER(_abi.Crystal), C.POINTER(_abi.Powder), C.POINTER(_abi.Opts),
                                     C.c_int64, C.c_int64, dp, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                     C.c_int]
    return L


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def fourier_lmn(eck, vi, inc):
    eck = np.asfortranarray(eck, dtype=np.float64).reshape(-1, order="F").copy()
    vi = np.asfortranarray(vi, dtype=np.float64).reshape(-1, order="F").copy()
    inc = np.asarray(inc, dtype=np.int32).copy()
    lmn = np.zeros(6, np.int32)
    off = np.zeros(9, np.float64)
    rc = lib().oc_fourier_lmn(_d(eck), _d(vi), _i(inc), _i(lmn), _d(off))
    return rc, lmn, off.reshape(3, 3, order="F")


def cexpt():
    cex = np.zeros(2 * _abi.I2PI)
    lib().oc_cexpt(_d(cex))
    return cex[0::2] + 1j * cex[1::2]


def stltab(grid, rten):
    g = grid.to_c()
    eck = np.array(g.eck[:], dtype=np.float64)
    vi = np.array(g.vi[:], dtype=np.float64)
    num = np.array(grid.inc, dtype=np.int32)
    rt = np.asarray(rten, dtype=np.float64).reshape(-1, order="F").copy()
    istl = np.zeros(int(np.prod(grid.inc)), np.int32)
    rc = lib().oc_stltab(_d(eck), _d(vi), _i(num), _d(rt), _i(istl))
    return rc, istl.reshape(grid.inc, order="F")


def formtab(cr, opts):
    c = cr.to_c()
    out = np.zeros(2 * (_abi.CFPKT + 1) * cr.nscat)
    lib().oc_formtab(C.byref(c), C.byref(opts), _d(out))
    z = out[0::2] + 1j * out[1::2]
    return z.reshape(cr.nscat, _abi.CFPKT + 1)


def increments(xat, uin, vin, win, off):
    """xat (n,3) -> int64 (6,n): iincu, iincv, iincw, jincu, jincv, jincw."""
    x = np.asfortranarray(xat, dtype=np.float64)
    n = x.shape[0]
    out = np.zeros(6 * n, np.int64)
    u, v, w = (np.asarray(a, dtype=np.float64).copy() for a in (uin, vin, win))
    o = np.asarray(off, dtype=np.float64).reshape(-1, order="F").copy()
    lib().oc_increments(_d(x), n, _d(u), _d(v), _d(w), _d(o), out.ctypes.data_as(C.POINTER(C.c_int64)))
    return out.reshape(6, n)


def four_strucf(xat, uin, vin, win, off, lmn, num, fnum, cfact=None, istl=None):
    x = np.asfortranarray(xat, dtype=np.float64)
    n = x.shape[0]
    u, v, w = (np.asarray(a, dtype=np.float64).copy() for a in (uin, vin, win))
    o = np.asarray(off, dtype=np.float64).reshape(-1, order="F").copy()
    lm = np.asarray(lmn, dtype=np.int32).copy()
    nm = np.asarray(num, dtype=np.int32).copy()
    fn = np.asarray(fnum, dtype=np.int32).copy()
    np_ = int(np.prod(num))
    out = np.zeros(2 * np_)
    cf = None if cfact is None else np.ascontiguousarray(np.stack([cfact.real, cfact.imag], -1).ravel())
    ist = None if istl is None else np.asfortranarray(istl, dtype=np.int32).reshape(-1, order="F").copy()
    lib().oc_four_strucf(_d(x), n, _d(u), _d(v), _d(w), _d(o), _i(lm), _i(nm), _i(fn),
                         _d(cf) if cf is not None else None, _i(ist) if ist is not None else None, _d(out))
    return (out[0::2] + 1j * out[1::2]).reshape(num, order="F")


def four_run(cr, grid, opts, nthreads=0, aver_cells=None, lot_origins=None):
    """Returns (rc, csf, acsf, dsi, info); arrays shaped grid.inc (Fortran order)."""
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    keep = []
    if aver_cells is not None:
        a = np.ascontiguousarray(np.asarray(aver_cells, dtype=np.uint8).reshape(-1, order="F"))
        opts.aver_cells = a.ctypes.data_as(C.POINTER(C.c_uint8))
        keep.append(a)
    if lot_origins is not None:
        o = np.ascontiguousarray(np.asarray(lot_origins, dtype=np.int32).reshape(-1, 3))
        opts.lot_origins = _i(o)
        opts.nlots = o.shape[0]
        keep.append(o)
    c = cr.to_c()
    g = grid.to_c()
    np_ = grid.npoints
    csf = np.zeros(2 * np_)
    acsf = np.zeros(2 * np_)
    dsi = np.zeros(np_)
    info = _abi.Info()
    rc = lib().oc_four_run(C.byref(c), C.byref(g), C.byref(opts), _d(csf), _d(acsf), _d(dsi),
                           C.byref(info), nthreads)
    del keep
    shp = grid.inc
    return (rc, (csf[0::2] + 1j * csf[1::2]).reshape(shp, order="F"),
            (acsf[0::2] + 1j * acsf[1::2]).reshape(shp, order="F"),
            dsi.reshape(shp, order="F"), info)


def chi2_grad(cr, grid, opts, i_target, weight=None, nthreads=0, aver_cells=None, lot_origins=None):
    """(chi2, grad_pos (N,3), grad_occ (N,)) in FP64; with opts.fave > 0 the
    <F> of the selected cells (aver_cells over csize when fave < 1) is
    subtracted from F as four_run does."""
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    keep = []
    if aver_cells is not None:
        a = np.ascontiguousarray(np.asarray(aver_cells, dtype=np.uint8).reshape(-1, order="F"))
        opts.aver_cells = a.ctypes.data_as(C.POINTER(C.c_uint8))
        keep.append(a)
    if lot_origins is not None:
        o = np.ascontiguousarray(np.asarray(lot_origins, dtype=np.int32).reshape(-1, 3))
        opts.lot_origins = _i(o)
        opts.nlots = o.shape[0]
        keep.append(o)
    c = cr.to_c()
    g = grid.to_c()
    it = np.asfortranarray(i_target, dtype=np.float64).reshape(-1, order="F").copy()
    wt = None if weight is None else np.asfortranarray(weight, dtype=np.float64).reshape(-1, order="F").copy()
    chi2 = np.zeros(1)
    gp = np.zeros(3 * cr.natoms)
    go = np.zeros(cr.natoms)
    rc = lib().oc_chi2_grad(C.byref(c), C.byref(g), C.byref(opts), _d(it),
                            _d(wt) if wt is not None else None, _d(chi2), _d(gp), _d(go), nthreads)
    del keep
    assert rc == 0
    return float(chi2[0]), gp.reshape(-1, 3), go


def time_ref_rows(cr, grid, row_lo, row_hi, nthreads=0, natoms=None):
    """Seconds and pairs for the REF22 type sums over abscissa rows [lo,hi)
    (over the first natoms atoms when given), in the build with the
    reference's release flags."""
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    c = cr.to_c()
    if natoms is not None:
        c.natoms = min(int(natoms), int(c.natoms))
    g = grid.to_c()
    pairs = C.c_int64(0)
    sec = timing_lib().oc_time_ref_rows(C.byref(c), C.byref(g), int(row_lo), int(row_hi), int(nthreads),
                                 C.byref(pairs))
    return sec, int(pairs.value)


def four_weight(cr, grid, dsi, opts):
    """(dsi3d, scalef) of four_weight."""
    c = cr.to_c()
    g = grid.to_c()
    d = np.asfortranarray(dsi, dtype=np.float64).reshape(-1, order="F").copy()
    out = np.zeros_like(d)
    sc = np.zeros(1)
    lib().oc_four_weight(C.byref(c), C.byref(g), C.byref(opts), _d(d), _d(out), _d(sc))
    return out.reshape(grid.inc, order="F"), float(sc[0])


def four_symm(grid, arr, mats):
    """four_symm_csf / four_symm_dsi on a grid array (real or complex, shaped
    grid.inc); mats (nops, 3, 3), the first the identity."""
    g = grid.to_c()
    m = np.asarray(mats, dtype=np.float64).reshape(-1, 3, 3)
    flat = np.ascontiguousarray(np.transpose(m, (0, 2, 1)).reshape(-1))
    a = np.asfortranarray(arr).reshape(-1, order="F")
    if np.iscomplexobj(a):
        buf = np.empty(2 * a.size)
        buf[0::2], buf[1::2] = a.real, a.imag
        lib().oc_four_symm(C.byref(g), m.shape[0], _d(flat), _d(buf), 2)
        return (buf[0::2] + 1j * buf[1::2]).reshape(grid.inc, order="F")
    buf = np.ascontiguousarray(a, dtype=np.float64).copy()
    lib().oc_four_symm(C.byref(g), m.shape[0], _d(flat), _d(buf), 1)
    return buf.reshape(grid.inc, order="F")


def fill_bragg(grid, arr):
    """four_fill_csf / four_fill_dsi (fave < 0) on a copy of arr."""
    g = grid.to_c()
    if np.iscomplexobj(arr):
        z = np.asfortranarray(arr).reshape(-1, order="F")
        buf = np.empty(2 * z.size)
        buf[0::2], buf[1::2] = z.real, z.imag
        lib().oc_fill_bragg(C.byref(g), _d(buf), 2)
        return (buf[0::2] + 1j * buf[1::2]).reshape(grid.inc, order="F")
    buf = np.asfortranarray(arr, dtype=np.float64).reshape(-1, order="F").copy()
    lib().oc_fill_bragg(C.byref(g), _d(buf), 1)
    return buf.reshape(grid.inc, order="F")


def qval(cr, grid, opts, value, csf, acsf, dsi, laver=False, rand=None):
    """qval of every grid point (arrays shaped grid.inc, Fortran order)."""
    c = cr.to_c()
    g = grid.to_c()
    def il(z):
        z = np.asfortranarray(z).reshape(-1, order="F")
        b = np.empty(2 * z.size)
        b[0::2], b[1::2] = z.real, z.imag
        return b
    cs, ac = il(csf), il(acsf)
    d = np.asfortranarray(dsi, dtype=np.float64).reshape(-1, order="F").copy()
    rn = None if rand is None else np.asfortranarray(rand, dtype=np.float64).reshape(-1, order="F").copy()
    out = np.zeros(grid.npoints)
    rc = lib().oc_qval(C.byref(c), C.byref(g), C.byref(opts), int(value), int(bool(laver)), _d(cs), _d(ac),
                       _d(d), _d(rn) if rn is not None else None, _d(out))
    return rc, out.reshape(grid.inc, order="F")


def calc_hkl(cr, opts, hkl, scale=1.0, exti=0.0, rlambda=0.70932, nthreads=0):
    """(rc, icalc, sigi, phase) at the reflections hkl (n, 3)."""
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    h = np.ascontiguousarray(np.asarray(hkl, dtype=np.int32).reshape(-1, 3))
    n = h.shape[0]
    ic, sg, ph = np.zeros(n), np.zeros(n), np.zeros(n)
    c = cr.to_c()
    rc = lib().oc_calc_hkl(C.byref(c), C.byref(opts), h.ctypes.data_as(C.POINTER(C.c_int32)), n, float(scale),
                           float(exti), float(rlambda), _d(ic), _d(sg), _d(ph), nthreads)
    return rc, ic, sg, ph


def powder_complete(cr, pw, opts, rod_lo=-1, rod_hi=-1, nthreads=0, timing=False):
    """powder_complete (powder.f90:1829-2593), literal rod loop: (rc, pow_qsp,
    rods, rod points evaluated).  rod_lo/rod_hi restrict the evaluation to
    the rods [rod_lo, rod_hi) of the reference's loop order (a bounded CPU
    sample); the half-volume doubling is applied either way.  timing: run
    the build with the reference's release flags (for timing only)."""
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    L = timing_lib() if timing else lib()
    p = pw.to_c()
    n = L.oc_powder_npkt(C.byref(p))
    if n < 0:
        return -1, None, 0, 0
    qsp = np.zeros(n + 1)
    c = cr.to_c()
    nr, npts = C.c_int64(0), C.c_int64(0)
    rc = L.oc_powder_complete(C.byref(c), C.byref(p), C.byref(opts), int(rod_lo), int(rod_hi), _d(qsp),
                                  C.byref(nr), C.byref(npts), nthreads)
    return rc, qsp, nr.value, npts.value


def lut_floor_tol(grid, lmn):
    """Tolerance of a comparison with the reference's table arithmetic
    (four_strucf_OMP_mod.f90:143-148,169): the 2^-16-turn table index is a
    truncation (uniform phase error, rms 2^-16/sqrt(12) turn; its mean is a
    phase common to all atoms and drops out of |F|^2) and each 2^-22-turn
    increment is rounded (+-2^-23 turn, times the point's index from the
    origin of the increments, lmn + n, largest at a corner of the grid).  A
    random per-atom phase error of
    rms sigma moves |F|^2 by at most ~ sigma times a Gaussian in units of
    I + N<|f|^2>; the tolerance is six sigma."""
    import numpy as _np
    n = _np.array([max(abs(lmn[k]), abs(lmn[k] + grid.inc[k] - 1)) for k in range(3)], float)
    s_tab = 2 ** -16 / _np.sqrt(12.0)
    s_inc = 2 ** -23 * _np.sqrt(_np.sum(n ** 2) / 3.0)
    return float(6.0 * 2 * _np.pi * _np.hypot(s_tab, s_inc))
