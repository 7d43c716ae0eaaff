"""Python mirror of DISCUS's `fourier` menu for the `run` path.

The menu state (discus/prog/fourier.f90:9-1062, defaults from
fourier_reset.f90:42-101) is kept in a `Fourier` object; `run()` calls the
C-ABI (dgpu_four_run) and returns csf, acsf, dsi shaped (num1, num2, num3)
in Fortran order, plus the four_qinfo values of res[].

    f = Fourier(crystal)
    f.ll, f.lr, f.ul = (-5,-5,0), (5,-5,0), (-5,5,0)
    f.nabs, f.nord = 201, 201
    f.temp = "use"
    out = f.run()
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._lib import default_context
from .structures import CrystalData, GridData, PowderSpec


@dataclass
class FourierResult:
    csf: np.ndarray
    acsf: np.ndarray
    dsi: np.ndarray
    info: _abi.Info
    status: int

    @property
    def res(self):
        """four_qinfo: res[0]=6, diffumin, diffumax, diffuave, diffusig, braggmin, braggmax."""
        return list(self.info.res)


def _cplx(buf, shape):
    return (buf[0::2] + 1j * buf[1::2]).reshape(shape, order="F")


class DiscambTables:
    """DISCAMB aspherical form factors (discus_discamb.f90:15-26): for every
    scattering type t (1..nscat) the symmetry operation numbers isymm[t-1]
    (cr_iscat(2,:) values) and one complex table per operation over integer
    h in [-maxhkl, maxhkl]^3, tables[t-1][k][h+m0, k+m1, l+m2]
    (disc_list(t)%four_form_tsc(h,k,l,k), discamb_set_form_tsc :447-546).
    attach(opts) points opts at the flattened copy."""

    def __init__(self, maxhkl, isymm, tables):
        self.maxhkl = tuple(int(m) for m in maxhkl)
        self.isymm = [list(int(y) for y in ys) for ys in isymm]
        shape = tuple(2 * m + 1 for m in self.maxhkl)
        flat = []
        for ts, ys in zip(tables, self.isymm):
            assert len(ts) == len(ys)
            for tab in ts:
                tab = np.asarray(tab, dtype=np.complex128)
                assert tab.shape == shape, (tab.shape, shape)
                flat.append(np.stack([tab.real, tab.imag], -1).transpose(2, 1, 0, 3).ravel())
        self.tables = [[np.asarray(t, dtype=np.complex128) for t in ts] for ts in tables]
        self._nsymm = np.asarray([len(ys) for ys in self.isymm], np.int32)
        self._isymm = np.asarray([y for ys in self.isymm for y in ys] or [0], np.int32)
        self._tsc = np.ascontiguousarray(np.concatenate(flat) if flat else np.zeros(2))
        self._c = _abi.Discamb()
        for k in range(3):
            self._c.maxhkl[k] = self.maxhkl[k]
        self._c.nsymm = _abi.iptr(self._nsymm)
        self._c.isymm = _abi.iptr(self._isymm)
        self._c.form_tsc = _abi.dptr(self._tsc)

    def attach(self, opts: _abi.Opts):
        """Points opts at the tables; opts keeps this object (and so the
        host arrays the library copies from) alive."""
        opts.discamb = C.pointer(self._c)
        opts._discamb_owner = self
        return self

    def value(self, t, k, hkl):
        """Table k (0-based) of type t (1-based) at integer hkl (nint of each component)."""
        ijk = tuple(int(np.sign(x) * np.floor(abs(x) + 0.5)) + m for x, m in zip(hkl, self.maxhkl))
        return self.tables[t - 1][k][ijk]


def attach_selections(opts: _abi.Opts, aver_cells=None, lot_origins=None):
    """Points opts at the caller's random draws: the <F> cell selection
    cells(csize1,csize2,csize3) (fourier_sup.f90:1235-1241) and the lot origins
    lbeg(3,nlots), 1-based (four_ranloc, fourier_sup.f90:2513-2530).  Returns
    the arrays, which must stay alive while opts is used."""
    keep = []
    if aver_cells is not None:
        a = np.ascontiguousarray(np.asarray(aver_cells, dtype=np.uint8).reshape(-1, order="F"))
        opts.aver_cells = a.ctypes.data_as(C.POINTER(C.c_uint8))
        keep.append(a)
    if lot_origins is not None:
        o = np.ascontiguousarray(np.asarray(lot_origins, dtype=np.int32).reshape(-1, 3))
        opts.lot_origins = _abi.iptr(o)
        opts.nlots = o.shape[0]
        keep.append(o)
    return keep


def four_run(cr: CrystalData, grid: GridData, opts: _abi.Opts, ctx=None, aver_cells=None, lot_origins=None):
    """four_run (discus/prog/fourier_sup.f90:11-323) on the GPU."""
    ctx = ctx or default_context()
    np_ = grid.npoints
    csf = np.zeros(2 * np_)
    acsf = np.zeros(2 * np_)
    dsi = np.zeros(np_)
    info = _abi.Info()
    c = cr.to_c()
    g = grid.to_c()
    keep = attach_selections(opts, aver_cells, lot_origins)
    rc = ctx.check(ctx.lib.dgpu_four_run(ctx.h, C.byref(c), C.byref(g), C.byref(opts), _abi.dptr(csf),
                                         _abi.dptr(acsf), _abi.dptr(dsi), C.byref(info)))
    del keep
    shp = grid.inc
    return FourierResult(_cplx(csf, shp), _cplx(acsf, shp), dsi.reshape(shp, order="F"), info, rc)


def calc_000(cr: CrystalData, opts: _abi.Opts, rhkl, ctx=None):
    """calc_000 (fourier_sup.f90:3149-3226): four_run at the single point
    rhkl (inc 1 1 1, every corner rhkl, vi = 0); res_para(0:4) = 4, Re F,
    Im F and both per unit cell (divided by cr_icc(1) cr_icc(2) cr_icc(3)).
    For a single point fourier_lmn keeps only the nearest integers of the
    corner (identity offsets), so in PHASE_REF22 the phases are those of the
    rounded hkl while istl (the form factors) follows rhkl itself, as in the
    reference; PHASE_EXACT64 takes the phases at rhkl."""
    h = np.asarray(rhkl, dtype=np.float64).reshape(3)
    grid = GridData(eck=np.repeat(h[:, None], 4, axis=1), vi=np.zeros((3, 3)), inc=(1, 1, 1))
    f = complex(four_run(cr, grid, opts, ctx=ctx).csf.reshape(-1)[0])
    ncell = float(cr.icc[0]) * float(cr.icc[1]) * float(cr.icc[2])
    return [4.0, f.real, f.imag, f.real / ncell, f.imag / ncell]


def four_weight(cr: CrystalData, grid: GridData, dsi, opts: _abi.Opts, ctx=None):
    """four_weight (fourier_sup.f90:1428-1643): the dsi3d copy of dsi with
    the Bragg points re-weighted."""
    ctx = ctx or default_context()
    d = np.asfortranarray(dsi, dtype=np.float64).reshape(-1, order="F").copy()
    out = np.zeros_like(d)
    c = cr.to_c()
    g = grid.to_c()
    ctx.check(ctx.lib.dgpu_four_weight(ctx.h, C.byref(c), C.byref(g), C.byref(opts), _abi.dptr(d),
                                       _abi.dptr(out)))
    return out.reshape(grid.inc, order="F")


def four_accumulate(mode, grid: GridData, csf=None, dsi=None, fave=0.0, symm=0, ctx=None):
    """four_accumulate (fourier_sup.f90:3784-3840).  ACCUM adds csf/dsi to the
    context's sums; FINISHED returns (csf_sum, dsi_sum) and clears them."""
    ctx = ctx or default_context()
    g = grid.to_c()
    np_ = grid.npoints
    if csf is None:
        cbuf, dbuf = np.zeros(2 * np_), np.zeros(np_)
    else:
        z = np.asfortranarray(csf).reshape(-1, order="F")
        cbuf = np.empty(2 * np_)
        cbuf[0::2], cbuf[1::2] = z.real, z.imag
        dbuf = np.asfortranarray(dsi, dtype=np.float64).reshape(-1, order="F").copy()
    ctx.check(ctx.lib.dgpu_four_accumulate(ctx.h, int(mode), int(symm), C.byref(g), float(fave),
                                           _abi.dptr(cbuf), _abi.dptr(dbuf)))
    return _cplx(cbuf, grid.inc), dbuf.reshape(grid.inc, order="F")


def set_symmetry(mats, ctx=None):
    """The point-group operations of four_symm (spc_mat(1:3,1:3,1:nops), the
    first the identity): an array (nops, 3, 3) of integer matrices."""
    ctx = ctx or default_context()
    m = np.asarray(mats, dtype=np.float64).reshape(-1, 3, 3)
    flat = np.ascontiguousarray(np.transpose(m, (0, 2, 1)).reshape(-1))     # column-major per matrix
    ctx.check(ctx.lib.dgpu_set_symmetry(ctx.h, int(m.shape[0]), _abi.dptr(flat)))


def _interleave(z):
    z = np.asfortranarray(z).reshape(-1, order="F")
    b = np.empty(2 * z.size)
    b[0::2], b[1::2] = z.real, z.imag
    return b


def four_filter(dsi, opts: _abi.Opts, ctx=None):
    """do_four_filter (fourier_sup.f90:1646-1803) on a copy of dsi(num), on
    the device (dgpu_four_filter): the Lanczos filter set by opts.filter,
    filter_width, filter_damp, filter_scale."""
    ctx = ctx or default_context()
    d = np.asfortranarray(np.asarray(dsi, dtype=np.float64))
    shape = d.shape + (1,) * (3 - d.ndim)
    flat = d.reshape(-1, order="F").copy()
    num = np.asarray(shape, dtype=np.int32)
    ctx.check(ctx.lib.dgpu_four_filter(ctx.h, _abi.iptr(num), C.byref(opts), _abi.dptr(flat)))
    return flat.reshape(d.shape, order="F")


def qval(cr: CrystalData, grid: GridData, opts: _abi.Opts, value, result: FourierResult, laver=False,
         rand=None, ctx=None):
    """qval (discus/prog/qval.f90:65-290) on the device: the output value of
    every grid point from a FourierResult (csf, acsf, dsi)."""
    ctx = ctx or default_context()
    c = cr.to_c()
    g = grid.to_c()
    csf = _interleave(result.csf)
    acsf = _interleave(result.acsf)
    dsi = np.asfortranarray(result.dsi, dtype=np.float64).reshape(-1, order="F").copy()
    rnd = None if rand is None else np.asfortranarray(rand, dtype=np.float64).reshape(-1, order="F").copy()
    out = np.zeros(grid.npoints)
    ctx.check(ctx.lib.dgpu_qval(ctx.h, C.byref(c), C.byref(g), C.byref(opts), int(value), int(bool(laver)),
                                _abi.dptr(csf), _abi.dptr(acsf), _abi.dptr(dsi), _abi.dptr(rnd), _abi.dptr(out)))
    return out.reshape(grid.inc, order="F")


def calc_hkl(cr: CrystalData, opts: _abi.Opts, hkl, scale=1.0, exti=0.0, rlambda=0.70932, ctx=None):
    """calc_hkl (fourier_sup.f90:3230-3549) core on the device: (icalc, sigi,
    phase) at the integer reflections hkl (n, 3)."""
    ctx = ctx or default_context()
    h = np.ascontiguousarray(np.asarray(hkl, dtype=np.int32).reshape(-1, 3))
    n = h.shape[0]
    ic, sg, ph = np.zeros(n), np.zeros(n), np.zeros(n)
    c = cr.to_c()
    ctx.check(ctx.lib.dgpu_calc_hkl(ctx.h, C.byref(c), C.byref(opts), _abi.iptr(h), n, float(scale), float(exti),
                                    float(rlambda), _abi.dptr(ic), _abi.dptr(sg), _abi.dptr(ph)))
    return ic, sg, ph


def powder_complete(cr: CrystalData, pw: PowderSpec, opts: _abi.Opts, ctx=None):
    """powder_complete (discus/prog/powder.f90:1829-2593), pow_four_mode =
    fourier, on the device: (pow_qsp[0..n_pkt], info)."""
    ctx = ctx or default_context()
    p = pw.to_c()
    n = ctx.lib.dgpu_powder_npkt(C.byref(p))
    if n < 0:
        raise ValueError("invalid Q range")
    qsp = np.zeros(n + 1)
    info = _abi.PowderInfo()
    c = cr.to_c()
    ctx.check(ctx.lib.dgpu_powder_complete(ctx.h, C.byref(c), C.byref(p), C.byref(opts), _abi.dptr(qsp),
                                           C.byref(info)))
    return qsp, info


def fourier_lmn(eck, vi, inc, ctx=None):
    """fourier_lmn (discus/prog/fourier_lmn_mod.f90:4-280): (rc, lmn[6], off_shift(3,3))."""
    ctx = ctx or default_context()
    e = np.asarray(eck, dtype=np.float64).reshape(-1, order="F").copy()
    v = np.asarray(vi, dtype=np.float64).reshape(-1, order="F").copy()
    i = np.asarray(inc, dtype=np.int32).copy()
    lmn = np.zeros(6, np.int32)
    off = np.zeros(9)
    rc = ctx.lib.dgpu_fourier_lmn(_abi.dptr(e), _abi.dptr(v), _abi.iptr(i), _abi.iptr(lmn), _abi.dptr(off))
    return rc, lmn, off.reshape(3, 3, order="F")


def four_stltab(grid: GridData, rten, ctx=None):
    """four_stltab (fourier_sup.f90:2637-2687) on the device: (rc, istl)."""
    ctx = ctx or default_context()
    g = grid.to_c()
    rt = np.asarray(rten, dtype=np.float64).reshape(-1, order="F").copy()
    istl = np.zeros(grid.npoints, np.int32)
    rc = ctx.lib.dgpu_four_stltab(ctx.h, C.byref(g), _abi.dptr(rt), _abi.iptr(istl))
    return rc, istl.reshape(grid.inc, order="F")


def four_formtab(cr: CrystalData, opts, ctx=None):
    """four_formtab (fourier_sup.f90:2691-2743): cfact (nscat, CFPKT+1) complex."""
    ctx = ctx or default_context()
    c = cr.to_c()
    out = np.zeros(2 * cr.nscat * (_abi.CFPKT + 1))
    ctx.check(ctx.lib.dgpu_four_formtab(ctx.h, C.byref(c), C.byref(opts), _abi.dptr(out)))
    return (out[0::2] + 1j * out[1::2]).reshape(cr.nscat, _abi.CFPKT + 1)


def four_increments(xat, uin, vin, win, off, ctx=None):
    """Per-atom REF22 increments (four_strucf_OMP_mod.f90:135-149): int64 (6, n)."""
    ctx = ctx or default_context()
    x = np.asfortranarray(xat, dtype=np.float64)
    n = x.shape[0]
    out = np.zeros(6 * max(n, 1), np.int64)
    u, v, w = (np.asarray(a, dtype=np.float64).copy() for a in (uin, vin, win))
    o = np.asarray(off, dtype=np.float64).reshape(-1, order="F").copy()
    ctx.check(ctx.lib.dgpu_four_increments(ctx.h, x.ctypes.data_as(C.POINTER(C.c_double)), n, _abi.dptr(u),
                                           _abi.dptr(v), _abi.dptr(w), _abi.dptr(o),
                                           out.ctypes.data_as(C.POINTER(C.c_int64))))
    return out[: 6 * n].reshape(6, n)


def four_strucf(xat, uin, vin, win, off, lmn, num, fnum, cfact=None, istl=None, ctx=None):
    """four_strucf (four_strucf_OMP_mod.f90:19-68) + tcsf_form_iso: tcsf(num)."""
    ctx = ctx or default_context()
    x = np.asfortranarray(xat, dtype=np.float64)
    n = x.shape[0]
    u, v, w = (np.asarray(a, dtype=np.float64).copy() for a in (uin, vin, win))
    o = np.asarray(off, dtype=np.float64).reshape(-1, order="F").copy()
    lm = np.asarray(lmn, dtype=np.int32).copy()
    nm = np.asarray(num, dtype=np.int32).copy()
    fn = np.asarray(fnum, dtype=np.int32).copy()
    np_ = int(np.prod(num))
    out = np.zeros(2 * np_)
    cf = None
    ist = None
    if cfact is not None:
        cf = np.ascontiguousarray(np.stack([np.real(cfact), np.imag(cfact)], -1).ravel())
        ist = np.asfortranarray(istl, dtype=np.int32).reshape(-1, order="F").copy()
    ctx.check(ctx.lib.dgpu_four_strucf(ctx.h, x.ctypes.data_as(C.POINTER(C.c_double)), n, _abi.dptr(u),
                                       _abi.dptr(v), _abi.dptr(w), _abi.dptr(o), _abi.iptr(lm), _abi.iptr(nm),
                                       _abi.iptr(fn), _abi.dptr(cf), _abi.iptr(ist), _abi.dptr(out)))
    return _cplx(out, tuple(num))


def batch_run(crystals, grids, opts, targets=None, weights=None, ctx=None):
    """A population of crystals in one captured launch sequence
    (dgpu_batch_run; options outside the graph run member by member).
    Returns (dsi list, chi2 array or None, grad_pos list, grad_occ list, ms
    of the graph launch or of the member loop)."""
    ctx = ctx or default_context()
    n = len(crystals)
    crs = (_abi.Crystal * n)(*[c.to_c() for c in crystals])
    grs = (_abi.Grid * n)(*[g.to_c() for g in grids])
    dp = C.POINTER(C.c_double)
    dsi = [np.zeros(g.npoints) for g in grids]
    dsi_p = (dp * n)(*[_abi.dptr(d) for d in dsi])
    it_p = wt_p = gp_p = go_p = None
    chi2 = None
    gps, gos = [], []
    keep = []
    if targets is not None:
        its = [np.asfortranarray(np.asarray(t, np.float64)).reshape(-1, order="F").copy() for t in targets]
        keep += its
        it_p = (dp * n)(*[_abi.dptr(t) for t in its])
        if weights is not None:
            wts = [np.asfortranarray(np.asarray(w, np.float64)).reshape(-1, order="F").copy() for w in weights]
            keep += wts
            wt_p = (dp * n)(*[_abi.dptr(w) for w in wts])
        chi2 = np.zeros(n)
        gps = [np.zeros(3 * c.natoms) for c in crystals]
        gos = [np.zeros(c.natoms) for c in crystals]
        gp_p = (dp * n)(*[_abi.dptr(x) for x in gps])
        go_p = (dp * n)(*[_abi.dptr(x) for x in gos])
    ctx.check(ctx.lib.dgpu_batch_run(ctx.h, n, crs, grs, C.byref(opts), dsi_p, it_p, wt_p,
                                     _abi.dptr(chi2), gp_p, go_p))
    ms = ctx.lib.dgpu_batch_last_ms(ctx.h)
    dsi = [d.reshape(g.inc, order="F") for d, g in zip(dsi, grids)]
    return dsi, chi2, [x.reshape(-1, 3) for x in gps], gos, ms


def batch_graph_nodes(ctx=None):
    """(all nodes, kernel nodes) of the graph the last batch_run launched."""
    ctx = ctx or default_context()
    k = C.c_int64(0)
    n = ctx.lib.dgpu_batch_graph_nodes(ctx.h, C.byref(k))
    return int(n), int(k.value)


class Fourier:
    """Menu state of `fourier` with its reset defaults (fourier_reset.f90:42-101)."""

    def __init__(self, crystal: CrystalData):
        self.crystal = crystal
        self.ll = (0.0, 0.0, 0.0)
        self.lr = (5.0, 0.0, 0.0)
        self.ul = (0.0, 5.0, 0.0)
        self.tl = None
        self.nabs, self.nord, self.ntop = 121, 121, 1
        self.radiation = "xray"     # xray | neut
        self.power = 4
        self.temp = "ignore"        # use | ignore
        self.aver = 0.0             # set aver
        self.friedel = True         # set friedel
        self.anomalous = False
        self.scale = 1.0
        self.phase = _abi.PHASE_EXACT64
        self.form = _abi.FORM_TABLE
        self.engine = _abi.ENGINE_AUTO

    def grid(self) -> GridData:
        return GridData.from_corners(self.ll, self.lr, self.ul, self.tl, inc=(self.nabs, self.nord, self.ntop))

    def opts(self) -> _abi.Opts:
        return _abi.default_opts(lxray=int(self.radiation == "xray"), power=self.power,
                                 ano=int(self.anomalous), ldbw=int(self.temp == "use"),
                                 friedel=int(self.friedel), fave=float(self.aver), diff_scale=self.scale,
                                 phase=self.phase, form=self.form, engine=self.engine)

    def run(self, ctx=None, aver_cells=None) -> FourierResult:
        return four_run(self.crystal, self.grid(), self.opts(), ctx=ctx, aver_cells=aver_cells)
