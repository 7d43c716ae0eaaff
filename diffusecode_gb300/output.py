"""The output menu's file writers and calc_hkl's files through the C-ABI
(dgpu_output_write, dgpu_calc_hkl_files; the writers are host code of the
library, the values come from qval on the device).

Mirrors discus/prog/graphic.f90's `output` menu: `format` is the menu's
format (standard, gnuplot, hklf4, list5, list9, 3d, vtk, mrc, hdf5, xplor), the
grid the last Fourier's (out_inc, out_eck, out_vi), `value` the qval code.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._lib import default_context, load

FORMATS = {"standard": _abi.OUT_STANDARD, "gnuplot": _abi.OUT_GNUPLOT, "hklf4": _abi.OUT_HKLF4,
           "shelx": _abi.OUT_HKLF4, "list5": _abi.OUT_LIST5, "list9": _abi.OUT_LIST9, "3d": _abi.OUT_NIPL3D,
           "vtk": _abi.OUT_VTK, "mrc": _abi.OUT_MRC, "hdf5": _abi.OUT_HDF5, "xplor": _abi.OUT_XPLOR}


def _flat(a):
    return None if a is None else np.asfortranarray(a, dtype=np.float64).reshape(-1, order="F").copy()


def nipl_info(cr, grid, four_last=None, lots=False, radiation=1, rlambda=0.70932, lambda_name="", ldbw=False,
              ano=False, names=None, amount=None):
    """write_discus_nipl_header's crystal and Fourier data (dict): names
    cr_at_lis(0:nscat) (default VOID and T1..), amount cr_amount(0:nscat)
    (default: the atom count per type); four_last as the fourier menu sets
    it (fourier.f90:733-742): the number of axes with inc > 1, negative
    with lots."""
    ns = int(cr.nscat)
    if four_last is None:
        four_last = sum(1 for x in grid.inc if x > 1) * (-1 if lots else 1)
    if names is None:
        names = ["VOID"] + [f"T{t}" for t in range(1, ns + 1)]
    if amount is None:
        amount = np.bincount(np.asarray(cr.iscat), minlength=ns + 1)[:ns + 1]
    return {"natoms": int(cr.iscat.shape[0]), "nscat": ns, "ncatoms": int(cr.ncatoms),
            "at_lis": [str(x) for x in names], "amount": [int(x) for x in amount],
            "dw": [float(x) for x in cr.dw[:ns + 1]], "four_last": int(four_last), "radiation": int(radiation),
            "rlambda": float(rlambda), "lambda": lambda_name, "ldbw": int(bool(ldbw)), "ano": int(bool(ano)),
            "inc": list(grid.inc), "eck": list(grid.eck.reshape(-1, order="F")),
            "vi": list(grid.vi.reshape(-1, order="F"))}


def _nipl_c(n, keep):
    s = _abi.Nipl()
    s.natoms, s.nscat, s.ncatoms = n["natoms"], n["nscat"], n["ncatoms"]
    names = b"".join(x.encode()[:4].ljust(4) for x in n["at_lis"])
    amount = np.asarray(n["amount"], dtype=np.int64)
    dw = np.asarray(n["dw"], dtype=np.float64)
    lam = n["lambda"].encode()
    keep += [names, amount, dw, lam]
    s.at_lis = names
    s.amount = amount.ctypes.data_as(C.POINTER(C.c_int64))
    s.dw = dw.ctypes.data_as(C.POINTER(C.c_double))
    s.four_last, s.radiation, s.rlambda = n["four_last"], n["radiation"], n["rlambda"]
    s.lambda_ = lam
    s.ldbw, s.ano = n["ldbw"], n["ano"]
    for k in range(3):
        s.inc[k] = int(n["inc"][k])
    for k in range(12):
        s.eck[k] = float(n["eck"][k])
    for k in range(9):
        s.vi[k] = float(n["vi"][k])
    return s


def output_spec(fmt, grid, value=1, extr=(1, 2, 3), cr=None, ar=(1.0, 1.0, 1.0), wrez=(90.0, 90.0, 90.0),
                valmax=0.0, f000=0.0, exti=0.0, rlambda=0.70932, name="crystal", lrange=0, lcenter=0, lpixel=0,
                center=(1, 1, 1), pixel=(1, 1, 1), quad="   ", nipl=None, scale=1.0, a0=None, win=None):
    """The output menu's settings as a dgpu_output struct (plus the objects
    its pointers refer to).  a0/win: cr_a0 and cr_win (HDF5 unit_cell); when
    omitted, the cell of cr's direct metric (the inverse of cr.rten), else
    1 and 90.  scale: out_scale (HDF5)."""
    o = _abi.Output()
    keep = []
    o.format = FORMATS[fmt] if isinstance(fmt, str) else int(fmt)
    o.value = int(value)
    for k in range(3):
        o.inc[k] = int(grid.inc[k])
    o.extr_abs, o.extr_ord, o.extr_top = (int(x) for x in extr)
    e, v = grid.eck.reshape(-1, order="F"), grid.vi.reshape(-1, order="F")
    for k in range(12):
        o.eck[k] = float(e[k])
    for k in range(9):
        o.vi[k] = float(v[k])
    rt = np.eye(3) if cr is None else np.asarray(cr.rten, dtype=np.float64)
    rt = rt.reshape(-1, order="F")
    for k in range(9):
        o.rten[k] = float(rt[k])
    for k in range(3):
        o.ar[k], o.wrez[k] = float(ar[k]), float(wrez[k])
        o.icc[k] = 1 if cr is None else int(cr.icc[k])
        o.center[k], o.pixel[k] = int(center[k]), int(pixel[k])
    o.lrange, o.lcenter, o.lpixel = int(lrange), int(lcenter), int(lpixel)
    o.quad = quad.encode()[:3].ljust(3)
    o.valmax, o.f000, o.exti, o.rlambda = float(valmax), float(f000), float(exti), float(rlambda)
    if (a0 is None or win is None) and cr is not None:
        g = np.linalg.inv(np.asarray(cr.rten, dtype=np.float64))
        la = np.sqrt(np.diag(g))
        ang = [np.degrees(np.arccos(g[(k + 1) % 3, (k + 2) % 3] / (la[(k + 1) % 3] * la[(k + 2) % 3])))
               for k in range(3)]
        a0 = la if a0 is None else a0
        win = ang if win is None else win
    for k in range(3):
        o.a0[k] = 1.0 if a0 is None else float(a0[k])
        o.win[k] = 90.0 if win is None else float(win[k])
    o.scale = float(scale)
    nm = name.encode()
    keep.append(nm)
    o.name = nm
    if nipl is not None:
        ns = _nipl_c(nipl, keep)
        keep.append(ns)
        o.nipl = C.pointer(ns)
    o._keep = keep
    return o


def write(path, spec, values=None, ampl=None, phase=None):
    """Write one output file (dgpu_output_write); returns the SHELX scale
    applied.  values/ampl/phase: qval arrays over the grid (VTK: dsi)."""
    L = load()
    v, a, p = _flat(values), _flat(ampl), _flat(phase)
    n = int(v.size) if v is not None else int(np.prod(list(spec.inc)))
    rc = L.dgpu_output_write(path.encode(), C.byref(spec), _abi.dptr(v), _abi.dptr(a), _abi.dptr(p), n)
    if rc != _abi.DGPU_OK:
        raise OSError(rc, f"dgpu_output_write failed ({rc}) for {path}")
    return spec.out_fac


def calc_hkl_files(cr, opts, infile, calcfile, style="hklf4", scale=1.0, exti=0.0, rlambda=0.70932, ctx=None):
    """calc_hkl with its files (dgpu_calc_hkl_files): reads infile (HKLF4 or
    CIF), writes calcfile and its .fcf list file."""
    ctx = ctx or default_context()
    st = {"hklf4": _abi.HKL_HKLF4, "cif": _abi.HKL_CIF}[style] if isinstance(style, str) else int(style)
    c = cr.to_c()
    ctx.check(ctx.lib.dgpu_calc_hkl_files(ctx.h, C.byref(c), C.byref(opts), infile.encode(), calcfile.encode(),
                                          st, float(scale), float(exti), float(rlambda)))
