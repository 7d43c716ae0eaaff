"""ctypes mirror of include/discus_gpu.h (structs, constants).

The C-ABI is the product boundary; this module only describes its plain-C
structs so that Python callers (the Fourier menu mirror, tests, bench) can
fill them from numpy arrays.
"""
import ctypes as C

import numpy as np

DGPU_OK = 0
DGPU_WARN_NO_CELL = 1
DGPU_ERR_ARG = -1
DGPU_ERR_CUDA = -2
DGPU_ERR_NOMEM = -3
DGPU_ERR_STL_RANGE = -4
DGPU_ERR_ZERO_INC = -5
DGPU_ERR_UNSUPPORTED = -6
DGPU_ERR_TIMEOUT = -7
DGPU_ERR_CANCELLED = -14
DGPU_ERR_NO_ATOMS = -198
DGPU_ERR_SCRATCH_SIZE = -20
DGPU_ERR_NO_ACCUM = -175
DGPU_ERR_IO = -21

CFPKT = 9999
CFINC = 0.001
I2PI = 65536

PHASE_REF22 = 0
PHASE_EXACT64 = 1
FORM_TABLE = 0
FORM_ANALYTIC = 1
ENGINE_AUTO = 0
ENGINE_DIRECT = 1
ENGINE_TC = 2
SPLIT_F16 = 0
SPLIT_BF16 = 1
VAL_INTEN = 1
VAL_AMPLI = 2
VAL_PHASE = 3
VAL_REAL = 4
VAL_IMAG = 5
VAL_RANPH = 6
VAL_SQ = 7
VAL_F2AVER = 9
VAL_FAVER2 = 10
VAL_FAVER = 11
VAL_IQ = 13
VAL_F2AVERB = 17
VAL_FAVER2B = 18
VAL_FAVERB = 19
ACCUM_INIT = -1
ACCUM_SINGLE = 0
ACCUM_ACCUM = 1
ACCUM_FINISHED = 2
LOT_OFF = 1
LOT_BOX = 2
LOT_ELI = 3
PREF_NONE = 0
PREF_RIETVELD = 1
PREF_MARCH = 2
FILTER_OFF = 0
FILTER_LANCZOS = 1
HKL_CIF = 1
HKL_HKLF4 = 4
OUT_STANDARD = 0
OUT_GNUPLOT = 3
OUT_HKLF4 = 6
OUT_LIST5 = 7
OUT_LIST9 = 8
OUT_NIPL3D = 9
OUT_VTK = 11
OUT_MRC = 12
OUT_HDF5 = 13
OUT_XPLOR = 14

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_fp = C.POINTER(C.c_float)


class Crystal(C.Structure):
    _fields_ = [
        ("natoms", C.c_int64),
        ("pos", _dp),
        ("iscat", _ip),
        ("atom_occ", _fp),
        ("nscat", C.c_int32),
        ("ncatoms", C.c_int32),
        ("icc", C.c_int32 * 3),
        ("dim0", C.c_double * 3),
        ("rten", C.c_double * 9),
        ("scat", _dp),
        ("occ", _dp),
        ("dw", _dp),
        ("delfr", _dp),
        ("delfi", _dp),
        ("is_anis", C.c_int32),
        ("nanis", C.c_int32),
        ("ianis", _ip),
        ("anis_full", _dp),
        ("ar", C.c_double * 3),
        ("dim_lo", C.c_double * 3),
        ("isym", _ip),
    ]


class Discamb(C.Structure):
    _fields_ = [
        ("maxhkl", C.c_int32 * 3),
        ("nsymm", _ip),
        ("isymm", _ip),
        ("form_tsc", _dp),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("eck", C.c_double * 12),
        ("vi", C.c_double * 9),
        ("inc", C.c_int32 * 3),
    ]


class Opts(C.Structure):
    _fields_ = [
        ("lxray", C.c_int32),
        ("power", C.c_int32),
        ("ano", C.c_int32),
        ("ldbw", C.c_int32),
        ("friedel", C.c_int32),
        ("fave", C.c_double),
        ("aver_cells", C.POINTER(C.c_uint8)),
        ("diff_scale", C.c_double),
        ("phase", C.c_int32),
        ("form", C.c_int32),
        ("engine", C.c_int32),
        ("split", C.c_int32),
        ("tc_tile_n", C.c_int32),
        ("tc_kslice", C.c_int32),
        ("tc_flush", C.c_int32),
        ("cancel", C.POINTER(C.c_int32)),
        ("ilots", C.c_int32),
        ("nlots", C.c_int32),
        ("ls_xyz", C.c_int32 * 3),
        ("lot_all", C.c_int32),
        ("lperiod", C.c_int32),
        ("lot_origins", _ip),
        ("tc_vimg", C.c_int32),
        ("tc_wait_us", C.c_int32),
        ("discamb", C.POINTER(Discamb)),
        ("filter", C.c_int32),
        ("filter_width", C.c_int32),
        ("filter_damp", C.c_double),
        ("filter_scale", C.c_double),
    ]


class Info(C.Structure):
    _fields_ = [
        ("fnum", C.c_int32 * 3),
        ("friedel_dim", C.c_int32),
        ("lmn", C.c_int32 * 6),
        ("off_shift", C.c_double * 9),
        ("ncell", C.c_int32),
        ("engine_used", C.c_int32),
        ("pairs", C.c_int64),
        ("pairs_aver", C.c_int64),
        ("res", C.c_double * 7),
        ("kernel_ms", C.c_double),
        ("total_ms", C.c_double),
        ("tc_config", C.c_int32 * 4),
        ("refined", C.c_int64),
    ]


class Powder(C.Structure):
    _fields_ = [
        ("hkl_del", C.c_double * 3),
        ("hkl_shift", C.c_double * 3),
        ("a0", C.c_double * 3),
        ("gten", C.c_double * 9),
        ("ds_max", C.c_double),
        ("qmin", C.c_double),
        ("qmax", C.c_double),
        ("deltaq", C.c_double),
        ("l_all", C.c_int32),
        ("pref_type", C.c_int32),
        ("pref_hkl", C.c_double * 3),
        ("pref_g1", C.c_double),
        ("pref_g2", C.c_double),
        ("slabs", C.c_int32),
    ]


class PowderInfo(C.Structure):
    _fields_ = [
        ("n_pkt", C.c_int32),
        ("nslab", C.c_int32),
        ("rods", C.c_int64),
        ("rod_points", C.c_int64),
        ("grid_points", C.c_int64),
        ("binned", C.c_int64),
        ("pairs", C.c_int64),
        ("kernel_ms", C.c_double),
        ("total_ms", C.c_double),
    ]


def dptr(a):
    """double* of a contiguous float64 numpy array (None -> NULL)."""
    if a is None:
        return C.cast(None, _dp)
    assert a.dtype == np.float64 and a.flags.c_contiguous or a.flags.f_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return C.cast(None, _ip)
    assert a.dtype == np.int32
    return a.ctypes.data_as(_ip)


def fptr(a):
    if a is None:
        return C.cast(None, _fp)
    assert a.dtype == np.float32
    return a.ctypes.data_as(_fp)


def default_opts(**kw):
    """fourier_reset.f90:42-101 defaults (xray, 4 Gaussians, temp ignore,
    Friedel on, aver off, scale 1) plus phase/form/engine choices."""
    o = Opts()
    o.lxray = 1
    o.power = 4
    o.ano = 0
    o.ldbw = 0
    o.friedel = 1
    o.fave = 0.0
    o.aver_cells = C.cast(None, C.POINTER(C.c_uint8))
    o.diff_scale = 1.0
    o.phase = PHASE_EXACT64
    o.form = FORM_TABLE
    o.engine = ENGINE_AUTO
    o.split = SPLIT_F16
    o.tc_tile_n = 0
    o.tc_kslice = 0
    o.tc_flush = 0
    o.cancel = C.cast(None, C.POINTER(C.c_int32))
    o.ilots = LOT_OFF
    o.nlots = 1
    for k in range(3):
        o.ls_xyz[k] = 5
    o.lot_all = 0
    o.lperiod = 1
    o.lot_origins = C.cast(None, _ip)
    o.tc_vimg = 0
    o.tc_wait_us = 0
    o.discamb = C.cast(None, C.POINTER(Discamb))
    o.filter = FILTER_OFF
    o.filter_width = 4
    o.filter_damp = 0.5
    o.filter_scale = 1.0
    for k, v in kw.items():
        if k in ("aver_cells", "lot_origins"):
            continue
        if k == "ls_xyz":
            for i in range(3):
                o.ls_xyz[i] = int(v[i])
            continue
        setattr(o, k, v)
    return o


class Nipl(C.Structure):
    _fields_ = [
        ("natoms", C.c_int64),
        ("nscat", C.c_int32),
        ("ncatoms", C.c_int32),
        ("at_lis", C.c_char_p),
        ("amount", C.POINTER(C.c_int64)),
        ("dw", _dp),
        ("four_last", C.c_int32),
        ("radiation", C.c_int32),
        ("rlambda", C.c_double),
        ("lambda_", C.c_char_p),
        ("ldbw", C.c_int32),
        ("ano", C.c_int32),
        ("inc", C.c_int32 * 3),
        ("eck", C.c_double * 12),
        ("vi", C.c_double * 9),
    ]


class Output(C.Structure):
    _fields_ = [
        ("format", C.c_int32),
        ("value", C.c_int32),
        ("inc", C.c_int32 * 3),
        ("extr_abs", C.c_int32),
        ("extr_ord", C.c_int32),
        ("extr_top", C.c_int32),
        ("eck", C.c_double * 12),
        ("vi", C.c_double * 9),
        ("rten", C.c_double * 9),
        ("ar", C.c_double * 3),
        ("wrez", C.c_double * 3),
        ("icc", C.c_int32 * 3),
        ("lrange", C.c_int32),
        ("lcenter", C.c_int32),
        ("lpixel", C.c_int32),
        ("center", C.c_int32 * 3),
        ("pixel", C.c_int32 * 3),
        ("quad", C.c_char * 4),
        ("valmax", C.c_double),
        ("f000", C.c_double),
        ("exti", C.c_double),
        ("rlambda", C.c_double),
        ("name", C.c_char_p),
        ("nipl", C.POINTER(Nipl)),
        ("out_fac", C.c_double),
        ("a0", C.c_double * 3),
        ("win", C.c_double * 3),
        ("scale", C.c_double),
    ]
