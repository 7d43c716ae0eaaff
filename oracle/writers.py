"""Restatement of the output menu's and calc_hkl's file writers -- TEST
INFRASTRUCTURE ONLY (tests/ compares the library's files with these bytes).

Independent of the library's C++: Fortran editing is done here with exact
decimal arithmetic (Decimal of the binary value, ROUND_HALF_EVEN, the
processor's default rounding on exact values), records are lists of str.
Each writer follows the reference routine it names:

  edit descriptors          Fortran 2008 10.7 (I, F, E, A, X), list-directed
                            layout of gfortran (10.10.4: integer I11 after a
                            blank, REAL(8) 17 digits in G25 after a blank)
  do_output                 discus/prog/graphic.f90:1515-2124
  output_save_file_1d/2d    discus/prog/discus_s_out_file.f90:11-260
  write_discus_nipl_header  discus/prog/discus_nipl_header.f90:5-172
  four_angles / do_bang     discus/prog/four_angles_mod.f90:7-106, metric.f90:35-86
  vtk_write                 discus/prog/vtk_mod.f90:4-35
  mrc_write                 lib_f90/mrc_data.f90:19-139
  xplor_write               discus/prog/discus_xplor.f90:16-139
  calc_hkl (files)          discus/prog/fourier_sup.f90:3230-3549
Parity unpinned: no Fortran compiler is available to run the reference's writers.
"""
import math
import struct
from decimal import ROUND_HALF_EVEN, Decimal

import numpy as np

CVALUE = ["undefined", "Intensity", "Amplitude", "Phase angle", "Real Part", "Imaginary Part", "Random Phase",
          "S(Q)", "F(Q)", "f2aver = <f^2>", "faver2 = <f>^2", "faver = <f>", "Normal Inten", "I(Q)", "PDF",
          "3DPDF", "3DBETA", "f2averb=<f^2>*DBW", "faver2b=<f>^2*DBW", "faverb = <F>"]


# ------------------------------------------------------------- editing

def _neg(x):
    return math.copysign(1.0, x) < 0


def I(w, v):
    s = str(int(v))
    return "*" * w if len(s) > w else s.rjust(w)


def I0(v):
    return str(int(v))


def _fixed(d, x):
    q = Decimal(abs(x)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
    return f"{q:.{d}f}"


def F(w, d, x):
    if math.isnan(x):
        return "NaN".rjust(w)
    m = _fixed(d, x)
    sg = "-" if _neg(x) else ""
    if len(sg + m) > w and m.startswith("0."):
        m = m[1:]
    s = sg + m
    return "*" * w if len(s) > w else s.rjust(w)


def F0(d, x):
    return ("-" if _neg(x) else "") + _fixed(d, x)


def _sig(x, d):
    """|x| = 0.d1..dd * 10**e, rounded to d significant digits"""
    if x == 0:
        return "0" * d, 0
    a = Decimal(abs(x))
    e = a.adjusted() + 1
    q = (a.scaleb(-e)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
    if q >= 1:
        e += 1
        q = (a.scaleb(-e)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
    digits = f"{q:.{d}f}"[2:]
    return digits, e


def E(w, d, x, e=0):
    if math.isnan(x):
        return "NaN".rjust(w)
    digits, ex = _sig(x, d)
    if e == 0:
        if abs(ex) <= 99:
            es = "E" + ("-" if ex < 0 else "+") + f"{abs(ex):02d}"
        elif abs(ex) <= 999:
            es = ("-" if ex < 0 else "+") + f"{abs(ex):03d}"
        else:
            return "*" * w
    else:
        if abs(ex) >= 10 ** e:
            return "*" * w
        es = "E" + ("-" if ex < 0 else "+") + str(abs(ex)).zfill(e)
    sg = "-" if _neg(x) else ""
    s = sg + "0." + digits + es
    if len(s) > w:
        s = sg + "." + digits + es
    return "*" * w if len(s) > w else s.rjust(w)


def A(w, s):
    return s[:w] if len(s) >= w else s.rjust(w)


def ld_int(v):
    return " " + str(int(v)).rjust(11)


def ld_real(x):
    """gfortran list-directed REAL(8): G25.17E3 (1P for the E form) after a blank"""
    if x == 0:
        return " " + "0.0000000000000000".rjust(20) + " " * 5
    digits, ex = _sig(x, 17)          # |x| = 0.d1..d17 * 10**ex
    sg = "-" if _neg(x) else ""
    if 0 <= ex < 18:                  # 0.1 <= |x| < 1e17 after rounding: F20.(17-ex)
        k = ex
        s = sg + (digits[:k] if k > 0 else "0") + "." + digits[k:]
        return " " + s.rjust(20) + " " * 5
    e1 = ex - 1
    s = sg + digits[0] + "." + digits[1:] + "E" + ("-" if e1 < 0 else "+") + f"{abs(e1):03d}"
    return " " + s.rjust(25)


def groups(items, n):
    """format reversion: n items per record (one empty record for none)"""
    recs = ["".join(items[k:k + n]) for k in range(0, len(items), n)]
    return recs or [""]


# ------------------------------------------------------------- helpers

class Spec:
    """output_mod's state for one write (out_inc, out_eck(3,4), out_vi(3,3), ...)"""

    def __init__(self, fmt, value, inc, eck, vi, extr=(1, 2, 3), rten=None, ar=(1, 1, 1), wrez=(90, 90, 90),
                 icc=(1, 1, 1), valmax=0.0, f000=0.0, exti=0.0, rlambda=0.70932, name="crystal", lrange=0,
                 lcenter=0, lpixel=0, center=(1, 1, 1), pixel=(1, 1, 1), quad="   ", nipl=None):
        self.fmt, self.value = fmt, value
        self.inc = [int(x) for x in inc]
        self.eck = np.asarray(eck, dtype=np.float64).reshape(4, 3).T      # eck[:, corner]
        self.vi = np.asarray(vi, dtype=np.float64).reshape(3, 3).T         # vi[:, axis]
        self.ea, self.eo, self.et = extr
        self.rten = np.eye(3) if rten is None else np.asarray(rten, dtype=np.float64).reshape(3, 3).T
        self.ar, self.wrez, self.icc = list(ar), list(wrez), list(icc)
        self.valmax, self.f000, self.exti, self.rlambda = valmax, f000, exti, rlambda
        self.name = name
        self.lrange, self.lcenter, self.lpixel = lrange, lcenter, lpixel
        self.center, self.pixel, self.quad = list(center), list(pixel), quad
        self.nipl = nipl

    def h(self, i, j, l, third=True):
        """out_eck(:,1) + out_vi(:,1) REAL(i-1) + ... (REAL: default kind)"""
        r = self.eck[:, 0] + self.vi[:, 0] * float(np.float32(i - 1)) + self.vi[:, 1] * float(np.float32(j - 1))
        if third:
            r = r + self.vi[:, 2] * float(np.float32(l - 1))
        return r


def at(v, spec, i, j, l):
    return float(v[(i - 1) + spec.inc[0] * ((j - 1) + spec.inc[1] * (l - 1))])


def dstar(rten, h):
    return math.sqrt(float(h @ (rten @ h)))


def ext_cor(exti, lam, qq, ds):
    th = 2.0 * math.degrees(math.asin(0.5 * lam * ds))
    return (1.0 / (1.0 + 0.001 * exti * qq ** 2 * lam ** 3 / math.sin(math.radians(th)))) ** 0.25


def int_h(h):
    return [int(x) for x in h]          # INT: toward zero


# ------------------------------------------------------------- NIPL header

def _bang(rten, u, w):
    x, y = -np.asarray(u), -np.asarray(w)
    xx, xy, yy = math.sqrt(x @ rten @ x), x @ rten @ y, math.sqrt(y @ rten @ y)
    if not (xx > 0 and yy > 0):
        return 0.0
    arg = xy / (xx * yy)
    if abs(arg) < 1.0:
        return math.acos(arg) / float(np.float32(math.pi / 180.0))
    return 0.0 if arg >= 1.0 else 180.0


def four_angles(n, spec):
    vi = np.asarray(n["vi"], dtype=np.float64).reshape(3, 3).T
    eck = np.asarray(n["eck"], dtype=np.float64).reshape(4, 3).T
    inc = n["inc"]
    hor, ver, top = vi[:, 0], vi[:, 1], vi[:, 2]
    ltop = not (eck[0, 0] == eck[0, 3] and eck[1, 0] == eck[1, 3] and eck[2, 0] == eck[2, 3]) or inc[2] > 1
    ln = [math.sqrt(vi[:, k] @ spec.rten @ vi[:, k]) if inc[k] > 1 else 0.0 for k in range(3)]

    def pair(inc2, inc1, v, h, l2, l1, e_o, e_a):
        if inc1 > 1 and inc2 > 1:
            a = _bang(spec.rten, h, v)
            av = (l2 / v[e_o - 1]) / (l1 / h[e_a - 1]) if abs(h[e_a - 1]) > 0 and abs(v[e_o - 1]) > 0 else 0.0
            return a, av
        return 0.0, 0.0

    a1, v1 = pair(inc[1], inc[0], ver, hor, ln[1], ln[0], spec.eo, spec.ea)
    if ltop and inc[2] > 1 and ln[2] > 0:
        a2, v2 = pair(inc[2], inc[0], hor, top, ln[0], ln[2], spec.ea, spec.et)
        a3, v3 = pair(inc[2], inc[1], top, ver, ln[2], ln[1], spec.et, spec.eo)
    else:
        a2 = a3 = 90.0
        v2 = v3 = 1.0
    return (a1, a2, a3), (v1, v2, v3)


def nipl_header(n, spec, layer):
    cry = ["# CRYSTAL : lines       ;1I:: " + I(8, 3 + n["nscat"]),
           "# CRYSTAL : no. atoms   ;3I:: " + I(12, n["natoms"]) + ", " + I(12, n["nscat"]) + ", "
           + I(12, n["ncatoms"])]
    for i in range(n["nscat"] + 1):
        cry.append("# CRYSTAL : type atom   ;1C 2I 1R:: " + A(5, n["at_lis"][i].ljust(4)[:4]) + ", " + I(12, i)
                   + ", " + I(12, n["amount"][i]) + ", " + F(8, 5, n["dw"][i]))
    four = abs(n["four_last"]) < 3
    fou = []
    if four:
        ang, avr = four_angles(n, spec)
        eck = np.asarray(n["eck"], dtype=np.float64).reshape(4, 3)

        def r3(v):
            return F(12, 5, v[0]) + ", " + F(12, 5, v[1]) + ", " + F(12, 5, v[2])

        lam = n["lambda"].rstrip()
        fou = ["# FOURIER : lines       ;1I:: " + I(8, 18),
               "# FOURIER : type        ;1C:: " + I(1, abs(n["four_last"]))
               + ("D Fourier with lots" if n["four_last"] < 0 else "D Fourier complete crystal"),
               "# FOURIER : radiation   ;1C:: " + ["xray", "neutron", "electron"][n["radiation"] - 1],
               "# FOURIER : wave length ;1R::" + F(12, 5, n["rlambda"]),
               "# FOURIER : wave name   ;" + I(1, 1 if lam else 0) + "C::" + lam,
               "# FOURIER : adp         ;1C:: " + ("used" if n["ldbw"] else "ignored"),
               "# FOURIER : dispersion  ;1C:: " + ("anomalous" if n["ano"] else "ignored"),
               "# FOURIER : lower left  ;3R::" + r3(eck[0]),
               "# FOURIER : lower right ;3R::" + r3(eck[1]),
               "# FOURIER : upper left  ;3R::" + r3(eck[2]),
               "# FOURIER : top   left  ;3R::" + r3(eck[3]),
               "# FOURIER : no. points  ;3I::" + ", ".join(I(12, x) for x in n["inc"]),
               "# FOURIER : abscissa    ;1C:: " + "hkl"[spec.ea - 1],
               "# FOURIER : ordinate    ;1C:: " + "hkl"[spec.eo - 1],
               "# FOURIER : top         ;1C:: " + "hkl"[spec.et - 1],
               "# FOURIER : current top ;1I:: " + I(12, layer),
               "# FOURIER : angles      ;3R::" + r3(ang),
               "# FOURIER : aver        ;3R::" + r3(avr)]
    nh = 2 + (1 if four else 0) + len(cry) + len(fou)
    out = ["# HEADER  : lines, sec  ;2I::" + I(8, nh) + ", " + I(8, 2 if four else 1),
           "# HEADER  : section     ;1C::CRYSTAL"]
    if four:
        out.append("# HEADER  : section     ;1C::FOURIER")
    return out + [s.rstrip() for s in cry + fou]


# ------------------------------------------------------------- writers

def _text(recs):
    return ("\n".join(recs) + "\n").encode()


def _save_2d(hdr, ranges, n1, n2, spec, v, l):
    r = list(hdr) + [" " + I(8, n1) + " " + I(8, n2), "".join(" " + E(12, 5, x) for x in ranges)]
    for j in range(1, n2 + 1):
        r += groups([" " + E(12, 5, at(v, spec, i, j, l)) for i in range(1, n1 + 1)], 5)
    return _text(r + [""])


def standard(spec, v):
    """{file suffix: bytes} of ityp 0"""
    inc = spec.inc
    if inc[1] == 1 and inc[2] == 1:
        ax = 1
    elif inc[0] == 1 and inc[2] == 1:
        ax = 2
    elif inc[0] == 1 and inc[1] == 1:
        ax = 3
    else:
        ax = 0
    if ax:
        recs = []
        for i in range(1, inc[ax - 1] + 1):
            loop = [1, 1, 1]
            loop[ax - 1] = i
            h = spec.h(*loop)
            recs.append(" " + E(12, 5, h[spec.ea - 1]) + " " + E(12, 5, at(v, spec, i, 1, 1)))
        return {"": _text(recs)}
    ranges = [spec.eck[spec.ea - 1, 0], spec.eck[spec.ea - 1, 1], spec.eck[spec.eo - 1, 0], spec.eck[spec.eo - 1, 2]]
    hdr = (lambda l: nipl_header(spec.nipl, spec, l) if spec.nipl else [])
    if inc[2] == 1:
        return {"": _save_2d(hdr(1), ranges, inc[0], inc[1], spec, v, 1)}
    return {".PART_%04d" % l: _save_2d(hdr(l), ranges, inc[0], inc[1], spec, v, l) for l in range(1, inc[2] + 1)}


def shelx_scale(spec, ampl):
    m = int(math.floor(abs(spec.valmax) + 0.5)) * (1 if spec.valmax >= 0 else -1)     # NINT
    cells = spec.icc[0] * spec.icc[1] * spec.icc[2]
    sh = spec.fmt in (6, 7)
    if m == -1 and sh:
        qq = (spec.f000 / spec.icc[0] / spec.icc[1] / spec.icc[2]) ** 2
        f = int(math.log(qq) / math.log(10.0)) - (3 if spec.fmt == 6 else 2)
        return 10.0 ** (-max(f, 0))
    if m == -2 and sh:
        qqmax = 0.0
        for l in range(1, spec.inc[2] + 1):
            for j in range(1, spec.inc[1] + 1):
                for i in range(1, spec.inc[0] + 1):
                    if any(int_h(spec.h(i, j, l))):
                        qqmax = max(qqmax, (at(ampl, spec, i, j, l) / spec.icc[0] / spec.icc[1] / spec.icc[2]) ** 2)
        f = int(math.log(qqmax) / math.log(10.0)) - 3
        if spec.fmt == 6:
            f = max(f, 0)
        return 10.0 ** (-f)
    del cells
    if spec.valmax > 0 and sh:
        return spec.valmax
    return 1.0


def other(spec, v, ampl=None, phase=None):
    """(bytes, out_fac) of ityp 3, 6, 7, 8, 9"""
    inc, fmt = spec.inc, spec.fmt
    fac = shelx_scale(spec, ampl)
    cells = spec.icc[0] * spec.icc[1] * spec.icc[2]

    def pc(a):
        return a / spec.icc[0] / spec.icc[1] / spec.icc[2]

    def pos(p):
        return p + 360.0 if p < 0.0 else p

    del cells
    r = []
    if inc[0] > 1 and inc[1] > 1:
        if fmt == 9:
            e = spec.eck
            r.append(ld_int(inc[0]) + ld_int(inc[1]) + ld_int(inc[2]))
            r.append("".join(ld_real(x) for x in (e[spec.ea - 1, 0], e[spec.ea - 1, 1], e[spec.eo - 1, 0],
                                                   e[spec.eo - 1, 2], e[spec.et - 1, 0], e[spec.et - 1, 3])))
            for j in range(1, inc[1] + 1):
                r += groups([" " + E(12, 5, at(v, spec, i, j, 1)) for i in range(1, inc[0] + 1)], 5)
                r.append("")
        elif fmt in (6, 7, 8):
            for l in range(1, inc[2] + 1):
                for j in range(1, inc[1] + 1):
                    for i in range(1, inc[0] + 1):
                        h = spec.h(i, j, l)
                        ih = int_h(h)
                        if not any(ih):
                            continue
                        qq = pc(at(ampl, spec, i, j, l))
                        ds = dstar(spec.rten, h)
                        if fmt == 6:
                            ec = ext_cor(spec.exti, spec.rlambda, qq, ds) if spec.exti > 0.00001 else 1.0
                            sq = max(qq * math.sqrt(ec) * fac * 0.10, 0.01)
                            qq = (qq * ec) ** 2 * fac
                            r.append(I(4, ih[0]) + I(4, ih[1]) + I(4, ih[2]) + F(8, 2, qq) + F(8, 2, sq))
                        else:
                            try:
                                ec = ext_cor(spec.exti, spec.rlambda, qq, ds)
                            except (ValueError, ZeroDivisionError):
                                ec = float("nan")
                            qq = qq * ec * fac
                            sq = pos(at(phase, spec, i, j, l))
                            if fmt == 7:
                                r.append(I(4, ih[0]) + I(4, ih[1]) + I(4, ih[2]) + F(10, 2, qq) + F(10, 2, qq)
                                         + F(7, 2, sq))
                            else:
                                r.append(F(10, 6, h[0]) + " " + F(10, 6, h[1]) + " " + F(10, 6, h[2]) + " "
                                         + E(12, 5, qq) + " " + E(12, 5, qq) + " " + F(7, 2, sq))
        elif fmt == 3:
            ima = 6 - spec.ea - spec.eo
            for j in range(1, inc[1] + 1):
                for i in range(1, inc[0] + 1):
                    h = spec.h(i, j, 1, third=False)
                    r.append(" " + E(12, 5, h[spec.ea - 1]) + " " + E(12, 5, h[spec.eo - 1]) + " "
                             + E(12, 5, at(v, spec, i, j, 1)) + " " + E(12, 5, h[ima - 1]))
                r.append("")
    elif inc[0] == 1 or inc[1] == 1:
        along_j = inc[0] == 1
        src = v
        if fmt in (6, 7) and int(math.floor(abs(spec.valmax) + 0.5)) * (1 if spec.valmax >= 0 else -1) == -1:
            src = ampl
        for t in range(1, (inc[1] if along_j else inc[0]) + 1):
            i, j = (1, t) if along_j else (t, 1)
            h = spec.h(i, j, 1, third=False)
            ih = int_h(h)
            if not any(ih):
                continue
            val = at(src, spec, i, j, 1)
            if fmt == 6:
                qq = pc(val) * fac
                r.append(I(4, ih[0]) + I(4, ih[1]) + I(4, ih[2]) + F(8, 2, qq) + F(8, 2, math.sqrt(qq)))
            elif fmt == 7:
                qq = pc(val) * fac
                r.append(I(4, ih[0]) + I(4, ih[1]) + I(4, ih[2]) + F(10, 2, qq) + F(10, 2, qq)
                         + F(7, 2, pos(at(phase, spec, i, j, 1))))
            elif fmt == 8:
                qq = pc(val)
                r.append(F(10, 6, h[0]) + " " + F(10, 6, h[1]) + " " + F(10, 6, h[2]) + " " + E(12, 5, qq) + " "
                         + E(12, 5, qq) + " " + F(7, 2, pos(at(phase, spec, i, j, 1))))
    return (_text(r) if r else b""), fac


def vtk(spec, dsi):
    d = [math.sqrt(float(spec.vi[:, k] @ spec.vi[:, k])) for k in range(3)]
    r = ["# vtk DataFile Version 3.0", "DISCUS OUTPUT", "ASCII", "DATASET STRUCTURED_POINTS",
         "DIMENSIONS " + " ".join(I0(x) for x in spec.inc),
         "ORIGIN " + " ".join(F0(4, x) for x in spec.eck[:, 0]),
         "SPACING " + " ".join(F0(4, x) for x in d),
         "POINT_DATA " + I0(spec.inc[0] * spec.inc[1] * spec.inc[2]),
         "SCALARS values float", "LOOKUP_TABLE default"]
    r += [E(13, 6, float(x), 2) for x in dsi]
    return _text(r)


def mrc(spec, v):
    words = [b"\0\0\0\0"] * 1024

    def i4(k, x):
        words[k - 1] = struct.pack("<i", int(x))

    def r4(k, x):
        words[k - 1] = struct.pack("<f", float(np.float32(x)))

    n = spec.inc
    arr = np.asarray(v, dtype=np.float64)
    for k, x in enumerate([n[0], n[1], n[2], 2, 0, 0, 0, n[0] - 1, n[1] - 1, n[2] - 1]):
        i4(k + 1, x)
    for k in range(3):
        r4(11 + k, spec.ar[k])
        r4(14 + k, spec.wrez[k])
    r4(17, spec.ea)
    r4(18, spec.eo)
    r4(19, spec.et)
    r4(20, arr.min())
    r4(21, arr.max())
    r4(22, arr.sum() / (n[0] * n[1] * n[2]))
    i4(23, 0)
    i4(24, 3072)
    words[52] = b"MAP\0"
    i4(54, 4 + 4 * 16 + 68 * 256)
    return b"".join(words) + arr.astype("<f4").tobytes()


def xplor_name(path):
    return path if path[-6:].upper() == ".XPLOR" else path + ".xplor"


def xplor(spec, v):
    inc = spec.inc
    start, fini = [1, 1, 1], list(inc)
    if spec.lrange != 0:
        center, pixel = list(spec.center), list(spec.pixel)
        if spec.lcenter == 0:
            center = [max(1, int(math.floor(x / 2.0 + 0.5))) for x in inc]
        if spec.lpixel == 0:
            pixel = list(inc)
        if spec.lrange == 2:
            for k in range(3):
                e = inc[k] + inc[k] % 2
                if spec.quad[k] == "l":
                    pixel[k], center[k] = e // 2, e // 4 + 1
                elif spec.quad[k] == "r":
                    pixel[k] = e // 2
                    center[k] = e // 4 + pixel[k] + 1 - inc[k] % 2
        for k in range(3):
            m1 = pixel[k] // 2
            m2 = pixel[k] // 2 - (1 if pixel[k] % 2 == 0 else 0)
            start[k] = min(max(1, center[k] - m1), inc[k])
            fini[k] = min(max(1, center[k] + m2), inc[k])
    title = ("TITLE " + spec.name.rstrip() + " " + CVALUE[spec.value].ljust(17) + " written by DISCUS ")
    r = ["", title.ljust(80)[:80],
         "".join(I(8, fini[k] - start[k] + 1) + I(8, 1) + I(8, fini[k] - start[k] + 1) for k in range(3))]
    if spec.value != 14:
        r.append("".join(E(12, 5, x) for x in list(spec.ar) + list(spec.wrez)))
    r.append("  ZYX")
    for l in range(start[2], fini[2] + 1):
        r.append(I(8, l - start[2] + 1))
        items = [E(12, 5, at(v, spec, i, j, l)) for j in range(start[1], fini[1] + 1)
                 for i in range(start[0], fini[0] + 1)]
        r += groups(items, 6)
    r.append(I(8, -9999))
    r.append(E(12, 4, 1.0) + " " + E(12, 4, 1.0))
    return _text(r)


# ------------------------------------------------------------- calc_hkl

def read_hklf4(text):
    """(3I4,2F8.2) records: [(h, k, l, rint, sint)]"""
    out = []
    for ln in text.splitlines():
        f = [ln[0:4], ln[4:8], ln[8:12], ln[12:20], ln[20:28]]
        vals = []
        for k, s in enumerate(f):
            s = s.replace(" ", "")
            if not s:
                vals.append(0)
            elif k < 3:
                vals.append(int(s))
            else:
                vals.append(float(s) if "." in s else int(s) / 100.0)
        out.append(tuple(vals))
    return out


def calc_hkl_files(style, infile_text, icalc, sigi, phase):
    """(calcfile bytes, listfile bytes) from calc_hkl's per-reflection values
    (in the order of the input's reflections)"""
    cf, lf = [], []
    if style == 4:
        rows = read_hklf4(infile_text)
        for r, (h, k, l, rint, _) in enumerate(rows):
            ihkl = I(4, h) + I(4, k) + I(4, l)
            if h == 0 and k == 0 and l == 0:
                cf.append(ihkl + F(8, 2, 0.0) + F(8, 2, 0.0))
                continue
            cf.append(ihkl + F(8, 2, icalc[r]) + F(8, 2, sigi[r]))
            lf.append(ihkl + F(10, 2, math.sqrt(abs(rint))) + F(10, 2, math.sqrt(abs(icalc[r])))
                      + F(7, 2, phase[r]))
    else:
        lines = infile_text.splitlines()
        k = next(i for i, s in enumerate(lines) if s.startswith("_refln_index_h"))
        names = []
        while k < len(lines) and (lines[k].startswith("_refln_") or lines[k].startswith("#") or not lines[k].strip()):
            if lines[k].startswith("_refln_"):
                names.append(lines[k].split()[0])
            k += 1
        jc = names.index("_refln_F_squared_calc") if "_refln_F_squared_calc" in names else -1
        r = 0
        for ln in lines[k:]:
            t = ln.split()
            if not t:
                continue
            vals = [float(x) for x in t[:len(names) - 1]]
            h, kk, l = (int(math.copysign(math.floor(abs(x) + 0.5), x)) for x in vals[:3])     # NINT
            ihkl = I(4, h) + I(4, kk) + I(4, l)
            if h == 0 and kk == 0 and l == 0:
                cf.append(ihkl + F(8, 2, 0.0) + F(8, 2, 0.0))
                r += 1
                continue
            if 0 <= jc < len(vals):
                vals[jc] = icalc[r]
            cf.append(ihkl + "".join(F(12, 2, x) for x in vals[3:]))
            lf.append(ihkl + F(10, 2, vals[0]) + F(10, 2, math.sqrt(abs(icalc[r]))) + F(7, 2, phase[r]))
            r += 1
    return _text(cf) if cf else b"", _text(lf) if lf else b""
