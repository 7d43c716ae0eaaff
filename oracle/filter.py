"""Restatement of four_run's Lanczos filter -- TEST INFRASTRUCTURE ONLY.

do_four_filter (discus/prog/fourier_sup.f90:1646-1803) with the FFT
variants do_lanczos_{1,2,3}d_fft (lib_f90/lib_lanczos.f90:224-426), the
kernel functions wsinc/lqgm (:428-604), sinc (lib_f90/lib_functions.f90:10-30),
the FFT convolution do_convolute_{1,2,3}d_real (lib_f90/lib_conv.f90) and
the index maps maptofftfd / mapfftfdtoline (lib_f90/map_1dtofield.f90:39-62,
165-199, 325-364, 411-430, 556-593, 718-755), step by step: the kernel table
with the reference's 1-based loops, the forward maps, numpy's unnormalised
forward FFT for FFTW_FORWARD (applied a second time for the "back" FFT, as
the reference does), the back maps, the weight and the sum normalisation.
Parity unpinned: no Fortran compiler is available to run the reference's filter.
"""
import math

import numpy as np

PI = 3.1415926535897932384626433832795028841971693993751


def sinc(x):
    return 1.0 if abs(x) < 1.0e-7 else math.sin(x) / x


def _table(dims, rcut, m, nscale=1.0):
    """sinc_table(1:idims) of do_lanczos_{1,2,3}d_fft (0-based array)"""
    nd = len(dims)
    tab = np.zeros(dims)
    c = [(n + 1) // 2 for n in dims]                       # i1 = (idims+1)/2
    lo = [int(np.rint(-nscale * m - 1.0)) + ck for ck in c]
    hi = [int(np.rint(nscale * m + 1.0)) + ck for ck in c]
    q = [ck / nscale for ck in c]
    ranges = [range(lo[k], hi[k] + 1) for k in range(nd)]
    for idx in np.ndindex(*[len(r) for r in ranges]):
        t = [ranges[k][idx[k]] for k in range(nd)]
        g = [tk / nscale for tk in t]
        d = [q[k] - g[k] for k in range(nd)]
        if nd == 1:
            ws = sinc(PI * d[0] * rcut) * sinc(PI * d[0] * rcut)
            lq = sinc(PI * d[0] / m) if abs(d[0]) < m else 0.0
        else:
            ws = 1.0
            for k in range(nd):
                ws *= sinc(PI * d[k] * rcut)
            if all(abs(x) < m for x in d):
                lq = 1.0
                for k in range(nd):
                    lq *= sinc(PI * d[k] / m)
            else:
                lq = 0.0
        if any(tk < 1 or tk > dims[k] for k, tk in enumerate(t)):
            raise ValueError("kernel table outside its bounds (the reference writes out of range)")
        tab[tuple(tk - 1 for tk in t)] = ws * lq
    return tab


def _map_to_fft(a):
    """maptofftfd (dsort = identity): field index i -> mod(i + n/2 - l, n) + 1"""
    out = np.zeros(a.shape, dtype=complex)
    idx = []
    for n in a.shape:
        l_ = (n - 1) % 2
        idx.append(np.array([(i + n // 2 - l_) % n for i in range(1, n + 1)]))
    out[np.ix_(*idx)] = a
    return out


def _map_back(r, one_d):
    """mapfftfdtoline: FFT index ii -> n + 1 - (mod(ii + n/2 - l - 1, n) + 1)
    (2D/3D), n + 1 - (mod(ii - 1 + n/2, n) + 1) (1D)"""
    out = np.zeros(r.shape)
    idx = []
    for n in r.shape:
        l_ = 0 if one_d else (n - 1) % 2
        idx.append(np.array([n + 1 - (((ii + n // 2 - l_ - 1) % n) + 1) - 1 for ii in range(1, n + 1)]))
    out[np.ix_(*idx)] = r.real
    return out


def lanczos(field, rcut, m, nscale=1.0):
    """do_lanczos_{1,2,3}d_fft with inc = idims = field.shape"""
    a = np.asarray(field, dtype=np.float64)
    dims = a.shape
    tab = _table(dims, rcut, m, nscale)
    out = np.zeros(dims)
    sl = tuple(slice(0, n, int(round(nscale))) for n in dims)
    out[sl] = a
    # do_convolute_*_real(idims, outfield, sinc_table)
    t = np.fft.fftn(_map_to_fft(tab))
    o = np.fft.fftn(_map_to_fft(out))
    r = np.fft.fftn(t * o)
    res = _map_back(r, len(dims) == 1)
    w = 1.0
    for n in dims:
        w *= math.sqrt(float(n) ** 3)
    res = res / w
    factor = a.sum() / res.sum() * nscale
    return res * factor


def four_filter(dsi, rcut=0.5, m=4, nscale=1.0):
    """do_four_filter on dsi(num) (Fortran-ordered 3D array), FOUR_FILTER_LANCZOS"""
    d = np.array(dsi, dtype=np.float64, copy=True)
    num = d.shape
    dim = sum(1 for n in num if n > 1)
    w2 = 2 * m + 1
    if dim == 3:
        if all(n > w2 for n in num):
            d[...] = lanczos(d, rcut, m, nscale)
        elif num[2] <= w2:
            for k in range(num[2]):
                d[:, :, k] = lanczos(d[:, :, k], rcut, m, nscale)
        elif num[1] <= w2:
            for j in range(num[1]):
                d[:, j, :] = lanczos(d[:, j, :], rcut, m, nscale)
        elif num[0] <= w2:
            for i in range(num[0]):
                d[i, :, :] = lanczos(d[i, :, :], rcut, m, nscale)
    elif dim == 2:
        d[:, :, 0] = lanczos(d[:, :, 0], rcut, m, nscale)
    elif dim == 1:
        d[:, 0, 0] = lanczos(d[:, 0, 0], rcut, m, nscale)
    return d
