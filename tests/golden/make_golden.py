"""Known-answer vectors for DISCUS's Fourier path, from closed forms.

The reference ships no tests or golden data for this path and cannot be
compiled here, so these fixtures are derived independently of any
implementation:

  * single_atom_ref -- one atom at the origin: every REF22 phase index is 0,
    cex(0) = 1, so csf(h) = cfact(istl(h)) exactly (four_strucf_OMP_mod.f90:169,
    fourier_form.f90:172); istl from h rounded to REAL(4) (fourier_sup.f90:2668-2674).
  * laue_exact -- a perfect primitive lattice of n1 x n2 x n3 cells with one
    atom per cell at r0: F(h) = f(s) exp(2 pi i h.r0) prod_a G(h_a, n_a),
    G = sum_m exp(2 pi i x m) (Laue interference function).
  * two_atoms_exact -- F(h) = sum_k f_k(s) exp(2 pi i h.r_k).
  * lmn -- hand-derived decompositions of standard grids (fourier_lmn_mod.f90).

    python tests/golden/make_golden.py   (writes kat.npz and lmn.json here)
"""
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def form(scat_t, s2, power=4):
    f = scat_t[0]
    for i in range(1, power + 1):
        f = f + scat_t[2 * i - 1] * np.exp(-scat_t[2 * i] * s2)
    return f


def cfact(scat_t, occ, b, s2, ldbw=True):
    sb = np.exp(-b * s2) * occ if ldbw else occ
    return sb * form(scat_t, s2)


def hgrid(eck, vi, inc):
    i = np.arange(inc[0])[:, None, None]
    j = np.arange(inc[1])[None, :, None]
    k = np.arange(inc[2])[None, None, :]
    return np.stack([eck[a] + vi[0][a] * i + vi[1][a] * j + vi[2][a] * k for a in range(3)])


def nint(x):
    return np.where(x >= 0, np.floor(x + 0.5), -np.floor(-x + 0.5)).astype(np.int64)


def main():
    out = {}
    rng = np.random.Generator(np.random.PCG64(20240601))
    scat = np.zeros((4, 11))
    for t in range(1, 4):
        scat[t, 0] = rng.uniform(0, 2)
        for i in range(1, 5):
            scat[t, 2 * i - 1] = rng.uniform(0.5, 10)
            scat[t, 2 * i] = rng.uniform(0.5, 50)
    a = 4.0
    rten = np.diag([1 / a ** 2] * 3)
    out["scat"] = scat
    out["rten_cubic4"] = rten

    # --- single atom at the origin, REF22, 21x21 hk0 plane centred on 0
    eck = np.array([-1.0, -1.0, 0.0])
    vi = np.array([[0.1, 0, 0], [0, 0.1, 0], [0, 0, 0]])
    inc = (21, 21, 1)
    h = hgrid(eck, vi, inc).astype(np.float32).astype(np.float64)
    q2 = np.einsum("a...,ab,b...->...", h, rten, h) / 4.0
    istl = nint(np.sqrt(q2) * 1000.0)
    s2 = (istl * 0.001) ** 2
    out["single_atom_istl"] = istl
    out["single_atom_csf"] = cfact(scat[1], 1.0, 0.5, s2).astype(np.complex128)
    out["single_atom_eck"] = eck
    out["single_atom_vi"] = vi
    out["single_atom_inc"] = np.array(inc)

    # --- Laue function, exact phases, analytic form factor, general 3D grid
    n = (4, 5, 3)
    r0 = np.array([0.1, 0.2, 0.3])
    eck = np.array([-0.73, 0.41, -0.37])
    vi = np.array([[0.113, 0.0, 0.0], [0.0, 0.097, 0.0], [0.0, 0.0, 0.21]])
    inc = (9, 7, 5)
    h = hgrid(eck, vi, inc)
    s2 = np.einsum("a...,ab,b...->...", h, rten, h) / 4.0

    def G(x, m):
        xr = x - np.round(x)
        with np.errstate(invalid="ignore", divide="ignore"):
            r = np.sin(math.pi * m * xr) / np.sin(math.pi * xr)
        r = np.where(xr == 0, m, r)
        return r * np.exp(1j * math.pi * xr * (m - 1))

    F = cfact(scat[1], 1.0, 0.5, s2) * np.exp(2j * math.pi * np.einsum("a...,a->...", h, r0))
    for ax in range(3):
        F = F * G(h[ax], n[ax])
    cells = np.stack(np.meshgrid(*[np.arange(m) for m in n], indexing="ij"), -1).reshape(-1, 3, order="F")
    out["laue_pos"] = cells + r0
    out["laue_icc"] = np.array(n)
    out["laue_eck"] = eck
    out["laue_vi"] = vi
    out["laue_inc"] = np.array(inc)
    out["laue_csf"] = F

    # --- two atoms of different types, exact, analytic, 2D plane
    pos2 = np.array([[0.123, -0.456, 0.789], [1.5, 0.25, -0.75]])
    eck = np.array([-2.0, -1.5, 0.3])
    vi = np.array([[0.2, 0.05, 0.0], [-0.04, 0.25, 0.01], [0, 0, 0]])
    inc = (17, 13, 1)
    h = hgrid(eck, vi, inc)
    s2 = np.einsum("a...,ab,b...->...", h, rten, h) / 4.0
    F = (cfact(scat[1], 1.0, 0.5, s2) * np.exp(2j * math.pi * np.einsum("a...,a->...", h, pos2[0]))
         + cfact(scat[2], 1.0, 0.5, s2) * np.exp(2j * math.pi * np.einsum("a...,a->...", h, pos2[1])))
    out["two_pos"] = pos2
    out["two_eck"] = eck
    out["two_vi"] = vi
    out["two_inc"] = np.array(inc)
    out["two_csf"] = F
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **out)

    # --- fourier_lmn decompositions (eck(3,4) as ll only; vi columns)
    lmn_cases = [
        dict(name="hk0_centred", eck=[-5, -5, 0], vi=[[0.05, 0, 0], [0, 0.05, 0], [0, 0, 0]], inc=[201, 201, 1],
             lmn=[-100, -100, 0, 0, 0, 0], off=[[0, 0, 0], [0, 0, 0], [0, 0, 0.001]], rc=0),
        dict(name="cube_centred", eck=[-4, -4, -4], vi=[[0.08, 0, 0], [0, 0.08, 0], [0, 0, 0.08]],
             inc=[101, 101, 101], lmn=[-50, -50, -50, 0, 0, 0], off=[[0, 0, 0]] * 3, rc=0),
        dict(name="h0l_offplane", eck=[-10, 0.5, -10], vi=[[0.02, 0, 0], [0, 0, 0], [0, 0, 0.02]],
             inc=[1001, 1, 1001], lmn=[-500, 0, -500, 0, -500, 0], off=[[0, 0, 0], [0, -0.001, 0], [0, 0, 0]],
             rc=0),
        dict(name="row_a_star", eck=[-2.5, 1, 0], vi=[[0.05, 0, 0], [0, 0, 0], [0, 0, 0]], inc=[101, 1, 1],
             lmn=[-50, 0, 0, 0, 1, 1], off=[[0, 0, 0], [0, 1, 0], [0, 0, 0]], rc=0),
        dict(name="zero_increment", eck=[0, 0, 0], vi=[[0, 0, 0], [0, 0.05, 0], [0, 0, 0]], inc=[11, 11, 1],
             lmn=[0] * 6, off=[[0, 0, 0]] * 3, rc=-5),
    ]
    with open(os.path.join(HERE, "lmn.json"), "w") as f:
        json.dump(lmn_cases, f, indent=1)


if __name__ == "__main__":
    main()
