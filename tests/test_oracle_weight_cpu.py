"""four_weight and the Bragg fill of four_accumulate in the oracle, against
closed forms (CPU only).

The voxel of four_weight is the reciprocal volume of the grid steps
(do_volume from lengths and angles); divided by the reciprocal cell volume
it is |det(bases)| exactly, so scalef = ncells * |det(bases)| up to the
reference's single-precision degree conversion (1e-6 here).
"""
import numpy as np

from diffusecode_gb300 import _abi
from diffusecode_gb300.structures import GridData, reciprocal_metric, small_lots_anis
from oracle import oracle as O


def _grid(vi, inc, lo=(-1.0, -1.0, 0.0)):
    vi = np.asarray(vi, dtype=np.float64)
    lo = np.asarray(lo, dtype=np.float64)
    eck = np.stack([lo, lo + vi[:, 0] * (inc[0] - 1), lo + vi[:, 1] * (inc[1] - 1), lo + vi[:, 2] * (inc[2] - 1)],
                   axis=1)
    return GridData(eck=eck, vi=vi, inc=inc)


def _crystal(icc, rten):
    cr, _ = small_lots_anis(anis=False, icc=icc)
    cr.rten = rten
    return cr


def test_weight_scale_closed_forms():
    rt = reciprocal_metric(4.1, 4.6, 5.3, 90, 103, 90)
    cr = _crystal((5, 4, 3), rt)
    cases = [
        # 3D, oblique steps: bases = vi
        (np.array([[0.1, 0.02, 0.0], [0.0, 0.2, 0.01], [0.03, 0.0, 0.25]]), (9, 7, 5), 60),
        # hk0 plane: the flat column is (0, 0, 1)
        (np.array([[0.05, 0.0, 0.0], [0.0, 0.05, 0.0], [0.0, 0.0, 0.0]]), (21, 21, 1), 20),
        # h0l plane
        (np.array([[0.05, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.04]]), (21, 1, 21), 15),
        # row along a*: columns v, e2, e3
        (np.array([[0.05, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]), (41, 1, 1), 5),
    ]
    for vi, inc, ncells in cases:
        g = _grid(vi, inc)
        B = vi.copy()
        if inc[2] == 1 and inc[1] > 1:
            B[:, 2] = [0, 0, 1]
        elif inc[1] == 1 and inc[2] > 1:
            B[:, 1] = [0, 1, 0]
        elif inc[1] == 1 and inc[2] == 1:
            B[:, 1], B[:, 2] = [0, 1, 0], [0, 0, 1]
        dsi = np.random.default_rng(1).random(inc) + 1.0
        d3, scalef = O.four_weight(cr, g, dsi, _abi.default_opts())
        assert abs(scalef - ncells * abs(np.linalg.det(B))) <= 1e-6 * scalef, (inc, scalef)
        hkl = g.hkl()
        bragg = np.all(np.abs(hkl - np.rint(hkl)) < np.float32(1e-4), axis=0)
        assert bragg.any()
        np.testing.assert_allclose(d3[bragg], dsi[bragg] / scalef, rtol=1e-15)
        np.testing.assert_array_equal(d3[~bragg], dsi[~bragg])


def test_weight_lots_and_aver():
    cr = _crystal((6, 5, 4), reciprocal_metric(4, 4, 4, 90, 90, 90))
    g = _grid(np.diag([0.1, 0.1, 0.1]), (11, 11, 11))
    dsi = np.ones(g.inc)
    _, s_all = O.four_weight(cr, g, dsi, _abi.default_opts())
    op = _abi.default_opts(ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), nlots=7)
    _, s_lot = O.four_weight(cr, g, dsi, op)
    assert abs(s_all - 120 * 1e-3) < 1e-9 and abs(s_lot - 12 * 1e-3) < 1e-9
    d3, s = O.four_weight(cr, g, dsi, _abi.default_opts(fave=1.0))
    assert s == 1.0 and np.array_equal(d3, dsi)


def test_fill_bragg_neighbour_mean():
    g = _grid(np.diag([0.25, 0.25, 0.0]), (9, 9, 1), lo=(-1.0, -1.0, 0.0))
    rng = np.random.default_rng(2)
    d = rng.random(g.inc)
    out = O.fill_bragg(g, d)
    z = d + 1j * rng.random(g.inc)
    zout = O.fill_bragg(g, z)
    hkl = g.hkl()
    ref, zref = d.copy(), z.copy()
    for h in range(9):                      # reference order: h slowest (no Bragg neighbours here)
        for k in range(9):
            x = hkl[:, h, k, 0]
            if np.all(np.abs(x - np.rint(x)) < [0.25 * np.float32(0.005)] * 2 + [np.float32(1e-4)]):
                nb = [(h + a, k + b) for a, b in ((-1, 0), (1, 0), (0, -1), (0, 1))
                      if 0 <= h + a < 9 and 0 <= k + b < 9]
                ref[h, k, 0] = np.mean([ref[p, q, 0] for p, q in nb])
                zref[h, k, 0] = np.mean([zref[p, q, 0] for p, q in nb])
    np.testing.assert_allclose(out, ref, rtol=1e-14)
    np.testing.assert_allclose(zout, zref, rtol=1e-14)
    assert not np.array_equal(out, d)


def test_closed_form_gradient_reference_matches_oracle(oracle):
    """bench.fp64_gradient_perfect_lattice (F of a perfect lattice in closed
    form, the FP64 reference of the adjoint at the 100 000-atom scale) against
    the oracle's direct FP64 gradient on a 3 x 3 x 3-cell rock salt."""
    import bench
    from diffusecode_gb300 import _abi
    from diffusecode_gb300 import structures as S
    cr, g = S.rocksalt_volume(cells=(3, 3, 3), inc=9, step=0.3)
    tgt = S.perturbed_copy(cr, 3, 0.05, 5.64, 0.1)
    op = _abi.default_opts(ldbw=1, phase=_abi.PHASE_EXACT64)
    rc, csf, acsf, it, info = oracle.four_run(tgt, g, op)
    wt = 1.0 / (it + 1.0)
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, op, it, wt)
    atoms = np.arange(0, cr.natoms, 7)
    c2, gp, go = bench.fp64_gradient_perfect_lattice(cr, g, it, wt, atoms)
    assert abs(c2 - oc2) <= 1e-10 * oc2
    np.testing.assert_allclose(gp, ogp[atoms], rtol=0, atol=1e-9 * np.abs(ogp).max())
    np.testing.assert_allclose(go, ogo[atoms], rtol=0, atol=1e-9 * np.abs(ogo).max())


def _point_group_mmm():
    ops = []
    for sx in (1, -1):
        for sy in (1, -1):
            for sz in (1, -1):
                ops.append(np.diag([sx, sy, sz]).astype(float))
    return np.array(ops)


def test_four_symm_known_answers():
    """four_symm on a centred 5 x 5 x 1 grid: a 2-fold axis along z averages
    each pixel with its mirror through the centre and divides by the two
    operations as well (csf_sym / weight / nops, fourier_sup.f90:4161); the
    identity alone returns the array; an off-centre grid leaves the pixels
    whose image falls outside with weight 1."""
    g = _grid(np.diag([0.5, 0.5, 0.0]), (5, 5, 1), lo=(-1.0, -1.0, 0.0))
    rng = np.random.default_rng(4)
    d = rng.random(g.inc)
    two = np.array([np.eye(3), np.diag([-1.0, -1.0, 1.0])])
    out = O.four_symm(g, d, two)
    want = (d + d[::-1, ::-1, :]) / 2 / 2
    np.testing.assert_allclose(out, want, rtol=1e-15)
    np.testing.assert_array_equal(O.four_symm(g, d, np.eye(3)[None]), d)
    z = d + 1j * rng.random(g.inc)
    np.testing.assert_allclose(O.four_symm(g, z, two), (z + z[::-1, ::-1, :]) / 4, rtol=1e-15)
    # off centre by one pixel along x: pixel column 0 has no image inside
    g2 = _grid(np.diag([0.5, 0.5, 0.0]), (5, 5, 1), lo=(-0.5, -1.0, 0.0))
    out2 = O.four_symm(g2, d, two)
    # hkl = 0 at pixel (1, 2): h -> 2 - h along x, k -> 4 - k along y
    for h in range(5):
        for k in range(5):
            hh = 2 - h
            if 0 <= hh < 5:
                assert abs(out2[h, k, 0] - (d[h, k, 0] + d[hh, 4 - k, 0]) / 2 / 2) < 1e-15
            else:
                assert abs(out2[h, k, 0] - d[h, k, 0] / 1 / 2) < 1e-15
