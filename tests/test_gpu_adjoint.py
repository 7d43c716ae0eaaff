"""Adjoint (dgpu_chi2_grad): against the oracle's FP64 gradient, against
central finite differences, and through the autograd wrapper."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S

pytestmark = pytest.mark.gpu


def _target(cr, grid, ctx, seed=3, sigma=0.05, occ_pm=0.1, a_lat=4.0):
    tgt = S.perturbed_copy(cr, seed, sigma, a_lat, occ_pm)
    r = FR.four_run(tgt, grid, K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT, friedel=0), ctx=ctx)
    return r.dsi, 1.0 / (r.dsi + 1.0)


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_gradient_vs_oracle_fp64(oracle, ctx, engine):
    from diffusecode_gb300.autograd import chi2_grad
    cr, g = S.small_random(seed=8, natoms=120, nscat=2, inc=(9, 7, 5))
    cr.atom_occ = np.linspace(0.9, 1.1, cr.natoms).astype(np.float32)
    it, wt = _target(cr, g, ctx)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine)
    c2, gp, go, _ = chi2_grad(cr, g, op, it, wt, ctx=ctx)
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, op, it, wt)
    assert abs(c2 - oc2) <= 1e-4 * oc2
    assert np.max(np.abs(gp - ogp)) <= 2e-4 * np.abs(ogp).max()
    assert np.max(np.abs(go - ogo)) <= 2e-4 * np.abs(ogo).max()
    assert np.all(gp[cr.iscat == 0] == 0) and np.all(go[cr.iscat == 0] == 0)


@pytest.mark.parametrize("inc", [(97, 5, 3), (9, 71, 69)], ids=["two-column-chunks", "many-rows"])
def test_tc_adjoint_shapes(oracle, ctx, inc):
    """Tensor-core adjoint on boxes with more than 64 columns on every axis
    choice (two column chunks) and with many row tiles, three atom types,
    against the oracle's FP64 gradient."""
    from diffusecode_gb300.autograd import chi2_grad
    cr, _ = S.small_random(seed=21, natoms=300, nscat=3, span=4.0)
    st = [4.0 / (n - 1) for n in inc]              # about 4 reciprocal units along every axis
    vi = np.array([[st[0], 0.2 * st[1], 0.1 * st[2]],
                   [0.1 * st[0], st[1], -0.1 * st[2]],
                   [0.05 * st[0], 0.1 * st[1], st[2]]])
    eck = np.zeros((3, 4))
    eck[:, 0] = -0.5 * (vi @ (np.asarray(inc) - 1)) + np.array([0.013, -0.021, 0.017])
    g = S.GridData(eck=eck, vi=vi, inc=inc)
    cr.atom_occ = np.linspace(0.8, 1.2, cr.natoms).astype(np.float32)
    it, wt = _target(cr, g, ctx)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC, friedel=0)
    c2, gp, go, _ = chi2_grad(cr, g, op, it, wt, ctx=ctx)
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, op, it, wt)
    assert abs(c2 - oc2) <= 1e-4 * oc2
    assert np.max(np.abs(gp - ogp)) <= 2e-4 * np.abs(ogp).max()
    assert np.max(np.abs(go - ogo)) <= 2e-4 * np.abs(ogo).max()


def test_gradient_with_friedel_reduction(oracle, ctx):
    """Centred odd grid: the GPU sums over half the grid with mirror weights."""
    from diffusecode_gb300.autograd import chi2_grad
    cr, g = S.perovskite_plane(cells=2)
    g = S.GridData.from_corners((-2, -2, 0), (2, -2, 0), (-2, 2, 0), inc=(21, 21, 1))
    it, wt = _target(cr, g, ctx)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT)
    c2, gp, go, info = chi2_grad(cr, g, op, it, wt, ctx=ctx)
    assert info.friedel_dim == 1
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, op, it, wt)
    assert abs(c2 - oc2) <= 1e-4 * oc2
    assert np.max(np.abs(gp - ogp)) <= 2e-4 * np.abs(ogp).max()
    assert np.max(np.abs(go - ogo)) <= 2e-4 * np.abs(ogo).max()


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_central_finite_differences(ctx, engine):
    """d chi2 / d x by central differences on seeded atoms: a 1e-4 A step for
    the CUDA-core engine; 1e-3 A for the tensor-core engine, whose ~1e-6
    relative noise in chi2 would otherwise dominate the difference (the
    truncation error of the central difference stays ~1e-6 relative)."""
    from diffusecode_gb300.autograd import chi2_grad
    a = 5.64
    cr, g = S.rocksalt_volume(cells=(3, 3, 3), inc=17, step=0.2)
    it, wt = _target(cr, g, ctx, a_lat=a)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine)
    c2, gp, go, _ = chi2_grad(cr, g, op, it, wt, ctx=ctx)
    rng = np.random.Generator(np.random.PCG64(12))
    h = (1e-4 if engine == _abi.ENGINE_DIRECT else 1e-3) / a
    scale = np.abs(gp).max()
    for atom in rng.choice(cr.natoms, 6, replace=False):
        for k in range(3):
            vals = []
            for sgn in (1, -1):
                p = cr.pos.copy()
                p[atom, k] += sgn * h
                c, _, _, _ = chi2_grad(cr.with_positions(p), g, op, it, wt, ctx=ctx)
                vals.append(c)
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - gp[atom, k]) <= 1e-3 * scale + 1e-3 * abs(gp[atom, k])


def test_autograd_wrapper(ctx):
    import torch
    from diffusecode_gb300.autograd import chi2, chi2_grad
    cr, g = S.small_random(seed=4, natoms=60, nscat=2, inc=(7, 5, 3))
    it, wt = _target(cr, g, ctx)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT)
    pos = torch.tensor(cr.pos, requires_grad=True)
    occ = torch.ones(cr.natoms, dtype=torch.float64, requires_grad=True)
    val = chi2(pos, occ, cr, g, op, it, wt)
    val.backward()
    c2, gp, go, _ = chi2_grad(cr.with_positions(cr.pos, np.ones(cr.natoms, np.float32)), g, op, it, wt, ctx=ctx)
    assert abs(val.item() - c2) <= 1e-12 * c2
    np.testing.assert_allclose(pos.grad.numpy(), gp, rtol=1e-12)
    np.testing.assert_allclose(occ.grad.numpy(), go, rtol=1e-12)


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_autograd_wrapper_device_tensors(ctx, engine):
    """CUDA tensors take the device-resident entry (dgpu_chi2_grad_device):
    the same chi2 and gradients as the host entry on the same context (whose
    tuned tensor-core tile both then use), and a second call reusing the
    context's buffers agrees with the first."""
    import torch
    from diffusecode_gb300.autograd import chi2, chi2_grad
    cr, g = S.small_random(seed=5, natoms=200, nscat=2, inc=(11, 9, 5))
    it, wt = _target(cr, g, ctx)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine)
    dev = torch.device("cuda:0")
    occ_h = np.linspace(0.9, 1.1, cr.natoms).astype(np.float32)
    c2, gp, go, _ = chi2_grad(cr.with_positions(cr.pos, occ_h), g, op, it, wt)     # the default context
    for _ in range(2):
        pos = torch.tensor(cr.pos, device=dev, requires_grad=True)
        occ = torch.tensor(occ_h, device=dev, requires_grad=True)
        val = chi2(pos, occ, cr, g, op, torch.from_numpy(it).to(dev), torch.from_numpy(wt).to(dev))
        val.backward()
        assert abs(val.item() - c2) <= 1e-12 * c2
        np.testing.assert_allclose(pos.grad.cpu().numpy(), gp, rtol=1e-12, atol=1e-12 * np.abs(gp).max())
        np.testing.assert_allclose(occ.grad.cpu().numpy(), go, rtol=1e-6, atol=1e-9 * np.abs(go).max())


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_gradient_vs_fp64_closed_form_rocksalt(ctx, engine):
    """A 10 x 10 x 8-cell rock salt (6400 atoms) on a 33^3 grid: the gradient
    of 300 seeded atoms against the FP64 closed-form reference of a perfect
    lattice (bench.fp64_gradient_perfect_lattice, itself pinned to the
    oracle), within 2e-4 of the largest component.  chi2 within 1e-6 on the
    CUDA-core engine and 1e-4 on the tensor cores: on a perfect lattice the
    Bragg peaks dominate chi2, where the tensor-core sums are coherent and
    carry a relative error of ~1e-6, and chi2 amplifies it by I / (I - I_t)."""
    import bench
    from diffusecode_gb300.autograd import chi2_grad
    cr, g = S.rocksalt_volume(cells=(10, 10, 8), inc=33, step=0.2)
    it, wt = _target(cr, g, ctx, a_lat=5.64)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine)
    c2, gp, go, _ = chi2_grad(cr, g, op, it, wt, ctx=ctx)
    atoms = np.sort(np.random.Generator(np.random.PCG64(6)).choice(cr.natoms, 300, replace=False))
    c64, gp64, go64 = bench.fp64_gradient_perfect_lattice(cr, g, it, wt, atoms)
    assert abs(c2 - c64) <= (1e-6 if engine == _abi.ENGINE_DIRECT else 1e-4) * c64
    assert np.max(np.abs(gp[atoms] - gp64)) <= 2e-4 * np.abs(gp64).max()
    assert np.max(np.abs(go[atoms] - go64)) <= 2e-4 * np.abs(go64).max()


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
@pytest.mark.parametrize("fave", [1.0, 0.5])
def test_gradient_with_average_vs_oracle(oracle, ctx, engine, fave):
    """<F> subtracted (four_aver): every atom of a selected cell enters A(h)
    a second time, moved into one cell, and the gradient adds that term.
    A perturbed 3 x 3 x 3-cell rock salt on a centred 9^3 grid (Friedel-
    reduced), all cells (fave = 1) or a seeded half (fave = 0.5), against
    the oracle's FP64 gradient with the same subtraction; an occupancy-weight
    target makes the chi^2 diffuse, so the main and the folded sums cancel
    at the Bragg points as in an RMC fit."""
    from diffusecode_gb300.autograd import chi2_grad
    cr0, g = S.rocksalt_volume(cells=(3, 3, 3), inc=9, step=0.37)
    cr = S.perturbed_copy(cr0, 5, 0.04, 5.64, 0.1)
    tgt = S.perturbed_copy(cr0, 3, 0.05, 5.64, 0.1)
    cells = None
    if fave < 1.0:
        cells = (np.random.default_rng(1).random(27) < 0.5).astype(np.uint8).reshape((3, 3, 3), order="F")
    rc, _, _, it, _ = oracle.four_run(tgt, g, K.opts(phase=_abi.PHASE_EXACT64, fave=fave), aver_cells=cells)
    wt = 1.0 / (it + 1.0)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine, fave=fave)
    c2, gp, go, info = chi2_grad(cr, g, op, it, wt, ctx=ctx, aver_cells=cells)
    assert info.friedel_dim >= 1 and info.ncell == (27 if cells is None else int(cells.sum()))
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, K.opts(phase=_abi.PHASE_EXACT64, fave=fave), it, wt, aver_cells=cells)
    _, gp0, _ = oracle.chi2_grad(cr, g, K.opts(phase=_abi.PHASE_EXACT64), it, wt)
    assert np.abs(ogp - gp0).max() > 0.1 * np.abs(ogp).max()       # the <F> term matters here
    assert abs(c2 - oc2) <= 1e-4 * oc2
    assert np.max(np.abs(gp - ogp)) <= 2e-4 * np.abs(ogp).max()
    assert np.max(np.abs(go - ogo)) <= 2e-4 * np.abs(ogo).max()


def test_gradient_with_average_no_cell(oracle, ctx):
    """fave < 0 selects no cell: <F> = 0, the plain gradient."""
    from diffusecode_gb300.autograd import chi2_grad
    cr, g = S.small_random(seed=4, natoms=30, inc=(5, 5, 3))
    it, wt = _target(cr, g, ctx)
    c2, gp, go, info = chi2_grad(cr, g, K.opts(phase=_abi.PHASE_EXACT64, fave=-1.0), it, wt, ctx=ctx)
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, K.opts(phase=_abi.PHASE_EXACT64), it, wt)
    assert info.ncell == 0
    assert abs(c2 - oc2) <= 1e-4 * oc2
    assert np.max(np.abs(gp - ogp)) <= 2e-4 * np.abs(ogp).max()


def test_gradient_rejects_average_of_ref22(ctx):
    """<F> of the REF22 phases is a table sum, not a closed-form lattice: the
    gradient needs EXACT64 phases and says so."""
    from diffusecode_gb300.autograd import chi2_grad
    cr, g = S.small_random(seed=4, natoms=30, inc=(5, 5, 3))
    with pytest.raises(Exception) as e:
        chi2_grad(cr, g, K.opts(fave=1.0, phase=_abi.PHASE_REF22), np.zeros(g.inc), ctx=ctx)
    assert getattr(e.value, "code", None) == _abi.DGPU_ERR_UNSUPPORTED


LOT_CASES = {
    "box": dict(anis=False, opts=dict(ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2)), origins=[(1, 1, 1), (4, 3, 2), (5, 4, 3)]),
    "box-aver-anis": dict(anis=True, opts=dict(ilots=_abi.LOT_BOX, ls_xyz=(3, 2, 2), fave=1.0),
                          origins=[(1, 1, 1), (4, 3, 2), (5, 4, 3)]),
    "eli-all": dict(anis=False, opts=dict(ilots=_abi.LOT_ELI, ls_xyz=(3, 3, 2), lot_all=1, lperiod=0)),
}


@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
@pytest.mark.parametrize("name", sorted(LOT_CASES))
def test_gradient_with_lots_vs_oracle(oracle, ctx, engine, name):
    """Lots (box with wrap and interstitial atoms, the box with <F> of the lot
    lattice and anisotropic ADPs, every ellipsoid of a non-periodic csize):
    the per-lot sums are redone chunk by chunk after the forward pass and each
    lot's weights reach the atoms it holds; against the oracle's FP64
    gradient with the same lots."""
    from diffusecode_gb300.autograd import chi2_grad
    case = LOT_CASES[name]
    cr, g = S.small_lots_anis(anis=case["anis"], icc=(5, 4, 3), inc=(9, 9, 5))
    origins = case.get("origins")
    tgt = cr.with_positions(cr.pos + np.random.default_rng(2).normal(0, 0.01, cr.pos.shape))
    rc, _, _, it, _ = oracle.four_run(tgt, g, K.opts(phase=_abi.PHASE_EXACT64, **case["opts"]), lot_origins=origins)
    assert rc == 0
    wt = 1.0 / (it + 1.0)
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=engine, **case["opts"])
    c2, gp, go, info = chi2_grad(cr, g, op, it, wt, ctx=ctx, lot_origins=origins)
    assert info.engine_used == engine
    oc2, ogp, ogo = oracle.chi2_grad(cr, g, K.opts(phase=_abi.PHASE_EXACT64, **case["opts"]), it, wt,
                                     lot_origins=origins)
    assert abs(c2 - oc2) <= 1e-4 * oc2
    assert np.max(np.abs(gp - ogp)) <= 2e-4 * np.abs(ogp).max()
    assert np.max(np.abs(go - ogo)) <= 2e-4 * np.abs(ogo).max()
