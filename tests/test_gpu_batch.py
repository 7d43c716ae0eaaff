"""Batched population (dgpu_batch_run): every member against the oracle's
exact FP64 intensity, gradients against the single-crystal adjoint, and a
second call (graph replay) with moved atoms."""
import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _members():
    pop = S.population(seed=9, count=5, nmin=200, nmax=4000)
    out = []
    for cr, g in pop:
        n = min(g.inc[0], 41)
        n = n if n % 2 else n - 1
        hm = 1.5
        g2 = S.GridData.from_corners((-hm, -hm, 0), (hm, -hm, 0), (-hm, hm, 0), inc=(n, n, 1))
        out.append((cr, g2))
    return out


def test_batch_forward_vs_oracle(oracle, ctx):
    mem = _members()
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC)
    dsi, chi2, gp, go, ms = FR.batch_run([m[0] for m in mem], [m[1] for m in mem], op, ctx=ctx)
    assert ms > 0
    for (cr, g), d in zip(mem, dsi):
        rc, csf, acsf, ref, info = oracle.four_run(cr, g, op)
        assert K.rel_err(d, ref, K.incoherent_floor(cr, g, op)) <= TOL


def test_batch_graph_size_does_not_grow_with_members(ctx):
    """Every stage is one member-indexed launch: the forward graph has the
    same nodes for 2 and for 5 members (under 20), and the gradient graph
    adds a fixed set."""
    mem = _members()
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC)
    counts = {}
    for k in (2, 5):
        crs, grids = [m[0] for m in mem[:k]], [m[1] for m in mem[:k]]
        FR.batch_run(crs, grids, op, ctx=ctx)
        fwd = FR.batch_graph_nodes(ctx)
        FR.batch_run(crs, grids, op, [np.ones(g.inc) for g in grids], None, ctx=ctx)
        counts[k] = (fwd, FR.batch_graph_nodes(ctx))
    assert counts[2] == counts[5]
    (nf, kf), (ng, kg) = counts[5]
    assert nf < 20 and kf <= 8
    assert ng > nf and kg <= kf + 6


def test_batch_gradients_and_replay(ctx):
    from diffusecode_gb300.autograd import chi2_grad
    mem = _members()
    crs = [m[0] for m in mem]
    grids = [m[1] for m in mem]
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC)
    targets, weights = [], []
    for i, (cr, g) in enumerate(mem):
        tgt = S.perturbed_copy(cr, 100 + i, 0.03, 4.0, 0.0)
        it = FR.four_run(tgt, g, K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_DIRECT), ctx=ctx).dsi
        targets.append(it)
        weights.append(1.0 / (it + 1.0))
    for step in range(2):
        if step == 1:     # same shapes, moved atoms: the captured graph is replayed
            rng = np.random.Generator(np.random.PCG64(77))
            crs = [c.with_positions(c.pos + rng.normal(0, 0.002, c.pos.shape)) for c in crs]
        dsi, chi2, gp, go, ms = FR.batch_run(crs, grids, op, targets, weights, ctx=ctx)
        for i, (cr, g) in enumerate(zip(crs, grids)):
            c2, gps, gos, _ = chi2_grad(cr, g, op, targets[i], weights[i], ctx=ctx)
            assert abs(chi2[i] - c2) <= 1e-4 * c2
            assert np.max(np.abs(gp[i] - gps)) <= 1e-3 * np.abs(gps).max()
            assert np.max(np.abs(go[i] - gos)) <= 1e-3 * np.abs(gos).max()


def test_population_members_vs_fp64_sampled(ctx):
    """The 64-crystal population of the bench (2 000 - 200 000 atoms, planes of
    129^2 - 257^2 points, one graph launch): every member's |F|^2 against an
    FP64 numpy sum at 16 sampled points, within 1e-5 of I + N<|f|^2>."""
    import bench
    pop = S.population()
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC)
    dsi, chi2, gp, go, ms = FR.batch_run([c for c, g in pop], [g for c, g in pop], op, ctx=ctx)
    worst = 0.0
    for k, ((cr, g), d) in enumerate(zip(pop, dsi)):
        rng = np.random.Generator(np.random.PCG64(2000 + k))
        idx = np.stack([rng.integers(0, n, 16) for n in g.inc], 1)
        i64, fl = bench.fp64_points(cr, g, idx)
        worst = max(worst, float(np.max(np.abs(d[idx[:, 0], idx[:, 1], idx[:, 2]] - i64) / (i64 + fl))))
    assert worst <= TOL


def test_batch_anisotropic_members(oracle, ctx):
    """Members with anisotropic ADPs (three ADP types) beside isotropic ones:
    each summed per (type, ADP type) group with its four_dbw term, against
    the oracle; gradients against the single-crystal adjoint."""
    from diffusecode_gb300.autograd import chi2_grad
    mem = []
    for k, icc in enumerate([(5, 4, 3), (4, 4, 2), (6, 3, 3)]):
        cr, g = S.small_lots_anis(seed=7 + k, icc=icc, anis=(k != 1))
        mem.append((cr, g))
    op = K.opts(phase=_abi.PHASE_EXACT64, engine=_abi.ENGINE_TC, ldbw=1)
    crs, grids = [m[0] for m in mem], [m[1] for m in mem]
    dsi, _, _, _, _ = FR.batch_run(crs, grids, op, ctx=ctx)
    for (cr, g), d in zip(mem, dsi):
        rc, csf, acsf, ref, info = oracle.four_run(cr, g, op)
        assert rc == 0
        assert K.rel_err(d, ref, K.incoherent_floor(cr, g, K.opts(ldbw=0))) <= TOL
    targets = [d * 1.1 for d in dsi]
    weights = [1.0 / (t + 1.0) for t in targets]
    _, chi2, gp, go, _ = FR.batch_run(crs, grids, op, targets, weights, ctx=ctx)
    for k, (cr, g) in enumerate(mem):
        c2, gp1, go1, _ = chi2_grad(cr, g, op, targets[k], weights[k], ctx=ctx)
        # the two runs may pick different tensor-core tiles (rounding ~1e-7
        # of I, amplified by I / (I - I_t) = 10 in chi^2): the bounds of the
        # isotropic batch test
        assert abs(chi2[k] - c2) <= 1e-4 * c2
        assert np.max(np.abs(gp[k] - gp1)) <= 1e-3 * np.abs(gp1).max()
        assert np.max(np.abs(go[k] - go1)) <= 1e-3 * np.abs(go1).max()
