"""Powder "complete" mode (discus/prog/powder.f90:1829-2593): the oracle's
literal rod loop against an independent numpy restatement (CPU), and the
device's slab evaluation against the oracle (GPU).

The numpy restatement below follows powder_complete, do_proj
(metric.f90:337-548), four_run_powder (powder.f90:3143-3206), powder_split
(:2975-3008) and calc_preferred (:3332-3376) with plain loops, numpy
exp(2 pi i h.x) sums and neutron scattering lengths (lxray = 0, so cfact is
occ * c and needs no sin(theta)/lambda table).
"""
import math

import numpy as np
import pytest

from diffusecode_gb300 import _abi
from diffusecode_gb300 import structures as S
from oracle import oracle as O


# ---------------------------------------------------------------------------
# independent restatement

def _do_proj(u, v, sp, rten, gten):
    """res_para(1:6) of do_proj for the space letters sp."""
    u, v = np.array(u, float), np.array(v, float)
    if sp[0] == "r":
        u = rten @ u
    if sp[1] == "r":
        v = rten @ v
    uv = u @ (gten @ v)
    vv = v @ (gten @ v)
    with np.errstate(divide="ignore", invalid="ignore"):
        w = v / uv / vv
    if sp[2] == "r":
        w = gten @ w
    h = gten @ v
    uh = u @ h
    hh = h @ (rten @ h)
    w2 = u - uh * v / hh
    if sp[3] == "r":
        w2 = gten @ w2
    return np.concatenate([w, w2])


def _rods(rten, pw, ano):
    dh, dk, dl = pw.hkl_del
    s1, s2, s3 = pw.hkl_shift
    hmax = pw.a0[0] * pw.ds_max
    h_end = int(hmax / dh)
    rods = []
    for ih in range(-h_end if ano else 0, h_end + 1):
        hh = ih * dh + s1
        if hh == 0.0:
            u, u2 = np.zeros(3), 0.0
        else:
            u = _do_proj((hh, 0, 0), (1, 0, 0), "rdrr", rten, pw.gten)[:3]
            u2 = u @ (rten @ u)
        v = _do_proj((0, 1, 0), (1, 0, 0), "ddrr", rten, pw.gten)[3:]
        v = v / math.sqrt(v @ (rten @ v))
        rr = pw.ds_max ** 2 - u2
        if not rr > 0:
            continue
        wmin, wmax = u - math.sqrt(rr) * v, u + math.sqrt(rr) * v
        k_start = 0 if (not ano and ih == 0) else int(wmin[1] / dk)
        for ik in range(k_start, int(wmax[1] / dk) + 1):
            kk = ik * dk + s2
            a = rten[2, 2]
            b = 2.0 * (rten[0, 2] * hh + rten[1, 2] * kk)
            c = rten[0, 0] * hh ** 2 + 2.0 * rten[0, 1] * hh * kk + rten[1, 1] * kk ** 2 - pw.ds_max ** 2
            disc = b * b - 4.0 * a * c
            if not disc > 0:
                continue
            lo, hi = (-b - math.sqrt(disc)) / 2 / a, (-b + math.sqrt(disc)) / 2 / a
            l0 = 0 if (not ano and ih == 0 and ik == 0) else int(lo / dl)
            l1 = int(hi / dl)
            n = int(np.rint((l1 * dl - l0 * dl) / dl)) + 1
            rods.append((ih, ik, hh, kk, l0, n))
    return rods


def _angle_direct(w, pref, gten):
    x, y = -np.asarray(w, float), -np.asarray(pref, float)
    xx, yy, xy = math.sqrt(x @ gten @ x), math.sqrt(y @ gten @ y), x @ gten @ y
    if not (xx > 0 and yy > 0):
        return 0.0
    arg = xy / (xx * yy)
    if abs(arg) < 1:
        return math.acos(arg) / float(np.float32(math.pi / 180))
    return 0.0 if arg >= 1 else 180.0


def _pref(hkl, pw):
    alpha = _angle_direct(hkl, pw.pref_hkl, pw.gten)
    if pw.pref_type == _abi.PREF_RIETVELD:
        a2 = alpha ** 2 if alpha <= 90 else (180 - alpha) ** 2
        return pw.pref_g2 + (1 - pw.pref_g2) * math.exp(pw.pref_g1 * a2)
    if pw.pref_type == _abi.PREF_MARCH:
        r = math.radians(alpha)
        return pw.pref_g2 + (1 - pw.pref_g2) * ((pw.pref_g1 * math.cos(r)) ** 2 + math.sin(r) ** 2 / pw.pref_g1) ** -1.5
    return 1.0


def numpy_powder(cr, pw, ano):
    """pow_qsp of powder_complete, neutron lengths, no Debye-Waller."""
    cf = np.array([0.0] + [cr.occ[t] * cr.scat[t, 0] for t in range(1, cr.nscat + 1)])
    keep = cr.iscat > 0
    pos, f = cr.pos[keep], cf[cr.iscat[keep]]
    qsp = np.zeros(pw.n_pkt + 1)
    rods = _rods(cr.rten, pw, ano)
    dl = pw.hkl_del[2]
    for ih, ik, hh, kk, l0, n in rods:
        e31 = l0 * dl + pw.hkl_shift[2]
        ll = e31 + np.arange(n) * dl
        hkl = np.stack([np.full(n, hh), np.full(n, kk), ll], axis=1)
        F = np.exp(2j * np.pi * (hkl @ pos.T)) @ f
        hreal = abs((round(hh) - hh) / pw.hkl_del[0]) > 0.51
        kreal = abs((round(kk) - kk) / pw.hkl_del[1]) > 0.51
        for i in range(n):
            lreal = abs((np.round(ll[i]) - ll[i]) / dl) > 0.51
            if not (pw.l_all or hreal or kreal or lreal):
                continue
            q = 2 * math.pi * math.sqrt(hkl[i] @ cr.rten @ hkl[i])
            if not (pw.qmin <= q <= pw.qmax + pw.deltaq):
                continue
            inten = abs(F[i]) ** 2 * _pref(hkl[i], pw)
            x = (q - pw.qmin) / pw.deltaq
            it = int(x)
            qsp[it] += inten * (1 - (x - it))
            qsp[it + 1] += inten * (x - it)
    if not ano:
        qsp *= 2
    return qsp, rods


# ---------------------------------------------------------------------------
# cases

def _neutron_crystal(hexagonal=False):
    cr, _ = S.small_lots_anis(anis=False, lxray=False)
    if hexagonal:
        cr.rten = S.reciprocal_metric(4.0, 4.0, 5.0, 90, 90, 120)
        pw = S.PowderSpec.for_lattice(4.0, 4.0, 5.0, 90, 90, 120)
    else:
        pw = S.PowderSpec.for_lattice(4.0, 4.5, 5.0)
    return cr, pw


CASES = {
    "ortho": dict(hexagonal=False, ano=0, hkl_del=(0.25, 0.25, 0.1), ds_max=0.9, l_all=True),
    "ortho-bragg-excluded": dict(hexagonal=False, ano=0, hkl_del=(1.0, 0.5, 0.05), ds_max=1.0, l_all=False),
    "hex-ano-shift": dict(hexagonal=True, ano=1, hkl_del=(0.5, 0.5, 0.1), hkl_shift=(0.01, -0.02, 0.003),
                          ds_max=0.8, l_all=False),
    "rietveld": dict(hexagonal=False, ano=0, hkl_del=(0.5, 0.5, 0.1), ds_max=0.8, l_all=True,
                     pref_type=_abi.PREF_RIETVELD, pref_hkl=(0, 0, 1), pref_g1=-0.0005, pref_g2=0.3),
    "march": dict(hexagonal=True, ano=0, hkl_del=(0.5, 0.5, 0.1), ds_max=0.8, l_all=True,
                  pref_type=_abi.PREF_MARCH, pref_hkl=(1, 1, 0), pref_g1=0.7, pref_g2=0.1),
}


def _case(name):
    kw = dict(CASES[name])
    cr, pw = _neutron_crystal(kw.pop("hexagonal"))
    ano = kw.pop("ano")
    for k, v in kw.items():
        setattr(pw, k, v)
    pw.qmin, pw.qmax, pw.deltaq = 0.3, 5.5, 0.01
    op = _abi.default_opts(lxray=0, ldbw=0, ano=ano)
    op.phase = _abi.PHASE_EXACT64
    op.form = _abi.FORM_ANALYTIC
    return cr, pw, op, ano


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_powder_vs_numpy(name):
    cr, pw, op, ano = _case(name)
    want, rods = numpy_powder(cr, pw, ano)
    rc, got, nr, npts = O.powder_complete(cr, pw, op)
    assert rc == 0
    assert nr == len(rods) and npts == sum(r[5] for r in rods)
    assert want.max() > 0
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-11 * want.max())


def test_oracle_powder_rod_sample():
    """A rod range evaluates only those rods (the bounded CPU sample)."""
    cr, pw, op, _ = _case("ortho")
    _, full, nr, npts = O.powder_complete(cr, pw, op)
    _, a, _, na = O.powder_complete(cr, pw, op, 0, nr // 2)
    _, b, _, nb = O.powder_complete(cr, pw, op, nr // 2, nr)
    assert na + nb == npts
    np.testing.assert_allclose(a + b, full, rtol=1e-12, atol=1e-13 * full.max())


def test_do_proj_parallel_part_quirk():
    """do_proj's parallel part is v / (u.v) / |v|^2 (metric.f90:337-548): the
    plane hh = 0.25 is placed as if it were hh = 4, outside the d* = 0.9
    sphere, so powder_complete evaluates no rod in it although the sphere
    crosses it; hh = 1 is placed correctly."""
    cr, pw = _neutron_crystal()
    pw.hkl_del, pw.ds_max = (0.25, 0.25, 0.1), 0.9
    u = _do_proj((0.25, 0, 0), (1, 0, 0), "rdrr", cr.rten, pw.gten)[:3]
    np.testing.assert_allclose(u, [4.0, 0, 0], atol=1e-12)
    u1 = _do_proj((1.0, 0, 0), (1, 0, 0), "rdrr", cr.rten, pw.gten)[:3]
    np.testing.assert_allclose(u1, [1.0, 0, 0], atol=1e-12)
    rods = _rods(cr.rten, pw, 0)
    assert 0.25 ** 2 * cr.rten[0, 0] < pw.ds_max ** 2
    assert not [r for r in rods if r[0] == 1]
    assert [r for r in rods if r[0] == 4]


def test_oracle_powder_centrosymmetric():
    """Without anomalous terms |F|^2 is centrosymmetric: the full sphere
    (ano) equals the doubled half sphere on an orthogonal lattice."""
    cr, pw, op, _ = _case("ortho")
    op0 = _abi.default_opts(lxray=0, ldbw=0, ano=0)
    op1 = _abi.default_opts(lxray=0, ldbw=0, ano=1)
    for o in (op0, op1):
        o.phase, o.form = _abi.PHASE_EXACT64, _abi.FORM_ANALYTIC
    cr.delfr = np.zeros(cr.nscat + 1)
    cr.delfi = np.zeros(cr.nscat + 1)
    _, a, _, _ = O.powder_complete(cr, pw, op0)
    _, b, _, _ = O.powder_complete(cr, pw, op1)
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-11 * a.max())


def test_oracle_powder_needs_smallest_dl():
    cr, pw, op, _ = _case("ortho")
    pw.hkl_del = (0.1, 0.25, 0.25)
    rc, _, _, _ = O.powder_complete(cr, pw, op)
    assert rc == _abi.DGPU_ERR_UNSUPPORTED


# ---------------------------------------------------------------------------
# device

def _tol(engine):
    return 2e-6 if engine == _abi.ENGINE_DIRECT else 2e-5


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
@pytest.mark.parametrize("name", sorted(CASES))
def test_powder_vs_oracle(ctx, name, engine):
    from diffusecode_gb300 import fourier as FR
    cr, pw, op, _ = _case(name)
    op.engine = engine
    rc, want, nr, npts = O.powder_complete(cr, pw, op)
    assert rc == 0
    got, info = FR.powder_complete(cr, pw, op, ctx=ctx)
    assert info.rods == nr and info.rod_points == npts and info.n_pkt == pw.n_pkt
    assert info.grid_points >= npts and info.binned > 0
    t = _tol(engine)
    np.testing.assert_allclose(got, want, rtol=10 * t, atol=t * want.max())
    assert abs(got.sum() - want.sum()) <= t * want.sum()


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_powder_xray_anis_vs_oracle(ctx, engine):
    """X-ray form factors on the sin(theta)/lambda table, Debye-Waller on, and
    an anisotropic crystal (which powder_complete evaluates without any
    Debye-Waller factor)."""
    from diffusecode_gb300 import fourier as FR
    for anis in (False, True):
        cr, _ = S.small_lots_anis(anis=anis, lxray=True)
        pw = S.PowderSpec.for_lattice(4.0, 4.5, 5.0, hkl_del=(0.25, 0.25, 0.05), ds_max=0.9, qmin=0.3,
                                      qmax=5.5, deltaq=0.005, l_all=True)
        op = _abi.default_opts(lxray=1, ldbw=1, ano=0)
        op.phase, op.form, op.engine = _abi.PHASE_EXACT64, _abi.FORM_TABLE, engine
        rc, want, nr, npts = O.powder_complete(cr, pw, op)
        assert rc == 0
        got, info = FR.powder_complete(cr, pw, op, ctx=ctx)
        assert info.rods == nr and info.rod_points == npts
        t = _tol(engine)
        np.testing.assert_allclose(got, want, rtol=10 * t, atol=t * want.max())


@pytest.mark.gpu
def test_powder_centrosymmetric_large(ctx):
    """Size-independent property on a 108 000-atom alloy: without anomalous
    terms the ano (full sphere) and half-sphere patterns agree."""
    from diffusecode_gb300 import fourier as FR
    cr, _ = S.fcc_alloy_volume(seed=5, cells=30, sweeps=2, inc=3)
    cr.delfr = np.zeros(cr.nscat + 1)
    cr.delfi = np.zeros(cr.nscat + 1)
    pw = S.PowderSpec.for_lattice(3.6, 3.6, 3.6, hkl_del=(0.1, 0.1, 0.05), ds_max=0.75, qmin=0.5, qmax=4.5,
                                  deltaq=0.002, l_all=True)
    out = []
    for ano in (0, 1):
        op = _abi.default_opts(lxray=1, ldbw=1, ano=ano)
        op.phase, op.form = _abi.PHASE_EXACT64, _abi.FORM_TABLE
        q, info = FR.powder_complete(cr, pw, op, ctx=ctx)
        out.append(q)
    np.testing.assert_allclose(out[0], out[1], rtol=1e-3, atol=2e-5 * out[0].max())


@pytest.mark.gpu
def test_powder_errors(ctx):
    from diffusecode_gb300 import fourier as FR
    from diffusecode_gb300._lib import DiscusGpuError
    cr, pw, op, _ = _case("ortho")

    def code(**kw):
        o = _abi.default_opts(lxray=0)
        o.phase = _abi.PHASE_EXACT64
        p = S.PowderSpec(**{**pw.__dict__})
        for k, v in kw.items():
            if hasattr(o, k):
                setattr(o, k, v)
            else:
                setattr(p, k, v)
        try:
            FR.powder_complete(cr, p, o, ctx=ctx)
            return 0
        except DiscusGpuError as e:
            return e.code

    assert code(phase=_abi.PHASE_REF22) == _abi.DGPU_ERR_UNSUPPORTED
    assert code(hkl_del=(0.1, 0.25, 0.25)) == _abi.DGPU_ERR_UNSUPPORTED
    assert code(pref_type=7) == _abi.DGPU_ERR_ARG
    assert code(pref_type=_abi.PREF_MARCH, pref_g1=0.0) == _abi.DGPU_ERR_ARG
    assert code(ds_max=-1.0) == _abi.DGPU_ERR_ARG
    assert code(power=9) == _abi.DGPU_ERR_ARG
    assert code(form=5) == _abi.DGPU_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_powder_slab_count_invariance(ctx, engine):
    """The slab partition is a device detail: 1, 3, 8 and one slab per plane
    give the same pattern (the CUDA-core engine evaluates the slabs one after
    another, the tensor-core engine all of them in one launch with shared V
    images; they differ by FP32 rounding and the order of the FP64 bin sums)."""
    from diffusecode_gb300 import fourier as FR
    cr, pw, op, _ = _case("hex-ano-shift")
    op.engine = engine
    out = []
    for n in (1, 3, 8, 1000):
        pw.slabs = n
        q, info = FR.powder_complete(cr, pw, op, ctx=ctx)
        assert info.nslab <= n
        out.append(q)
    t = 1e-6 if engine == _abi.ENGINE_DIRECT else 2e-5
    for q in out[1:]:
        np.testing.assert_allclose(q, out[0], rtol=10 * t, atol=t * out[0].max())


def test_oracle_powder_empty():
    """Only the origin inside a tiny sphere (its Q = 0 is below qmin), or every
    Q outside the range: a zero pattern of n_pkt + 1 points."""
    cr, pw, op, _ = _case("ortho")
    pw.ds_max = 1e-3
    rc, q, nr, npts = O.powder_complete(cr, pw, op)
    assert rc == 0 and nr == 1 and npts == 1 and q.shape == (pw.n_pkt + 1,) and not q.any()
    cr, pw, op, _ = _case("ortho")
    pw.qmin, pw.qmax = 20.0, 21.0
    rc, q, nr, npts = O.powder_complete(cr, pw, op)
    assert rc == 0 and nr > 0 and not q.any()


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [_abi.ENGINE_DIRECT, _abi.ENGINE_TC])
def test_powder_empty(ctx, engine):
    from diffusecode_gb300 import fourier as FR
    cr, pw, op, _ = _case("ortho")
    op.engine = engine
    pw.ds_max = 1e-3
    q, info = FR.powder_complete(cr, pw, op, ctx=ctx)
    assert info.rods == 1 and info.binned == 0 and q.shape == (pw.n_pkt + 1,) and not q.any()
    cr, pw, op, _ = _case("ortho")
    op.engine = engine
    pw.qmin, pw.qmax = 20.0, 21.0
    q, info = FR.powder_complete(cr, pw, op, ctx=ctx)
    assert info.rods > 0 and info.binned == 0 and not q.any()
