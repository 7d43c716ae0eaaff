"""The allocation-free per-type sum (dgpu_four_strucf_noalloc).

It exists for callers that cannot allocate device memory -- e.g. a reverse
Monte Carlo loop that re-evaluates a few atoms per move and cannot afford a
synchronising cudaMalloc per call.  Its working memory is a fixed __device__
array, so it must agree with the oracle's four_strucf (the reference's REF22
arithmetic) and with the allocating entry point dgpu_four_strucf, and keep
agreeing on consecutive calls that reuse that array.  This file is collected
last so that a failure here never hides the other tests.

Tolerance: max |tcsf - ref| <= 1e-5 max |ref| (FP32 phasors, FP64 across
chunks; the tables are the same 2^-16-turn ones as the oracle's).
"""
import ctypes as C

import numpy as np
import pytest

import kat_cases as K
from diffusecode_gb300 import _abi
from diffusecode_gb300 import fourier as FR
from diffusecode_gb300 import structures as S

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _dev(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(torch.device("cuda:0"))


def _enqueue(ctx, xat, g, off, lmn, fnum, cf, istl, stream=None):
    """Device copies of the inputs, one call enqueued (no synchronize);
    returns (rc, output tensor, the tensors that must outlive the call)."""
    import torch
    dev = torch.device("cuda:0")
    x = _dev(np.asfortranarray(xat).reshape(-1, order="F"), np.float64) if xat.shape[0] else None
    cft = _dev(np.stack([cf.real, cf.imag], -1).ravel(), np.float64) if cf is not None else None
    ist = _dev(np.asarray(istl, np.int32).reshape(-1, order="F"), np.int32) if istl is not None else None
    out = torch.full((2 * g.npoints,), 7.0, dtype=torch.float64, device=dev)   # stale content on purpose
    u, v, w = (np.ascontiguousarray(g.vi[:, k]) for k in range(3))
    o = np.asarray(off, dtype=np.float64).reshape(-1, order="F").copy()
    lm = np.asarray(lmn, np.int32).copy()
    nm = np.asarray(g.inc, np.int32)
    fn = np.asarray(fnum, np.int32)
    st = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    rc = ctx.lib.dgpu_four_strucf_noalloc(C.c_void_p(st), ptr(x), xat.shape[0], _abi.dptr(u), _abi.dptr(v),
                                          _abi.dptr(w), _abi.dptr(o), _abi.iptr(lm), _abi.iptr(nm), _abi.iptr(fn),
                                          ptr(cft), ptr(ist), C.c_void_p(out.data_ptr()))
    return rc, out, (x, cft, ist)


def _host(out, g):
    o = out.cpu().numpy()
    return (o[0::2] + 1j * o[1::2]).reshape(g.inc, order="F")


def _noalloc(ctx, xat, g, off, lmn, fnum, cf, istl):
    import torch
    rc, out, keep = _enqueue(ctx, xat, g, off, lmn, fnum, cf, istl)
    assert rc == 0
    torch.cuda.synchronize()
    return _host(out, g)


def _plane(ctx, cells=4):
    cr, g = S.perovskite_plane(cells=cells)
    rc, lmn, off = FR.fourier_lmn(g.eck, g.vi, g.inc, ctx=ctx)
    rc, istl = FR.four_stltab(g, cr.rten, ctx=ctx)
    cfact = FR.four_formtab(cr, K.opts(), ctx=ctx)
    fnum = ((g.inc[0] + 1) // 2, g.inc[1], g.inc[2])
    return cr, g, lmn, off, istl, cfact, fnum


def test_noalloc_matches_oracle_and_allocating_entry_twice(oracle, ctx):
    cr, g, lmn, off, istl, cfact, fnum = _plane(ctx)
    for t in (3, 1):                 # two calls in a row, different atoms
        xat = cr.pos[cr.iscat == t]
        ref = oracle.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, g.inc, fnum, cfact[t - 1], istl)
        alloc = FR.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, g.inc, fnum, cfact[t - 1], istl,
                               ctx=ctx)
        got = _noalloc(ctx, xat, g, off, lmn, fnum, cfact[t - 1], istl)
        assert np.all(got[fnum[0]:] == 0)
        assert np.max(np.abs(got - ref)) <= TOL * np.abs(ref).max()
        assert np.max(np.abs(got - alloc)) <= TOL * np.abs(ref).max()


def test_noalloc_coherent_bragg_row(oracle, ctx):
    """A perfect 20 x 20 x 20 lattice on a row through Bragg points (h = 0..4
    in steps of 0.01 at k = 1, l = 0): at the peaks all 8000 terms add up in
    phase, the case where uncompensated FP32 chunk sums round with a bias."""
    icc = (20, 20, 20)
    gi, gj, gk = np.meshgrid(*(np.arange(n, dtype=np.float64) for n in icc), indexing="ij")
    xat = np.stack([gi.ravel(order="F"), gj.ravel(order="F"), gk.ravel(order="F")], 1)
    g = S.GridData.from_corners((0, 1, 0), (4, 1, 0), (0, 1, 0), inc=(401, 1, 1))
    rc, lmn, off = FR.fourier_lmn(g.eck, g.vi, g.inc, ctx=ctx)
    fnum = g.inc
    ref = oracle.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, g.inc, fnum)
    got = _noalloc(ctx, xat, g, off, lmn, fnum, None, None)
    assert abs(ref[0, 0, 0] - xat.shape[0]) < 1e-6 * xat.shape[0]      # a Bragg peak of all atoms
    assert np.max(np.abs(got - ref)) <= 1e-6 * np.abs(ref).max()


def test_noalloc_edge_cases(oracle, ctx):
    cr, g, lmn, off, istl, cfact, fnum = _plane(ctx, cells=2)
    xat = cr.pos[cr.iscat == 1]
    # no form-factor table: the raw sums
    ref = oracle.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, g.inc, fnum)
    got = _noalloc(ctx, xat, g, off, lmn, fnum, None, None)
    assert np.max(np.abs(got - ref)) <= TOL * np.abs(ref).max()
    # no atoms: zeros everywhere (the stale output is overwritten)
    got = _noalloc(ctx, np.zeros((0, 3)), g, off, lmn, fnum, cfact[0], istl)
    assert np.all(got == 0)
    # an istl value outside the table: NaN there, the other points unchanged
    bad = np.array(istl, copy=True)
    bad[3, 5, 0] = _abi.CFPKT + 1
    ok = _noalloc(ctx, xat, g, off, lmn, fnum, cfact[0], istl)
    got = _noalloc(ctx, xat, g, off, lmn, fnum, cfact[0], bad)
    assert np.isnan(got[3, 5, 0].real)
    mask = np.ones(g.inc, bool)
    mask[3, 5, 0] = False
    np.testing.assert_array_equal(got[mask], ok[mask])


def test_noalloc_two_calls_queued_on_one_stream(oracle, ctx):
    """Two calls enqueued back to back on one stream, one synchronize after
    both: the second reuses the array the first has written, in stream order."""
    import torch
    cr, g, lmn, off, istl, cfact, fnum = _plane(ctx)
    s = torch.cuda.Stream(device=torch.device("cuda:0"))
    outs = []
    with torch.cuda.stream(s):
        for t in (2, 3):
            xat = cr.pos[cr.iscat == t]
            rc, out, keep = _enqueue(ctx, xat, g, off, lmn, fnum, cfact[t - 1], istl, stream=s.cuda_stream)
            assert rc == 0
            outs.append((t, out, keep))
    s.synchronize()
    for t, out, keep in outs:
        xat = cr.pos[cr.iscat == t]
        ref = oracle.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, g.inc, fnum, cfact[t - 1], istl)
        assert np.max(np.abs(_host(out, g) - ref)) <= TOL * np.abs(ref).max()


def test_noalloc_rejects_oversize(ctx):
    g = S.GridData.from_corners((-1, -1, 0), (1, -1, 0), (-1, 1, 0), inc=(11, 11, 1))
    big = np.zeros(9)
    lmn = np.zeros(6, np.int32)
    num = np.asarray(g.inc, np.int32)
    u = np.ascontiguousarray(g.vi[:, 0])
    rc = ctx.lib.dgpu_four_strucf_noalloc(None, C.c_void_p(16), 131073, _abi.dptr(u), _abi.dptr(u), _abi.dptr(u),
                                          _abi.dptr(big), _abi.iptr(lmn), _abi.iptr(num), _abi.iptr(num), None, None,
                                          C.c_void_p(16))
    assert rc == _abi.DGPU_ERR_SCRATCH_SIZE
    huge = np.asarray([1001, 1001, 1], np.int32)
    rc = ctx.lib.dgpu_four_strucf_noalloc(None, C.c_void_p(16), 10, _abi.dptr(u), _abi.dptr(u), _abi.dptr(u),
                                          _abi.dptr(big), _abi.iptr(lmn), _abi.iptr(huge), _abi.iptr(huge), None,
                                          None, C.c_void_p(16))
    assert rc == _abi.DGPU_ERR_SCRATCH_SIZE
