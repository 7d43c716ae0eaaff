"""The allocation-free per-type sum (dgpu_four_strucf_noalloc).

It exists for callers that cannot allocate device memory -- e.g. a reverse
Monte Carlo loop that re-evaluates a few atoms per move and cannot afford a
synchronising cudaMalloc per call.  Its working memory is a fixed __device__
array, so it must agree with the allocating entry point dgpu_four_strucf and
keep agreeing on consecutive calls that reuse that array.  This file is
collected last so that a failure here never hides the other tests.
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


def _noalloc(ctx, xat, g, off, lmn, fnum, cf, istl):
    import torch
    dev = torch.device("cuda:0")
    x = torch.from_numpy(np.asfortranarray(xat).reshape(-1, order="F").copy()).to(dev)
    cft = torch.from_numpy(np.stack([cf.real, cf.imag], -1).ravel().copy()).to(dev)
    ist = torch.from_numpy(np.asarray(istl, np.int32).reshape(-1, order="F").copy()).to(dev)
    out = torch.full((2 * g.npoints,), 7.0, dtype=torch.float64, device=dev)   # stale content on purpose
    u, v, w = (np.ascontiguousarray(g.vi[:, k]) for k in range(3))
    o = np.asarray(off, dtype=np.float64).reshape(-1, order="F").copy()
    lm = np.asarray(lmn, np.int32).copy()
    nm = np.asarray(g.inc, np.int32)
    fn = np.asarray(fnum, np.int32)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = ctx.lib.dgpu_four_strucf_noalloc(C.c_void_p(stream), C.c_void_p(x.data_ptr()), xat.shape[0],
                                          _abi.dptr(u), _abi.dptr(v), _abi.dptr(w), _abi.dptr(o), _abi.iptr(lm),
                                          _abi.iptr(nm), _abi.iptr(fn), C.c_void_p(cft.data_ptr()),
                                          C.c_void_p(ist.data_ptr()), C.c_void_p(out.data_ptr()))
    assert rc == 0
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    return (o[0::2] + 1j * o[1::2]).reshape(g.inc, order="F")


def test_noalloc_matches_allocating_entry_twice(ctx):
    cr, g = S.perovskite_plane(cells=4)
    rc, lmn, off = FR.fourier_lmn(g.eck, g.vi, g.inc, ctx=ctx)
    rc, istl = FR.four_stltab(g, cr.rten, ctx=ctx)
    cfact = FR.four_formtab(cr, K.opts(), ctx=ctx)
    fnum = ((g.inc[0] + 1) // 2, g.inc[1], g.inc[2])
    for t in (3, 1):                 # two calls in a row, different atoms
        xat = cr.pos[cr.iscat == t]
        ref = FR.four_strucf(xat, g.vi[:, 0], g.vi[:, 1], g.vi[:, 2], off, lmn, g.inc, fnum,
                             cfact[t - 1], istl, ctx=ctx)
        got = _noalloc(ctx, xat, g, off, lmn, fnum, cfact[t - 1], istl)
        assert np.all(got[fnum[0]:] == 0)
        assert np.max(np.abs(got - ref)) <= TOL * np.abs(ref).max()


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
