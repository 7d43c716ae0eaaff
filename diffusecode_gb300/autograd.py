"""chi^2 of the diffuse intensity and its gradient as a torch.autograd.Function.

chi2 = sum_h w(h) (I(h) - I_target(h))^2 over the grid, I = diff_scale |F|^2
as four_run computes it.  The gradient with respect to every atom position
(lattice units, shape (N, 3)) and per-atom occupancy weight (N,) comes from
the library's adjoint kernel (dgpu_chi2_grad) -- the analytic replacement for
the finite differences REFINE/RMC take by re-running macros
(refine/prog/refine_run.f90:491-759).

CUDA tensors go through dgpu_chi2_grad_device: positions, types,
occupancies, target, weights and both gradients stay in device memory, and
one double (chi2) comes back to the host per call.  CPU tensors go through
the host entry dgpu_chi2_grad.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _abi
from ._lib import default_context
from .fourier import attach_selections
from .structures import CrystalData, GridData


def chi2_grad(cr: CrystalData, grid: GridData, opts, i_target, weight=None, ctx=None, aver_cells=None,
              lot_origins=None):
    """(chi2, grad_pos (N,3), grad_occ (N,), info) through the host C-ABI.
    opts.fave > 0 subtracts <F> (aver_cells: the cells drawn over csize when
    fave < 1) and differentiates through it; with lots (opts.ilots) the
    intensity is the lots' normalised sum and an atom's gradient adds its
    terms over the lots that hold it (lot_origins: lbeg(3,nlots))."""
    ctx = ctx or default_context()
    keep = attach_selections(opts, aver_cells, lot_origins)
    it = np.asfortranarray(np.asarray(i_target, dtype=np.float64)).reshape(-1, order="F").copy()
    wt = None if weight is None else np.asfortranarray(np.asarray(weight, np.float64)).reshape(-1, order="F").copy()
    chi2 = np.zeros(1)
    gp = np.zeros(3 * cr.natoms)
    go = np.zeros(cr.natoms)
    info = _abi.Info()
    c = cr.to_c()
    g = grid.to_c()
    ctx.check(ctx.lib.dgpu_chi2_grad(ctx.h, C.byref(c), C.byref(g), C.byref(opts), _abi.dptr(it), _abi.dptr(wt),
                                     _abi.dptr(chi2), _abi.dptr(gp), _abi.dptr(go), C.byref(info)))
    del keep
    return float(chi2[0]), gp.reshape(-1, 3), go, info


def grid_flat(a, device):
    """A grid array shaped grid.inc (numpy or torch) as a contiguous float64
    device tensor in the library's order (first axis fastest)."""
    t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.asarray(a, dtype=np.float64))
    t = t.to(device=device, dtype=torch.float64)
    return t.permute(*reversed(range(t.dim()))).contiguous().view(-1)


def chi2_grad_device(cr: CrystalData, grid: GridData, opts, pos, occ, i_target, weight=None, iscat=None,
                     ctx=None, aver_cells=None):
    """(chi2, grad_pos (N,3), grad_occ (N,), info) with the per-atom and
    per-point arrays on the GPU: pos (N,3) float64 and occ (N,) CUDA tensors,
    i_target / weight shaped grid.inc (torch or numpy).  iscat: a cached
    device copy of cr.iscat (made here when None).  aver_cells as for
    chi2_grad."""
    ctx = ctx or default_context()
    keep = attach_selections(opts, aver_cells)
    dev = pos.device
    p = pos.detach().to(torch.float64).contiguous()
    o = occ.detach().to(torch.float32).contiguous()
    isc = iscat if iscat is not None else torch.from_numpy(np.asarray(cr.iscat, np.int32)).to(dev)
    it = grid_flat(i_target, dev)
    wt = None if weight is None else grid_flat(weight, dev)
    gp = torch.zeros((cr.natoms, 3), dtype=torch.float64, device=dev)
    go = torch.zeros(cr.natoms, dtype=torch.float64, device=dev)
    chi2 = np.zeros(1)
    info = _abi.Info()
    ian = None if cr.ianis is None else torch.from_numpy(np.asarray(cr.ianis, np.int32)).to(dev)
    c = cr.to_c(pos_ptr=C.cast(p.data_ptr(), C.POINTER(C.c_double)),
                iscat_ptr=C.cast(isc.data_ptr(), C.POINTER(C.c_int32)),
                occ_ptr=C.cast(o.data_ptr(), C.POINTER(C.c_float)),
                ianis_ptr=None if ian is None else C.cast(ian.data_ptr(), C.POINTER(C.c_int32)))
    g = grid.to_c()
    torch.cuda.synchronize(dev)          # the library's stream reads what torch's stream wrote
    ctx.check(ctx.lib.dgpu_chi2_grad_device(ctx.h, C.byref(c), C.byref(g), C.byref(opts),
                                            C.c_void_p(it.data_ptr()),
                                            C.c_void_p(wt.data_ptr()) if wt is not None else None,
                                            _abi.dptr(chi2), C.c_void_p(gp.data_ptr()), C.c_void_p(go.data_ptr()),
                                            C.byref(info)))
    del keep
    return float(chi2[0]), gp, go, info


class StructureFactorChi2(torch.autograd.Function):
    """chi2(pos, occ); pos (N,3) float64 in lattice units, occ (N,) float32/64."""

    @staticmethod
    def forward(fctx, pos, occ, cr: CrystalData, grid: GridData, opts, i_target, weight):
        if pos.is_cuda:
            chi2, gp, go, _ = chi2_grad_device(cr, grid, opts, pos, occ, i_target, weight)
            fctx.save_for_backward(gp.to(pos.dtype), go.to(occ.dtype))
            return torch.tensor(chi2, dtype=torch.float64, device=pos.device)
        p = pos.detach().cpu().numpy().astype(np.float64)
        o = occ.detach().cpu().numpy().astype(np.float32)
        cur = cr.with_positions(np.ascontiguousarray(p), o)
        chi2, gp, go, _ = chi2_grad(cur, grid, opts, i_target, weight)
        fctx.save_for_backward(torch.from_numpy(gp).to(pos.device, pos.dtype),
                               torch.from_numpy(go).to(occ.device, occ.dtype))
        return torch.tensor(chi2, dtype=torch.float64, device=pos.device)

    @staticmethod
    def backward(fctx, gout):
        gp, go = fctx.saved_tensors
        return gout * gp, gout * go, None, None, None, None, None


def chi2(pos, occ, cr, grid, opts, i_target, weight=None):
    return StructureFactorChi2.apply(pos, occ, cr, grid, opts, i_target, weight)
