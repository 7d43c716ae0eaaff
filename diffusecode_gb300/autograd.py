"""chi^2 of the diffuse intensity and its gradient as a torch.autograd.Function.

chi2 = sum_h w(h) (I(h) - I_target(h))^2 over the grid, I = diff_scale |F|^2
as four_run computes it.  The gradient with respect to every atom position
(lattice units, shape (N, 3)) and per-atom occupancy weight (N,) comes from
the library's adjoint kernel (dgpu_chi2_grad) -- the analytic replacement for
the finite differences REFINE/RMC take by re-running macros
(refine/prog/refine_run.f90:491-759).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _abi
from ._lib import default_context
from .structures import CrystalData, GridData


def chi2_grad(cr: CrystalData, grid: GridData, opts, i_target, weight=None, ctx=None):
    """(chi2, grad_pos (N,3), grad_occ (N,), info) through the C-ABI."""
    ctx = ctx or default_context()
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
    return float(chi2[0]), gp.reshape(-1, 3), go, info


class StructureFactorChi2(torch.autograd.Function):
    """chi2(pos, occ); pos (N,3) float64 in lattice units, occ (N,) float32/64."""

    @staticmethod
    def forward(fctx, pos, occ, cr: CrystalData, grid: GridData, opts, i_target, weight):
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
