"""torch.autograd binding of the BSE eigenvalue adjoint (thin test binding).

BSEEigenvalues.apply(mmn, hqp, w, opt, nroots, coef, tol) solves the TDA BSE
eigenproblem on the GPU (bse_davidson_solve) and returns the lowest nroots
eigenvalues; its backward pass calls the hand-written Hellmann-Feynman
gradient entry point (bse_op_eig_gradient) with grad_output as the weights,
giving d/dMmn (reference slice layout), d/dHqp (window) and d/dscreening.
BSEFullEigenvalues does the same for the full (non-TDA) BSE: the forward pass is
BSE::Solve_nonhermitian_Davidson's solve (xtp/src/libxtp/gwbse/bse.cc:315-360) on
the GPU, the backward pass bse_op_eig_gradient_full (X^T dA X + Y^T dA Y + 2 X^T dB Y).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .bse_operator import BSE_OPERATOR, BSEOperator_Options, GpuBSEContext, TCMatrix_gwbse, _p
from .davidson import DavidsonSolver


class BSEEigenvalues(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mmn, hqp, w, opt: BSEOperator_Options, nroots: int, coef=(1, 2, 1, 0), tol=1e-10,
                precision=0):
        mmn_np = mmn.detach().cpu().numpy()
        hqp_np = hqp.detach().cpu().numpy()
        w_np = w.detach().cpu().numpy()
        dense = w_np.ndim == 2
        gctx = GpuBSEContext(None if dense else w_np, TCMatrix_gwbse(mmn_np), hqp_np, opt, precision=precision,
                             dense_screening=w_np if dense else None)
        ds = DavidsonSolver()
        ds.set_tolerance(tol)
        ds.set_max_search_space(max(10 * nroots, 40))
        evals, evecs = ds.solve(BSE_OPERATOR(gctx, *coef), nroots)
        if ds.info() != "Success":
            raise RuntimeError("BSE Davidson did not converge")
        ctx.gctx = gctx
        ctx.evecs = np.asfortranarray(evecs)
        ctx.coef = coef
        ctx.shapes = (mmn.shape, hqp.shape, w.shape)
        return torch.from_numpy(evals.copy())

    @staticmethod
    def backward(ctx, grad_out):
        g = np.ascontiguousarray(grad_out.detach().cpu().numpy(), dtype=np.float64)
        gctx = ctx.gctx
        mmn_shape, hqp_shape, w_shape = ctx.shapes
        gm = np.zeros(mmn_shape)
        # window gradient of Hqp: (vt + ct)^2
        dim = gctx.size
        nh = gctx.opt.cmax - gctx.opt.vmin + 1
        gh_win = np.zeros((nh, nh), order="F")
        gw = np.zeros(w_shape)
        X = ctx.evecs
        _lib.check(gctx._L.bse_op_eig_gradient(gctx.handle, *ctx.coef, _p(X), dim, X.shape[1], _p(g), _p(gm),
                                               _p(gh_win), _p(gw)))
        gh = np.zeros(hqp_shape)
        gh[:nh, :nh] = gh_win
        return (torch.from_numpy(gm), torch.from_numpy(gh), torch.from_numpy(gw), None, None, None, None, None)


def bse_eigenvalues(mmn, hqp, w, opt, nroots, coef=(1, 2, 1, 0), tol=1e-10, precision=0):
    return BSEEigenvalues.apply(mmn, hqp, w, opt, nroots, coef, tol, precision)


class BSEFullEigenvalues(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mmn, hqp, w, opt: BSEOperator_Options, nroots: int, a_coef=(1, 2, 1, 0), b_coef=(0, 2, 0, 1),
                tol=1e-10, precision=0):
        from .bse import DavidsonOptions, solve_nonhermitian_davidson

        mmn_np = mmn.detach().cpu().numpy()
        hqp_np = hqp.detach().cpu().numpy()
        w_np = w.detach().cpu().numpy()
        dense = w_np.ndim == 2
        gctx = GpuBSEContext(None if dense else w_np, TCMatrix_gwbse(mmn_np), hqp_np, opt, precision=precision,
                             dense_screening=w_np if dense else None)
        lam, X, Y, ds = solve_nonhermitian_davidson(BSE_OPERATOR(gctx, *a_coef), BSE_OPERATOR(gctx, *b_coef),
                                                    DavidsonOptions(davidson_tolerance=tol, nmax=nroots))
        if ds.info() != "Success":
            raise RuntimeError("BSE Davidson did not converge")
        ctx.gctx = gctx
        ctx.X, ctx.Y = np.asfortranarray(X), np.asfortranarray(Y)
        ctx.coefs = (a_coef, b_coef)
        ctx.shapes = (mmn.shape, hqp.shape, w.shape)
        return torch.from_numpy(np.asarray(lam).copy())

    @staticmethod
    def backward(ctx, grad_out):
        g = np.ascontiguousarray(grad_out.detach().cpu().numpy(), dtype=np.float64)
        gctx = ctx.gctx
        mmn_shape, hqp_shape, w_shape = ctx.shapes
        gm = np.zeros(mmn_shape)
        nh = gctx.opt.cmax - gctx.opt.vmin + 1
        gh_win = np.zeros((nh, nh), order="F")
        gw = np.zeros(w_shape)
        a = (ctypes.c_int32 * 4)(*ctx.coefs[0])
        b = (ctypes.c_int32 * 4)(*ctx.coefs[1])
        _lib.check(gctx._L.bse_op_eig_gradient_full(gctx.handle, a, b, _p(ctx.X), _p(ctx.Y), gctx.size,
                                                    ctx.X.shape[1], _p(g), _p(gm), _p(gh_win), _p(gw)))
        gh = np.zeros(hqp_shape)
        gh[:nh, :nh] = gh_win
        return (torch.from_numpy(gm), torch.from_numpy(gh), torch.from_numpy(gw), None, None, None, None, None, None)


def bse_full_eigenvalues(mmn, hqp, w, opt, nroots, a_coef=(1, 2, 1, 0), b_coef=(0, 2, 0, 1), tol=1e-10,
                         precision=0):
    return BSEFullEigenvalues.apply(mmn, hqp, w, opt, nroots, a_coef, b_coef, tol, precision)
