"""Gradient of a miniFE box solve with respect to per-element conductivity.

The reference assembles with a constant conductivity k = 1.0
(ref/fem/Hex8.hpp:273).  With one conductivity kappa_e per element the
assembled operator is K(kappa) = sum_e kappa_e Khat_e (Khat_e: the k = 1
element matrix), the Dirichlet lifting moves kappa-dependent boundary columns
into b (ref/src/SparseMatrix_functions.hpp:460-479), and the solution u of the
lifted system A(kappa) u = b(kappa) is differentiable in kappa.

For a scalar loss L(u):
    A lambda = dL/du with lambda = 0 on the Dirichlet rows,
    dL/dkappa_e = -lambda_e^T Khat_e u_e          (u including boundary values)
A is symmetric (Dirichlet rows are identity rows and the matching columns are
zeroed), so the adjoint solve reuses the forward matrix and the same CG.

`BoxSolve` is the torch.autograd.Function: forward assembles and solves on the
GPU (mfe_assemble + mfe_cg_solve), backward zeroes the Dirichlet rows of the
incoming gradient (mfe_box_zero_boundary), runs the adjoint CG and contracts
element by element in the hand-written kernel k_elem_grad
(mfe_element_gradient).
"""
from __future__ import annotations

import torch

from . import (box_zero_boundary, build_system, cg_solve, element_gradient)


class BoxSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kappa, dims, tol, max_iter, precision):
        nx, ny, nz = dims
        kap = kappa.detach().to(torch.float64).contiguous()
        A, b = build_system(nx, ny, nz, kappa=kap)
        u = torch.zeros_like(b)
        res = cg_solve(A, b, u, max_iter=max_iter, tol=tol, tol_mode="relative",
                       precision=precision, allow_breakdown=False)
        if res.status != 0:
            raise RuntimeError("forward CG did not converge (status %d)" % res.status)
        ctx.A = A
        ctx.dims = dims
        ctx.tol = tol
        ctx.max_iter = max_iter
        ctx.precision = precision
        ctx.save_for_backward(u)
        return u

    @staticmethod
    def backward(ctx, grad_u):
        (u,) = ctx.saved_tensors
        nx, ny, nz = ctx.dims
        rhs = grad_u.detach().to(torch.float64).contiguous().clone()
        box_zero_boundary(nx, ny, nz, rhs)
        lam = torch.zeros_like(rhs)
        if float(rhs.abs().max()) > 0.0:
            res = cg_solve(ctx.A, rhs, lam, max_iter=ctx.max_iter, tol=ctx.tol,
                           tol_mode="relative", precision=ctx.precision, allow_breakdown=False)
            if res.status != 0:
                raise RuntimeError("adjoint CG did not converge (status %d)" % res.status)
        g = element_gradient(nx, ny, nz, u, lam)
        return g, None, None, None, None


def solve(kappa, dims, tol=1e-10, max_iter=20000, precision="f64"):
    """u = solution of the miniFE box problem with per-element conductivity
    kappa (nx*ny*nz, element-id order); differentiable in kappa."""
    return BoxSolve.apply(kappa, tuple(int(d) for d in dims), float(tol), int(max_iter),
                          precision)


def grad_l2(kappa, dims, u_target, tol=1e-10, max_iter=20000, precision="f64", ctx=None):
    """(loss, grad, u) of L = 1/2 ||u - u_target||^2 in one native call
    (mfe_adjoint_grad): forward solve, adjoint solve and element contraction
    without the autograd tape."""
    import ctypes
    from . import MfeCgResult, _opts, _ptr, default_context
    ctx = ctx or default_context()
    nx, ny, nz = (int(d) for d in dims)
    kap = kappa.detach().to(torch.float64).contiguous()
    tgt = u_target.detach().to(torch.float64).contiguous()
    u = torch.empty_like(tgt)
    g = torch.empty_like(kap)
    o, _ = _opts(max_iter, tol, "relative", precision)
    loss = ctypes.c_double()
    rf, ra = MfeCgResult(), MfeCgResult()
    ctx.check(ctx.lib.mfe_adjoint_grad(ctx.h, nx, ny, nz, _ptr(kap), _ptr(tgt), ctypes.byref(o),
                                       _ptr(u), _ptr(g), ctypes.byref(loss), ctypes.byref(rf),
                                       ctypes.byref(ra)), "mfe_adjoint_grad")
    return loss.value, g, u


def loss_l2(u, u_target):
    return 0.5 * torch.sum((u - u_target) ** 2)


def finite_difference(kappa, dims, u_target, elements, h=1e-6, tol=1e-13, max_iter=20000):
    """Central differences (L(kappa + h e_i) - L(kappa - h e_i)) / 2h of
    loss_l2 for the listed elements.  Each perturbed solve starts from the
    unperturbed solution, so its relative tolerance is relative to a residual
    of order h and the difference of the two losses is resolved far below
    the loss itself."""
    nx, ny, nz = dims
    kap = kappa.detach().to(torch.float64).contiguous()
    A, b = build_system(nx, ny, nz, kappa=kap)
    u0 = torch.zeros_like(b)
    cg_solve(A, b, u0, max_iter=max_iter, tol=1e-14, tol_mode="relative")
    out = []
    for e in elements:
        vals = []
        for s in (+1.0, -1.0):
            kp = kap.clone()
            kp[int(e)] += s * h
            Ap, bp = build_system(nx, ny, nz, kappa=kp)
            up = u0.clone()
            cg_solve(Ap, bp, up, max_iter=max_iter, tol=tol, tol_mode="relative")
            vals.append(float(loss_l2(up, u_target)))
            del Ap, bp
        out.append((vals[0] - vals[1]) / (2.0 * h))
    return torch.tensor(out, dtype=torch.float64)
