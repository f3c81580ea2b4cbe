"""torch.autograd wrapper of the friction solve (no counterpart in the reference).

    r = friction_solve(HA, HB, w, mu, f, minv=..., objA=..., objB=..., coulomb=False)

solves min 1/2 r^T W r + b^T r over r_i in K_mu_i (coulomb=False, the SOC problem) or the Coulomb friction
problem (coulomb=True) with W = H M^-1 H^T + c I (c: compliance) and b = w - H M^-1 f on the GPU, and
differentiates r with respect to HA, HB, w, mu and f through the library's adjoint (bogus_gpu_adjoint /
bogus_gpu_adjoint_primal). Tensors are float64 (host or device; they are moved through host memory). The
forward solve is Gauss-Seidel with the chosen law run to `tol` (it reaches the FP64 floor), since the gradient
is that of the fixed point at the returned r.
"""
from __future__ import annotations

import numpy as np
import torch

from . import DualFrictionProblem, GaussSeidel, PrimalFrictionProblem


def _np(t: torch.Tensor) -> np.ndarray:
    return t.detach().to("cpu", torch.float64).contiguous().numpy()


class FrictionSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, HA, HB, w, mu, f, minv, objA, objB, compliance, tol, max_sweeps, device, coulomb):
        P = PrimalFrictionProblem(minv, objA, objB, _np(HA), _np(HB), _np(w), _np(mu), f=_np(f), device=device)
        D = DualFrictionProblem(device)
        D.computeFrom(P)
        if compliance:
            D.add_compliance(compliance)
        gs = GaussSeidel()
        gs.setTol(tol)
        gs.setMaxIters(max_sweeps)
        r = np.zeros(3 * P.objA.size)
        D.solveWith(gs, r, staticProblem=not coulomb)
        ctx.D, ctx.P, ctx.r, ctx.coulomb = D, P, r, coulomb
        ctx.like = w
        return torch.as_tensor(r, dtype=torch.float64, device=w.device)

    @staticmethod
    def backward(ctx, grad_r):
        D, P = ctx.D, ctx.P
        _, dmu = D.adjoint(ctx.r, _np(grad_r), tol=1e-13, coulomb=ctx.coulomb)
        dHA, dHB, dw, df = D.adjoint_primal(P)
        dev = ctx.like.device
        t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)
        return t(dHA), t(dHB), t(dw), t(dmu), t(df), None, None, None, None, None, None, None, None


def friction_solve(HA, HB, w, mu, f, *, minv, objA, objB, compliance: float = 0.0, tol: float = 1e-30,
                   max_sweeps: int = 5000, device: int = 0, coulomb: bool = False) -> torch.Tensor:
    """Differentiable friction solve (see the module docstring). minv [nbodies, ndof, ndof], objA/objB [n]
    (objB = -1: no second body) are constants; HA, HB [n, 3, ndof], w [3n], mu [n], f [nbodies * ndof]."""
    return FrictionSolve.apply(HA, HB, w, mu, f, np.asarray(minv, np.float64), np.asarray(objA, np.int32),
                               np.asarray(objB, np.int32), float(compliance), float(tol), int(max_sweeps),
                               int(device), bool(coulomb))
