"""Dense FP64 implicit-function gradients of the SOC and Coulomb friction solves. Test infrastructure only (the
checker of the GPU adjoint; only tests/ import it).

The reference has no differentiation; this oracle defines what the GPU adjoint must compute, independently of
the GPU's formulation:

  r solves  min 1/2 r^T W r + b^T r  over  r_i in K_mu_i = {x : |x_T| <= mu x_N}   (SOCLaw<3>, the static
  problem DualFrictionProblem::solveWith(ProjectedGradient&, r) solves), i.e. the fixed point
  r = P_K(r - alpha (W r + b)) for any alpha > 0.

Differentiating the fixed point at x* = r - alpha (W r + b) with J = dP/dx(x*), K = dP/dmu(x*) (block
diagonal) gives (I - J + alpha J W) dr = -alpha J (dW r + db) + K dmu, so for a loss L with g = dL/dr:
  B^T lam = g  (B = I - J + alpha J W, solved densely),
  dL/db = -alpha J^T lam,   dL/dmu_i = K_i^T lam_i,   dL/dW = (dL/db) r^T,
and through W = H M^-1 H^T + C (C constant) and b = w - H M^-1 f, with s = dL/db, v_r = M^-1 H^T r,
v_s = M^-1 H^T s:
  dL/dH_ik = s_i (v_r - M^-1 f)_k^T + r_i (v_s)_k^T,   dL/dw = s,   dL/df = -v_s.
The projection Jacobian is written from the closed form of the projection (its values are checked against
finite differences of the projection in the tests). The Coulomb problem adds the De Saxce term to the fixed
point (implicit_gradient(coulomb=True)); the primal gradients are the same functions of s = dL/db.
"""
from __future__ import annotations

import numpy as np


def project(mu: float, x: np.ndarray) -> np.ndarray:
    """Projection on the second-order cone K_mu (3-vector, normal first), as SOCLaw::projectOnConstraint."""
    xn, xt = x[0], x[1:]
    t = np.linalg.norm(xt)
    if mu < 0:
        return np.zeros(3)
    if t <= mu * xn:
        return x.copy()
    if mu * t <= -xn:
        return np.zeros(3)
    pn = (xn + mu * t) / (1 + mu * mu)
    return np.concatenate([[pn], mu * pn * xt / t])


def projection_jacobian(mu: float, x: np.ndarray):
    """(J, K): dP/dx (3 x 3) and dP/dmu (3) at x."""
    xn, xt = x[0], x[1:]
    t = np.linalg.norm(xt)
    if mu < 0 or (mu * t <= -xn):
        return np.zeros((3, 3)), np.zeros(3)
    if t <= mu * xn:
        return np.eye(3), np.zeros(3)
    c = 1.0 / (1 + mu * mu)
    u = xt / t
    pn = (xn + mu * t) * c
    J = np.zeros((3, 3))
    J[0, 0] = c
    J[0, 1:] = mu * c * u
    J[1:, 0] = mu * c * u
    J[1:, 1:] = mu * mu * c * np.outer(u, u) + (mu * pn / t) * (np.eye(2) - np.outer(u, u))
    dpn = t * c - 2 * mu * (xn + mu * t) * c * c
    K = np.concatenate([[dpn], (pn + mu * dpn) * u])
    return J, K


def implicit_gradient(W: np.ndarray, b: np.ndarray, mu: np.ndarray, r: np.ndarray, g: np.ndarray,
                      alpha: float = 1.0, coulomb: bool = False):
    """Dense implicit gradients at the solution r: returns (dL/db, dL/dmu, dL/dW dense).

    coulomb=True: r solves the Coulomb friction problem, the fixed point r = P(r - alpha (u + s(u))) with
    u = W r + b and the De Saxce term s(u) = (mu |u_T|, 0, 0) (SOCLaw::dualityCOV, SOCLaw.hpp:92-99). With
    T = I + e_N tau^T, tau = (0, mu u_T / |u_T|) (0 where u_T = 0), the linearisation is
      (I - J + alpha J T W) dr = -alpha J T (dW r + db) + (K - alpha |u_T| J e_N) dmu,
    so B = I - J + alpha J T W, B^T lam = g, dL/db = -alpha T^T J^T lam,
    dL/dmu_i = K_i^T lam_i - alpha |u_T,i| (J lam)_i,N and dL/dW = (dL/db) r^T."""
    n = mu.size
    u = W @ r + b
    T = np.eye(3 * n)
    tn = np.zeros(n)
    x = r - alpha * u
    if coulomb:
        for i in range(n):
            ui = u[3 * i:3 * i + 3]
            t = np.linalg.norm(ui[1:])
            tn[i] = t
            x[3 * i] -= alpha * mu[i] * t
            if t > 0:
                T[3 * i, 3 * i + 1:3 * i + 3] = mu[i] * ui[1:] / t
    J = np.zeros((3 * n, 3 * n))
    K = np.zeros((n, 3))
    for i in range(n):
        Ji, Ki = projection_jacobian(mu[i], x[3 * i:3 * i + 3])
        J[3 * i:3 * i + 3, 3 * i:3 * i + 3] = Ji
        K[i] = Ki
    B = np.eye(3 * n) - J + alpha * J @ T @ W
    lam = np.linalg.solve(B.T, g)
    s = -alpha * T.T @ (J.T @ lam)
    dmu = np.einsum("ik,ik->i", K, lam.reshape(n, 3)) - alpha * tn * (J @ lam).reshape(n, 3)[:, 0]
    return s, dmu, np.outer(s, r)


def dense_H(objA, objB, HA, HB, nbodies: int, ndof: int) -> np.ndarray:
    """H (3n x nbodies ndof) from per-contact blocks (a body repeated in one contact counts once: slot A)."""
    n = len(objA)
    H = np.zeros((3 * n, nbodies * ndof))
    for i in range(n):
        a, bb = objA[i], objB[i]
        H[3 * i:3 * i + 3, ndof * a:ndof * a + ndof] += HA[i]
        if bb >= 0 and bb != a:
            H[3 * i:3 * i + 3, ndof * bb:ndof * bb + ndof] += HB[i]
    return H


def primal_gradients(s, r, minv, objA, objB, HA, HB, f=None):
    """dL/dHA, dL/dHB, dL/dw, dL/df from s = dL/db and the solution r (formulas in the module docstring)."""
    nb, d = minv.shape[0], minv.shape[1]
    n = len(objA)
    H = dense_H(objA, objB, HA, HB, nb, d)
    Mi = np.zeros((nb * d, nb * d))
    for k in range(nb):
        Mi[d * k:d * k + d, d * k:d * k + d] = minv[k]
    vr = Mi @ (H.T @ r)
    vs = Mi @ (H.T @ s)
    if f is not None:
        vr = vr - Mi @ f
    dHA = np.zeros_like(HA)
    dHB = np.zeros_like(HB)
    for i in range(n):
        a, bb = objA[i], objB[i]
        si, ri = s[3 * i:3 * i + 3], r[3 * i:3 * i + 3]
        dHA[i] = np.outer(si, vr[d * a:d * a + d]) + np.outer(ri, vs[d * a:d * a + d])
        if bb >= 0 and bb != a:
            dHB[i] = np.outer(si, vr[d * bb:d * bb + d]) + np.outer(ri, vs[d * bb:d * bb + d])
    return dHA, dHB, s.copy(), -vs
