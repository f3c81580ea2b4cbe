"""Seeded synthetic friction problems (rigid bodies, 6 dofs, diagonal mass matrices).

The reference ships no benchmark data; these generators produce the workload shapes used to measure the
friction-solve path:

* ``random_pairs``  — contacts between random distinct bodies (10 % against the ground), random
  orthonormal contact frames, contact points uniform in a unit cube (the 500-contact / 200-body case);
* ``grid``          — bodies on a jittered 3-D grid, contacts between grid neighbours (10 % against the
  ground), normals along the neighbour direction (the 200 000-contact / 50 000-body case).

Per contact and body the Jacobian block is H = s [R^T, -R^T [r]_x] (3 x 6), r the lever arm from the body
centre to the contact point, s = +1 for body A and -1 for body B, so u = H v is the relative velocity in
the contact frame (normal first). M = diag(m, m, m, I, I, I) with m ~ U[0.5, 2], I ~ U[0.05, 0.5].
b has normal part ~ U[-1, 0.5] and tangential parts ~ N(0, 0.3); mu ~ U[0.3, 0.8].
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class PrimalData:
    minv: np.ndarray   # (nbodies, 6, 6)
    objA: np.ndarray   # (n,) int32
    objB: np.ndarray   # (n,) int32, -1 = ground
    HA: np.ndarray     # (n, 3, 6)
    HB: np.ndarray     # (n, 3, 6)
    b: np.ndarray      # (n, 3)  free relative velocity in the contact frame (dual rhs)
    mu: np.ndarray     # (n,)
    seed: int
    kind: str

    @property
    def n(self) -> int:
        return int(self.objA.shape[0])

    @property
    def nbodies(self) -> int:
        return int(self.minv.shape[0])


def _skew(r: np.ndarray) -> np.ndarray:
    z = np.zeros(r.shape[0])
    return np.stack([np.stack([z, -r[:, 2], r[:, 1]], 1),
                     np.stack([r[:, 2], z, -r[:, 0]], 1),
                     np.stack([-r[:, 1], r[:, 0], z], 1)], 1)


def _random_frames(rng: np.random.Generator, n: int) -> np.ndarray:
    q, rr = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    d = np.sign(np.einsum("nii->ni", rr))
    d[d == 0] = 1.0
    return q * d[:, None, :]


def _frames_from_normals(rng: np.random.Generator, nrm: np.ndarray) -> np.ndarray:
    nrm = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    a = rng.standard_normal(nrm.shape)
    t1 = a - np.sum(a * nrm, 1, keepdims=True) * nrm
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(nrm, t1)
    return np.stack([nrm, t1, t2], 2)  # columns: normal, t1, t2


def _jacobian(R: np.ndarray, r: np.ndarray, sign: float) -> np.ndarray:
    Rt = np.transpose(R, (0, 2, 1))
    H = np.concatenate([Rt, -Rt @ _skew(r)], axis=2)
    return sign * H


def _masses(rng: np.random.Generator, nb: int) -> np.ndarray:
    m = rng.uniform(0.5, 2.0, nb)
    inertia = rng.uniform(0.05, 0.5, nb)
    minv = np.zeros((nb, 6, 6))
    for k in range(3):
        minv[:, k, k] = 1.0 / m
        minv[:, 3 + k, 3 + k] = 1.0 / inertia
    return minv


def _rhs(rng: np.random.Generator, n: int):
    b = np.empty((n, 3))
    b[:, 0] = rng.uniform(-1.0, 0.5, n)
    b[:, 1:] = rng.normal(0.0, 0.3, (n, 2))
    mu = rng.uniform(0.3, 0.8, n)
    return b, mu


def random_pairs(nbodies: int = 200, ncontacts: int = 500, seed: int = 0, ground_fraction: float = 0.1) -> PrimalData:
    rng = np.random.default_rng(seed)
    minv = _masses(rng, nbodies)
    objA = rng.integers(0, nbodies, ncontacts)
    objB = rng.integers(0, nbodies - 1, ncontacts)
    objB = np.where(objB >= objA, objB + 1, objB)
    ground = rng.random(ncontacts) < ground_fraction
    objB = np.where(ground, -1, objB)
    R = _random_frames(rng, ncontacts)
    p = rng.random((ncontacts, 3)) - 0.5
    HA = _jacobian(R, p, 1.0)
    HB = np.where(ground[:, None, None], 0.0, _jacobian(R, p, -1.0))
    b, mu = _rhs(rng, ncontacts)
    return PrimalData(minv, objA.astype(np.int32), objB.astype(np.int32), HA, HB, b, mu, seed, "random_pairs")


def grid(nbodies: int = 50_000, ncontacts: int = 200_000, seed: int = 1, ground_fraction: float = 0.1,
         jitter: float = 0.1) -> PrimalData:
    rng = np.random.default_rng(seed)
    side = int(np.ceil(nbodies ** (1.0 / 3.0)))
    idx = np.arange(nbodies)
    ijk = np.stack([idx % side, (idx // side) % side, idx // (side * side)], 1)
    centres = ijk + rng.uniform(-jitter, jitter, (nbodies, 3))
    minv = _masses(rng, nbodies)
    # neighbour pairs on the 18-neighbourhood (faces + edges), each listed once
    offs = [o for o in np.array(np.meshgrid([-1, 0, 1], [-1, 0, 1], [-1, 0, 1])).reshape(3, -1).T
            if 0 < np.abs(o).sum() <= 2 and tuple(o) > (0, 0, 0)]
    lookup = -np.ones((side, side, side), np.int64)
    lookup[ijk[:, 0], ijk[:, 1], ijk[:, 2]] = idx
    pairs = []
    for o in offs:
        nb = ijk + o
        ok = np.all((nb >= 0) & (nb < side), 1)
        j = np.full(nbodies, -1)
        j[ok] = lookup[nb[ok, 0], nb[ok, 1], nb[ok, 2]]
        sel = j >= 0
        pairs.append(np.stack([idx[sel], j[sel]], 1))
    pairs = np.concatenate(pairs)
    n_ground = int(round(ground_fraction * ncontacts))
    n_pair = ncontacts - n_ground
    if n_pair > len(pairs):
        raise ValueError("not enough neighbour pairs for the requested contact count")
    chosen = pairs[np.sort(rng.choice(len(pairs), n_pair, replace=False))]
    gb = np.sort(rng.choice(nbodies, n_ground, replace=n_ground > nbodies))
    objA = np.concatenate([chosen[:, 0], gb])
    objB = np.concatenate([chosen[:, 1], -np.ones(n_ground, np.int64)])
    # spatial contact order (by the first body): the natural order of a broad phase
    order = np.lexsort((objB, objA))
    objA, objB = objA[order], objB[order]
    n = ncontacts
    cA = centres[objA]
    cB = np.where(objB[:, None] >= 0, centres[np.maximum(objB, 0)], cA - np.array([0.0, 0.0, 1.0]))
    nrm = cB - cA
    R = _frames_from_normals(rng, nrm)
    p = 0.5 * (cA + cB) + rng.uniform(-0.05, 0.05, (n, 3))
    HA = _jacobian(R, p - cA, 1.0)
    HB = np.where(objB[:, None, None] >= 0, _jacobian(R, p - cB, -1.0), 0.0)
    b, mu = _rhs(rng, n)
    return PrimalData(minv, objA.astype(np.int32), objB.astype(np.int32), HA, HB, b, mu, seed, "grid")


def batch(nproblems: int = 4096, nmin: int = 16, nmax: int = 4096, seed: int = 4, ground_fraction: float = 0.1):
    """Independent problems with contact counts log-uniform in [nmin, nmax] and bodies = contacts / 3
    (random pairs), concatenated into one primal problem whose contact groups share no body. Returns
    (PrimalData, contact_ptr)."""
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1), nproblems))).astype(int)
    sizes = np.clip(sizes, nmin, nmax)
    parts, body_off = [], 0
    for p, n in enumerate(sizes):
        d = random_pairs(nbodies=max(2, int(n) // 3), ncontacts=int(n), seed=seed * 100003 + p,
                         ground_fraction=ground_fraction)
        parts.append((d, body_off))
        body_off += d.nbodies
    minv = np.concatenate([d.minv for d, _ in parts])
    objA = np.concatenate([d.objA + off for d, off in parts]).astype(np.int32)
    objB = np.concatenate([np.where(d.objB >= 0, d.objB + off, -1) for d, off in parts]).astype(np.int32)
    HA = np.concatenate([d.HA for d, _ in parts])
    HB = np.concatenate([d.HB for d, _ in parts])
    b = np.concatenate([d.b for d, _ in parts])
    mu = np.concatenate([d.mu for d, _ in parts])
    contact_ptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    return PrimalData(minv, objA, objB, HA, HB, b, mu, seed, "batch"), contact_ptr


def adjoint_batch(nproblems: int = 64, ncontacts: int = 20_000, seed: int = 5, ground_fraction: float = 0.1):
    """Independent random-pairs problems of `ncontacts` contacts each with bodies = contacts / 3 (each body in
    about 6 contacts), concatenated like batch(). With 3 n constraint rows on 2 n body dofs, H M^-1 H^T is
    singular; the gradient workload adds a compliance term (ADJOINT_COMPLIANCE I) so that each solution is
    unique and differentiable. Returns (PrimalData, contact_ptr)."""
    parts, body_off = [], 0
    for p in range(nproblems):
        d = random_pairs(nbodies=max(2, ncontacts // 3), ncontacts=ncontacts, seed=seed * 100003 + p,
                         ground_fraction=ground_fraction)
        parts.append((d, body_off))
        body_off += d.nbodies
    minv = np.concatenate([d.minv for d, _ in parts])
    objA = np.concatenate([d.objA + off for d, off in parts]).astype(np.int32)
    objB = np.concatenate([np.where(d.objB >= 0, d.objB + off, -1) for d, off in parts]).astype(np.int32)
    HA = np.concatenate([d.HA for d, _ in parts])
    HB = np.concatenate([d.HB for d, _ in parts])
    b = np.concatenate([d.b for d, _ in parts])
    mu = np.concatenate([d.mu for d, _ in parts])
    contact_ptr = (np.arange(nproblems + 1) * ncontacts).astype(np.int32)
    return PrimalData(minv, objA, objB, HA, HB, b, mu, seed, "adjoint_batch"), contact_ptr


ADJOINT_COMPLIANCE = 0.05

CONFIGS = {
    "c1": dict(fn=random_pairs, kw=dict(nbodies=200, ncontacts=500, seed=0)),
    "c2": dict(fn=grid, kw=dict(nbodies=50_000, ncontacts=200_000, seed=1)),
}


def make(name: str, **overrides) -> PrimalData:
    c = CONFIGS[name]
    kw = dict(c["kw"])
    kw.update(overrides)
    return c["fn"](**kw)
