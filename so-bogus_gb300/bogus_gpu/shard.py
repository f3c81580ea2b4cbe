"""Sharding of batches of independent friction problems over ranks (one process per GPU).

A single friction problem does not shard: every APGD phase needs the whole iterate. A batch of independent
problems does: each rank solves a subset, with no collective on the data path. The subsets balance the work
by a greedy bin-pack on the problems' W blocks (each pass over W dominates a solve's cost): problems are taken
by decreasing block count and each goes to the rank with the least work so far (ties: the lowest rank). Every
rank computes the same partition from the same inputs, so no partition is exchanged; only the per-problem
results (residual, iterations, and where wanted r) are gathered at the end.
"""
from __future__ import annotations

import numpy as np

from .generator import PrimalData


def w_blocks_per_problem(data: PrimalData, contact_ptr) -> np.ndarray:
    """Stored blocks of the both-triangle W = H M^-1 H^T of each problem of a batch, from its contacts' bodies:
    block (i, j) exists when contacts i and j share a body, so the count is sum_k c_k^2 over bodies (c_k contacts
    on body k) minus sum over body pairs of m_ab^2 (m_ab contacts joining a and b, counted once per shared body)."""
    cptr = np.asarray(contact_ptr, np.int64)
    nprob = cptr.size - 1
    prob_of_contact = np.repeat(np.arange(nprob), np.diff(cptr))
    a = data.objA.astype(np.int64)
    b = data.objB.astype(np.int64)
    has_b = (b >= 0) & (b != a)
    bodies = np.concatenate([a, b[has_b]])
    probs = np.concatenate([prob_of_contact, prob_of_contact[has_b]])
    per_body = np.bincount(bodies, minlength=data.nbodies).astype(np.int64)
    body_prob = np.full(data.nbodies, -1, np.int64)
    body_prob[bodies] = probs
    used = per_body > 0
    out = np.bincount(body_prob[used], weights=(per_body[used] ** 2).astype(np.float64), minlength=nprob)
    if has_b.any():
        lo = np.minimum(a[has_b], b[has_b])
        hi = np.maximum(a[has_b], b[has_b])
        key = lo * (data.nbodies + 1) + hi
        uniq, inv, cnt = np.unique(key, return_inverse=True, return_counts=True)
        first = np.zeros(uniq.size, np.int64)
        first[inv] = prob_of_contact[has_b]
        out -= np.bincount(first, weights=(cnt.astype(np.float64) ** 2), minlength=nprob)
    return np.rint(out).astype(np.int64)


def partition(costs, nparts: int) -> list[np.ndarray]:
    """Greedy longest-processing-time bin-pack: problems by decreasing cost (ties: lower index first), each to the
    part with the least total cost so far (ties: the lowest part). Returns the problem indices of each part,
    in increasing order."""
    costs = np.asarray(costs, np.float64)
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    order = np.lexsort((np.arange(costs.size), -costs))
    load = np.zeros(nparts)
    parts: list[list[int]] = [[] for _ in range(nparts)]
    for p in order:
        k = int(np.argmin(load))
        parts[k].append(int(p))
        load[k] += costs[p]
    return [np.array(sorted(q), np.int64) for q in parts]


def subset(data: PrimalData, contact_ptr, problems) -> tuple[PrimalData, np.ndarray]:
    """The sub-batch made of `problems` (indices into the batch, kept in that order): contacts, bodies renumbered
    from 0, and its own contact_ptr."""
    cptr = np.asarray(contact_ptr, np.int64)
    problems = np.asarray(problems, np.int64)
    sel = np.concatenate([np.arange(cptr[p], cptr[p + 1]) for p in problems]) if problems.size else np.zeros(0, np.int64)
    a = data.objA[sel].astype(np.int64)
    b = data.objB[sel].astype(np.int64)
    used = np.unique(np.concatenate([a, b[b >= 0]])) if sel.size else np.zeros(0, np.int64)
    remap = np.full(data.nbodies, -1, np.int64)
    remap[used] = np.arange(used.size)
    sizes = np.diff(cptr)[problems]
    sub = PrimalData(minv=data.minv[used], objA=remap[a].astype(np.int32),
                     objB=np.where(b >= 0, remap[np.maximum(b, 0)], -1).astype(np.int32), HA=data.HA[sel],
                     HB=data.HB[sel], b=data.b[sel], mu=data.mu[sel], seed=data.seed, kind=data.kind + "_subset")
    return sub, np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)


def gather_results(local_problems, local_values: np.ndarray, nproblems: int, world: int) -> np.ndarray | None:
    """Gathers per-problem rows (local_values[k] belongs to problem local_problems[k]) from every rank into one
    array ordered by problem index, returned on rank 0 (None elsewhere). Uses torch.distributed (any backend);
    with world == 1 it only reorders."""
    local_problems = np.asarray(local_problems, np.int64)
    local_values = np.asarray(local_values, np.float64).reshape(local_problems.size, -1)
    width = local_values.shape[1]
    if world <= 1:
        out = np.zeros((nproblems, width))
        out[local_problems] = local_values
        return out
    import torch.distributed as dist

    rows = [None] * world
    dist.all_gather_object(rows, (local_problems.tolist(), local_values.tolist()))
    if dist.get_rank() != 0:
        return None
    out = np.full((nproblems, width), np.nan)
    for probs, vals in rows:
        if probs:
            out[np.asarray(probs, np.int64)] = np.asarray(vals, np.float64).reshape(len(probs), width)
    return out
