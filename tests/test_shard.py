"""Sharding of independent problems over ranks (bogus_gpu.shard), on the CPU: the W-block count of each problem
(the bin-pack's cost) against the oracle's assembly, the greedy bin-pack's coverage and balance, the sub-batch
extraction, and on two gloo ranks the whole path: every rank takes its share of a batch, solves it (with the
oracle, no GPU), and rank 0 gathers residuals, iteration counts and r in problem order; the gathered results
equal a single process solving every problem."""
import json
import os
import socket
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _batch(nproblems=12, seed=7):
    from bogus_gpu import generator

    return generator.batch(nproblems, nmin=16, nmax=120, seed=seed)


def test_w_blocks_per_problem_matches_the_assembly(oracle):
    from bogus_gpu import shard

    d, cptr = _batch()
    est = shard.w_blocks_per_problem(d, cptr)
    for p in range(len(cptr) - 1):
        sub, _ = shard.subset(d, cptr, [p])
        rp, cl, vl = oracle.PrimalProblem(sub.minv, sub.objA, sub.objB, sub.HA, sub.HB).assemble()
        assert est[p] == 2 * len(cl) - sub.n  # both triangles from the lower one


def test_partition_covers_every_problem_once_and_balances():
    from bogus_gpu import shard

    rng = np.random.default_rng(3)
    costs = rng.integers(1, 1000, 257)
    for nparts in (1, 2, 3, 8):
        parts = shard.partition(costs, nparts)
        allp = np.sort(np.concatenate(parts))
        assert np.array_equal(allp, np.arange(costs.size))
        loads = np.array([costs[q].sum() for q in parts])
        # the greedy longest-first bound: no part exceeds the mean by more than the largest cost
        assert loads.max() <= costs.sum() / nparts + costs.max()
        again = shard.partition(costs, nparts)  # deterministic: every rank computes the same split
        assert all(np.array_equal(a, b) for a, b in zip(parts, again))


def test_subset_keeps_the_problems_and_renumbers_bodies():
    from bogus_gpu import shard

    d, cptr = _batch()
    probs = [3, 0, 11]
    sub, sc = shard.subset(d, cptr, probs)
    assert np.array_equal(np.diff(sc), np.diff(cptr)[probs])
    for k, p in enumerate(probs):
        c0, c1 = cptr[p], cptr[p + 1]
        assert np.array_equal(sub.b[sc[k]:sc[k + 1]], d.b[c0:c1])
        assert np.array_equal(sub.HA[sc[k]:sc[k + 1]], d.HA[c0:c1])
        # the same bodies (through the renumbering): their inverse masses agree
        assert np.array_equal(sub.minv[sub.objA[sc[k]:sc[k + 1]]], d.minv[d.objA[c0:c1]])
    assert sub.objA.max() < sub.nbodies and sub.objB.max() < sub.nbodies


def _solve_problems(oracle, d, cptr, probs):
    """(residual, iterations, r) of each problem, APGD with the oracle (one thread: the ranks share the cores)."""
    from bogus_gpu import shard

    threads = oracle.num_threads()
    oracle.set_num_threads(1)
    out = []
    try:
        for p in probs:
            sub, _ = shard.subset(d, cptr, [p])
            P = oracle.PrimalProblem(sub.minv, sub.objA, sub.objB, sub.HA, sub.HB)
            rp, cl, vl = P.assemble()
            O = oracle.DualProblem(rp, cl, vl, sub.b, sub.mu)
            res, r, it = O.solve_pg(np.zeros(3 * sub.n), variant=3, coulomb=False, tol=1e-6, max_iters=100)
            out.append((res, it, r))
    finally:
        oracle.set_num_threads(threads)
    return out


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, outdir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    for p in (REPO, os.path.join(REPO, "so-bogus_gb300"), os.path.join(REPO, "oracle")):
        sys.path.insert(0, p)
    import pyoracle

    from bogus_gpu import shard

    pyoracle.build()
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        d, cptr = _batch()
        parts = shard.partition(shard.w_blocks_per_problem(d, cptr), world)
        mine = parts[rank]
        local = _solve_problems(pyoracle, d, cptr, mine)
        sizes = np.diff(cptr)
        width = 2 + 3 * int(sizes.max())
        rows = np.zeros((len(mine), width))
        for k, (res, it, r) in enumerate(local):
            rows[k, 0], rows[k, 1] = res, it
            rows[k, 2:2 + r.size] = r
        got = shard.gather_results(mine, rows, len(cptr) - 1, world)
        with open(os.path.join(outdir, f"rank{rank}.json"), "w") as fh:
            json.dump({"mine": mine.tolist(), "gathered": None if got is None else got.tolist()}, fh)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_solve_and_gather(tmp_path, oracle):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    out = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    assert out[1]["gathered"] is None
    mine = [set(o["mine"]) for o in out]
    assert mine[0] and mine[1] and not (mine[0] & mine[1])
    d, cptr = _batch()
    assert mine[0] | mine[1] == set(range(len(cptr) - 1))
    got = np.array(out[0]["gathered"])
    ref = _solve_problems(oracle, d, cptr, range(len(cptr) - 1))
    for p, (res, it, r) in enumerate(ref):
        assert got[p, 0] == res and got[p, 1] == it
        assert np.array_equal(got[p, 2:2 + r.size], r)
