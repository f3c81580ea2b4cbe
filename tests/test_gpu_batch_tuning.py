"""Launch shapes of the batched solve, the tuner that picks one, and the graph-captured batched solve.

Every shape (one CTA per problem at 1..2 CTAs per SM, the kernel's occupancy; teams of 2..16 CTAs at 2 or 3 CTAs per SM) must give the
same residuals, iteration counts and iterates bit for bit, since each problem's reductions follow its fixed
32-contact chunk order; the tuner measures the candidates on the batch and keeps one; the captured CUDA graph
replays the solve with the same results as the plain call.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(oracle):
    import bogus_gpu
    from bogus_gpu import generator

    d, cptr = generator.batch(nproblems=40, nmin=16, nmax=1500, seed=21)
    D = bogus_gpu.DualFrictionProblem()
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(1e-8)
    pg.setMaxIters(120)
    r0 = np.random.default_rng(3).standard_normal(3 * d.n) * 0.01
    r = r0.copy()
    res, its = D.solveBatchWith(pg, r, staticProblem=False)
    return d, cptr, D, pg, r0, (res, its, r)


def _solve(D, pg, r0, **kw):
    r = r0.copy()
    res, its = D.solveBatchWith(pg, r, staticProblem=False, **kw)
    return res, its, r


def _same(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_every_launch_shape_gives_the_same_results(batch):
    d, cptr, D, pg, r0, ref = batch
    shapes = [(0, k, 1) for k in (1, 2)] + [(1, k, t) for t in (2, 4, 8, 16) for k in (2, 3)]
    try:
        for sh in shapes:
            D.setBatchShape(*sh)
            got = _solve(D, pg, r0)
            assert D.batchShape() == sh
            assert _same(got, ref), sh
    finally:
        D.setBatchShape(None)


def test_every_launch_shape_gives_the_same_fp32_refined_results(batch):
    d, cptr, D, _, r0, _ = batch
    import bogus_gpu

    pgm = bogus_gpu.ProjectedGradient()
    pgm.setTol(1e-8)
    pgm.setMaxIters(60)
    pgm.setMixedPrecision(True, 30)
    ref = _solve(D, pgm, r0)
    try:
        for sh in [(0, 1, 1), (0, 2, 1), (1, 2, 4), (1, 3, 16)]:
            D.setBatchShape(*sh)
            assert _same(_solve(D, pgm, r0), ref), sh
    finally:
        D.setBatchShape(None)


def test_tuner_measures_the_candidates_keeps_the_fastest_and_caches_it(batch):
    d, cptr, D, pg, r0, ref = batch
    D.setBatchTuning(True)
    try:
        got = _solve(D, pg, r0)
        assert _same(got, ref)  # tuning runs restore the starting iterate
        log = D.batchTuningLog()
        assert len(log) >= 5
        best = min(log, key=lambda e: e[1])[0]
        assert D.batchShape() == best
        got = _solve(D, pg, r0)  # no second tuning: the same log, the same shape
        assert D.batchTuningLog() == log and D.batchShape() == best
        assert _same(got, ref)
    finally:
        D.setBatchTuning(False)


def test_graph_capture_replays_bit_for_bit(batch):
    torch = pytest.importorskip("torch")
    import bogus_gpu

    d, cptr, D, pg, r0, ref = batch
    buf = torch.empty(3 * d.n, dtype=torch.float64, pin_memory=True)
    rp = buf.numpy()
    for k in range(3):  # the first call captures, the others replay
        rp[...] = r0
        res, its = D.solveBatchGraph(pg, rp, staticProblem=False)
        assert _same((res, its, rp), ref), k
    # another warm start in the same buffer: the replay reads it
    r1 = r0 * 0.5
    ref1 = _solve(D, pg, r1)
    rp[...] = r1
    res, its = D.solveBatchGraph(pg, rp, staticProblem=False)
    assert _same((res, its, rp), ref1)
    # the team schedule (a cooperative launch) captured as well
    try:
        D.setBatchShape(1, 2, 4)
        rp[...] = r0
        res, its = D.solveBatchGraph(pg, rp, staticProblem=False)
        assert _same((res, its, rp), ref)
    finally:
        D.setBatchShape(None)
    # pageable memory is refused
    with pytest.raises(bogus_gpu.BogusGpuError) as e:
        D.solveBatchGraph(pg, r0.copy(), staticProblem=False)
    assert e.value.status == bogus_gpu.BAD_INPUT
