"""The stall test of the FP32-refined solves (an addition with no counterpart in the reference): the FP32 part
ends once FP32 rounding stops its progress, that is when its residual has repeated bit for bit, or its line
search has run out of trials, on fp32_stall_iters consecutive iterations. The FP64 iterations then start from
the best FP32 iterate.

Ending the FP32 part at the top of iteration k (residuals 0..k evaluated) keeps the same best iterate as a
fixed FP32 budget of k + 1 iterations, so the two solves must agree bit for bit; the batched forms (one CTA per
problem, and teams of CTAs for large problems) must stop each problem where its own single-problem solve stops.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BUDGET = 6000


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


@pytest.fixture(scope="module")
def c1(oracle):
    from bogus_gpu import generator

    d = generator.make("c1")
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    rp, cl, vl = P.assemble()
    return d, rp, cl, vl


def _fp32_iterations(st):
    return st["iterations"] - st["refine_iterations"]


@pytest.mark.parametrize("variant", [3, 1])  # APGD, Descent
@pytest.mark.parametrize("static", [True, False])
def test_fp32_refined_bitwise_against_the_oracle(bg, oracle, c1, variant, static):
    """The FP32 part against the oracle's restatement of it (float W, iterates and law; double reductions and
    step decisions; the stall test), then the FP64 part from its best iterate: iterates, residual and iteration
    counts bit for bit."""
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setTol(1e-10)
    pg.setMaxIters(3000)
    pg.setMixedPrecision(True, 400)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=static)
    st = D.solve_stats()
    _, r32, k = O.solve_pg_fp32(np.zeros(3 * d.n), apgd=variant == 3, coulomb=not static, tol=1e-10, max_iters=3000,
                                stall_iters=4)
    assert k == _fp32_iterations(st)
    res_o, r_o, it_o = O.solve_pg(r32, variant=variant, coulomb=not static, tol=1e-10, max_iters=400)
    assert it_o == st["refine_iterations"] and res == res_o and np.array_equal(r, r_o)


@pytest.mark.parametrize("static", [True, False])
def test_stall_ends_the_fp32_part_like_a_budget(bg, oracle, c1, static):
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-13)
    pg.setMaxIters(BUDGET)
    pg.setMixedPrecision(True, 300)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=static)
    st = D.solve_stats()
    k = _fp32_iterations(st)
    assert 0 < k < BUDGET, k  # the FP32 part cannot reach 1e-13: it stalls before its budget
    assert res == O.eval(r, coulomb=not static)
    # a fixed FP32 budget of k + 1 iterations keeps the same best FP32 iterate: the same solve bit for bit
    pg.setFp32StallIterations(0)
    pg.setMaxIters(k + 1)
    r2 = np.zeros(3 * d.n)
    res2 = D.solveWith(pg, r2, staticProblem=static)
    st2 = D.solve_stats()
    assert _fp32_iterations(st2) == k + 1
    assert res2 == res and np.array_equal(r2, r) and st2["refine_iterations"] == st["refine_iterations"]
    # with the test off the FP32 part runs its whole budget
    pg.setMaxIters(k + 200)
    D.solveWith(pg, np.zeros(3 * d.n), staticProblem=static)
    assert _fp32_iterations(D.solve_stats()) == k + 200
    # repeatable
    pg.setFp32StallIterations(4)
    pg.setMaxIters(BUDGET)
    r3 = np.zeros(3 * d.n)
    assert D.solveWith(pg, r3, staticProblem=static) == res and np.array_equal(r3, r)


@pytest.mark.parametrize("sizes", [(16, 16, 300), (5, 1500, 3000)])  # one CTA per problem; teams of CTAs
def test_batched_stall_matches_single_problem_solves(bg, sizes):
    from bogus_gpu import generator

    nproblems, nmin, nmax = sizes
    d, cptr = generator.batch(nproblems=nproblems, nmin=nmin, nmax=nmax, seed=21)
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-13)
    pg.setMaxIters(3000)
    pg.setMixedPrecision(True, 60)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r, staticProblem=True)
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    single = bg.DualFrictionProblem()
    stalled = 0
    for p in range(len(cptr) - 1):
        c0, c1_ = cptr[p], cptr[p + 1]
        single.set(rp[c0:c1_ + 1] - rp[c0], cl[rp[c0]:rp[c1_]] - c0, vl[rp[c0]:rp[c1_]].reshape(-1), d.b[c0:c1_],
                   d.mu[c0:c1_])
        rs = np.zeros(3 * (c1_ - c0))
        res_s = single.solveWith(pg, rs)
        assert res[p] == res_s and its[p] == single.last_iterations, p
        assert np.array_equal(r[3 * c0:3 * c1_], rs), p
        stalled += _fp32_iterations(single.solve_stats()) < 3000
    assert stalled > 0
