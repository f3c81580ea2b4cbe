"""FP32 correction products in the FP64 iterations of the FP32-refined solve (an addition with no counterpart in
the reference): after the FP32 part, APGD keeps FP64 iterates, law and reductions but forms its products as
W x_ref + W32 (v - x_ref), the correction rounded to FP32 and multiplied by the FP32 copy of W, with x_ref and
W x_ref refreshed in FP64; a plain FP64 solve then checks the tolerance with the exact error function.

The results are not the reference's iterates (the products are rounded differently). The oracle restates the
form (ProjectedGradient::hyRefresh), and without an FP32 part the GPU iterations equal it bit for bit; beyond
that the tests check what the form promises: the returned residual is the oracle's FP64 error function at the
returned iterate, below the tolerance; the solve repeats bit for bit; a stalled correction part hands over to
the plain FP64 iterations; the batched forms stop each problem where its own solve stops; the forms it does
not cover refuse it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("fp32_iters", [400, 0])  # with and without the FP32 part
@pytest.mark.parametrize("static", [True, False])
def test_correction_products_reach_the_fp64_tolerance(bg, oracle, c1, fp32_iters, static):
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-10)
    pg.setMaxIters(fp32_iters)
    pg.setMixedPrecision(True, 4000)
    pg.setFp32CorrectionProducts(50)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=static)
    st = D.solve_stats()
    assert res == O.eval(r, coulomb=not static) and res < 1e-10
    assert st["fp32_product_iterations"] > 0 and st["refine_iterations"] >= st["fp32_product_iterations"]
    assert st["kernel_launches"] == 3
    r2 = np.zeros(3 * d.n)
    assert D.solveWith(pg, r2, staticProblem=static) == res and np.array_equal(r2, r)


@pytest.mark.parametrize("refresh, tol, budget", [(7, 1e-10, 3000), (50, 1e-10, 3000), (1000, 1e-14, 30000)])
@pytest.mark.parametrize("static", [True, False])
def test_correction_products_bitwise_against_the_oracle(bg, oracle, c1, refresh, tol, budget, static):
    """Without an FP32 part (max_iters = 0, r = 0) the correction iterations equal the oracle's restatement of
    them bit for bit (iteration count, refreshes, stall rule), and so does the plain FP64 check that follows from
    their best iterate (iterate, residual, iteration count)."""
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setTol(tol)
    pg.setMaxIters(0)
    pg.setMixedPrecision(True, budget)
    pg.setFp32CorrectionProducts(refresh)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=static)
    st = D.solve_stats()
    ith = st["fp32_product_iterations"]
    _, r_h, it_h = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=not static, tol=tol, max_iters=budget,
                              hy_refresh=refresh)
    assert ith == it_h
    res_c, r_c, it_c = O.solve_pg(r_h, variant=3, coulomb=not static, tol=tol, max_iters=max(1, budget - it_h))
    assert st["refine_iterations"] - ith == it_c
    assert res == res_c and np.array_equal(r, r_c)


@pytest.mark.parametrize("static", [True, False])
def test_fp32_refined_pipeline_bitwise_against_the_oracle(bg, oracle, c1, static):
    """The whole FP32-refined solve with correction products (FP32 part with its stall test, correction
    iterations, plain FP64 check) against the oracle's restatements of the three parts, bit for bit."""
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    tol, budget = 1e-10, 3000
    pg = bg.ProjectedGradient()
    pg.setTol(tol)
    pg.setMaxIters(2000)
    pg.setMixedPrecision(True, budget)
    pg.setFp32CorrectionProducts(20)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=static)
    st = D.solve_stats()
    _, r32, k = O.solve_pg_fp32(np.zeros(3 * d.n), coulomb=not static, tol=tol, max_iters=2000, stall_iters=4)
    assert k == st["iterations"] - st["refine_iterations"]
    _, r_h, it_h = O.solve_pg(r32, variant=3, coulomb=not static, tol=tol, max_iters=budget, hy_refresh=20)
    assert it_h == st["fp32_product_iterations"]
    res_c, r_c, it_c = O.solve_pg(r_h, variant=3, coulomb=not static, tol=tol, max_iters=max(1, budget - it_h))
    assert st["refine_iterations"] - it_h == it_c
    assert res == res_c and np.array_equal(r, r_c)


def test_stalled_corrections_hand_over_to_fp64(bg, oracle, c1):
    """A refresh interval too long for the tolerance: the correction part stops once its best residual has not
    improved by 1 % in 10 intervals, and the plain FP64 iterations go on from its best iterate."""
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-14)
    pg.setMaxIters(200)
    pg.setMixedPrecision(True, 30000)
    pg.setFp32CorrectionProducts(1000)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=True)
    st = D.solve_stats()
    assert 0 < st["fp32_product_iterations"] < 30000
    assert st["refine_iterations"] > st["fp32_product_iterations"]  # plain FP64 iterations followed
    assert res == O.eval(r, coulomb=False)


def test_full_size_correction_products(bg, oracle):
    """200 000 contacts to 1e-6: the FP64 error function of the returned iterate meets the tolerance."""
    from bogus_gpu import generator

    d = generator.make("c2")
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    rp, cl, vl = D.W_lower()
    O = oracle.DualProblem(rp, cl, vl.reshape(-1), d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-6)
    pg.setMaxIters(20000)
    pg.setMixedPrecision(True, 20000)
    pg.setFp32CorrectionProducts(50)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=True)
    st = D.solve_stats()
    assert res < 1e-6 and res == O.eval(r, coulomb=False)
    assert st["fp32_product_iterations"] > 0


def test_correction_products_refused_where_not_built(bg, c1):
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    for setup in (lambda pg: None,                                                  # no FP32-refined solve
                  lambda pg: (pg.setMixedPrecision(True, 50), pg.setDefaultVariant(4)),  # SPG
                  lambda pg: (pg.setMixedPrecision(True, 50), pg.setMomentumByLinearity(True))):
        pg = bg.ProjectedGradient()
        setup(pg)
        pg.setFp32CorrectionProducts(50)
        with pytest.raises(bg.BogusGpuError):
            D.solveWith(pg, np.zeros(3 * d.n))


@pytest.mark.parametrize("sizes", [(16, 16, 300), (5, 1500, 3000)])  # one CTA per problem; teams of CTAs
def test_batched_correction_products_match_single_problem_solves(bg, sizes):
    """The batched forms (plain FP32 copy of W, one CTA or a team per problem) stop, refresh and round each
    problem's correction products as its single-problem solve does (interleaved copy): bit for bit."""
    from bogus_gpu import generator

    nproblems, nmin, nmax = sizes
    d, cptr = generator.batch(nproblems=nproblems, nmin=nmin, nmax=nmax, seed=23)
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-9)
    pg.setMaxIters(100)
    pg.setMixedPrecision(True, 1500)
    pg.setFp32CorrectionProducts(20)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r, staticProblem=True)
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    single = bg.DualFrictionProblem()
    for p in range(len(cptr) - 1):
        c0, c1_ = cptr[p], cptr[p + 1]
        single.set(rp[c0:c1_ + 1] - rp[c0], cl[rp[c0]:rp[c1_]] - c0, vl[rp[c0]:rp[c1_]].reshape(-1), d.b[c0:c1_],
                   d.mu[c0:c1_])
        rs = np.zeros(3 * (c1_ - c0))
        res_s = single.solveWith(pg, rs)
        st = single.solve_stats()
        assert res[p] == res_s, p
        assert np.array_equal(r[3 * c0:3 * c1_], rs), p
        assert st["fp32_product_iterations"] > 0, p
