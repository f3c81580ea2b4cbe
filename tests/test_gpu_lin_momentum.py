"""APGD with the momentum product formed by linearity (an option with no counterpart in the reference):
W x = W xs + beta (W xs - W prev) in place of the product of ProjectedGradient.impl.hpp:141.

The oracle restates the same variant with the same operations, so the GPU solve is checked bit for bit against
it, as the reference's arithmetic is in test_gpu_parity.py; the single-problem (FP64 and FP32-refined) and the
batched forms are covered, and at full size the option's deviation from the reference's iterates is bounded
through the residual, not the iterate (W is singular there).
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


@pytest.mark.parametrize("static", [True, False])
@pytest.mark.parametrize("variant", [3, 1, 4])  # APGD (uses it), Descent and SPG (no momentum product: no effect)
def test_lin_momentum_bitwise(bg, oracle, c1, static, variant):
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setTol(1e-8)
    pg.setMaxIters(400)
    pg.setMomentumByLinearity(True)
    trace = []
    pg.callback().connect(lambda it, res: trace.append((it, res)))
    r0 = np.random.default_rng(2).standard_normal(3 * d.n) * 0.1
    r = r0.copy()
    res = D.solveWith(pg, r, staticProblem=static)
    tr = oracle.Trace()
    res_o, r_o, it_o = O.solve_pg(r0, variant=variant, coulomb=not static, tol=1e-8, max_iters=400, trace=tr,
                                  lin_momentum=True)
    assert res == res_o and D.last_iterations == it_o
    assert np.array_equal(r, r_o)
    assert trace == tr.items
    if variant != 3:  # nothing to form by linearity: the reference's iterates
        res_ref, r_ref, _ = O.solve_pg(r0, variant=variant, coulomb=not static, tol=1e-8, max_iters=400)
        assert res_ref == res_o and np.array_equal(r_ref, r_o)


def test_lin_momentum_saves_products(bg, c1):
    """Same problem, same budget: with the option the solve makes fewer passes over W per iteration."""
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    passes = {}
    for lin in (False, True):
        pg = bg.ProjectedGradient()
        pg.setTol(1e-30)
        pg.setMaxIters(200)
        pg.setMomentumByLinearity(lin)
        D.solveWith(pg, np.zeros(3 * d.n), staticProblem=True)
        st = D.solve_stats()
        passes[lin] = st["w_passes"] / st["iterations"]
    assert passes[True] < passes[False] - 0.5


def test_lin_momentum_full_size(bg, oracle):
    """200 000 contacts, 300 iterations: bit-identical to the oracle's variant; against the reference's
    iterates the residual stays within a factor 2 (two rounding forms of one method)."""
    from bogus_gpu import generator

    d = generator.make("c2")
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    O = oracle.DualProblem(*P.assemble(), d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setMaxIters(300)
    pg.setMomentumByLinearity(True)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=True)
    res_o, r_o, it_o = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=False, max_iters=300, lin_momentum=True)
    assert res == res_o and D.last_iterations == it_o and np.array_equal(r, r_o)
    res_ref, _, _ = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=False, max_iters=300)
    assert 0.5 * res_ref < res < 2.0 * res_ref


def test_lin_momentum_mixed_precision(bg, oracle, c1):
    """FP32-refined with the option (applied to the FP64 iterations: the FP32 part is the plain FP32-refined
    one): the returned residual meets the tolerance and equals the oracle's error function at the returned
    iterate up to rounding (it is evaluated with the product formed by linearity), the FP32 part makes as many
    passes over W as without the option, and the solve repeats bit for bit."""
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-10)
    pg.setMaxIters(400)
    pg.setMixedPrecision(True, 200)
    pg.setMomentumByLinearity(True)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=True)
    assert res < 1e-10 and abs(res - O.eval(r, coulomb=False)) <= 1e-9 * res
    st = D.solve_stats()
    r2 = np.zeros(3 * d.n)
    assert D.solveWith(pg, r2, staticProblem=True) == res and np.array_equal(r, r2)
    pg.setMomentumByLinearity(False)
    D.solveWith(pg, np.zeros(3 * d.n), staticProblem=True)
    plain = D.solve_stats()
    assert plain["fp32_device_ms"] > 0 and st["iterations"] - st["refine_iterations"] == \
        plain["iterations"] - plain["refine_iterations"]


def test_lin_momentum_batched(bg, oracle):
    """One launch over 24 problems: each equals the oracle's variant on that problem."""
    from bogus_gpu import generator

    d, cptr = generator.batch(nproblems=24, nmin=16, nmax=400, seed=7)
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-8)
    pg.setMaxIters(300)
    pg.setMomentumByLinearity(True)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r, staticProblem=False)
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    for p in range(len(cptr) - 1):
        c0, c1_ = cptr[p], cptr[p + 1]
        O = oracle.DualProblem(rp[c0:c1_ + 1] - rp[c0], cl[rp[c0]:rp[c1_]] - c0, vl[rp[c0]:rp[c1_]].reshape(-1),
                               d.b[c0:c1_], d.mu[c0:c1_])
        res_o, r_o, it_o = O.solve_pg(np.zeros(3 * (c1_ - c0)), variant=3, coulomb=True, tol=1e-8, max_iters=300,
                                      lin_momentum=True)
        assert res[p] == res_o and its[p] == it_o, p
        assert np.array_equal(r[3 * c0:3 * c1_], r_o), p


@pytest.mark.parametrize("mixed", [False, True])
def test_lin_momentum_team_batch(bg, oracle, mixed):
    """Few large problems (several CTAs per problem, the team schedule): each problem equals its own
    single-problem solve with the option and, in FP64, the oracle's variant."""
    from bogus_gpu import generator

    d, cptr = generator.batch(nproblems=5, nmin=1500, nmax=3000, seed=13)
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-8)
    pg.setMaxIters(150)
    pg.setMomentumByLinearity(True)
    if mixed:
        pg.setMixedPrecision(True, 40)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r, staticProblem=True)
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    single = bg.DualFrictionProblem()
    for p in range(len(cptr) - 1):
        c0, c1_ = cptr[p], cptr[p + 1]
        prp, pcl, pvl = rp[c0:c1_ + 1] - rp[c0], cl[rp[c0]:rp[c1_]] - c0, vl[rp[c0]:rp[c1_]].reshape(-1)
        single.set(prp, pcl, pvl, d.b[c0:c1_], d.mu[c0:c1_])
        rs = np.zeros(3 * (c1_ - c0))
        res_s = single.solveWith(pg, rs)
        assert res[p] == res_s and its[p] == single.last_iterations, p
        assert np.array_equal(r[3 * c0:3 * c1_], rs), p
        if not mixed:
            O = oracle.DualProblem(prp, pcl, pvl, d.b[c0:c1_], d.mu[c0:c1_])
            res_o, r_o, it_o = O.solve_pg(np.zeros(3 * (c1_ - c0)), variant=3, coulomb=False, tol=1e-8,
                                          max_iters=150, lin_momentum=True)
            assert res[p] == res_o and its[p] == it_o and np.array_equal(rs, r_o), p


def test_noalloc_rejects_lin_momentum(bg):
    """The allocation-free entry point has no room for the two extra product buffers: BAD_INPUT before anything
    runs (an empty problem, so no device pointer is needed)."""
    import ctypes as C

    L = bg.lib()
    pg = bg.ProjectedGradient()
    pg.setMomentumByLinearity(True)
    o = pg.options(True)
    st = L.bogus_gpu_solve_pg_noalloc(0, 0, 0, None, None, None, None, None, C.byref(o), None, None, None, None)
    assert st == 2 and b"momentum_by_linearity" in L.bogus_gpu_last_error()
