"""GPU matrix-free Gauss-Seidel (PrimalFrictionProblem::solveWith(ProductGaussSeidel&, r, staticProblem)) against
the oracle's restatement: iterates, error, iteration count and callback trace bit-identical. The oracle itself
reaches the reference's SmallFrictionPb solution (test_oracle_golden.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


def run_pair(bg, oracle, minv, objA, objB, HA, HB, w, mu, f, r0, static=False, strategy=3, tol=1e-8,
             max_iters=100, auto_reg=0.0, try_zero=True, inf_norm=False, eval_every=25):
    P = bg.PrimalFrictionProblem(minv, objA, objB, HA, HB, w, mu, f=f)
    gs = bg.ProductGaussSeidel()
    gs.setTol(tol)
    gs.setMaxIters(max_iters)
    gs.setAutoRegularization(auto_reg)
    gs.doTryZeroAsWell(try_zero)
    gs.useInfinityNorm(inf_norm)
    gs.setLocalStrategy(strategy)
    gs.setEvalEvery(eval_every)
    trace = []
    gs.callback().connect(lambda it, res: trace.append((it, res)))
    r = r0.copy()
    res = P.solveWith(gs, r, staticProblem=static)
    O = oracle.PrimalProblem(minv, objA, objB, HA, HB)
    tr = oracle.Trace()
    fo = np.zeros(minv.shape[0] * minv.shape[1]) if f is None else f
    res_o, r_o, it_o = O.solve_product_gs(fo, w, mu, r0, coulomb=not static, strategy=strategy, tol=tol,
                                          max_iters=max_iters, eval_every=eval_every, auto_reg=auto_reg,
                                          try_zero=try_zero, inf_norm=inf_norm, trace=tr)
    assert res == res_o
    assert P.last_iterations == it_o
    assert np.array_equal(r, r_o)
    assert trace == tr.items
    return res


def test_small_friction_bitwise(bg, oracle, golden):
    s = golden["small_friction_pb"]
    res = run_pair(bg, oracle, np.array(s["minv"]), np.array(s["objA"]), np.array(s["objB"]), np.array(s["HA"]),
                   np.array(s["HB"]), np.array(s["w"]), np.array(s["mu"]), np.array(s["f_padded"]), np.ones(6),
                   tol=1e-8, max_iters=250)
    assert res < 1e-8


@pytest.mark.parametrize("static, strategy, auto_reg, inf_norm", [
    (False, 3, 0.0, False), (True, 3, 0.0, False), (False, 0, 1e-3, False), (False, 2, 0.0, True)])
def test_random_pairs_bitwise(bg, oracle, static, strategy, auto_reg, inf_norm):
    from bogus_gpu import generator

    d = generator.make("c1")
    f = np.random.default_rng(8).standard_normal(6 * d.nbodies) * 0.1
    r0 = np.abs(np.random.default_rng(9).standard_normal(3 * d.n)) * 0.01
    run_pair(bg, oracle, d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu, f, r0, static=static,
             strategy=strategy, auto_reg=auto_reg, inf_norm=inf_norm, max_iters=60, eval_every=10)


def test_full_size_first_sweeps_bitwise(bg, oracle):
    """200 000 contacts / 50 000 bodies: 25 matrix-free sweeps bit-identical to the oracle."""
    from bogus_gpu import generator

    d = generator.make("c2")
    run_pair(bg, oracle, d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu, None, np.zeros(3 * d.n),
             max_iters=25, tol=1e-12)
