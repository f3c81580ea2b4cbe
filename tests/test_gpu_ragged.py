"""Ragged sizes against the oracle, bit for bit: problems of 1, 2, 31, 32, 33 and 65 contacts (a partial chunk, a
full one, one past it, two and one past), on few bodies so that W rows are long (up to every contact coupled:
segments of many blocks per lane) and on many bodies (short rows). Every solver family that runs over 32-contact
chunks: the product, the error function, APGD / SPG / Standard / Conjugated (APGD also with the momentum
product by linearity), Gauss-Seidel (natural and colored), and primal ADMM.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 31, 32, 33, 65]


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


def _problem(oracle, n, dense):
    from bogus_gpu import generator

    nbodies = 3 if dense else max(2, 2 * n)
    d = generator.random_pairs(nbodies=nbodies, ncontacts=n, seed=1000 + 7 * n + (1 if dense else 0))
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    rp, cl, vl = P.assemble()
    return d, rp, cl, vl


@pytest.mark.parametrize("dense", [True, False])
@pytest.mark.parametrize("n", SIZES)
def test_ragged_product_eval_pg(bg, oracle, n, dense):
    d, rp, cl, vl = _problem(oracle, n, dense)
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    x = np.random.default_rng(n).standard_normal(3 * n)
    assert np.array_equal(D.multiply(x), O.spmv(x))
    for static in (True, False):
        pg = bg.ProjectedGradient()
        assert D.evalWith(pg, x, staticProblem=static) == O.eval(x, coulomb=not static)
    for variant, lin in ((3, False), (3, True), (4, False), (0, False), (2, False)):
        pg = bg.ProjectedGradient()
        pg.setDefaultVariant(variant)
        pg.setTol(1e-10)
        pg.setMaxIters(200)
        pg.setMomentumByLinearity(lin)
        r = np.zeros(3 * n)
        res = D.solveWith(pg, r, staticProblem=False)
        res_o, r_o, it_o = O.solve_pg(np.zeros(3 * n), variant=variant, coulomb=True, tol=1e-10, max_iters=200,
                                      lin_momentum=lin)
        assert res == res_o and D.last_iterations == it_o and np.array_equal(r, r_o), (variant, lin)


@pytest.mark.parametrize("coloring", [False, True])
@pytest.mark.parametrize("dense", [True, False])
@pytest.mark.parametrize("n", SIZES)
def test_ragged_gauss_seidel(bg, oracle, n, dense, coloring):
    d, rp, cl, vl = _problem(oracle, n, dense)
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    gs = bg.GaussSeidel()
    gs.coloring().update(coloring)
    gs.setTol(1e-10)
    gs.setMaxIters(60)
    r = np.zeros(3 * n)
    res = D.solveWith(gs, r)
    res_o, r_o, it_o = O.solve_gs(np.zeros(3 * n), coulomb=True, tol=1e-10, max_iters=60, coloring=coloring)
    assert res == res_o and D.last_iterations == it_o and np.array_equal(r, r_o)


@pytest.mark.parametrize("dense", [True, False])
@pytest.mark.parametrize("n", SIZES)
def test_ragged_admm(bg, oracle, n, dense):
    d, _, _, _ = _problem(oracle, n, dense)
    P = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b, d.mu)
    admm = bg.ADMM()
    admm.setTol(1e-12)
    admm.setMaxIters(80)
    v, r = np.zeros(6 * d.nbodies), np.zeros(3 * n)
    res = P.solveWith(admm, 0.0, v, r)
    O = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    res_o, v_o, r_o, it_o = O.solve_admm(d.minv, 0.0, d.mu, np.zeros(6 * d.nbodies), d.b, np.zeros(6 * d.nbodies),
                                         np.zeros(3 * n), tol=1e-12, max_iters=80)
    assert res == res_o and P.last_iterations == it_o
    assert np.array_equal(v, v_o) and np.array_equal(r, r_o)
