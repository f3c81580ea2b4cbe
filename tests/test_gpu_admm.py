"""GPU primal ADMM (PrimalFrictionProblem::solveWith(ADMM&, lambda, v, r)) against the CPU oracle.

The kernel follows the oracle's evaluation order, so v, r, the residual, the iteration count and the
callback trace are bit-identical (exact equality). The oracle itself is pinned on the reference's ADMM test
(tests/ADMM.cpp:16-60) in test_oracle_golden.py.
"""
import numpy as np
import pytest

from test_oracle_golden import _small_primal, admm_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


def _run_both(bg, oracle, data, lam, prox, v0, r0, f, accelerated=True, inf_norm=False, tol=1e-10,
              max_iters=300, step=1e-2):
    minv, objA, objB, HA, HB, w, mu = data
    P = bg.PrimalFrictionProblem(minv, objA, objB, HA, HB, w, mu, f=f)
    admm = bg.ADMM()
    admm.setTol(tol)
    admm.setMaxIters(max_iters)
    admm.setStepSize(step)
    admm.setDefaultVariant(bg.ADMM_ACCELERATED if accelerated else bg.ADMM_STANDARD)
    admm.useInfinityNorm(inf_norm)
    trace = []
    admm.callback().connect(lambda it, res: trace.append((it, res)))
    v, r = v0.copy(), r0.copy()
    res = P.solveWith(admm, lam, v, r, prox=prox)
    O = oracle.PrimalProblem(minv, objA, objB, HA, HB)
    tr = oracle.Trace()
    fo = np.zeros(v0.size) if f is None else f
    po = minv if prox is None else prox
    res_o, v_o, r_o, it_o = O.solve_admm(po, lam, mu, fo, w, v0, r0, tol=tol, max_iters=max_iters, step=step,
                                         accelerated=accelerated, inf_norm=inf_norm, trace=tr)
    return (res, v, r, P.last_iterations, trace), (res_o, v_o, r_o, it_o, tr.items)


def _assert_same(g, o):
    assert g[0] == o[0]
    assert np.array_equal(g[1], o[1])
    assert np.array_equal(g[2], o[2])
    assert g[3] == o[3]
    assert g[4] == o[4]


@pytest.mark.parametrize("lam", [0.0, 0.1])
def test_small_friction_admm_bitwise(bg, oracle, golden, lam):
    s, _, minv, Hd = _small_primal(oracle, golden)
    prox, v, r, f = admm_inputs(s, minv, Hd, lam)
    data = (minv, np.array(s["objA"]), np.array(s["objB"]), np.array(s["HA"]), np.array(s["HB"]),
            np.array(s["w"]), np.array(s["mu"]))
    g, o = _run_both(bg, oracle, data, lam, prox, v, r, f, tol=1e-8, max_iters=1000)
    _assert_same(g, o)
    assert g[0] < 1e-8


@pytest.fixture(scope="module")
def c1_primal():
    from bogus_gpu import generator

    d = generator.make("c1")
    rng = np.random.default_rng(11)
    f = rng.standard_normal(d.nbodies * 6) * 0.1
    return d, f


@pytest.mark.parametrize("accelerated", [True, False])
@pytest.mark.parametrize("inf_norm", [False, True])
def test_admm_bitwise_random_pairs(bg, oracle, c1_primal, accelerated, inf_norm):
    d, f = c1_primal
    data = (d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    rng = np.random.default_rng(3)
    v0 = rng.standard_normal(d.nbodies * 6) * 0.01
    r0 = np.abs(rng.standard_normal(3 * d.n)) * 0.01
    g, o = _run_both(bg, oracle, data, 0.0, None, v0, r0, f, accelerated=accelerated, inf_norm=inf_norm)
    _assert_same(g, o)


def test_admm_bitwise_lambda_with_default_prox(bg, oracle, c1_primal):
    """lambda > 0 with the M^-1 operator PrimalFrictionProblem::solveWith passes whatever lambda, f = 0 (NULL
    on the GPU). That operator does not match lambda and the iteration diverges, in the reference as here:
    the first iterations, still finite, are compared."""
    d, _ = c1_primal
    data = (d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    g, o = _run_both(bg, oracle, data, 0.5, None, np.zeros(d.nbodies * 6), np.zeros(3 * d.n), None, max_iters=4)
    assert np.isfinite(g[0])
    _assert_same(g, o)


def test_admm_bitwise_lambda_with_matching_prox(bg, oracle, c1_primal):
    """lambda = 0.1 with the operator (M + I / lambda)^-1 of the reference's ADMM test, random f."""
    d, f = c1_primal
    data = (d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    prox = np.linalg.inv(np.linalg.inv(d.minv) + np.eye(6)[None] / 0.1)
    g, o = _run_both(bg, oracle, data, 0.1, prox, np.zeros(d.nbodies * 6), np.zeros(3 * d.n), f, max_iters=200)
    assert np.isfinite(g[0])
    _assert_same(g, o)


def test_admm_zero_iterations_and_bad_inputs(bg, c1_primal):
    d, _ = c1_primal
    P = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    admm = bg.ADMM()
    admm.setMaxIters(0)
    v, r = np.zeros(d.nbodies * 6), np.zeros(3 * d.n)
    assert P.solveWith(admm, 0.0, v, r) == -1.0  # the reference returns its initial -1
    with pytest.raises(bg.BogusGpuError):
        P.solveWith(bg.ADMM(), -1.0, v, r)
    bad = bg.ADMM()
    bad.setStepSize(0.0)
    with pytest.raises(bg.BogusGpuError):
        P.solveWith(bad, 0.0, v, r)
    with pytest.raises(ValueError):
        P.solveWith(bg.ADMM(), 0.0, v[:-1].copy(), r)


def test_full_size_admm_first_iterations(bg, oracle):
    """200 000 contacts / 50 000 bodies: 25 iterations bit-identical to the oracle."""
    from bogus_gpu import generator

    d = generator.make("c2")
    data = (d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    g, o = _run_both(bg, oracle, data, 0.0, None, np.zeros(d.nbodies * 6), np.zeros(3 * d.n), None, max_iters=25)
    _assert_same(g, o)
