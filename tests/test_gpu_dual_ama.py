"""GPU DualAMA (PrimalFrictionProblem::solveWith(DualAMAType&, v, r, staticProblem)) against the CPU oracle.

The kernel follows the oracle's evaluation order, so v, r, the residual, the iteration count and the callback
trace are bit-identical (exact equality). The oracle itself is pinned on the reference's DualAMA tests
(tests/ADMM.cpp:135-189) in test_oracle_golden.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


def _run_both(bg, oracle, data, mass, f, v0, r0, static=False, accelerated=True, ls=6, fp=1e-1, proj=1e-1,
              inf_norm=False, tol=1e-10, max_iters=300, body_dofs=None):
    minv, objA, objB, HA, HB, w, mu = data
    P = bg.PrimalFrictionProblem(minv, objA, objB, HA, HB, w, mu, f=f, M=mass, body_dofs=body_dofs)
    dama = bg.DualAMA()
    dama.setTol(tol)
    dama.setMaxIters(max_iters)
    dama.setFpStepSize(fp)
    dama.setProjStepSize(proj)
    dama.setLineSearchIterations(ls)
    dama.setDefaultVariant(bg.ADMM_ACCELERATED if accelerated else bg.ADMM_STANDARD)
    dama.useInfinityNorm(inf_norm)
    trace = []
    dama.callback().connect(lambda it, res: trace.append((it, res)))
    v, r = v0.copy(), r0.copy()
    res = P.solveWith(dama, v, r, staticProblem=static)
    O = oracle.PrimalProblem(minv, objA, objB, HA, HB)
    tr = oracle.Trace()
    fo = np.zeros(v0.size) if f is None else f
    res_o, v_o, r_o, it_o = O.solve_dual_ama(mass, mu, fo, w, v0, r0, static=static, tol=tol, max_iters=max_iters,
                                             fp_step=fp, proj_step=proj, ls_iters=ls, accelerated=accelerated,
                                             inf_norm=inf_norm, true_dofs=body_dofs, trace=tr)
    return (res, v, r, P.last_iterations, trace), (res_o, v_o, r_o, it_o, tr.items)


def _assert_same(g, o):
    assert g[0] == o[0]
    assert np.array_equal(g[1], o[1])
    assert np.array_equal(g[2], o[2])
    assert g[3] == o[3]
    assert g[4] == o[4]


@pytest.mark.parametrize("name, accelerated, ls, proj, coulomb", [
    ("Std-Kmu", False, 4, 1.0, False), ("Std-Cmu", False, 4, 1.0, True),
    ("Acc-Kmu", True, 0, 1e-1, False), ("Acc-Cmu", True, 0, 1e-2, True)])
def test_small_friction_dual_ama_bitwise(bg, oracle, golden, name, accelerated, ls, proj, coulomb):
    """The four DualAMA cases of tests/ADMM.cpp:135-189 on SmallFrictionPb (bodies of 4 and 2 dofs: H square at
    the block level, so the error function is scaled)."""
    s = golden["small_friction_pb"]
    minv = np.array(s["minv"])
    dofs, nd = s["dofs"], s["ndof_padded"]
    mass = np.zeros_like(minv)
    for k, dk in enumerate(dofs):
        mass[k, :dk, :dk] = np.linalg.inv(minv[k, :dk, :dk])
    f = np.array(s["f_padded"])
    v0 = np.concatenate([-(minv[k] @ f[nd * k:nd * k + nd]) for k in range(2)])
    data = (minv, np.array(s["objA"], np.int32), np.array(s["objB"], np.int32), np.array(s["HA"]),
            np.array(s["HB"]), np.array(s["w"]), np.array(s["mu"]))
    g, o = _run_both(bg, oracle, data, mass, f, v0, np.zeros(6), static=not coulomb, accelerated=accelerated,
                     ls=ls, proj=proj, tol=1e-16, body_dofs=dofs)
    _assert_same(g, o)
    assert g[0] < 1e-8, name


@pytest.fixture(scope="module")
def c1_primal():
    from bogus_gpu import generator

    d = generator.make("c1")
    rng = np.random.default_rng(11)
    f = rng.standard_normal(d.nbodies * 6) * 0.1
    return d, f


@pytest.mark.parametrize("static, accelerated, ls, inf_norm", [
    (True, True, 6, False), (False, True, 0, False), (False, False, 6, True), (True, False, 0, True),
    (False, True, 6, False)])
def test_dual_ama_bitwise_random_pairs(bg, oracle, c1_primal, static, accelerated, ls, inf_norm):
    d, f = c1_primal
    data = (d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    mass = np.linalg.inv(d.minv)
    rng = np.random.default_rng(3)
    v0 = rng.standard_normal(d.nbodies * 6) * 0.01
    r0 = np.abs(rng.standard_normal(3 * d.n)) * 0.01
    g, o = _run_both(bg, oracle, data, mass, f, v0, r0, static=static, accelerated=accelerated, ls=ls,
                     proj=1e-2 if ls == 0 else 1e-1, inf_norm=inf_norm, max_iters=200)
    _assert_same(g, o)
    assert np.isfinite(g[0])


def square_problem(n=96, seed=4):
    """H square at the block level: n contacts, n bodies of 3 dofs, contact i on body i (diagonal block of
    trace near 12, so its error-function scaling is about 4) and on another body or the ground."""
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, 3, 3)) * 0.3
    minv = np.linalg.inv(A @ A.transpose(0, 2, 1) + np.eye(3)[None] * 2.0)
    objA = np.arange(n, dtype=np.int32)
    objB = rng.integers(0, n - 1, n).astype(np.int32)
    objB = np.where(objB >= objA, objB + 1, objB).astype(np.int32)
    objB[rng.random(n) < 0.2] = -1
    HA = np.eye(3)[None] * 4.0 + rng.standard_normal((n, 3, 3)) * 0.2
    HB = np.where((objB < 0)[:, None, None], 0.0, rng.standard_normal((n, 3, 3)) * 0.5)
    w = np.stack([rng.uniform(-1.0, 0.5, n), rng.normal(0, 0.3, n), rng.normal(0, 0.3, n)], 1).reshape(-1)
    mu = rng.uniform(0.3, 0.8, n)
    assert np.all(np.trace(HA, axis1=1, axis2=2) / 3.0 > 1.0)
    return (minv, objA, objB, HA, HB, w, mu), np.linalg.inv(minv)


@pytest.mark.parametrize("static", [True, False])
def test_dual_ama_scaled_error_function(bg, oracle, static):
    data, mass = square_problem()
    n = data[1].size
    rng = np.random.default_rng(8)
    f = rng.standard_normal(3 * n) * 0.1
    g, o = _run_both(bg, oracle, data, mass, f, np.zeros(3 * n), np.zeros(3 * n), static=static, max_iters=150)
    _assert_same(g, o)


def test_admm_scaled_error_function(bg, oracle):
    """ADMM scales its error function the same way (ConstrainedSolverBase::updateScalings on H)."""
    data, _ = square_problem()
    minv, objA, objB, HA, HB, w, mu = data
    n = objA.size
    P = bg.PrimalFrictionProblem(minv, objA, objB, HA, HB, w, mu)
    admm = bg.ADMM()
    admm.setTol(1e-12)
    admm.setMaxIters(120)
    trace = []
    admm.callback().connect(lambda it, res: trace.append((it, res)))
    v, r = np.zeros(3 * n), np.zeros(3 * n)
    res = P.solveWith(admm, 0.0, v, r)
    O = oracle.PrimalProblem(minv, objA, objB, HA, HB)
    tr = oracle.Trace()
    res_o, v_o, r_o, it_o = O.solve_admm(minv, 0.0, mu, np.zeros(3 * n), w, np.zeros(3 * n), np.zeros(3 * n),
                                         tol=1e-12, max_iters=120, trace=tr)
    _assert_same((res, v, r, P.last_iterations, trace), (res_o, v_o, r_o, it_o, tr.items))


def test_dual_ama_zero_iterations_and_bad_inputs(bg, c1_primal):
    d, _ = c1_primal
    mass = np.linalg.inv(d.minv)
    P = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu, M=mass)
    dama = bg.DualAMA()
    dama.setMaxIters(0)
    v, r = np.full(d.nbodies * 6, 0.5), np.full(3 * d.n, 0.25)
    assert P.solveWith(dama, v, r) == -1.0  # the reference returns its initial -1 and the initial iterate
    assert np.all(v == 0.5) and np.all(r == 0.25)
    bad = bg.DualAMA()
    bad.setFpStepSize(0.0)
    with pytest.raises(bg.BogusGpuError):
        P.solveWith(bad, v, r)
    with pytest.raises(ValueError):
        P.solveWith(bg.DualAMA(), v[:-1].copy(), r)
    no_mass = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    with pytest.raises(ValueError):
        no_mass.solveWith(bg.DualAMA(), v, r)
    with pytest.raises(bg.BogusGpuError):
        bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu, M=mass,
                                 body_dofs=np.full(d.nbodies, 7)).solveWith(bg.DualAMA(), v, r)
