"""Pins the CPU oracle against So-bogus's own unit tests (values in tests/golden/reference_fixtures.json).

Each test names the reference test it restates; thresholds are the reference's.
"""
import numpy as np
import pytest

from conftest import small_friction_dual


def isApprox(a, b, prec):
    """Eigen's isApprox: |a - b| <= prec * min(|a|, |b|)."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.linalg.norm(a - b) <= prec * min(np.linalg.norm(a), np.linalg.norm(b))


# ---- tests/ProjectedGradient.cpp:85-108 ----------------------------------------------------------
def test_projection_cases(oracle, golden):
    for case in golden["projection"]["cases"]:
        out = oracle.project(case["mu"], case["x"])
        exp = np.array(case["expected"], float)
        if case["exact"]:
            assert np.array_equal(out, exp)
        elif np.all(exp == 0):
            assert np.all(np.abs(out) < 1e-12)  # x.isZero()
        else:
            assert isApprox(out, exp, 1e-12)


# ---- tests/Polynomial.cpp:17-38 -------------------------------------------------------------------
def test_quadratic_roots(oracle, golden):
    for case in golden["polynomial"]["quadratic"]:
        roots = oracle.real_roots(case["coeffs"], degenerate=False, filt=case["filter"])
        assert len(roots) == len(case["roots"])
        # EXPECT_DOUBLE_EQ: within 4 ulps
        for got, exp in zip(sorted(roots), sorted(case["roots"])):
            assert abs(got - exp) <= 4 * np.spacing(abs(exp))


# ---- tests/Polynomial.cpp:40-94: 3D SOC local problem by the enumerative solver ------------------
def test_soc_quartic_pure_enumerative(oracle, golden):
    chk = golden["polynomial"]["soc_quartic_checks"]
    for case in golden["polynomial"]["soc_quartic"]:
        W = np.array(case["W"], float).reshape(3, 3)
        b = np.array(case["b"], float)
        res, r = oracle.local_solve(W, b, np.zeros(3), case["mu"], coulomb=False, strategy=1, tol=1e-12)
        u = W @ r + b
        assert res < chk["res_below"]
        assert r[0] > 0
        assert u[0] > 0
        assert np.float32(u[0]) == pytest.approx(np.float32(np.linalg.norm(u[1:]) * case["mu"]), rel=4 * 2 ** -23)
        assert u @ r < chk["complementarity_below"]


# ---- tests/BlockMV.cpp:193-296: symmetric 3x3-block products ---------------------------------------
def test_block_mv_symmetric(oracle, golden):
    g = golden["block_mv_symmetric"]
    D = oracle.DualProblem(g["rowptr"], g["col"], g["val"], np.zeros(9), np.ones(3))
    rhs = np.array(g["rhs"], float)
    assert np.array_equal(D.spmv(rhs), np.array(g["expected_product"], float))
    res = np.zeros(9)
    for k in range(3):
        res[3 * k:3 * k + 3] = D.split_row(k, rhs, res[3 * k:3 * k + 3])
    assert np.array_equal(res, np.array(g["expected_split_row"], float))
    # accumulating into the previous result doubles it (the "ussbm" case of the same test)
    res2 = res.copy()
    for k in range(3):
        res2[3 * k:3 * k + 3] = D.split_row(k, rhs, res2[3 * k:3 * k + 3])
    assert np.array_equal(res2, 2 * np.array(g["expected_split_row"], float))


# ---- tests/SparseBlock.cpp:464-498: permutation of a symmetric matrix ---------------------------------
def test_symmetric_permutation(oracle, golden):
    perm = np.array(golden["permutation"]["perm"])
    n = len(perm)
    # symmetric matrix whose block (i, j) is diag(i + j, j + i): the test's sbm += sbm^T, lower part stored
    rowptr = np.arange(0, (n + 1) * (n + 2) // 2, 1)
    rp, cl, vl = [0], [], []
    for i in range(n):
        for j in range(i + 1):
            cl.append(j)
            vl.extend([i + j, 0, 0, 0, j + i, 0, 0, 0, 0])
        rp.append(len(cl))
    del rowptr
    D = oracle.DualProblem(rp, cl, vl, np.zeros(3 * n), np.ones(n))
    # new (i, j) = old (perm[i], perm[j]): check through products with unit vectors on the full view
    frp, fcl, fvl = D.full()
    dense = np.zeros((3 * n, 3 * n))
    for i in range(n):
        for k in range(frp[i], frp[i + 1]):
            dense[3 * i:3 * i + 3, 3 * fcl[k]:3 * fcl[k] + 3] = fvl[9 * k:9 * k + 9].reshape(3, 3)
    P = np.zeros((3 * n, 3 * n))
    for i in range(n):
        P[3 * i:3 * i + 3, 3 * perm[i]:3 * perm[i] + 3] = np.eye(3)
    permuted = P @ dense @ P.T
    for i in range(n):
        for j in range(i + 1):
            blk = permuted[3 * i:3 * i + 3, 3 * j:3 * j + 3]
            assert blk[0, 0] == perm[i] + perm[j]
            assert blk[1, 1] == perm[j] + perm[i]


# ---- tests/SparseBlock.cpp:16-60: H H^T ----------------------------------------------------------------
def test_sparse_product_hht(oracle, golden):
    g = golden["sparse_product"]["blocks"]
    ones = np.ones((3, 4))
    # block rows 0..2 as "contacts"; block cols 0..1 as 4-dof "bodies"; M^-1 = I
    minv = np.stack([np.eye(4), np.eye(4)])
    objA = [1, 0, 0]
    objB = [-1, -1, 1]
    HA = np.stack([np.array(g["0,1"]), np.array(g["1,0"]), np.array(g["2,0"])])
    HB = np.stack([np.zeros((3, 4)), np.zeros((3, 4)), np.array(g["2,1"])])
    P = oracle.PrimalProblem(minv, objA, objB, HA, HB)
    rp, cl, vl = P.assemble()
    blocks = {(i, cl[k]): vl[9 * k:9 * k + 9].reshape(3, 3) for i in range(3) for k in range(rp[i], rp[i + 1])}
    assert np.array_equal(blocks[(2, 2)], np.full((3, 3), golden["sparse_product"]["diag2_value"]))
    H = np.zeros((9, 8))
    H[0:3, 4:8] = ones
    H[3:6, 0:4] = np.array(g["1,0"])
    H[6:9, 0:4] = 3 * ones
    H[6:9, 4:8] = 5 * ones
    dense = H @ H.T
    for (i, j), blk in blocks.items():
        assert np.array_equal(blk, dense[3 * i:3 * i + 3, 3 * j:3 * j + 3])
    assert (1, 0) not in blocks or np.array_equal(blocks[(1, 0)], dense[3:6, 0:3])


# ---- tests/SmallFrictionPb.hpp + tests/GaussSeidel.cpp:19-65 -------------------------------------------
def test_small_friction_assembly(oracle, golden):
    s = golden["small_friction_pb"]
    rp, cl, vl, b, mu = small_friction_dual(golden, oracle)
    Wd = np.array(s["W_dense"])
    for i in range(2):
        for k in range(rp[i], rp[i + 1]):
            j = cl[k]
            assert np.allclose(vl[9 * k:9 * k + 9].reshape(3, 3), Wd[3 * i:3 * i + 3, 3 * j:3 * j + 3], rtol=0,
                               atol=1e-12)
    assert np.allclose(b, s["b"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("strategy", [0, 1, 2, 3])
def test_small_friction_gauss_seidel(oracle, golden, strategy):
    s = golden["small_friction_pb"]
    D = oracle.DualProblem(*small_friction_dual(golden, oracle))
    res, r, _ = D.solve_gs(np.ones(6), coulomb=True, strategy=strategy, coloring=False)
    assert res < s["res_tol"]
    assert isApprox(s["sol"], r, s["sol_rel_tol"])


def test_small_friction_gauss_seidel_soc(oracle, golden):
    D = oracle.DualProblem(*small_friction_dual(golden, oracle))
    res, r, _ = D.solve_gs(np.ones(6), coulomb=False, tol=1e-8, coloring=False)
    assert res < 1e-8


# ---- tests/ProjectedGradient.cpp:16-61 ---------------------------------------------------------------
@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4])
def test_small_friction_projected_gradient(oracle, golden, variant):
    D = oracle.DualProblem(*small_friction_dual(golden, oracle))
    res, r, _ = D.solve_pg(np.ones(6), variant=variant, coulomb=False, tol=1e-8)
    assert res < 1e-8


# ---- Cadoux fixed point (Interfaces/Cadoux.hpp:44-91); the reference has no test of its own, so the result is
# held to the Coulomb solution of tests/SmallFrictionPb.hpp (the one GaussSeidel.cpp checks) ------------------
@pytest.mark.parametrize("minimizer", ["gs", "pg"])
def test_small_friction_cadoux_reaches_the_coulomb_solution(oracle, golden, minimizer):
    s = golden["small_friction_pb"]
    D = oracle.DualProblem(*small_friction_dual(golden, oracle))
    if minimizer == "gs":
        res, r, it = D.solve_cadoux_gs(np.ones(6), 50, tol=1e-10, max_iters=1000)
    else:
        res, r, it = D.solve_cadoux_pg(np.ones(6), 50, tol=1e-10, max_iters=3000)
    assert res < 1e-10 and it <= 50
    assert isApprox(s["sol"], r, s["sol_rel_tol"])
    assert D.eval(r, coulomb=True) < 1e-9


# ---- tests/ADMM.cpp:16-60 (primal AMA with lambda = 0, ADMM with lambda = 0.1) ---------------------------
def _small_primal(oracle, golden):
    s = golden["small_friction_pb"]
    minv = np.array(s["minv"])
    P = oracle.PrimalProblem(minv, s["objA"], s["objB"], np.array(s["HA"]), np.array(s["HB"]))
    HA, HB = np.array(s["HA"]), np.array(s["HB"])
    nd = s["ndof_padded"]
    Hd = np.zeros((6, 2 * nd))  # dense H of the padded layout
    for i in range(2):
        Hd[3 * i:3 * i + 3, nd * s["objA"][i]:nd * s["objA"][i] + nd] += HA[i]
        if s["objB"][i] >= 0:
            Hd[3 * i:3 * i + 3, nd * s["objB"][i]:nd * s["objB"][i] + nd] += HB[i]
    return s, P, minv, Hd


def admm_inputs(s, minv, Hd, lam):
    """The reference test's start (r = 1, v = M^-1 (H^T r - f)) and prox operator: M^-1 for lambda = 0, else
    (M + I / lambda)^-1 per body (inert padded dofs: 0)."""
    f = np.array(s["f_padded"])
    nd = s["ndof_padded"]
    r = np.ones(6)
    Minv = np.zeros((2 * nd, 2 * nd))
    for k in range(2):
        Minv[nd * k:nd * k + nd, nd * k:nd * k + nd] = minv[k]
    v = Minv @ (Hd.T @ r - f)
    if lam == 0:
        return minv.copy(), v, r, f
    prox = np.zeros_like(minv)
    for k, dk in enumerate(s["dofs"]):
        Mk = np.linalg.inv(minv[k, :dk, :dk])
        prox[k, :dk, :dk] = np.linalg.inv(Mk + np.eye(dk) / lam)
    return prox, v, r, f


@pytest.mark.parametrize("lam", [0.0, 0.1])
def test_small_friction_admm(oracle, golden, lam):
    s, P, minv, Hd = _small_primal(oracle, golden)
    prox, v, r, f = admm_inputs(s, minv, Hd, lam)
    res, v, r, it = P.solve_admm(prox, lam, np.array(s["mu"]), f, np.array(s["w"]), v, r, tol=1e-8, max_iters=1000,
                                 step=1e-2, accelerated=True)
    assert 0 <= res < 1e-8 and it < 1000


def test_coloring_is_valid_and_follows_reference_rule(oracle):
    from bogus_gpu import generator

    d = generator.make("c1")
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    rp, cl, vl = P.assemble()
    D = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    perm, colors = D.coloring()
    assert sorted(perm.tolist()) == list(range(d.n))
    color_of = np.empty(d.n, int)
    for c in range(len(colors) - 1):
        members = perm[colors[c]:colors[c + 1]]
        assert np.all(np.diff(members) > 0)
        color_of[members] = c
    for i in range(d.n):
        for k in range(rp[i], rp[i + 1]):
            j = cl[k]
            if j < i:
                assert color_of[i] != color_of[j]
                # the reference's lower_bound test: no member of i's color lies in [j, i)
                members = perm[colors[color_of[i]]:colors[color_of[i] + 1]]
                assert not np.any((members >= j) & (members < i))


def test_canonical_sum_matches_its_definition(oracle):
    rng = np.random.default_rng(3)
    for n in [0, 1, 31, 32, 33, 1000, 5000]:
        v = rng.standard_normal(n)
        C = (n + 31) // 32
        pad = np.zeros(C * 32)
        pad[:n] = v
        sums = []
        for c in range(C):
            w = list(pad[32 * c:32 * c + 32])
            for off in (16, 8, 4, 2, 1):
                w = [w[l] + w[l ^ off] for l in range(32)]
            sums.append(w[0])
        per = (C + 7) // 8
        total = 0.0
        for k in range(8):
            lanes = []
            for l in range(32):
                p = 0.0
                for c in range(k * per + l, min(C, (k + 1) * per), 32):
                    p = p + sums[c]
                lanes.append(p)
            for off in (16, 8, 4, 2, 1):
                lanes = [lanes[l] + lanes[l ^ off] for l in range(32)]
            total = lanes[0] if k == 0 else total + lanes[0]
        got = oracle.canonical_sum(v)
        assert got == total
        assert got == pytest.approx(float(np.sum(v)), abs=1e-9 * max(1, n))


# ---- MecheFrictionProblem (Interfaces/MecheInterface.cpp:97-367); the reference has no test of its own, so the
# facade is held to the Coulomb solution of tests/SmallFrictionPb.hpp, posed in world coordinates ------------
def small_friction_world():
    """SmallFrictionPb in world coordinates: contact frames E_i (a random rotation, the fixture's own frame),
    world Jacobians HA = E H_A, HB = -E H_B, world w = E w_local. Returns the Meche inputs and the frames."""
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_fixtures.json")) as fh:
        s = json.load(fh)["small_friction_pb"]
    nd = s["ndof_padded"]
    dofs = s["dofs"]
    minv = np.array(s["minv"])
    mass = [np.linalg.inv(minv[k, :dofs[k], :dofs[k]]) for k in range(2)]
    HA = np.array(s["HA"])
    HB = np.array(s["HB"])
    q, _ = np.linalg.qr(np.random.default_rng(3).standard_normal((3, 3)))
    E = np.stack([q, np.array([[0.0, 0, 1], [1, 0, 0], [0, 1, 0]])])
    HAw = [E[0] @ HA[0][:, :dofs[0]], E[1] @ HA[1][:, :dofs[0]]]
    HBw = [-(E[0] @ HB[0][:, :dofs[1]]), None]
    w = np.array(s["w"])
    ww = np.concatenate([E[i] @ w[3 * i:3 * i + 3] for i in range(2)])
    f = np.array(s["f_padded"])
    fp = np.concatenate([f[:dofs[0]], f[nd:nd + dofs[1]]])
    return s, dict(mass=mass, f=fp, mu=np.array(s["mu"]), E=E, w=ww, objA=[0, 0], objB=[1, -1], HA=HAw, HB=HBw)


@pytest.mark.parametrize("algorithm, cadoux", [(0, 0), (1, 40)])  # Gauss-Seidel; projected gradient + Cadoux
def test_meche_reaches_the_coulomb_solution(oracle, algorithm, cadoux):
    s, inp = small_friction_world()
    M = oracle.MecheProblem(**inp)
    res, r, v = M.solve(np.zeros(6), algorithm=algorithm, cadoux_iters=cadoux, tolerance=1e-10, max_iters=3000,
                        pg_variant=3)
    assert res < 1e-10
    E = inp["E"]
    r_loc = np.concatenate([E[i].T @ r[3 * i:3 * i + 3] for i in range(2)])
    assert isApprox(s["sol"], r_loc, s["sol_rel_tol"])
    # v = M^-1 (H^T r - f) in the bodies' own dofs
    Hd = np.zeros((6, 6))
    Hd[0:3, 0:4] = E[0].T @ inp["HA"][0]
    Hd[0:3, 4:6] = -(E[0].T @ inp["HB"][0])
    Hd[3:6, 0:4] = E[1].T @ inp["HA"][1]
    Mi = np.zeros((6, 6))
    Mi[:4, :4] = np.linalg.inv(inp["mass"][0])
    Mi[4:, 4:] = np.linalg.inv(inp["mass"][1])
    assert np.allclose(v, Mi @ (Hd.T @ r_loc - inp["f"]), rtol=0, atol=1e-12)


def test_meche_admm_matches_the_primal_solver(oracle):
    """Algorithm ADMM: PrimalFrictionProblem::solveWith(ADMM&, 0, v, E^T r) on the local problem."""
    s, inp = small_friction_world()
    M = oracle.MecheProblem(**inp)
    res, r, v = M.solve(np.zeros(6), algorithm=3, tolerance=1e-9, max_iters=2000, admm_step=1e-2, static=True)
    assert res < 1e-9
    P = oracle.PrimalProblem(np.array(s["minv"]), s["objA"], s["objB"], np.array(s["HA"]), np.array(s["HB"]))
    minv = np.array(s["minv"])
    res_o, v_o, r_o, _ = P.solve_admm(minv, 0.0, np.array(s["mu"]), np.array(s["f_padded"]), np.array(s["w"]),
                                      np.zeros(8), np.zeros(6), tol=1e-9, max_iters=2000, step=1e-2,
                                      true_dofs=[4, 2])
    E = inp["E"]
    r_loc = np.concatenate([E[i].T @ r[3 * i:3 * i + 3] for i in range(2)])
    assert np.allclose(r_loc, r_o, rtol=0, atol=1e-6)


def test_meche_dual_ama_reaches_the_coulomb_solution(oracle):
    """Algorithm DualAMA (MecheInterface.cpp:249-261: no line search, admmProjStepSize / admmFpStepSize) on the
    Coulomb problem reaches the reference solution of tests/SmallFrictionPb.hpp."""
    s, inp = small_friction_world()
    M = oracle.MecheProblem(**inp)
    res, r, v = M.solve(np.zeros(6), with_v=False, algorithm=4, tolerance=1e-12, max_iters=3000, admm_step=1e-2,
                        admm_fp_step=1e-1)
    assert res < 1e-12
    E = inp["E"]
    r_loc = np.concatenate([E[i].T @ r[3 * i:3 * i + 3] for i in range(2)])
    assert isApprox(s["sol"], r_loc, s["sol_rel_tol"])


# ---- ProductGaussSeidel (Core/BlockSolvers/ProductGaussSeidel.impl.hpp): the matrix-free sweep reaches the
# Coulomb solution of tests/SmallFrictionPb.hpp, as Gauss-Seidel on the assembled W does ---------------------
@pytest.mark.parametrize("strategy", [0, 3])
def test_small_friction_product_gauss_seidel(oracle, golden, strategy):
    s = golden["small_friction_pb"]
    P = oracle.PrimalProblem(np.array(s["minv"]), s["objA"], s["objB"], np.array(s["HA"]), np.array(s["HB"]))
    res, r, _ = P.solve_product_gs(np.array(s["f_padded"]), np.array(s["w"]), np.array(s["mu"]), np.ones(6),
                                   coulomb=True, strategy=strategy, tol=1e-8)
    assert res < s["res_tol"]
    assert isApprox(s["sol"], r, s["sol_rel_tol"])


# ---- tests/ADMM.cpp:135-189: DualAMA on SmallFrictionPb (its own 4 + 2 dofs), Standard with line search and
# Accelerated without, on the SOC cone and the Coulomb law; the Coulomb results at the reference solution -----
@pytest.mark.parametrize("name, variant_acc, ls, proj, coulomb", [
    ("Std-Kmu", False, 4, 1.0, False), ("Std-Cmu", False, 4, 1.0, True),
    ("Acc-Kmu", True, 0, 1e-1, False), ("Acc-Cmu", True, 0, 1e-2, True)])
def test_small_friction_dual_ama(oracle, golden, name, variant_acc, ls, proj, coulomb):
    s = golden["small_friction_pb"]
    minv = np.array(s["minv"])
    P = oracle.PrimalProblem(minv, s["objA"], s["objB"], np.array(s["HA"]), np.array(s["HB"]))
    dofs = s["dofs"]
    nd = s["ndof_padded"]
    mass = np.zeros_like(minv)
    for k, dk in enumerate(dofs):
        mass[k, :dk, :dk] = np.linalg.inv(minv[k, :dk, :dk])
    f = np.array(s["f_padded"])
    v0 = np.concatenate([-(minv[k] @ f[nd * k:nd * k + nd]) for k in range(2)])  # M^-1 (H^T 0 - f)
    res, v, r, _ = P.solve_dual_ama(mass, np.array(s["mu"]), f, np.array(s["w"]), v0, np.zeros(6),
                                    static=not coulomb, tol=1e-16, fp_step=1e-1, proj_step=proj, ls_iters=ls,
                                    optimistic=1.25, accelerated=variant_acc, true_dofs=dofs)
    assert res < 1e-8, name
    if coulomb:
        assert isApprox(s["sol"], r, 1e-4), name


def test_oracle_threads_do_not_change_primal_solvers(oracle):
    """The oracle's ADMM and DualAMA run their H, H^T, body and contact loops on OpenMP threads; every result
    must be the same bit for bit whatever the thread count (H^T r gathers each body's contacts in the order
    of the sequential scatter), since the GPU parity tests compare against it."""
    from bogus_gpu import generator

    d = generator.grid(nbodies=600, ncontacts=2_400, seed=9)
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    mass = np.linalg.inv(d.minv)
    f = np.random.default_rng(2).standard_normal(d.nbodies * 6) * 0.1
    w = d.b.reshape(-1)
    saved = oracle.num_threads()
    outs = []
    try:
        for t in (1, 3, max(2, saved)):
            oracle.set_num_threads(t)
            a = P.solve_admm(d.minv, 0.0, d.mu, np.zeros(d.nbodies * 6), w, np.zeros(d.nbodies * 6),
                             np.zeros(3 * d.n), max_iters=30)
            b = P.solve_dual_ama(mass, d.mu, f, w, np.zeros(d.nbodies * 6), np.zeros(3 * d.n), max_iters=30)
            outs.append((a, b))
    finally:
        oracle.set_num_threads(saved)
    for (a, b) in outs[1:]:
        assert a[0] == outs[0][0][0] and a[3] == outs[0][0][3]
        assert np.array_equal(a[1], outs[0][0][1]) and np.array_equal(a[2], outs[0][0][2])
        assert b[0] == outs[0][1][0] and b[3] == outs[0][1][3]
        assert np.array_equal(b[1], outs[0][1][1]) and np.array_equal(b[2], outs[0][1][2])


def test_parallel_colored_gauss_seidel_timing_path(oracle):
    """The timing-only per-color OpenMP sweep (the reference's parallel loop) reaches the sequential sweep's
    accuracy; its iterates may differ (the shared step-size reference decides which contacts skip)."""
    from bogus_gpu import generator

    d = generator.grid(nbodies=1_500, ncontacts=6_000, seed=3)
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    rp, cl, vl = P.assemble()
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    res_seq, _, _ = O.solve_gs(np.zeros(3 * d.n), max_iters=50, coloring=True)
    assert oracle.last_gs_sweep_ms() > 0.0
    try:
        oracle.set_gs_threads(4)
        res_par, r_par, _ = O.solve_gs(np.zeros(3 * d.n), max_iters=50, coloring=True)
    finally:
        oracle.set_gs_threads(1)
    assert np.all(np.isfinite(r_par))
    assert res_par < 2.0 * res_seq + 1e-12
    res_again, _, _ = O.solve_gs(np.zeros(3 * d.n), max_iters=50, coloring=True)
    assert res_again == res_seq  # back to the sequential sweep
