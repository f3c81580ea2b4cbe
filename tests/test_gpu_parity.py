"""GPU kernels (through the C ABI) against the CPU oracle on identical inputs.

The kernels follow the oracle's evaluation order, so products, residuals, iterates, iteration counts and
callback traces must be bit-identical (exact equality; +0.0 and -0.0 compare equal). At the full
200 000-contact size, where running the whole oracle solve would take minutes, the checks are
size-independent: bit-identical assembly and products, the returned residual equal to the oracle's
error function at the returned iterate, and the first iterations of the solve bit-identical.
"""
import numpy as np
import pytest

from conftest import small_friction_dual

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


def _gpu_dual(bg, rp, cl, vl, b, mu):
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, b, mu)
    return D


def test_spmv_bitwise(bg, oracle, c1):
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    rng = np.random.default_rng(0)
    for _ in range(3):
        x = rng.standard_normal(3 * d.n)
        assert np.array_equal(D.multiply(x), O.spmv(x))


def test_assembly_bitwise(bg, oracle, c1):
    d, rp, cl, vl = c1
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    grp, gcl, gvl = D.W_lower()
    assert np.array_equal(grp, rp) and np.array_equal(gcl, cl)
    assert np.array_equal(gvl.reshape(-1), vl)
    # b = w - H M^-1 f with f given
    f = np.random.default_rng(5).standard_normal(6 * d.nbodies)
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    b_oracle = P.rhs(f, d.b)
    pr = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b, d.mu, f=f)
    D2 = bg.DualFrictionProblem()
    D2.computeFrom(pr)
    r = np.zeros(3 * d.n)
    # W r + b at r = 0 is b: read it through the error function's input path via a product
    O = oracle.DualProblem(rp, cl, vl, b_oracle, d.mu)
    for coulomb in (True, False):
        assert D2.evalWith(bg.GaussSeidel(), r, staticProblem=not coulomb) == O.eval(r, coulomb=coulomb)


@pytest.mark.parametrize("inf_norm", [False, True])
def test_eval_bitwise(bg, oracle, c1, inf_norm):
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    r = np.random.default_rng(1).standard_normal(3 * d.n)
    pg = bg.ProjectedGradient()
    pg.useInfinityNorm(inf_norm)
    for static in (True, False):
        assert D.evalWith(pg, r, staticProblem=static) == O.eval(r, coulomb=not static, inf_norm=inf_norm)


@pytest.mark.parametrize("variant", [3, 1, 4, 0, 2])  # APGD, Descent, SPG, Standard, Conjugated
@pytest.mark.parametrize("static", [True, False])
def test_projected_gradient_bitwise(bg, oracle, c1, variant, static):
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setTol(1e-8)
    pg.setMaxIters(400)
    trace_gpu = []
    pg.callback().connect(lambda it, res: trace_gpu.append((it, res)))
    r0 = np.random.default_rng(2).standard_normal(3 * d.n) * 0.1
    r = r0.copy()
    res = D.solveWith(pg, r, staticProblem=static)
    tr = oracle.Trace()
    res_o, r_o, it_o = O.solve_pg(r0, variant=variant, coulomb=not static, tol=1e-8, max_iters=400, trace=tr)
    assert res == res_o
    assert D.last_iterations == it_o
    assert np.array_equal(r, r_o)
    assert trace_gpu == tr.items


@pytest.mark.parametrize("static", [True, False])
def test_mixed_precision_converges_to_fp64_residual(bg, oracle, c1, static):
    """FP32 iterations then FP64 refinement: the returned residual is the FP64 error function of the returned
    iterate (bit-identical to the oracle's), it meets the tolerance the FP64 solve meets, and the solve is
    repeatable bit for bit."""
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-10)
    pg.setMaxIters(400)
    pg.setMixedPrecision(True, 200)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=static)
    st = D.solve_stats()
    assert res == O.eval(r, coulomb=not static)
    res_o, _, _ = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=not static, tol=1e-10, max_iters=600)
    assert res_o < 1e-10 and res < 1e-10
    assert 1 <= st["refine_iterations"] <= 201 and st["iterations"] >= st["refine_iterations"]
    assert st["fp32_device_ms"] > 0 and st["kernel_launches"] >= 2
    r2 = np.zeros(3 * d.n)
    assert D.solveWith(pg, r2, staticProblem=static) == res and np.array_equal(r, r2)
    # the FP64 path is untouched by the FP32 copies: a plain solve afterwards is still the oracle's
    pg64 = bg.ProjectedGradient()
    pg64.setTol(1e-8)
    pg64.setMaxIters(400)
    r3 = np.zeros(3 * d.n)
    res3 = D.solveWith(pg64, r3, staticProblem=static)
    res3_o, r3_o, _ = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=not static, tol=1e-8, max_iters=400)
    assert res3 == res3_o and np.array_equal(r3, r3_o)


@pytest.mark.parametrize("minimizer", ["gs", "gs_colored", "pg"])
def test_cadoux_bitwise(bg, oracle, c1, minimizer):
    """DualFrictionProblem::solveCadoux with each minimizer: iterate, Coulomb error, fixed-point iteration count
    and the per-iteration trace equal the oracle's."""
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    trace_gpu = []
    tr = oracle.Trace()
    r0 = np.zeros(3 * d.n)
    if minimizer == "pg":
        solver = bg.ProjectedGradient()
        solver.setTol(1e-8)
        solver.setMaxIters(200)
        solver.callback().connect(lambda it, res: trace_gpu.append((it, res)))
        r = r0.copy()
        res = D.solveCadoux(solver, r, 6)
        res_o, r_o, it_o = O.solve_cadoux_pg(r0, 6, tol=1e-8, max_iters=200, trace=tr)
    else:
        solver = bg.GaussSeidel()
        solver.setTol(1e-8)
        solver.setMaxIters(100)
        solver.doTryZeroAsWell(False)
        solver.coloring().update(minimizer == "gs_colored")
        solver.callback().connect(lambda it, res: trace_gpu.append((it, res)))
        r = r0.copy()
        res = D.solveCadoux(solver, r, 6)
        res_o, r_o, it_o = O.solve_cadoux_gs(r0, 6, tol=1e-8, max_iters=100, coloring=minimizer == "gs_colored",
                                             trace=tr)
    assert res == res_o
    assert D.last_iterations == it_o
    assert np.array_equal(r, r_o)
    assert trace_gpu == tr.items
    # the problem's own right-hand side is intact afterwards: a plain solve still matches the oracle
    pg = bg.ProjectedGradient()
    pg.setMaxIters(50)
    r2 = np.zeros(3 * d.n)
    res2 = D.solveWith(pg, r2)
    res2_o, r2_o, _ = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=False, max_iters=50)
    assert res2 == res2_o and np.array_equal(r2, r2_o)


def test_mixed_precision_rejects_zero_refinement(bg, c1):
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setMixedPrecision(True, 0)
    with pytest.raises(bg.BogusGpuError):
        D.solveWith(pg, np.zeros(3 * d.n))


@pytest.mark.parametrize("strategy", [3, 0, 2])
@pytest.mark.parametrize("static", [False, True])
@pytest.mark.parametrize("coloring", [False, True])
def test_gauss_seidel_bitwise(bg, oracle, c1, strategy, static, coloring):
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    gs = bg.GaussSeidel()
    gs.coloring().update(coloring)
    gs.setLocalStrategy(strategy)
    gs.setTol(1e-8)
    gs.setMaxIters(150)
    trace_gpu = []
    gs.callback().connect(lambda it, res: trace_gpu.append((it, res)))
    r0 = np.zeros(3 * d.n)
    r = r0.copy()
    res = D.solveWith(gs, r, staticProblem=static)
    tr = oracle.Trace()
    res_o, r_o, it_o = O.solve_gs(r0, coulomb=not static, strategy=strategy, tol=1e-8, max_iters=150,
                                  coloring=coloring, trace=tr)
    assert res == res_o
    assert D.last_iterations == it_o
    assert np.array_equal(r, r_o)
    assert trace_gpu == tr.items


def test_gauss_seidel_options_bitwise(bg, oracle, c1):
    """Skip heuristic off, auto-regularization on, infinity norm, no tryZero."""
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    gs = bg.GaussSeidel()
    gs.setSkipTol(0.0)
    gs.setAutoRegularization(1e-3)
    gs.useInfinityNorm(True)
    gs.doTryZeroAsWell(False)
    gs.setEvalEvery(10)
    gs.setMaxIters(60)
    gs.coloring().update(True)
    r = np.ones(3 * d.n)
    res = D.solveWith(gs, r)
    res_o, r_o, it_o = O.solve_gs(np.ones(3 * d.n), coulomb=True, skip_tol=0.0, auto_reg=1e-3, inf_norm=True,
                                  try_zero=False, eval_every=10, max_iters=60, coloring=True)
    assert res == res_o and D.last_iterations == it_o and np.array_equal(r, r_o)


def test_coloring_matches_oracle(bg, oracle, c1):
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    perm, colors = D.coloring()
    perm_o, colors_o = oracle.DualProblem(rp, cl, vl, d.b, d.mu).coloring()
    assert np.array_equal(perm, perm_o) and np.array_equal(colors, colors_o)


# ---- the reference's SmallFrictionPb known answers, solved on the GPU ----------------------------------
def test_small_friction_known_answers(bg, oracle, golden):
    s = golden["small_friction_pb"]
    rp, cl, vl, b, mu = small_friction_dual(golden, oracle)
    D = _gpu_dual(bg, rp, cl, vl, b, mu)
    for strategy in range(4):
        gs = bg.GaussSeidel()
        gs.setLocalStrategy(strategy)
        r = np.ones(6)
        res = D.solveWith(gs, r)
        assert res < s["res_tol"]
        sol = np.array(s["sol"])
        assert np.linalg.norm(sol - r) <= s["sol_rel_tol"] * min(np.linalg.norm(sol), np.linalg.norm(r))
    for variant in (3, 1, 4):
        pg = bg.ProjectedGradient()
        pg.setTol(1e-8)
        pg.setDefaultVariant(variant)
        r = np.ones(6)
        assert D.solveWith(pg, r) < 1e-8


# ---- edge cases ------------------------------------------------------------------------------------------
def test_empty_problem(bg):
    D = bg.DualFrictionProblem()
    D.set(np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), np.zeros(0), np.zeros(0))
    r = np.zeros(0)
    assert D.solveWith(bg.ProjectedGradient(), r) == 0.0
    assert D.solveWith(bg.GaussSeidel(), r) == 0.0


def test_missing_diagonal_negative_mu_and_zero_iterations(bg, oracle):
    # 3 contacts; contact 1 has no diagonal block; contact 2 has mu < 0
    rng = np.random.default_rng(9)
    G = rng.standard_normal((3, 3))
    A = G @ G.T + np.eye(3)
    rp = np.array([0, 1, 1, 3], np.int32)
    cl = np.array([0, 0, 2], np.int32)
    vl = np.concatenate([A.reshape(-1), 0.1 * G.reshape(-1), A.reshape(-1)])
    b = rng.standard_normal(9)
    mu = np.array([0.5, 0.3, -1.0])
    D = _gpu_dual(bg, rp, cl, vl, b, mu)
    O = oracle.DualProblem(rp, cl, vl, b, mu)
    for variant in (3, 4):
        pg = bg.ProjectedGradient()
        pg.setDefaultVariant(variant)
        pg.setMaxIters(50)
        r = np.ones(9)
        res = D.solveWith(pg, r, staticProblem=False)
        res_o, r_o, it_o = O.solve_pg(np.ones(9), variant=variant, coulomb=True, max_iters=50)
        assert res == res_o and np.array_equal(r, r_o)
    for coloring in (False, True):
        gs = bg.GaussSeidel()
        gs.setMaxIters(50)
        gs.coloring().update(coloring)
        r = np.ones(9)
        res = D.solveWith(gs, r)
        res_o, r_o, _ = O.solve_gs(np.ones(9), max_iters=50, coloring=coloring)
        assert res == res_o and np.array_equal(r, r_o)
    # maxIters = 0: the iterate is only projected and the residual is -1, as in the reference
    pg = bg.ProjectedGradient()
    pg.setMaxIters(0)
    r = np.ones(9)
    res = D.solveWith(pg, r)
    res_o, r_o, _ = O.solve_pg(np.ones(9), max_iters=0)
    assert res == res_o == -1.0 and np.array_equal(r, r_o)


def test_bad_inputs_raise(bg):
    D = bg.DualFrictionProblem()
    with pytest.raises(bg.BogusGpuError) as e:  # block above the diagonal in lower storage
        D.set([0, 1, 1], [1], np.eye(3).reshape(-1), np.zeros(6), np.ones(2))
    assert e.value.status == bg.BAD_INPUT
    with pytest.raises(bg.BogusGpuError) as e:
        D.set([0, 1], [0], np.eye(3).reshape(-1), np.array([np.nan, 0, 0]), np.ones(1))
    assert e.value.status == bg.NONFINITE
    D.set([0, 1], [0], np.eye(3).reshape(-1), np.zeros(3), np.ones(1))
    pg = bg.ProjectedGradient()
    pg.setLineSearchIterations(0)
    with pytest.raises(bg.BogusGpuError):
        D.solveWith(pg, np.zeros(3))
    # blocks are checked on the device after the upload, in a staging copy: a rejected W leaves the problem set
    D.set([0, 1], [0], np.eye(3).reshape(-1), np.array([-1.0, 0, 0]), np.ones(1))
    blocks = np.eye(3).reshape(-1).copy()
    blocks[4] = np.inf
    with pytest.raises(bg.BogusGpuError) as e:
        D.set([0, 1], [0], blocks, np.zeros(3), np.ones(1))
    assert e.value.status == bg.NONFINITE
    with pytest.raises(bg.BogusGpuError) as e:  # columns not increasing in row 1
        D.set([0, 1, 3], [0, 1, 0], np.tile(np.eye(3).reshape(-1), 3), np.zeros(6), np.ones(2))
    assert e.value.status == bg.BAD_INPUT and "row 1" in str(e.value)
    r = np.zeros(3)
    assert D.solveWith(bg.GaussSeidel(), r) < 1e-12 and np.allclose(r, [1.0, 0, 0])
    rp, cl, vl = D.W_lower()
    assert list(rp) == [0, 1] and list(cl) == [0] and np.array_equal(vl.reshape(-1), np.eye(3).reshape(-1))


def test_lower_upload_expands_like_the_host(bg, oracle, c1):
    """W from the lower triangle, expanded on the device: the same both-triangle matrix as the oracle's
    expansion (products bit-identical), and the host copy of the lower triangle (downloaded at first use)
    equal to what was uploaded."""
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    x = np.random.default_rng(2).standard_normal(3 * d.n)
    assert np.array_equal(D.multiply(x), O.spmv(x))
    rp2, cl2, vl2 = D.W_lower()
    assert np.array_equal(rp2, rp) and np.array_equal(cl2, cl) and np.array_equal(vl2.reshape(-1), vl.reshape(-1))


def test_repeatable(bg, c1):
    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    outs = []
    for _ in range(2):
        r = np.zeros(3 * d.n)
        outs.append((D.solveWith(bg.ProjectedGradient(), r, staticProblem=False), r.copy()))
    assert outs[0][0] == outs[1][0] and np.array_equal(outs[0][1], outs[1][1])


# ---- full size (200 000 contacts): size-independent checks -----------------------------------------------
@pytest.fixture(scope="module")
def c2(bg, oracle):
    from bogus_gpu import generator

    d = generator.make("c2")
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    return d, D


def test_full_size_assembly_and_product(bg, oracle, c2):
    d, D = c2
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    rp, cl, vl = P.assemble()
    grp, gcl, gvl = D.W_lower()
    assert np.array_equal(grp, rp) and np.array_equal(gcl, cl) and np.array_equal(gvl.reshape(-1), vl)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    x = np.random.default_rng(4).standard_normal(3 * d.n)
    assert np.array_equal(D.multiply(x), O.spmv(x))


def test_full_size_apgd(bg, oracle, c2):
    """500 APGD iterations on 200 000 contacts with both laws: iterate, residual, iteration count and callback
    trace bit-identical to the oracle's (the oracle's OpenMP loops give thread-count-independent results)."""
    d, D = c2
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    O = oracle.DualProblem(*P.assemble(), d.b, d.mu)
    for static in (True, False):
        pg = bg.ProjectedGradient()
        pg.setMaxIters(500)
        trace = []
        pg.callback().connect(lambda it, res: trace.append((it, res)))
        r = np.zeros(3 * d.n)
        res = D.solveWith(pg, r, staticProblem=static)
        tr = oracle.Trace()
        res_o, r_o, it_o = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=not static, max_iters=500, trace=tr)
        assert res == res_o and D.last_iterations == it_o
        assert np.array_equal(r, r_o)
        assert trace == tr.items
        # the returned residual is the error function at the returned iterate
        assert res == O.eval(r, coulomb=not static)


@pytest.mark.parametrize("variant", [0, 2])  # Standard, Conjugated
def test_full_size_standard_and_conjugated(bg, oracle, c2, variant):
    """The projected-gradient variants with an Armijo line search, 40 iterations on 200 000 contacts (Coulomb
    law): iterate, residual, iteration count and trace bit-identical to the oracle's."""
    d, D = c2
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    O = oracle.DualProblem(*P.assemble(), d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setMaxIters(40)
    trace = []
    pg.callback().connect(lambda it, res: trace.append((it, res)))
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=False)
    tr = oracle.Trace()
    res_o, r_o, it_o = O.solve_pg(np.zeros(3 * d.n), variant=variant, coulomb=True, max_iters=40, trace=tr)
    assert res == res_o and D.last_iterations == it_o
    assert np.array_equal(r, r_o)
    assert trace == tr.items


def test_standard_and_conjugated_rejected_where_not_built(bg, c1):
    """Standard and Conjugated run in FP64 single-problem solves: the FP32-refined and batched forms refuse them."""
    from bogus_gpu import generator

    d, rp, cl, vl = c1
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    for variant in (0, 2):
        pg = bg.ProjectedGradient()
        pg.setDefaultVariant(variant)
        pg.setMixedPrecision(True, 10)
        with pytest.raises(bg.BogusGpuError):
            D.solveWith(pg, np.zeros(3 * d.n))
    db, cptr = generator.batch(nproblems=3, nmin=16, nmax=40, seed=3)
    B = bg.DualFrictionProblem()
    B.computeFrom(bg.PrimalFrictionProblem.from_generated(db))
    B.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setDefaultVariant(2)
    with pytest.raises(bg.BogusGpuError):
        B.solveBatchWith(pg, np.zeros(3 * db.n))


def test_full_size_mixed_precision(bg, oracle, c2):
    """500 FP32 iterations + up to 50 FP64 ones on 200 000 contacts: the returned residual is the oracle's
    FP64 error function at the returned iterate, and it is no worse than a tenth of the FP64 solve's
    improvement over the start (the FP32 part does the work of the FP64 one)."""
    d, D = c2
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    O = oracle.DualProblem(*P.assemble(), d.b, d.mu)
    pg = bg.ProjectedGradient()
    pg.setMaxIters(500)
    pg.setMixedPrecision(True, 50)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=True)
    assert res == O.eval(r, coulomb=False)
    pg64 = bg.ProjectedGradient()
    pg64.setMaxIters(500)
    r64 = np.zeros(3 * d.n)
    res64 = D.solveWith(pg64, r64, staticProblem=True)
    res0 = O.eval(np.zeros(3 * d.n), coulomb=False)
    assert res <= res0 - 0.9 * (res0 - res64)


def test_full_size_gauss_seidel_first_sweeps(bg, oracle, c2):
    d, D = c2
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    O = oracle.DualProblem(*P.assemble(), d.b, d.mu)
    for coloring in (False, True):
        gs = bg.GaussSeidel()
        gs.coloring().update(coloring)
        gs.setMaxIters(2)
        gs.setEvalEvery(1)
        r = np.zeros(3 * d.n)
        res = D.solveWith(gs, r)
        res_o, r_o, _ = O.solve_gs(np.zeros(3 * d.n), max_iters=2, eval_every=1, coloring=coloring)
        assert res == res_o and np.array_equal(r, r_o)


# ---- batched solves: one launch, each problem bit-identical to its own solve --------------------------
@pytest.mark.parametrize("variant", [3, 4])
def test_batched_matches_single_problem_solves(bg, oracle, variant):
    from bogus_gpu import generator

    d, cptr = generator.batch(nproblems=24, nmin=16, nmax=400, seed=7)
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setTol(1e-8)
    pg.setMaxIters(300)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r, staticProblem=False)
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    for p in range(len(cptr) - 1):
        c0, c1 = cptr[p], cptr[p + 1]
        prp = rp[c0:c1 + 1] - rp[c0]
        pcl = cl[rp[c0]:rp[c1]] - c0
        pvl = vl[rp[c0]:rp[c1]].reshape(-1)
        O = oracle.DualProblem(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
        res_o, r_o, it_o = O.solve_pg(np.zeros(3 * (c1 - c0)), variant=variant, coulomb=True, tol=1e-8,
                                      max_iters=300)
        assert res[p] == res_o and its[p] == it_o, p
        assert np.array_equal(r[3 * c0:3 * c1], r_o), p


def test_batched_mixed_precision_matches_single_problem_solves(bg):
    """FP32-refined batch: each problem's residual, iteration count and iterate equal its own FP32-refined
    single-problem solve (same FP32 order, same FP64 refinement)."""
    from bogus_gpu import generator

    d, cptr = generator.batch(nproblems=16, nmin=16, nmax=300, seed=9)
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setTol(1e-8)
    pg.setMaxIters(200)
    pg.setMixedPrecision(True, 40)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r, staticProblem=True)
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    single = bg.DualFrictionProblem()
    for p in range(len(cptr) - 1):
        c0, c1 = cptr[p], cptr[p + 1]
        single.set(rp[c0:c1 + 1] - rp[c0], cl[rp[c0]:rp[c1]] - c0, vl[rp[c0]:rp[c1]].reshape(-1), d.b[c0:c1],
                   d.mu[c0:c1])
        rs = np.zeros(3 * (c1 - c0))
        res_s = single.solveWith(pg, rs)
        assert res[p] == res_s and its[p] == single.last_iterations, p
        assert np.array_equal(r[3 * c0:3 * c1], rs), p


@pytest.mark.parametrize("variant, mixed", [(3, False), (4, False), (3, True)])
def test_team_batch_matches_single_problem_solves(bg, oracle, variant, mixed):
    """Few large problems: the batch runs several CTAs per problem (team schedule); each problem's result equals
    its own single-problem solve (and, in FP64, the oracle's) bit for bit."""
    from bogus_gpu import generator

    d, cptr = generator.batch(nproblems=5, nmin=1500, nmax=3000, seed=13)
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bg.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setTol(1e-8)
    pg.setMaxIters(150)
    if mixed:
        pg.setMixedPrecision(True, 40)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r, staticProblem=True)
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    single = bg.DualFrictionProblem()
    for p in range(len(cptr) - 1):
        c0, c1 = cptr[p], cptr[p + 1]
        prp, pcl, pvl = rp[c0:c1 + 1] - rp[c0], cl[rp[c0]:rp[c1]] - c0, vl[rp[c0]:rp[c1]].reshape(-1)
        single.set(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
        rs = np.zeros(3 * (c1 - c0))
        res_s = single.solveWith(pg, rs)
        assert res[p] == res_s and its[p] == single.last_iterations, p
        assert np.array_equal(r[3 * c0:3 * c1], rs), p
        if not mixed and p == 0:
            O = oracle.DualProblem(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
            res_o, r_o, it_o = O.solve_pg(np.zeros(3 * (c1 - c0)), variant=variant, coulomb=False, tol=1e-8,
                                          max_iters=150)
            assert res[p] == res_o and its[p] == it_o and np.array_equal(rs, r_o)


def test_batch_rejects_coupled_partition(bg):
    from bogus_gpu import generator

    d = generator.make("c1")
    D = bg.DualFrictionProblem()
    D.computeFrom(bg.PrimalFrictionProblem.from_generated(d))
    with pytest.raises(bg.BogusGpuError) as e:
        D.setBatch([0, 250, d.n])  # random pairs couple the two halves
    assert e.value.status == bg.BAD_INPUT


@pytest.fixture(scope="module")
def grid20k(oracle):
    """A 20 000-contact grid problem: 625 chunks, enough CTAs that the reductions run on 8 combining CTAs."""
    from bogus_gpu import generator

    d = generator.grid(nbodies=5_000, ncontacts=20_000, seed=7)
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    rp, cl, vl = P.assemble()
    return d, rp, cl, vl


@pytest.mark.parametrize("variant", [3, 1])  # APGD, Descent: reductions after the A phases are split
@pytest.mark.parametrize("tol, max_iters", [(1e3, 50), (1e-30, 1), (1e-30, 2), (1e-30, 3), (1e-30, 7), (0.1, 60)])
def test_projected_gradient_early_exits_bitwise(bg, oracle, grid20k, variant, tol, max_iters):
    """Solves that stop at the first residual check (the warps drop the trial product they started before
    the residual was published), after a few iterations, or on convergence part way: iterate, residual,
    iteration count and callback trace equal the oracle's."""
    d, rp, cl, vl = grid20k
    D = _gpu_dual(bg, rp, cl, vl, d.b, d.mu)
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    for static in (True, False):
        pg = bg.ProjectedGradient()
        pg.setDefaultVariant(variant)
        pg.setTol(tol)
        pg.setMaxIters(max_iters)
        trace_gpu = []
        pg.callback().connect(lambda it, res: trace_gpu.append((it, res)))
        r0 = np.random.default_rng(5).standard_normal(3 * d.n) * 0.05
        r = r0.copy()
        res = D.solveWith(pg, r, staticProblem=static)
        tr = oracle.Trace()
        res_o, r_o, it_o = O.solve_pg(r0, variant=variant, coulomb=not static, tol=tol, max_iters=max_iters, trace=tr)
        assert res == res_o
        assert D.last_iterations == it_o
        assert np.array_equal(r, r_o)
        assert trace_gpu == tr.items
