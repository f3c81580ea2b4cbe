"""Parity at the configurations' own sizes.

* The 4096-problem batch (16..4096 contacts, log-uniform, 3.09 M contacts): one batched launch, and every
  problem's residual, iteration count and iterate equal its own single-problem solve bit for bit; the oracle
  agrees on a stratified sample (every 64th problem by size). The FP32-refined batch equals the FP32-refined
  single-problem solves on every 16th problem by size.
* The gradient workload's problem size (20 000 contacts): the adjoint against central differences.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6
MAX_ITERS = 500


@pytest.fixture(scope="module")
def batch4096(oracle):
    import bogus_gpu
    from bogus_gpu import generator

    d, cptr = generator.batch(4096)
    D = bogus_gpu.DualFrictionProblem()
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    rp, cl, vl = D.W_lower()
    return d, cptr, D, rp, cl, vl.reshape(-1, 9)


def _problem(d, cptr, rp, cl, vl, p):
    c0, c1 = int(cptr[p]), int(cptr[p + 1])
    return c0, c1, rp[c0:c1 + 1] - rp[c0], cl[rp[c0]:rp[c1]] - c0, vl[rp[c0]:rp[c1]].reshape(-1)


def test_batch_4096_every_problem_equals_its_single_solve(batch4096, oracle):
    import bogus_gpu

    d, cptr, D, rp, cl, vl = batch4096
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(MAX_ITERS)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r)
    assert len(res) == 4096 and d.n > 3_000_000
    sizes = np.diff(cptr)
    order = np.argsort(-sizes, kind="stable")  # largest first: the single handle's buffers grow once
    single = bogus_gpu.DualFrictionProblem()
    for p in order:
        c0, c1, prp, pcl, pvl = _problem(d, cptr, rp, cl, vl, p)
        single.set(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
        rs = np.zeros(3 * (c1 - c0))
        res_s = single.solveWith(pg, rs)
        assert res[p] == res_s and its[p] == single.last_iterations, p
        assert np.array_equal(r[3 * c0:3 * c1], rs), p
    for p in np.argsort(sizes, kind="stable")[::64]:
        c0, c1, prp, pcl, pvl = _problem(d, cptr, rp, cl, vl, p)
        O = oracle.DualProblem(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
        res_o, r_o, it_o = O.solve_pg(np.zeros(3 * (c1 - c0)), variant=3, coulomb=False, tol=TOL, max_iters=MAX_ITERS)
        assert res[p] == res_o and its[p] == it_o and np.array_equal(r[3 * c0:3 * c1], r_o), p


def test_batch_4096_fp32_refined_equals_single_solves(batch4096):
    import bogus_gpu

    d, cptr, D, rp, cl, vl = batch4096
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(200)
    pg.setMixedPrecision(True, MAX_ITERS - 200)
    r = np.zeros(3 * d.n)
    res, its = D.solveBatchWith(pg, r)
    sizes = np.diff(cptr)
    single = bogus_gpu.DualFrictionProblem()
    for p in np.argsort(-sizes, kind="stable")[::16]:
        c0, c1, prp, pcl, pvl = _problem(d, cptr, rp, cl, vl, p)
        single.set(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
        rs = np.zeros(3 * (c1 - c0))
        res_s = single.solveWith(pg, rs)
        assert res[p] == res_s and its[p] == single.last_iterations, p
        assert np.array_equal(r[3 * c0:3 * c1], rs), p


# ---- the gradient workload's problem size: central differences at 20 000 contacts --------------------------
def test_adjoint_20000_contacts_matches_central_differences():
    """One problem of the gradient workload (20 000 contacts, bodies = contacts / 3, compliance 0.05, SOC law):
    dL/db, dL/dmu and dL/dH of the GPU adjoint against central differences (step 1e-6) of the forward solve, on a
    random sample of the entries whose gradient is not negligible, within 1e-5 relative (of the entry, or of 1 % of
    the largest gradient entry where the entry is smaller). Differences at step 1e-6 need the iterate to about 1e-14: APGD stops near residual 1e-15
    (iterate near 1e-8), so each solve is APGD to that floor and then Gauss-Seidel, warm started, to residual
    below 1e-24 (1200 sweeps)."""
    import bogus_gpu
    from bogus_gpu import generator

    d = generator.random_pairs(nbodies=20_000 // 3, ncontacts=20_000, seed=5 * 100003)
    n = d.n
    b0 = d.b.reshape(-1)
    D = bogus_gpu.DualFrictionProblem()
    gs = bogus_gpu.GaussSeidel()
    gs.setTol(1e-32)
    gs.setMaxIters(1200)
    gs.setEvalEvery(50)

    def forward(HA, w, mu, r0=None):
        P = bogus_gpu.PrimalFrictionProblem(d.minv, d.objA, d.objB, HA, d.HB, w, mu)
        D.computeFrom(P)
        D.add_compliance(generator.ADJOINT_COMPLIANCE)
        if r0 is None:
            pg = bogus_gpu.ProjectedGradient()
            pg.setTol(1e-30)
            pg.setMaxIters(600)
            r0 = np.zeros(3 * n)
            D.solveWith(pg, r0, staticProblem=True)
        r = r0.copy()
        res = D.solveWith(gs, r, staticProblem=True)
        assert res < 1e-24, res
        return r, P

    r, P = forward(d.HA, b0, d.mu)
    g = np.random.default_rng(6).standard_normal(3 * n)
    s, dmu = D.adjoint(r, g, tol=1e-13)
    assert D.last_adjoint_residual <= 1e-13
    dHA, _, _, _ = D.adjoint_primal(P)
    h = 1e-6
    L = lambda rr: float(g @ rr)
    rng = np.random.default_rng(11)

    def check(fd, ref, scale):
        assert abs(fd - ref) <= 1e-5 * max(abs(ref), 1e-2 * scale), (fd, ref)

    # entries are drawn where the gradient is not negligible (a separated contact's entries are exactly zero)
    for k in rng.choice(np.nonzero(np.abs(s) > 1e-3 * np.abs(s).max())[0], 8, replace=False):
        e = np.zeros(3 * n)
        e[k] = h
        fd = (L(forward(d.HA, b0 + e, d.mu, r)[0]) - L(forward(d.HA, b0 - e, d.mu, r)[0])) / (2 * h)
        check(fd, s[k], np.abs(s).max())
    for i in rng.choice(np.nonzero(np.abs(dmu) > 1e-3 * np.abs(dmu).max())[0], 4, replace=False):
        e = np.zeros(n)
        e[i] = h
        fd = (L(forward(d.HA, b0, d.mu + e, r)[0]) - L(forward(d.HA, b0, d.mu - e, r)[0])) / (2 * h)
        check(fd, dmu[i], np.abs(dmu).max())
    big = np.argwhere(np.abs(dHA) > 1e-3 * np.abs(dHA).max())
    for i, a, m in big[rng.choice(len(big), 6, replace=False)]:
        E = np.zeros_like(d.HA)
        E[i, a, m] = h
        fd = (L(forward(d.HA + E, b0, d.mu, r)[0]) - L(forward(d.HA - E, b0, d.mu, r)[0])) / (2 * h)
        check(fd, dHA[i, a, m], np.abs(dHA).max())
