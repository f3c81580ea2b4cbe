"""DualFrictionProblem::applyPermutation / undoPermutation on the GPU: the stored problem is P W P^T, P b, P mu
(blocks moved above the diagonal stored transposed), and the solves take and return r in the caller's order.
Checked bit for bit against the oracle solving the permuted problem with r permuted in and out."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


def permuted_lower(rp, cl, vl, perm):
    """Lower triangle of P W P^T: new (k, l), k >= l, is old (perm[k], perm[l]), transposed when that lies
    above the old diagonal."""
    n = len(rp) - 1
    vl = np.asarray(vl).reshape(-1, 3, 3)
    blocks = {}
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            blocks[(i, cl[k])] = vl[k]
    inv = np.empty(n, int)
    inv[perm] = np.arange(n)
    rows = [[] for _ in range(n)]
    for (i, j), B in blocks.items():
        ni, nj = inv[i], inv[j]
        if nj > ni:
            rows[nj].append((ni, B.T))
        else:
            rows[ni].append((nj, B))
    nrp, ncl, nvl = [0], [], []
    for r in rows:
        r.sort(key=lambda t: t[0])
        ncl += [c for c, _ in r]
        nvl += [B for _, B in r]
        nrp.append(len(ncl))
    return np.array(nrp, np.int32), np.array(ncl, np.int32), np.array(nvl).reshape(-1)


@pytest.fixture(scope="module")
def problem():
    from bogus_gpu import generator
    import bogus_gpu

    d = generator.make("c1")
    D = bogus_gpu.DualFrictionProblem()
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    rp, cl, vl = D.W_lower()
    perm = np.random.default_rng(12).permutation(d.n).astype(np.int32)
    return d, rp, cl, np.asarray(vl).reshape(-1), perm


def test_permuted_solves_bitwise(bg, oracle, problem):
    d, rp, cl, vl, perm = problem
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    D.applyPermutation(perm)
    assert D.permuted()
    prp, pcl, pvl = permuted_lower(rp, cl, vl, perm)
    grp, gcl, gvl = D.W_lower()
    assert np.array_equal(grp, prp) and np.array_equal(gcl, pcl) and np.array_equal(gvl.reshape(-1), pvl)
    pb = d.b.reshape(-1, 3)[perm].reshape(-1)
    O = oracle.DualProblem(prp, pcl, pvl, pb, d.mu[perm])
    r0 = np.abs(np.random.default_rng(3).standard_normal(3 * d.n)) * 0.01
    r0p = r0.reshape(-1, 3)[perm].reshape(-1)
    # Gauss-Seidel (Coulomb) and projected gradient (SOC), r in the caller's order
    gs = bg.GaussSeidel()
    gs.setMaxIters(50)
    r = r0.copy()
    res = D.solveWith(gs, r)
    res_o, r_o, _ = O.solve_gs(r0p, max_iters=50, coloring=False)
    back = np.empty_like(r_o.reshape(-1, 3))
    back[perm] = r_o.reshape(-1, 3)
    assert res == res_o and np.array_equal(r, back.reshape(-1))
    pg = bg.ProjectedGradient()
    pg.setMaxIters(100)
    r = r0.copy()
    res = D.solveWith(pg, r)
    res_o, r_o, _ = O.solve_pg(r0p, max_iters=100)
    back[perm] = r_o.reshape(-1, 3)
    assert res == res_o and np.array_equal(r, back.reshape(-1))
    # evalWith at the caller's r equals the error of the permuted problem at the permuted r
    assert D.evalWith(pg, r) == O.eval(r.reshape(-1, 3)[perm].reshape(-1), coulomb=False)
    # undo: the original problem, solved as before the permutation
    D.undoPermutation()
    assert not D.permuted()
    grp, gcl, gvl = D.W_lower()
    assert np.array_equal(grp, rp) and np.array_equal(gcl, cl) and np.array_equal(gvl.reshape(-1), vl)
    E = bg.DualFrictionProblem()
    E.set(rp, cl, vl, d.b, d.mu)
    r1, r2 = r0.copy(), r0.copy()
    assert D.solveWith(gs, r1) == E.solveWith(gs, r2) and np.array_equal(r1, r2)


def test_permutation_rejections(bg, problem):
    d, rp, cl, vl, perm = problem
    D = bg.DualFrictionProblem()
    D.set(rp, cl, vl, d.b, d.mu)
    bad = perm.copy()
    bad[0] = bad[1]
    with pytest.raises(bg.BogusGpuError):
        D.applyPermutation(bad)
    D.applyPermutation(perm)
    with pytest.raises(bg.BogusGpuError):  # already permuted
        D.applyPermutation(perm)
    D.set(rp, cl, vl, d.b, d.mu)  # a new problem clears the permutation
    assert not D.permuted()
