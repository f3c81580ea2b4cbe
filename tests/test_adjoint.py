"""Adjoint of the SOC friction solve: the dense implicit-function oracle against central finite differences of
the oracle's forward solve (CPU), and the GPU adjoint against the dense oracle (GPU).

The reference has no differentiation, so the gradient is pinned by finite differences: the forward solve is
the oracle's Gauss-Seidel with the SOC law run to residual 1e-30 (APGD stalls near 1e-16 on these problems),
differences are central with step 1e-6, and the problems carry a compliance term (W + 0.05 I) so that the
solution is unique and differentiable.
"""
import numpy as np
import pytest

EPS_COMPLIANCE = 0.05
FD_STEP = 1e-6


def _lower_to_dense(rp, cl, vl, n):
    W = np.zeros((3 * n, 3 * n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            j = cl[k]
            B = vl[9 * k:9 * k + 9].reshape(3, 3)
            W[3 * i:3 * i + 3, 3 * j:3 * j + 3] = B
            if i != j:
                W[3 * j:3 * j + 3, 3 * i:3 * i + 3] = B.T
    return W


class Problem:
    """A random-pairs problem (300 contacts, 150 bodies) with compliance, solved tightly by the oracle."""

    def __init__(self, oracle, n=300, nb=150, seed=7):
        from bogus_gpu import generator

        self.oracle = oracle
        self.d = generator.random_pairs(nbodies=nb, ncontacts=n, seed=seed)
        self.n = n
        rng = np.random.default_rng(seed + 1)
        self.f = rng.standard_normal(nb * 6) * 0.1
        self.w = self.d.b.reshape(-1).copy()
        self.mu = self.d.mu.copy()
        self.g = rng.standard_normal(3 * n)
        self.rp, self.cl, self.vl, self.b = self.assemble(self.d.HA, self.d.HB, self.w, self.f)
        self.W = _lower_to_dense(self.rp, self.cl, self.vl, n)
        self.r = self.solve(self.b, self.mu)

    def assemble(self, HA, HB, w, f):
        P = self.oracle.PrimalProblem(self.d.minv, self.d.objA, self.d.objB, HA, HB)
        rp, cl, vl = P.assemble()
        vl = vl.copy()
        for i in range(self.n):
            k = rp[i + 1] - 1
            for e in (0, 4, 8):
                vl[9 * k + e] += EPS_COMPLIANCE
        return rp, cl, vl, P.rhs(f, w)

    def solve(self, b, mu, lower=None, coulomb=False):
        rp, cl, vl = lower if lower is not None else (self.rp, self.cl, self.vl)
        O = self.oracle.DualProblem(rp, cl, vl, b, mu)
        res, r, _ = O.solve_gs(np.zeros(3 * self.n), coulomb=coulomb, tol=1e-34, max_iters=5000 if coulomb else 3000,
                               coloring=False)
        assert res < 1e-26
        return r

    def loss(self, r):
        return float(self.g @ r)


@pytest.fixture(scope="module")
def prob(oracle):
    return Problem(oracle)


@pytest.fixture(scope="module")
def prob_coulomb(prob):
    """The same problem under the Coulomb law (De Saxce fixed point), solved by Gauss-Seidel to the FP64 floor."""
    prob.rc = prob.solve(prob.b, prob.mu, coulomb=True)
    return prob


@pytest.fixture(scope="module")
def adj():
    import adjoint  # oracle/adjoint.py (the oracle directory is on sys.path, see conftest.py)

    return adjoint


def test_projection_jacobian_matches_differences(adj):
    rng = np.random.default_rng(0)
    h = 1e-7
    seen = set()
    for _ in range(300):
        mu = rng.uniform(0.2, 1.0)
        x = rng.standard_normal(3)
        J, K = adj.projection_jacobian(mu, x)
        seen.add("I" if np.array_equal(J, np.eye(3)) else ("0" if not J.any() else "B"))
        Jfd = np.stack([(adj.project(mu, x + h * e) - adj.project(mu, x - h * e)) / (2 * h) for e in np.eye(3)], 1)
        Kfd = (adj.project(mu + h, x) - adj.project(mu - h, x)) / (2 * h)
        assert np.allclose(J, Jfd, atol=1e-6) and np.allclose(K, Kfd, atol=1e-6)
        assert np.allclose(J, J.T)
    assert seen == {"I", "0", "B"}


def test_dense_gradient_matches_finite_differences(adj, prob):
    """dL/db, dL/dmu, dL/dHA, dL/dw, dL/df of the dense oracle against central differences (1e-5)."""
    s, dmu, _ = adj.implicit_gradient(prob.W, prob.b, prob.mu, prob.r, prob.g)
    d = prob.d
    dHA, dHB, dw, df = adj.primal_gradients(s, prob.r, d.minv, d.objA, d.objB, d.HA, d.HB, prob.f)
    rng = np.random.default_rng(5)
    h = FD_STEP

    def fd(fn):
        return (prob.loss(fn(+h)) - prob.loss(fn(-h))) / (2 * h)

    for k in rng.choice(3 * prob.n, 4, replace=False):
        e = np.zeros(3 * prob.n)
        e[k] = 1
        assert abs(fd(lambda t: prob.solve(prob.b + t * e, prob.mu)) - s[k]) <= 1e-5 * max(1.0, abs(s[k]))
    for i in rng.choice(prob.n, 3, replace=False):
        e = np.zeros(prob.n)
        e[i] = 1
        assert abs(fd(lambda t: prob.solve(prob.b, prob.mu + t * e)) - dmu[i]) <= 1e-5 * max(1.0, abs(dmu[i]))

    def primal_fd(HA=None, HB=None, w=None, f=None):
        rp, cl, vl, b = prob.assemble(d.HA if HA is None else HA, d.HB if HB is None else HB,
                                      prob.w if w is None else w, prob.f if f is None else f)
        return prob.solve(b, prob.mu, (rp, cl, vl))

    for _ in range(3):
        i, a, m = rng.integers(prob.n), rng.integers(3), rng.integers(6)
        E = np.zeros_like(d.HA)
        E[i, a, m] = 1
        assert abs(fd(lambda t: primal_fd(HA=d.HA + t * E)) - dHA[i, a, m]) <= 1e-5 * max(1.0, abs(dHA[i, a, m]))
    k = rng.integers(3 * prob.n)
    e = np.zeros(3 * prob.n)
    e[k] = 1
    assert abs(fd(lambda t: primal_fd(w=prob.w + t * e)) - dw[k]) <= 1e-5 * max(1.0, abs(dw[k]))
    k = rng.integers(prob.f.size)
    e = np.zeros(prob.f.size)
    e[k] = 1
    assert abs(fd(lambda t: primal_fd(f=prob.f + t * e)) - df[k]) <= 1e-5 * max(1.0, abs(df[k]))


def test_dense_coulomb_gradient_matches_finite_differences(adj, prob_coulomb):
    """The Coulomb problem: dL/db, dL/dmu and dL/dHA of the dense oracle (with the De Saxce term) against central
    differences of the oracle's Coulomb Gauss-Seidel solve (1e-5), and independent of the fixed-point step."""
    prob = prob_coulomb
    s, dmu, _ = adj.implicit_gradient(prob.W, prob.b, prob.mu, prob.rc, prob.g, coulomb=True)
    s2, dmu2, _ = adj.implicit_gradient(prob.W, prob.b, prob.mu, prob.rc, prob.g, alpha=0.37, coulomb=True)
    assert np.abs(s - s2).max() <= 1e-10 * np.abs(s).max() and np.abs(dmu - dmu2).max() <= 1e-10 * np.abs(dmu).max()
    d = prob.d
    dHA, dHB, dw, df = adj.primal_gradients(s, prob.rc, d.minv, d.objA, d.objB, d.HA, d.HB, prob.f)
    rng = np.random.default_rng(15)
    h = FD_STEP

    def fd(fn):
        return (prob.loss(fn(+h)) - prob.loss(fn(-h))) / (2 * h)

    nonzero_b = np.nonzero(np.abs(s) > 1e-3 * np.abs(s).max())[0]
    for k in rng.choice(nonzero_b, 4, replace=False):
        e = np.zeros(3 * prob.n)
        e[k] = 1
        assert abs(fd(lambda t: prob.solve(prob.b + t * e, prob.mu, coulomb=True)) - s[k]) <= 1e-5 * max(1.0, abs(s[k]))
    nonzero_mu = np.nonzero(np.abs(dmu) > 1e-3 * np.abs(dmu).max())[0]
    for i in rng.choice(nonzero_mu, 3, replace=False):
        e = np.zeros(prob.n)
        e[i] = 1
        got = fd(lambda t: prob.solve(prob.b, prob.mu + t * e, coulomb=True))
        assert abs(got - dmu[i]) <= 1e-5 * max(1.0, abs(dmu[i]))
    for _ in range(2):
        i, a, m = rng.integers(prob.n), rng.integers(3), rng.integers(6)
        E = np.zeros_like(d.HA)
        E[i, a, m] = 1

        def primal(t):
            rp, cl, vl, b = prob.assemble(d.HA + t * E, d.HB, prob.w, prob.f)
            return prob.solve(b, prob.mu, (rp, cl, vl), coulomb=True)

        assert abs(fd(primal) - dHA[i, a, m]) <= 1e-5 * max(1.0, abs(dHA[i, a, m]))


# ---- GPU adjoint ---------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def gpu_prob(prob):
    import bogus_gpu

    d = prob.d
    P = bogus_gpu.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, prob.w, prob.mu, f=prob.f)
    D = bogus_gpu.DualFrictionProblem()
    D.computeFrom(P)
    D.add_compliance(EPS_COMPLIANCE)
    return D, P


@pytest.mark.gpu
def test_gpu_adjoint_matches_dense_oracle(adj, prob, gpu_prob):
    D, P = gpu_prob
    rp, cl, vl = D.W_lower()
    assert np.array_equal(vl.reshape(-1), prob.vl)  # the GPU assembly + compliance is the oracle's W
    s_o, dmu_o, dW_o = adj.implicit_gradient(prob.W, prob.b, prob.mu, prob.r, prob.g)
    s, dmu = D.adjoint(prob.r, prob.g, tol=1e-13)
    assert D.last_adjoint_residual <= 1e-13
    scale = np.abs(s_o).max()
    assert np.abs(s - s_o).max() <= 1e-8 * scale
    assert np.abs(dmu - dmu_o).max() <= 1e-8 * max(1.0, np.abs(dmu_o).max())
    # dL/dW on the stored lower blocks: G_ij + G_ji^T off the diagonal
    G = D.adjoint_dual_lower()
    for i in range(prob.n):
        for k in range(rp[i], rp[i + 1]):
            j = cl[k]
            ref = dW_o[3 * i:3 * i + 3, 3 * j:3 * j + 3] + (dW_o[3 * j:3 * j + 3, 3 * i:3 * i + 3].T if i != j else 0)
            assert np.allclose(G[k], ref, rtol=0, atol=1e-8 * scale * np.abs(prob.r).max() + 1e-300)
    d = prob.d
    dHA, dHB, dw, df = D.adjoint_primal(P)
    rHA, rHB, rw, rf = adj.primal_gradients(s_o, prob.r, d.minv, d.objA, d.objB, d.HA, d.HB, prob.f)
    for got, ref in ((dHA, rHA), (dHB, rHB), (dw, rw), (df, rf)):
        assert np.abs(got - ref).max() <= 1e-7 * max(1.0, np.abs(ref).max())


@pytest.mark.gpu
def test_gpu_coulomb_adjoint_matches_dense_oracle(adj, prob_coulomb, gpu_prob):
    """The Coulomb adjoint (bi-conjugate gradients stabilised on the De Saxce linearisation) against the dense
    oracle: dL/db, dL/dmu and the primal gradients within 1e-8 relative."""
    prob = prob_coulomb
    D, P = gpu_prob
    s_o, dmu_o, _ = adj.implicit_gradient(prob.W, prob.b, prob.mu, prob.rc, prob.g, coulomb=True)
    s, dmu = D.adjoint(prob.rc, prob.g, tol=1e-13, coulomb=True)
    assert D.last_adjoint_residual <= 1e-13
    scale = np.abs(s_o).max()
    assert np.abs(s - s_o).max() <= 1e-8 * scale
    assert np.abs(dmu - dmu_o).max() <= 1e-8 * max(1.0, np.abs(dmu_o).max())
    d = prob.d
    dHA, dHB, dw, df = D.adjoint_primal(P)
    rHA, rHB, rw, rf = adj.primal_gradients(s_o, prob.rc, d.minv, d.objA, d.objB, d.HA, d.HB, prob.f)
    for got, ref in ((dHA, rHA), (dHB, rHB), (dw, rw), (df, rf)):
        assert np.abs(got - ref).max() <= 1e-7 * max(1.0, np.abs(ref).max())


@pytest.mark.gpu
def test_gpu_adjoint_is_linear_in_the_loss(prob, gpu_prob):
    D, _ = gpu_prob
    rng = np.random.default_rng(9)
    g1, g2 = rng.standard_normal(3 * prob.n), rng.standard_normal(3 * prob.n)
    s1, m1 = D.adjoint(prob.r, g1, tol=1e-13)
    s2, m2 = D.adjoint(prob.r, g2, tol=1e-13)
    s3, m3 = D.adjoint(prob.r, 2.0 * g1 - 3.0 * g2, tol=1e-13)
    assert np.allclose(s3, 2.0 * s1 - 3.0 * s2, rtol=0, atol=1e-9 * np.abs(s3).max())
    assert np.allclose(m3, 2.0 * m1 - 3.0 * m2, rtol=0, atol=1e-9 * max(1.0, np.abs(m3).max()))


@pytest.mark.gpu
def test_torch_gradcheck_small_problem():
    """torch.autograd.gradcheck of friction_solve (forward: GPU Gauss-Seidel with the SOC law to the FP64
    floor, backward: the GPU adjoint) with respect to w, mu and f on 12 contacts / 8 bodies."""
    torch = pytest.importorskip("torch")
    from bogus_gpu import generator
    from bogus_gpu.autograd import friction_solve

    d = generator.random_pairs(nbodies=8, ncontacts=12, seed=3)
    rng = np.random.default_rng(4)
    HA = torch.tensor(d.HA)
    HB = torch.tensor(d.HB)
    w = torch.tensor(d.b.reshape(-1), requires_grad=True)
    mu = torch.tensor(d.mu, requires_grad=True)
    f = torch.tensor(rng.standard_normal(8 * 6) * 0.1, requires_grad=True)
    gw = torch.tensor(rng.standard_normal(36))

    def fn(w_, mu_, f_):
        r = friction_solve(HA, HB, w_, mu_, f_, minv=d.minv, objA=d.objA, objB=d.objB, compliance=EPS_COMPLIANCE)
        return (gw * r).sum()

    assert torch.autograd.gradcheck(fn, (w, mu, f), eps=1e-6, atol=1e-6, rtol=1e-5)
    # H through the same path, a few entries against central differences
    HAg = HA.clone().requires_grad_(True)
    L = (gw * friction_solve(HAg, HB, w.detach(), mu.detach(), f.detach(), minv=d.minv, objA=d.objA, objB=d.objB,
                              compliance=EPS_COMPLIANCE)).sum()
    L.backward()
    for (i, a, m) in [(0, 0, 0), (3, 1, 4), (7, 2, 5)]:
        E = torch.zeros_like(HA)
        E[i, a, m] = 1e-6
        Lp = (gw * friction_solve(HA + E, HB, w.detach(), mu.detach(), f.detach(), minv=d.minv, objA=d.objA,
                                  objB=d.objB, compliance=EPS_COMPLIANCE)).sum()
        Lm = (gw * friction_solve(HA - E, HB, w.detach(), mu.detach(), f.detach(), minv=d.minv, objA=d.objA,
                                  objB=d.objB, compliance=EPS_COMPLIANCE)).sum()
        fd = float((Lp - Lm) / 2e-6)
        assert abs(fd - float(HAg.grad[i, a, m])) <= 1e-5 * max(1.0, abs(fd))
