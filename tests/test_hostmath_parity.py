"""The library's per-contact device mathematics (csrc/soc_device.cuh, compiled here for the host) against the
CPU oracle: bit-identical on random local problems, including the reference's edge cases (take-off,
frictionless, mu < 0, singular diagonal blocks, zero vectors)."""
import numpy as np
import pytest


def _random_local(rng, k):
    """SPD-ish 3x3 blocks (some singular), right-hand sides spanning take-off / stick / slide."""
    out = []
    for t in range(k):
        G = rng.standard_normal((3, 3))
        A = G @ G.T
        if t % 17 == 0:
            A = np.outer(G[0], G[0])  # rank one
        if t % 23 == 0:
            A = np.zeros((3, 3))
        b = rng.standard_normal(3)
        if t % 5 == 0:
            b[0] = abs(b[0])  # take-off
        mu = rng.uniform(0.1, 1.0)
        if t % 13 == 0:
            mu = 0.0
        if t % 29 == 0:
            mu = -1.0
        x0 = rng.standard_normal(3) if t % 3 else np.zeros(3)
        out.append((A, b, mu, x0, rng.uniform(1.0, 3.0)))
    return out


def _same(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.array_equal(a, b) or np.array_equal(np.nan_to_num(a, nan=7.0), np.nan_to_num(b, nan=7.0))


@pytest.mark.parametrize("coulomb", [True, False])
@pytest.mark.parametrize("strategy", [0, 1, 2, 3])
def test_local_solver_bitwise(oracle, hostmath, coulomb, strategy):
    rng = np.random.default_rng(100 + 10 * strategy + int(coulomb))
    for A, b, mu, x0, sc in _random_local(rng, 400):
        res_o, x_o = oracle.local_solve(A, b, x0, mu, coulomb=coulomb, strategy=strategy, scaling=sc)
        x_h = x0.copy()
        res_h = hostmath.hm_local_solve(int(coulomb), strategy, A.reshape(-1).copy(), b.copy(), x_h, mu,
                                        1.8189894035458565e-12, sc)
        assert _same(res_o, res_h), (A, b, mu, x0)
        assert _same(x_o, x_h), (A, b, mu, x0)


def test_law_eval_projection_roots_bitwise(oracle, hostmath):
    rng = np.random.default_rng(7)
    for t in range(2000):
        mu = [0.0, -0.5, rng.uniform(0.05, 2.0)][t % 3]
        x = rng.standard_normal(3) * (0 if t % 11 == 0 else 1)
        y = rng.standard_normal(3)
        for coulomb in (True, False):
            assert _same(oracle.law_eval(mu, x, y, coulomb), hostmath.hm_law_eval(int(coulomb), mu, x, y))
        xp = x.copy()
        hostmath.hm_project(mu, xp)
        assert _same(oracle.project(mu, x), xp)
    for t in range(500):
        dim = [2, 3, 4][t % 3]
        c = rng.standard_normal(dim + 1)
        if t % 7 == 0:
            c[-1] = 0.0
        for deg in (0, 1):
            cc = c if deg else c[:dim]
            ro = oracle.real_roots(cc, degenerate=bool(deg), filt=t % 3)
            rh = np.zeros(4)
            nh = hostmath.hm_real_roots(np.ascontiguousarray(cc), dim, deg, t % 3, rh)
            assert len(ro) == nh
            assert _same(ro, rh[:nh])


def test_fb_jacobian_bitwise(oracle, hostmath):
    import ctypes as C

    L = oracle.lib()
    rng = np.random.default_rng(11)
    for t in range(1000):
        A = rng.standard_normal((3, 3))
        A = A @ A.T
        b = rng.standard_normal(3)
        x = rng.standard_normal(3) if t % 9 else np.zeros(3)
        mu = [0.0, rng.uniform(0.1, 1.0)][t % 2]
        for coulomb in (0, 1):
            fo, jo = np.zeros(3), np.zeros(9)
            L.oracle_fb_jacobian(coulomb, mu, 1.5, A.reshape(-1).copy(), b, x, fo, jo)
            fh, jh = np.zeros(3), np.zeros(9)
            hostmath.hm_fb_jacobian(coulomb, mu, 1.5, A.reshape(-1).copy(), b, x, fh, jh)
            assert _same(fo, fh) and _same(jo, jh)
    del C
