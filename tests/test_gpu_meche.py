"""GPU MecheFrictionProblem facade (fromPrimal / solve) against the oracle's restatement of it.

Both follow the same evaluation order (frames, Jacobian rotation, mass inverses, assembly, solvers, velocity
recovery), so r, v and the residual are bit-identical. The oracle facade itself is pinned on the reference's
SmallFrictionPb solution in world coordinates (test_oracle_golden.py).
"""
import numpy as np
import pytest

from test_oracle_golden import small_friction_world

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


def random_world_problem():
    """The 500-contact random-pairs problem posed in world coordinates: random contact frames E_i, world
    Jacobians E_i H_A and -E_i H_B, masses from the inverse-mass blocks, a random f."""
    from bogus_gpu import generator

    d = generator.make("c1")
    rng = np.random.default_rng(21)
    q, rr = np.linalg.qr(rng.standard_normal((d.n, 3, 3)))
    E = q * np.sign(np.einsum("nii->ni", rr))[:, None, :]
    mass = [np.linalg.inv(m) for m in d.minv]
    HA = [E[i] @ d.HA[i] for i in range(d.n)]
    HB = [None if d.objB[i] < 0 else -(E[i] @ d.HB[i]) for i in range(d.n)]
    w = np.concatenate([E[i] @ d.b[i] for i in range(d.n)])
    f = rng.standard_normal(6 * d.nbodies) * 0.1
    return dict(mass=mass, f=f, mu=d.mu, E=E, w=w, objA=d.objA, objB=d.objB, HA=HA, HB=HB)


def run_pair(bg, oracle, inp, r0, with_v=True, static=False, regularization=0.0, v0=None, **opts):
    M = bg.MecheFrictionProblem()
    M.fromPrimal(**inp)
    o = bg.MecheOptions()
    names = {"max_threads": "maxThreads", "max_iters": "maxIters", "cadoux_iters": "cadouxIters",
             "tolerance": "tolerance", "algorithm": "algorithm", "gs_coloring": "gsColoring",
             "pg_variant": "pgVariant", "admm_step": "admmProjStepSize", "admm_fp_step": "admmFpStepSize",
             "inf_norm": "useInfinityNorm",
             "gs_regularization": "gsRegularization", "try_zero": "tryZeroAsWell"}
    for k, val in opts.items():
        setattr(o, names[k], val)
    r = r0.copy()
    v = None
    if with_v:
        v = np.zeros(M.nDegreesOfFreedom()) if v0 is None else v0.copy()
    res = M.solve(r, v, o, staticProblem=static, problemRegularization=regularization)
    O = oracle.MecheProblem(**inp)
    res_o, r_o, v_o = O.solve(r0, with_v=with_v, static=static, regularization=regularization, v=v0, **opts)
    return (res, r, v), (res_o, r_o, v_o)


def assert_same(g, o):
    assert g[0] == o[0]
    assert np.array_equal(g[1], o[1])
    if g[2] is not None:
        assert np.array_equal(g[2], o[2])


@pytest.mark.parametrize("algorithm, extra", [
    (0, {}),                                    # Gauss-Seidel, Coulomb
    (1, {"pg_variant": 3}),                     # projected gradient (APGD)
    (1, {"pg_variant": 0}),                     # projected gradient (Standard)
    (1, {"pg_variant": 2, "cadoux_iters": 5}),  # projected gradient (Conjugated) + Cadoux
    (1, {"cadoux_iters": 8}),                   # projected gradient (SPG, the facade's default) + Cadoux
    (0, {"cadoux_iters": 5}),                   # Gauss-Seidel + Cadoux
    (2, {}),                                    # matrix-free Gauss-Seidel
])
def test_small_friction_world_bitwise(bg, oracle, algorithm, extra):
    _, inp = small_friction_world()
    g, o = run_pair(bg, oracle, inp, np.zeros(6), algorithm=algorithm, tolerance=1e-10, max_iters=500, **extra)
    assert_same(g, o)


def test_small_friction_world_admm_bitwise(bg, oracle):
    _, inp = small_friction_world()
    g, o = run_pair(bg, oracle, inp, np.zeros(6), static=True, algorithm=3, tolerance=1e-9, max_iters=2000,
                    admm_step=1e-2)
    assert_same(g, o)
    assert g[0] < 1e-9


@pytest.mark.parametrize("static, with_v", [(True, True), (False, False)])
def test_small_friction_world_dual_ama_bitwise(bg, oracle, static, with_v):
    """Algorithm DualAMA (MecheInterface.cpp:249-261): no line search, the facade's two step sizes."""
    _, inp = small_friction_world()
    g, o = run_pair(bg, oracle, inp, np.zeros(6), with_v=with_v, static=static, algorithm=4, tolerance=1e-12,
                    max_iters=3000, admm_step=1e-2, admm_fp_step=1e-1)
    assert_same(g, o)


@pytest.mark.parametrize("case", ["gs", "gs_colored_regularized", "pg_static", "gs_cadoux", "admm_v0", "matrix_free",
                                  "dual_ama"])
def test_random_world_problem_bitwise(bg, oracle, case):
    inp = random_world_problem()
    n = len(inp["objA"])
    r0 = np.random.default_rng(5).standard_normal(3 * n) * 0.01
    if case == "gs":
        g, o = run_pair(bg, oracle, inp, r0, algorithm=0, tolerance=1e-8, max_iters=100)
    elif case == "gs_colored_regularized":
        g, o = run_pair(bg, oracle, inp, r0, algorithm=0, tolerance=1e-8, max_iters=100, max_threads=0,
                        gs_coloring=True, gs_regularization=1e-3, regularization=1e-2)
    elif case == "pg_static":
        g, o = run_pair(bg, oracle, inp, r0, static=True, algorithm=1, pg_variant=3, tolerance=1e-8,
                        max_iters=300, inf_norm=True)
    elif case == "matrix_free":
        g, o = run_pair(bg, oracle, inp, r0, algorithm=2, tolerance=1e-8, max_iters=75, gs_regularization=1e-3)
    elif case == "dual_ama":
        g, o = run_pair(bg, oracle, inp, r0, algorithm=4, tolerance=1e-10, max_iters=150, admm_step=1e-2,
                        admm_fp_step=1e-1)
    elif case == "gs_cadoux":
        g, o = run_pair(bg, oracle, inp, r0, algorithm=0, cadoux_iters=4, tolerance=1e-8, max_iters=60)
    else:
        v0 = np.random.default_rng(6).standard_normal(6 * (len(inp["mass"]))) * 0.01
        g, o = run_pair(bg, oracle, inp, r0, static=True, algorithm=3, tolerance=1e-10, max_iters=150,
                        admm_step=1e-2, v0=v0)
    assert_same(g, o)


def test_meche_rejects_unknown_algorithms_and_singular_mass(bg):
    _, inp = small_friction_world()
    M = bg.MecheFrictionProblem()
    M.fromPrimal(**inp)
    for alg in (-1, 5):
        o = bg.MecheOptions()
        o.algorithm = alg
        with pytest.raises(bg.BogusGpuError):
            M.solve(np.zeros(6), None, o)
    bad = dict(inp)
    bad["mass"] = [np.zeros((4, 4)), inp["mass"][1]]
    with pytest.raises(bg.BogusGpuError):
        bg.MecheFrictionProblem().fromPrimal(**bad)
