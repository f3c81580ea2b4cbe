"""Edge cases of the primal solvers on the GPU against the oracle: problems without contacts (ADMM, DualAMA,
the matrix-free Gauss-Seidel, the Meche facade) and bodies without contacts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bogus_gpu

    bogus_gpu.lib()
    return bogus_gpu


def _bodies(nb=5, d=6, seed=1):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((nb, d, d)) * 0.3
    M = A @ A.transpose(0, 2, 1) + np.eye(d)[None]
    return M, np.linalg.inv(M)


def _no_contacts(bg, nb=5, d=6):
    M, minv = _bodies(nb, d)
    e = np.zeros(0, np.int32)
    H = np.zeros((0, 3, d))
    f = np.random.default_rng(2).standard_normal(nb * d)
    P = bg.PrimalFrictionProblem(minv, e, e, H, H, np.zeros(0), np.zeros(0), f=f, M=M)
    return P, M, minv, f


def test_admm_without_contacts(bg, oracle):
    P, M, minv, f = _no_contacts(bg)
    v, r = np.zeros(f.size), np.zeros(0)
    admm = bg.ADMM()
    admm.setMaxIters(20)
    res = P.solveWith(admm, 0.0, v, r)
    O = oracle.PrimalProblem(minv, np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, 3, 6)), np.zeros((0, 3, 6)))
    res_o, v_o, r_o, it_o = O.solve_admm(minv, 0.0, np.zeros(0), f, np.zeros(0), np.zeros(f.size), np.zeros(0),
                                         max_iters=20)
    assert res == res_o and np.array_equal(v, v_o)
    assert np.allclose(v, -(minv @ f.reshape(-1, 6)[..., None])[..., 0].reshape(-1), rtol=0, atol=1e-14)


def test_dual_ama_without_contacts(bg, oracle):
    P, M, minv, f = _no_contacts(bg)
    v, r = np.zeros(f.size), np.zeros(0)
    dama = bg.DualAMA()
    dama.setMaxIters(30)
    res = P.solveWith(dama, v, r)
    O = oracle.PrimalProblem(minv, np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, 3, 6)), np.zeros((0, 3, 6)))
    res_o, v_o, r_o, it_o = O.solve_dual_ama(M, np.zeros(0), f, np.zeros(0), np.zeros(f.size), np.zeros(0),
                                             max_iters=30)
    assert res == res_o and np.array_equal(v, v_o) and P.last_iterations == it_o


def test_product_gs_without_contacts(bg):
    P, M, minv, f = _no_contacts(bg)
    r = np.zeros(0)
    assert P.solveWith(bg.ProductGaussSeidel(), r) == 0.0


def test_bodies_without_contacts(bg, oracle):
    """Bodies 3 and 4 touch no contact: their velocities follow from f alone."""
    M, minv = _bodies(5)
    rng = np.random.default_rng(4)
    objA = np.array([0, 1, 2, 0], np.int32)
    objB = np.array([1, 2, -1, 2], np.int32)
    HA = rng.standard_normal((4, 3, 6))
    HB = np.where((objB < 0)[:, None, None], 0.0, rng.standard_normal((4, 3, 6)))
    w = rng.standard_normal(12)
    mu = rng.uniform(0.3, 0.8, 4)
    f = rng.standard_normal(30) * 0.1
    P = bg.PrimalFrictionProblem(minv, objA, objB, HA, HB, w, mu, f=f, M=M)
    O = oracle.PrimalProblem(minv, objA, objB, HA, HB)
    v, r = np.zeros(30), np.zeros(12)
    dama = bg.DualAMA()
    dama.setMaxIters(200)
    res = P.solveWith(dama, v, r)
    res_o, v_o, r_o, _ = O.solve_dual_ama(M, mu, f, w, np.zeros(30), np.zeros(12), max_iters=200)
    assert res == res_o and np.array_equal(v, v_o) and np.array_equal(r, r_o)
    v, r = np.zeros(30), np.zeros(12)
    admm = bg.ADMM()
    admm.setMaxIters(200)
    res = P.solveWith(admm, 0.0, v, r)
    res_o, v_o, r_o, _ = O.solve_admm(minv, 0.0, mu, f, w, np.zeros(30), np.zeros(12), max_iters=200)
    assert res == res_o and np.array_equal(v, v_o) and np.array_equal(r, r_o)


@pytest.mark.parametrize("algorithm", [0, 1, 2, 3, 4])
def test_meche_without_contacts(bg, oracle, algorithm):
    M, minv = _bodies(3, 4)
    f = np.random.default_rng(6).standard_normal(12)
    inp = dict(mass=[M[k] for k in range(3)], f=f, mu=np.zeros(0), E=np.zeros((0, 3, 3)), w=np.zeros(0),
               objA=np.zeros(0, np.int32), objB=np.zeros(0, np.int32), HA=[], HB=[])
    P = bg.MecheFrictionProblem()
    P.fromPrimal(**inp)
    o = bg.MecheOptions()
    o.algorithm = algorithm
    v = np.zeros(12)
    res = P.solve(np.zeros(0), v, o)
    O = oracle.MecheProblem(**inp)
    res_o, r_o, v_o = O.solve(np.zeros(0), algorithm=algorithm)
    assert res == res_o and np.array_equal(v, v_o)


def test_frames_rotate_w(bg, oracle):
    """PrimalFrictionProblem::E: w in world coordinates, taken to the contact basis as E^T w by the assembly and
    the primal solvers; the same as the problem posed with the rotated w."""
    from bogus_gpu import generator

    d = generator.make("c1")
    rng = np.random.default_rng(31)
    q, rr = np.linalg.qr(rng.standard_normal((d.n, 3, 3)))
    E = q * np.sign(np.einsum("nii->ni", rr))[:, None, :]
    w_world = rng.standard_normal(3 * d.n)
    w_loc = oracle.frame_t(E, w_world)
    f = rng.standard_normal(d.nbodies * 6) * 0.1
    M = np.linalg.inv(d.minv)
    PE = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, w_world, d.mu, f=f, M=M, E=E)
    PL = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, w_loc, d.mu, f=f, M=M)
    # assembly: b = E^T w - H M^-1 f
    DE, DL = bg.DualFrictionProblem(), bg.DualFrictionProblem()
    DE.computeFrom(PE)
    DL.computeFrom(PL)
    r = np.abs(rng.standard_normal(3 * d.n)) * 0.01
    pg = bg.ProjectedGradient()
    assert DE.evalWith(pg, r) == DL.evalWith(pg, r)
    # primal solvers
    for solver, args in ((bg.ADMM(), (0.0,)), (bg.DualAMA(), ()), (bg.ProductGaussSeidel(), ())):
        solver.setMaxIters(40)
        outs = []
        for P in (PE, PL):
            v, rr_ = np.zeros(d.nbodies * 6), np.zeros(3 * d.n)
            if isinstance(solver, bg.ProductGaussSeidel):
                res = P.solveWith(solver, rr_)
            elif args:
                res = P.solveWith(solver, *args, v, rr_)
            else:
                res = P.solveWith(solver, v, rr_)
            outs.append((res, v, rr_))
        assert outs[0][0] == outs[1][0] and np.array_equal(outs[0][2], outs[1][2])
        assert np.array_equal(outs[0][1], outs[1][1])


def test_destroyed_handles_return_their_device_memory(bg):
    """Handles that ran every solver family (projected gradient, Gauss-Seidel, ADMM, DualAMA, the matrix-free
    Gauss-Seidel, the adjoint) give all their device arrays back when destroyed: the free device memory after
    a few create / solve / destroy rounds is what it was after the first round."""
    import gc

    import torch
    from bogus_gpu import generator

    d = generator.make("c1")
    mass = np.linalg.inv(d.minv)

    def one_round():
        P = bg.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b, d.mu, M=mass,
                                     f=np.zeros(6 * d.nbodies))
        D = bg.DualFrictionProblem()
        D.computeFrom(P)
        r = np.zeros(3 * d.n)
        pg = bg.ProjectedGradient()
        pg.setTol(1e-10)
        D.solveWith(pg, r, staticProblem=True)
        D.solveWith(bg.GaussSeidel(), np.zeros(3 * d.n))
        D.adjoint(r, np.ones(3 * d.n), tol=1e-8)
        v = np.zeros(6 * d.nbodies)
        P.solveWith(bg.ADMM(), 0.0, v, np.zeros(3 * d.n))
        P.solveWith(bg.DualAMA(), np.zeros(6 * d.nbodies), np.zeros(3 * d.n))
        P.solveWith(bg.ProductGaussSeidel(), np.zeros(3 * d.n))
        del D, P
        gc.collect()
        torch.cuda.synchronize()

    one_round()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        one_round()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 >= free0 - (2 << 20), (free0, free1)
