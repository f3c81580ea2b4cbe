"""The oracle's APGD with FP32 correction products (no counterpart in the reference; the GPU form is checked
against it bit for bit in test_gpu_fp32_products.py): W v = W x_ref + W32 (v - x_ref)_32, x_ref refreshed at
the first momentum step on or after every hy_refresh iterations. On the 500-contact problem it reaches the
tolerance of the FP64 solve with the reported residual equal to the exact error function up to the products'
rounding; a refresh interval too long for the tolerance stalls above it, and the solve stops on the 1 %-in-10-
intervals rule instead of running its budget."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def c1_dual(oracle):
    from bogus_gpu import generator

    d = generator.make("c1")
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    return d, oracle.DualProblem(*P.assemble(), d.b, d.mu)


@pytest.mark.parametrize("coulomb", [False, True])
@pytest.mark.parametrize("refresh", [7, 50])
def test_correction_products_reach_the_tolerance(c1_dual, coulomb, refresh):
    d, O = c1_dual
    res_ref, r_ref, it_ref = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=coulomb, tol=1e-8, max_iters=3000)
    res, r, it = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=coulomb, tol=1e-8, max_iters=3000,
                            hy_refresh=refresh)
    assert res_ref < 1e-8 and res < 1e-8 and it < 3000
    # the reported residual comes from the corrected products: the exact error function differs by their rounding
    assert abs(res - O.eval(r, coulomb=coulomb)) <= 1e-3 * res
    assert np.linalg.norm(r - r_ref) <= 1e-3 * np.linalg.norm(r_ref)


def test_long_refresh_interval_stops_on_the_stall_rule(c1_dual):
    d, O = c1_dual
    budget = 40000
    res, r, it = O.solve_pg(np.zeros(3 * d.n), variant=3, tol=1e-16, max_iters=budget, hy_refresh=1000)
    assert 10000 <= it < budget


def test_zero_refresh_is_the_fp64_solve(c1_dual):
    d, O = c1_dual
    a = O.solve_pg(np.zeros(3 * d.n), variant=3, tol=1e-8, max_iters=400)
    b = O.solve_pg(np.zeros(3 * d.n), variant=3, tol=1e-8, max_iters=400, hy_refresh=0)
    assert a[0] == b[0] and a[2] == b[2] and np.array_equal(a[1], b[1])
