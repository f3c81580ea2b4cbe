"""The oracle's APGD variant with the momentum product formed by linearity (no counterpart in the reference):
same method, other rounding. On the 500-contact problem it converges like the reference's form, with iterates
that differ by rounding only; the variants without a momentum product ignore the option. The residual a solve
reports is evaluated with the product it carries (formed by linearity after a momentum step), so it equals the
error function recomputed at the returned iterate up to rounding, not bit for bit."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def c1_dual(oracle):
    from bogus_gpu import generator

    d = generator.make("c1")
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    return d, oracle.DualProblem(*P.assemble(), d.b, d.mu)


@pytest.mark.parametrize("coulomb", [False, True])
def test_lin_momentum_converges_like_the_reference_form(c1_dual, coulomb):
    d, O = c1_dual
    res_ref, r_ref, it_ref = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=coulomb, tol=1e-8, max_iters=2000)
    res, r, it = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=coulomb, tol=1e-8, max_iters=2000,
                            lin_momentum=True)
    assert res < 1e-8 and res_ref < 1e-8
    assert abs(int(it) - int(it_ref)) <= 5
    assert np.linalg.norm(r - r_ref) <= 1e-10 * np.linalg.norm(r_ref)
    # the reported residual is evaluated with the product formed by linearity: the error function recomputed at
    # the returned iterate differs from it by rounding only
    assert abs(res - O.eval(r, coulomb=coulomb)) <= 1e-9 * res


@pytest.mark.parametrize("variant", [1, 4])  # Descent, SPG
def test_lin_momentum_ignored_without_momentum_product(c1_dual, variant):
    d, O = c1_dual
    a = O.solve_pg(np.zeros(3 * d.n), variant=variant, tol=1e-8, max_iters=300)
    b = O.solve_pg(np.zeros(3 * d.n), variant=variant, tol=1e-8, max_iters=300, lin_momentum=True)
    assert a[0] == b[0] and a[2] == b[2] and np.array_equal(a[1], b[1])
