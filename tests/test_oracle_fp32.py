"""The oracle's restatement of the FP32 part of the FP32-refined solve (no counterpart in the reference; the GPU
FP32 kernel is checked against it bit for bit in test_gpu_fp32_stall.py): on the 500-contact problem it makes
progress from r = 0 to the FP32 floor, its stall test ends it before a budget it cannot use, and with the test
off it runs the whole budget."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def c1_dual(oracle):
    from bogus_gpu import generator

    d = generator.make("c1")
    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    return d, oracle.DualProblem(*P.assemble(), d.b, d.mu)


@pytest.mark.parametrize("apgd", [True, False])
def test_fp32_part_stalls_before_its_budget(c1_dual, apgd):
    d, O = c1_dual
    res0 = O.eval(np.zeros(3 * d.n), coulomb=False)
    res, r, it = O.solve_pg_fp32(np.zeros(3 * d.n), apgd=apgd, tol=1e-13, max_iters=6000, stall_iters=4)
    assert 0 < it < 6000
    assert O.eval(r, coulomb=False) < 1e-3 * res0  # the FP32 part's best iterate, judged by the FP64 error function
    assert np.all(r == r.astype(np.float32))  # a float iterate widened
    _, _, it_off = O.solve_pg_fp32(np.zeros(3 * d.n), apgd=apgd, tol=1e-13, max_iters=it + 50, stall_iters=0)
    assert it_off == it + 50
