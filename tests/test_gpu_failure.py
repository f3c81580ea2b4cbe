"""Failure handling on the GPU, without faulting it: a bounded device-side wait that runs out, and malformed
problems handed over in device memory.

* The timeout path: bogus_gpu_test_wait_timeout makes the persistent projected-gradient kernel wait at its first
  barrier for one CTA more than the launch holds (a count that nothing completes). With a short wait limit
  (bogus_gpu_set_wait_limit) the wait runs out, every CTA returns, the solve reports BOGUS_GPU_TIMEOUT and leaves
  r untouched; the same handle then solves normally, bit for bit like the oracle.
* bogus_gpu_set_dual_device checks the caller's device arrays before copying them: malformed row pointers,
  columns out of range or out of order, a missing diagonal block (BAD_INPUT) and non-finite values (NONFINITE)
  are rejected and the handle keeps the problem it had.
"""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1(oracle):
    import bogus_gpu
    from bogus_gpu import generator

    bogus_gpu.lib()
    d = generator.make("c1")
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    rp, cl, vl = D.W_lower()
    O = oracle.DualProblem(rp, cl, vl.reshape(-1), d.b, d.mu)
    return d, D, O


def test_wait_timeout_then_solve_on_the_same_handle(c1):
    import bogus_gpu

    L = bogus_gpu.lib()
    d, D, O = c1
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(1e-8)
    opts = pg.options(False)
    try:
        assert L.bogus_gpu_set_wait_limit(0, 0.05) == bogus_gpu.OK
        assert L.bogus_gpu_test_wait_timeout(D.handle, 1) == bogus_gpu.OK
        r = np.full(3 * d.n, 0.25)
        res, it = C.c_double(-1.0), C.c_uint(7)
        t0 = time.perf_counter()
        st = L.bogus_gpu_solve_pg(D.handle, C.byref(opts), r, C.byref(res), C.byref(it))
        elapsed = time.perf_counter() - t0
        assert st == bogus_gpu.TIMEOUT, L.bogus_gpu_last_error()
        assert b"timed out" in L.bogus_gpu_last_error()
        assert elapsed < 2.0  # the 0.05 s limit, not the 4 s default
        assert np.all(r == 0.25)  # r untouched
    finally:
        L.bogus_gpu_test_wait_timeout(D.handle, 0)
        assert L.bogus_gpu_set_wait_limit(0, 4.0) == bogus_gpu.OK
    # the context and the handle are still usable: the same solve, bit for bit like the oracle
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r, staticProblem=False)
    res_o, r_o, it_o = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=True, tol=1e-8)
    assert res == res_o and np.array_equal(r, r_o) and D.last_iterations == it_o


def test_wait_limit_rejects_bad_values():
    import bogus_gpu

    L = bogus_gpu.lib()
    assert L.bogus_gpu_set_wait_limit(0, 0.0) == bogus_gpu.BAD_INPUT
    assert L.bogus_gpu_set_wait_limit(0, float("nan")) == bogus_gpu.BAD_INPUT
    assert L.bogus_gpu_set_wait_limit(0, 1e9) == bogus_gpu.BAD_INPUT
    assert L.bogus_gpu_set_wait_limit(99, 1.0) == bogus_gpu.NO_DEVICE


def _device_full(torch, O, d):
    frp, fcl, fvl = O.full()
    dev = "cuda:0"
    return {
        "rowptr": torch.tensor(frp, dtype=torch.int32, device=dev),
        "col": torch.tensor(fcl, dtype=torch.int32, device=dev),
        "val": torch.tensor(np.asarray(fvl).reshape(-1), dtype=torch.float64, device=dev),
        "b": torch.tensor(d.b.reshape(-1), dtype=torch.float64, device=dev),
        "mu": torch.tensor(d.mu, dtype=torch.float64, device=dev),
    }


def _set_device(L, h, n, p):
    return L.bogus_gpu_set_dual_device(h, n, int(p["col"].numel()), p["rowptr"].data_ptr(), p["col"].data_ptr(),
                                       p["val"].data_ptr(), p["b"].data_ptr(), p["mu"].data_ptr())


def test_set_dual_device_checks_structure_and_keeps_the_problem(c1):
    torch = pytest.importorskip("torch")
    import bogus_gpu

    L = bogus_gpu.lib()
    d, D, O = c1
    n = d.n
    p = _device_full(torch, O, d)
    E = bogus_gpu.DualFrictionProblem(0)
    assert _set_device(L, E.handle, n, p) == bogus_gpu.OK
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(1e-8)
    r = np.zeros(3 * n)
    res = E.solveWith(pg, r, staticProblem=False)
    res_o, r_o, _ = O.solve_pg(np.zeros(3 * n), variant=3, coulomb=True, tol=1e-8)
    assert res == res_o and np.array_equal(r, r_o)

    rowptr = p["rowptr"].cpu().numpy()
    row = 7
    k0, k1 = int(rowptr[row]), int(rowptr[row + 1])
    diag_k = k0 + int(np.nonzero(p["col"][k0:k1].cpu().numpy() == row)[0][0])
    assert k1 - k0 >= 2
    cases = []
    q = dict(p, col=p["col"].clone())
    q["col"][k0] = n  # column out of range
    cases.append(("range", q, bogus_gpu.BAD_INPUT))
    q = dict(p, col=p["col"].clone())
    q["col"][k0], q["col"][k0 + 1] = p["col"][k0 + 1], p["col"][k0]  # columns out of order
    cases.append(("order", q, bogus_gpu.BAD_INPUT))
    q = dict(p, col=p["col"].clone())
    q["col"][diag_k] = -1  # negative column
    cases.append(("negative", q, bogus_gpu.BAD_INPUT))
    q = dict(p, rowptr=p["rowptr"].clone())
    q["rowptr"][row + 1] = q["rowptr"][row] - 1  # row pointers out of order
    cases.append(("rowptr", q, bogus_gpu.BAD_INPUT))
    q = dict(p, rowptr=p["rowptr"].clone())
    q["rowptr"][n] = q["rowptr"][n] + 5  # rowptr[n] beyond nnzb
    cases.append(("rowptr_end", q, bogus_gpu.BAD_INPUT))
    q = dict(p, val=p["val"].clone())
    q["val"][40] = float("nan")
    cases.append(("nan", q, bogus_gpu.NONFINITE))
    for name, q, want in cases:
        st = _set_device(L, E.handle, n, q)
        assert st == want, (name, L.bogus_gpu_last_error())
    # a well-ordered 2-contact W whose row 0 has no diagonal block
    dev = "cuda:0"
    q = {"rowptr": torch.tensor([0, 1, 3], dtype=torch.int32, device=dev),
         "col": torch.tensor([1, 0, 1], dtype=torch.int32, device=dev),
         "val": torch.tensor(np.tile(np.eye(3).reshape(-1), 3), dtype=torch.float64, device=dev),
         "b": torch.zeros(6, dtype=torch.float64, device=dev),
         "mu": torch.full((2,), 0.5, dtype=torch.float64, device=dev)}
    assert _set_device(L, E.handle, 2, q) == bogus_gpu.BAD_INPUT
    assert b"row 0" in L.bogus_gpu_last_error()
    # the handle still holds the first problem
    r = np.zeros(3 * n)
    assert E.solveWith(pg, r, staticProblem=False) == res_o and np.array_equal(r, r_o)
