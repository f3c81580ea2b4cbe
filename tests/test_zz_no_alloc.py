"""Allocation-free projected-gradient solve (bogus_gpu_solve_pg_noalloc) against the handle-based solve.

The allocation-free entry point exists for callers that cannot allocate GPU memory while they solve (fixed
memory budgets, real-time loops, hosts that own every buffer): it keeps its temporaries in one array inside
the library. Two calls in a row through the C ABI must give exactly what DualFrictionProblem.solveWith gives
for the same inputs (the kernels are the same, so the tolerance is exact equality), which also shows that the
second call is not disturbed by what the first one left in the shared array. This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_problem(torch, oracle, d, rp, cl, vl):
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    frp, fcl, fvl = O.full()
    dev = "cuda:0"
    return {
        "n": d.n,
        "nnzb": int(fcl.size),
        "rowptr": torch.tensor(frp, dtype=torch.int32, device=dev),
        "col": torch.tensor(fcl, dtype=torch.int32, device=dev),
        "val": torch.tensor(fvl, dtype=torch.float64, device=dev),
        "b": torch.tensor(d.b.reshape(-1), dtype=torch.float64, device=dev),
        "mu": torch.tensor(d.mu, dtype=torch.float64, device=dev),
    }


@pytest.mark.parametrize("variant", [3, 4])  # APGD, SPG
def test_noalloc_matches_handle_solve_on_two_calls(oracle, variant):
    torch = pytest.importorskip("torch")
    import bogus_gpu
    from bogus_gpu import generator

    L = bogus_gpu.lib()
    d = generator.make("c1")
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    rp, cl, vl = D.W_lower()
    pg = bogus_gpu.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setTol(1e-8)
    r_ref = np.zeros(3 * d.n)
    res_ref = D.solveWith(pg, r_ref, staticProblem=False)
    it_ref = D.last_iterations

    p = _device_problem(torch, oracle, d, rp, cl, vl.reshape(-1))
    opts = pg.options(False)
    for call in range(2):
        r = torch.zeros(3 * d.n, dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        res, it = C.c_double(), C.c_uint()
        st = L.bogus_gpu_solve_pg_noalloc(0, p["n"], p["nnzb"], p["rowptr"].data_ptr(), p["col"].data_ptr(),
                                          p["val"].data_ptr(), p["b"].data_ptr(), p["mu"].data_ptr(), C.byref(opts),
                                          r.data_ptr(), C.byref(res), C.byref(it), None)
        assert st in (bogus_gpu.OK, bogus_gpu.NOT_CONVERGED), L.bogus_gpu_last_error()
        assert res.value == res_ref, f"call {call}"
        assert it.value == it_ref, f"call {call}"
        assert np.array_equal(r.cpu().numpy(), r_ref), f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_capacity():
    import bogus_gpu

    L = bogus_gpu.lib()
    o = bogus_gpu.PgOptions()
    L.bogus_gpu_pg_options_default(C.byref(o))
    res, it = C.c_double(), C.c_uint()
    st = L.bogus_gpu_solve_pg_noalloc(0, 65537, 0, None, None, None, None, None, C.byref(o), None, C.byref(res),
                                      C.byref(it), None)
    assert st == bogus_gpu.BAD_INPUT
    assert b"exceed" in L.bogus_gpu_last_error()
    o.max_iters = 65537
    st = L.bogus_gpu_solve_pg_noalloc(0, 10, 0, None, None, None, None, None, C.byref(o), None, C.byref(res),
                                      C.byref(it), None)
    assert st == bogus_gpu.BAD_INPUT
