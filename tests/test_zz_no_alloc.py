"""Allocation-free projected-gradient solve (bogus_gpu_solve_pg_noalloc) against the handle-based solve.

The allocation-free entry point exists for callers that cannot allocate GPU memory while they solve (fixed
memory budgets, real-time loops, hosts that own every buffer): it keeps its temporaries in one array inside
the library. Calls in a row through the C ABI must give exactly what DualFrictionProblem.solveWith gives for the
same inputs (the kernels are the same, so the tolerance is exact equality):

* at the array's capacity (65 536 contacts), then on a 500-contact problem twice, so that the small solves
  run over what the large one left in the shared array;
* for APGD, Descent and SPG;
* without changing the device's free memory once the library is loaded;
* rejecting a malformed W with BAD_INPUT before any solve, r untouched.

The capacity problem is also compared with the oracle. This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAPACITY = 65536
CAP_ITERS = 200


def _device_problem(torch, oracle, d, rp, cl, vl):
    O = oracle.DualProblem(rp, cl, vl, d.b, d.mu)
    frp, fcl, fvl = O.full()
    dev = "cuda:0"
    return {
        "n": d.n,
        "nnzb": int(fcl.size),
        "rowptr": torch.tensor(frp, dtype=torch.int32, device=dev),
        "col": torch.tensor(fcl, dtype=torch.int32, device=dev),
        "val": torch.tensor(np.asarray(fvl).reshape(-1), dtype=torch.float64, device=dev),
        "b": torch.tensor(d.b.reshape(-1), dtype=torch.float64, device=dev),
        "mu": torch.tensor(d.mu, dtype=torch.float64, device=dev),
        "oracle": O,
    }


@pytest.fixture(scope="module")
def problems(oracle):
    torch = pytest.importorskip("torch")
    import bogus_gpu
    from bogus_gpu import generator

    out = {}
    for name, d, tol, max_iters, static in (
            ("capacity", generator.random_pairs(nbodies=CAPACITY // 3, ncontacts=CAPACITY, seed=11), 1e-6, CAP_ITERS,
             True),
            ("c1", generator.make("c1"), 1e-8, 300, False)):
        D = bogus_gpu.DualFrictionProblem(0)
        D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
        rp, cl, vl = D.W_lower()
        p = _device_problem(torch, oracle, d, rp, cl, vl.reshape(-1))
        p.update(d=d, D=D, tol=tol, max_iters=max_iters, static=static)
        out[name] = p
    assert out["capacity"]["n"] == CAPACITY
    return out


def _solver(p, variant):
    import bogus_gpu

    pg = bogus_gpu.ProjectedGradient()
    pg.setDefaultVariant(variant)
    pg.setTol(p["tol"])
    pg.setMaxIters(p["max_iters"])
    return pg


def _noalloc(p, pg, r):
    import bogus_gpu

    L = bogus_gpu.lib()
    opts = pg.options(p["static"])
    res, it = C.c_double(), C.c_uint()
    st = L.bogus_gpu_solve_pg_noalloc(0, p["n"], p["nnzb"], p["rowptr"].data_ptr(), p["col"].data_ptr(),
                                      p["val"].data_ptr(), p["b"].data_ptr(), p["mu"].data_ptr(), C.byref(opts),
                                      r.data_ptr(), C.byref(res), C.byref(it), None)
    return st, res.value, it.value


@pytest.mark.parametrize("variant", [3, 1, 4])  # APGD, Descent, SPG
def test_noalloc_matches_handle_solve_large_then_small(problems, variant):
    import torch

    import bogus_gpu

    L = bogus_gpu.lib()
    for call, name in enumerate(("capacity", "c1", "c1")):
        p = problems[name]
        pg = _solver(p, variant)
        r_ref = np.zeros(3 * p["n"])
        res_ref = p["D"].solveWith(pg, r_ref, staticProblem=p["static"])
        it_ref = p["D"].last_iterations
        r = torch.zeros(3 * p["n"], dtype=torch.float64, device="cuda:0")
        torch.cuda.synchronize()
        st, res, it = _noalloc(p, pg, r)
        assert st in (bogus_gpu.OK, bogus_gpu.NOT_CONVERGED), L.bogus_gpu_last_error()
        assert res == res_ref, f"call {call} ({name})"
        assert it == it_ref, f"call {call} ({name})"
        assert np.array_equal(r.cpu().numpy(), r_ref), f"call {call} ({name})"


def test_noalloc_at_capacity_matches_oracle(problems):
    import torch

    import bogus_gpu

    p = problems["capacity"]
    pg = _solver(p, 3)
    r = torch.zeros(3 * p["n"], dtype=torch.float64, device="cuda:0")
    st, res, it = _noalloc(p, pg, r)
    assert st in (bogus_gpu.OK, bogus_gpu.NOT_CONVERGED)
    res_o, r_o, it_o = p["oracle"].solve_pg(np.zeros(3 * p["n"]), variant=3, coulomb=False, tol=p["tol"],
                                            max_iters=p["max_iters"])
    assert res == res_o and it == it_o
    assert np.array_equal(r.cpu().numpy(), r_o)


def test_noalloc_allocates_nothing(problems):
    import torch

    import bogus_gpu

    p = problems["c1"]
    pg = _solver(p, 3)
    r = torch.zeros(3 * p["n"], dtype=torch.float64, device="cuda:0")
    assert _noalloc(p, pg, r)[0] == bogus_gpu.OK  # the library and its kernels are loaded
    r.zero_()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert _noalloc(p, pg, r)[0] == bogus_gpu.OK
        r.zero_()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_a_malformed_w(problems):
    import torch

    import bogus_gpu

    L = bogus_gpu.lib()
    p = dict(problems["c1"])
    p["col"] = p["col"].clone()
    p["col"][3] = p["n"] + 4  # column out of range
    pg = _solver(p, 3)
    r = torch.full((3 * p["n"],), 0.5, dtype=torch.float64, device="cuda:0")
    st, _, _ = _noalloc(p, pg, r)
    assert st == bogus_gpu.BAD_INPUT
    assert b"malformed" in L.bogus_gpu_last_error()
    assert bool(torch.all(r == 0.5))


def test_noalloc_rejects_sizes_beyond_its_capacity():
    import bogus_gpu

    L = bogus_gpu.lib()
    o = bogus_gpu.PgOptions()
    L.bogus_gpu_pg_options_default(C.byref(o))
    res, it = C.c_double(), C.c_uint()
    st = L.bogus_gpu_solve_pg_noalloc(0, CAPACITY + 1, 0, None, None, None, None, None, C.byref(o), None, C.byref(res),
                                      C.byref(it), None)
    assert st == bogus_gpu.BAD_INPUT
    assert b"exceed" in L.bogus_gpu_last_error()
    o.max_iters = 65537
    st = L.bogus_gpu_solve_pg_noalloc(0, 10, 0, None, None, None, None, None, C.byref(o), None, C.byref(res),
                                      C.byref(it), None)
    assert st == bogus_gpu.BAD_INPUT
