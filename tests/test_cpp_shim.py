"""The C++ caller's path: include/bogus_gpu.hpp (the reference's API names over the C ABI) compiled with g++ and
linked against libbogus_gpu.so.

* CPU: the program compiles and links; the solver objects carry the reference's defaults; the host-side
  BAD_INPUT paths throw bogus_gpu::Error; without a usable GPU a solve reports NO_DEVICE (on a GPU it solves).
* GPU: DualFrictionProblem<3>::computeFrom and solveWith (Gauss-Seidel, APGD), evalWith, solveCadoux, a changed b,
  and PrimalFrictionProblem<3>::solveWith(ADMM) on the 500-contact problem, bit for bit against the oracle.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO

SRC = os.path.join(REPO, "tests", "cpp", "shim_check.cpp")
OUT_DIR = os.path.join(REPO, "tests", "cpp", "build")
EXE = os.path.join(OUT_DIR, "shim_check")


@pytest.fixture(scope="module")
def shim_exe():
    import sys

    sys.path.insert(0, os.path.join(REPO, "so-bogus_gb300"))
    import build as gpu_build

    lib = gpu_build.build()
    libdir = os.path.dirname(lib)
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, lib, os.path.join(REPO, "include", "bogus_gpu.hpp"), os.path.join(REPO, "include", "bogus_gpu.h")]
    if not os.path.exists(EXE) or any(os.path.getmtime(d) > os.path.getmtime(EXE) for d in deps):
        subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(REPO, "include"),
                        SRC, "-o", EXE, "-L" + libdir, "-lbogus_gpu", "-Wl,-rpath," + libdir], check=True)
    return EXE


def test_shim_compiles_links_and_keeps_the_reference_defaults(shim_exe):
    r = subprocess.run([shim_exe, "defaults"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "defaults ok" in r.stdout


@pytest.mark.gpu
def test_shim_solves_bitwise_like_the_oracle(shim_exe, oracle, tmp_path):
    from bogus_gpu import generator

    d = generator.make("c1")
    n, nb, dof = d.n, d.nbodies, 6
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as fh:
        np.array([n, nb, dof], np.int32).tofile(fh)
        np.ascontiguousarray(d.minv, np.float64).tofile(fh)
        np.ascontiguousarray(d.objA, np.int32).tofile(fh)
        np.ascontiguousarray(d.objB, np.int32).tofile(fh)
        np.ascontiguousarray(d.HA, np.float64).tofile(fh)
        np.ascontiguousarray(d.HB, np.float64).tofile(fh)
        np.ascontiguousarray(d.b, np.float64).tofile(fh)
        np.ascontiguousarray(d.mu, np.float64).tofile(fh)
    r = subprocess.run([shim_exe, "solve", str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(out, "rb").read()
    pos = 0

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos)
        pos += a.nbytes
        return a

    nnz = int(take(np.int32, 1)[0])
    rp, cl, vl = take(np.int32, n + 1), take(np.int32, nnz), take(np.float64, 9 * nnz)
    b = take(np.float64, 3 * n)
    res_gs, r_gs, ev_gs, ncalls = take(np.float64, 1)[0], take(np.float64, 3 * n), take(np.float64, 1)[0], \
        take(np.float64, 1)[0]
    res_pg, r_pg = take(np.float64, 1)[0], take(np.float64, 3 * n)
    res_cad, r_cad = take(np.float64, 1)[0], take(np.float64, 3 * n)
    res_pg2, r_pg2 = take(np.float64, 1)[0], take(np.float64, 3 * n)
    res_admm, v_admm, r_admm = take(np.float64, 1)[0], take(np.float64, nb * dof), take(np.float64, 3 * n)
    assert pos == len(raw)

    P = oracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    orp, ocl, ovl = P.assemble()
    assert np.array_equal(rp, orp) and np.array_equal(cl, ocl) and np.array_equal(vl, ovl)
    ob = P.rhs(np.zeros(nb * dof), d.b)
    assert np.array_equal(b, ob)
    O = oracle.DualProblem(orp, ocl, ovl, ob, d.mu)
    trace = oracle.Trace()
    res_o, r_o, _ = O.solve_gs(np.zeros(3 * n), coulomb=True, tol=1e-8, coloring=False, trace=trace)
    assert res_gs == res_o and np.array_equal(r_gs, r_o)
    assert ev_gs == O.eval(r_o, coulomb=True)
    assert ncalls > 0
    res_o, r_o, _ = O.solve_pg(np.zeros(3 * n), variant=3, coulomb=False, tol=1e-8)
    assert res_pg == res_o and np.array_equal(r_pg, r_o)
    res_o, r_o, _ = O.solve_cadoux_pg(np.zeros(3 * n), 10, variant=3, tol=1e-8)
    assert res_cad == res_o and np.array_equal(r_cad, r_o)
    b2 = ob.copy()
    b2[0::3] += 0.125
    O2 = oracle.DualProblem(orp, ocl, ovl, b2, d.mu)
    res_o, r_o, _ = O2.solve_pg(np.zeros(3 * n), variant=3, coulomb=False, tol=1e-8)
    assert res_pg2 == res_o and np.array_equal(r_pg2, r_o)
    res_o, v_o, r_o, _ = P.solve_admm(d.minv, 0.0, d.mu, np.zeros(nb * dof), d.b, np.zeros(nb * dof), np.zeros(3 * n),
                                      max_iters=50)
    assert res_admm == res_o and np.array_equal(v_admm, v_o) and np.array_equal(r_admm, r_o)
