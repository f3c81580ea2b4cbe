"""Shared test setup: the `gpu` marker, import paths, and builders for the CPU-side helpers.

CPU tests (`-m "not gpu"`) pin the oracle against the reference's own known answers, check that the
library's per-contact device math (compiled for the host) matches the oracle bit for bit, and check that
the C-ABI library loads and exports every declared symbol. GPU tests (`-m gpu`) compare the kernels,
through the C ABI, with the oracle on identical inputs.
"""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "so-bogus_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

HOSTMATH_SRC = os.path.join(REPO, "tests", "hostmath", "hostmath.cpp")
HOSTMATH_LIB = os.path.join(REPO, "tests", "hostmath", "build", "libhostmath.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")


def build_hostmath() -> str:
    deps = [HOSTMATH_SRC, os.path.join(REPO, "so-bogus_gb300", "csrc", "soc_device.cuh")]
    if not os.path.exists(HOSTMATH_LIB) or any(os.path.getmtime(d) > os.path.getmtime(HOSTMATH_LIB) for d in deps):
        os.makedirs(os.path.dirname(HOSTMATH_LIB), exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                        "-I" + os.path.join(REPO, "so-bogus_gb300", "csrc"), "-o", HOSTMATH_LIB, HOSTMATH_SRC],
                       check=True)
    return HOSTMATH_LIB


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(REPO, "tests", "golden", "reference_fixtures.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def hostmath():
    import ctypes as C

    import numpy as np

    L = C.CDLL(build_hostmath())
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    L.hm_local_solve.restype = C.c_double
    L.hm_local_solve.argtypes = [C.c_int, C.c_int, dp, dp, dp, C.c_double, C.c_double, C.c_double]
    L.hm_law_solve_local.restype = C.c_int
    L.hm_law_solve_local.argtypes = [C.c_int, C.c_int, dp, dp, dp, C.c_double, C.c_double]
    L.hm_law_eval.restype = C.c_double
    L.hm_law_eval.argtypes = [C.c_int, C.c_double, dp, dp]
    L.hm_project.argtypes = [C.c_double, dp]
    L.hm_real_roots.restype = C.c_int
    L.hm_real_roots.argtypes = [dp, C.c_int, C.c_int, C.c_int, dp]
    L.hm_fb_jacobian.argtypes = [C.c_int, C.c_double, C.c_double, dp, dp, dp, dp, dp]
    L.hm_min_eigen_symmetric3.restype = C.c_double
    L.hm_min_eigen_symmetric3.argtypes = [dp]
    return L


def small_friction_dual(golden, oracle_mod):
    """The reference's SmallFrictionPb fixture as (lower BSR, b, mu) through the oracle's assembly."""
    import numpy as np

    s = golden["small_friction_pb"]
    P = oracle_mod.PrimalProblem(np.array(s["minv"]), s["objA"], s["objB"], np.array(s["HA"]), np.array(s["HB"]))
    rp, cl, vl = P.assemble()
    b = P.rhs(np.array(s["f_padded"]), np.array(s["w"]))
    return rp, cl, vl, b, np.array(s["mu"])
