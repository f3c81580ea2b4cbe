"""The C-ABI library builds, loads and exports every function include/bogus_gpu.h declares (no GPU needed;
nothing here launches a kernel)."""
import ctypes as C
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "bogus_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(bogus_gpu_[a-z0-9_]+)\s*\(", text))
    names.discard("bogus_gpu_callback")
    return sorted(names)


@pytest.fixture(scope="module")
def built_lib():
    import sys

    sys.path.insert(0, os.path.join(REPO, "so-bogus_gb300"))
    import build as gpu_build

    return gpu_build.build()


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("bogus_gpu_create", "bogus_gpu_set_dual", "bogus_gpu_solve_pg", "bogus_gpu_solve_gs",
                     "bogus_gpu_eval", "bogus_gpu_spmv", "bogus_gpu_assemble_dual"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_binding_lists_every_symbol():
    import bogus_gpu

    assert sorted(bogus_gpu.EXPORTED) == declared_functions()


def test_defaults_match_reference(built_lib):
    import bogus_gpu

    L = bogus_gpu.lib()
    o = bogus_gpu.PgOptions()
    L.bogus_gpu_pg_options_default(C.byref(o))
    assert (o.tol, o.max_iters, o.ls_iters) == (1e-6, 300, 8)
    assert (o.ls_optimistic_factor, o.ls_pessimistic_factor, o.ls_armijo_coefficient) == (1.25, 0.5, 0.5)
    assert o.variant == bogus_gpu.APGD and o.static_problem == 1
    assert o.mixed_precision == 0 and o.momentum_by_linearity == 0  # the drop-in: the reference's arithmetic
    assert o.fp32_stall_iters == 4  # FP32-refined solves only
    g = bogus_gpu.GsOptions()
    L.bogus_gpu_gs_options_default(C.byref(g))
    assert (g.tol, g.max_iters, g.eval_every, g.skip_tol, g.skip_iters) == (1e-6, 250, 25, 1e-6, 10)
    assert g.try_zero_as_well == 1 and g.static_problem == 0 and g.local_strategy == bogus_gpu.REV_HYBRID
    assert L.bogus_gpu_status_string(5) == b"device wait timed out"
