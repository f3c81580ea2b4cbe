"""ctypes binding of the CPU oracle (oracle/src). Test infrastructure only.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py import this module, as the
checker. The oracle restates So-bogus's friction-solve path in plain C++ (see oracle/src/*.hpp for the
reference files each part follows).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")
_lib = None

CALLBACK = C.CFUNCTYPE(None, C.c_uint, C.c_double, C.c_void_p)

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build() -> str:
    """Compile liboracle.so with the committed Makefile (g++, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        build()
    L = C.CDLL(_LIB_PATH)
    vp = C.c_void_p
    L.oracle_num_threads.restype = C.c_int
    L.oracle_set_num_threads.argtypes = [C.c_int]
    L.oracle_set_gs_threads.argtypes = [C.c_int]
    L.oracle_last_gs_sweep_ms.restype = C.c_double
    L.oracle_dual_create.restype = vp
    L.oracle_dual_create.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp]
    L.oracle_dual_destroy.argtypes = [vp]
    L.oracle_dual_nnz_full.restype = C.c_int
    L.oracle_dual_nnz_full.argtypes = [vp]
    L.oracle_dual_full.argtypes = [vp, _ip, _ip, _dp]
    L.oracle_dual_spmv.argtypes = [vp, _dp, _dp, C.c_void_p]
    L.oracle_dual_split_row.argtypes = [vp, C.c_int, _dp, _dp]
    L.oracle_dual_eval.restype = C.c_double
    L.oracle_dual_eval.argtypes = [vp, C.c_int, _dp, C.c_int]
    L.oracle_dual_solve_pg.restype = C.c_double
    L.oracle_dual_solve_pg.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_uint, C.c_double, C.c_double,
                                       C.c_double, C.c_int, C.c_int, C.c_uint, _dp, C.POINTER(C.c_uint), CALLBACK,
                                       C.c_void_p]
    L.oracle_dual_solve_pg_fp32.restype = C.c_double
    L.oracle_dual_solve_pg_fp32.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_uint, C.c_double,
                                            C.c_double, C.c_int, C.c_uint, _dp, C.POINTER(C.c_uint)]
    L.oracle_dual_coloring.restype = C.c_int
    L.oracle_dual_coloring.argtypes = [vp, _ip, _ip]
    L.oracle_dual_solve_cadoux_gs.restype = C.c_double
    L.oracle_dual_solve_cadoux_gs.argtypes = [vp, C.c_int, C.c_double, C.c_uint, C.c_uint, C.c_double, C.c_uint,
                                              C.c_double, C.c_int, C.c_int, C.c_int, C.c_uint, _dp,
                                              C.POINTER(C.c_uint), CALLBACK, vp]
    L.oracle_dual_solve_cadoux_pg.restype = C.c_double
    L.oracle_dual_solve_cadoux_pg.argtypes = [vp, C.c_int, C.c_double, C.c_uint, C.c_uint, C.c_double, C.c_double,
                                              C.c_double, C.c_int, C.c_uint, _dp, C.POINTER(C.c_uint), CALLBACK, vp]
    L.oracle_meche_create.restype = vp
    L.oracle_meche_create.argtypes = [C.c_int, np.ctypeslib.ndpointer(dtype=np.uint32), _dp, _dp, C.c_int, _dp, _dp,
                                      _dp, _ip, _ip, _dp, _dp]
    L.oracle_meche_destroy.argtypes = [vp]
    L.oracle_frame_t.restype = None
    L.oracle_frame_t.argtypes = [C.c_int, _dp, _dp, _dp]
    L.oracle_meche_solve.restype = C.c_double
    L.oracle_meche_solve.argtypes = [vp, _dp, vp, C.c_int, C.c_uint, C.c_uint, C.c_double, C.c_int, C.c_int,
                                     C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                     C.c_double, CALLBACK, vp]
    L.oracle_primal_solve_product_gs.restype = C.c_double
    L.oracle_primal_solve_product_gs.argtypes = [vp, _dp, _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_uint,
                                                 C.c_double, C.c_uint, C.c_double, C.c_int, C.c_int, _dp,
                                                 C.POINTER(C.c_uint), CALLBACK, vp]
    L.oracle_primal_solve_dual_ama.restype = C.c_double
    L.oracle_primal_solve_dual_ama.argtypes = [vp, _dp, _dp, _dp, _dp, C.c_int, C.c_double, C.c_uint, C.c_double,
                                               C.c_double, C.c_uint, C.c_double, C.c_double, C.c_int, C.c_int, vp,
                                               _dp, _dp, C.POINTER(C.c_uint), CALLBACK, vp]
    L.oracle_dual_solve_gs.restype = C.c_double
    L.oracle_dual_solve_gs.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_uint, C.c_uint, C.c_double, C.c_uint,
                                       C.c_double, C.c_int, C.c_int, C.c_int, _dp, C.POINTER(C.c_uint), CALLBACK,
                                       C.c_void_p]
    L.oracle_local_solve.restype = C.c_double
    L.oracle_local_solve.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double]
    L.oracle_law_solve_local.restype = C.c_int
    L.oracle_law_solve_local.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_double, C.c_double]
    L.oracle_real_roots.restype = C.c_int
    L.oracle_real_roots.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp]
    L.oracle_project.argtypes = [C.c_double, _dp]
    L.oracle_law_eval.restype = C.c_double
    L.oracle_law_eval.argtypes = [C.c_int, C.c_double, _dp, _dp]
    L.oracle_fb_jacobian.argtypes = [C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp]
    L.oracle_canonical_sum.restype = C.c_double
    L.oracle_canonical_sum.argtypes = [_dp, C.c_size_t]
    L.oracle_primal_create.restype = vp
    L.oracle_primal_create.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, _ip, _dp, _dp]
    L.oracle_primal_destroy.argtypes = [vp]
    L.oracle_primal_assemble.restype = C.c_int
    L.oracle_primal_assemble.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p]
    L.oracle_primal_rhs.argtypes = [vp, _dp, _dp, _dp]
    L.oracle_primal_solve_admm.restype = C.c_double
    L.oracle_primal_solve_admm.argtypes = [vp, _dp, C.c_double, _dp, _dp, _dp, C.c_double, C.c_uint, C.c_double,
                                           C.c_int, C.c_int, vp, _dp, _dp, C.POINTER(C.c_uint), CALLBACK, C.c_void_p]
    _lib = L
    return L


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def set_num_threads(t: int) -> None:
    lib().oracle_set_num_threads(int(t))


def set_gs_threads(t: int) -> None:
    """Threads of the colored Gauss-Seidel sweeps that follow: 1 (default) is the sequential sweep the tests
    compare against; more runs the reference's per-color OpenMP loop, whose iterates depend on the thread
    timing (CPU timing baseline only)."""
    lib().oracle_set_gs_threads(int(t))


def last_gs_sweep_ms() -> float:
    """Wall time (ms) of the sweeps and evaluations of the last dual Gauss-Seidel solve, without its setup."""
    return float(lib().oracle_last_gs_sweep_ms())


def num_threads() -> int:
    return lib().oracle_num_threads()


class Trace:
    """Collects (iteration, residual) pairs from a solver callback."""

    def __init__(self):
        self.items = []
        self._cb = CALLBACK(lambda it, r, _u: self.items.append((int(it), float(r))))


_NO_CB = CALLBACK(0)


class DualProblem:
    """DualFrictionProblem<3>: W (lower-triangle BSR), b, mu."""

    def __init__(self, rowptr, col, val, b, mu):
        self.rowptr, self.col, self.val = _i32(rowptr), _i32(col), _f64(val).reshape(-1)
        self.b, self.mu = _f64(b).reshape(-1), _f64(mu).reshape(-1)
        self.n = len(self.rowptr) - 1
        self.h = lib().oracle_dual_create(self.n, self.rowptr, self.col, self.val, self.b, self.mu)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_dual_destroy(self.h)
            self.h = None

    def full(self):
        L = lib()
        nnz = L.oracle_dual_nnz_full(self.h)
        rp = np.zeros(self.n + 1, np.int32)
        cl = np.zeros(nnz, np.int32)
        vl = np.zeros(9 * nnz, np.float64)
        L.oracle_dual_full(self.h, rp, cl, vl)
        return rp, cl, vl

    def spmv(self, x, init=None):
        y = np.zeros(3 * self.n)
        xi = _f64(x)
        ii = None if init is None else _f64(init)
        lib().oracle_dual_spmv(self.h, xi, y, None if ii is None else ii.ctypes.data_as(C.c_void_p))
        return y

    def split_row(self, row, x, res):
        res = _f64(res).copy()
        lib().oracle_dual_split_row(self.h, int(row), _f64(x), res)
        return res

    def eval(self, r, coulomb=True, inf_norm=False):
        return lib().oracle_dual_eval(self.h, int(coulomb), _f64(r), int(inf_norm))

    def coloring(self):
        perm = np.zeros(self.n, np.int32)
        colors = np.zeros(self.n + 1, np.int32)
        nc = lib().oracle_dual_coloring(self.h, perm, colors)
        return perm, colors[: nc + 1]

    def solve_pg(self, r, variant=3, coulomb=False, tol=1e-6, max_iters=300, ls_iters=8, optimistic=1.25,
                 pessimistic=0.5, armijo=0.5, inf_norm=False, trace: Trace | None = None, lin_momentum=False,
                 hy_refresh=0):
        """lin_momentum: APGD's momentum product by linearity; hy_refresh: FP32 correction products refreshed
        every hy_refresh iterations (neither is in the reference; see ProjectedGradient)."""
        r = _f64(r).copy()
        it = C.c_uint(0)
        cb = trace._cb if trace else _NO_CB
        res = lib().oracle_dual_solve_pg(self.h, variant, int(coulomb), tol, max_iters, ls_iters, optimistic,
                                         pessimistic, armijo, int(inf_norm), int(lin_momentum), int(hy_refresh), r,
                                         C.byref(it), cb, None)
        return res, r, it.value

    def solve_pg_fp32(self, r, apgd=True, coulomb=False, tol=1e-6, max_iters=300, ls_iters=8, optimistic=1.25,
                      pessimistic=0.5, inf_norm=False, stall_iters=4):
        """The FP32 part of the FP32-refined solve (not in the reference): returns (residual, best iterate widened
        to double, iterations)."""
        r = _f64(r).copy()
        it = C.c_uint(0)
        res = lib().oracle_dual_solve_pg_fp32(self.h, int(apgd), int(coulomb), tol, max_iters, ls_iters, optimistic,
                                              pessimistic, int(inf_norm), int(stall_iters), r, C.byref(it))
        return res, r, it.value

    def solve_cadoux_gs(self, r, cadoux_iters, strategy=3, tol=1e-6, max_iters=250, eval_every=25, skip_tol=1e-6,
                        skip_iters=10, auto_reg=0.0, try_zero=False, inf_norm=False, coloring=False,
                        trace: Trace | None = None):
        """DualFrictionProblem::solveCadoux(gs, r, cadoux_iters): returns (residual, r, cadoux iterations run)."""
        r = _f64(r).copy()
        it = C.c_uint(0)
        cb = trace._cb if trace else _NO_CB
        res = lib().oracle_dual_solve_cadoux_gs(self.h, strategy, tol, max_iters, eval_every, skip_tol, skip_iters,
                                                auto_reg, int(try_zero), int(inf_norm), int(coloring), cadoux_iters,
                                                r, C.byref(it), cb, None)
        return res, r, it.value

    def solve_cadoux_pg(self, r, cadoux_iters, variant=3, tol=1e-6, max_iters=300, ls_iters=8, optimistic=1.25,
                        pessimistic=0.5, armijo=0.5, inf_norm=False, trace: Trace | None = None):
        r = _f64(r).copy()
        it = C.c_uint(0)
        cb = trace._cb if trace else _NO_CB
        res = lib().oracle_dual_solve_cadoux_pg(self.h, variant, tol, max_iters, ls_iters, optimistic, pessimistic,
                                                armijo, int(inf_norm), cadoux_iters, r, C.byref(it), cb, None)
        return res, r, it.value

    def solve_gs(self, r, coulomb=True, strategy=3, tol=1e-6, max_iters=250, eval_every=25, skip_tol=1e-6,
                 skip_iters=10, auto_reg=0.0, try_zero=True, inf_norm=False, coloring=True,
                 trace: Trace | None = None):
        r = _f64(r).copy()
        it = C.c_uint(0)
        cb = trace._cb if trace else _NO_CB
        res = lib().oracle_dual_solve_gs(self.h, int(coulomb), strategy, tol, max_iters, eval_every, skip_tol,
                                         skip_iters, auto_reg, int(try_zero), int(inf_norm), int(coloring), r,
                                         C.byref(it), cb, None)
        return res, r, it.value


def local_solve(A, b, x, mu, coulomb=True, strategy=3, tol=1.8189894035458565e-12, scaling=1.0):
    x = _f64(x).copy()
    res = lib().oracle_local_solve(int(coulomb), strategy, _f64(A).reshape(-1), _f64(b), x, mu, tol, scaling)
    return res, x


def law_solve_local(A, b, x, mu, coulomb=True, strategy=3, scaling=1.0):
    x = _f64(x).copy()
    ok = lib().oracle_law_solve_local(int(coulomb), strategy, _f64(A).reshape(-1), _f64(b), x, mu, scaling)
    return bool(ok), x


def real_roots(coeffs, degenerate=False, filt=0):
    c = _f64(coeffs)
    dim = len(c) - (1 if degenerate else 0)
    roots = np.zeros(max(dim, 1))
    n = lib().oracle_real_roots(c, dim, int(degenerate), filt, roots)
    return roots[:n]


def project(mu, x):
    x = _f64(x).copy()
    lib().oracle_project(mu, x)
    return x


def law_eval(mu, x, y, coulomb=True):
    return lib().oracle_law_eval(int(coulomb), mu, _f64(x), _f64(y))


def canonical_sum(v):
    v = _f64(v)
    return lib().oracle_canonical_sum(v, v.size)


class PrimalProblem:
    """Rigid-body primal data: uniform ndof per body, block-diagonal M^-1, contacts with 1 or 2 bodies."""

    def __init__(self, minv, objA, objB, HA, HB):
        self.minv = _f64(minv)
        self.nbodies, self.ndof = self.minv.shape[0], self.minv.shape[1]
        self.objA, self.objB = _i32(objA), _i32(objB)
        self.HA, self.HB = _f64(HA), _f64(HB)
        self.n = len(self.objA)
        self.h = lib().oracle_primal_create(self.nbodies, self.ndof, self.minv.reshape(-1), self.n, self.objA,
                                            self.objB, self.HA.reshape(-1), self.HB.reshape(-1))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_primal_destroy(self.h)
            self.h = None

    def assemble(self):
        L = lib()
        nnz = L.oracle_primal_assemble(self.h, None, None, None)
        rp = np.zeros(self.n + 1, np.int32)
        cl = np.zeros(nnz, np.int32)
        vl = np.zeros(9 * nnz)
        L.oracle_primal_assemble(self.h, rp.ctypes.data_as(C.c_void_p), cl.ctypes.data_as(C.c_void_p),
                                 vl.ctypes.data_as(C.c_void_p))
        return rp, cl, vl

    def rhs(self, f, w):
        b = np.zeros(3 * self.n)
        lib().oracle_primal_rhs(self.h, _f64(f).reshape(-1), _f64(w).reshape(-1), b)
        return b

    def solve_product_gs(self, f, w, mu, r, coulomb=True, strategy=3, tol=1e-6, max_iters=250, eval_every=25,
                         skip_tol=1e-6, skip_iters=10, auto_reg=0.0, try_zero=True, inf_norm=False,
                         trace: Trace | None = None):
        """PrimalFrictionProblem::solveWith(ProductGaussSeidelType&, r, staticProblem = not coulomb)."""
        r = _f64(r).copy()
        it = C.c_uint(0)
        cb = trace._cb if trace else _NO_CB
        res = lib().oracle_primal_solve_product_gs(self.h, _f64(f).reshape(-1), _f64(w).reshape(-1), _f64(mu),
                                                   int(coulomb), strategy, tol, max_iters, eval_every, skip_tol,
                                                   skip_iters, auto_reg, int(try_zero), int(inf_norm), r,
                                                   C.byref(it), cb, None)
        return res, r, it.value

    def solve_dual_ama(self, mass, mu, f, w, v, r, static=False, tol=1e-6, max_iters=300, fp_step=0.1,
                       proj_step=0.1, ls_iters=6, optimistic=1.25, pessimistic=0.5, accelerated=True, inf_norm=False,
                       true_dofs=None, trace: Trace | None = None):
        """PrimalFrictionProblem::solveWith(DualAMAType&, v, r, staticProblem): returns (res, v, r, iterations)."""
        v = _f64(v).copy()
        r = _f64(r).copy()
        it = C.c_uint(0)
        cb = trace._cb if trace else _NO_CB
        td = None if true_dofs is None else _i32(true_dofs)
        res = lib().oracle_primal_solve_dual_ama(self.h, _f64(mass).reshape(-1), _f64(mu), _f64(f).reshape(-1),
                                                 _f64(w).reshape(-1), int(static), tol, max_iters, fp_step, proj_step,
                                                 ls_iters, optimistic, pessimistic, int(accelerated), int(inf_norm),
                                                 None if td is None else td.ctypes.data_as(C.c_void_p), v, r,
                                                 C.byref(it), cb, None)
        return res, v, r, it.value

    def solve_admm(self, prox_inv, lam, mu, f, w, v, r, tol=1e-6, max_iters=300, step=1e-2, accelerated=True,
                   inf_norm=False, true_dofs=None, trace: Trace | None = None):
        """PrimalFrictionProblem::solveWith(ADMM&, lambda, v, r): returns (res, v, r, iterations). true_dofs: the
        bodies' own dof counts of a padded problem (the error function's scalings), default all ndof."""
        v = _f64(v).copy()
        r = _f64(r).copy()
        it = C.c_uint(0)
        cb = trace._cb if trace else _NO_CB
        td = None if true_dofs is None else _i32(true_dofs)
        res = lib().oracle_primal_solve_admm(self.h, _f64(prox_inv).reshape(-1), lam, _f64(mu), _f64(f).reshape(-1),
                                             _f64(w).reshape(-1), tol, max_iters, step, int(accelerated),
                                             int(inf_norm), None if td is None else td.ctypes.data_as(C.c_void_p),
                                             v, r, C.byref(it), cb, None)
        return res, v, r, it.value


def frame_t(E, x):
    """E^T x per contact (E: (n, 3, 3), x: 3n) with the facade's frame chain."""
    E = _f64(E).reshape(-1)
    x = _f64(x).reshape(-1)
    y = np.zeros_like(x)
    lib().oracle_frame_t(x.size // 3, E, x, y)
    return y


class MecheProblem:
    """MecheFrictionProblem::fromPrimal / solve (Interfaces/MecheInterface.cpp) restated (oracle/src/oracle_meche.hpp).
    mass: list of (ndof, ndof) arrays; HA / HB: lists of (3, ndof) arrays (HB[i] None when objB[i] == -1);
    E: (n, 3, 3) frames (rows: world -> local, E[i][a][b] as the reference's E block); f packed by body; w (3n)
    in world coordinates."""

    def __init__(self, mass, f, mu, E, w, objA, objB, HA, HB):
        ndof = np.array([m.shape[0] for m in mass], np.uint32)
        n = len(objA)
        Ecm = np.zeros((3, 3 * n))  # the reference's (3n x 3) column-major layout
        E = np.asarray(E, np.float64)
        for i in range(n):
            Ecm[:, 3 * i:3 * i + 3] = E[i].T
        self.h = lib().oracle_meche_create(len(mass), ndof, np.concatenate([np.asarray(m, np.float64).T.ravel()
                                                                             for m in mass]),
                                           _f64(f).reshape(-1), n, _f64(mu), Ecm.ravel(), _f64(w).reshape(-1),
                                           _i32(objA), _i32(objB),
                                           np.concatenate([np.zeros(0)] + [np.asarray(h, np.float64).T.ravel()
                                                                           for h in HA]),
                                           np.concatenate([np.zeros(0)] + [np.asarray(h, np.float64).T.ravel()
                                                                           for h in HB if h is not None]))
        if not self.h:
            raise ValueError("singular mass block")
        self.m = int(ndof.sum())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_meche_destroy(self.h)
            self.h = None

    def solve(self, r, with_v=True, max_threads=0, max_iters=0, cadoux_iters=0, tolerance=0.0, inf_norm=False,
              algorithm=0, gs_regularization=0.0, gs_coloring=False, gs_skip_iters=-1, try_zero=True, pg_variant=4,
              admm_step=1.0, admm_fp_step=1e-3, static=False, regularization=0.0, v=None,
              trace: Trace | None = None):
        r = _f64(r).copy()
        vv = None
        if with_v:
            vv = np.zeros(self.m) if v is None else _f64(v).copy()
        cb = trace._cb if trace else _NO_CB
        res = lib().oracle_meche_solve(self.h, r, None if vv is None else vv.ctypes.data_as(C.c_void_p), max_threads,
                                       max_iters, cadoux_iters, tolerance, int(inf_norm), algorithm, gs_regularization,
                                       int(gs_coloring), gs_skip_iters, int(try_zero), pg_variant, admm_step,
                                       admm_fp_step, int(static), regularization, cb, None)
        return res, r, vv
