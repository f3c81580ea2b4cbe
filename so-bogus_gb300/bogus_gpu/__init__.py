"""bogus_gpu — Python host interface of the GB300 friction-solve library (ctypes over libbogus_gpu.so).

Mirrors So-bogus's friction-solve API (Interfaces/FrictionProblem.hpp, Core/BlockSolvers/*.hpp) with the
same names, defaults and argument meanings:

    problem = DualFrictionProblem()            # W (3x3-block BSR), b, mu on the GPU
    problem.computeFrom(primal)                # W = H M^-1 H^T, b = w - H M^-1 f   (on the GPU)
    pg = ProjectedGradient(); pg.setTol(1e-6)  # APGD by default
    res = problem.solveWith(pg, r)             # r: warm start in, solution out (staticProblem=True)
    gs = GaussSeidel()
    res = problem.solveWith(gs, r)             # colored GS, Coulomb law (staticProblem=False)

Every solve runs the CUDA kernels of libbogus_gpu.so; there is no CPU path. Importing this module on a
machine without the built library raises ImportError; calls without a usable sm_103 GPU raise BogusGpuError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libbogus_gpu.so")

OK, NOT_CONVERGED, BAD_INPUT, NONFINITE, CUDA_ERROR, TIMEOUT, NO_DEVICE, NO_PROBLEM = range(8)
STANDARD, DESCENT, CONJUGATED, APGD, SPG = range(5)            # projected_gradient::Variant
PURE_NEWTON, PURE_ENUMERATIVE, HYBRID, REV_HYBRID = range(4)   # local_soc_solver::Strategy
ADMM_STANDARD, ADMM_ACCELERATED = range(2)                     # admm::Variant
# MecheFrictionProblem::Algorithm
MECHE_GAUSS_SEIDEL, MECHE_PROJECTED_GRADIENT, MECHE_MATRIX_FREE_GAUSS_SEIDEL, MECHE_ADMM, MECHE_DUAL_AMA = range(5)


class BogusGpuError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"bogus_gpu status {status}: {message}")
        self.status = status


class PgOptions(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_uint), ("ls_iters", C.c_uint),
                ("ls_optimistic_factor", C.c_double), ("ls_pessimistic_factor", C.c_double),
                ("ls_armijo_coefficient", C.c_double), ("variant", C.c_int), ("use_infinity_norm", C.c_int),
                ("static_problem", C.c_int), ("mixed_precision", C.c_int), ("refine_max_iters", C.c_uint),
                ("momentum_by_linearity", C.c_int), ("fp32_stall_iters", C.c_uint),
                ("fp32_products_refresh", C.c_uint)]


class GsOptions(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_uint), ("eval_every", C.c_uint), ("skip_tol", C.c_double),
                ("skip_iters", C.c_uint), ("auto_regularization", C.c_double), ("try_zero_as_well", C.c_int),
                ("use_infinity_norm", C.c_int), ("static_problem", C.c_int), ("local_strategy", C.c_int),
                ("use_coloring", C.c_int)]


class AdmmOptions(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_uint), ("step_size", C.c_double), ("variant", C.c_int),
                ("use_infinity_norm", C.c_int)]


class DualAmaOptions(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_uint), ("fp_step_size", C.c_double),
                ("proj_step_size", C.c_double), ("ls_iters", C.c_uint), ("ls_optimistic_factor", C.c_double),
                ("ls_pessimistic_factor", C.c_double), ("variant", C.c_int), ("use_infinity_norm", C.c_int)]


class AdjointOptions(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iters", C.c_uint), ("coulomb", C.c_int)]


class MecheOptions(C.Structure):
    """MecheFrictionProblem::Options (Interfaces/MecheInterface.hpp:44-69) with the reference's defaults."""
    _fields_ = [("maxThreads", C.c_int), ("maxIters", C.c_uint), ("cadouxIters", C.c_uint), ("tolerance", C.c_double),
                ("useInfinityNorm", C.c_int), ("algorithm", C.c_int), ("gsRegularization", C.c_double),
                ("gsColoring", C.c_int), ("gsSkipIters", C.c_int), ("tryZeroAsWell", C.c_int),
                ("pgVariant", C.c_int), ("admmProjStepSize", C.c_double), ("admmFpStepSize", C.c_double)]

    def __init__(self):
        super().__init__()
        lib().bogus_gpu_meche_options_default(C.byref(self))


class BatchShape(C.Structure):
    _fields_ = [("schedule", C.c_int), ("ctas_per_sm", C.c_int), ("team_size", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("kernel_launches", C.c_uint), ("iterations", C.c_uint),
                ("w_passes", C.c_uint), ("algorithmic_bytes", C.c_double), ("fp64_fma", C.c_double),
                ("refine_iterations", C.c_uint), ("fp32_device_ms", C.c_double),
                ("fp32_product_iterations", C.c_uint)]


CALLBACK = C.CFUNCTYPE(None, C.c_uint, C.c_double, C.c_void_p)

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = None

EXPORTED = [
    "bogus_gpu_pg_options_default", "bogus_gpu_gs_options_default", "bogus_gpu_status_string",
    "bogus_gpu_last_error", "bogus_gpu_create", "bogus_gpu_destroy", "bogus_gpu_set_dual",
    "bogus_gpu_set_dual_device", "bogus_gpu_nnzb", "bogus_gpu_set_callback", "bogus_gpu_spmv", "bogus_gpu_eval",
    "bogus_gpu_solve_pg", "bogus_gpu_solve_pg_device", "bogus_gpu_solve_gs", "bogus_gpu_coloring",
    "bogus_gpu_set_primal", "bogus_gpu_assemble_dual", "bogus_gpu_get_dual_lower", "bogus_gpu_get_solve_stats",
    "bogus_gpu_get_stream", "bogus_gpu_measure_fp64_peak", "bogus_gpu_check_fp64_ops", "bogus_gpu_solve_pg_noalloc",
    "bogus_gpu_set_batch", "bogus_gpu_solve_pg_batch", "bogus_gpu_solve_pg_batch_device",
    "bogus_gpu_admm_options_default", "bogus_gpu_solve_admm", "bogus_gpu_adjoint_options_default",
    "bogus_gpu_adjoint", "bogus_gpu_adjoint_device", "bogus_gpu_adjoint_dual_lower", "bogus_gpu_adjoint_primal",
    "bogus_gpu_add_compliance", "bogus_gpu_solve_cadoux_gs", "bogus_gpu_solve_cadoux_pg",
    "bogus_gpu_meche_options_default", "bogus_gpu_meche_from_primal", "bogus_gpu_meche_solve",
    "bogus_gpu_solve_product_gs", "bogus_gpu_dual_ama_options_default", "bogus_gpu_solve_dual_ama",
    "bogus_gpu_set_body_dofs", "bogus_gpu_set_frames", "bogus_gpu_apply_permutation", "bogus_gpu_undo_permutation", "bogus_gpu_permuted",
    "bogus_gpu_set_wait_limit", "bogus_gpu_test_wait_timeout", "bogus_gpu_get_dual_rhs",
    "bogus_gpu_set_batch_tuning", "bogus_gpu_set_batch_shape", "bogus_gpu_get_batch_shape",
    "bogus_gpu_get_batch_tuning_log", "bogus_gpu_solve_pg_batch_graph",
]


def lib():
    """Loads libbogus_gpu.so (raises ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libbogus_gpu.so is not built ({LIB_PATH}); run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.bogus_gpu_pg_options_default.argtypes = [C.POINTER(PgOptions)]
    L.bogus_gpu_gs_options_default.argtypes = [C.POINTER(GsOptions)]
    L.bogus_gpu_status_string.restype = C.c_char_p
    L.bogus_gpu_status_string.argtypes = [C.c_int]
    L.bogus_gpu_last_error.restype = C.c_char_p
    L.bogus_gpu_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.bogus_gpu_destroy.argtypes = [vp]
    L.bogus_gpu_set_dual.argtypes = [vp, C.c_int, _ip, vp, vp, C.c_int, _dp, _dp]
    L.bogus_gpu_set_dual_device.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp]
    L.bogus_gpu_nnzb.argtypes = [vp, C.POINTER(C.c_int)]
    L.bogus_gpu_set_callback.argtypes = [vp, CALLBACK, vp]
    L.bogus_gpu_spmv.argtypes = [vp, _dp, _dp]
    L.bogus_gpu_eval.argtypes = [vp, _dp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.bogus_gpu_solve_pg.argtypes = [vp, C.POINTER(PgOptions), _dp, C.POINTER(C.c_double), C.POINTER(C.c_uint)]
    L.bogus_gpu_solve_pg_device.argtypes = [vp, C.POINTER(PgOptions), vp, C.POINTER(C.c_double), C.POINTER(C.c_uint)]
    L.bogus_gpu_solve_gs.argtypes = [vp, C.POINTER(GsOptions), _dp, C.POINTER(C.c_double), C.POINTER(C.c_uint)]
    L.bogus_gpu_coloring.argtypes = [vp, _ip, _ip, C.POINTER(C.c_int)]
    L.bogus_gpu_set_primal.argtypes = [vp, C.c_int, C.c_int, _dp, C.c_int, _ip, _ip, _dp, _dp]
    L.bogus_gpu_assemble_dual.argtypes = [vp, vp, _dp, _dp]
    L.bogus_gpu_get_dual_lower.argtypes = [vp, vp, vp, vp, C.POINTER(C.c_int)]
    L.bogus_gpu_get_solve_stats.argtypes = [vp, C.POINTER(SolveStats)]
    L.bogus_gpu_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.bogus_gpu_measure_fp64_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.bogus_gpu_check_fp64_ops.argtypes = [C.c_int, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    L.bogus_gpu_set_batch.argtypes = [vp, C.c_int, _ip]
    L.bogus_gpu_adjoint_options_default.argtypes = [C.POINTER(AdjointOptions)]
    L.bogus_gpu_adjoint_options_default.restype = None
    L.bogus_gpu_adjoint.argtypes = [vp, C.POINTER(AdjointOptions), _dp, _dp, _dp, _dp, C.POINTER(C.c_double),
                                    C.POINTER(C.c_uint)]
    L.bogus_gpu_adjoint_device.argtypes = [vp, C.POINTER(AdjointOptions), vp, vp, vp, vp, C.POINTER(C.c_double),
                                           C.POINTER(C.c_uint)]
    L.bogus_gpu_adjoint_dual_lower.argtypes = [vp, _dp]
    L.bogus_gpu_adjoint_primal.argtypes = [vp, vp, vp, vp, vp, vp]
    L.bogus_gpu_add_compliance.argtypes = [vp, _dp]
    L.bogus_gpu_solve_cadoux_gs.argtypes = [vp, C.POINTER(GsOptions), _dp, C.c_uint, C.POINTER(C.c_double),
                                            C.POINTER(C.c_uint)]
    L.bogus_gpu_solve_cadoux_pg.argtypes = [vp, C.POINTER(PgOptions), _dp, C.c_uint, C.POINTER(C.c_double),
                                            C.POINTER(C.c_uint)]
    L.bogus_gpu_meche_options_default.argtypes = [C.POINTER(MecheOptions)]
    L.bogus_gpu_meche_options_default.restype = None
    L.bogus_gpu_meche_from_primal.argtypes = [vp, C.c_uint, np.ctypeslib.ndpointer(dtype=np.uint32),
                                              C.POINTER(C.c_void_p), vp, C.c_uint, _dp, _dp, _dp, _ip, _ip,
                                              C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    L.bogus_gpu_meche_solve.argtypes = [vp, _dp, vp, C.POINTER(MecheOptions), C.c_int, C.c_double,
                                        C.POINTER(C.c_double)]
    L.bogus_gpu_solve_product_gs.argtypes = [vp, C.POINTER(GsOptions), vp, _dp, _dp, _dp, C.POINTER(C.c_double),
                                             C.POINTER(C.c_uint)]
    L.bogus_gpu_admm_options_default.argtypes = [C.POINTER(AdmmOptions)]
    L.bogus_gpu_admm_options_default.restype = None
    L.bogus_gpu_solve_admm.argtypes = [vp, C.POINTER(AdmmOptions), C.c_double, vp, vp, _dp, _dp, _dp, _dp,
                                       C.POINTER(C.c_double), C.POINTER(C.c_uint)]
    L.bogus_gpu_dual_ama_options_default.argtypes = [C.POINTER(DualAmaOptions)]
    L.bogus_gpu_dual_ama_options_default.restype = None
    L.bogus_gpu_solve_dual_ama.argtypes = [vp, C.POINTER(DualAmaOptions), _dp, vp, _dp, _dp, C.c_int, _dp, _dp,
                                           C.POINTER(C.c_double), C.POINTER(C.c_uint)]
    L.bogus_gpu_set_body_dofs.argtypes = [vp, _ip]
    L.bogus_gpu_set_frames.argtypes = [vp, _dp]
    L.bogus_gpu_apply_permutation.argtypes = [vp, _ip]
    L.bogus_gpu_undo_permutation.argtypes = [vp]
    L.bogus_gpu_permuted.argtypes = [vp, C.POINTER(C.c_int)]
    L.bogus_gpu_solve_pg_batch.argtypes = [vp, C.POINTER(PgOptions), _dp, _dp, np.ctypeslib.ndpointer(dtype=np.uint32)]
    L.bogus_gpu_solve_pg_batch_device.argtypes = [vp, C.POINTER(PgOptions), vp, _dp,
                                                  np.ctypeslib.ndpointer(dtype=np.uint32)]
    L.bogus_gpu_solve_pg_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, C.POINTER(PgOptions), vp,
                                             C.POINTER(C.c_double), C.POINTER(C.c_uint), vp]
    L.bogus_gpu_set_wait_limit.argtypes = [C.c_int, C.c_double]
    L.bogus_gpu_test_wait_timeout.argtypes = [vp, C.c_int]
    L.bogus_gpu_get_dual_rhs.argtypes = [vp, vp, vp]
    L.bogus_gpu_set_batch_tuning.argtypes = [vp, C.c_int]
    L.bogus_gpu_set_batch_shape.argtypes = [vp, C.POINTER(BatchShape)]
    L.bogus_gpu_get_batch_shape.argtypes = [vp, C.POINTER(BatchShape)]
    L.bogus_gpu_get_batch_tuning_log.argtypes = [vp, vp, vp, C.POINTER(C.c_int)]
    L.bogus_gpu_solve_pg_batch_graph.argtypes = [vp, C.POINTER(PgOptions), vp, _dp,
                                                 np.ctypeslib.ndpointer(dtype=np.uint32)]
    _lib = L
    return L


def _check(status: int, allow_not_converged: bool = True) -> int:
    if status == OK or (allow_not_converged and status == NOT_CONVERGED):
        return status
    L = lib()
    raise BogusGpuError(status, f"{L.bogus_gpu_status_string(status).decode()}: {L.bogus_gpu_last_error().decode()}")


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


class Signal:
    """Signal<unsigned, double> (Core/Utils/Signal.hpp): listeners receive (iteration, residual)."""

    def __init__(self):
        self._callees = []

    def connect(self, fn) -> None:
        self._callees.append(fn)

    def disconnectAll(self) -> None:
        self._callees.clear()

    def trigger(self, it: int, res: float) -> None:
        for fn in self._callees:
            fn(it, res)


class _SolverBase:
    def __init__(self, tol: float, max_iters: int):
        self._tol = tol
        self._max_iters = max_iters
        self._inf = False
        self._callback = Signal()

    def setTol(self, tol: float) -> None: self._tol = float(tol)
    def tol(self) -> float: return self._tol
    def setMaxIters(self, n: int) -> None: self._max_iters = int(n)
    def maxIters(self) -> int: return self._max_iters
    def useInfinityNorm(self, on: bool) -> None: self._inf = bool(on)
    def usesInfinityNorm(self) -> bool: return self._inf
    def callback(self) -> Signal: return self._callback


class ProjectedGradient(_SolverBase):
    """ProjectedGradient<WType> (Core/BlockSolvers/ProjectedGradient.hpp:21-107): tol 1e-6, 300 iterations,
    8 line-search iterations, factors 1.25 / 0.5 / 0.5, APGD."""

    def __init__(self):
        super().__init__(1e-6, 300)
        self._ls = 8
        self._opt, self._pess, self._armijo = 1.25, 0.5, 0.5
        self._variant = APGD
        self._mixed, self._refine = False, 50
        self._lin = False
        self._stall = 4
        self._hy = 0

    def setMomentumByLinearity(self, on: bool = True) -> None:
        """APGD's momentum product formed by linearity, W x = W xs + beta (W xs - W prev), instead of the product
        W x of ProjectedGradient.impl.hpp:141: one pass over W fewer per momentum step, iterates that differ
        from the reference's by rounding. No counterpart in the reference."""
        self._lin = bool(on)

    def setMixedPrecision(self, on: bool = True, refine_max_iters: int = 50) -> None:
        """FP32-refined solve: FP32 W / iterates / per-contact law (FP64 reductions and decisions), then up to
        refine_max_iters FP64 iterations from the FP32 result. No counterpart in the reference."""
        self._mixed, self._refine = bool(on), int(refine_max_iters)

    def setFp32StallIterations(self, n: int) -> None:
        """FP32-refined solve: end the FP32 part once its residual has repeated bit for bit on n consecutive
        iterations or its line search has run out of trials n times in a row (0: run it to max_iters). No
        counterpart in the reference."""
        self._stall = int(n)

    def setFp32CorrectionProducts(self, refresh: int = 100) -> None:
        """FP32-refined solve: the FP64 iterations after the FP32 part form their products as
        W x_ref + W32 (v - x_ref) (FP32 correction, FP64 iterates and law), x_ref refreshed every `refresh`
        iterations, then a plain FP64 solve checks the tolerance (0: plain FP64 iterations). APGD only. No
        counterpart in the reference."""
        self._hy = int(refresh)

    def setLineSearchIterations(self, n: int) -> None: self._ls = int(n)
    def setLineSearchOptimisticFactor(self, f: float) -> None: self._opt = float(f)
    def setLineSearchPessimisticFactor(self, f: float) -> None: self._pess = float(f)
    def setLineSearchArmijoCoefficient(self, f: float) -> None: self._armijo = float(f)
    def setDefaultVariant(self, v: int) -> None: self._variant = int(v)
    def lineSearchIterations(self) -> int: return self._ls

    def options(self, static_problem: bool) -> PgOptions:
        o = PgOptions()
        lib().bogus_gpu_pg_options_default(C.byref(o))
        o.tol, o.max_iters, o.ls_iters = self._tol, self._max_iters, self._ls
        o.ls_optimistic_factor, o.ls_pessimistic_factor, o.ls_armijo_coefficient = self._opt, self._pess, self._armijo
        o.variant, o.use_infinity_norm, o.static_problem = self._variant, int(self._inf), int(static_problem)
        o.mixed_precision, o.refine_max_iters = int(self._mixed), self._refine
        o.momentum_by_linearity = int(self._lin)
        o.fp32_stall_iters = self._stall
        o.fp32_products_refresh = self._hy
        return o


class Coloring:
    """GaussSeidel::coloring() (Core/BlockSolvers/Coloring.hpp): update(True) selects the order of
    Coloring::compute with the contact permutation (as MecheFrictionProblem::solve does with several threads);
    update(False) — the default — sweeps the contacts in their own order."""

    def __init__(self):
        self.enabled = False

    def update(self, enable: bool, matrix=None) -> None:
        self.enabled = bool(enable)


class GaussSeidel(_SolverBase):
    """GaussSeidel<WType> (Core/BlockSolvers/GaussSeidel.hpp, GaussSeidelBase.hpp:39-91): tol 1e-6,
    250 sweeps, evalEvery 25, skipTol 1e-6, skipIters 10, tryZeroAsWell; the sequential sweep of the reference,
    run on the GPU as one launch in which each contact waits only for its earlier neighbours (same result)."""

    def __init__(self):
        super().__init__(1e-6, 250)
        self._eval_every, self._skip_tol, self._skip_iters = 25, 1e-6, 10
        self._auto_reg, self._try_zero = 0.0, True
        self._strategy = REV_HYBRID
        self._coloring = Coloring()

    def coloring(self) -> Coloring:
        return self._coloring

    def setEvalEvery(self, n: int) -> None: self._eval_every = int(n)
    def setSkipTol(self, t: float) -> None: self._skip_tol = float(t)
    def setSkipIters(self, n: int) -> None: self._skip_iters = int(n)
    def setAutoRegularization(self, r: float) -> None: self._auto_reg = float(r)
    def doTryZeroAsWell(self, on: bool = True) -> None: self._try_zero = bool(on)
    def setLocalStrategy(self, s: int) -> None:
        """SOCLaw's Strat template argument (default RevHybrid)."""
        self._strategy = int(s)

    def options(self, static_problem: bool) -> GsOptions:
        o = GsOptions()
        lib().bogus_gpu_gs_options_default(C.byref(o))
        o.tol, o.max_iters, o.eval_every = self._tol, self._max_iters, self._eval_every
        o.skip_tol, o.skip_iters, o.auto_regularization = self._skip_tol, self._skip_iters, self._auto_reg
        o.try_zero_as_well, o.use_infinity_norm = int(self._try_zero), int(self._inf)
        o.static_problem, o.local_strategy = int(static_problem), self._strategy
        o.use_coloring = int(self._coloring.enabled)
        return o


class ProductGaussSeidel(GaussSeidel):
    """ProductGaussSeidel<HType, MInvType, true> (Core/BlockSolvers/ProductGaussSeidel.hpp): Gauss-Seidel on
    W = H M^-1 H^T without forming W, for PrimalFrictionProblem.solveWith(pgs, r, staticProblem). Same setters and
    defaults as GaussSeidel; the contacts are swept in their own order."""


class ADMM(_SolverBase):
    """ADMM<HType> (Core/BlockSolvers/ADMM.hpp:41-110): tol 1e-6, 300 iterations, step size 1e-2,
    Accelerated variant."""

    def __init__(self):
        super().__init__(1e-6, 300)
        self._step = 1e-2
        self._variant = ADMM_ACCELERATED

    def setStepSize(self, s: float) -> None: self._step = float(s)
    def stepSize(self) -> float: return self._step
    def setDefaultVariant(self, v: int) -> None: self._variant = int(v)

    def options(self) -> "AdmmOptions":
        o = AdmmOptions()
        lib().bogus_gpu_admm_options_default(C.byref(o))
        o.tol, o.max_iters, o.step_size = self._tol, self._max_iters, self._step
        o.variant, o.use_infinity_norm = self._variant, int(self._inf)
        return o


class DualAMA(_SolverBase):
    """DualAMA<HType> (Core/BlockSolvers/ADMM.hpp:170-236): tol 1e-6, 300 iterations, fp step size 1e-1,
    projection step size 1e-1, 6 line-search iterations (factors 1.25 / 0.5), Accelerated variant."""

    def __init__(self):
        super().__init__(1e-6, 300)
        self._fp, self._proj = 1e-1, 1e-1
        self._ls, self._opt, self._pess = 6, 1.25, .5
        self._variant = ADMM_ACCELERATED

    def setFpStepSize(self, s: float) -> None: self._fp = float(s)
    def setProjStepSize(self, s: float) -> None: self._proj = float(s)
    def setLineSearchIterations(self, n: int) -> None: self._ls = int(n)
    def setLineSearchOptimisticFactor(self, f: float) -> None: self._opt = float(f)
    def setLineSearchPessimisticFactor(self, f: float) -> None: self._pess = float(f)
    def setDefaultVariant(self, v: int) -> None: self._variant = int(v)
    def fpStepSize(self) -> float: return self._fp
    def projStepSize(self) -> float: return self._proj

    def options(self) -> "DualAmaOptions":
        o = DualAmaOptions()
        lib().bogus_gpu_dual_ama_options_default(C.byref(o))
        o.tol, o.max_iters, o.fp_step_size, o.proj_step_size = self._tol, self._max_iters, self._fp, self._proj
        o.ls_iters, o.ls_optimistic_factor, o.ls_pessimistic_factor = self._ls, self._opt, self._pess
        o.variant, o.use_infinity_norm = self._variant, int(self._inf)
        return o


class PrimalFrictionProblem:
    """PrimalFrictionProblem<3> for rigid bodies (Interfaces/FrictionProblem.hpp:55-116): M^-1 blocks,
    per-contact Jacobian blocks for one or two bodies, f, w (local contact basis), mu. The arrays are uploaded
    to the GPU on the first solveWith; call invalidate() after changing them. M: the mass blocks (DualAMA needs
    them; computeMInv(M) sets both). body_dofs: the bodies' own dof counts when they are padded to ndof (the
    reference's H has column blocks of varying width); default ndof each. E: per-contact frames (n, 3, 3),
    contact basis to world; w is then in world coordinates (default: E = I, w in the contact basis)."""

    def __init__(self, minv, objA, objB, HA, HB, w, mu, f=None, device: int = 0, M=None, body_dofs=None, E=None):
        self.minv = _f64(minv)
        self.E = None if E is None else _f64(E).reshape(-1, 3, 3)
        self.M = None if M is None else _f64(M)
        self.body_dofs = None if body_dofs is None else _i32(body_dofs)
        self.objA, self.objB = _i32(objA), _i32(objB)
        self.HA, self.HB = _f64(HA), _f64(HB)
        self.w, self.mu = _f64(w).reshape(-1), _f64(mu).reshape(-1)
        self.f = None if f is None else _f64(f).reshape(-1)
        self._device = int(device)
        self._gpu = None
        self.last_status = self.last_iterations = None

    def invalidate(self) -> None:
        self._gpu = None

    def _uploaded(self) -> "DualFrictionProblem":
        if self._gpu is None:
            g = DualFrictionProblem(self._device)
            nb, ndof = self.minv.shape[0], self.minv.shape[1]
            _check(lib().bogus_gpu_set_primal(g.handle, nb, ndof, self.minv.reshape(-1), self.objA.size, self.objA,
                                              self.objB, self.HA.reshape(-1), self.HB.reshape(-1)), False)
            if self.body_dofs is not None:
                _check(lib().bogus_gpu_set_body_dofs(g.handle, self.body_dofs), False)
            if self.E is not None:
                if self.E.shape[0] != self.objA.size:
                    raise ValueError("E must hold one 3 x 3 frame per contact")
                _check(lib().bogus_gpu_set_frames(g.handle, self.E.reshape(-1)), False)
            self._gpu = g
        return self._gpu

    def solveWith(self, solver, *args, **kwargs) -> float:
        """PrimalFrictionProblem::solveWith:
        - solveWith(ADMM, lambda_, v, r, prox=None): primal ADMM (see _solve_admm);
        - solveWith(ProductGaussSeidel, r, staticProblem=False): the matrix-free Gauss-Seidel;
        - solveWith(DualAMA, v, r, staticProblem=False): the dual AMA solver (see _solve_dual_ama)."""
        if isinstance(solver, ProductGaussSeidel):
            return self._solve_product_gs(solver, *args, **kwargs)
        if isinstance(solver, DualAMA):
            return self._solve_dual_ama(solver, *args, **kwargs)
        return self._solve_admm(solver, *args, **kwargs)

    def _solve_dual_ama(self, dama: "DualAMA", v, r, staticProblem: bool = False) -> float:
        """PrimalFrictionProblem::solveWith(DualAMAType&, v, r, staticProblem): v (nbodies * ndof) and r (3n) are
        solved in place (float64, C-contiguous; the iterate of least residual); returns the residual."""
        for a, name in ((v, "v"), (r, "r")):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise TypeError(f"{name} must be a C-contiguous float64 numpy array (solved in place)")
        if v.size != self.minv.shape[0] * self.minv.shape[1] or r.size != 3 * self.objA.size:
            raise ValueError("inconsistent v / r sizes")
        if self.M is None:
            raise ValueError("DualAMA needs the mass blocks M (constructor argument or computeMInv(M))")
        g = self._uploaded()
        g._bind(dama)
        o = dama.options()
        res = C.c_double()
        it = C.c_uint()
        fptr = None if self.f is None else self.f.ctypes.data_as(C.c_void_p)
        st = lib().bogus_gpu_solve_dual_ama(g.handle, C.byref(o), self.M.reshape(-1), fptr, self.w, self.mu,
                                            int(bool(staticProblem)), v.reshape(-1), r.reshape(-1), C.byref(res),
                                            C.byref(it))
        _check(st)
        self.last_status, self.last_iterations = st, it.value
        return res.value

    def _solve_product_gs(self, gs: "ProductGaussSeidel", r, staticProblem: bool = False) -> float:
        if not (isinstance(r, np.ndarray) and r.dtype == np.float64 and r.flags.c_contiguous):
            raise TypeError("r must be a C-contiguous float64 numpy array (solved in place)")
        if r.size != 3 * self.objA.size:
            raise ValueError("inconsistent r size")
        g = self._uploaded()
        g._bind(gs)
        o = gs.options(staticProblem)
        o.use_coloring = 0
        res = C.c_double()
        it = C.c_uint()
        fptr = None if self.f is None else self.f.ctypes.data_as(C.c_void_p)
        st = lib().bogus_gpu_solve_product_gs(g.handle, C.byref(o), fptr, self.w, self.mu, r.reshape(-1),
                                              C.byref(res), C.byref(it))
        _check(st)
        self.last_status, self.last_iterations = st, it.value
        return res.value

    def _solve_admm(self, admm: "ADMM", lambda_: float, v, r, prox=None) -> float:
        """PrimalFrictionProblem::solveWith(ADMMType&, lambda, v, r): v (nbodies * ndof) and r (3n) are solved in
        place (float64, C-contiguous); returns the residual. prox: the QuadraticProxOp operator blocks
        [nbodies, ndof, ndof] of ADMM::solve(law, op, w, v, r) (default M^-1, as the reference passes)."""
        for a, name in ((v, "v"), (r, "r")):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise TypeError(f"{name} must be a C-contiguous float64 numpy array (solved in place)")
        if v.size != self.minv.shape[0] * self.minv.shape[1] or r.size != 3 * self.objA.size:
            raise ValueError("inconsistent v / r sizes")
        g = self._uploaded()
        g._bind(admm)
        o = admm.options()
        res = C.c_double()
        it = C.c_uint()
        fptr = None if self.f is None else self.f.ctypes.data_as(C.c_void_p)
        pb = None if prox is None else _f64(prox).reshape(-1)
        if pb is not None and pb.size != self.minv.size:
            raise ValueError("prox must hold nbodies x ndof x ndof blocks")
        pptr = None if pb is None else pb.ctypes.data_as(C.c_void_p)
        st = lib().bogus_gpu_solve_admm(g.handle, C.byref(o), float(lambda_), pptr, fptr, self.w, self.mu,
                                         v.reshape(-1), r.reshape(-1), C.byref(res), C.byref(it))
        _check(st)
        self.last_status, self.last_iterations = st, it.value
        return res.value

    def solve_stats(self) -> dict:
        return self._uploaded().solve_stats()

    @classmethod
    def from_generated(cls, data) -> "PrimalFrictionProblem":
        """Wraps generator.PrimalData: w = b (free velocity, f = 0)."""
        return cls(data.minv, data.objA, data.objB, data.HA, data.HB, data.b, data.mu)

    def computeMInv(self, M) -> None:
        """Sets the mass blocks M[nbodies, ndof, ndof] and their inverses (PrimalFrictionProblem::computeMInv)."""
        self.M = _f64(M).copy()
        self.minv = _f64(np.linalg.inv(self.M))


class DualFrictionProblem:
    """DualFrictionProblem<3> (Interfaces/FrictionProblem.hpp:127-214) held on one GPU."""

    def __init__(self, device: int = 0):
        L = lib()
        h = C.c_void_p()
        _check(L.bogus_gpu_create(int(device), C.byref(h)), False)
        self._h = h
        self.n = 0
        self._cb_keep = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.bogus_gpu_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def set(self, rowptr, col, blocks, b, mu, symmetric_lower: bool = True) -> None:
        """Sets W (3x3-block BSR, lower triangle by default), b and mu from host arrays."""
        rowptr, col, blocks = _i32(rowptr), _i32(col), _f64(blocks).reshape(-1)
        b, mu = _f64(b).reshape(-1), _f64(mu).reshape(-1)
        n = len(rowptr) - 1
        if b.size != 3 * n or mu.size != n or blocks.size != 9 * col.size:
            raise ValueError("inconsistent W / b / mu sizes")
        _check(lib().bogus_gpu_set_dual(self._h, n, rowptr, col.ctypes.data_as(C.c_void_p),
                                        blocks.ctypes.data_as(C.c_void_p), int(symmetric_lower), b, mu), False)
        self.n = n

    def computeFrom(self, primal: PrimalFrictionProblem) -> None:
        """W = H M^-1 H^T and b = E^T w - H M^-1 f on the GPU (DualFrictionProblem::computeFrom)."""
        L = lib()
        nb, ndof = primal.minv.shape[0], primal.minv.shape[1]
        n = primal.objA.size
        _check(L.bogus_gpu_set_primal(self._h, nb, ndof, primal.minv.reshape(-1), n, primal.objA, primal.objB,
                                      primal.HA.reshape(-1), primal.HB.reshape(-1)), False)
        if primal.E is not None:
            _check(L.bogus_gpu_set_frames(self._h, primal.E.reshape(-1)), False)
        fptr = None if primal.f is None else primal.f.ctypes.data_as(C.c_void_p)
        _check(L.bogus_gpu_assemble_dual(self._h, fptr, primal.w, primal.mu), False)
        self.n = n

    def W_lower(self):
        """Lower triangle of W as (rowptr, col, blocks[nnzb, 3, 3])."""
        L = lib()
        nnz = C.c_int()
        _check(L.bogus_gpu_get_dual_lower(self._h, None, None, None, C.byref(nnz)), False)
        rp = np.zeros(self.n + 1, np.int32)
        cl = np.zeros(nnz.value, np.int32)
        vl = np.zeros(9 * nnz.value)
        _check(L.bogus_gpu_get_dual_lower(self._h, rp.ctypes.data_as(C.c_void_p), cl.ctypes.data_as(C.c_void_p),
                                          vl.ctypes.data_as(C.c_void_p), C.byref(nnz)), False)
        return rp, cl, vl.reshape(-1, 3, 3)

    def nnzb(self) -> int:
        v = C.c_int()
        _check(lib().bogus_gpu_nnzb(self._h, C.byref(v)), False)
        return v.value

    def applyPermutation(self, permutation) -> None:
        """DualFrictionProblem::applyPermutation: contact k of the stored problem becomes contact permutation[k];
        solveWith / evalWith keep taking r in the original order until undoPermutation()."""
        p = _i32(permutation)
        if p.size != self.n:
            raise ValueError("the permutation must have one entry per contact")
        _check(lib().bogus_gpu_apply_permutation(self._h, p), False)

    def undoPermutation(self) -> None:
        _check(lib().bogus_gpu_undo_permutation(self._h), False)

    def permuted(self) -> bool:
        out = C.c_int()
        _check(lib().bogus_gpu_permuted(self._h, C.byref(out)), False)
        return bool(out.value)

    def multiply(self, x) -> np.ndarray:
        """y = W x (the stored W: permuted while a permutation is applied)."""
        x = _f64(x).reshape(-1)
        y = np.zeros_like(x)
        _check(lib().bogus_gpu_spmv(self._h, x, y), False)
        return y

    def _bind(self, solver) -> None:
        sig = solver.callback()
        if sig._callees:
            cb = CALLBACK(lambda it, res, _u: sig.trigger(int(it), float(res)))
            self._cb_keep = cb
            lib().bogus_gpu_set_callback(self._h, cb, None)
        else:
            self._cb_keep = None
            lib().bogus_gpu_set_callback(self._h, CALLBACK(0), None)

    def solveWith(self, solver, r, staticProblem: bool | None = None) -> float:
        """Solves in place (r: float64 array of 3n entries, warm start and result); returns the residual.
        staticProblem defaults as in the reference: False for GaussSeidel, True for ProjectedGradient."""
        if not (isinstance(r, np.ndarray) and r.dtype == np.float64 and r.flags.c_contiguous):
            raise TypeError("r must be a C-contiguous float64 numpy array (solved in place)")
        res = C.c_double()
        it = C.c_uint()
        self._bind(solver)
        if isinstance(solver, GaussSeidel):
            sp = False if staticProblem is None else staticProblem
            o = solver.options(sp)
            st = lib().bogus_gpu_solve_gs(self._h, C.byref(o), r.reshape(-1), C.byref(res), C.byref(it))
        elif isinstance(solver, ProjectedGradient):
            sp = True if staticProblem is None else staticProblem
            o = solver.options(sp)
            st = lib().bogus_gpu_solve_pg(self._h, C.byref(o), r.reshape(-1), C.byref(res), C.byref(it))
        else:
            raise TypeError("solver must be GaussSeidel or ProjectedGradient")
        _check(st)
        self.last_status, self.last_iterations = st, it.value
        return res.value

    def solveCadoux(self, solver, r, cadouxIterations: int) -> float:
        """DualFrictionProblem::solveCadoux (Interfaces/FrictionProblem.impl.hpp:76-92): the Coulomb problem as a
        sequence of SOCQP solves with the De Saxce change of variable; r in place; returns the Coulomb error.
        The solver's callback fires once per fixed-point iteration."""
        if not (isinstance(r, np.ndarray) and r.dtype == np.float64 and r.flags.c_contiguous):
            raise TypeError("r must be a C-contiguous float64 numpy array (solved in place)")
        res = C.c_double()
        it = C.c_uint()
        self._bind(solver)
        if isinstance(solver, GaussSeidel):
            o = solver.options(True)
            st = lib().bogus_gpu_solve_cadoux_gs(self._h, C.byref(o), r.reshape(-1), int(cadouxIterations),
                                                 C.byref(res), C.byref(it))
        elif isinstance(solver, ProjectedGradient):
            o = solver.options(True)
            st = lib().bogus_gpu_solve_cadoux_pg(self._h, C.byref(o), r.reshape(-1), int(cadouxIterations),
                                                 C.byref(res), C.byref(it))
        else:
            raise TypeError("solver must be GaussSeidel or ProjectedGradient")
        _check(st)
        self.last_status, self.last_iterations = st, it.value
        return res.value

    def evalWith(self, solver, r, staticProblem: bool | None = None) -> float:
        """Error function at r with the solver's norm (DualFrictionProblem::evalWith)."""
        sp = staticProblem
        if sp is None:
            sp = isinstance(solver, ProjectedGradient)
        res = C.c_double()
        _check(lib().bogus_gpu_eval(self._h, _f64(r).reshape(-1), int(sp), int(solver.usesInfinityNorm()),
                                    C.byref(res)), False)
        return res.value

    # ---- adjoint of the SOC solve (no counterpart in the reference) ----
    def adjoint(self, r, dL_dr, tol: float = 1e-10, max_iters: int = 5000, coulomb: bool = False):
        """Implicit-function gradients at the solution r of the SOC problem (or, coulomb=True, of the Coulomb
        problem): returns (dL/db [3n], dL/dmu [n]); the final relative residual of the linear solve is in
        self.last_adjoint_residual."""
        o = AdjointOptions()
        lib().bogus_gpu_adjoint_options_default(C.byref(o))
        o.tol, o.max_iters, o.coulomb = float(tol), int(max_iters), int(bool(coulomb))
        db = np.zeros(3 * self.n)
        dmu = np.zeros(self.n)
        res = C.c_double()
        it = C.c_uint()
        st = lib().bogus_gpu_adjoint(self._h, C.byref(o), _f64(r).reshape(-1), _f64(dL_dr).reshape(-1), db, dmu,
                                     C.byref(res), C.byref(it))
        _check(st)
        self.last_adjoint_residual, self.last_adjoint_iterations = res.value, it.value
        return db, dmu

    def adjoint_dual_lower(self) -> np.ndarray:
        """dL/dW for the stored lower blocks of the last adjoint, [nnzb_lower, 3, 3]."""
        nnz = C.c_int()
        _check(lib().bogus_gpu_get_dual_lower(self._h, None, None, None, C.byref(nnz)), False)
        out = np.zeros(9 * nnz.value)
        _check(lib().bogus_gpu_adjoint_dual_lower(self._h, out), False)
        return out.reshape(-1, 3, 3)

    def adjoint_primal(self, primal: "PrimalFrictionProblem"):
        """dL/dHA, dL/dHB, dL/dw, dL/df of the last adjoint, for W and b assembled from `primal`."""
        n, nb, d = primal.objA.size, primal.minv.shape[0], primal.minv.shape[1]
        dHA = np.zeros((n, 3, d))
        dHB = np.zeros((n, 3, d))
        dw = np.zeros(3 * n)
        df = np.zeros(nb * d)
        fptr = None if primal.f is None else primal.f.ctypes.data_as(C.c_void_p)
        _check(lib().bogus_gpu_adjoint_primal(self._h, fptr, dHA.ctypes.data_as(C.c_void_p),
                                              dHB.ctypes.data_as(C.c_void_p), dw.ctypes.data_as(C.c_void_p),
                                              df.ctypes.data_as(C.c_void_p)), False)
        return dHA, dHB, dw, df

    def add_compliance(self, c) -> None:
        """W_ii += c_i I (c: one value per contact, or a scalar)."""
        c = np.broadcast_to(_f64(c), (self.n,)).copy()
        _check(lib().bogus_gpu_add_compliance(self._h, c), False)

    def coloring(self):
        perm = np.zeros(self.n, np.int32)
        colors = np.zeros(self.n + 1, np.int32)
        nc = C.c_int()
        _check(lib().bogus_gpu_coloring(self._h, perm, colors, C.byref(nc)), False)
        return perm, colors[: nc.value + 1]

    def solve_stats(self) -> dict:
        """Device time, launches, W passes, algorithmic bytes and FP64 FMAs of the last solve."""
        st = SolveStats()
        _check(lib().bogus_gpu_get_solve_stats(self._h, C.byref(st)), False)
        return {k: getattr(st, k) for k, _ in SolveStats._fields_}

    def stream(self) -> int:
        """The cudaStream_t (as an integer) this problem's kernels run on."""
        v = C.c_void_p()
        _check(lib().bogus_gpu_get_stream(self._h, C.byref(v)), False)
        return v.value or 0

    def solve_pg_device(self, solver: "ProjectedGradient", d_r_ptr: int, staticProblem: bool = True):
        """APGD / SPG with r already in device memory (pointer to 3n doubles); returns (residual, iterations)."""
        res = C.c_double()
        it = C.c_uint()
        self._bind(solver)
        o = solver.options(staticProblem)
        st = lib().bogus_gpu_solve_pg_device(self._h, C.byref(o), C.c_void_p(d_r_ptr), C.byref(res), C.byref(it))
        _check(st)
        self.last_status, self.last_iterations = st, it.value
        return res.value, it.value


    # ---- batches of independent problems -------------------------------------------------------------
    def setBatch(self, contact_ptr) -> None:
        """Marks W as block diagonal: problem p owns contacts [contact_ptr[p], contact_ptr[p+1])."""
        cp = _i32(contact_ptr)
        _check(lib().bogus_gpu_set_batch(self._h, cp.size - 1, cp), False)
        self.nproblems = cp.size - 1

    def solveBatchWith(self, solver: "ProjectedGradient", r, staticProblem: bool = True):
        """Solves every problem of the batch in one launch (r in place); returns (residuals, iterations)."""
        if not (isinstance(r, np.ndarray) and r.dtype == np.float64 and r.flags.c_contiguous):
            raise TypeError("r must be a C-contiguous float64 numpy array (solved in place)")
        res = np.zeros(self.nproblems)
        its = np.zeros(self.nproblems, np.uint32)
        o = solver.options(staticProblem)
        st = lib().bogus_gpu_solve_pg_batch(self._h, C.byref(o), r.reshape(-1), res, its)
        _check(st)
        self.last_status = st
        return res, its

    def solveBatch_device(self, solver: "ProjectedGradient", d_r_ptr: int, staticProblem: bool = True):
        res = np.zeros(self.nproblems)
        its = np.zeros(self.nproblems, np.uint32)
        o = solver.options(staticProblem)
        st = lib().bogus_gpu_solve_pg_batch_device(self._h, C.byref(o), C.c_void_p(d_r_ptr), res, its)
        _check(st)
        self.last_status = st
        return res, its

    def solveBatchGraph(self, solver: "ProjectedGradient", r_pinned, staticProblem: bool = True):
        """solveBatchWith through the captured CUDA graph (bogus_gpu_solve_pg_batch_graph): r_pinned is a float64
        array in page-locked memory (e.g. a pinned torch tensor's numpy view), solved in place."""
        res = np.zeros(self.nproblems)
        its = np.zeros(self.nproblems, np.uint32)
        o = solver.options(staticProblem)
        st = lib().bogus_gpu_solve_pg_batch_graph(self._h, C.byref(o), C.c_void_p(r_pinned.ctypes.data), res, its)
        _check(st)
        self.last_status = st
        return res, its

    def setBatchTuning(self, on: bool = True) -> None:
        """Tune the batched launch shape on the device at the next batched solve of each precision."""
        _check(lib().bogus_gpu_set_batch_tuning(self._h, int(bool(on))), False)

    def setBatchShape(self, schedule=None, ctas_per_sm: int = 0, team_size: int = 1) -> None:
        """Force the batched launch shape (schedule 0: one CTA per problem, 1: teams); None: back to the default."""
        if schedule is None:
            _check(lib().bogus_gpu_set_batch_shape(self._h, None), False)
            return
        sh = BatchShape(int(schedule), int(ctas_per_sm), int(team_size))
        _check(lib().bogus_gpu_set_batch_shape(self._h, C.byref(sh)), False)

    def batchShape(self) -> tuple:
        """(schedule, ctas_per_sm, team_size) of the last batched launch."""
        sh = BatchShape()
        _check(lib().bogus_gpu_get_batch_shape(self._h, C.byref(sh)), False)
        return sh.schedule, sh.ctas_per_sm, sh.team_size

    def batchTuningLog(self) -> list:
        """[((schedule, ctas_per_sm, team_size), ms), ...] measured by the last tuning."""
        k = C.c_int(0)
        _check(lib().bogus_gpu_get_batch_tuning_log(self._h, None, None, C.byref(k)), False)
        shapes = (BatchShape * max(1, k.value))()
        ms = np.zeros(max(1, k.value))
        _check(lib().bogus_gpu_get_batch_tuning_log(self._h, shapes, ms.ctypes.data_as(C.c_void_p), C.byref(k)), False)
        return [((shapes[i].schedule, shapes[i].ctas_per_sm, shapes[i].team_size), float(ms[i])) for i in range(k.value)]


def measure_fp64_peak(device: int = 0) -> float:
    """FP64 FMA throughput of the device in TFLOP/s (the ceiling of the FP64 kernels)."""
    v = C.c_double()
    _check(lib().bogus_gpu_measure_fp64_peak(int(device), C.byref(v)), False)
    return v.value


def check_fp64_ops(n: int, seed: int = 0, device: int = 0) -> tuple:
    """Mismatches (division, square root, scalings) of the integer-pipe FP64 operations against the GPU's IEEE
    operations on n generated operands; all zero when they are exact."""
    out = (C.c_longlong * 3)()
    _check(lib().bogus_gpu_check_fp64_ops(int(device), int(n), int(seed), out), False)
    return tuple(int(v) for v in out)


class MecheFrictionProblem:
    """MecheFrictionProblem (Interfaces/MecheInterface.hpp:40-170) on one GPU: fromPrimal() with world-coordinate
    data (contact frames E), solve(r, v, options, staticProblem, problemRegularization)."""

    def __init__(self, device: int = 0):
        self._dual = DualFrictionProblem(device)
        self._keep = None
        self.m = 0
        self.n = 0

    def fromPrimal(self, mass, f, mu, E, w, objA, objB, HA, HB) -> None:
        """mass: list of (ndof, ndof) arrays; f: (sum ndof) or None; mu: (n); E: (n, 3, 3) contact frames
        (world to local, E[i][a][b] as the reference's E blocks); w: (3n) world; objA / objB: (n) (-1: external);
        HA / HB: lists of (3, ndof) world Jacobian blocks (HB[i] None when objB[i] == -1)."""
        mass = [np.asfortranarray(np.asarray(m_, np.float64)) for m_ in mass]
        ndof = np.array([m_.shape[0] for m_ in mass], np.uint32)
        n = len(objA)
        E = np.asarray(E, np.float64).reshape(n, 3, 3)
        Ecm = np.zeros((3, 3 * n))
        for i in range(n):
            Ecm[:, 3 * i:3 * i + 3] = E[i].T
        HA = [np.asfortranarray(np.asarray(h, np.float64)) for h in HA]
        HB = [None if h is None else np.asfortranarray(np.asarray(h, np.float64)) for h in HB]
        fv = None if f is None else _f64(f).reshape(-1)
        mp = (C.c_void_p * len(mass))(*[m_.ctypes.data for m_ in mass])
        hap = (C.c_void_p * max(1, n))(*[h.ctypes.data for h in HA])
        hbp = (C.c_void_p * max(1, n))(*[0 if h is None else h.ctypes.data for h in HB])
        self._keep = (mass, HA, HB, fv)
        _check(lib().bogus_gpu_meche_from_primal(self._dual.handle, len(mass), ndof, mp,
                                                 None if fv is None else fv.ctypes.data_as(C.c_void_p), n,
                                                 _f64(mu), Ecm.ravel(), _f64(w).reshape(-1), _i32(objA), _i32(objB),
                                                 hap, hbp), False)
        self.m, self.n = int(ndof.sum()), n

    def solve(self, r, v=None, options: MecheOptions | None = None, staticProblem: bool = False,
              problemRegularization: float = 0.0) -> float:
        """r: (3n) world, solved in place; v: (sum ndof) array receiving the velocities (ADMM: also its warm
        start) or None. Returns the solver's residual; the callback connected through callback() fires per
        iteration."""
        if not (isinstance(r, np.ndarray) and r.dtype == np.float64 and r.flags.c_contiguous):
            raise TypeError("r must be a C-contiguous float64 numpy array (solved in place)")
        if v is not None and not (isinstance(v, np.ndarray) and v.dtype == np.float64 and v.flags.c_contiguous
                                  and v.size == self.m):
            raise TypeError("v must be a C-contiguous float64 numpy array of the problem's dofs")
        o = options or MecheOptions()
        res = C.c_double()
        st = lib().bogus_gpu_meche_solve(self._dual.handle, r.reshape(-1),
                                         None if v is None else v.ctypes.data_as(C.c_void_p), C.byref(o),
                                         int(staticProblem), float(problemRegularization), C.byref(res))
        _check(st)
        self.last_status = st
        return res.value

    def callback(self, fn) -> None:
        """Connects fn(iteration, residual) to the solver callbacks (MecheFrictionProblem::callback())."""
        sig = Signal()
        sig.connect(fn)

        class _Holder:
            def callback(self_inner):
                return sig

        self._dual._bind(_Holder())

    def nContacts(self) -> int:
        return self.n

    def nDegreesOfFreedom(self) -> int:
        return self.m
