/*
 * bogus_gpu — C ABI of the GB300 (sm_103a) friction-solve library.
 *
 * A drop-in for So-bogus's friction-solve path: 3x3-block sparse products, Delassus assembly
 * W = H M^-1 H^T, colored block Gauss-Seidel, projected gradient (APGD / SPG / ...) and the
 * SOCLaw<3> / Coulomb local solver, run by hand-written CUDA kernels on one GPU.
 *
 * Conventions (the reference's, Interfaces/FrictionProblem.hpp:127-214):
 *  - one handle = one dual problem  u = W r + b  on one device; contacts are 3-vectors in the local
 *    basis (normal first), arrays are contact-major: r[3*i + k];
 *  - W is given as 3x3-block BSR (row pointers, column indices, row-major blocks of 9 doubles), either
 *    the symmetric lower triangle (the reference's SparseBlockMatrix<Matrix3d, SYMMETRIC> storage) or
 *    both triangles;
 *  - the caller owns every array; r is in/out (warm start and result) as in solveWith();
 *  - every call returns a bogus_gpu_status; a solve also writes the reference's return value (the
 *    error function of ConstrainedSolverBase::eval) to *residual;
 *  - no CPU fallback: without a usable GPU, calls return BOGUS_GPU_NO_DEVICE or BOGUS_GPU_CUDA_ERROR;
 *  - a handle is not thread-safe; it owns one CUDA stream.
 */
#ifndef BOGUS_GPU_H
#define BOGUS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bogus_gpu_status {
  BOGUS_GPU_OK = 0,
  BOGUS_GPU_NOT_CONVERGED = 1, /* iteration budget exhausted; r holds the best iterate */
  BOGUS_GPU_BAD_INPUT = 2,     /* malformed sizes, indices or options */
  BOGUS_GPU_NONFINITE = 3,     /* NaN / Inf in the inputs */
  BOGUS_GPU_CUDA_ERROR = 4,    /* a CUDA call failed (see bogus_gpu_last_error) */
  BOGUS_GPU_TIMEOUT = 5,       /* a device-side wait ran out (the kernel stopped itself) */
  BOGUS_GPU_NO_DEVICE = 6,     /* no CUDA device / wrong architecture */
  BOGUS_GPU_NO_PROBLEM = 7     /* solve called before the problem was set */
} bogus_gpu_status;

/* projected_gradient::Variant (Core/BlockSolvers.fwd.hpp) */
typedef enum bogus_gpu_pg_variant {
  BOGUS_GPU_PG_STANDARD = 0,
  BOGUS_GPU_PG_DESCENT = 1,
  BOGUS_GPU_PG_CONJUGATED = 2,
  BOGUS_GPU_PG_APGD = 3,
  BOGUS_GPU_PG_SPG = 4
} bogus_gpu_pg_variant;

/* local_soc_solver::Strategy (Extra/SecondOrder.fwd.hpp:33-55) */
typedef enum bogus_gpu_local_strategy {
  BOGUS_GPU_LOCAL_PURE_NEWTON = 0,
  BOGUS_GPU_LOCAL_PURE_ENUMERATIVE = 1,
  BOGUS_GPU_LOCAL_HYBRID = 2,
  BOGUS_GPU_LOCAL_REV_HYBRID = 3
} bogus_gpu_local_strategy;

/* Signal<unsigned, double> listener (Core/Utils/Signal.hpp:25-54, BlockSolverBase::callback()).
 * Fired on the calling thread, in iteration order, when the solve returns. */
typedef void (*bogus_gpu_callback)(unsigned iteration, double residual, void* user);

/* ProjectedGradient setters and defaults (Core/BlockSolvers/ProjectedGradient.hpp:61-95,
 * BlockSolverBase.hpp:38-43, ConstrainedSolverBase.hpp:31). */
typedef struct bogus_gpu_pg_options {
  double tol;                     /* 1e-6 */
  unsigned max_iters;             /* 300 */
  unsigned ls_iters;              /* 8 */
  double ls_optimistic_factor;    /* 1.25 */
  double ls_pessimistic_factor;   /* 0.5 */
  double ls_armijo_coefficient;   /* 0.5 */
  int variant;                    /* bogus_gpu_pg_variant, APGD */
  int use_infinity_norm;          /* 0 */
  int static_problem;             /* 1: SOC law; 0: Coulomb (DualFrictionProblem::solveWith(pg) default 1) */
  int mixed_precision;            /* 0: FP64 throughout (the drop-in). 1: FP32-refined: W, the iterates and
                                     the per-contact law in FP32 (reductions and step decisions in FP64) for up
                                     to max_iters iterations, then up to refine_max_iters FP64 iterations from
                                     the FP32 result (the returned residual is the FP64 error function) */
  unsigned refine_max_iters;      /* 50 */
  int momentum_by_linearity;      /* 0: APGD's momentum step multiplies W by the new x, as the reference does
                                     (ProjectedGradient.impl.hpp:141). 1 (not in the reference): the product is
                                     formed by linearity, W x = W xs + beta (W xs - W prev), from the trial's
                                     product and the kept product of prev: one pass over W fewer per momentum
                                     step, iterates that differ from the reference's by rounding (and a returned
                                     residual evaluated with that product, equal to the error function at the
                                     returned iterate up to rounding). Single-problem and batched solves; with
                                     mixed_precision it applies to the FP64 iterations only (in FP32 the
                                     recombined product's rounding makes the line search retry more often); the
                                     allocation-free entry point rejects it */
  unsigned fp32_stall_iters;      /* 4 (not in the reference; mixed_precision only): the FP32 part ends before
                                     max_iters once FP32 rounding stops its progress, that is when its residual
                                     has repeated bit for bit on this many consecutive iterations or (APGD,
                                     Descent) its line search has run out of trials this many times in a row;
                                     the FP64 iterations then start from the best FP32 iterate. 0: the FP32 part
                                     runs to max_iters */
  unsigned fp32_products_refresh; /* 0 (not in the reference; mixed_precision with APGD only; single-problem and
                                     batched solves). N > 0: the FP64
                                     iterations after the FP32 part keep FP64 iterates, law and reductions but
                                     form their products as W x_ref + W32 (v - x_ref), the correction v - x_ref
                                     rounded to FP32 and multiplied by the FP32 copy of W, with x_ref and
                                     W x_ref (FP64) refreshed at the first momentum step on or after every N
                                     iterations; a plain FP64 solve from their best iterate then checks the
                                     tolerance with the exact error function (it runs on while the budget
                                     refine_max_iters lasts). The corrections leave a floor in the error
                                     function that grows with N (about 1e-8 N on a 200 000-contact problem):
                                     choose N well below tol / 1e-8 there; a part whose best residual stops
                                     improving (1 % in 10 N iterations) hands over early. max_iters = 0 skips
                                     the FP32 part */
} bogus_gpu_pg_options;

/* GaussSeidel setters and defaults (Core/BlockSolvers/GaussSeidelBase.hpp:39-91) plus the coloring switch
 * of MecheFrictionProblem::Options (Interfaces/MecheInterface.hpp:44-69). */
typedef struct bogus_gpu_gs_options {
  double tol;                     /* 1e-6 */
  unsigned max_iters;             /* 250 */
  unsigned eval_every;            /* 25 */
  double skip_tol;                /* 1e-6 */
  unsigned skip_iters;            /* 10 */
  double auto_regularization;     /* 0 */
  int try_zero_as_well;           /* 1 */
  int use_infinity_norm;          /* 0 */
  int static_problem;             /* 0: Coulomb law (DualFrictionProblem::solveWith(gs) default) */
  int local_strategy;             /* bogus_gpu_local_strategy, RevHybrid */
  int use_coloring;               /* 0: contacts swept in their own order, as DualFrictionProblem::solveWith(gs)
                                     does single-threaded; 1: Coloring::compute + contact permutation, as
                                     MecheFrictionProblem::solve does with maxThreads != 1 */
} bogus_gpu_gs_options;

/* admm::Variant (Core/BlockSolvers/ADMM.hpp:21-29) */
typedef enum bogus_gpu_admm_variant {
  BOGUS_GPU_ADMM_STANDARD = 0,
  BOGUS_GPU_ADMM_ACCELERATED = 1
} bogus_gpu_admm_variant;

/* ADMM setters and defaults (Core/BlockSolvers/ADMM.hpp:81-100, ConstrainedSolverBase.hpp:31). */
typedef struct bogus_gpu_admm_options {
  double tol;                     /* 1e-6 */
  unsigned max_iters;             /* 300 */
  double step_size;               /* 1e-2 */
  int variant;                    /* bogus_gpu_admm_variant, Accelerated */
  int use_infinity_norm;          /* 0 */
} bogus_gpu_admm_options;

/* DualAMA setters and defaults (Core/BlockSolvers/ADMM.hpp:170-236). */
typedef struct bogus_gpu_dual_ama_options {
  double tol;                     /* 1e-6 */
  unsigned max_iters;             /* 300 */
  double fp_step_size;            /* 1e-1 (gamma) */
  double proj_step_size;          /* 1e-1 (lambda) */
  unsigned ls_iters;              /* 6 (0: no line search) */
  double ls_optimistic_factor;    /* 1.25 */
  double ls_pessimistic_factor;   /* 0.5 */
  int variant;                    /* bogus_gpu_admm_variant, Accelerated */
  int use_infinity_norm;          /* 0 */
} bogus_gpu_dual_ama_options;

typedef struct bogus_gpu_problem bogus_gpu_problem;

/* Option defaults, identical to the reference's constructors. */
void bogus_gpu_pg_options_default(bogus_gpu_pg_options* opts);
void bogus_gpu_gs_options_default(bogus_gpu_gs_options* opts);
void bogus_gpu_admm_options_default(bogus_gpu_admm_options* opts);
void bogus_gpu_dual_ama_options_default(bogus_gpu_dual_ama_options* opts);

const char* bogus_gpu_status_string(int status);
/* Last CUDA / validation message recorded on this thread. */
const char* bogus_gpu_last_error(void);

/* Creates a problem handle on `device` (checks for an sm_103 device). */
int bogus_gpu_create(int device, bogus_gpu_problem** out);
int bogus_gpu_destroy(bogus_gpu_problem* h);

/* DualFrictionProblem<3> members W, b, mu (Interfaces/FrictionProblem.hpp:140-150), from host arrays.
 * symmetric_lower != 0: blocks hold the lower triangle incl. diagonal, rows sorted by column
 * (SparseBlockMatrix<Matrix3d RowMajor, SYMMETRIC>); 0: both triangles, rows sorted. A malformed structure
 * (BAD_INPUT) or a non-finite value (NONFINITE) is rejected and the handle keeps the problem it had. */
int bogus_gpu_set_dual(bogus_gpu_problem* h, int n, const int* rowptr, const int* colidx, const double* blocks,
                       int symmetric_lower, const double* b, const double* mu);

/* Same, from device pointers (full both-triangle BSR already on the device; copied into the handle). The
 * arrays are checked on the device before the copy: row pointers in order and in range, columns in range and
 * strictly increasing, a diagonal block in every row (BOGUS_GPU_BAD_INPUT otherwise), finite W, b and mu
 * (BOGUS_GPU_NONFINITE); a rejected problem leaves the handle's problem in place. */
int bogus_gpu_set_dual_device(bogus_gpu_problem* h, int n, int nnzb, const int* d_rowptr, const int* d_colidx,
                              const double* d_blocks, const double* d_b, const double* d_mu);

/* DualFrictionProblem::applyPermutation / undoPermutation / permuted (Interfaces/FrictionProblem.hpp:198-207,
 * FrictionProblem.cpp:102-125): contact k of the stored problem becomes contact perm[k] of the current one
 * (W' = P W P^T, b' = P b, mu' = P mu). While permuted, bogus_gpu_solve_gs / _pg / _pg_device / _cadoux_* and
 * bogus_gpu_eval take and return r in the caller's order (FrictionProblem.impl.hpp:38-91); bogus_gpu_spmv and
 * bogus_gpu_get_dual_lower work on the stored (permuted) W, as W.multiply does. Batched solves and the adjoint
 * need the contacts in their own order (BAD_INPUT while permuted). Setting a new problem clears the permutation. */
int bogus_gpu_apply_permutation(bogus_gpu_problem* h, const int* perm);
int bogus_gpu_undo_permutation(bogus_gpu_problem* h);
int bogus_gpu_permuted(const bogus_gpu_problem* h, int* permuted);

/* Number of stored blocks of the both-triangle W held on the device. */
int bogus_gpu_nnzb(const bogus_gpu_problem* h, int* nnzb);

/* BlockSolverBase::callback() (Core/BlockSolvers/BlockSolverBase.hpp:45-51). */
int bogus_gpu_set_callback(bogus_gpu_problem* h, bogus_gpu_callback cb, void* user);

/* y = W x (SparseBlockMatrixBase::multiply, Core/Block/SparseMatrixVectorProduct.impl.hpp:423-432); host arrays. */
int bogus_gpu_spmv(bogus_gpu_problem* h, const double* x, double* y);

/* DualFrictionProblem::evalWith (Interfaces/FrictionProblem.cpp:56-66): error function at r, u = W r + b. */
int bogus_gpu_eval(bogus_gpu_problem* h, const double* r, int static_problem, int use_infinity_norm,
                   double* residual);

/* DualFrictionProblem::solveWith(ProjectedGradient&, r, staticProblem) (Interfaces/FrictionProblem.cpp:49-54,
 * ProjectedGradient.impl.hpp:74-382). r: host array, in/out. iters may be NULL. All five variants; Standard
 * and Conjugated (Armijo line search) in FP64 single-problem solves only: the FP32-refined, batched and
 * allocation-free forms return BAD_INPUT for them. */
int bogus_gpu_solve_pg(bogus_gpu_problem* h, const bogus_gpu_pg_options* opts, double* r, double* residual,
                       unsigned* iters);

/* Same with r on the device (no host copies). */
int bogus_gpu_solve_pg_device(bogus_gpu_problem* h, const bogus_gpu_pg_options* opts, double* d_r, double* residual,
                              unsigned* iters);

/* DualFrictionProblem::solveWith(GaussSeidel&, r, staticProblem) (Interfaces/FrictionProblem.cpp:42-47,
 * GaussSeidel.impl.hpp:62-205): the reference's sequential sweep, in the contacts' own order or (use_coloring)
 * in the order of Coloring::compute with the contact permutation of MecheFrictionProblem::solve
 * (Interfaces/MecheInterface.cpp:326-337, Coloring.impl.hpp:20-62). Contacts are processed level by level:
 * a contact's level is one more than the highest level among its neighbours that precede it in the sweep, so
 * each launch solves contacts that share no block of W and every contact sees exactly the values the
 * sequential sweep would give it. Requires W set from host arrays or assembled (the schedule is built on the
 * host). */
int bogus_gpu_solve_gs(bogus_gpu_problem* h, const bogus_gpu_gs_options* opts, double* r, double* residual,
                       unsigned* iters);

/* ---- Batched solves (no counterpart in the reference, which solves one problem per call) ------------------
 * Marks the handle's W as block diagonal: problem p owns contacts [contact_ptr[p], contact_ptr[p+1]) and its
 * rows reference only columns of that range (for example a primal problem whose contact groups share no body,
 * assembled with bogus_gpu_assemble_dual). contact_ptr has nproblems + 1 entries, from 0 to n. */
int bogus_gpu_set_batch(bogus_gpu_problem* h, int nproblems, const int* contact_ptr);

/* Solves every problem of the batch in one persistent launch (one CTA per problem, largest first). Each
 * problem gets exactly the result DualFrictionProblem::solveWith(ProjectedGradient&, r) gives for it alone
 * (same iterates, residual and iteration count). r: all problems, contact-major, in/out; residuals and iters
 * hold one entry per problem (NULL allowed). Returns BOGUS_GPU_NOT_CONVERGED if any problem did not converge. */
int bogus_gpu_solve_pg_batch(bogus_gpu_problem* h, const bogus_gpu_pg_options* opts, double* r, double* residuals,
                             unsigned* iters);
/* Same with r on the device. */
int bogus_gpu_solve_pg_batch_device(bogus_gpu_problem* h, const bogus_gpu_pg_options* opts, double* d_r,
                                    double* residuals, unsigned* iters);

/* Launch shape of the batched solves. schedule 0: one CTA per problem, at most ctas_per_sm resident CTAs per SM;
 * schedule 1: teams of team_size CTAs per problem (a cooperative launch), at most ctas_per_sm CTAs per SM. Every
 * shape gives the same results bit for bit: each problem's reductions follow its fixed 32-contact chunk order. */
typedef struct bogus_gpu_batch_shape {
  int schedule;
  int ctas_per_sm;
  int team_size;
} bogus_gpu_batch_shape;

/* on != 0: the first batched solve of each precision after bogus_gpu_set_batch measures the candidate shapes on
 * the batch itself (one CTA per problem at 1..4 CTAs per SM; teams of 2, 4, 8, 16 CTAs at 2 and 3 CTAs per SM;
 * each run capped at 30 iterations from the same starting iterate, timed with CUDA events) and keeps the fastest,
 * which later solves reuse; the choice is also cached for the process by device, precision and the batch's size
 * class (problems, largest problem, total 32-contact chunks). 0 (default): a fixed rule (one CTA per problem when
 * there are at least half as many problems as resident CTAs, else teams). */
int bogus_gpu_set_batch_tuning(bogus_gpu_problem* h, int on);
/* Forces the shape of the following batched solves (NULL: back to tuning or the rule). */
int bogus_gpu_set_batch_shape(bogus_gpu_problem* h, const bogus_gpu_batch_shape* shape);
/* The shape of the last batched launch. */
int bogus_gpu_get_batch_shape(const bogus_gpu_problem* h, bogus_gpu_batch_shape* shape);
/* The tuner's last measurements: *count shapes and their times in ms (pass NULL arrays to get the count). */
int bogus_gpu_get_batch_tuning_log(const bogus_gpu_problem* h, bogus_gpu_batch_shape* shapes, double* ms, int* count);

/* bogus_gpu_solve_pg_batch (FP64) with the whole sequence (upload of r, the solve, download of r and of the
 * per-problem results) captured once into a CUDA graph and replayed by later calls with the same options, host
 * buffer and batch: for a simulation that solves the same batch layout every step, one graph launch replaces the
 * separate copies, memsets and kernel launch. r must be page-locked host memory (cudaHostAlloc /
 * cudaHostRegister; BOGUS_GPU_BAD_INPUT otherwise). The shape (and tuning, when enabled) is settled before the
 * capture. Results are those of bogus_gpu_solve_pg_batch, bit for bit. */
int bogus_gpu_solve_pg_batch_graph(bogus_gpu_problem* h, const bogus_gpu_pg_options* opts, double* r,
                                   double* residuals, unsigned* iters);

/* DualFrictionProblem::solveCadoux (Interfaces/FrictionProblem.impl.hpp:76-92, Interfaces/Cadoux.hpp:44-91): the
 * Coulomb problem solved as up to cadoux_iters SOCQP problems u = W r + (b + COV(u_prev)), each by the
 * Gauss-Seidel or projected-gradient minimizer with its tolerance tightened to 0.1 max(tol, min(res, 1)). r is
 * in/out; *residual is the Coulomb error function at the result; *iters the fixed-point iterations run. The
 * callback fires once per fixed-point iteration (0 = the initial error). The options' static_problem is ignored
 * (inner problems use the SOC law). */
int bogus_gpu_solve_cadoux_gs(bogus_gpu_problem* h, const bogus_gpu_gs_options* opts, double* r,
                              unsigned cadoux_iters, double* residual, unsigned* iters);
int bogus_gpu_solve_cadoux_pg(bogus_gpu_problem* h, const bogus_gpu_pg_options* opts, double* r,
                              unsigned cadoux_iters, double* residual, unsigned* iters);

/* PrimalFrictionProblem::solveWith(ProductGaussSeidelType&, r, staticProblem) (Interfaces/PrimalFrictionProblem.cpp:
 * 41-59, Core/BlockSolvers/ProductGaussSeidel.impl.hpp:108-296): Gauss-Seidel on W = H M^-1 H^T without forming W,
 * on the handle's primal data (bogus_gpu_set_primal), b = w - H M^-1 f (f NULL: 0). The contacts are swept in their
 * own order (use_coloring must be 0); the other options as bogus_gpu_solve_gs (static_problem 0: Coulomb). */
int bogus_gpu_solve_product_gs(bogus_gpu_problem* h, const bogus_gpu_gs_options* opts, const double* f,
                               const double* w, const double* mu, double* r, double* residual, unsigned* iters);

/* Greedy coloring used by bogus_gpu_solve_gs: perm[n] (contact order, colors contiguous) and colors[ncolors+1]
 * offsets; colors must hold n + 1 ints. */
int bogus_gpu_coloring(bogus_gpu_problem* h, int* perm, int* colors, int* ncolors);

/* PrimalFrictionProblem data (Interfaces/FrictionProblem.hpp:55-116) for rigid bodies with a uniform number
 * of dofs: minv[nbodies][ndof][ndof] (M^-1 blocks), contact i couples body objA[i] and objB[i] (-1: none)
 * through 3 x ndof Jacobian blocks HA[i], HB[i] (row-major, local contact basis). */
int bogus_gpu_set_primal(bogus_gpu_problem* h, int nbodies, int ndof, const double* minv, int ncontacts,
                         const int* objA, const int* objB, const double* HA, const double* HB);

/* The bodies' own dof counts of a padded primal problem. The reference's H has column blocks of varying
 * width (PrimalFrictionProblem<3>::HType, Interfaces/FrictionProblem.hpp:65-66); bogus_gpu_set_primal pads every
 * body to ndof dofs, and body k then uses its first ndof_k <= ndof dofs, the Jacobian columns and M^-1 entries
 * past them being zero. Only the error-function scalings of ADMM / DualAMA (their square-matrix test,
 * ConstrainedSolverBase.impl.hpp:84-118) and DualAMA's gap normalisation depend on it. Default: ndof each. */
int bogus_gpu_set_body_dofs(bogus_gpu_problem* h, const int* ndof_k);

/* PrimalFrictionProblem::E (Interfaces/FrictionProblem.hpp:62-63): per-contact frames, contact basis to world
 * coordinates, n x 3 x 3 row-major (E_i[a][b]); NULL: identity (the default). With frames set, the w given to
 * bogus_gpu_assemble_dual, _solve_admm, _solve_dual_ama and _solve_product_gs is in world coordinates and is
 * taken to the contact basis as E^T w (PrimalFrictionProblem.cpp:44, 64, 82; FrictionProblem.cpp:35-36), each
 * component the chain fma(E[2][a], w2, fma(E[1][a], w1, E[0][a] w0)). H is given in the contact basis. */
int bogus_gpu_set_frames(bogus_gpu_problem* h, const double* E);

/* DualFrictionProblem::computeFrom (Interfaces/FrictionProblem.cpp:30-40): W = H M^-1 H^T assembled on the
 * device and b = w - H M^-1 f (w in the local basis, E = I; f may be NULL for f = 0); mu copied. The result
 * replaces the handle's dual problem. */
int bogus_gpu_assemble_dual(bogus_gpu_problem* h, const double* f, const double* w, const double* mu);

/* PrimalFrictionProblem::solveWith(ADMMType&, lambda, v, r) (Interfaces/PrimalFrictionProblem.cpp:61-73), or
 * ADMM::solve(law, QuadraticProxOp(prox, lambda, f), w, v, r) (Core/BlockSolvers/ADMM.impl.hpp:54-127) with
 * an explicit prox operator: primal ADMM on the handle's primal data (bogus_gpu_set_primal), law
 * SOCLaw<3, false> on 1 / mu, J(v) = v^T M v / 2 + f^T v.
 *  - prox: nbodies x ndof x ndof blocks of the linear operator of QuadraticProxOp (row-major), or NULL for the
 *    M^-1 blocks of bogus_gpu_set_primal (what PrimalFrictionProblem::solveWith passes, whatever lambda);
 *  - f: nbodies x ndof (NULL: 0); w: 3 n (local basis, E = I); mu: n;
 *  - v (nbodies x ndof) and r (3 n) are in/out (warm start and result);
 *  - the callback, when set, fires once per iteration. */
int bogus_gpu_solve_admm(bogus_gpu_problem* h, const bogus_gpu_admm_options* opts, double lambda,
                         const double* prox, const double* f, const double* w, const double* mu, double* v,
                         double* r, double* residual, unsigned* iters);

/* PrimalFrictionProblem::solveWith(DualAMAType&, v, r, staticProblem) (Interfaces/PrimalFrictionProblem.cpp:
 * 78-99), DualAMA::solve(law, M, f, w, v, r) (Core/BlockSolvers/ADMM.impl.hpp:128-303): dual accelerated
 * minimisation on the handle's primal data, law SOCLaw<3, !static_problem> on mu.
 *  - mass: nbodies x ndof x ndof mass blocks M (row-major; required);
 *  - f: nbodies x ndof (NULL: 0); w: 3 n (local basis); mu: n;
 *  - v (nbodies x ndof) and r (3 n) are in/out; on return they hold the iterate of least residual;
 *  - the error function's scalings are 1 unless H is square at the block level (3 n == the bodies' dofs and
 *    n == nbodies), as ConstrainedSolverBase::updateScalings sets them;
 *  - the callback, when set, fires once per iteration. */
int bogus_gpu_solve_dual_ama(bogus_gpu_problem* h, const bogus_gpu_dual_ama_options* opts, const double* mass,
                             const double* f, const double* w, const double* mu, int static_problem, double* v,
                             double* r, double* residual, unsigned* iters);

/* ---- Adjoint of the SOC and Coulomb solves (no counterpart in the reference, which has no differentiation) --
 * r solves min 1/2 r^T W r + b^T r over r_i in K_mu_i = {|x_T| <= mu x_N} (the SOCLaw<3> problem that
 * bogus_gpu_solve_pg solves with static_problem = 1), or (options.coulomb) the Coulomb friction problem
 * (static_problem = 0). Given that solution r and g = dL/dr of a loss L, the implicit-function gradients dL/db and
 * dL/dmu follow from one linear solve on the device, to relative residual tol. r should be solved tightly: the
 * gradients are those of the fixed point at r. W must be positive definite on the contacts' active
 * directions (add a compliance term, bogus_gpu_add_compliance, where H M^-1 H^T is singular). */
typedef struct bogus_gpu_adjoint_options {
  double tol;                     /* 1e-10 */
  unsigned max_iters;             /* 5000 */
  int coulomb;                    /* 0: the SOC problem (conjugate gradients). 1: the Coulomb problem that
                                     bogus_gpu_solve_pg / _gs solve with static_problem = 0, the fixed point
                                     r = P(r - A (u + s(u))) with the De Saxce term s(u) = (mu |u_T|, 0, 0)
                                     (SOCLaw::dualityCOV); its linearisation is not symmetric and is solved by
                                     bi-conjugate gradients stabilised, two passes over W per iteration */
} bogus_gpu_adjoint_options;
void bogus_gpu_adjoint_options_default(bogus_gpu_adjoint_options* opts);
/* dL_db (3 n) and dL_dmu (n) from r and dL_dr (host arrays); residual: final relative CG residual. */
int bogus_gpu_adjoint(bogus_gpu_problem* h, const bogus_gpu_adjoint_options* opts, const double* r,
                      const double* dL_dr, double* dL_db, double* dL_dmu, double* residual, unsigned* iters);
/* Same with device arrays. */
int bogus_gpu_adjoint_device(bogus_gpu_problem* h, const bogus_gpu_adjoint_options* opts, const double* d_r,
                             const double* d_dL_dr, double* d_dL_db, double* d_dL_dmu, double* residual,
                             unsigned* iters);
/* After bogus_gpu_adjoint: dL/dW for the stored lower blocks (the order of bogus_gpu_get_dual_lower; block
 * W_ij, i > j, stands for W_ji = W_ij^T too): s_i r_j^T + r_i s_j^T off the diagonal, s_i r_i^T on it. */
int bogus_gpu_adjoint_dual_lower(bogus_gpu_problem* h, double* dL_dW_lower);
/* After bogus_gpu_adjoint on a W assembled from the handle's primal data (W = H M^-1 H^T, plus compliance,
 * b = w - H M^-1 f): dL/dHA, dL/dHB (n x 3 x ndof, zero where the contact has no body B), dL/dw (3 n) and
 * dL/df (nbodies x ndof); f: the f of the assembly (NULL: 0). Any output may be NULL. */
int bogus_gpu_adjoint_primal(bogus_gpu_problem* h, const double* f, double* dL_dHA, double* dL_dHB, double* dL_dw,
                             double* dL_df);
/* W_ii += c_i I for every contact (a compliance term); c: n values >= 0. */
int bogus_gpu_add_compliance(bogus_gpu_problem* h, const double* c);

/* Copies the lower triangle of the device-held W back (rowptr[n+1], colidx/blocks sized by *nnzb_lower;
 * pass NULL arrays first to get the size). */
int bogus_gpu_get_dual_lower(bogus_gpu_problem* h, int* rowptr, int* colidx, double* blocks, int* nnzb_lower);

/* Copies the device-held b (3 n) and mu (n) back, in the stored order of bogus_gpu_get_dual_lower: the
 * DualFrictionProblem members b and mu (Interfaces/FrictionProblem.hpp:145-150) after bogus_gpu_assemble_dual
 * computed them. Either output may be NULL. */
int bogus_gpu_get_dual_rhs(bogus_gpu_problem* h, double* b, double* mu);

/* Measurements of the last solve, spmv or assembly (no counterpart in the reference, which only offers
 * MecheFrictionProblem::lastSolveTime, Interfaces/MecheInterface.hpp:173). */
typedef struct bogus_gpu_solve_stats {
  double device_ms;          /* device time between CUDA events around the solver kernels */
  unsigned kernel_launches;  /* kernels launched */
  unsigned iterations;
  unsigned w_passes;         /* full passes over W (products) */
  double algorithmic_bytes;  /* bytes the passes had to move: W (values + indices) + vector streams */
  double fp64_fma;           /* FP64 fused multiply-adds of the W passes */
  unsigned refine_iterations; /* FP64 iterations after the FP32 ones (mixed precision), else 0 */
  double fp32_device_ms;      /* device time of the FP32 part (mixed precision), else 0 */
  unsigned fp32_product_iterations; /* of refine_iterations, those with FP32 correction products */
} bogus_gpu_solve_stats;
int bogus_gpu_get_solve_stats(const bogus_gpu_problem* h, bogus_gpu_solve_stats* out);

/* The CUDA stream (cudaStream_t) the handle launches on, so callers can order and time their own work
 * with it (no counterpart in the reference). */
int bogus_gpu_get_stream(const bogus_gpu_problem* h, void** stream);

/* Limit of every device-side wait of the library's kernels on `device` (grid barriers of the persistent
 * solvers, the Gauss-Seidel sweep's flag waits), in seconds within [1e-6, 3600]; default 4. A wait that runs
 * out makes the kernel record BOGUS_GPU_TIMEOUT and return, and the call reports TIMEOUT; the CUDA context
 * stays usable. The setting holds for every handle and the allocation-free entry point on that device until
 * changed; set it while no solve runs there. The caller's current device is left as it was. No counterpart
 * in the reference (its solvers run on the host). */
int bogus_gpu_set_wait_limit(int device, double seconds);

/* Test of the timeout path (no counterpart in the reference). While `on` is non-zero, the single-problem
 * projected-gradient solves of this handle (bogus_gpu_solve_pg / _pg_device, FP64) launch their kernel with
 * barriers that wait for one CTA more than the launch holds: the first barrier can never complete, its
 * bounded wait runs out after the wait limit, and the solve returns BOGUS_GPU_TIMEOUT without touching r.
 * Turn it off to solve normally again on the same handle. */
int bogus_gpu_test_wait_timeout(bogus_gpu_problem* h, int on);

/* Measures the FP64 fused multiply-add throughput of `device` in TFLOP/s: the ceiling of the FP64 kernels
 * on GPUs whose FP64 rate is below their memory bandwidth's need (no counterpart in the reference). */
int bogus_gpu_measure_fp64_peak(int device, double* tflops);

/* Compares the library's integer-pipe FP64 division, square root and exact scalings (by 1/2, by 2, + 0.0),
 * used by the solvers' per-contact law work, with the GPU's own IEEE operations on n generated operands;
 * mismatches[0..2] receive the differing results of division, square root and scalings (all zero when the
 * implementation is exact). A diagnostic with no counterpart in the reference. */
int bogus_gpu_check_fp64_ops(int device, long long n, unsigned long long seed, long long* mismatches);

/* ---- Allocation-free projected-gradient solve (no counterpart in the reference) --------------------------
 * For callers that must not allocate GPU memory while solving: simulation steps run under a fixed device-memory
 * budget, real-time loops where cudaMalloc's implicit synchronisation would stall the frame, or hosts that hand
 * the library only buffers they own. Same solve as bogus_gpu_solve_pg_device (APGD, Descent or SPG; the same
 * iterates and residual), but W (both triangles, as in bogus_gpu_set_dual_device), b, mu and r are caller-owned
 * device arrays, no handle is needed, and every temporary lives in one fixed array inside the library
 * (about 14.2 MB of device memory, held on every GPU that loads the library until the process exits).
 *  - Limits: at most BOGUS_GPU_NOALLOC_MAX_CONTACTS contacts and BOGUS_GPU_NOALLOC_MAX_ITERS iterations;
 *    larger requests return BOGUS_GPU_BAD_INPUT without launching anything.
 *  - The first call on a device looks up the array's device address (cudaGetSymbolAddress) with that device
 *    current; make that first call before any stream capture.
 *  - Calls on one device share the array and it keeps the last call's contents (each call clears what must
 *    start at zero): calls whose GPU work overlaps race and must not be issued.
 *  - The remembered address lives in the device's CUDA context: after cudaDeviceReset on that device the
 *    entry point must not be called again in the process.
 *  - W, b, mu and r are checked on the device first (row pointers in order and in range, columns in range and
 *    strictly increasing, a diagonal block in every row, finite values); a malformed W returns
 *    BOGUS_GPU_BAD_INPUT and a non-finite value BOGUS_GPU_NONFINITE, with r untouched.
 *  - `device` is made current for the call's work; the caller's current device is restored before returning.
 *  - No callback. stream: a cudaStream_t, or NULL for the default stream; the call returns when the solve is
 *    done and r holds the result. */
#define BOGUS_GPU_NOALLOC_MAX_CONTACTS 65536
#define BOGUS_GPU_NOALLOC_MAX_ITERS 65536
int bogus_gpu_solve_pg_noalloc(int device, int n, int nnzb, const int* d_rowptr, const int* d_colidx,
                               const double* d_blocks, const double* d_b, const double* d_mu,
                               const bogus_gpu_pg_options* opts, double* d_r, double* residual, unsigned* iters,
                               void* stream);

/* ---- MecheFrictionProblem facade (Interfaces/MecheInterface.hpp:40-170, MecheInterface.cpp:97-367) ---------
 * The raw-pointer caller of the reference: a primal problem in world coordinates (contact frames E), solved
 * with the dual assembled on the device. Per handle; bogus_gpu_meche_from_primal replaces the handle's
 * primal and dual problems. */
typedef enum bogus_gpu_meche_algorithm { /* MecheFrictionProblem::Algorithm */
  BOGUS_GPU_MECHE_GAUSS_SEIDEL = 0,
  BOGUS_GPU_MECHE_PROJECTED_GRADIENT = 1,
  BOGUS_GPU_MECHE_MATRIX_FREE_GAUSS_SEIDEL = 2,
  BOGUS_GPU_MECHE_ADMM = 3,
  BOGUS_GPU_MECHE_DUAL_AMA = 4
} bogus_gpu_meche_algorithm;

/* MecheFrictionProblem::Options (MecheInterface.hpp:44-69) and its defaults (MecheInterface.cpp:51-63). */
typedef struct bogus_gpu_meche_options {
  int max_threads;            /* 0; Gauss-Seidel uses the coloring order when != 1 and gs_coloring */
  unsigned max_iters;         /* 0: the solver's default */
  unsigned cadoux_iters;      /* 0; > 0 with a non-static problem: the Cadoux fixed point */
  double tolerance;           /* 0: the solver's default */
  int use_infinity_norm;      /* 0 */
  int algorithm;              /* bogus_gpu_meche_algorithm, Gauss-Seidel */
  double gs_regularization;   /* 0: GaussSeidel::setAutoRegularization */
  int gs_coloring;            /* 0 */
  int gs_skip_iters;          /* -1: the solver's default */
  int try_zero_as_well;       /* 1 */
  int pg_variant;             /* bogus_gpu_pg_variant, SPG */
  double admm_proj_step_size; /* 1 */
  double admm_fp_step_size;   /* 1e-3 (DualAMA only) */
} bogus_gpu_meche_options;
void bogus_gpu_meche_options_default(bogus_gpu_meche_options* opts);

/* MecheFrictionProblem::fromPrimal: nobj objects with ndof[k] (1..12) degrees of freedom and column-major mass
 * matrices mass[k]; f: sum of ndof entries (NULL: 0); n contacts with friction mu, frames E ((3n x 3) column-
 * major: the n local-basis blocks, world to local), w (3n, world), objects objA[i] and objB[i] (-1: external)
 * and column-major 3 x ndof Jacobian blocks HA[i], HB[i] in world coordinates. The mass blocks are inverted and
 * H = E^T HA / -E^T HB (E^T (HA - HB) when objA[i] == objB[i]) is formed on the device. */
int bogus_gpu_meche_from_primal(bogus_gpu_problem* h, unsigned nobj, const unsigned* ndof, const double* const* mass,
                                const double* f, unsigned n, const double* mu, const double* E, const double* w,
                                const int* objA, const int* objB, const double* const* HA, const double* const* HB);

/* MecheFrictionProblem::solve(r, v, options, staticProblem, problemRegularization): r (3n, world) is in/out;
 * v (sum of ndof; NULL: not returned) receives M^-1 (H^T r - f), or is ADMM's warm start and result. The dual,
 * with problem_regularization added to W's diagonal, is computed at the first Gauss-Seidel or projected-gradient
 * solve after fromPrimal and kept, as in the reference. *residual: the solver's error. */
int bogus_gpu_meche_solve(bogus_gpu_problem* h, double* r, double* v, const bogus_gpu_meche_options* opts,
                          int static_problem, double problem_regularization, double* residual);

#ifdef __cplusplus
}
#endif

#endif /* BOGUS_GPU_H */
