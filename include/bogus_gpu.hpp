/*
 * bogus_gpu.hpp — header-only C++ layer over the bogus_gpu C ABI that restores the reference's API names, so a
 * caller of So-bogus's friction-solve path keeps its code shape:
 *
 *   bogus_gpu::PrimalFrictionProblem<3> primal;   // MInv, H (two 3 x ndof blocks per contact), f, w, mu
 *   bogus_gpu::DualFrictionProblem<3> dual;
 *   dual.computeFrom(primal);                     // W = H M^-1 H^T, b = E^T w - H M^-1 f (assembled on the GPU)
 *   bogus_gpu::DualFrictionProblem<3>::GaussSeidelType gs;
 *   gs.setTol(1e-8);
 *   double res = dual.solveWith(gs, r.data());    // the error function, as the reference returns it
 *
 * Names, arguments, defaults and return values follow Interfaces/FrictionProblem.hpp:55-214 (PrimalFrictionProblem,
 * DualFrictionProblem: computeFrom, solveWith, evalWith, solveCadoux, applyPermutation / undoPermutation),
 * Core/BlockSolvers/GaussSeidelBase.hpp:39-91 and GaussSeidel.hpp:122 (setters, coloring()),
 * ProjectedGradient.hpp:61-95, ADMM.hpp:81-100 and 170-236 (DualAMA), ConstrainedSolverBase.hpp:31-32
 * (useInfinityNorm), BlockSolverBase.hpp:38-51 (setTol, setMaxIters, callback()) and Core/Utils/Signal.hpp
 * (Signal<unsigned, double>::connect).
 *
 * Differences, since Eigen is not a dependency: vectors are bogus_gpu::VectorXd (owned, with data(), rows(),
 * size(), operator[], setZero()); W is a SymmetricBlockMatrix3 (the compressed lower triangle of
 * SparseBlockMatrix<Matrix3d, SYMMETRIC>: outer / inner indices and row-major 3x3 blocks); the primal problem
 * holds uniform-width bodies (ndof dofs each, at most 12). Errors that the reference only asserts, and CUDA
 * errors, throw bogus_gpu::Error carrying the bogus_gpu_status. A solve that ends its iteration budget returns
 * its residual like the reference (no exception). The GPU handle is created on first use, so option objects and
 * problems can be built on machines without a GPU.
 */
#ifndef BOGUS_GPU_HPP
#define BOGUS_GPU_HPP

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bogus_gpu.h"

namespace bogus_gpu {

// ---- errors ------------------------------------------------------------------------------------------------
class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline int check(int status, bool allow_not_converged = true) {
  if (status == BOGUS_GPU_OK || (allow_not_converged && status == BOGUS_GPU_NOT_CONVERGED)) return status;
  const char* last = bogus_gpu_last_error();
  throw Error(status, std::string(bogus_gpu_status_string(status)) + (last && *last ? std::string(": ") + last : ""));
}

// ---- minimal owned containers ------------------------------------------------------------------------------
// A dense vector of doubles. Every non-const access bumps a generation counter, so a problem knows when its data
// changed and must be uploaded again.
class VectorXd {
 public:
  VectorXd() = default;
  explicit VectorXd(std::size_t n, double value = 0.0) : v_(n, value) {}
  std::size_t rows() const { return v_.size(); }
  std::size_t size() const { return v_.size(); }
  void resize(std::size_t n) {
    ++gen_;
    v_.resize(n);
  }
  void setZero() {
    ++gen_;
    std::fill(v_.begin(), v_.end(), 0.0);
  }
  double* data() {
    ++gen_;
    return v_.data();
  }
  const double* data() const { return v_.data(); }
  double& operator[](std::size_t i) {
    ++gen_;
    return v_[i];
  }
  double operator[](std::size_t i) const { return v_[i]; }
  unsigned long long generation() const { return gen_; }

 private:
  std::vector<double> v_;
  unsigned long long gen_ = 0;
};

// Signal<unsigned, double> (Core/Utils/Signal.hpp:25-54): listeners called in iteration order.
template <class... Args>
class Signal {
 public:
  void connect(std::function<void(Args...)> fn) { callees_.push_back(std::move(fn)); }
  void disconnectAll() { callees_.clear(); }
  void trigger(Args... args) const {
    for (const auto& f : callees_) f(args...);
  }
  bool empty() const { return callees_.empty(); }

 private:
  std::vector<std::function<void(Args...)>> callees_;
};

// SparseBlockMatrix<Matrix3d RowMajor, SYMMETRIC> in compressed form: the lower triangle with the diagonal,
// rows sorted by column (outer[n + 1], inner[nnzb], 9 doubles per block, row-major).
class SymmetricBlockMatrix3 {
 public:
  int rowsOfBlocks() const { return outer_.empty() ? 0 : (int)outer_.size() - 1; }
  int nonZeros() const { return (int)inner_.size(); }
  void setFromLower(int n, const int* outer, const int* inner, const double* blocks) {
    ++gen_;
    outer_.assign(outer, outer + n + 1);
    const int nnz = n > 0 ? outer[n] : 0;
    inner_.assign(inner, inner + nnz);
    blocks_.assign(blocks, blocks + 9 * (std::size_t)nnz);
  }
  int* outerIndexPtr() { return (++gen_, outer_.data()); }
  int* innerIndexPtr() { return (++gen_, inner_.data()); }
  double* blockPtr() { return (++gen_, blocks_.data()); }
  const int* outerIndexPtr() const { return outer_.data(); }
  const int* innerIndexPtr() const { return inner_.data(); }
  const double* blockPtr() const { return blocks_.data(); }
  unsigned long long generation() const { return gen_; }

 private:
  std::vector<int> outer_, inner_;
  std::vector<double> blocks_;
  unsigned long long gen_ = 0;
};

// ---- solvers (option holders: the solve runs on the GPU through the problem) ----------------------------
namespace projected_gradient {
enum Variant { Standard = BOGUS_GPU_PG_STANDARD, Descent = BOGUS_GPU_PG_DESCENT, Conjugated = BOGUS_GPU_PG_CONJUGATED,
               APGD = BOGUS_GPU_PG_APGD, SPG = BOGUS_GPU_PG_SPG };
}
namespace admm {
enum Variant { Standard = BOGUS_GPU_ADMM_STANDARD, Accelerated = BOGUS_GPU_ADMM_ACCELERATED };
}
namespace local_soc_solver {
enum Strategy { PureNewton = BOGUS_GPU_LOCAL_PURE_NEWTON, PureEnumerative = BOGUS_GPU_LOCAL_PURE_ENUMERATIVE,
                Hybrid = BOGUS_GPU_LOCAL_HYBRID, RevHybrid = BOGUS_GPU_LOCAL_REV_HYBRID };
}

// BlockSolverBase + ConstrainedSolverBase: tolerance, iteration budget, norm, callback.
class SolverBase {
 public:
  using CallBackType = Signal<unsigned, double>;
  void setTol(double tol) { tol_ = tol; }
  double tol() const { return tol_; }
  void setMaxIters(unsigned n) { max_iters_ = n; }
  unsigned maxIters() const { return max_iters_; }
  void useInfinityNorm(bool on) { inf_ = on; }
  bool usesInfinityNorm() const { return inf_; }
  CallBackType& callback() { return callback_; }
  const CallBackType& callback() const { return callback_; }

 protected:
  SolverBase(double tol, unsigned max_iters) : tol_(tol), max_iters_(max_iters) {}
  double tol_;
  unsigned max_iters_;
  bool inf_ = false;
  CallBackType callback_;
};

// Coloring (Core/BlockSolvers/Coloring.hpp): update(true, W) turns the coloring order on.
class Coloring {
 public:
  template <class Matrix>
  void update(bool enable, const Matrix&) { enabled_ = enable; }
  void update(bool enable) { enabled_ = enable; }
  bool enabled() const { return enabled_; }

 private:
  bool enabled_ = false;
};

// GaussSeidel<WType> (GaussSeidelBase.hpp:39-91, GaussSeidel.hpp:122), defaults of GaussSeidelBase().
class GaussSeidel : public SolverBase {
 public:
  GaussSeidel() : SolverBase(1e-6, 250) {
    bogus_gpu_gs_options o;
    bogus_gpu_gs_options_default(&o);
    tol_ = o.tol;
    max_iters_ = o.max_iters;
    eval_every_ = o.eval_every;
    skip_tol_ = o.skip_tol;
    skip_iters_ = o.skip_iters;
    auto_reg_ = o.auto_regularization;
    try_zero_ = o.try_zero_as_well != 0;
    strategy_ = o.local_strategy;
  }
  void setMaxThreads(unsigned n = 0) { max_threads_ = n; }
  void setAutoRegularization(double r) { auto_reg_ = r; }
  void setEvalEvery(unsigned n) { eval_every_ = n; }
  void setSkipTol(double t) { skip_tol_ = t; }
  void setSkipIters(unsigned n) { skip_iters_ = n; }
  void doTryZeroAsWell(bool on = true) { try_zero_ = on; }
  void setLocalStrategy(local_soc_solver::Strategy s) { strategy_ = s; }
  Coloring& coloring() { return coloring_; }
  const Coloring& coloring() const { return coloring_; }
  unsigned evalEvery() const { return eval_every_; }
  double skipTol() const { return skip_tol_; }
  unsigned skipIters() const { return skip_iters_; }
  double autoRegularization() const { return auto_reg_; }
  bool tryZeroAsWell() const { return try_zero_; }

  bogus_gpu_gs_options options(bool static_problem) const {
    bogus_gpu_gs_options o;
    bogus_gpu_gs_options_default(&o);
    o.tol = tol_;
    o.max_iters = max_iters_;
    o.eval_every = eval_every_;
    o.skip_tol = skip_tol_;
    o.skip_iters = skip_iters_;
    o.auto_regularization = auto_reg_;
    o.try_zero_as_well = try_zero_ ? 1 : 0;
    o.use_infinity_norm = inf_ ? 1 : 0;
    o.static_problem = static_problem ? 1 : 0;
    o.local_strategy = strategy_;
    o.use_coloring = coloring_.enabled() ? 1 : 0;
    return o;
  }

 private:
  unsigned max_threads_ = 0, eval_every_ = 25, skip_iters_ = 10;
  double skip_tol_ = 1e-6, auto_reg_ = 0.0;
  bool try_zero_ = true;
  int strategy_ = BOGUS_GPU_LOCAL_REV_HYBRID;
  Coloring coloring_;
};

// ProductGaussSeidel<HType, MInvType, true>: the same setters, solved without forming W.
class ProductGaussSeidel : public GaussSeidel {};

// ProjectedGradient<WType> (ProjectedGradient.hpp:61-95), defaults of init().
class ProjectedGradient : public SolverBase {
 public:
  ProjectedGradient() : SolverBase(1e-6, 300) {
    bogus_gpu_pg_options o;
    bogus_gpu_pg_options_default(&o);
    tol_ = o.tol;
    max_iters_ = o.max_iters;
    ls_iters_ = o.ls_iters;
    opt_ = o.ls_optimistic_factor;
    pess_ = o.ls_pessimistic_factor;
    armijo_ = o.ls_armijo_coefficient;
    variant_ = o.variant;
    refine_ = o.refine_max_iters;
  }
  void setLineSearchIterations(unsigned n) { ls_iters_ = n; }
  void setLineSearchOptimisticFactor(double f) { opt_ = f; }
  void setLineSearchPessimisticFactor(double f) { pess_ = f; }
  void setLineSearchArmijoCoefficient(double f) { armijo_ = f; }
  void setDefaultVariant(projected_gradient::Variant v) { variant_ = v; }
  unsigned lineSearchIterations() const { return ls_iters_; }
  double lineSearchOptimisticFactor() const { return opt_; }
  double lineSearchPessimisticFactor() const { return pess_; }
  double lineSearchArmijoCoefficient() const { return armijo_; }
  projected_gradient::Variant defaultVariant() const { return (projected_gradient::Variant)variant_; }
  // extension: the FP32-refined solve (FP32 iterations, then up to refine_max_iters FP64 ones)
  void setMixedPrecision(bool on, unsigned refine_max_iters = 50) {
    mixed_ = on;
    refine_ = refine_max_iters;
  }
  // extension: APGD's momentum product by linearity (one pass over W fewer per momentum step)
  void setMomentumByLinearity(bool on) { lin_ = on; }
  // extension: the FP32 part of the FP32-refined solve ends once FP32 rounding stops its progress (0: never)
  void setFp32StallIterations(unsigned n) { stall_ = n; }
  // extension: FP32 correction products in the FP64 iterations of the FP32-refined solve (0: off)
  void setFp32CorrectionProducts(unsigned refresh = 100) { hy_ = refresh; }

  bogus_gpu_pg_options options(bool static_problem) const {
    bogus_gpu_pg_options o;
    bogus_gpu_pg_options_default(&o);
    o.tol = tol_;
    o.max_iters = max_iters_;
    o.ls_iters = ls_iters_;
    o.ls_optimistic_factor = opt_;
    o.ls_pessimistic_factor = pess_;
    o.ls_armijo_coefficient = armijo_;
    o.variant = variant_;
    o.use_infinity_norm = inf_ ? 1 : 0;
    o.static_problem = static_problem ? 1 : 0;
    o.mixed_precision = mixed_ ? 1 : 0;
    o.refine_max_iters = refine_;
    o.momentum_by_linearity = lin_ ? 1 : 0;
    o.fp32_stall_iters = stall_;
    o.fp32_products_refresh = hy_;
    return o;
  }

 private:
  unsigned ls_iters_ = 8, refine_ = 50, stall_ = 4, hy_ = 0;
  double opt_ = 1.25, pess_ = 0.5, armijo_ = 0.5;
  int variant_ = BOGUS_GPU_PG_APGD;
  bool mixed_ = false, lin_ = false;
};

// ADMM<HType> (ADMM.hpp:81-100), defaults of init().
class ADMM : public SolverBase {
 public:
  ADMM() : SolverBase(1e-6, 300) {
    bogus_gpu_admm_options o;
    bogus_gpu_admm_options_default(&o);
    tol_ = o.tol;
    max_iters_ = o.max_iters;
    step_ = o.step_size;
    variant_ = o.variant;
  }
  void setStepSize(double s) { step_ = s; }
  double stepSize() const { return step_; }
  void setDefaultVariant(admm::Variant v) { variant_ = v; }

  bogus_gpu_admm_options options() const {
    bogus_gpu_admm_options o;
    bogus_gpu_admm_options_default(&o);
    o.tol = tol_;
    o.max_iters = max_iters_;
    o.step_size = step_;
    o.variant = variant_;
    o.use_infinity_norm = inf_ ? 1 : 0;
    return o;
  }

 private:
  double step_ = 1e-2;
  int variant_ = BOGUS_GPU_ADMM_ACCELERATED;
};

// DualAMA<HType> (ADMM.hpp:170-236), defaults of init().
class DualAMA : public SolverBase {
 public:
  DualAMA() : SolverBase(1e-6, 300) {
    bogus_gpu_dual_ama_options o;
    bogus_gpu_dual_ama_options_default(&o);
    tol_ = o.tol;
    max_iters_ = o.max_iters;
    fp_ = o.fp_step_size;
    proj_ = o.proj_step_size;
    ls_iters_ = o.ls_iters;
    opt_ = o.ls_optimistic_factor;
    pess_ = o.ls_pessimistic_factor;
    variant_ = o.variant;
  }
  void setFpStepSize(double s) { fp_ = s; }
  void setProjStepSize(double s) { proj_ = s; }
  void setLineSearchIterations(unsigned n) { ls_iters_ = n; }
  void setLineSearchOptimisticFactor(double f) { opt_ = f; }
  void setLineSearchPessimisticFactor(double f) { pess_ = f; }
  void setDefaultVariant(admm::Variant v) { variant_ = v; }
  double fpStepSize() const { return fp_; }
  double projStepSize() const { return proj_; }

  bogus_gpu_dual_ama_options options() const {
    bogus_gpu_dual_ama_options o;
    bogus_gpu_dual_ama_options_default(&o);
    o.tol = tol_;
    o.max_iters = max_iters_;
    o.fp_step_size = fp_;
    o.proj_step_size = proj_;
    o.ls_iters = ls_iters_;
    o.ls_optimistic_factor = opt_;
    o.ls_pessimistic_factor = pess_;
    o.variant = variant_;
    o.use_infinity_norm = inf_ ? 1 : 0;
    return o;
  }

 private:
  double fp_ = 1e-1, proj_ = 1e-1, opt_ = 1.25, pess_ = 0.5;
  unsigned ls_iters_ = 6;
  int variant_ = BOGUS_GPU_ADMM_ACCELERATED;
};

// ---- the GPU handle ----------------------------------------------------------------------------------------
namespace detail {
class Handle {
 public:
  explicit Handle(int device) : device_(device) {}
  Handle(const Handle&) = delete;
  Handle& operator=(const Handle&) = delete;
  ~Handle() {
    if (h_) bogus_gpu_destroy(h_);
  }
  bogus_gpu_problem* get() {
    if (!h_) check(bogus_gpu_create(device_, &h_), false);
    return h_;
  }
  int device() const { return device_; }

 private:
  int device_;
  bogus_gpu_problem* h_ = nullptr;
};

struct CallbackBridge {
  static void fire(unsigned it, double res, void* user) { static_cast<const Signal<unsigned, double>*>(user)->trigger(it, res); }
  static void bind(bogus_gpu_problem* h, const Signal<unsigned, double>& s) {
    if (s.empty()) check(bogus_gpu_set_callback(h, nullptr, nullptr), false);
    else check(bogus_gpu_set_callback(h, &CallbackBridge::fire, const_cast<Signal<unsigned, double>*>(&s)), false);
  }
};
}  // namespace detail

// ---- PrimalFrictionProblem<3> (Interfaces/FrictionProblem.hpp:55-116) ----------------------------------------
template <unsigned Dimension>
struct PrimalFrictionProblem;

template <>
struct PrimalFrictionProblem<3> {
  using ADMMType = ADMM;
  using DualAMAType = DualAMA;
  using ProductGaussSeidelType = ProductGaussSeidel;

  explicit PrimalFrictionProblem(int device = 0) : handle_(new detail::Handle(device)) {}

  unsigned ndof = 6;            // dofs per body (uniform), at most 12
  std::vector<double> M;        // nbodies x ndof x ndof mass blocks, row-major (needed by DualAMA, computeMInv)
  std::vector<double> MInv;     // nbodies x ndof x ndof inverse mass blocks, row-major
  std::vector<double> E;        // n x 3 x 3 contact frames (contact basis to world), row-major; empty: identity
  std::vector<int> objA, objB;  // per contact: body A, body B (-1: none)
  std::vector<double> HA, HB;   // per contact: 3 x ndof Jacobian blocks, row-major, contact basis
  const double* f = nullptr;    // external forces (nbodies x ndof), NULL: 0
  const double* w = nullptr;    // free velocity in world coordinates (3 n), u = H v + E^T w
  const double* mu = nullptr;   // friction coefficients (n)

  unsigned nBodies() const { return ndof ? (unsigned)(MInv.empty() ? M.size() : MInv.size()) / (ndof * ndof) : 0; }
  unsigned nContacts() const { return (unsigned)objA.size(); }

  // MInv = M^-1 block by block (Gauss-Jordan elimination with partial pivoting).
  void computeMInv() {
    const unsigned d = ndof, nb = d ? (unsigned)M.size() / (d * d) : 0;
    MInv.assign(M.size(), 0.0);
    std::vector<double> a(2 * d * d);
    for (unsigned k = 0; k < nb; ++k) {
      for (unsigned i = 0; i < d; ++i)
        for (unsigned j = 0; j < 2 * d; ++j) a[i * 2 * d + j] = j < d ? M[(k * d + i) * d + j] : (j - d == i ? 1.0 : 0.0);
      for (unsigned c = 0; c < d; ++c) {
        unsigned p = c;
        for (unsigned i = c + 1; i < d; ++i)
          if (std::fabs(a[i * 2 * d + c]) > std::fabs(a[p * 2 * d + c])) p = i;
        if (a[p * 2 * d + c] == 0.0) throw Error(BOGUS_GPU_BAD_INPUT, "singular mass block");
        if (p != c)
          for (unsigned j = 0; j < 2 * d; ++j) std::swap(a[p * 2 * d + j], a[c * 2 * d + j]);
        const double inv = 1.0 / a[c * 2 * d + c];
        for (unsigned j = 0; j < 2 * d; ++j) a[c * 2 * d + j] *= inv;
        for (unsigned i = 0; i < d; ++i) {
          if (i == c) continue;
          const double s = a[i * 2 * d + c];
          if (s != 0.0)
            for (unsigned j = 0; j < 2 * d; ++j) a[i * 2 * d + j] -= s * a[c * 2 * d + j];
        }
      }
      for (unsigned i = 0; i < d; ++i)
        for (unsigned j = 0; j < d; ++j) MInv[(k * d + i) * d + j] = a[i * 2 * d + d + j];
    }
  }

  // solveWith(ADMMType&, lambda, v, r): primal ADMM on the SOC (static) problem, M^-1 as the prox operator
  // (PrimalFrictionProblem.cpp:61-73).
  double solveWith(ADMM& admm, double lambda, double* v, double* r) const {
    bogus_gpu_problem* h = upload();
    const bogus_gpu_admm_options o = admm.options();
    detail::CallbackBridge::bind(h, admm.callback());
    double res = 0.0;
    unsigned it = 0;
    check(bogus_gpu_solve_admm(h, &o, lambda, nullptr, f, w, mu, v, r, &res, &it));
    return res;
  }
  // solveWith(DualAMAType&, v, r, staticProblem) (PrimalFrictionProblem.cpp:78-99); needs M.
  double solveWith(DualAMA& dama, double* v, double* r, bool staticProblem = false) const {
    if (M.empty()) throw Error(BOGUS_GPU_BAD_INPUT, "DualAMA needs the mass blocks M");
    bogus_gpu_problem* h = upload();
    const bogus_gpu_dual_ama_options o = dama.options();
    detail::CallbackBridge::bind(h, dama.callback());
    double res = 0.0;
    unsigned it = 0;
    check(bogus_gpu_solve_dual_ama(h, &o, M.data(), f, w, mu, staticProblem ? 1 : 0, v, r, &res, &it));
    return res;
  }
  // solveWith(ProductGaussSeidelType&, r, staticProblem) (PrimalFrictionProblem.cpp:41-59).
  double solveWith(ProductGaussSeidel& pgs, double* r, bool staticProblem = false) const {
    bogus_gpu_problem* h = upload();
    bogus_gpu_gs_options o = pgs.options(staticProblem);
    o.use_coloring = 0;
    detail::CallbackBridge::bind(h, pgs.callback());
    double res = 0.0;
    unsigned it = 0;
    check(bogus_gpu_solve_product_gs(h, &o, f, w, mu, r, &res, &it));
    return res;
  }

 private:
  template <unsigned>
  friend struct DualFrictionProblem;
  // Uploads the primal data to `h` (the problem's own handle, or a dual problem's).
  void validate() const {
    const std::size_t n = objA.size();
    if (ndof == 0 || ndof > 12) throw Error(BOGUS_GPU_BAD_INPUT, "ndof must lie in 1..12");
    if (objB.size() != n || HA.size() != n * 3 * ndof || HB.size() != HA.size())
      throw Error(BOGUS_GPU_BAD_INPUT, "primal arrays of inconsistent sizes");
    if (MInv.empty() || MInv.size() % (ndof * ndof) != 0)
      throw Error(BOGUS_GPU_BAD_INPUT, "MInv not set (call computeMInv())");
    if (!E.empty() && E.size() != 9 * n) throw Error(BOGUS_GPU_BAD_INPUT, "E must hold 9 values per contact");
  }
  void upload_to(bogus_gpu_problem* h) const {
    const int n = (int)objA.size();
    check(bogus_gpu_set_primal(h, (int)nBodies(), (int)ndof, MInv.data(), n, objA.data(), objB.data(), HA.data(),
                               HB.data()),
          false);
    check(bogus_gpu_set_frames(h, E.empty() ? nullptr : E.data()), false);
  }
  bogus_gpu_problem* upload() const {
    validate();
    bogus_gpu_problem* h = handle_->get();
    upload_to(h);
    return h;
  }
  std::shared_ptr<detail::Handle> handle_;
};

// ---- DualFrictionProblem<3> (Interfaces/FrictionProblem.hpp:127-214) -----------------------------------------
template <unsigned Dimension>
struct DualFrictionProblem;

template <>
struct DualFrictionProblem<3> {
  using WType = SymmetricBlockMatrix3;
  using GaussSeidelType = GaussSeidel;
  using ProjectedGradientType = ProjectedGradient;

  explicit DualFrictionProblem(int device = 0) : handle_(new detail::Handle(device)) {}

  WType W;      // Delassus operator, lower triangle
  VectorXd b;   // u = W r + b
  VectorXd mu;  // friction coefficients

  // computeFrom (FrictionProblem.cpp:30-40): W = H M^-1 H^T and b = E^T w - H M^-1 f, assembled on the GPU; W,
  // b and mu are copied back into the members.
  void computeFrom(const PrimalFrictionProblem<3>& primal) {
    primal.validate();
    const int n = (int)primal.nContacts();
    if (n > 0 && (!primal.w || !primal.mu)) throw Error(BOGUS_GPU_BAD_INPUT, "w and mu must be set");
    bogus_gpu_problem* h = handle_->get();
    primal.upload_to(h);
    check(bogus_gpu_assemble_dual(h, primal.f, primal.w, primal.mu), false);
    download();
  }

  // solveWith(GaussSeidelType&, r, staticProblem = false) (FrictionProblem.cpp:42-47).
  double solveWith(GaussSeidel& gs, double* r, bool staticProblem = false) const {
    bogus_gpu_problem* h = sync();
    const bogus_gpu_gs_options o = gs.options(staticProblem);
    detail::CallbackBridge::bind(h, gs.callback());
    double res = 0.0;
    unsigned it = 0;
    check(bogus_gpu_solve_gs(h, &o, r, &res, &it));
    return res;
  }
  // solveWith(ProjectedGradientType&, r, staticProblem = true) (FrictionProblem.cpp:49-54).
  double solveWith(ProjectedGradient& pg, double* r, bool staticProblem = true) const {
    bogus_gpu_problem* h = sync();
    const bogus_gpu_pg_options o = pg.options(staticProblem);
    detail::CallbackBridge::bind(h, pg.callback());
    double res = 0.0;
    unsigned it = 0;
    check(bogus_gpu_solve_pg(h, &o, r, &res, &it));
    return res;
  }
  // evalWith (FrictionProblem.cpp:56-66): the solver's error function at r.
  double evalWith(const GaussSeidel& gs, const double* r, bool staticProblem = false) const {
    return eval(r, staticProblem, gs.usesInfinityNorm());
  }
  double evalWith(const ProjectedGradient& pg, const double* r, bool staticProblem = true) const {
    return eval(r, staticProblem, pg.usesInfinityNorm());
  }
  // solveCadoux (FrictionProblem.impl.hpp:76-92, Cadoux.hpp:44-91): the Coulomb problem as a sequence of SOCQPs.
  double solveCadoux(GaussSeidel& gs, double* r, unsigned cadouxIterations) const {
    bogus_gpu_problem* h = sync();
    const bogus_gpu_gs_options o = gs.options(true);
    detail::CallbackBridge::bind(h, gs.callback());
    double res = 0.0;
    unsigned it = 0;
    check(bogus_gpu_solve_cadoux_gs(h, &o, r, cadouxIterations, &res, &it));
    return res;
  }
  double solveCadoux(ProjectedGradient& pg, double* r, unsigned cadouxIterations) const {
    bogus_gpu_problem* h = sync();
    const bogus_gpu_pg_options o = pg.options(true);
    detail::CallbackBridge::bind(h, pg.callback());
    double res = 0.0;
    unsigned it = 0;
    check(bogus_gpu_solve_cadoux_pg(h, &o, r, cadouxIterations, &res, &it));
    return res;
  }
  // applyPermutation / undoPermutation / permuted (FrictionProblem.hpp:198-207): W, b and mu are permuted in
  // place; the solves keep taking r in the original order.
  void applyPermutation(const std::vector<std::size_t>& permutation) {
    bogus_gpu_problem* h = sync();
    std::vector<int> p(permutation.begin(), permutation.end());
    check(bogus_gpu_apply_permutation(h, p.data()), false);
    download();
  }
  void undoPermutation() {
    bogus_gpu_problem* h = sync();
    check(bogus_gpu_undo_permutation(h), false);
    download();
  }
  bool permuted() const {
    int p = 0;
    check(bogus_gpu_permuted(handle_->get(), &p), false);
    return p != 0;
  }
  // The underlying C handle (for the C ABI's extensions: batches, adjoint, device pointers).
  bogus_gpu_problem* handle() const { return sync(); }

 private:
  double eval(const double* r, bool static_problem, bool inf) const {
    bogus_gpu_problem* h = sync();
    double res = 0.0;
    check(bogus_gpu_eval(h, r, static_problem ? 1 : 0, inf ? 1 : 0, &res), false);
    return res;
  }
  // Uploads W, b and mu when they changed since the last upload or download.
  bogus_gpu_problem* sync() const {
    const bool stale = !synced_ || W.generation() != w_gen_ || b.generation() != b_gen_ || mu.generation() != mu_gen_;
    const int n = W.rowsOfBlocks();
    if (stale && (b.size() != 3 * (std::size_t)n || mu.size() != (std::size_t)n))
      throw Error(BOGUS_GPU_BAD_INPUT, "b must hold 3 n values and mu n values");
    bogus_gpu_problem* h = handle_->get();
    if (stale) {
      check(bogus_gpu_set_dual(h, n, W.outerIndexPtr(), W.innerIndexPtr(), W.blockPtr(), 1, b.data(), mu.data()),
            false);
      mark();
    }
    return h;
  }
  // Copies the device-held problem (stored order) into W, b and mu.
  void download() {
    bogus_gpu_problem* h = handle_->get();
    int nnzb = 0;
    check(bogus_gpu_get_dual_lower(h, nullptr, nullptr, nullptr, &nnzb), false);
    int n = 0;
    {
      int full = 0;
      check(bogus_gpu_nnzb(h, &full), false);
      n = 2 * nnzb - full;  // the lower triangle holds (full + n) / 2 blocks
    }
    std::vector<int> outer(n + 1), inner(nnzb);
    std::vector<double> blocks(9 * (std::size_t)nnzb);
    check(bogus_gpu_get_dual_lower(h, outer.data(), inner.data(), blocks.data(), &nnzb), false);
    W.setFromLower(n, outer.data(), inner.data(), blocks.data());
    b.resize(3 * (std::size_t)n);
    mu.resize((std::size_t)n);
    check(bogus_gpu_get_dual_rhs(h, b.data(), mu.data()), false);
    mark();
  }
  void mark() const {
    synced_ = true;
    w_gen_ = W.generation();
    b_gen_ = b.generation();
    mu_gen_ = mu.generation();
  }
  std::shared_ptr<detail::Handle> handle_;
  mutable bool synced_ = false;
  mutable unsigned long long w_gen_ = 0, b_gen_ = 0, mu_gen_ = 0;
};

}  // namespace bogus_gpu

#endif  // BOGUS_GPU_HPP
