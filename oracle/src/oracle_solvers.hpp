// ORACLE — test infrastructure only (see oracle_math.hpp).
//
// CPU restatement of the reference's block solvers on a dual friction problem (W, b, mu):
//   ConstrainedSolverBase  (Core/BlockSolvers/ConstrainedSolverBase.impl.hpp)
//   GaussSeidel            (Core/BlockSolvers/GaussSeidel.impl.hpp, GaussSeidelBase.impl.hpp)
//   ProjectedGradient      (Core/BlockSolvers/ProjectedGradient.impl.hpp), all five variants
//   ADMM / QuadraticProxOp (Core/BlockSolvers/ADMM.impl.hpp:29-127)
// Vectors are contact-major: x[3i + k]. Every global dot product or residual is the canonicalSum() of
// per-contact values; per-contact values use the evaluation order of oracle_math.hpp.
#pragma once

#include <chrono>
#include <cfloat>
#include <functional>
#include <vector>

#include "oracle_math.hpp"
#include "oracle_sparse.hpp"

namespace oracle {

using Callback = std::function<void(unsigned, double)>;

struct Law {
  bool desaxce;        // Coulomb (De Saxce change of variable) or plain SOC
  int strat;           // local_soc_solver::Strategy
  const double* mu;
};

struct SolverBase {
  const BSR* W = nullptr;  // full view (both triangles)
  std::vector<double> scaling;
  bool useInfinityNorm = false;
  double tol = 1e-6;
  unsigned maxIters = 300;
  Callback callback;

  // updateScalings (ConstrainedSolverBase.impl.hpp:78-118): max(1, trace(W_ii)/3), 1 without a diagonal block
  void setMatrix(const BSR& M) {
    W = &M;
    scaling.assign(M.n, 1.0);
    for (int i = 0; i < M.n; ++i) {
      const int p = M.diagPtr(i);
      if (p >= 0) {
        const double* B = M.block(p);
        scaling[i] = dmax(1.0, ((B[0] + B[4]) + B[8]) / 3.0);
      }
    }
  }
  int n() const { return W->n; }

  // eval (ConstrainedSolverBase.impl.hpp:21-74)
  double eval(const Law& law, const double* y, const double* x) const {
    const int N = n();
    std::vector<double> v(N);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
      const double s = scaling[i];
      const double lx[3] = {x[3 * i] * s, x[3 * i + 1] * s, x[3 * i + 2] * s};
      v[i] = lawEval(law.desaxce, law.mu[i], lx, &y[3 * i]);
    }
    if (useInfinityNorm) return maxOf(v.data(), N);
    return canonicalSum(v.data(), N) / (double)(1 + N);
  }
  void projectOnConstraints(const Law& law, double* x) const {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n(); ++i) projectCone(law.mu[i], &x[3 * i]);
  }
  void dualityCOVAll(const Law& law, const double* y, double* s) const {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n(); ++i) dualityCOV(law.desaxce, law.mu[i], &y[3 * i], &s[3 * i]);
  }
  void trigger(unsigned it, double r) const {
    if (callback) callback(it, r);
  }
};

// Per-contact reduction helpers (canonical)
template <typename F>
inline double reduceContacts(int n, F f) {
  std::vector<double> v(n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) v[i] = f(i);
  return canonicalSum(v.data(), n);
}

// ---------------------------------------------------------------------------------------------
// Gauss-Seidel (GaussSeidel.impl.hpp:62-205, GaussSeidelBase.impl.hpp:21-77)
// ---------------------------------------------------------------------------------------------
struct GaussSeidel : SolverBase {
  unsigned evalEvery = 25;
  double skipTol = 1e-6;
  unsigned skipIters = 10;
  double autoRegularization = 0.0;
  bool tryZeroAsWell = true;
  std::vector<int> perm, colors;   // Coloring: permutation + color offsets
  std::vector<double> local;       // 9 n, diagonal blocks (+ regularization)
  std::vector<double> reg;         // n
  // > 1: with two colors or more, each color's contacts are updated by that many OpenMP threads, as
  // GaussSeidel::innerLoop does with maxThreads != 1 (GaussSeidel.impl.hpp:77-114, one `omp for` per color).
  // The step-size reference ndxRef is shared between the threads, as there, so which contacts skip the next
  // sweeps, and hence the iterates, depend on the thread timing: a CPU timing baseline only, never a parity
  // reference.
  int threads = 1;
  mutable double sweepSeconds = 0.0;  // wall time of the last solve's sweeps and evaluations (no setup)

  GaussSeidel() { tol = 1e-6; maxIters = 250; }

  // setMatrix + updateLocalMatrices + processLocalMatrices; coloring reset to one color (natural order)
  void setMatrix(const BSR& M) {
    SolverBase::setMatrix(M);
    const int N = M.n;
    if ((int)perm.size() != N) {
      perm.resize(N);
      std::iota(perm.begin(), perm.end(), 0);
      colors = {0, N};
    }
    local.assign(9 * (size_t)N, 0.0);
    reg.assign(N, 0.0);
    for (int i = 0; i < N; ++i) {
      const int p = M.diagPtr(i);
      if (p >= 0) std::copy(M.block(p), M.block(p) + 9, &local[9 * (size_t)i]);
      const double* D = &local[9 * (size_t)i];
      scaling[i] = dmax(1.0, ((D[0] + D[4]) + D[8]) / 3.0);
      if (autoRegularization > 0.) {
        const double lmin = minEigenSymmetric3(D);
        reg[i] = dmax(0.0, autoRegularization - lmin);
        local[9 * (size_t)i + 0] += reg[i];
        local[9 * (size_t)i + 4] += reg[i];
        local[9 * (size_t)i + 8] += reg[i];
      }
    }
  }

  // Smallest eigenvalue of a symmetric 3x3 block by cyclic Jacobi rotations (the reference takes the real
  // parts of Eigen's general eigenvalues; W_ii is symmetric so both agree up to rounding).
  static double minEigenSymmetric3(const double* D) {
    double a[9];
    for (int k = 0; k < 9; ++k) a[k] = D[k];
    for (int sweep = 0; sweep < 50; ++sweep) {
      const double off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
      if (off == 0.0) break;
      for (int p = 0; p < 2; ++p)
        for (int q = p + 1; q < 3; ++q) {
          const double apq = a[3 * p + q];
          if (apq == 0.0) continue;
          const double theta = (a[3 * q + q] - a[3 * p + p]) / (2.0 * apq);
          const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
          const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
          for (int k = 0; k < 3; ++k) {  // A <- A J
            const double akp = a[3 * k + p], akq = a[3 * k + q];
            a[3 * k + p] = c * akp - s * akq;
            a[3 * k + q] = s * akp + c * akq;
          }
          for (int k = 0; k < 3; ++k) {  // A <- J^T A
            const double apk = a[3 * p + k], aqk = a[3 * q + k];
            a[3 * p + k] = c * apk - s * aqk;
            a[3 * q + k] = s * apk + c * aqk;
          }
        }
    }
    return dmin(dmin(a[0], a[4]), a[8]);
  }

  double evalAndKeepBest(const Law& law, const double* x, const double* y, std::vector<double>& x_best,
                         double& err_best) const {
    const double err = eval(law, y, x);
    if (err < err_best) {
      x_best.assign(x, x + 3 * (size_t)n());
      err_best = err;
    }
    return err;
  }

  void innerLoop(const Law& law, const double* b, std::vector<unsigned char>& skip, double& ndxRef, double* x) const {
    const double absSkipTol = dmin(skipTol, tol);
    const double absSkipIters = dmin((double)skipIters, (double)(unsigned)std::sqrt((double)skip.size()));
    if (threads > 1 && colors.size() > 2 && (size_t)n() > (size_t)threads * (size_t)threads) {
      double ndx = ndxRef;
#pragma omp parallel num_threads(threads)
      for (size_t c = 0; c + 1 < colors.size(); ++c) {
#pragma omp for schedule(static)
        for (int pi = colors[c]; pi < colors[c + 1]; ++pi) {
          const int i = perm[pi];
          if (skip[i]) {
            --skip[i];
            continue;
          }
          double lx[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
          double lb[3];
          for (int k = 0; k < 3; ++k) lb[k] = b[3 * i + k] - reg[i] * lx[k];
          splitRowMultiply(*W, i, x, lb);
          double ldx[3] = {-lx[0], -lx[1], -lx[2]};
          const bool ok = lawSolveLocal(law.desaxce, law.strat, &local[9 * (size_t)i], lb, lx, law.mu[i], scaling[i]);
          for (int k = 0; k < 3; ++k) ldx[k] = ldx[k] + lx[k];
          if (!ok) {
            ldx[0] *= .5; ldx[1] *= .5; ldx[2] *= .5;
          }
          for (int k = 0; k < 3; ++k) x[3 * i + k] = x[3 * i + k] + ldx[k];
          const double s2 = scaling[i] * scaling[i];
          const double nx2 = s2 * sq3(lx);
          const double ndx2 = s2 * sq3(ldx);
          double ref;
#pragma omp atomic read
          ref = ndx;
          if (ndx2 > ref) {
#pragma omp atomic write
            ndx = ndx2;
            ref = ndx2;
          }
          if (dmin(nx2, ndx2) < absSkipTol || ndx2 < skipTol * dmin(nx2, ref))
            skip[i] = (unsigned char)absSkipIters;
        }
      }
      ndxRef = ndx;
      return;
    }
    for (size_t c = 0; c + 1 < colors.size(); ++c) {
      for (int pi = colors[c]; pi < colors[c + 1]; ++pi) {
        const int i = perm[pi];
        if (skip[i]) {
          --skip[i];
          continue;
        }
        double lx[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
        double lb[3];
        for (int k = 0; k < 3; ++k) lb[k] = b[3 * i + k] - reg[i] * lx[k];
        splitRowMultiply(*W, i, x, lb);
        double ldx[3] = {-lx[0], -lx[1], -lx[2]};
        const bool ok = lawSolveLocal(law.desaxce, law.strat, &local[9 * (size_t)i], lb, lx, law.mu[i], scaling[i]);
        for (int k = 0; k < 3; ++k) ldx[k] = ldx[k] + lx[k];
        if (!ok) {
          ldx[0] *= .5; ldx[1] *= .5; ldx[2] *= .5;
        }
        for (int k = 0; k < 3; ++k) x[3 * i + k] = x[3 * i + k] + ldx[k];
        const double s2 = scaling[i] * scaling[i];
        const double nx2 = s2 * sq3(lx);
        const double ndx2 = s2 * sq3(ldx);
        if (ndx2 > ndxRef) ndxRef = ndx2;
        if (dmin(nx2, ndx2) < absSkipTol || ndx2 < skipTol * dmin(nx2, ndxRef))
          skip[i] = (unsigned char)absSkipIters;
      }
    }
  }

  // solve(law, b, x, tryZeroAsWell) == solveWithLinearConstraints(law, Zero, b, x, tryZero, 0)
  double solve(const Law& law, const double* b, double* x, unsigned* itersOut = nullptr) const {
    const int N = n();
    const size_t n3 = 3 * (size_t)N;
    std::vector<double> y(n3), x_best;
    double err_best = DBL_MAX;
    spmv(*W, x, y.data(), b);
    evalAndKeepBest(law, x, y.data(), x_best, err_best);
    if (tryZeroAsWell) {  // tryZero (GaussSeidelBase.impl.hpp:61-77)
      std::vector<double> zero(n3, 0.0);
      const double err_zero = eval(law, b, zero.data());
      if (err_zero < err_best) {
        err_best = err_zero;
        x_best.assign(n3, 0.0);
        std::fill(x, x + n3, 0.0);
      } else {
        std::copy(x_best.begin(), x_best.end(), x);
      }
    }
    trigger(0, err_best);
    std::vector<unsigned char> skip(N, 0);
    double ndxRef = 0;
    unsigned GSIter;
    const auto t0 = std::chrono::steady_clock::now();
    for (GSIter = 1; GSIter <= maxIters; ++GSIter) {
      innerLoop(law, b, skip, ndxRef, x);
      if (0 == (GSIter % evalEvery)) {
        spmv(*W, x, y.data(), b);
        const double err = evalAndKeepBest(law, x, y.data(), x_best, err_best);
        trigger(GSIter, err);
        if (err < tol) break;
        ndxRef /= evalEvery;
      }
    }
    sweepSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (GSIter > maxIters) std::copy(x_best.begin(), x_best.end(), x);
    if (itersOut) *itersOut = GSIter > maxIters ? maxIters : GSIter;
    return err_best;
  }
};

// ---------------------------------------------------------------------------------------------
// Projected gradient (ProjectedGradient.impl.hpp)
// ---------------------------------------------------------------------------------------------
enum PGVariant { Standard = 0, Descent = 1, Conjugated = 2, APGD = 3, SPG = 4 };  // projected_gradient::Variant

struct ProjectedGradient : SolverBase {
  unsigned lsIters = 8;
  double lsOptimisticFactor = 1.25, lsPessimisticFactor = .5, lsArmijoCoefficient = .5;
  int variant = APGD;
  // Not in the reference: APGD's momentum product formed by linearity, W x = W xs + beta (W xs - W prev) with
  // x = xs + beta (xs - prev), from the trial's product W xs and the kept product of prev, in place of the
  // product W x of ProjectedGradient.impl.hpp:141 (same fma form as x itself). One pass over W fewer per
  // momentum step; the iterates differ from the reference's by the rounding of the two forms.
  bool linMomentum = false;
  // Not in the reference: FP32 correction products (APGD). Each trial and momentum product is
  // W x_ref + W32 (v - x_ref)_32 (spmv32 on the correction rounded to float, added to the FP64 W x_ref); the
  // first momentum step on or after every hyRefresh iterations takes the FP64 product instead, which becomes
  // W x_ref with x_ref = x. The solve ends (not converged) when its best residual has not improved by 1 % in
  // 10 hyRefresh iterations. 0: off.
  unsigned hyRefresh = 0;

  ProjectedGradient() { tol = 1e-6; maxIters = 300; }

  bool testResidual(const Law& law, unsigned it, const double* x, const double* y, std::vector<double>& x_best,
                    double& min_res, double* resOut = nullptr) const {
    const double res = eval(law, y, x);
    if (resOut) *resOut = res;
    trigger(it, res);
    if (0 == it || res < min_res) {
      x_best.assign(x, x + 3 * (size_t)n());
      min_res = res;
    }
    return res < tol;
  }

  // guess_alpha (:21-28)
  void guessAlpha(const double* x, double& alpha) const {
    const int N = n();
    std::vector<double> d(3 * (size_t)N), Md(3 * (size_t)N);
    for (size_t k = 0; k < d.size(); ++k) d[k] = x[k] - 1.0;
    spmv(*W, d.data(), Md.data());
    const double nMx = reduceContacts(N, [&](int i) { return sq3(&Md[3 * i]); });
    if (nMx > 1.e-16) alpha = dmin(1., reduceContacts(N, [&](int i) { return sq3(&d[3 * i]); }) / nMx);
  }

  double objective(const double* x, const double* Mx, const double* b, const double* s) const {
    return reduceContacts(n(), [&](int i) {
      double t[3];
      for (int k = 0; k < 3; ++k) t[k] = (0.5 * Mx[3 * i + k] + b[3 * i + k]) + s[3 * i + k];
      return dot3(&x[3 * i], t);
    });
  }

  double solve(const Law& law, const double* b, double* x, unsigned* itersOut = nullptr) const {
    switch (variant) {
      case APGD: return solveAPGD(law, b, x, true, itersOut);
      case Descent: return solveAPGD(law, b, x, false, itersOut);
      case SPG: return solveSPG(law, b, x, itersOut);
      case Standard: return solveStandard(law, b, x, itersOut);
      case Conjugated: return solveConjugated(law, b, x, itersOut);
    }
    return -1;
  }

  // PgMethod<APGD / Descent> (:74-155)
  double solveAPGD(const Law& law, const double* b, double* x, bool apgd, unsigned* itersOut) const {
    const int N = n();
    const size_t n3 = 3 * (size_t)N;
    std::vector<double> Mx(n3), y(n3), xs(n3), s(n3), prev, x_best, Mprev;
    projectOnConstraints(law, x);
    spmv(*W, x, Mx.data());
    double theta = 1., q = 0;
    prev.assign(x, x + n3);
    if (linMomentum) Mprev = Mx;  // W prev
    // FP32 correction products (hyRefresh > 0)
    std::vector<float> W32, d32, p32;
    std::vector<double> xref, wxref;
    unsigned nextRefresh = hyRefresh, hyBestIt = 0;
    double hyBest = 0.0;
    if (hyRefresh) {
      W32.resize(W->val.size());
      for (size_t k = 0; k < W32.size(); ++k) W32[k] = (float)W->val[k];
      d32.resize(n3);
      p32.resize(n3);
      xref.assign(x, x + n3);
      wxref = Mx;
    }
    auto product = [&](const double* v, double* out) {
      if (!hyRefresh) {
        spmv(*W, v, out);
        return;
      }
      for (size_t k = 0; k < n3; ++k) d32[k] = (float)(v[k] - xref[k]);
      spmv32(*W, W32.data(), d32.data(), p32.data());
      for (size_t k = 0; k < n3; ++k) out[k] = wxref[k] + (double)p32[k];
    };
    double alpha = 1.;
    guessAlpha(x, alpha);
    double min_res = -1;
    unsigned it;
    for (it = 0; it < maxIters; ++it) {
      for (size_t k = 0; k < n3; ++k) y[k] = Mx[k] + b[k];
      double res = 0.0;
      if (testResidual(law, it, x, y.data(), x_best, min_res, &res)) break;
      if (hyRefresh) {
        if (it == 0 || res < 0.99 * hyBest) {
          hyBest = res;
          hyBestIt = it;
        }
        if (it - hyBestIt >= 10u * hyRefresh) break;
      }
      dualityCOVAll(law, y.data(), s.data());
      for (size_t k = 0; k < n3; ++k) y[k] = y[k] + s[k];
      const double J = objective(x, Mx.data(), b, s.data());
      double Js = J;
      alpha *= lsOptimisticFactor;
      for (unsigned ls = 0; ls < lsIters; ++ls, alpha *= lsPessimisticFactor) {
        for (size_t k = 0; k < n3; ++k) xs[k] = std::fma(-alpha, y[k], x[k]);
        projectOnConstraints(law, xs.data());
        product(xs.data(), Mx.data());
        Js = objective(xs.data(), Mx.data(), b, s.data());
        const double decr = reduceContacts(N, [&](int i) {
          const double d[3] = {xs[3 * i] - x[3 * i], xs[3 * i + 1] - x[3 * i + 1], xs[3 * i + 2] - x[3 * i + 2]};
          return dot3(&y[3 * i], d);
        });
        const double nrm = reduceContacts(N, [&](int i) {
          const double d[3] = {xs[3 * i] - x[3 * i], xs[3 * i + 1] - x[3 * i + 1], xs[3 * i + 2] - x[3 * i + 2]};
          return sq3(d);
        });
        if (Js < (J + decr) + (.5 / alpha) * nrm) break;
      }
      const double decr2 = reduceContacts(N, [&](int i) {
        const double d[3] = {xs[3 * i] - prev[3 * i], xs[3 * i + 1] - prev[3 * i + 1], xs[3 * i + 2] - prev[3 * i + 2]};
        return dot3(d, &y[3 * i]);
      });
      if (apgd && decr2 < 0) {
        const double beta = nesterovInertia(theta, q);
        for (size_t k = 0; k < n3; ++k) x[k] = std::fma(beta, xs[k] - prev[k], xs[k]);
        if (linMomentum) {
          // Mx holds W xs (the accepted trial's product)
          for (size_t k = 0; k < n3; ++k) {
            const double mxs = Mx[k];
            Mx[k] = std::fma(beta, mxs - Mprev[k], mxs);
            Mprev[k] = mxs;
          }
        } else if (hyRefresh && it + 1 >= nextRefresh) {
          spmv(*W, x, Mx.data());  // refresh: x_ref = x, W x_ref = W x
          xref.assign(x, x + n3);
          wxref = Mx;
          nextRefresh = it + 1 + hyRefresh;
        } else {
          product(x, Mx.data());
        }
      } else {
        std::copy(xs.begin(), xs.end(), x);
        theta = 1.;
        if (linMomentum) Mprev = Mx;
      }
      prev = xs;
    }
    std::copy(x_best.begin(), x_best.end(), x);
    if (itersOut) *itersOut = it;
    return min_res;
  }

  // PgMethod<SPG> (:288-351)
  double solveSPG(const Law& law, const double* b, double* x, unsigned* itersOut) const {
    const int N = n();
    const size_t n3 = 3 * (size_t)N;
    std::vector<double> Mx(n3), y(n3), xs(n3), s(n3), z(n3), w(n3), prev, x_best;
    projectOnConstraints(law, x);
    prev.assign(x, x + n3);
    spmv(*W, x, Mx.data());
    double theta = 1, q = 0;
    const double a_min = 1.e-6, a_max = 1.e6;
    double alpha = 1;
    guessAlpha(x, alpha);
    double min_res = -1;
    unsigned it;
    for (it = 0; it < maxIters; ++it) {
      for (size_t k = 0; k < n3; ++k) y[k] = Mx[k] + b[k];
      if (testResidual(law, it, x, y.data(), x_best, min_res)) break;
      dualityCOVAll(law, y.data(), s.data());
      for (size_t k = 0; k < n3; ++k) y[k] = y[k] + s[k];
      for (size_t k = 0; k < n3; ++k) xs[k] = std::fma(-alpha, y[k], x[k]);
      projectOnConstraints(law, xs.data());
      const double decr = reduceContacts(N, [&](int i) {
        const double d[3] = {xs[3 * i] - prev[3 * i], xs[3 * i + 1] - prev[3 * i + 1], xs[3 * i + 2] - prev[3 * i + 2]};
        return dot3(d, &y[3 * i]);
      });
      if (decr < 0.) {
        const double beta = nesterovInertia(theta, q);
        for (size_t k = 0; k < n3; ++k) {
          w[k] = std::fma(beta, xs[k] - prev[k], xs[k]) - x[k];
          x[k] = x[k] + w[k];
        }
      } else {
        for (size_t k = 0; k < n3; ++k) {
          w[k] = xs[k] - x[k];
          x[k] = xs[k];
        }
        theta = 1.;
      }
      for (size_t k = 0; k < n3; ++k) z[k] = -Mx[k];
      spmv(*W, x, Mx.data());
      prev = xs;
      for (size_t k = 0; k < n3; ++k) z[k] = z[k] + Mx[k];
      const double wz = reduceContacts(N, [&](int i) { return dot3(&w[3 * i], &z[3 * i]); });
      const double zz = reduceContacts(N, [&](int i) { return sq3(&z[3 * i]); });
      alpha = wz / zz;
      alpha = dmin(a_max, dmax(a_min, alpha));
    }
    std::copy(x_best.begin(), x_best.end(), x);
    if (itersOut) *itersOut = it;
    return min_res;
  }

  // armijo_ls (:54-72) on the objective with linear part bs = b + s
  void armijoLS(const Law& law, const double* x, const double* bs, const double* dir, const double* grad, double J,
                double& alpha, double* xs, double& Js, double* Mx) const {
    const int N = n();
    const size_t n3 = 3 * (size_t)N;
    Js = J;
    std::vector<double> zero(n3, 0.0);
    for (unsigned ls = 0; ls < lsIters; ++ls, alpha *= lsPessimisticFactor) {
      for (size_t k = 0; k < n3; ++k) xs[k] = std::fma(alpha, dir[k], x[k]);
      projectOnConstraints(law, xs);
      spmv(*W, xs, Mx);
      Js = objective(xs, Mx, bs, zero.data());
      const double decr = reduceContacts(N, [&](int i) {
        const double d[3] = {xs[3 * i] - x[3 * i], xs[3 * i + 1] - x[3 * i + 1], xs[3 * i + 2] - x[3 * i + 2]};
        return dot3(&grad[3 * i], d);
      });
      if (Js < J + lsArmijoCoefficient * decr) break;
    }
  }

  // PgMethod<Standard> (:157-209)
  double solveStandard(const Law& law, const double* b, double* x, unsigned* itersOut) const {
    const int N = n();
    const size_t n3 = 3 * (size_t)N;
    std::vector<double> Mx(n3), y(n3), xs(n3), s(n3), pg(n3), Mpg(n3), bs(n3), x_best;
    projectOnConstraints(law, x);
    spmv(*W, x, Mx.data());
    double alpha = 1;
    double min_res = -1;
    unsigned it;
    for (it = 0; it < maxIters; ++it) {
      for (size_t k = 0; k < n3; ++k) y[k] = Mx[k] + b[k];
      if (testResidual(law, it, x, y.data(), x_best, min_res)) break;
      dualityCOVAll(law, y.data(), s.data());
      for (size_t k = 0; k < n3; ++k) y[k] = y[k] + s[k];
      const double J = objective(x, Mx.data(), b, s.data());
      for (size_t k = 0; k < n3; ++k) xs[k] = x[k] - y[k];
      projectOnConstraints(law, xs.data());
      for (size_t k = 0; k < n3; ++k) pg[k] = x[k] - xs[k];
      spmv(*W, pg.data(), Mpg.data());
      const double num = reduceContacts(N, [&](int i) { return dot3(&y[3 * i], &pg[3 * i]); });
      const double den = reduceContacts(N, [&](int i) { return dot3(&pg[3 * i], &Mpg[3 * i]); });
      const double beta = -num / den;
      for (size_t k = 0; k < n3; ++k) pg[k] *= beta;
      double Js;
      alpha = dmin(1., alpha * lsOptimisticFactor);
      for (size_t k = 0; k < n3; ++k) bs[k] = b[k] + s[k];
      armijoLS(law, x, bs.data(), pg.data(), y.data(), J, alpha, xs.data(), Js, Mx.data());
      std::copy(xs.begin(), xs.end(), x);
    }
    std::copy(x_best.begin(), x_best.end(), x);
    if (itersOut) *itersOut = it;
    return min_res;
  }

  // PgMethod<Conjugated> (:211-286)
  double solveConjugated(const Law& law, const double* b, double* x, unsigned* itersOut) const {
    const int N = n();
    const size_t n3 = 3 * (size_t)N;
    std::vector<double> Mx(n3), y(n3), xs(n3), s(n3), dir(n3), prev_dir(n3), prev_pg, bs(n3), x_best;
    projectOnConstraints(law, x);
    spmv(*W, x, Mx.data());
    prev_pg.assign(x, x + n3);
    double prev_n2 = 0;
    double alpha = 1.;
    double min_res = -1;
    unsigned it;
    for (it = 0; it < maxIters; ++it) {
      for (size_t k = 0; k < n3; ++k) y[k] = Mx[k] + b[k];
      if (testResidual(law, it, x, y.data(), x_best, min_res)) break;
      dualityCOVAll(law, y.data(), s.data());
      for (size_t k = 0; k < n3; ++k) y[k] = y[k] + s[k];
      const double J = objective(x, Mx.data(), b, s.data());
      {
        for (size_t k = 0; k < n3; ++k) xs[k] = x[k] - y[k];
        projectOnConstraints(law, xs.data());
        for (size_t k = 0; k < n3; ++k) xs[k] = x[k] - xs[k];
        const double ng2 = reduceContacts(N, [&](int i) { return sq3(&xs[3 * i]); });
        if (prev_n2 == 0.) {
          for (size_t k = 0; k < n3; ++k) dir[k] = -y[k];
        } else {
          const double den = reduceContacts(N, [&](int i) {
            const double d[3] = {xs[3 * i] - prev_pg[3 * i], xs[3 * i + 1] - prev_pg[3 * i + 1],
                                 xs[3 * i + 2] - prev_pg[3 * i + 2]};
            return dot3(&prev_dir[3 * i], d);
          });
          const double xp = reduceContacts(N, [&](int i) { return dot3(&xs[3 * i], &prev_pg[3 * i]); });
          const double beta = (den < 1.e-12) ? dmax(0., (ng2 - xp)) / prev_n2 : dmax(0., (ng2 - xp)) / den;
          for (size_t k = 0; k < n3; ++k) dir[k] = beta * prev_dir[k] - y[k];
          const double dy = reduceContacts(N, [&](int i) { return dot3(&dir[3 * i], &y[3 * i]); });
          if (dy >= 0.)
            for (size_t k = 0; k < n3; ++k) dir[k] = -y[k];
        }
        prev_pg = xs;
        prev_n2 = ng2;
      }
      double Js;
      alpha = alpha * lsOptimisticFactor;
      for (size_t k = 0; k < n3; ++k) bs[k] = b[k] + s[k];
      armijoLS(law, x, bs.data(), dir.data(), y.data(), J, alpha, xs.data(), Js, Mx.data());
      for (size_t k = 0; k < n3; ++k) prev_dir[k] = (xs[k] - x[k]) / alpha;
      std::copy(xs.begin(), xs.end(), x);
    }
    std::copy(x_best.begin(), x_best.end(), x);
    if (itersOut) *itersOut = it;
    return min_res;
  }
};

// ---------------------------------------------------------------------------------------------
// ProductGaussSeidel<HType, MInvType, true> (Core/BlockSolvers/ProductGaussSeidel.impl.hpp:108-296), as
// PrimalFrictionProblem::solveWith(ProductGaussSeidelType&, r, staticProblem) (PrimalFrictionProblem.cpp:41-59)
// runs it: Gauss-Seidel on W = H M^-1 H^T without forming W. It keeps Mx = M^-1 H^T x (DMt x) per body:
//   local_i = sum_t H_t T_t (T = M^-1 H^T per slot; W's diagonal block as assembleW forms it) + reg I;
//   contact i: lb = b_i - local_i x_i + H_i Mx (rowMultiply), local solve, x_i += dx, Mx += T_i dx (colMultiply);
//   every evalEvery sweeps Mx is recomputed from x and y = b + H Mx gives the error.
// Orders: Mx_b chains over b's contacts in increasing index, then the 3 components; H_i Mx adds, slot by slot
// in body order, the dof chain sum to lb; T_i dx is the dot3 chain, added to Mx; local_i x_i is the dot3 chain
// per row, subtracted from b_i. The sweep visits the contacts in their own order (no coloring).
// ---------------------------------------------------------------------------------------------
struct ProductGaussSeidel : SolverBase {
  unsigned evalEvery = 25;
  double skipTol = 1e-6;
  unsigned skipIters = 10;
  double autoRegularization = 0.0;
  bool tryZeroAsWell = true;
  const Primal* P = nullptr;
  BSR shape;                  // n only (SolverBase::eval)
  std::vector<double> T;      // slots, d x 3
  std::vector<double> local;  // 9 n (+ regularization)
  std::vector<double> reg;    // n
  std::vector<std::vector<std::pair<int, int>>> byBody;  // (contact, slot), increasing contact

  ProductGaussSeidel() { tol = 1e-6; maxIters = 250; }

  void setPrimal(const Primal& Pr) {
    P = &Pr;
    const int n = Pr.ncontacts, d = Pr.ndof;
    shape.n = n;
    W = &shape;
    T = slotT(Pr);
    byBody.assign(Pr.nbodies, {});
    local.assign(9 * (size_t)n, 0.0);
    reg.assign(n, 0.0);
    scaling.assign(n, 1.0);
    for (int i = 0; i < n; ++i) {
      int bodies[2]; const double* H[2]; int nb;
      contactBodies(Pr, i, bodies, H, nb);
      for (int t = 0; t < nb; ++t) byBody[bodies[t]].push_back({i, t});
      double* L = &local[9 * (size_t)i];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          double a = 0.0;
          for (int t = 0; t < nb; ++t) {
            const double* Tt = &T[((size_t)i * 2 + t) * d * 3];
            for (int m = 0; m < d; ++m) a = std::fma(H[t][r * d + m], Tt[m * 3 + c], a);
          }
          L[3 * r + c] = a;
        }
      scaling[i] = dmax(1.0, ((L[0] + L[4]) + L[8]) / 3.0);
      if (autoRegularization > 0.) {
        reg[i] = dmax(0.0, autoRegularization - GaussSeidel::minEigenSymmetric3(L));
        L[0] += reg[i];
        L[4] += reg[i];
        L[8] += reg[i];
      }
    }
  }

  void computeMx(const double* x, double* Mx) const {
    const int d = P->ndof;
    for (int b = 0; b < P->nbodies; ++b)
      for (int m = 0; m < d; ++m) {
        double a = 0.0;
        for (const auto& it : byBody[b]) {
          const double* Tt = &T[((size_t)it.first * 2 + it.second) * d * 3];
          const double* xi = &x[3 * (size_t)it.first];
          a = std::fma(Tt[m * 3], xi[0], a);
          a = std::fma(Tt[m * 3 + 1], xi[1], a);
          a = std::fma(Tt[m * 3 + 2], xi[2], a);
        }
        Mx[(size_t)b * d + m] = a;
      }
  }
  void rowMul(int i, const double* Mx, double* v) const {
    const int d = P->ndof;
    int bodies[2]; const double* H[2]; int nb;
    contactBodies(*P, i, bodies, H, nb);
    for (int t = 0; t < nb; ++t)
      for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int m = 0; m < d; ++m) s = std::fma(H[t][r * d + m], Mx[(size_t)bodies[t] * d + m], s);
        v[r] = v[r] + s;
      }
  }
  void colMul(int i, const double* dx, double* Mx) const {
    const int d = P->ndof;
    int bodies[2]; const double* H[2]; int nb;
    contactBodies(*P, i, bodies, H, nb);
    for (int t = 0; t < nb; ++t) {
      const double* Tt = &T[((size_t)i * 2 + t) * d * 3];
      for (int m = 0; m < d; ++m) {
        const double s = std::fma(Tt[m * 3 + 2], dx[2], std::fma(Tt[m * 3 + 1], dx[1], Tt[m * 3] * dx[0]));
        Mx[(size_t)bodies[t] * d + m] = Mx[(size_t)bodies[t] * d + m] + s;
      }
    }
  }
  void velocity(const double* b, const double* Mx, double* y) const {  // y = b + H Mx
    std::copy(b, b + 3 * (size_t)P->ncontacts, y);
    for (int i = 0; i < P->ncontacts; ++i) rowMul(i, Mx, &y[3 * (size_t)i]);
  }

  double solve(const Law& law, const double* b, double* x, unsigned* itersOut = nullptr) const {
    const int N = P->ncontacts;
    const size_t n3 = 3 * (size_t)N;
    std::vector<double> Mx((size_t)P->nbodies * P->ndof), y(n3), x_best;
    double err_best = DBL_MAX;
    computeMx(x, Mx.data());
    velocity(b, Mx.data(), y.data());
    {
      const double err = eval(law, y.data(), x);
      if (err < err_best) {
        x_best.assign(x, x + n3);
        err_best = err;
      }
    }
    if (tryZeroAsWell) {
      std::vector<double> zero(n3, 0.0);
      const double err_zero = eval(law, b, zero.data());
      if (err_zero < err_best) {
        err_best = err_zero;
        x_best.assign(n3, 0.0);
        std::fill(x, x + n3, 0.0);
        std::fill(Mx.begin(), Mx.end(), 0.0);
      } else {
        std::copy(x_best.begin(), x_best.end(), x);
      }
    }
    trigger(0, err_best);
    std::vector<unsigned char> skip(N, 0);
    double ndxRef = 0;
    const double absSkipTol = dmin(skipTol, tol);
    const double absSkipIters = dmin((double)skipIters, (double)(unsigned)std::sqrt((double)N));
    unsigned GSIter;
    for (GSIter = 1; GSIter <= maxIters; ++GSIter) {
      for (int i = 0; i < N; ++i) {
        if (skip[i]) {
          --skip[i];
          continue;
        }
        double lx[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
        const double* L = &local[9 * (size_t)i];
        double lb[3];
        for (int r = 0; r < 3; ++r) lb[r] = b[3 * i + r] - dot3(&L[3 * r], lx);
        rowMul(i, Mx.data(), lb);
        double ldx[3] = {-lx[0], -lx[1], -lx[2]};
        const bool ok = lawSolveLocal(law.desaxce, law.strat, L, lb, lx, law.mu[i], scaling[i]);
        for (int k = 0; k < 3; ++k) ldx[k] = ldx[k] + lx[k];
        if (!ok) {
          ldx[0] *= .5; ldx[1] *= .5; ldx[2] *= .5;
        }
        for (int k = 0; k < 3; ++k) x[3 * i + k] = x[3 * i + k] + ldx[k];
        colMul(i, ldx, Mx.data());
        const double s2 = scaling[i] * scaling[i];
        const double nx2 = s2 * sq3(lx);
        const double ndx2 = s2 * sq3(ldx);
        if (ndx2 > ndxRef) ndxRef = ndx2;
        if (dmin(nx2, ndx2) < absSkipTol || ndx2 < skipTol * dmin(nx2, ndxRef))
          skip[i] = (unsigned char)absSkipIters;
      }
      if (0 == (GSIter % evalEvery)) {
        computeMx(x, Mx.data());
        velocity(b, Mx.data(), y.data());
        const double err = eval(law, y.data(), x);
        if (err < err_best) {
          x_best.assign(x, x + n3);
          err_best = err;
        }
        trigger(GSIter, err);
        if (err < tol) break;
        ndxRef /= evalEvery;
      }
    }
    if (GSIter > maxIters) std::copy(x_best.begin(), x_best.end(), x);
    if (itersOut) *itersOut = GSIter > maxIters ? maxIters : GSIter;
    return err_best;
  }
};

// ---------------------------------------------------------------------------------------------
// Cadoux fixed point (Interfaces/Cadoux.hpp:44-91): a Coulomb problem solved as a sequence of SOCQP problems
// whose right-hand side carries the De Saxce change of variable of the previous velocity:
//   s = W r + b, res = eval(Coulomb, s, r)
//   repeat: tol_inner = tolTighten * max(tol, min(res, 1)); s = COV(s) + b; solve SOC with rhs s from r;
//           s = W r + b; res = eval(Coulomb, s, r); stop when res < tol
// `m` is the inner minimizer (GaussSeidel or ProjectedGradient) set up on W; its tolerance is restored.
// W r + b is formed as the product with b as its initial value (spmv with init).
// ---------------------------------------------------------------------------------------------
template <class Minimizer>
double solveCadoux(Minimizer& m, const BSR& W, const double* b, const double* mu, int strat, double* r,
                   unsigned cadouxIterations, const Callback& callback, unsigned* itersOut = nullptr,
                   double tolTighten = 1.e-1) {
  const int n = W.n;
  const size_t n3 = 3 * (size_t)n;
  const Law coulomb{true, strat, mu};
  const Law soc{false, strat, mu};
  std::vector<double> s(n3);
  spmv(W, r, s.data(), b);
  double res = m.eval(coulomb, s.data(), r);
  if (callback) callback(0, res);
  const double tol = m.tol;
  unsigned it = 0;
  for (; it < cadouxIterations; ++it) {
    m.tol = tolTighten * dmax(tol, dmin(res, 1.));
    for (int i = 0; i < n; ++i) {
      double c[3];
      dualityCOV(true, mu[i], &s[3 * i], c);
      s[3 * i] = c[0];
      s[3 * i + 1] = c[1];
      s[3 * i + 2] = c[2];
    }
    for (size_t k = 0; k < n3; ++k) s[k] = s[k] + b[k];
    m.solve(soc, s.data(), r);
    spmv(W, r, s.data(), b);
    res = m.eval(coulomb, s.data(), r);
    if (callback) callback(it + 1, res);
    if (res < tol) {
      ++it;
      break;
    }
  }
  m.tol = tol;
  if (itersOut) *itersOut = it;
  return res;
}

// ---------------------------------------------------------------------------------------------
// Primal ADMM / AMA (ADMM.impl.hpp:54-127) with QuadraticProxOp (:29-38), as called by
// PrimalFrictionProblem::solveWith(ADMM&, lambda, v, r) (Interfaces/PrimalFrictionProblem.cpp:61-76):
// law SOCLaw<3, false> on 1/mu, operator H (contacts x bodies, 3 x ndof blocks), prox operator
// (M + lambda I)^-1 given as block-diagonal dense inverses `proxInv` (M^-1 when lambda == 0).
// The residual uses the error function of a non-square matrix: all scalings are 1.
// ---------------------------------------------------------------------------------------------
struct ADMMSolver {
  const Primal* P = nullptr;
  double tol = 1e-6;
  unsigned maxIters = 300;
  double stepSize = 1e-2;
  bool accelerated = true;
  bool useInfinityNorm = false;
  Callback callback;

  // ut = w + H v (contacts independent; OpenMP threads)
  void Hmul(const double* v, const double* w, double* ut) const {
    const int n = P->ncontacts, d = P->ndof;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      int bodies[2]; const double* H[2]; int nb;
      contactBodies(*P, i, bodies, H, nb);
      for (int r = 0; r < 3; ++r) {
        double a = w ? w[3 * i + r] : 0.0;
        for (int t = 0; t < nb; ++t)
          for (int m = 0; m < d; ++m) a = std::fma(H[t][r * d + m], v[(size_t)bodies[t] * d + m], a);
        ut[3 * i + r] = a;
      }
    }
  }
  // out = init + H^T r, accumulated body by body over its (contact, slot) pairs in increasing contact index,
  // then slot: each body gathers its own pairs (bodyPairs), so the bodies run on OpenMP threads with the order
  // of the sequential scatter over contacts.
  mutable std::vector<int> pairPtr, pairContact, pairSlot;
  void bodyPairs() const {
    if (!pairPtr.empty()) return;
    const int n = P->ncontacts, nbod = P->nbodies;
    pairPtr.assign(nbod + 1, 0);
    for (int i = 0; i < n; ++i) {
      int bodies[2]; const double* H[2]; int nb;
      contactBodies(*P, i, bodies, H, nb);
      for (int t = 0; t < nb; ++t) ++pairPtr[bodies[t] + 1];
    }
    for (int b = 0; b < nbod; ++b) pairPtr[b + 1] += pairPtr[b];
    pairContact.assign(pairPtr[nbod], 0);
    pairSlot.assign(pairPtr[nbod], 0);
    std::vector<int> cur(pairPtr.begin(), pairPtr.end() - 1);
    for (int i = 0; i < n; ++i) {
      int bodies[2]; const double* H[2]; int nb;
      contactBodies(*P, i, bodies, H, nb);
      for (int t = 0; t < nb; ++t) {
        const int p = cur[bodies[t]]++;
        pairContact[p] = i;
        pairSlot[p] = t;
      }
    }
  }
  void HTmul(const double* r, const double* init, double* out) const {
    const int d = P->ndof, nbod = P->nbodies;
    bodyPairs();
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nbod; ++b) {
      for (int q = 0; q < d; ++q) out[(size_t)b * d + q] = init ? init[(size_t)b * d + q] : 0.0;
      for (int p = pairPtr[b]; p < pairPtr[b + 1]; ++p) {
        const int i = pairContact[p];
        int bodies[2]; const double* H[2]; int nb;
        contactBodies(*P, i, bodies, H, nb);
        const double* Ht = H[pairSlot[p]];
        for (int q = 0; q < d; ++q) {
          double a = out[(size_t)b * d + q];
          for (int rr = 0; rr < 3; ++rr) a = std::fma(Ht[rr * d + q], r[3 * i + rr], a);
          out[(size_t)b * d + q] = a;
        }
      }
    }
  }
  // res = proxInv (rhs - f), block diagonal
  void prox(const std::vector<double>& proxInv, const double* rhs, const double* f, double* res) const {
    const int d = P->ndof;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < P->nbodies; ++k) {
      double t[16];
      for (int q = 0; q < d; ++q) t[q] = rhs[(size_t)k * d + q] - f[(size_t)k * d + q];
      for (int m = 0; m < d; ++m) {
        double a = 0.0;
        for (int q = 0; q < d; ++q) a = std::fma(proxInv[(size_t)k * d * d + m * d + q], t[q], a);
        res[(size_t)k * d + m] = a;
      }
    }
  }

  // Scalings of ConstrainedSolverBase::updateScalings for H (ConstrainedSolverBase.impl.hpp:84-118): 1, unless
  // H is square at the block level (3 n == total dofs and n == nbodies), where contact i takes
  // max(1, trace(H_(i, body i)) / 3) when it involves body i. trueDofs: the bodies' own dof counts (unpadded).
  std::vector<double> scalings;
  void setScalings(const std::vector<int>& trueDofs) {
    const int n = P->ncontacts, d = P->ndof;
    scalings.assign(n, 1.0);
    long long m = 0;
    for (int k : trueDofs) m += k;
    if (!(3LL * n == m && n == P->nbodies)) return;
    for (int i = 0; i < n; ++i) {
      int bodies[2]; const double* H[2]; int nb;
      contactBodies(*P, i, bodies, H, nb);
      for (int t = 0; t < nb; ++t)
        if (bodies[t] == i) {
          const int kk = std::min(3, trueDofs[i]);
          double tr = 0.0;
          for (int k = 0; k < kk; ++k) tr = tr + H[t][k * d + k];
          scalings[i] = dmax(1.0, tr / 3.0);
        }
    }
  }

  double solve(const double* invMu, const std::vector<double>& proxInv, double lambda, const double* f,
               const double* w, double* x, double* r, unsigned* itersOut = nullptr) const {
    const int n = P->ncontacts;
    const size_t n3 = 3 * (size_t)n, m = (size_t)P->nbodies * P->ndof;
    const double gamma = stepSize, inv_gamma = 1. / gamma;
    double res = -1;
    std::vector<double> ut(n3), prox_arg(m), z(n3), y(n3), y_prev(n3), zacc, z_prev, tmp(n3);
    Hmul(x, w, ut.data());
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n3; ++k) z[k] = ut[k] - inv_gamma * r[k];
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) projectCone(invMu[i], &z[3 * i]);
    #pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n3; ++k) y_prev[k] = -inv_gamma * r[k];
    zacc = z;
    z_prev = z;
    double theta_prev = 1.;
    double res_prev = -1;
    unsigned it;
    std::vector<double> ev(n);
    for (it = 0; it < maxIters; ++it) {
      if (lambda < kEps) {
        HTmul(r, nullptr, prox_arg.data());
      } else {
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n3; ++k) tmp[k] = std::fma(gamma, zacc[k] - ut[k], r[k]);
        // prox_arg = x / lambda ... multiply<true>(ut, prox_arg, 1, 1/lambda): prox_arg = (1/lambda) x + H^T ut
        std::vector<double> sx(m);
        const double il = 1. / lambda;
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < m; ++k) sx[k] = il * x[k];
        HTmul(tmp.data(), sx.data(), prox_arg.data());
      }
      prox(proxInv, prox_arg.data(), f, x);
      Hmul(x, w, ut.data());
      // eval(law, r, ut): per contact FB(1/mu, ut_i (scaling 1), r_i) with SOC law
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) {
        const double sc = scalings.empty() ? 1.0 : scalings[i];
        const double lx[3] = {ut[3 * i] * sc, ut[3 * i + 1] * sc, ut[3 * i + 2] * sc};
        ev[i] = lawEval(false, invMu[i], lx, &r[3 * i]);
      }
      double e = useInfinityNorm ? maxOf(ev.data(), n) : canonicalSum(ev.data(), n) / (double)(1 + n);
      std::vector<double> gap(n);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) {
        const double d3[3] = {ut[3 * i] - z[3 * i], ut[3 * i + 1] - z[3 * i + 1], ut[3 * i + 2] - z[3 * i + 2]};
        gap[i] = useInfinityNorm ? dmax(dmax(std::fabs(d3[0]), std::fabs(d3[1])), std::fabs(d3[2])) : sq3(d3);
      }
      res = e + (useInfinityNorm ? maxOf(gap.data(), n) : canonicalSum(gap.data(), n) / (double)(1 + n3));
      if (callback) callback(it, res);
      if (res < tol) break;
      #pragma omp parallel for schedule(static)
      for (size_t k = 0; k < n3; ++k) z[k] = ut[k] - inv_gamma * r[k];
      #pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) projectCone(invMu[i], &z[3 * i]);
      if (accelerated && res < res_prev) {
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n3; ++k) y[k] = (ut[k] - z[k]) - inv_gamma * r[k];
        const double beta = nesterovInertia(theta_prev, 0.);
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n3; ++k) r[k] = -gamma * std::fma(beta, y[k] - y_prev[k], y[k]);
        y_prev = y;
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n3; ++k) zacc[k] = std::fma(beta, z[k] - z_prev[k], z[k]);
        z_prev = z;
      } else {
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n3; ++k) r[k] = std::fma(gamma, z[k] - ut[k], r[k]);
        zacc = z;
        z_prev = z;
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n3; ++k) y_prev[k] = -inv_gamma * r[k];
        theta_prev = 1;
      }
      res_prev = res;
    }
    if (itersOut) *itersOut = it;
    return res;
  }
};

// ---------------------------------------------------------------------------------------------
// DualAMA (Core/BlockSolvers/ADMM.hpp:170-236, ADMM.impl.hpp:128-303) as
// PrimalFrictionProblem::solveWith(DualAMAType&, v, r, staticProblem) (PrimalFrictionProblem.cpp:78-99) calls
// it: A = M, B = 0, trivial preconditioner, law SOCLaw<3> on mu (with the De Saxce change of variable unless
// static). Per iteration: x = f + M v, z = H^T r - x, u = w + H v, res = eval(u, r) + |z|^2 / (1 + m) (max
// norms with the infinity norm), g = u + COV(u) + gamma H z, then r = P(r - lambda g) with the line search on
// |H^T r - f - M y|^2 (y = v + gamma z over-relaxed by beta), z = H^T r - x, y = v + gamma z,
// v = y + beta (y - y_prev). The best (r, v) by residual is returned.
// Orders: M v and H z as fma chains from 0, then added (x = f + Mv, gap = (H^T r - f) - My, g = fma(gamma, Hz, g));
// H v and H^T r as the ADMM restatement's products; dof norms |z|^2 and |gap|^2 as each body's dofs summed
// left to right, then the canonical sum over bodies; over-relaxation y + beta (y - y_prev) unfused.
// ---------------------------------------------------------------------------------------------
struct DualAMASolver {
  const Primal* P = nullptr;
  double tol = 1e-6;
  unsigned maxIters = 300;
  double fpStepSize = 1.e-1;    // gamma
  double projStepSize = 1.e-1;  // lambda
  unsigned lsIters = 6;
  double lsOptimisticFactor = 1.25;
  double lsPessimisticFactor = .5;
  bool accelerated = true;
  bool useInfinityNorm = false;
  Callback callback;
  std::vector<double> scalings;  // as ADMMSolver::setScalings
  long long mTrue = -1;          // the bodies' own dof count (the gap term's 1 + m); -1: nbodies x ndof

  void Mmul(const std::vector<double>& M, const double* v, double* out) const {
    const int d = P->ndof;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < P->nbodies; ++k)
      for (int a = 0; a < d; ++a) {
        double acc = 0.0;
        for (int q = 0; q < d; ++q) acc = std::fma(M[(size_t)k * d * d + a * d + q], v[(size_t)k * d + q], acc);
        out[(size_t)k * d + a] = acc;
      }
  }

  double solve(const double* mu, bool desaxce, const std::vector<double>& M, const double* f, const double* w,
               double* v, double* r, unsigned* itersOut = nullptr) const {
    ADMMSolver h;
    h.P = P;
    const int n = P->ncontacts;
    const size_t n3 = 3 * (size_t)n, m = (size_t)P->nbodies * P->ndof;
    double lambda = projStepSize;
    const double gamma = fpStepSize;
    double res = -1, min_res = -1;
    std::vector<double> r_best(r, r + n3), v_best(v, v + m);
    std::vector<double> z(m), x(m), ut(n3), gap(m), HrBp(m), g(n3), Mv(m), y(m), y_prev(v, v + m), rs(n3);
    const int nb = P->nbodies, d = P->ndof;
    std::vector<double> tmp(m), zz(nb), ev(n), Hz(n3);
    double theta_prev = 1., res_prev = -1;
    // dof norms: each body's dofs left to right, then the canonical sum over bodies (or the maximum)
    auto dofnorm = [&](const std::vector<double>& a) {
      #pragma omp parallel for schedule(static)
      for (int b = 0; b < nb; ++b) {
        double p = 0.0;
        for (int k = 0; k < d; ++k) {
          const double e = a[(size_t)b * d + k];
          p = useInfinityNorm ? dmax(std::fabs(e), p) : p + e * e;
        }
        zz[b] = p;
      }
      return useInfinityNorm ? maxOf(zz.data(), nb) : canonicalSum(zz.data(), nb);
    };
    auto sqnorm = [&](const std::vector<double>& a) {
      #pragma omp parallel for schedule(static)
      for (int b = 0; b < nb; ++b) {
        double p = 0.0;
        for (int k = 0; k < d; ++k) p = p + a[(size_t)b * d + k] * a[(size_t)b * d + k];
        zz[b] = p;
      }
      return canonicalSum(zz.data(), nb);
    };
    h.HTmul(r, nullptr, HrBp.data());
    unsigned it;
    for (it = 0; it < maxIters; ++it) {
      Mmul(M, v, Mv.data());
      #pragma omp parallel for schedule(static)
      for (size_t k = 0; k < m; ++k) x[k] = f[k] + Mv[k];
      #pragma omp parallel for schedule(static)
      for (size_t k = 0; k < m; ++k) z[k] = HrBp[k] - x[k];
      h.Hmul(v, w, ut.data());
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) {
        const double sc = scalings.empty() ? 1.0 : scalings[i];
        const double lx[3] = {r[3 * i] * sc, r[3 * i + 1] * sc, r[3 * i + 2] * sc};
        ev[i] = lawEval(desaxce, mu[i], lx, &ut[3 * i]);
      }
      res = useInfinityNorm ? maxOf(ev.data(), n) : canonicalSum(ev.data(), n) / (double)(1 + n);
      const double zn = dofnorm(z);
      res += useInfinityNorm ? zn : zn / (double)(1 + (mTrue >= 0 ? (size_t)mTrue : m));
      if (callback) callback(it, res);
      if (res < min_res || it == 0) {
        std::copy(r, r + n3, r_best.begin());
        std::copy(v, v + m, v_best.begin());
        min_res = res;
        if (res < tol) break;
      } else if (res > 1.e50) {
        break;
      }
      double beta = 0;
      if (accelerated && res < res_prev) beta = nesterovInertia(theta_prev, 0.);
      else theta_prev = 1;
      // g = ut + COV(ut) + gamma H z
      h.Hmul(z.data(), nullptr, Hz.data());
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) {
        double s[3];
        dualityCOV(desaxce, mu[i], &ut[3 * i], s);
        for (int k = 0; k < 3; ++k) g[3 * i + k] = std::fma(gamma, Hz[3 * i + k], ut[3 * i + k] + s[k]);
      }
      if (lsIters == 0) {
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n3; ++k) r[k] = r[k] - lambda * g[k];
        #pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) projectCone(mu[i], &r[3 * i]);
        h.HTmul(r, nullptr, HrBp.data());
      } else {
        #pragma omp parallel for schedule(static)
        for (size_t k = 0; k < m; ++k) gap[k] = HrBp[k] - x[k];
        const double h0 = sqnorm(gap);  // the squared norm, whatever the residual's norm
        lambda *= lsOptimisticFactor;
        for (unsigned ls = 0; ls < lsIters; ++ls) {
          #pragma omp parallel for schedule(static)
          for (size_t k = 0; k < n3; ++k) rs[k] = r[k] - lambda * g[k];
#pragma omp parallel for schedule(static)
          for (int i = 0; i < n; ++i) projectCone(mu[i], &rs[3 * i]);
          h.HTmul(rs.data(), nullptr, HrBp.data());
          #pragma omp parallel for schedule(static)
          for (size_t k = 0; k < m; ++k) {
            const double zk = HrBp[k] - x[k];
            const double yk = v[k] + gamma * zk;
            y[k] = yk + beta * (yk - y_prev[k]);
          }
          Mmul(M, y.data(), tmp.data());
          #pragma omp parallel for schedule(static)
          for (size_t k = 0; k < m; ++k) gap[k] = (HrBp[k] - f[k]) - tmp[k];
          const double hh = sqnorm(gap);
          if (hh < h0) break;
          lambda *= lsPessimisticFactor;
        }
        std::copy(rs.begin(), rs.end(), r);
      }
      #pragma omp parallel for schedule(static)
      for (size_t k = 0; k < m; ++k) {
        z[k] = HrBp[k] - x[k];
        const double yk = v[k] + gamma * z[k];
        v[k] = yk + beta * (yk - y_prev[k]);
        y_prev[k] = yk;
      }
      res_prev = res;
    }
    std::copy(r_best.begin(), r_best.end(), r);
    std::copy(v_best.begin(), v_best.end(), v);
    if (itersOut) *itersOut = it;
    return min_res;
  }
};

}  // namespace oracle
