// ORACLE — test infrastructure only. Nothing in the shipped library includes, links or calls this code;
// only tests/, the smoke check and the CPU-baseline leg of bench.py use it, as the checker.
//
// CPU restatement of So-bogus's per-contact mathematics (3D second-order-cone / Coulomb law):
// Fischer-Burmeister function and Jacobian, non-smooth Newton, real roots of the local quartic,
// full-pivoting LU, the analytic local solvers and the local solver strategies.
//
// Evaluation order. The reference evaluates these formulas through Eigen expression templates, whose
// rounding order depends on Eigen's version and vectorisation; it cannot be reproduced bit for bit.
// This restatement fixes one order and the GPU kernels follow exactly the same one:
//   * dot3(a,b) = fma(a2,b2, fma(a1,b1, a0*b0)); squared norms are dot3(a,a);
//   * 3x3 matrix-vector rows are computed with the same chain;
//   * a value divided by the same denominator more than once is multiplied by that denominator's
//     reciprocal (one correctly rounded division);
//   * no other fused operations: every translation unit is built with -ffp-contract=off.
// Division and sqrt are IEEE correctly rounded on both the host and the GPU, so equal inputs give
// bit-identical outputs.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

// DBL_EPSILON, the reference's NumTraits<double>::epsilon() (Core/Utils/NumTraits.hpp:19-24)
constexpr double kEps = 2.220446049250313080847e-16;
// pow(eps, 0.75) == 2^-39 exactly: SOCLaw's local tolerance (Extra/SOC/SOCLaw.impl.hpp:33-35)
constexpr double kLocalTol = 1.8189894035458565e-12;

inline bool isZero(double s) { return std::fabs(s) < kEps; }  // NumTraits::isZero
inline double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max semantics
inline double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min semantics

inline double dot3(const double* a, const double* b) { return std::fma(a[2], b[2], std::fma(a[1], b[1], a[0] * b[0])); }
inline double sq3(const double* a) { return dot3(a, a); }
inline double dot2(double a0, double a1, double b0, double b1) { return std::fma(a1, b1, a0 * b0); }
inline double norm2(double a0, double a1) { return std::sqrt(dot2(a0, a1, a0, a1)); }

// y = A x, A row-major 3x3
inline void matvec3(const double* A, const double* x, double* y) {
  for (int r = 0; r < 3; ++r) y[r] = std::fma(A[3 * r + 2], x[2], std::fma(A[3 * r + 1], x[1], A[3 * r] * x[0]));
}

// ---------------------------------------------------------------------------------------------
// Full-pivoting LU (Gaussian elimination with complete pivoting), the decomposition the reference
// uses for every small dense solve (Eigen::FullPivLU through Core/Eigen/EigenLinearSolvers.hpp:21-63).
// P A Q = L U. Pivot: largest |a_ij| of the trailing submatrix, first in row-major order on ties.
// Elimination stops at an exactly zero pivot. solve() treats pivots with
// |p| <= eps * n * |p_0| as zero and sets the matching unknowns to 0.
// ---------------------------------------------------------------------------------------------
struct FullPivLU {
  int n = 0;
  int nonzero = 0;  // pivots actually eliminated
  int rank = 0;
  double lu[36];
  double inv_piv[6];
  int rowt[6], colt[6];

  void compute(const double* A, int n_) {
    n = n_;
    std::memcpy(lu, A, sizeof(double) * n * n);
    nonzero = n;
    for (int k = 0; k < n; ++k) {
      int pi = k, pj = k;
      double best = -1.0;
      for (int i = k; i < n; ++i)
        for (int j = k; j < n; ++j) {
          const double a = std::fabs(lu[i * n + j]);
          if (a > best) { best = a; pi = i; pj = j; }
        }
      rowt[k] = pi;
      colt[k] = pj;
      if (best == 0.0) {
        nonzero = k;
        for (int kk = k; kk < n; ++kk) { rowt[kk] = kk; colt[kk] = kk; }
        break;
      }
      if (pi != k)
        for (int j = 0; j < n; ++j) { const double t = lu[k * n + j]; lu[k * n + j] = lu[pi * n + j]; lu[pi * n + j] = t; }
      if (pj != k)
        for (int i = 0; i < n; ++i) { const double t = lu[i * n + k]; lu[i * n + k] = lu[i * n + pj]; lu[i * n + pj] = t; }
      const double inv = 1.0 / lu[k * n + k];
      inv_piv[k] = inv;
      for (int i = k + 1; i < n; ++i) lu[i * n + k] *= inv;
      for (int i = k + 1; i < n; ++i) {
        const double l = lu[i * n + k];
        for (int j = k + 1; j < n; ++j) lu[i * n + j] = std::fma(-l, lu[k * n + j], lu[i * n + j]);
      }
    }
    rank = 0;
    if (nonzero > 0) {
      const double thr = kEps * (double)n * std::fabs(lu[0]);
      for (int k = 0; k < nonzero; ++k)
        if (std::fabs(lu[k * n + k]) > thr) ++rank;
    }
  }

  // x = A^-1 b (least-norm-free basic solution when rank deficient); b and x may alias
  void solve(const double* b, double* x) const {
    double c[6];
    for (int i = 0; i < n; ++i) c[i] = b[i];
    for (int k = 0; k < n; ++k) { const int p = rowt[k]; if (p != k) { const double t = c[k]; c[k] = c[p]; c[p] = t; } }
    for (int i = 1; i < n; ++i)
      for (int j = 0; j < i; ++j) c[i] = std::fma(-lu[i * n + j], c[j], c[i]);
    for (int i = rank - 1; i >= 0; --i) {
      for (int j = i + 1; j < rank; ++j) c[i] = std::fma(-lu[i * n + j], c[j], c[i]);
      c[i] = c[i] * inv_piv[i];
    }
    for (int i = rank; i < n; ++i) c[i] = 0.0;
    for (int k = n - 1; k >= 0; --k) { const int p = colt[k]; if (p != k) { const double t = c[k]; c[k] = c[p]; c[p] = t; } }
    for (int i = 0; i < n; ++i) x[i] = c[i];
  }
};

// ---------------------------------------------------------------------------------------------
// Real roots of a polynomial as the real eigenvalues of its companion matrix
// (Core/Utils/Polynomial.impl.hpp:34-75): last column = -coefficients, unit sub-diagonal.
// The eigenvalues are found with the Francis implicit double-shift QR iteration on the upper
// Hessenberg companion matrix (the published EISPACK "hqr" method: deflation on negligible
// sub-diagonal entries, exceptional shifts after 10 and 20 stalled sweeps). An eigenvalue is real
// when its imaginary part is NumTraits::isZero, as in the reference.
// ---------------------------------------------------------------------------------------------
enum RootsFilter { AllRoots = 0, StrictlyNegativeRoots = 1, StrictlyPositiveRoots = 2 };  // Polynomial.hpp

inline int hessenbergEigenvalues(double* a, int n, double* wr, double* wi) {
  // a: n x n row-major upper Hessenberg, destroyed. Returns 0 on success, -1 if not converged.
  auto A = [&](int i, int j) -> double& { return a[i * n + j]; };
  double anorm = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = (i > 0 ? i - 1 : 0); j < n; ++j) anorm += std::fabs(A(i, j));
  int nn = n - 1;
  double t = 0.0;
  int total = 0;
  while (nn >= 0) {
    int its = 0, l;
    for (;;) {
      for (l = nn; l >= 1; --l) {
        double s = std::fabs(A(l - 1, l - 1)) + std::fabs(A(l, l));
        if (s == 0.0) s = anorm;
        if (std::fabs(A(l, l - 1)) + s == s) { A(l, l - 1) = 0.0; break; }
      }
      double x = A(nn, nn);
      if (l == nn) {  // one real root
        wr[nn] = x + t;
        wi[nn] = 0.0;
        --nn;
        break;
      }
      double y = A(nn - 1, nn - 1);
      double w = A(nn, nn - 1) * A(nn - 1, nn);
      if (l == nn - 1) {  // a 2x2 block
        const double p = 0.5 * (y - x);
        const double q = p * p + w;
        double z = std::sqrt(std::fabs(q));
        x += t;
        if (q >= 0.0) {
          z = p + (p >= 0.0 ? std::fabs(z) : -std::fabs(z));
          wr[nn - 1] = wr[nn] = x + z;
          if (z != 0.0) wr[nn] = x - w / z;
          wi[nn - 1] = wi[nn] = 0.0;
        } else {
          wr[nn - 1] = wr[nn] = x + p;
          wi[nn - 1] = -z;
          wi[nn] = z;
        }
        nn -= 2;
        break;
      }
      if (its == 30 || total >= 40 * n) return -1;
      if (its == 10 || its == 20) {  // exceptional shift
        t += x;
        for (int i = 0; i <= nn; ++i) A(i, i) -= x;
        const double s = std::fabs(A(nn, nn - 1)) + std::fabs(A(nn - 1, nn - 2));
        x = y = 0.75 * s;
        w = -0.4375 * s * s;
      }
      ++its;
      ++total;
      int m;
      double p = 0, q = 0, r = 0, z;
      for (m = nn - 2; m >= l; --m) {
        z = A(m, m);
        const double rr = x - z;
        const double ss = y - z;
        p = (rr * ss - w) / A(m + 1, m) + A(m, m + 1);
        q = A(m + 1, m + 1) - z - rr - ss;
        r = A(m + 2, m + 1);
        const double sc = std::fabs(p) + std::fabs(q) + std::fabs(r);
        p /= sc;
        q /= sc;
        r /= sc;
        if (m == l) break;
        const double u = std::fabs(A(m, m - 1)) * (std::fabs(q) + std::fabs(r));
        const double v = std::fabs(p) * (std::fabs(A(m - 1, m - 1)) + std::fabs(z) + std::fabs(A(m + 1, m + 1)));
        if (u + v == v) break;
      }
      for (int i = m + 2; i <= nn; ++i) {
        A(i, i - 2) = 0.0;
        if (i != m + 2) A(i, i - 3) = 0.0;
      }
      for (int k = m; k <= nn - 1; ++k) {
        if (k != m) {
          p = A(k, k - 1);
          q = A(k + 1, k - 1);
          r = 0.0;
          if (k != nn - 1) r = A(k + 2, k - 1);
          x = std::fabs(p) + std::fabs(q) + std::fabs(r);
          if (x != 0.0) { p /= x; q /= x; r /= x; }
        }
        const double nrm = std::sqrt(p * p + q * q + r * r);
        const double s = (p >= 0.0 ? nrm : -nrm);
        if (s != 0.0) {
          if (k == m) {
            if (l != m) A(k, k - 1) = -A(k, k - 1);
          } else {
            A(k, k - 1) = -s * x;
          }
          p += s;
          x = p / s;
          y = q / s;
          z = r / s;
          q /= p;
          r /= p;
          for (int j = k; j <= nn; ++j) {  // row transformation
            p = A(k, j) + q * A(k + 1, j);
            if (k != nn - 1) {
              p += r * A(k + 2, j);
              A(k + 2, j) -= p * z;
            }
            A(k + 1, j) -= p * y;
            A(k, j) -= p * x;
          }
          const int mmin = nn < k + 3 ? nn : k + 3;
          for (int i = l; i <= mmin; ++i) {  // column transformation
            p = x * A(i, k) + y * A(i, k + 1);
            if (k != nn - 1) {
              p += z * A(i, k + 2);
              A(i, k + 2) -= p * r;
            }
            A(i, k + 1) -= p * q;
            A(i, k) -= p;
          }
        }
      }
    }
  }
  return 0;
}

// Monic polynomial x^dim + c[dim-1] x^(dim-1) + ... + c[0] (RootsFinder::getRealRoots).
inline int realRootsMonic(const double* c, int dim, double* roots, RootsFilter filter) {
  double a[16];
  for (int i = 0; i < dim * dim; ++i) a[i] = 0.0;
  for (int i = 1; i < dim; ++i) a[i * dim + (i - 1)] = 1.0;
  for (int i = 0; i < dim; ++i) a[i * dim + (dim - 1)] = -c[i];
  double wr[4], wi[4];
  if (hessenbergEigenvalues(a, dim, wr, wi) != 0) {
    // not converged: report no root (the reference ignores Eigen's NoConvergence flag; its values are then
    // unspecified)
    return 0;
  }
  int count = 0;
  for (int i = 0; i < dim; ++i) {
    if (isZero(wi[i])) {
      const bool discard = (filter == StrictlyPositiveRoots && wr[i] <= 0) || (filter == StrictlyNegativeRoots && wr[i] >= 0);
      if (!discard) roots[count++] = wr[i];
    }
  }
  return count;
}

// Arbitrary leading coefficient c[dim] (PossiblyDegenerateRootsFinder, Polynomial.impl.hpp:86-109). c modified.
inline int realRootsDegenerate(double* c, int dim, double* roots, RootsFilter filter) {
  while (dim > 0 && isZero(c[dim])) --dim;
  if (dim == 0) {
    roots[0] = 0.0;
    return (filter == AllRoots && isZero(c[0])) ? 1 : 0;
  }
  const double inv = 1.0 / c[dim];
  for (int k = 0; k < dim; ++k) c[k] *= inv;
  return realRootsMonic(c, dim, roots, filter);
}

// ---------------------------------------------------------------------------------------------
// Fischer-Burmeister function on the second-order cone (Extra/SOC/FischerBurmeister.impl.hpp)
// ---------------------------------------------------------------------------------------------

// FBBaseFunction::compute<JacobianAsWell>(x, y, fb, dFb_dx, dFb_dy) on the canonical cone (:69-140)
template <bool Jac>
inline void fbCanonical(const double* x, const double* y, double* fb, double* dx, double* dy) {
  double z2[3];
  z2[0] = sq3(x) + sq3(y);
  z2[1] = std::fma(x[0], x[1], y[0] * y[1]);
  z2[2] = std::fma(x[0], x[2], y[0] * y[2]);
  const double nz2t = norm2(z2[1], z2[2]);
  double om1[3], om2[3];
  om1[0] = om2[0] = 0.5;
  if (isZero(nz2t)) {
    om1[1] = -0.5; om1[2] = 0.0;
    om2[1] = 0.5;  om2[2] = 0.0;
  } else {
    const double inv = 1.0 / nz2t;
    const double t1 = z2[1] * inv, t2 = z2[2] * inv;
    om1[1] = -0.5 * t1; om1[2] = -0.5 * t2;
    om2[1] = 0.5 * t1;  om2[2] = 0.5 * t2;
  }
  const double l1 = z2[0] - 2.0 * nz2t;
  const double rl1 = std::sqrt(l1 > 0.0 ? l1 : 0.0);
  const double rl2 = std::sqrt(z2[0] + 2.0 * nz2t);
  double z[3];
  for (int k = 0; k < 3; ++k) z[k] = std::fma(rl2, om2[k], rl1 * om1[k]);
  for (int k = 0; k < 3; ++k) fb[k] = (x[k] + y[k]) - z[k];
  if (!Jac) return;
  if (isZero(rl2)) {
    for (int k = 0; k < 9; ++k) dx[k] = dy[k] = 0.0;
    return;
  }
  if (isZero(rl1)) {
    const double izn = 1.0 / dot2(x[0], y[0], x[0], y[0]);
    const double cx = 1.0 - x[0] * izn, cy = 1.0 - y[0] * izn;
    for (int k = 0; k < 9; ++k) dx[k] = dy[k] = 0.0;
    dx[0] = dx[4] = dx[8] = cx;
    dy[0] = dy[4] = dy[8] = cy;
    return;
  }
  const double det = rl1 * rl2;
  const double inv_det = 1.0 / det;
  const double inv_z0 = 1.0 / z[0];
  double iL[9];
  iL[0] = z[0] * inv_det;
  iL[1] = -z[1] * inv_det;
  iL[2] = -z[2] * inv_det;
  iL[3] = iL[1];
  iL[6] = iL[2];
  iL[4] = (std::fma(z[1], z[1], det) * inv_z0) * inv_det;
  iL[5] = ((z[1] * z[2]) * inv_z0) * inv_det;
  iL[7] = iL[5];
  iL[8] = (std::fma(z[2], z[2], det) * inv_z0) * inv_det;
  const double* vs[2] = {x, y};
  double* outs[2] = {dx, dy};
  for (int w = 0; w < 2; ++w) {
    const double* v = vs[w];
    const double L[9] = {v[0], v[1], v[2], v[1], v[0], 0.0, v[2], 0.0, v[0]};
    double* o = outs[w];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        const double p = std::fma(iL[3 * r + 2], L[6 + c], std::fma(iL[3 * r + 1], L[3 + c], iL[3 * r] * L[c]));
        o[3 * r + c] = (r == c ? 1.0 : 0.0) - p;
      }
  }
}

// FBBaseFunction::compute(mu, x, y, fb) (:29-41)
inline void fbMu(double mu, const double* x, const double* y, double* fb) {
  if (isZero(mu)) {
    fb[0] = (x[0] + y[0]) - std::sqrt(dot2(x[0], y[0], x[0], y[0]));
    fb[1] = x[1];
    fb[2] = x[2];
  } else {
    const double xh[3] = {mu * x[0], x[1], x[2]};
    const double yh[3] = {y[0], mu * y[1], mu * y[2]};
    fbCanonical<false>(xh, yh, fb, nullptr, nullptr);
  }
}

// FBBaseFunction::computeJacobian(mu, x, y, fb, dFb_dx, dFb_dy) (:43-67)
inline void fbMuJacobian(double mu, const double* x, const double* y, double* fb, double* dx, double* dy) {
  if (isZero(mu)) {
    const double z = std::sqrt(dot2(x[0], y[0], x[0], y[0]));
    fb[0] = (x[0] + y[0]) - z;
    fb[1] = x[1];
    fb[2] = x[2];
    for (int k = 0; k < 9; ++k) { dx[k] = 0.0; dy[k] = 0.0; }
    dx[0] = dx[4] = dx[8] = 1.0;
    if (!isZero(z)) {
      const double iz = 1.0 / z;
      dx[0] = 1.0 - x[0] * iz;
      dy[0] = 1.0 - y[0] * iz;
    }
  } else {
    const double xh[3] = {mu * x[0], x[1], x[2]};
    const double yh[3] = {y[0], mu * y[1], mu * y[2]};
    fbCanonical<true>(xh, yh, fb, dx, dy);
    for (int r = 0; r < 3; ++r) {
      dx[3 * r] *= mu;
      dy[3 * r + 1] *= mu;
      dy[3 * r + 2] *= mu;
    }
  }
}

// FischerBurmeister<3, double, DeSaxceCOV>::compute(mu, x, y, fb) (:142-151)
inline void fbLaw(bool desaxce, double mu, const double* x, const double* y, double* fb) {
  if (desaxce) {
    const double yt[3] = {std::fma(mu, norm2(y[1], y[2]), y[0]), y[1], y[2]};
    fbMu(mu, x, yt, fb);
  } else {
    fbMu(mu, x, y, fb);
  }
}

// SOCLaw::eval (Extra/SOC/SOCLaw.hpp:55-64): |fb(mu, x, y)|^2, or |y|^2 for mu < 0
inline double lawEval(bool desaxce, double mu, const double* x, const double* y) {
  if (mu < 0) return sq3(y);
  double fb[3];
  fbLaw(desaxce, mu, x, y, fb);
  return sq3(fb);
}

// SOCLaw::projectOnConstraint (Extra/SOC/SOCLaw.impl.hpp:46-72)
inline void projectCone(double mu, double* x) {
  const double nxt = norm2(x[1], x[2]);
  const double xn = x[0];
  if (mu < 0) { x[0] = x[1] = x[2] = 0.0; return; }
  if (nxt <= mu * xn) return;
  if (mu * nxt <= -xn) { x[0] = x[1] = x[2] = 0.0; return; }
  const double den2 = std::fma(mu, mu, 1.0);
  const double proj = std::fma(mu, nxt, xn) / den2;
  x[0] = proj;
  const double f = (proj * mu) / nxt;
  x[1] *= f;
  x[2] *= f;
}

// SOCLaw::dualityCOV (Extra/SOC/SOCLaw.hpp:92-99)
inline void dualityCOV(bool desaxce, double mu, const double* y, double* s) {
  if (desaxce) {
    s[0] = mu * norm2(y[1], y[2]);
  } else {
    s[0] = 0.0;
  }
  s[1] = s[2] = 0.0;
}

// ---------------------------------------------------------------------------------------------
// Local problem function x -> FB(mu, scaling x, A x + b) (FischerBurmeister.impl.hpp:153-187)
// ---------------------------------------------------------------------------------------------
struct LocalFB {
  bool desaxce;
  double mu, scaling;
  const double* A;  // 3x3 row-major
  const double* b;

  void y_of(const double* x, double* y) const {
    double ax[3];
    matvec3(A, x, ax);
    for (int k = 0; k < 3; ++k) y[k] = ax[k] + b[k];
  }
  void compute(const double* x, double* fb) const {
    double y[3];
    y_of(x, y);
    const double xs[3] = {scaling * x[0], scaling * x[1], scaling * x[2]};
    fbLaw(desaxce, mu, xs, y, fb);
  }
  void computeJacobian(const double* x, double* fb, double* dFdx) const {
    const double xs[3] = {scaling * x[0], scaling * x[1], scaling * x[2]};
    double y[3];
    y_of(x, y);
    double s = 0.0;
    if (desaxce) {
      s = norm2(y[1], y[2]);
      y[0] = std::fma(mu, s, y[0]);
    }
    double dy[9];
    fbMuJacobian(mu, xs, y, fb, dFdx, dy);
    if (desaxce && !isZero(s)) {
      const double c = mu / s;
      for (int r = 0; r < 3; ++r) {
        const double t = dy[3 * r] * c;
        dy[3 * r + 1] = std::fma(t, y[1], dy[3 * r + 1]);
        dy[3 * r + 2] = std::fma(t, y[2], dy[3 * r + 2]);
      }
    }
    for (int k = 0; k < 9; ++k) dFdx[k] *= scaling;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        const double p = std::fma(dy[3 * r + 2], A[6 + c], std::fma(dy[3 * r + 1], A[3 + c], dy[3 * r] * A[c]));
        dFdx[3 * r + c] = dFdx[3 * r + c] + p;
      }
  }
};

// NonSmoothNewton::solve (Core/Utils/NonSmoothNewton.impl.hpp:23-79), maxIters 20 (NonSmoothNewton.hpp:31).
// Keeps the reference's descent test on dPhi_dx = dF_dx^T x (:67).
inline double newtonSolve(const LocalFB& f, double tol, double* x, int maxIters = 20) {
  const double sigma2 = 1.e-4, alpha = 0.5;
  double F[3];
  f.compute(x, F);
  const double Phi_init = 0.5 * sq3(F);
  if (Phi_init < tol) return Phi_init;
  double x_best[3] = {0.0, 0.0, 0.0};
  f.compute(x_best, F);
  const double Phi_zero = 0.5 * sq3(F);
  double Phi_best;
  if (Phi_zero < Phi_init) {
    Phi_best = Phi_zero;
    x[0] = x[1] = x[2] = 0.0;
  } else {
    Phi_best = Phi_init;
    x_best[0] = x[0]; x_best[1] = x[1]; x_best[2] = x[2];
  }
  if (Phi_zero < tol) return Phi_zero;
  double dF[9];
  FullPivLU lu;
  for (int iter = 0; iter < maxIters; ++iter) {
    f.computeJacobian(x, F, dF);
    const double Phi = 0.5 * sq3(F);
    if (Phi < tol) return Phi;
    if (Phi < Phi_best) {
      Phi_best = Phi;
      x_best[0] = x[0]; x_best[1] = x[1]; x_best[2] = x[2];
    }
    double dPhi[3];
    for (int k = 0; k < 3; ++k) dPhi[k] = std::fma(dF[6 + k], x[2], std::fma(dF[3 + k], x[1], dF[k] * x[0]));
    lu.compute(dF, 3);
    const double mF[3] = {-F[0], -F[1], -F[2]};
    double dx[3];
    lu.solve(mF, dx);
    const double proj = dot3(dx, dPhi);
    if (proj > 0 || proj * proj < (sigma2 * sq3(dx)) * sq3(dPhi)) {
      dx[0] *= alpha; dx[1] *= alpha; dx[2] *= alpha;
    }
    x[0] += dx[0]; x[1] += dx[1]; x[2] += dx[2];
  }
  x[0] = x_best[0]; x[1] = x_best[1]; x[2] = x_best[2];
  return Phi_best;
}

// AnalyticLocalSOCSolver<3, double, true>::solveOrthogonality (Extra/SOC/LocalSOCSolver.impl.hpp:47-103)
inline bool analyticCoulomb(const double* W, const double* b, double* r, double mu) {
  const double wN = W[0];
  if (wN < kEps) return false;
  const double wT0 = W[3], wT1 = W[6];
  const double bN = b[0];
  const double inv_wN = 1.0 / wN;
  const double wTwN0 = wT0 * inv_wN, wTwN1 = wT1 * inv_wN;
  const double Wb00 = std::fma(-wTwN0, wT0, W[4]);
  const double Wb01 = std::fma(-wTwN0, wT1, W[5]);
  const double Wb10 = std::fma(-wTwN1, wT0, W[7]);
  const double Wb11 = std::fma(-wTwN1, wT1, W[8]);
  const double inv_bN = 1.0 / bN;
  const double bb0 = b[1] * inv_bN - wTwN0;
  const double bb1 = b[2] * inv_bN - wTwN1;
  const double A = (Wb00 + Wb11) - dot2(wT0, wT1, bb0, bb1);
  const double B0 = Wb11 * bb0 - Wb10 * bb1;
  const double B1 = Wb00 * bb1 - Wb01 * bb0;
  const double det = Wb00 * Wb11 - Wb10 * Wb01;
  const double C = det - dot2(wT0, wT1, B0, B1);
  const double D = (wN * wN) / (mu * mu);
  double coeffs[4];
  coeffs[0] = C * C - D * dot2(B0, B1, B0, B1);
  coeffs[1] = 2.0 * (C * A - D * dot2(bb0, bb1, B0, B1));
  coeffs[2] = (2.0 * C + A * A) - D * dot2(bb0, bb1, bb0, bb1);
  coeffs[3] = 2.0 * A;
  double roots[4];
  const int nRoots = realRootsMonic(coeffs, 4, roots, StrictlyPositiveRoots);
  if (nRoots == 0) return false;
  double alpha = roots[0];
  for (int i = 1; i < nRoots; ++i)
    if (roots[i] < alpha) alpha = roots[i];
  const double M[4] = {Wb00 + alpha, Wb01, Wb10, Wb11 + alpha};
  FullPivLU lu;
  lu.compute(M, 2);
  const double rhs[2] = {(-bN) * bb0, (-bN) * bb1};
  double rt[2];
  lu.solve(rhs, rt);
  r[1] = rt[0];
  r[2] = rt[1];
  r[0] = norm2(rt[0], rt[1]) / mu;
  return true;
}

// AnalyticLocalSOCSolver<3, double, false>::solveOrthogonality (LocalSOCSolver.impl.hpp:139-199)
inline bool analyticSOC(const double* W, const double* b, double* r, double mu) {
  auto w = [&](int i, int j) { return W[3 * i + j]; };
  const double A = ((b[1] * w(1, 2) - b[2] * w(1, 1)) * mu * mu + b[0] * w(0, 2)) - b[2] * w(0, 0);
  const double B = ((b[0] * w(1, 2) + b[1] * w(0, 2)) - 2.0 * b[2] * w(0, 1)) * mu;
  const double C = 2.0 * ((((b[1] * w(2, 2) - b[2] * w(1, 2)) * mu * mu) - b[0] * w(0, 1)) + b[1] * w(0, 0));
  const double D = 2.0 * ((b[0] * (w(1, 1) - w(2, 2)) - b[1] * w(0, 1)) + b[2] * w(0, 2)) * mu;
  const double E = -6.0 * (b[0] * w(1, 2) - b[1] * w(0, 2)) * mu;
  double coeffs[5] = {A + B, C - D, E, C + D, B - A};
  double roots[4];
  const int nRoots = realRootsDegenerate(coeffs, 4, roots, AllRoots);
  for (int i = 0; i < nRoots; ++i) {
    const double t = roots[i];
    const double den = 1.0 + t * t;
    const double CT = (1.0 - t * t) / den;
    const double ST = (2.0 * t) / den;
    const double dir[3] = {1.0, mu * CT, mu * ST};
    const double v0[3] = {mu * w(0, 1) + CT * w(0, 0), mu * w(1, 1) + CT * w(1, 0), mu * w(2, 1) + CT * w(2, 0)};
    const double v1[3] = {mu * w(0, 2) + ST * w(0, 0), mu * w(1, 2) + ST * w(1, 0), mu * w(2, 2) + ST * w(2, 0)};
    const double den0 = dot3(v0, dir);
    const double den1 = dot3(v1, dir);
    double rN;
    if (std::fabs(den0) > std::fabs(den1)) {
      if (isZero(den0)) continue;
      rN = -(CT * b[0] + b[1] * mu) / den0;
    } else {
      if (isZero(den1)) continue;
      rN = -(ST * b[0] + b[2] * mu) / den1;
    }
    if (rN <= 0) continue;
    r[0] = rN * dir[0];
    r[1] = rN * dir[1];
    r[2] = rN * dir[2];
    const double col0[3] = {w(0, 0), w(1, 0), w(2, 0)};
    const double uN = dot3(col0, r) + b[0];
    if (uN > 0) return true;
  }
  return false;
}

// local_soc_solver::Strategy (Extra/SecondOrder.fwd.hpp:33-55)
enum Strategy { PureNewton = 0, PureEnumerative = 1, Hybrid = 2, RevHybrid = 3 };

// LocalSOCSolver<3, double, DeSaxceCOV, Strat>::solve (Extra/SOC/LocalSOCSolver.impl.hpp:243-318).
// For mu < 0 the reference solves A x = -b with a full-pivoting Householder QR; this restatement uses
// the full-pivoting LU (same solution for non-singular A).
inline double localSolve(bool desaxce, int strat, const double* A, const double* b, double* x, double mu, double tol,
                         double scaling) {
  if (mu < 0) {
    FullPivLU lu;
    lu.compute(A, 3);
    const double mb[3] = {-b[0], -b[1], -b[2]};
    lu.solve(mb, x);
    double ax[3];
    matvec3(A, x, ax);
    const double res[3] = {ax[0] + b[0], ax[1] + b[1], ax[2] + b[2]};
    return sq3(res);
  }
  LocalFB fb{desaxce, mu, scaling, A, b};
  if (strat == PureNewton) return newtonSolve(fb, tol, x);
  const double thr = desaxce ? 0.0 : mu * norm2(b[1], b[2]);
  if (b[0] >= thr) {  // take-off
    x[0] = x[1] = x[2] = 0.0;
    return 0.0;
  }
  if (isZero(mu)) {  // frictionless
    if (A[0] < kEps) {
      x[0] = x[1] = x[2] = 0.0;
      return b[0] * b[0];
    }
    x[1] = x[2] = 0.0;
    x[0] = (-b[0]) / A[0];
    return 0.0;
  }
  double res = 0.0;
  if (strat == Hybrid) {
    res = newtonSolve(fb, tol, x);
    if (res < tol) return res;
  }
  const double x0[3] = {x[0], x[1], x[2]};
  {
    FullPivLU lu;
    lu.compute(A, 3);
    const double mb[3] = {-b[0], -b[1], -b[2]};
    lu.solve(mb, x);
  }
  if (mu * x[0] >= norm2(x[1], x[2])) return 0.0;  // stick
  const bool ok = desaxce ? analyticCoulomb(A, b, x, mu) : analyticSOC(A, b, x, mu);
  if (!ok) { x[0] = x0[0]; x[1] = x0[1]; x[2] = x0[2]; }
  if (strat == RevHybrid) {
    res = newtonSolve(fb, tol, x);
  } else if (strat == Hybrid) {
    const double refined = newtonSolve(fb, tol, x);
    if (refined <= res) return refined;
    x[0] = x0[0]; x[1] = x0[1]; x[2] = x0[2];
  }
  return res;
}

// SOCLaw::solveLocal (SOCLaw.impl.hpp:37-44): success when the local residual is below the local tolerance
inline bool lawSolveLocal(bool desaxce, int strat, const double* A, const double* b, double* x, double mu, double scaling) {
  return kLocalTol > localSolve(desaxce, strat, A, b, x, mu, kLocalTol, scaling);
}

// nesterov_inertia (Core/BlockSolvers/ProjectedGradient.impl.hpp:30-39)
inline double nesterovInertia(double& theta, double q) {
  const double theta_prev = theta;
  const double theta_p2 = theta_prev * theta_prev;
  const double bb = theta_p2 - q;
  const double delta = std::sqrt(bb * bb + 4.0 * theta_p2);
  theta = 0.5 * (delta - bb);
  return (theta_prev - theta_p2) / (theta_p2 + theta);
}

}  // namespace oracle
