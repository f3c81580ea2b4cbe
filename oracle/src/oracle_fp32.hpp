// ORACLE — test infrastructure only (see oracle_math.hpp).
//
// The FP32 part of the FP32-refined projected-gradient solve (no counterpart in the reference), restated for the
// tests: PgMethod<APGD> (ProjectedGradient.impl.hpp:74-155, as solveAPGD in oracle_solvers.hpp) with W, the
// iterates and the per-contact law in single precision, and the reductions, the residual and the step decisions
// in double, converting at the same points as the GPU's FP32 kernel: each per-contact value is formed in float
// and widened for the canonical sum; a double step scalar (alpha, beta) is rounded to float where it enters
// float arithmetic. The law functions are the single-precision forms of SOCLaw::eval, dualityCOV and
// projectOnConstraint (float epsilon in the zero tests, NumTraits<float>). The solve also carries the FP32
// stall test: it stops once its residual has repeated bit for bit, or its line search has run out of trials,
// on stallIters consecutive iterations.
#pragma once

#include <cfloat>
#include <cmath>
#include <vector>

#include "oracle_solvers.hpp"

namespace oracle {
namespace fp32 {

inline bool isZero(float s) { return std::fabs(s) < FLT_EPSILON; }
inline float dot3(const float* a, const float* b) { return std::fma(a[2], b[2], std::fma(a[1], b[1], a[0] * b[0])); }
inline float sq3(const float* a) { return dot3(a, a); }
inline float norm2(float a0, float a1) { return std::sqrt(std::fma(a1, a1, a0 * a0)); }

inline void fbCanonical(const float* x, const float* y, float* fb) {
  float z2[3];
  z2[0] = sq3(x) + sq3(y);
  z2[1] = std::fma(x[0], x[1], y[0] * y[1]);
  z2[2] = std::fma(x[0], x[2], y[0] * y[2]);
  const float nz2t = norm2(z2[1], z2[2]);
  float om1[3], om2[3];
  om1[0] = om2[0] = 0.5f;
  if (isZero(nz2t)) {
    om1[1] = -0.5f; om1[2] = 0.f;
    om2[1] = 0.5f;  om2[2] = 0.f;
  } else {
    const float inv = 1.f / nz2t;
    const float t1 = z2[1] * inv, t2 = z2[2] * inv;
    om1[1] = -0.5f * t1; om1[2] = -0.5f * t2;
    om2[1] = 0.5f * t1;  om2[2] = 0.5f * t2;
  }
  const float l1 = z2[0] - 2.f * nz2t;
  const float rl1 = std::sqrt(l1 > 0.f ? l1 : 0.f);
  const float rl2 = std::sqrt(z2[0] + 2.f * nz2t);
  for (int k = 0; k < 3; ++k) fb[k] = (x[k] + y[k]) - std::fma(rl2, om2[k], rl1 * om1[k]);
}

// SOCLaw::eval in float: |fb|^2, |y|^2 when mu < 0
inline float lawEval(bool desaxce, float mu, const float* x, const float* y) {
  if (mu < 0.f) return sq3(y);
  float yy[3] = {y[0], y[1], y[2]};
  if (desaxce) yy[0] = std::fma(mu, norm2(y[1], y[2]), y[0]);
  float fb[3];
  if (isZero(mu)) {
    fb[0] = (x[0] + yy[0]) - std::sqrt(std::fma(yy[0], yy[0], x[0] * x[0]));
    fb[1] = x[1];
    fb[2] = x[2];
  } else {
    const float xh[3] = {mu * x[0], x[1], x[2]};
    const float yh[3] = {yy[0], mu * yy[1], mu * yy[2]};
    fbCanonical(xh, yh, fb);
  }
  return sq3(fb);
}
inline float cov(bool desaxce, float mu, const float* y) { return desaxce ? mu * norm2(y[1], y[2]) : 0.f; }
inline void project(float mu, float* x) {
  const float nxt = norm2(x[1], x[2]);
  const float xn = x[0];
  if (mu < 0.f) {
    x[0] = x[1] = x[2] = 0.f;
    return;
  }
  if (nxt <= mu * xn) return;
  if (mu * nxt <= -xn) {
    x[0] = x[1] = x[2] = 0.f;
    return;
  }
  const float proj = std::fma(mu, nxt, xn) / std::fma(mu, mu, 1.f);
  x[0] = proj;
  const float f = (proj * mu) / nxt;
  x[1] *= f;
  x[2] *= f;
}

// APGD (apgd) or Descent in float from x (float, 3n, projected first); returns the best residual and leaves the
// best iterate in x. mu, b, scaling are the double data, rounded to float as the FP32 copies are.
inline double solveAPGD32(const ProjectedGradient& pg, const BSR& W, bool desaxce, const double* mu64,
                          const double* b64, float* x, bool apgd, unsigned stallIters, unsigned* itersOut) {
  const int N = W.n;
  const size_t n3 = 3 * (size_t)N;
  std::vector<float> W32(W.val.size()), mu(N), b(n3), sc(N);
  for (size_t k = 0; k < W32.size(); ++k) W32[k] = (float)W.val[k];
  for (int i = 0; i < N; ++i) {
    mu[i] = (float)mu64[i];
    sc[i] = (float)pg.scaling[i];
  }
  for (size_t k = 0; k < n3; ++k) b[k] = (float)b64[k];
  auto product = [&](const float* v, float* out) { spmv32(W, W32.data(), v, out); };
  auto projectAll = [&](float* v) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) project(mu[i], &v[3 * i]);
  };
  // error function: per-contact values in float, the sum (or maximum) in double
  auto eval = [&](const float* y, const float* xv) {
    std::vector<double> v(N);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
      const float lx[3] = {xv[3 * i] * sc[i], xv[3 * i + 1] * sc[i], xv[3 * i + 2] * sc[i]};
      v[i] = (double)lawEval(desaxce, mu[i], lx, &y[3 * i]);
    }
    if (pg.useInfinityNorm) return maxOf(v.data(), N);
    return canonicalSum(v.data(), N) / (double)(1 + N);
  };
  auto objective = [&](const float* xv, const float* Mx, const float* s) {
    return reduceContacts(N, [&](int i) {
      float t[3];
      for (int k = 0; k < 3; ++k) t[k] = (0.5f * Mx[3 * i + k] + b[3 * i + k]) + s[3 * i + k];
      return (double)dot3(&xv[3 * i], t);
    });
  };
  std::vector<float> Mx(n3), y(n3), xs(n3), s(n3, 0.f), prev, x_best;
  projectAll(x);
  product(x, Mx.data());
  double theta = 1., q = 0;
  prev.assign(x, x + n3);
  double alpha = 1.;
  {  // guess_alpha (:21-28)
    std::vector<float> d(n3), Md(n3);
    for (size_t k = 0; k < n3; ++k) d[k] = x[k] - 1.f;
    product(d.data(), Md.data());
    const double nMx = reduceContacts(N, [&](int i) { return (double)sq3(&Md[3 * i]); });
    if (nMx > 1.e-16) alpha = dmin(1., reduceContacts(N, [&](int i) { return (double)sq3(&d[3 * i]); }) / nMx);
  }
  double min_res = -1, prev_res = 0.0;
  unsigned stallRun = 0;
  bool exhausted = false;
  unsigned it;
  for (it = 0; it < pg.maxIters; ++it) {
    for (size_t k = 0; k < n3; ++k) y[k] = Mx[k] + b[k];
    const double res = eval(y.data(), x);
    pg.trigger(it, res);
    if (0 == it || res < min_res) {
      x_best.assign(x, x + n3);
      min_res = res;
    }
    if (res < pg.tol) break;
    if (stallIters) {
      stallRun = ((it > 0 && res == prev_res) || exhausted) ? stallRun + 1 : 0;
      prev_res = res;
      if (stallRun >= stallIters) break;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) s[3 * i] = cov(desaxce, mu[i], &y[3 * i]);
    for (size_t k = 0; k < n3; ++k) y[k] = y[k] + s[k];
    const double J = objective(x, Mx.data(), s.data());
    alpha *= pg.lsOptimisticFactor;
    unsigned ls;
    for (ls = 0; ls < pg.lsIters; ++ls, alpha *= pg.lsPessimisticFactor) {
      const float na = (float)(-alpha);
      for (size_t k = 0; k < n3; ++k) xs[k] = std::fma(na, y[k], x[k]);
      projectAll(xs.data());
      product(xs.data(), Mx.data());
      const double Js = objective(xs.data(), Mx.data(), s.data());
      const double decr = reduceContacts(N, [&](int i) {
        const float d[3] = {xs[3 * i] - x[3 * i], xs[3 * i + 1] - x[3 * i + 1], xs[3 * i + 2] - x[3 * i + 2]};
        return (double)dot3(&y[3 * i], d);
      });
      const double nrm = reduceContacts(N, [&](int i) {
        const float d[3] = {xs[3 * i] - x[3 * i], xs[3 * i + 1] - x[3 * i + 1], xs[3 * i + 2] - x[3 * i + 2]};
        return (double)sq3(d);
      });
      if (Js < (J + decr) + (.5 / alpha) * nrm) break;
    }
    exhausted = pg.lsIters > 0 && ls >= pg.lsIters;
    const double decr2 = reduceContacts(N, [&](int i) {
      const float d[3] = {xs[3 * i] - prev[3 * i], xs[3 * i + 1] - prev[3 * i + 1], xs[3 * i + 2] - prev[3 * i + 2]};
      return (double)dot3(d, &y[3 * i]);
    });
    if (apgd && decr2 < 0) {
      const float beta = (float)nesterovInertia(theta, q);
      for (size_t k = 0; k < n3; ++k) x[k] = std::fma(beta, xs[k] - prev[k], xs[k]);
      product(x, Mx.data());
    } else {
      std::copy(xs.begin(), xs.end(), x);
      theta = 1.;
    }
    prev = xs;
  }
  std::copy(x_best.begin(), x_best.end(), x);
  if (itersOut) *itersOut = it;
  return min_res;
}

}  // namespace fp32
}  // namespace oracle
