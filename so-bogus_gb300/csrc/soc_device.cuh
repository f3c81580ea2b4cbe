// Per-contact mathematics of the 3D Coulomb / second-order-cone law, on the device.
//
// Follows So-bogus's formulas (Extra/SOC/FischerBurmeister.impl.hpp, SOCLaw.impl.hpp,
// LocalSOCSolver.impl.hpp, Core/Utils/NonSmoothNewton.impl.hpp, Core/Utils/Polynomial.impl.hpp) with one
// fixed evaluation order, chosen for the FP64 pipe (fused multiply-adds, one reciprocal per repeated
// denominator):
//   dot3(a,b) = fma(a2,b2, fma(a1,b1, a0*b0)),  3x3 rows the same, squared norms dot3(a,a).
// The translation unit is compiled with --fmad=false, so no other contraction happens; division and
// sqrt are IEEE correctly rounded: in the law and projection functions (the per-iteration work of the
// iterative solvers, throughput bound) through the integer-pipe implementations of fp64_int.cuh, elsewhere
// (the local solvers' QR, LU and closed forms, latency bound along the Gauss-Seidel chains, where the
// integer sequence is slower than the hardware's) the CUDA operations. Multiplications by 1/2 and 2 and the
// zero test are exact bit operations. Every
// function is __host__ __device__ so the CPU test helper can run the identical code.
#pragma once

#include <cmath>

#include "fp64_int.cuh"

#ifdef __CUDACC__
#define BG_HD __host__ __device__ __forceinline__
#else
#define BG_HD inline
#endif

namespace bogus_gpu {

constexpr double kEps = 2.220446049250313080847e-16;       // NumTraits<double>::epsilon()
constexpr double kLocalTol = 1.8189894035458565e-12;      // pow(eps, 0.75) == 2^-39 (SOCLaw local tolerance)

// fabs(s) < eps, compared as bit patterns (non-negative doubles order like their bits; NaN compares false)
BG_HD bool is_zero(double s) {
  return (ipipe::to_bits(s) & ~(uint64_t(1) << 63)) < ipipe::to_bits(kEps);
}
BG_HD double dmax(double a, double b) { return (a < b) ? b : a; }
BG_HD double dmin(double a, double b) { return (b < a) ? b : a; }
BG_HD double dot3(const double* a, const double* b) { return fma(a[2], b[2], fma(a[1], b[1], a[0] * b[0])); }
BG_HD double sq3(const double* a) { return dot3(a, a); }
BG_HD double dot2(double a0, double a1, double b0, double b1) { return fma(a1, b1, a0 * b0); }
BG_HD double norm2(double a0, double a1) { return ipipe::sqrt_rn(dot2(a0, a1, a0, a1)); }
BG_HD void matvec3(const double* A, const double* x, double* y) {
#pragma unroll
  for (int r = 0; r < 3; ++r) y[r] = fma(A[3 * r + 2], x[2], fma(A[3 * r + 1], x[1], A[3 * r] * x[0]));
}

// ------------------------------------------------------------------------------------------------
// Full-pivoting LU for n = 2, 3 (FullPivLU semantics: complete pivoting, first maximum in row-major
// order, elimination stops at an exactly zero pivot, pivots below eps*n*|p0| count as zero in solve)
// ------------------------------------------------------------------------------------------------
template <int N>
struct SmallLU {
  double lu[N * N];
  double inv_piv[N];
  int rowt[N], colt[N];
  int rank;

  BG_HD void compute(const double* A) {
#pragma unroll
    for (int k = 0; k < N * N; ++k) lu[k] = A[k];
    int nonzero = N;
    for (int k = 0; k < N; ++k) {
      int pi = k, pj = k;
      double best = -1.0;
      for (int i = k; i < N; ++i)
        for (int j = k; j < N; ++j) {
          const double a = fabs(lu[i * N + j]);
          if (a > best) { best = a; pi = i; pj = j; }
        }
      rowt[k] = pi;
      colt[k] = pj;
      if (best == 0.0) {
        nonzero = k;
        for (int kk = k; kk < N; ++kk) { rowt[kk] = kk; colt[kk] = kk; }
        break;
      }
      if (pi != k)
        for (int j = 0; j < N; ++j) { const double t = lu[k * N + j]; lu[k * N + j] = lu[pi * N + j]; lu[pi * N + j] = t; }
      if (pj != k)
        for (int i = 0; i < N; ++i) { const double t = lu[i * N + k]; lu[i * N + k] = lu[i * N + pj]; lu[i * N + pj] = t; }
      const double inv = 1.0 / lu[k * N + k];
      inv_piv[k] = inv;
      for (int i = k + 1; i < N; ++i) lu[i * N + k] *= inv;
      for (int i = k + 1; i < N; ++i) {
        const double l = lu[i * N + k];
        for (int j = k + 1; j < N; ++j) lu[i * N + j] = fma(-l, lu[k * N + j], lu[i * N + j]);
      }
    }
    rank = 0;
    if (nonzero > 0) {
      const double thr = kEps * (double)N * fabs(lu[0]);
      for (int k = 0; k < nonzero; ++k)
        if (fabs(lu[k * N + k]) > thr) ++rank;
    }
  }

  BG_HD void solve(const double* b, double* x) const {
    double c[N];
#pragma unroll
    for (int i = 0; i < N; ++i) c[i] = b[i];
    for (int k = 0; k < N; ++k) { const int p = rowt[k]; if (p != k) { const double t = c[k]; c[k] = c[p]; c[p] = t; } }
    for (int i = 1; i < N; ++i)
      for (int j = 0; j < i; ++j) c[i] = fma(-lu[i * N + j], c[j], c[i]);
    for (int i = rank - 1; i >= 0; --i) {
      for (int j = i + 1; j < rank; ++j) c[i] = fma(-lu[i * N + j], c[j], c[i]);
      c[i] = c[i] * inv_piv[i];
    }
    for (int i = rank; i < N; ++i) c[i] = 0.0;
    for (int k = N - 1; k >= 0; --k) { const int p = colt[k]; if (p != k) { const double t = c[k]; c[k] = c[p]; c[p] = t; } }
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = c[i];
  }
};

// ------------------------------------------------------------------------------------------------
// Real eigenvalues of an upper Hessenberg matrix (n <= 4) by the Francis implicit double-shift QR
// iteration (the published EISPACK hqr method); companion matrices give polynomial roots
// (RootsFinder::getRealRoots: real when |imag| < eps).
// ------------------------------------------------------------------------------------------------
enum { kAllRoots = 0, kStrictlyNegativeRoots = 1, kStrictlyPositiveRoots = 2 };

BG_HD int hessenberg_eigenvalues(double* a, int n, double* wr, double* wi) {
#define BG_A(i, j) a[(i) * n + (j)]
  double anorm = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = (i > 0 ? i - 1 : 0); j < n; ++j) anorm += fabs(BG_A(i, j));
  int nn = n - 1;
  double t = 0.0;
  int total = 0;
  while (nn >= 0) {
    int its = 0, l;
    for (;;) {
      for (l = nn; l >= 1; --l) {
        double s = fabs(BG_A(l - 1, l - 1)) + fabs(BG_A(l, l));
        if (s == 0.0) s = anorm;
        if (fabs(BG_A(l, l - 1)) + s == s) { BG_A(l, l - 1) = 0.0; break; }
      }
      double x = BG_A(nn, nn);
      if (l == nn) {
        wr[nn] = x + t;
        wi[nn] = 0.0;
        --nn;
        break;
      }
      double y = BG_A(nn - 1, nn - 1);
      double w = BG_A(nn, nn - 1) * BG_A(nn - 1, nn);
      if (l == nn - 1) {
        const double p = 0.5 * (y - x);
        const double q = p * p + w;
        double z = sqrt(fabs(q));
        x += t;
        if (q >= 0.0) {
          z = p + (p >= 0.0 ? fabs(z) : -fabs(z));
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
      if (its == 10 || its == 20) {
        t += x;
        for (int i = 0; i <= nn; ++i) BG_A(i, i) -= x;
        const double s = fabs(BG_A(nn, nn - 1)) + fabs(BG_A(nn - 1, nn - 2));
        x = y = 0.75 * s;
        w = -0.4375 * s * s;
      }
      ++its;
      ++total;
      int m;
      double p = 0, q = 0, r = 0, z;
      for (m = nn - 2; m >= l; --m) {
        z = BG_A(m, m);
        const double rr = x - z;
        const double ss = y - z;
        p = (rr * ss - w) / BG_A(m + 1, m) + BG_A(m, m + 1);
        q = BG_A(m + 1, m + 1) - z - rr - ss;
        r = BG_A(m + 2, m + 1);
        const double sc = fabs(p) + fabs(q) + fabs(r);
        p /= sc;
        q /= sc;
        r /= sc;
        if (m == l) break;
        const double u = fabs(BG_A(m, m - 1)) * (fabs(q) + fabs(r));
        const double v = fabs(p) * (fabs(BG_A(m - 1, m - 1)) + fabs(z) + fabs(BG_A(m + 1, m + 1)));
        if (u + v == v) break;
      }
      for (int i = m + 2; i <= nn; ++i) {
        BG_A(i, i - 2) = 0.0;
        if (i != m + 2) BG_A(i, i - 3) = 0.0;
      }
      for (int k = m; k <= nn - 1; ++k) {
        if (k != m) {
          p = BG_A(k, k - 1);
          q = BG_A(k + 1, k - 1);
          r = 0.0;
          if (k != nn - 1) r = BG_A(k + 2, k - 1);
          x = fabs(p) + fabs(q) + fabs(r);
          if (x != 0.0) { p /= x; q /= x; r /= x; }
        }
        const double nrm = sqrt(p * p + q * q + r * r);
        const double s = (p >= 0.0 ? nrm : -nrm);
        if (s != 0.0) {
          if (k == m) {
            if (l != m) BG_A(k, k - 1) = -BG_A(k, k - 1);
          } else {
            BG_A(k, k - 1) = -s * x;
          }
          p += s;
          x = p / s;
          y = q / s;
          z = r / s;
          q /= p;
          r /= p;
          for (int j = k; j <= nn; ++j) {
            p = BG_A(k, j) + q * BG_A(k + 1, j);
            if (k != nn - 1) {
              p += r * BG_A(k + 2, j);
              BG_A(k + 2, j) -= p * z;
            }
            BG_A(k + 1, j) -= p * y;
            BG_A(k, j) -= p * x;
          }
          const int mmin = nn < k + 3 ? nn : k + 3;
          for (int i = l; i <= mmin; ++i) {
            p = x * BG_A(i, k) + y * BG_A(i, k + 1);
            if (k != nn - 1) {
              p += z * BG_A(i, k + 2);
              BG_A(i, k + 2) -= p * r;
            }
            BG_A(i, k + 1) -= p * q;
            BG_A(i, k) -= p;
          }
        }
      }
    }
  }
  return 0;
#undef BG_A
}

#ifdef __CUDACC__
// hessenberg_eigenvalues run by a whole (converged) warp on a matrix in the warp's shared memory. Every lane
// holds the same scalars and follows the same control flow; the independent operations of a step run on
// different lanes of one instruction: the deflation tests of every row, the three (or five) divisions by the
// scale (or by s and p), the three squares of the norm, one column of the row modification, one row of the
// column modification. On GB300 an FP64 instruction occupies the sub-partition's FP64 unit for the same time
// with one active lane or many, so a step costs a fraction of the scalar chain. Each value goes through the
// same operations in the same order as in the scalar version, so the eigenvalues are identical.
__device__ __forceinline__ double warp_bcast(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

__device__ inline int hessenberg_eigenvalues_warp(double* a, int n, double* wr, double* wi) {
#define BG_A(i, j) a[(i) * n + (j)]
  const int lane = threadIdx.x & 31;
  double anorm = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = (i > 0 ? i - 1 : 0); j < n; ++j) anorm += fabs(BG_A(i, j));
  int nn = n - 1;
  double t = 0.0;
  int total = 0;
  while (nn >= 0) {
    int its = 0, l;
    for (;;) {
      {  // lane c tests l = c + 1; the scalar search stops at the largest l that passes (0 when none does)
        const int L = lane + 1;
        bool pass = false;
        if (L <= nn) {
          double s = fabs(BG_A(L - 1, L - 1)) + fabs(BG_A(L, L));
          if (s == 0.0) s = anorm;
          pass = fabs(BG_A(L, L - 1)) + s == s;
        }
        const unsigned m = __ballot_sync(0xffffffffu, pass);
        l = m ? 32 - __clz((int)m) : 0;
        __syncwarp();
        if (l >= 1 && lane == 0) BG_A(l, l - 1) = 0.0;
        __syncwarp();
      }
      double x = BG_A(nn, nn);
      if (l == nn) {
        wr[nn] = x + t;
        wi[nn] = 0.0;
        --nn;
        break;
      }
      double y = BG_A(nn - 1, nn - 1);
      double w = BG_A(nn, nn - 1) * BG_A(nn - 1, nn);
      if (l == nn - 1) {
        const double p = 0.5 * (y - x);
        const double q = p * p + w;
        double z = sqrt(fabs(q));
        x += t;
        if (q >= 0.0) {
          z = p + (p >= 0.0 ? fabs(z) : -fabs(z));
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
      if (its == 10 || its == 20) {
        t += x;
        __syncwarp();
        if (lane <= nn) BG_A(lane, lane) -= x;
        __syncwarp();
        const double s = fabs(BG_A(nn, nn - 1)) + fabs(BG_A(nn - 1, nn - 2));
        x = y = 0.75 * s;
        w = -0.4375 * s * s;
      }
      ++its;
      ++total;
      int m;
      double p = 0, q = 0, r = 0, z;
      {
        // The scalar search tries m = nn - 2, nn - 3, ..., l and stops at the first m that passes its test (m = l
        // always does). Candidate values do not depend on one another: lane group g (lanes 3g..3g+2) evaluates
        // m = nn - 2 - g, lane 3g + c normalising component c; the search's m is the first group that passes.
        const int g = lane / 3, c = lane - 3 * g;
        const bool valid = lane < 30 && nn - 2 - g >= l;
        const int mc = valid ? nn - 2 - g : l;
        const double zc = BG_A(mc, mc);
        const double rr = x - zc;
        const double ss = y - zc;
        const double pc = (rr * ss - w) / BG_A(mc + 1, mc) + BG_A(mc, mc + 1);
        const double qc = BG_A(mc + 1, mc + 1) - zc - rr - ss;
        const double rc = BG_A(mc + 2, mc + 1);
        const double sc = fabs(pc) + fabs(qc) + fabs(rc);
        const double vn = (c == 0 ? pc : (c == 1 ? qc : rc)) / sc;
        const int g0 = lane < 30 ? 3 * g : 0;
        const double pn = __shfl_sync(0xffffffffu, vn, g0);
        const double qn = __shfl_sync(0xffffffffu, vn, g0 + 1);
        const double rn = __shfl_sync(0xffffffffu, vn, g0 + 2);
        bool stop = valid && mc == l;
        if (valid && mc != l) {
          const double u = fabs(BG_A(mc, mc - 1)) * (fabs(qn) + fabs(rn));
          const double v = fabs(pn) * (fabs(BG_A(mc - 1, mc - 1)) + fabs(zc) + fabs(BG_A(mc + 1, mc + 1)));
          stop = u + v == v;
        }
        const unsigned hit = __ballot_sync(0xffffffffu, stop && c == 0);
        const int src = __ffs((int)hit) - 1;  // the leader lane of the first group that stops
        m = nn - 2 - src / 3;
        p = __shfl_sync(0xffffffffu, pn, src);
        q = __shfl_sync(0xffffffffu, qn, src);
        r = __shfl_sync(0xffffffffu, rn, src);
        z = __shfl_sync(0xffffffffu, zc, src);
      }
      __syncwarp();
      {
        const int i = m + 2 + lane;
        if (i <= nn) {
          BG_A(i, i - 2) = 0.0;
          if (i != m + 2) BG_A(i, i - 3) = 0.0;
        }
      }
      __syncwarp();
      for (int k = m; k <= nn - 1; ++k) {
        if (k != m) {
          p = BG_A(k, k - 1);
          q = BG_A(k + 1, k - 1);
          r = 0.0;
          if (k != nn - 1) r = BG_A(k + 2, k - 1);
          x = fabs(p) + fabs(q) + fabs(r);
          if (x != 0.0) {
            const double v = (lane == 0 ? p : (lane == 1 ? q : r)) / x;
            p = warp_bcast(v, 0);
            q = warp_bcast(v, 1);
            r = warp_bcast(v, 2);
          }
        }
        double nrm;
        {  // sqrt(p * p + q * q + r * r), evaluated as (p*p + q*q) + r*r
          const double c = lane == 0 ? p : (lane == 1 ? q : r);
          const double sq = c * c;
          nrm = sqrt((warp_bcast(sq, 0) + warp_bcast(sq, 1)) + warp_bcast(sq, 2));
        }
        const double s = (p >= 0.0 ? nrm : -nrm);
        if (s != 0.0) {
          __syncwarp();
          if (lane == 0) {
            if (k == m) {
              if (l != m) BG_A(k, k - 1) = -BG_A(k, k - 1);
            } else {
              BG_A(k, k - 1) = -s * x;
            }
          }
          p += s;
          {  // x = p / s, y = q / s, z = r / s, q = q / p, r = r / p
            const double num = lane == 0 ? p : (lane == 1 || lane == 3 ? q : r);
            const double v = num / (lane < 3 ? s : p);
            x = warp_bcast(v, 0);
            y = warp_bcast(v, 1);
            z = warp_bcast(v, 2);
            q = warp_bcast(v, 3);
            r = warp_bcast(v, 4);
          }
          __syncwarp();
          // Row and column modifications: lane 4u + c takes column (row) c of the step and, once every lane has
          // read the old values, applies the u-th of its three independent updates; the updates are selected
          // without branching, so the three run as one instruction stream (x 1.0 is exact: a - p * 1.0 = a - p).
          const int c4 = lane & 3, u4 = lane >> 2;
          {  // row modification, column j = k + c4
            const int j = k + c4;
            const bool on = lane < 12 && j <= nn;
            double pj = 0.0;
            if (on) {
              pj = BG_A(k, j) + q * BG_A(k + 1, j);
              if (k != nn - 1) pj += r * BG_A(k + 2, j);
            }
            __syncwarp();
            if (on && (u4 != 0 || k != nn - 1)) {
              const int row = k + 2 - u4;
              const double f = u4 == 0 ? z : (u4 == 1 ? y : x);
              BG_A(row, j) -= pj * f;
            }
          }
          __syncwarp();
          const int mmin = nn < k + 3 ? nn : k + 3;
          {  // column modification, row i = l + c4
            const int i = l + c4;
            const bool on = lane < 12 && i <= mmin;
            double pi = 0.0;
            if (on) {
              pi = x * BG_A(i, k) + y * BG_A(i, k + 1);
              if (k != nn - 1) pi += z * BG_A(i, k + 2);
            }
            __syncwarp();
            if (on && (u4 != 0 || k != nn - 1)) {
              const int col = k + 2 - u4;
              const double f = u4 == 0 ? r : (u4 == 1 ? q : 1.0);
              BG_A(i, col) -= pi * f;
            }
          }
          __syncwarp();
        }
      }
    }
  }
  return 0;
#undef BG_A
}
#endif

// Eigenvalues of the companion matrix of the monic polynomial c[0] + c[1] t + ... + t^dim. Warp: the whole
// warp runs hessenberg_eigenvalues_warp on the matrix in sa (its shared memory, dim * dim doubles).
template <bool Warp>
BG_HD int companion_eigenvalues(const double* c, int dim, double* wr, double* wi, double* sa) {
#ifdef __CUDA_ARCH__
  if constexpr (Warp) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    for (int e = lane; e < dim * dim; e += 32) {
      const int i = e / dim, j = e - (e / dim) * dim;
      sa[e] = (j == dim - 1) ? -c[i] : (j == i - 1 ? 1.0 : 0.0);
    }
    __syncwarp();
    return hessenberg_eigenvalues_warp(sa, dim, wr, wi);
  }
#endif
  (void)sa;
  double a[16];
  for (int i = 0; i < dim * dim; ++i) a[i] = 0.0;
  for (int i = 1; i < dim; ++i) a[i * dim + (i - 1)] = 1.0;
  for (int i = 0; i < dim; ++i) a[i * dim + (dim - 1)] = -c[i];
  return hessenberg_eigenvalues(a, dim, wr, wi);
}

template <bool Warp = false>
BG_HD int real_roots_monic(const double* c, int dim, double* roots, int filter, double* sa = nullptr) {
  double wr[4], wi[4];
  if (companion_eigenvalues<Warp>(c, dim, wr, wi, sa) != 0) return 0;
  int count = 0;
  for (int i = 0; i < dim; ++i) {
    if (is_zero(wi[i])) {
      const bool discard = (filter == kStrictlyPositiveRoots && wr[i] <= 0) || (filter == kStrictlyNegativeRoots && wr[i] >= 0);
      if (!discard) roots[count++] = wr[i];
    }
  }
  return count;
}

template <bool Warp = false>
BG_HD int real_roots_degenerate(double* c, int dim, double* roots, int filter, double* sa = nullptr) {
  while (dim > 0 && is_zero(c[dim])) --dim;
  if (dim == 0) {
    roots[0] = 0.0;
    return (filter == kAllRoots && is_zero(c[0])) ? 1 : 0;
  }
  const double inv = 1.0 / c[dim];
  for (int k = 0; k < dim; ++k) c[k] *= inv;
  return real_roots_monic<Warp>(c, dim, roots, filter, sa);
}

// ------------------------------------------------------------------------------------------------
// Fischer-Burmeister function and Jacobian
// ------------------------------------------------------------------------------------------------
template <bool Jac>
BG_HD void fb_canonical(const double* x, const double* y, double* fb, double* dx, double* dy) {
  double z2[3];
  z2[0] = sq3(x) + sq3(y);
  z2[1] = fma(x[0], x[1], y[0] * y[1]);
  z2[2] = fma(x[0], x[2], y[0] * y[2]);
  const double nz2t = norm2(z2[1], z2[2]);
  double om1[3], om2[3];
  om1[0] = om2[0] = 0.5;
  if (is_zero(nz2t)) {
    om1[1] = -0.5; om1[2] = 0.0;
    om2[1] = 0.5;  om2[2] = 0.0;
  } else {
    const double inv = ipipe::div_rn(1.0, nz2t);
    const double t1 = z2[1] * inv, t2 = z2[2] * inv;
    om2[1] = ipipe::scale2<-1>(t1);  om2[2] = ipipe::scale2<-1>(t2);
    om1[1] = -om2[1]; om1[2] = -om2[2];  // -0.5 t == -(0.5 t) exactly
  }
  const double nz2t2 = ipipe::scale2<1>(nz2t);
  const double l1 = z2[0] - nz2t2;
  const double rl1 = ipipe::sqrt_rn(l1 > 0.0 ? l1 : 0.0);
  const double rl2 = ipipe::sqrt_rn(z2[0] + nz2t2);
  double z[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) z[k] = fma(rl2, om2[k], rl1 * om1[k]);
#pragma unroll
  for (int k = 0; k < 3; ++k) fb[k] = (x[k] + y[k]) - z[k];
  if (!Jac) return;
  if (is_zero(rl2)) {
#pragma unroll
    for (int k = 0; k < 9; ++k) dx[k] = dy[k] = 0.0;
    return;
  }
  if (is_zero(rl1)) {
    const double izn = ipipe::div_rn(1.0, dot2(x[0], y[0], x[0], y[0]));
    const double cx = 1.0 - x[0] * izn, cy = 1.0 - y[0] * izn;
#pragma unroll
    for (int k = 0; k < 9; ++k) dx[k] = dy[k] = 0.0;
    dx[0] = dx[4] = dx[8] = cx;
    dy[0] = dy[4] = dy[8] = cy;
    return;
  }
  const double det = rl1 * rl2;
  const double inv_det = ipipe::div_rn(1.0, det);
  const double inv_z0 = ipipe::div_rn(1.0, z[0]);
  double iL[9];
  iL[0] = z[0] * inv_det;
  iL[1] = -z[1] * inv_det;
  iL[2] = -z[2] * inv_det;
  iL[3] = iL[1];
  iL[6] = iL[2];
  iL[4] = (fma(z[1], z[1], det) * inv_z0) * inv_det;
  iL[5] = ((z[1] * z[2]) * inv_z0) * inv_det;
  iL[7] = iL[5];
  iL[8] = (fma(z[2], z[2], det) * inv_z0) * inv_det;
#pragma unroll
  for (int w = 0; w < 2; ++w) {
    const double* v = w == 0 ? x : y;
    double* o = w == 0 ? dx : dy;
    const double L[9] = {v[0], v[1], v[2], v[1], v[0], 0.0, v[2], 0.0, v[0]};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double p = fma(iL[3 * r + 2], L[6 + c], fma(iL[3 * r + 1], L[3 + c], iL[3 * r] * L[c]));
        o[3 * r + c] = (r == c ? 1.0 : 0.0) - p;
      }
  }
}

BG_HD void fb_mu(double mu, const double* x, const double* y, double* fb) {
  if (is_zero(mu)) {
    fb[0] = (x[0] + y[0]) - ipipe::sqrt_rn(dot2(x[0], y[0], x[0], y[0]));
    fb[1] = x[1];
    fb[2] = x[2];
  } else {
    const double xh[3] = {mu * x[0], x[1], x[2]};
    const double yh[3] = {y[0], mu * y[1], mu * y[2]};
    fb_canonical<false>(xh, yh, fb, nullptr, nullptr);
  }
}

BG_HD void fb_mu_jacobian(double mu, const double* x, const double* y, double* fb, double* dx, double* dy) {
  if (is_zero(mu)) {
    const double z = ipipe::sqrt_rn(dot2(x[0], y[0], x[0], y[0]));
    fb[0] = (x[0] + y[0]) - z;
    fb[1] = x[1];
    fb[2] = x[2];
#pragma unroll
    for (int k = 0; k < 9; ++k) { dx[k] = 0.0; dy[k] = 0.0; }
    dx[0] = dx[4] = dx[8] = 1.0;
    if (!is_zero(z)) {
      const double iz = ipipe::div_rn(1.0, z);
      dx[0] = 1.0 - x[0] * iz;
      dy[0] = 1.0 - y[0] * iz;
    }
  } else {
    const double xh[3] = {mu * x[0], x[1], x[2]};
    const double yh[3] = {y[0], mu * y[1], mu * y[2]};
    fb_canonical<true>(xh, yh, fb, dx, dy);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      dx[3 * r] *= mu;
      dy[3 * r + 1] *= mu;
      dy[3 * r + 2] *= mu;
    }
  }
}

BG_HD void fb_law(bool desaxce, double mu, const double* x, const double* y, double* fb) {
  if (desaxce) {
    const double yt[3] = {fma(mu, norm2(y[1], y[2]), y[0]), y[1], y[2]};
    fb_mu(mu, x, yt, fb);
  } else {
    fb_mu(mu, x, y, fb);
  }
}

// SOCLaw::eval: |fb|^2, |y|^2 when mu < 0
BG_HD double law_eval(bool desaxce, double mu, const double* x, const double* y) {
  if (mu < 0) return sq3(y);
  double fb[3];
  fb_law(desaxce, mu, x, y, fb);
  return sq3(fb);
}

// SOCLaw::projectOnConstraint
BG_HD void project_cone(double mu, double* x) {
  const double nxt = norm2(x[1], x[2]);
  const double xn = x[0];
  if (mu < 0) { x[0] = x[1] = x[2] = 0.0; return; }
  if (nxt <= mu * xn) return;
  if (mu * nxt <= -xn) { x[0] = x[1] = x[2] = 0.0; return; }
  const double den2 = fma(mu, mu, 1.0);
  const double proj = ipipe::div_rn(fma(mu, nxt, xn), den2);
  x[0] = proj;
  const double f = ipipe::div_rn(proj * mu, nxt);
  x[1] *= f;
  x[2] *= f;
}

// SOCLaw::dualityCOV: first component only (the tangential part is zero)
BG_HD double duality_cov(bool desaxce, double mu, const double* y) { return desaxce ? mu * norm2(y[1], y[2]) : 0.0; }

// ------------------------------------------------------------------------------------------------
// Local problem x -> FB(mu, scaling x, A x + b) and its non-smooth Newton solver
// ------------------------------------------------------------------------------------------------
struct LocalFB {
  bool desaxce;
  double mu, scaling;
  const double* A;
  const double* b;

  BG_HD void y_of(const double* x, double* y) const {
    double ax[3];
    matvec3(A, x, ax);
#pragma unroll
    for (int k = 0; k < 3; ++k) y[k] = ax[k] + b[k];
  }
  BG_HD void compute(const double* x, double* fb) const {
    double y[3];
    y_of(x, y);
    const double xs[3] = {scaling * x[0], scaling * x[1], scaling * x[2]};
    fb_law(desaxce, mu, xs, y, fb);
  }
  BG_HD void jacobian(const double* x, double* fb, double* dFdx) const {
    const double xs[3] = {scaling * x[0], scaling * x[1], scaling * x[2]};
    double y[3];
    y_of(x, y);
    double s = 0.0;
    if (desaxce) {
      s = norm2(y[1], y[2]);
      y[0] = fma(mu, s, y[0]);
    }
    double dy[9];
    fb_mu_jacobian(mu, xs, y, fb, dFdx, dy);
    if (desaxce && !is_zero(s)) {
      const double c = mu / s;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const double t = dy[3 * r] * c;
        dy[3 * r + 1] = fma(t, y[1], dy[3 * r + 1]);
        dy[3 * r + 2] = fma(t, y[2], dy[3 * r + 2]);
      }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) dFdx[k] *= scaling;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double p = fma(dy[3 * r + 2], A[6 + c], fma(dy[3 * r + 1], A[3 + c], dy[3 * r] * A[c]));
        dFdx[3 * r + c] = dFdx[3 * r + c] + p;
      }
  }
};

// NonSmoothNewton::solve, 20 iterations, Armijo-like damping on dPhi_dx = dF_dx^T x (reference quirk kept)
BG_HD double newton_solve(const LocalFB& f, double tol, double* x) {
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
  for (int iter = 0; iter < 20; ++iter) {
    f.jacobian(x, F, dF);
    const double Phi = 0.5 * sq3(F);
    if (Phi < tol) return Phi;
    if (Phi < Phi_best) {
      Phi_best = Phi;
      x_best[0] = x[0]; x_best[1] = x[1]; x_best[2] = x[2];
    }
    double dPhi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dPhi[k] = fma(dF[6 + k], x[2], fma(dF[3 + k], x[1], dF[k] * x[0]));
    SmallLU<3> lu;
    lu.compute(dF);
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

template <bool Warp = false>
BG_HD bool analytic_coulomb(const double* W, const double* b, double* r, double mu, double* sa = nullptr) {
  const double wN = W[0];
  if (wN < kEps) return false;
  const double wT0 = W[3], wT1 = W[6];
  const double bN = b[0];
  const double inv_wN = 1.0 / wN;
  const double wTwN0 = wT0 * inv_wN, wTwN1 = wT1 * inv_wN;
  const double Wb00 = fma(-wTwN0, wT0, W[4]);
  const double Wb01 = fma(-wTwN0, wT1, W[5]);
  const double Wb10 = fma(-wTwN1, wT0, W[7]);
  const double Wb11 = fma(-wTwN1, wT1, W[8]);
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
  const int nRoots = real_roots_monic<Warp>(coeffs, 4, roots, kStrictlyPositiveRoots, sa);
  if (nRoots == 0) return false;
  double alpha = roots[0];
  for (int i = 1; i < nRoots; ++i)
    if (roots[i] < alpha) alpha = roots[i];
  const double M[4] = {Wb00 + alpha, Wb01, Wb10, Wb11 + alpha};
  SmallLU<2> lu;
  lu.compute(M);
  const double rhs[2] = {(-bN) * bb0, (-bN) * bb1};
  double rt[2];
  lu.solve(rhs, rt);
  r[1] = rt[0];
  r[2] = rt[1];
  r[0] = norm2(rt[0], rt[1]) / mu;
  return true;
}

template <bool Warp = false>
BG_HD bool analytic_soc(const double* W, const double* b, double* r, double mu, double* sa = nullptr) {
#define BG_W(i, j) W[3 * (i) + (j)]
  const double A = ((b[1] * BG_W(1, 2) - b[2] * BG_W(1, 1)) * mu * mu + b[0] * BG_W(0, 2)) - b[2] * BG_W(0, 0);
  const double B = ((b[0] * BG_W(1, 2) + b[1] * BG_W(0, 2)) - 2.0 * b[2] * BG_W(0, 1)) * mu;
  const double C = 2.0 * ((((b[1] * BG_W(2, 2) - b[2] * BG_W(1, 2)) * mu * mu) - b[0] * BG_W(0, 1)) + b[1] * BG_W(0, 0));
  const double D = 2.0 * ((b[0] * (BG_W(1, 1) - BG_W(2, 2)) - b[1] * BG_W(0, 1)) + b[2] * BG_W(0, 2)) * mu;
  const double E = -6.0 * (b[0] * BG_W(1, 2) - b[1] * BG_W(0, 2)) * mu;
  double coeffs[5] = {A + B, C - D, E, C + D, B - A};
  double roots[4];
  const int nRoots = real_roots_degenerate<Warp>(coeffs, 4, roots, kAllRoots, sa);
  for (int i = 0; i < nRoots; ++i) {
    const double t = roots[i];
    const double den = 1.0 + t * t;
    const double CT = (1.0 - t * t) / den;
    const double ST = (2.0 * t) / den;
    const double dir[3] = {1.0, mu * CT, mu * ST};
    const double v0[3] = {mu * BG_W(0, 1) + CT * BG_W(0, 0), mu * BG_W(1, 1) + CT * BG_W(1, 0), mu * BG_W(2, 1) + CT * BG_W(2, 0)};
    const double v1[3] = {mu * BG_W(0, 2) + ST * BG_W(0, 0), mu * BG_W(1, 2) + ST * BG_W(1, 0), mu * BG_W(2, 2) + ST * BG_W(2, 0)};
    const double den0 = dot3(v0, dir);
    const double den1 = dot3(v1, dir);
    double rN;
    if (fabs(den0) > fabs(den1)) {
      if (is_zero(den0)) continue;
      rN = -(CT * b[0] + b[1] * mu) / den0;
    } else {
      if (is_zero(den1)) continue;
      rN = -(ST * b[0] + b[2] * mu) / den1;
    }
    if (rN <= 0) continue;
    r[0] = rN * dir[0];
    r[1] = rN * dir[1];
    r[2] = rN * dir[2];
    const double col0[3] = {BG_W(0, 0), BG_W(1, 0), BG_W(2, 0)};
    const double uN = dot3(col0, r) + b[0];
    if (uN > 0) return true;
  }
  return false;
#undef BG_W
}

enum { kPureNewton = 0, kPureEnumerative = 1, kHybrid = 2, kRevHybrid = 3 };

// LocalSOCSolver<3, double, DeSaxce, Strat>::solve (mu < 0: full-pivoting LU solve of A x = -b)
// Warp: called by a whole converged warp with identical arguments (every lane computes the same values; the
// companion-matrix eigenvalues use the warp's shared scratch sa, 16 doubles).
template <bool Warp = false>
BG_HD double local_solve(bool desaxce, int strat, const double* A, const double* b, double* x, double mu, double tol,
                         double scaling, double* sa = nullptr) {
  if (mu < 0) {
    SmallLU<3> lu;
    lu.compute(A);
    const double mb[3] = {-b[0], -b[1], -b[2]};
    lu.solve(mb, x);
    double ax[3];
    matvec3(A, x, ax);
    const double res[3] = {ax[0] + b[0], ax[1] + b[1], ax[2] + b[2]};
    return sq3(res);
  }
  LocalFB fb{desaxce, mu, scaling, A, b};
  if (strat == kPureNewton) return newton_solve(fb, tol, x);
  const double thr = desaxce ? 0.0 : mu * norm2(b[1], b[2]);
  if (b[0] >= thr) {
    x[0] = x[1] = x[2] = 0.0;
    return 0.0;
  }
  if (is_zero(mu)) {
    if (A[0] < kEps) {
      x[0] = x[1] = x[2] = 0.0;
      return b[0] * b[0];
    }
    x[1] = x[2] = 0.0;
    x[0] = (-b[0]) / A[0];
    return 0.0;
  }
  double res = 0.0;
  if (strat == kHybrid) {
    res = newton_solve(fb, tol, x);
    if (res < tol) return res;
  }
  const double x0[3] = {x[0], x[1], x[2]};
  {
    SmallLU<3> lu;
    lu.compute(A);
    const double mb[3] = {-b[0], -b[1], -b[2]};
    lu.solve(mb, x);
  }
  if (mu * x[0] >= norm2(x[1], x[2])) return 0.0;
  const bool ok = desaxce ? analytic_coulomb<Warp>(A, b, x, mu, sa) : analytic_soc<Warp>(A, b, x, mu, sa);
  if (!ok) { x[0] = x0[0]; x[1] = x0[1]; x[2] = x0[2]; }
  if (strat == kRevHybrid) {
    res = newton_solve(fb, tol, x);
  } else if (strat == kHybrid) {
    const double refined = newton_solve(fb, tol, x);
    if (refined <= res) return refined;
    x[0] = x0[0]; x[1] = x0[1]; x[2] = x0[2];
  }
  return res;
}

template <bool Warp = false>
BG_HD bool law_solve_local(bool desaxce, int strat, const double* A, const double* b, double* x, double mu,
                           double scaling, double* sa = nullptr) {
  return kLocalTol > local_solve<Warp>(desaxce, strat, A, b, x, mu, kLocalTol, scaling, sa);
}

BG_HD double nesterov_inertia(double& theta, double q) {
  const double theta_prev = theta;
  const double theta_p2 = theta_prev * theta_prev;
  const double bb = theta_p2 - q;
  const double delta = sqrt(bb * bb + 4.0 * theta_p2);
  theta = 0.5 * (delta - bb);
  return (theta_prev - theta_p2) / (theta_p2 + theta);
}

// Smallest eigenvalue of a symmetric 3x3 block by cyclic Jacobi rotations (used for
// GaussSeidelBase::setAutoRegularization; the reference takes the real parts of the general eigenvalues,
// which coincide for the symmetric diagonal blocks of W up to rounding).
BG_HD double min_eigen_symmetric3(const double* D) {
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
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {
          const double akp = a[3 * k + p], akq = a[3 * k + q];
          a[3 * k + p] = c * akp - s * akq;
          a[3 * k + q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = a[3 * p + k], aqk = a[3 * q + k];
          a[3 * p + k] = c * apk - s * aqk;
          a[3 * q + k] = s * apk + c * aqk;
        }
      }
  }
  return dmin(dmin(a[0], a[4]), a[8]);
}

}  // namespace bogus_gpu
