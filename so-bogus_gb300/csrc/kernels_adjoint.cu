// Adjoint of the SOC friction solve and of the Coulomb friction solve (no counterpart in the reference, which has
// no differentiation).
//
// r solves min 1/2 r^T W r + b^T r over r_i in K_mu_i (SOCLaw<3>, the problem ProjectedGradient solves with
// staticProblem), i.e. the fixed point r = P(x), x = r - A (W r + b) for any positive diagonal step A (here
// alpha_i = 1 / scaling_i, the diagonal scalings of ConstrainedSolverBase; the gradient does not depend on the
// choice). With J = dP/dx(x) (block diagonal, symmetric) the adjoint system is (I - J + W A J) lam = g
// (g = dL/dr). Per contact
// J = V diag(theta) V^T in closed form:
//   interior (|x_T| <= mu x_N):      V = I, theta = (1, 1, 1)
//   polar (mu |x_T| <= -x_N, mu < 0): theta = (0, 0, 0)
//   boundary, c = 1 / (1 + mu^2), u = x_T / |x_T|, p_N = c (x_N + mu |x_T|):
//     v1 = sqrt(c) (1, mu u), theta 1;  v2 = (0, u_perp), theta = mu p_N / |x_T|;  v3 = sqrt(c) (-mu, u), theta 0.
// Writing lam in the V basis, the components with theta = 0 ("masked") decouple and the others, scaled as
// p = alpha theta lam_hat, solve the symmetric positive definite system
//   S p = D p + M V^T W V M p = M V^T g,   D = (1 / theta - 1) / alpha,  M = the unmasked components,
// by conjugate gradients (one pass over W per iteration) preconditioned with the inverse of S's 3 x 3
// diagonal blocks diag(D_i) + V_i^T W_ii V_i (D grows without bound as theta -> 0 near a regime change, which
// leaves plain CG unable to converge). Then
//   dL/db = s = -V M p,   lam_hat (masked) = v_k^T (g + W s),   lam_hat (unmasked) = p_k / (alpha theta_k),
//   dL/dmu_i = K_i^T V_i lam_hat_i with K = dP/dmu(x).
// A persistent cooperative kernel runs the setup, the CG iterations and the final pass; reductions use the
// canonical order of the solver kernels, waits are bounded (grid_barrier).
#include "internal.h"
#include "soc_device.cuh"
#include "spmv_chunk.cuh"

namespace bogus_gpu {

namespace {

__device__ __forceinline__ void ld3(const double* p, int i, double* v) {
  v[0] = ldcg(p + 3 * i);
  v[1] = ldcg(p + 3 * i + 1);
  v[2] = ldcg(p + 3 * i + 2);
}
__device__ __forceinline__ void st3(double* p, int i, const double* v) {
  p[3 * i] = v[0];
  p[3 * i + 1] = v[1];
  p[3 * i + 2] = v[2];
}

// Closed-form eigenbasis of the projection Jacobian at x: V (row-major 3x3, columns v1 v2 v3), D (negative
// for a masked component) and K = dP/dmu.
__device__ void projection_basis(double mu, const double* x, double alpha, double* V, double* D, double* K) {
  const double xn = x[0];
  const double t = sqrt(x[1] * x[1] + x[2] * x[2]);
#pragma unroll
  for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? 1.0 : 0.0;
  K[0] = K[1] = K[2] = 0.0;
  if (mu < 0.0 || mu * t <= -xn) {  // polar cone: J = 0
    D[0] = D[1] = D[2] = -1.0;
    return;
  }
  if (t <= mu * xn) {  // interior: J = I
    D[0] = D[1] = D[2] = 0.0;
    return;
  }
  const double c = 1.0 / (1.0 + mu * mu);
  const double sc = sqrt(c);
  const double u1 = x[1] / t, u2 = x[2] / t;
  const double pn = (xn + mu * t) * c;
  // columns: v1 = sc (1, mu u), v2 = (0, -u2, u1), v3 = sc (-mu, u)
  V[0] = sc;          V[1] = 0.0;  V[2] = -mu * sc;
  V[3] = sc * mu * u1; V[4] = -u2; V[5] = sc * u1;
  V[6] = sc * mu * u2; V[7] = u1;  V[8] = sc * u2;
  const double rho = mu * pn / t;
  D[0] = 0.0;
  D[1] = rho > 0.0 ? (1.0 / rho - 1.0) / alpha : -1.0;
  D[2] = -1.0;
  const double dpn = t * c - 2.0 * mu * (xn + mu * t) * c * c;
  const double kt = pn + mu * dpn;
  K[0] = dpn;
  K[1] = kt * u1;
  K[2] = kt * u2;
}

// Inverse of the SPD block diag(D) + V^T Wii V restricted to the unmasked components (identity on the
// masked ones), by Cholesky factorisation.
__device__ void precond_block(const double* V, const double* D, const double* Wii, double* Pinv) {
  double A[9];
  double T[9];  // Wii V
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) T[3 * r + k] = Wii[3 * r] * V[k] + Wii[3 * r + 1] * V[3 + k] + Wii[3 * r + 2] * V[6 + k];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double v = V[j] * T[k] + V[3 + j] * T[3 + k] + V[6 + j] * T[6 + k];
      const bool mj = D[j] < 0.0, mk = D[k] < 0.0;
      A[3 * j + k] = (mj || mk) ? (j == k ? 1.0 : 0.0) : v + (j == k ? D[j] : 0.0);
    }
  // symmetrise (V^T Wii V is symmetric up to rounding), then Cholesky A = L L^T
  const double a10 = 0.5 * (A[3] + A[1]), a20 = 0.5 * (A[6] + A[2]), a21 = 0.5 * (A[7] + A[5]);
  const double l00 = sqrt(fmax(A[0], 1e-300));
  const double l10 = a10 / l00, l20 = a20 / l00;
  const double l11 = sqrt(fmax(A[4] - l10 * l10, 1e-300));
  const double l21 = (a21 - l20 * l10) / l11;
  const double l22 = sqrt(fmax(A[8] - l20 * l20 - l21 * l21, 1e-300));
  // L^-1 (lower triangular)
  const double i00 = 1.0 / l00, i11 = 1.0 / l11, i22 = 1.0 / l22;
  const double i10 = -l10 * i00 * i11;
  const double i21 = -l21 * i11 * i22;
  const double i20 = -(l20 * i00 + l21 * i10) * i22;
  // A^-1 = L^-T L^-1
  Pinv[0] = i00 * i00 + i10 * i10 + i20 * i20;
  Pinv[1] = i10 * i11 + i20 * i21;
  Pinv[2] = i20 * i22;
  Pinv[4] = i11 * i11 + i21 * i21;
  Pinv[5] = i21 * i22;
  Pinv[8] = i22 * i22;
  Pinv[3] = Pinv[1];
  Pinv[6] = Pinv[2];
  Pinv[7] = Pinv[5];
}

__device__ __forceinline__ void mat3_apply(const double* M, const double* x, double* y) {
#pragma unroll
  for (int r = 0; r < 3; ++r) y[r] = M[3 * r] * x[0] + M[3 * r + 1] * x[1] + M[3 * r + 2] * x[2];
}

// y = V (m o p)
__device__ __forceinline__ void basis_apply(const double* V, const double* D, const double* p, double* y) {
  double q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) q[k] = D[k] < 0.0 ? 0.0 : p[k];
#pragma unroll
  for (int r = 0; r < 3; ++r) y[r] = V[3 * r] * q[0] + V[3 * r + 1] * q[1] + V[3 * r + 2] * q[2];
}
// p = m o (V^T y)
__device__ __forceinline__ void basis_apply_t(const double* V, const double* D, const double* y, double* p) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double v = V[k] * y[0] + V[3 + k] * y[1] + V[6 + k] * y[2];
    p[k] = D[k] < 0.0 ? 0.0 : v;
  }
}

// Warps take chunks from ticket counters (Tickets: dynamic balance; the chunk sums stay in chunk order).
struct AdjCtx {
  const AdjArgs& a;
  double* smem8;
  Tickets tk{a.tickets};
  __device__ int next() { return tk.next(); }
  __device__ bool sync() {
    const bool ok = grid_barrier(a.gb, [&] { tk.clear(); });
    ++tk.phase;
    return ok;
  }
  __device__ bool sync_reduce(int K) {
    const bool ok = grid_barrier_combine(a.gb, a.combine_count, a.csum, (size_t)a.nchunks, a.nchunks, a.nchunks, K,
                                         0u, a.stripes, a.scal, [&] { tk.clear(); });
    ++tk.phase;
    return ok;
  }
};

__global__ void __launch_bounds__(256) k_adjoint(AdjArgs a) {
  __shared__ double smem8[8];
  __shared__ ChunkScratch cs[8];
  AdjCtx ctx{a, smem8};
  ChunkScratch& sh = cs[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int C = a.nchunks;
  const bool writer = blockIdx.x == 0 && threadIdx.x == 0;
  auto put = [&](int q, int c, double v) {
    v = warp_sum_butterfly(v);
    if (lane == 0) a.csum[q * C + c] = v;
  };
  auto product = [&](int c, const double* src, double* acc) {
    spmv_chunk<1>(a.rowptr, InterleavedBlocks<double>{a.icol, a.ival, a.slot0}, a.n, c, sh,
                  [&](int j, double* x) { ld3(src, j, x); }, acc);
  };

  // setup: x = r - alpha (W r + b), the basis, the preconditioner, rhs c = m o V^T g; p = 0, res = c,
  // z = Pinv c, dir = z, Y = V (m o dir)
  for (int c = ctx.next(); c < C; c = ctx.next()) {
    const int i = 32 * c + lane;
    double acc[3] = {0.0, 0.0, 0.0};
    product(c, a.r, acc);
    double rr = 0.0, rz = 0.0;
    if (i < a.n) {
      double r[3], x[3], V[9], D[3], K[3], g[3], cv[3], y[3], Wii[9], Pinv[9], z[3];
      ld3(a.r, i, r);
      const double al = 1.0 / __ldg(a.scaling + i);
      for (int k = 0; k < 3; ++k) x[k] = r[k] - al * (acc[k] + __ldg(a.b + 3 * i + k));
      projection_basis(__ldg(a.mu + i), x, al, V, D, K);
      const int dk = __ldg(a.diag + i);
      for (int k = 0; k < 9; ++k) Wii[k] = dk >= 0 ? __ldg(a.val + 9 * (size_t)dk + k) : 0.0;
      precond_block(V, D, Wii, Pinv);
      for (int k = 0; k < 9; ++k) {
        a.V[9 * (size_t)i + k] = V[k];
        a.Pc[9 * (size_t)i + k] = Pinv[k];
      }
      st3(a.D, i, D);
      st3(a.K, i, K);
      ld3(a.g, i, g);
      basis_apply_t(V, D, g, cv);
      mat3_apply(Pinv, cv, z);
      const double zero[3] = {0.0, 0.0, 0.0};
      st3(a.P, i, zero);
      st3(a.R, i, cv);
      st3(a.Dir, i, z);
      basis_apply(V, D, z, y);
      st3(a.Y, i, y);
      rr = cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2];
      rz = cv[0] * z[0] + cv[1] * z[1] + cv[2] * z[2];
    }
    put(0, c, rr);
    put(1, c, rz);
  }
  if (!ctx.sync_reduce(2)) return;
  const double rr0 = ldcg(a.scal);
  double rr = rr0;
  double rz = ldcg(a.scal + 1);
  unsigned it = 0;
  const double stop = a.tol * a.tol * rr0;
  for (; it < a.max_iters; ++it) {
    if (!(rr > stop)) break;
    // q = D o dir + m o V^T W Y, dir . q
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      double acc[3] = {0.0, 0.0, 0.0};
      product(c, a.Y, acc);
      double dq = 0.0;
      if (i < a.n) {
        double V[9], D[3], d[3], t[3], q[3];
        for (int k = 0; k < 9; ++k) V[k] = ldcg(a.V + 9 * (size_t)i + k);
        ld3(a.D, i, D);
        ld3(a.Dir, i, d);
        basis_apply_t(V, D, acc, t);
        for (int k = 0; k < 3; ++k) q[k] = (D[k] < 0.0 ? 0.0 : D[k] * d[k]) + t[k];
        st3(a.Q, i, q);
        dq = d[0] * q[0] + d[1] * q[1] + d[2] * q[2];
      }
      put(0, c, dq);
    }
    if (!ctx.sync_reduce(1)) return;
    const double dq = ldcg(a.scal);
    if (!(dq > 0.0)) break;  // S is positive definite on the unmasked components; guards exact convergence
    const double step = rz / dq;
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      double v = 0.0, w = 0.0;
      if (i < a.n) {
        double p[3], res[3], d[3], q[3], Pinv[9], z[3];
        ld3(a.P, i, p);
        ld3(a.R, i, res);
        ld3(a.Dir, i, d);
        ld3(a.Q, i, q);
        for (int k = 0; k < 9; ++k) Pinv[k] = ldcg(a.Pc + 9 * (size_t)i + k);
        for (int k = 0; k < 3; ++k) {
          p[k] = fma(step, d[k], p[k]);
          res[k] = fma(-step, q[k], res[k]);
        }
        mat3_apply(Pinv, res, z);
        st3(a.P, i, p);
        st3(a.R, i, res);
        st3(a.Z, i, z);
        v = res[0] * res[0] + res[1] * res[1] + res[2] * res[2];
        w = res[0] * z[0] + res[1] * z[1] + res[2] * z[2];
      }
      put(0, c, v);
      put(1, c, w);
    }
    if (!ctx.sync_reduce(2)) return;
    rr = ldcg(a.scal);
    const double rz_new = ldcg(a.scal + 1);
    const double beta = rz_new / rz;
    rz = rz_new;
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      if (i < a.n) {
        double V[9], D[3], z[3], d[3], y[3];
        for (int k = 0; k < 9; ++k) V[k] = ldcg(a.V + 9 * (size_t)i + k);
        ld3(a.D, i, D);
        ld3(a.Z, i, z);
        ld3(a.Dir, i, d);
        for (int k = 0; k < 3; ++k) d[k] = fma(beta, d[k], z[k]);
        st3(a.Dir, i, d);
        basis_apply(V, D, d, y);
        st3(a.Y, i, y);
      }
    }
    if (!ctx.sync()) return;
  }
  // s = dL/db = -V (m o p)
  for (int c = ctx.next(); c < C; c = ctx.next()) {
    const int i = 32 * c + lane;
    if (i < a.n) {
      double V[9], D[3], p[3], y[3];
      for (int k = 0; k < 9; ++k) V[k] = ldcg(a.V + 9 * (size_t)i + k);
      ld3(a.D, i, D);
      ld3(a.P, i, p);
      basis_apply(V, D, p, y);
      const double s[3] = {-y[0], -y[1], -y[2]};
      st3(a.S, i, s);
    }
  }
  if (!ctx.sync()) return;
  // lam_hat and dL/dmu = K^T V lam_hat
  for (int c = ctx.next(); c < C; c = ctx.next()) {
    const int i = 32 * c + lane;
    double acc[3] = {0.0, 0.0, 0.0};
    product(c, a.S, acc);
    if (i < a.n) {
      double V[9], D[3], p[3], g[3], K[3], e[3], lh[3];
      for (int k = 0; k < 9; ++k) V[k] = ldcg(a.V + 9 * (size_t)i + k);
      ld3(a.D, i, D);
      ld3(a.P, i, p);
      ld3(a.g, i, g);
      ld3(a.K, i, K);
      const double al = 1.0 / __ldg(a.scaling + i);
      for (int k = 0; k < 3; ++k) e[k] = g[k] + acc[k];
      for (int k = 0; k < 3; ++k) {
        if (D[k] < 0.0) lh[k] = V[k] * e[0] + V[3 + k] * e[1] + V[6 + k] * e[2];
        else lh[k] = p[k] * (1.0 + al * D[k]) / al;  // p / (alpha theta), theta = 1 / (1 + alpha D)
      }
      double dm = 0.0;
      for (int r2 = 0; r2 < 3; ++r2) dm += K[r2] * (V[3 * r2] * lh[0] + V[3 * r2 + 1] * lh[1] + V[3 * r2 + 2] * lh[2]);
      a.dmu[i] = dm;
    }
  }
  if (writer) {
    a.out->iters = it;
    a.out->rel_res = rr0 > 0.0 ? sqrt(rr / rr0) : 0.0;
  }
}

// ---- Coulomb law ----------------------------------------------------------------------------------------
// With the De Saxce change of variable the fixed point is r = P(x), x = r - A (u + s(u)), u = W r + b,
// s(u) = (mu |u_T|, 0, 0) (SOCLaw::dualityCOV). Its derivative ds/du = e_N tau^T with tau = (0, mu u_T / |u_T|)
// (zero where u_T = 0) makes the linearised map non-symmetric: with T = I + e_N tau^T the adjoint system is
// (I - J + W T^T A J) lam = g. In the basis of J as above, the unmasked components of p = alpha theta lam_hat solve
//   (D + M V^T W T^T V M) p = M V^T g,
// by bi-conjugate gradients stabilised (two passes over W per iteration), right-preconditioned with the inverse
// of the 3 x 3 diagonal blocks diag(D_i) + V_i^T W_ii T_i^T V_i. Then
//   dL/db = s = -T^T V M p,   lam_hat (masked) = v_k^T (g + W s),   lam_hat (unmasked) = p_k / (alpha theta_k),
//   dL/dmu_i = K_i^T V_i lam_hat_i - |u_T,i| (V_i M p_i)_N.

// y = T^T V (m o p), T^T y = y + tau y_N (tc = (|u_T|, tau_1, tau_2))
__device__ __forceinline__ void coulomb_apply(const double* V, const double* D, const double* tc, const double* p,
                                              double* y) {
  basis_apply(V, D, p, y);
  y[1] = fma(tc[1], y[0], y[1]);
  y[2] = fma(tc[2], y[0], y[2]);
}

// Inverse of diag(D) + V^T Wii T^T V on the unmasked components (identity on the masked ones), by Gauss-Jordan
// elimination with partial pivoting; a zero pivot leaves that component unpreconditioned.
__device__ void precond_block_coulomb(const double* V, const double* D, const double* tc, const double* Wii,
                                      double* Pinv) {
  double TV[9];  // T^T V, column k = T^T v_k
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    TV[k] = V[k];
    TV[3 + k] = fma(tc[1], V[k], V[3 + k]);
    TV[6 + k] = fma(tc[2], V[k], V[6 + k]);
  }
  double WT[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) WT[3 * r + k] = Wii[3 * r] * TV[k] + Wii[3 * r + 1] * TV[3 + k] + Wii[3 * r + 2] * TV[6 + k];
  double A[3][6];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double v = V[j] * WT[k] + V[3 + j] * WT[3 + k] + V[6 + j] * WT[6 + k];
      const bool mj = D[j] < 0.0, mk = D[k] < 0.0;
      A[j][k] = (mj || mk) ? (j == k ? 1.0 : 0.0) : v + (j == k ? D[j] : 0.0);
      A[j][3 + k] = j == k ? 1.0 : 0.0;
    }
  for (int c = 0; c < 3; ++c) {
    int piv = c;
    for (int r = c + 1; r < 3; ++r)
      if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
    if (!(fabs(A[piv][c]) > 0.0)) continue;
    if (piv != c)
      for (int k = 0; k < 6; ++k) {
        const double t = A[c][k];
        A[c][k] = A[piv][k];
        A[piv][k] = t;
      }
    const double inv = 1.0 / A[c][c];
    for (int k = 0; k < 6; ++k) A[c][k] *= inv;
    for (int r = 0; r < 3; ++r) {
      if (r == c) continue;
      const double f = A[r][c];
      if (f != 0.0)
        for (int k = 0; k < 6; ++k) A[r][k] = fma(-f, A[c][k], A[r][k]);
    }
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) Pinv[3 * j + k] = A[j][3 + k];
}

__global__ void __launch_bounds__(256) k_adjoint_coulomb(AdjArgs a) {
  __shared__ double smem8[8];
  __shared__ ChunkScratch cs[8];
  AdjCtx ctx{a, smem8};
  ChunkScratch& sh = cs[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int C = a.nchunks;
  const bool writer = blockIdx.x == 0 && threadIdx.x == 0;
  auto put = [&](int q, int c, double v) {
    v = warp_sum_butterfly(v);
    if (lane == 0) a.csum[q * C + c] = v;
  };
  auto product = [&](int c, const double* src, double* acc) {
    spmv_chunk<1>(a.rowptr, InterleavedBlocks<double>{a.icol, a.ival, a.slot0}, a.n, c, sh,
                  [&](int j, double* x) { ld3(src, j, x); }, acc);
  };
  auto load_basis = [&](int i, double* V, double* D, double* tc) {
    for (int k = 0; k < 9; ++k) V[k] = ldcg(a.V + 9 * (size_t)i + k);
    ld3(a.D, i, D);
    ld3(a.Tc, i, tc);
  };
  // A q for the current W-operand product: D o q + m o V^T (W Y)
  auto op_tail = [&](int i, const double* acc, const double* q, double* out) {
    double V[9], D[3], tc[3], t[3];
    load_basis(i, V, D, tc);
    basis_apply_t(V, D, acc, t);
    for (int k = 0; k < 3; ++k) out[k] = (D[k] < 0.0 ? 0.0 : D[k] * q[k]) + t[k];
  };
  // setup: u = W r + b, s(u), x = r - alpha (u + s(u)), the basis, tau, the preconditioner; rhs c = m o V^T g;
  // p = 0, residual = shadow = c, direction = v = 0
  for (int c = ctx.next(); c < C; c = ctx.next()) {
    const int i = 32 * c + lane;
    double acc[3] = {0.0, 0.0, 0.0};
    product(c, a.r, acc);
    double rr = 0.0;
    if (i < a.n) {
      double r[3], u[3], x[3], V[9], D[3], K[3], g[3], cv[3], Wii[9], Pinv[9], tc[3];
      ld3(a.r, i, r);
      const double mu = __ldg(a.mu + i);
      const double al = 1.0 / __ldg(a.scaling + i);
      for (int k = 0; k < 3; ++k) u[k] = acc[k] + __ldg(a.b + 3 * i + k);
      const double t = sqrt(u[1] * u[1] + u[2] * u[2]);
      const double sN = mu * t;
      x[0] = r[0] - al * (u[0] + sN);
      x[1] = r[1] - al * u[1];
      x[2] = r[2] - al * u[2];
      tc[0] = t;
      tc[1] = t > 0.0 ? mu * u[1] / t : 0.0;
      tc[2] = t > 0.0 ? mu * u[2] / t : 0.0;
      projection_basis(mu, x, al, V, D, K);
      const int dk = __ldg(a.diag + i);
      for (int k = 0; k < 9; ++k) Wii[k] = dk >= 0 ? __ldg(a.val + 9 * (size_t)dk + k) : 0.0;
      precond_block_coulomb(V, D, tc, Wii, Pinv);
      for (int k = 0; k < 9; ++k) {
        a.V[9 * (size_t)i + k] = V[k];
        a.Pc[9 * (size_t)i + k] = Pinv[k];
      }
      st3(a.D, i, D);
      st3(a.K, i, K);
      st3(a.Tc, i, tc);
      ld3(a.g, i, g);
      basis_apply_t(V, D, g, cv);
      const double zero[3] = {0.0, 0.0, 0.0};
      st3(a.P, i, zero);
      st3(a.R, i, cv);
      st3(a.Rh, i, cv);
      st3(a.Dir, i, zero);
      st3(a.Q, i, zero);
      rr = cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2];
    }
    put(0, c, rr);
  }
  if (!ctx.sync_reduce(1)) return;
  const double rr0 = ldcg(a.scal);
  double rr = rr0, rho_old = 1.0, alpha = 1.0, omega = 1.0, rho = rr0;
  unsigned it = 0;
  const double stop = a.tol * a.tol * rr0;
  for (; it < a.max_iters; ++it) {
    if (!(rr > stop)) break;
    const double beta = (rho / rho_old) * (alpha / omega);
    // direction = r + beta (direction - omega v); ph = Pinv direction; Y = T^T V (m o ph)
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      if (i < a.n) {
        double res[3], d[3], v[3], Pinv[9], ph[3], V[9], D[3], tc[3], y[3];
        ld3(a.R, i, res);
        ld3(a.Dir, i, d);
        ld3(a.Q, i, v);
        for (int k = 0; k < 9; ++k) Pinv[k] = ldcg(a.Pc + 9 * (size_t)i + k);
        for (int k = 0; k < 3; ++k) d[k] = fma(beta, fma(-omega, v[k], d[k]), res[k]);
        mat3_apply(Pinv, d, ph);
        load_basis(i, V, D, tc);
        coulomb_apply(V, D, tc, ph, y);
        st3(a.Dir, i, d);
        st3(a.Ph, i, ph);
        st3(a.Y, i, y);
      }
    }
    if (!ctx.sync()) return;
    // v = A ph; shadow . v
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      double acc[3] = {0.0, 0.0, 0.0};
      product(c, a.Y, acc);
      double hv = 0.0;
      if (i < a.n) {
        double ph[3], v[3], rh[3];
        ld3(a.Ph, i, ph);
        op_tail(i, acc, ph, v);
        st3(a.Q, i, v);
        ld3(a.Rh, i, rh);
        hv = rh[0] * v[0] + rh[1] * v[1] + rh[2] * v[2];
      }
      put(0, c, hv);
    }
    if (!ctx.sync_reduce(1)) return;
    const double hv = ldcg(a.scal);
    if (!(hv != 0.0)) break;  // breakdown (or exact convergence)
    alpha = rho / hv;
    // s = r - alpha v; sh = Pinv s; Y = T^T V (m o sh)
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      if (i < a.n) {
        double res[3], v[3], sv[3], Pinv[9], shv[3], V[9], D[3], tc[3], y[3];
        ld3(a.R, i, res);
        ld3(a.Q, i, v);
        for (int k = 0; k < 3; ++k) sv[k] = fma(-alpha, v[k], res[k]);
        for (int k = 0; k < 9; ++k) Pinv[k] = ldcg(a.Pc + 9 * (size_t)i + k);
        mat3_apply(Pinv, sv, shv);
        load_basis(i, V, D, tc);
        coulomb_apply(V, D, tc, shv, y);
        st3(a.Sv, i, sv);
        st3(a.Sh, i, shv);
        st3(a.Y, i, y);
      }
    }
    if (!ctx.sync()) return;
    // t = A sh; t . s, t . t
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      double acc[3] = {0.0, 0.0, 0.0};
      product(c, a.Y, acc);
      double ts = 0.0, tt = 0.0;
      if (i < a.n) {
        double shv[3], tv[3], sv[3];
        ld3(a.Sh, i, shv);
        op_tail(i, acc, shv, tv);
        st3(a.Tv, i, tv);
        ld3(a.Sv, i, sv);
        ts = tv[0] * sv[0] + tv[1] * sv[1] + tv[2] * sv[2];
        tt = tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2];
      }
      put(0, c, ts);
      put(1, c, tt);
    }
    if (!ctx.sync_reduce(2)) return;
    const double ts = ldcg(a.scal), tt = ldcg(a.scal + 1);
    omega = tt > 0.0 ? ts / tt : 0.0;
    // p += alpha ph + omega sh; r = s - omega t; shadow . r, r . r
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      double hr = 0.0, r2 = 0.0;
      if (i < a.n) {
        double p[3], ph[3], shv[3], sv[3], tv[3], res[3], rh[3];
        ld3(a.P, i, p);
        ld3(a.Ph, i, ph);
        ld3(a.Sh, i, shv);
        ld3(a.Sv, i, sv);
        ld3(a.Tv, i, tv);
        ld3(a.Rh, i, rh);
        for (int k = 0; k < 3; ++k) {
          p[k] = fma(omega, shv[k], fma(alpha, ph[k], p[k]));
          res[k] = fma(-omega, tv[k], sv[k]);
        }
        st3(a.P, i, p);
        st3(a.R, i, res);
        hr = rh[0] * res[0] + rh[1] * res[1] + rh[2] * res[2];
        r2 = res[0] * res[0] + res[1] * res[1] + res[2] * res[2];
      }
      put(0, c, hr);
      put(1, c, r2);
    }
    if (!ctx.sync_reduce(2)) return;
    rho_old = rho;
    rho = ldcg(a.scal);
    rr = ldcg(a.scal + 1);
    if (!(omega != 0.0)) {
      ++it;
      break;
    }
  }
  // s = dL/db = -T^T V (m o p)
  for (int c = ctx.next(); c < C; c = ctx.next()) {
    const int i = 32 * c + lane;
    if (i < a.n) {
      double V[9], D[3], tc[3], p[3], y[3];
      load_basis(i, V, D, tc);
      ld3(a.P, i, p);
      coulomb_apply(V, D, tc, p, y);
      const double s[3] = {-y[0], -y[1], -y[2]};
      st3(a.S, i, s);
    }
  }
  if (!ctx.sync()) return;
  // lam_hat and dL/dmu = K^T V lam_hat - |u_T| (V m o p)_N
  for (int c = ctx.next(); c < C; c = ctx.next()) {
    const int i = 32 * c + lane;
    double acc[3] = {0.0, 0.0, 0.0};
    product(c, a.S, acc);
    if (i < a.n) {
      double V[9], D[3], tc[3], p[3], g[3], K[3], e[3], lh[3], vp[3];
      load_basis(i, V, D, tc);
      ld3(a.P, i, p);
      ld3(a.g, i, g);
      ld3(a.K, i, K);
      const double al = 1.0 / __ldg(a.scaling + i);
      for (int k = 0; k < 3; ++k) e[k] = g[k] + acc[k];
      for (int k = 0; k < 3; ++k) {
        if (D[k] < 0.0) lh[k] = V[k] * e[0] + V[3 + k] * e[1] + V[6 + k] * e[2];
        else lh[k] = p[k] * (1.0 + al * D[k]) / al;  // p / (alpha theta), theta = 1 / (1 + alpha D)
      }
      double dm = 0.0;
      for (int r2 = 0; r2 < 3; ++r2) dm += K[r2] * (V[3 * r2] * lh[0] + V[3 * r2 + 1] * lh[1] + V[3 * r2 + 2] * lh[2]);
      basis_apply(V, D, p, vp);
      a.dmu[i] = dm - tc[0] * vp[0];
    }
  }
  if (writer) {
    a.out->iters = it;
    a.out->rel_res = rr0 > 0.0 ? sqrt(rr / rr0) : 0.0;
  }
}

}  // namespace

cudaError_t launch_adjoint(const AdjArgs& a, int grid, cudaStream_t s) {
  AdjArgs copy = a;
  void* args[] = {&copy};
  return cudaLaunchCooperativeKernel((const void*)k_adjoint, dim3(grid), dim3(256), args, 0, s);
}

cudaError_t launch_adjoint_coulomb(const AdjArgs& a, int grid, cudaStream_t s) {
  AdjArgs copy = a;
  void* args[] = {&copy};
  return cudaLaunchCooperativeKernel((const void*)k_adjoint_coulomb, dim3(grid), dim3(256), args, 0, s);
}

int adjoint_max_grid(int device) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_adjoint, 256, 0) != cudaSuccess) return 0;
  int per_c = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_c, k_adjoint_coulomb, 256, 0) != cudaSuccess) return 0;
  if (per_c < per) per = per_c;
  if (per > 2) per = 2;
  return per * sms;
}

// Sets this file's copy of the device-side wait limit on the current device.
BOGUS_GPU_WAIT_LIMIT_SETTER(set_wait_limit_adjoint)

}  // namespace bogus_gpu
