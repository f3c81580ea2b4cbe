// Persistent primal ADMM / AMA solver: the whole ADMM::solve (Core/BlockSolvers/ADMM.impl.hpp:54-127) with
// QuadraticProxOp::eval (:29-38) in one cooperative launch, as PrimalFrictionProblem::solveWith(ADMM&,
// lambda, v, r) (Interfaces/PrimalFrictionProblem.cpp:61-73) sets it up: law SOCLaw<3, false> on 1 / mu,
// constraint matrix H (contacts x bodies, 3 x d blocks), prox operator M^-1 (the reference passes MInv
// whatever lambda), affine part f, offset w.
//
// Phases of one iteration (ADMM.impl.hpp line numbers):
//   P1 bodies    prox_arg = H^T r (lambda = 0, :85) or x / lambda + H^T (r + gamma (zacc - ut)) (:87-89),
//                x = prox (prox_arg - f) (:91) .............................................. barrier
//   P2 contacts  ut = w + H x (:93), error terms FB(1/mu; ut_i, r_i) and |ut_i - z_i|^2 (:95-98), then
//                P3 on the same contact: z = P(ut - r / gamma) (:102-103) and the r / y / zacc update of
//                both branches (:105-122) ................................................... barrier
//                + reduce: res (:95-98), tolerance test (:100), branch (accelerated when res < res_prev)
// P3 reads only its own contact's values, so it runs in P2's pass; its branch depends on the reduced
// residual, so both outcomes are formed: r into two spare buffers (three rotate; the one the branch picks
// becomes the current r, and a converged solve keeps the r it was tested on), y and zacc of the accelerated
// branch into their buffers in place, while after a plain step they are derived where they are read
// (y_prev = -r / gamma with the current r, zacc = z), the same operations the plain branch would store.
// z_prev is always z (both branches and the setup store the same z in both), so z serves for it.
// Body b's H^T accumulation runs over its contacts in increasing contact index, rows 0..2, one FMA chain
// per dof; contact rows accumulate w, then the slots in body order, dofs 0..d-1; the prox product is an FMA
// chain over the dofs. Sums use the canonical order (32-contact butterflies, 8 stripes), so the GPU's
// iterates and residuals equal the CPU oracle's bit for bit. Waits are bounded (grid_barrier).
#include "internal.h"
#include "soc_device.cuh"

namespace bogus_gpu {

namespace {

constexpr int kMaxDof = 12;

struct AdmmCtx {
  const ADMMArgs& a;
  double* smem8;
  int nchunks;
  Tickets tk{a.tickets};
  __device__ int next() { return tk.next(); }
  __device__ bool sync() {
    const bool ok = grid_barrier(a.gb, [&] { tk.clear(); });
    ++tk.phase;
    return ok;
  }
  __device__ bool sync_reduce2(unsigned maxmask) {
    const bool ok = grid_barrier_combine(a.gb, a.combine_count, a.csum, (size_t)nchunks, nchunks, nchunks, 2, maxmask,
                                         a.stripes, a.scal, [&] { tk.clear(); });
    ++tk.phase;
    return ok;
  }
};

// D > 0: d fixed at compile time (registers); D == 0: runtime d <= kMaxDof.
template <int D>
__device__ __forceinline__ int dofs(const ADMMArgs& a) {
  return D > 0 ? D : a.d;
}

// ut_i = w_i + H_i x (ADMM.impl.hpp:93 via the reference's multiply<false>(x, ut, 1, 1) after ut = w)
template <int D>
__device__ __forceinline__ void contact_velocity(const ADMMArgs& a, int i, double* ut) {
  const int d = dofs<D>(a);
  const size_t hs = 3 * (size_t)d;
#pragma unroll
  for (int r = 0; r < 3; ++r) ut[r] = __ldg(a.w + 3 * i + r);
  for (int t = 0; t < 2; ++t) {
    const int body = __ldg(a.cb + 2 * i + t);
    if (body < 0) continue;
    const double* Hb = a.H + (2 * (size_t)i + t) * hs;
    const double* xb = a.x + (size_t)body * d;
    double xv[D > 0 ? D : kMaxDof];
#pragma unroll
    for (int m = 0; m < (D > 0 ? D : kMaxDof); ++m)
      if (m < d) xv[m] = ldcg(xb + m);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double acc = ut[r];
#pragma unroll
      for (int m = 0; m < (D > 0 ? D : kMaxDof); ++m)
        if (m < d) acc = fma(__ldg(Hb + r * d + m), xv[m], acc);
      ut[r] = acc;
    }
  }
}

__device__ __forceinline__ void load3(const double* p, int i, double* v) {
  v[0] = ldcg(p + 3 * i);
  v[1] = ldcg(p + 3 * i + 1);
  v[2] = ldcg(p + 3 * i + 2);
}
__device__ __forceinline__ void store3(double* p, int i, const double* v) {
  p[3 * i] = v[0];
  p[3 * i + 1] = v[1];
  p[3 * i + 2] = v[2];
}

template <int D>
__device__ void admm_body(const ADMMArgs& a, AdmmCtx& ctx) {
  constexpr int DM = D > 0 ? D : kMaxDof;
  constexpr bool kPair = D > 0 && D % 2 == 0;
  const int d = dofs<D>(a);
  const int lane = threadIdx.x & 31;
  const int C = ctx.nchunks;
  const int CB = (a.nbodies + 31) / 32;
  const double gamma = a.gamma;
  const double inv_gamma = 1. / gamma;
  const bool with_lambda = !(a.lambda < kEps);
  const double il = with_lambda ? 1. / a.lambda : 0.0;
  const bool writer = blockIdx.x == 0 && threadIdx.x == 0;
  auto put = [&](int q, int c, double v, bool is_max) {
    v = is_max ? warp_max_butterfly(v) : warp_sum_butterfly(v);
    if (lane == 0) a.csum[q * C + c] = v;
  };

  // Setup (:64-77): ut = w + H x, z = P(ut - r / gamma), y_prev = -r / gamma, zacc = z_prev = z (the last two
  // derived: plain = true)
  for (int c = ctx.next(); c < C; c = ctx.next()) {
    const int i = 32 * c + lane;
    if (i < a.n) {
      const double im = 1. / __ldg(a.mu + i);
      a.inv_mu[i] = im;
      double ut[3], r[3], z[3];
      contact_velocity<D>(a, i, ut);
      load3(a.r, i, r);
      for (int k = 0; k < 3; ++k) z[k] = ut[k] - inv_gamma * r[k];
      project_cone(im, z);
      store3(a.ut, i, ut);
      store3(a.z, i, z);
    }
  }
  if (!ctx.sync()) return;

  double* rb[3] = {a.r, a.r_spare[0], a.r_spare[1]};
  int cur = 0;
  bool plain = true;  // y_prev = -r / gamma and zacc = z (the setup, or the last update took the plain branch)
  double theta_prev = 1., res_prev = -1., res = -1.;
  unsigned it = 0;
  for (it = 0; it < a.max_iters; ++it) {
    const double* rc = rb[cur];
    // P1: x = prox(prox_arg) per body (lane order a.border: bodies of similar contact counts share a warp).
    // Even compile-time d: a lane pair per body, each lane the FMA chains of half the dofs (16 bodies per warp,
    // twice the chunks to spread over the warps), the halves exchanged exactly for the prox product.
    if (kPair) {
      constexpr int H2 = kPair ? D / 2 : 1;
      const int half = lane & 1;
      const int CB2 = (a.nbodies + 15) / 16;
      for (int c = ctx.next(); c < CB2; c = ctx.next()) {
        const int slot = 16 * c + (lane >> 1);
        const bool on = slot < a.nbodies;
        const int b = on ? (a.border ? __ldg(a.border + slot) : slot) : 0;
        const int q0 = half * H2;
        double acc[H2];
#pragma unroll
        for (int k = 0; k < H2; ++k) acc[k] = (on && with_lambda) ? il * ldcg(a.x + (size_t)b * D + q0 + k) : 0.0;
        const int e0 = on ? __ldg(a.bptr + b) : 0, e1 = on ? __ldg(a.bptr + b + 1) : 0;
        // the incidence indices two steps ahead, this lane's H columns and r one step ahead of the accumulation
        int ent1 = e0 < e1 ? __ldg(a.bent + e0) : 0;
        int ent2 = e0 + 1 < e1 ? __ldg(a.bent + e0 + 1) : 0;
        double Hn[3 * H2], rn[3] = {0.0, 0.0, 0.0};
        auto load_inc = [&](int ent, double* Hv, double* rv) {
          const double* Hb = a.H + (size_t)ent * 3 * D + q0;
#pragma unroll
          for (int rr = 0; rr < 3; ++rr)
#pragma unroll
            for (int k = 0; k < H2; ++k) Hv[rr * H2 + k] = __ldg(Hb + rr * D + k);
          load3(rc, ent >> 1, rv);
        };
        if (e0 < e1) load_inc(ent1, Hn, rn);
        for (int e = e0; e < e1; ++e) {
          const int ent = ent1;
          ent1 = ent2;
          ent2 = e + 2 < e1 ? __ldg(a.bent + e + 2) : 0;
          double Hc[3 * H2], rv[3] = {rn[0], rn[1], rn[2]};
#pragma unroll
          for (int k = 0; k < 3 * H2; ++k) Hc[k] = Hn[k];
          if (e + 1 < e1) load_inc(ent1, Hn, rn);
          if (with_lambda) {
            const int i = ent >> 1;
            double za[3], ut[3];
            load3(plain ? a.z : a.zacc, i, za);
            load3(a.ut, i, ut);
            for (int k = 0; k < 3; ++k) rv[k] = fma(gamma, za[k] - ut[k], rv[k]);
          }
#pragma unroll
          for (int k = 0; k < H2; ++k) {
            double s = acc[k];
#pragma unroll
            for (int rr = 0; rr < 3; ++rr) s = fma(Hc[rr * H2 + k], rv[rr], s);
            acc[k] = s;
          }
        }
        // QuadraticProxOp::eval: res = prox (rhs - f)
        if (on && a.f) {
#pragma unroll
          for (int k = 0; k < H2; ++k) acc[k] = acc[k] - __ldg(a.f + (size_t)b * D + q0 + k);
        }
        double full[kPair ? D : 1];
#pragma unroll
        for (int k = 0; k < H2; ++k) {
          const double other = __shfl_xor_sync(0xffffffffu, acc[k], 1);
          full[k] = half ? other : acc[k];
          full[H2 + k] = half ? acc[k] : other;
        }
        if (on) {
          const double* P = a.prox + (size_t)b * D * D;
#pragma unroll
          for (int k = 0; k < H2; ++k) {
            const int m = q0 + k;
            double sum = 0.0;
#pragma unroll
            for (int q = 0; q < D; ++q) sum = fma(__ldg(P + m * D + q), full[q], sum);
            a.x[(size_t)b * D + m] = sum;
          }
        }
      }
    } else {
      for (int c = ctx.next(); c < CB; c = ctx.next()) {
        const int slot = 32 * c + lane;
        if (slot < a.nbodies) {
          const int b = a.border ? __ldg(a.border + slot) : slot;
          double acc[DM];
          const double* xb = a.x + (size_t)b * d;
  #pragma unroll
          for (int q = 0; q < DM; ++q)
            if (q < d) acc[q] = with_lambda ? il * ldcg(xb + q) : 0.0;
          const int e0 = __ldg(a.bptr + b), e1 = __ldg(a.bptr + b + 1);
          // Loads run ahead of the accumulation (its order is unchanged): the incidence indices two steps
          // ahead and, for a compile-time d, the H rows and r of the next incidence, so that no step waits on
          // the dependent index -> H / r load chain.
          constexpr bool kPre = D > 0;
          int ent1 = e0 < e1 ? __ldg(a.bent + e0) : 0;
          int ent2 = e0 + 1 < e1 ? __ldg(a.bent + e0 + 1) : 0;
          double Hn[kPre ? 3 * DM : 1], rn[3] = {0.0, 0.0, 0.0};
          if (kPre && e0 < e1) {
            const double* Hb = a.H + (size_t)ent1 * 3 * DM;
  #pragma unroll
            for (int k = 0; k < (kPre ? 3 * DM : 1); ++k) Hn[k] = __ldg(Hb + k);
            load3(rc, ent1 >> 1, rn);
          }
          for (int e = e0; e < e1; ++e) {
            const int ent = ent1;
            ent1 = ent2;
            ent2 = e + 2 < e1 ? __ldg(a.bent + e + 2) : 0;
            const int i = ent >> 1;
            double Hc[kPre ? 3 * DM : 1];
            double rv[3];
            if (kPre) {
  #pragma unroll
              for (int k = 0; k < (kPre ? 3 * DM : 1); ++k) Hc[k] = Hn[k];
              rv[0] = rn[0]; rv[1] = rn[1]; rv[2] = rn[2];
              if (e + 1 < e1) {
                const double* Hb = a.H + (size_t)ent1 * 3 * DM;
  #pragma unroll
                for (int k = 0; k < (kPre ? 3 * DM : 1); ++k) Hn[k] = __ldg(Hb + k);
                load3(rc, ent1 >> 1, rn);
              }
            } else {
              load3(rc, i, rv);
            }
            if (with_lambda) {
              double za[3], ut[3];
              load3(plain ? a.z : a.zacc, i, za);
              load3(a.ut, i, ut);
              for (int k = 0; k < 3; ++k) rv[k] = fma(gamma, za[k] - ut[k], rv[k]);
            }
            const double* Hb = a.H + (size_t)ent * 3 * d;
  #pragma unroll
            for (int q = 0; q < DM; ++q) {
              if (q < d) {
                double s = acc[q];
                for (int rr = 0; rr < 3; ++rr) s = fma(kPre ? Hc[rr * DM + q] : __ldg(Hb + rr * d + q), rv[rr], s);
                acc[q] = s;
              }
            }
          }
          // QuadraticProxOp::eval: res = prox (rhs - f)
          if (a.f) {
  #pragma unroll
            for (int q = 0; q < DM; ++q)
              if (q < d) acc[q] = acc[q] - __ldg(a.f + (size_t)b * d + q);
          }
          const double* P = a.prox + (size_t)b * d * d;
          double xn[DM];
  #pragma unroll
          for (int m = 0; m < DM; ++m) {
            if (m < d) {
              double s = 0.0;
  #pragma unroll
              for (int q = 0; q < DM; ++q)
                if (q < d) s = fma(__ldg(P + m * d + q), acc[q], s);
              xn[m] = s;
            }
          }
          double* xw = a.x + (size_t)b * d;
  #pragma unroll
          for (int m = 0; m < DM; ++m)
            if (m < d) xw[m] = xn[m];
        }
      }
    }
    if (!ctx.sync()) return;

    // P2 + P3: ut = w + H x, error terms; z and both branches' updates
    double theta_spec = theta_prev;
    const double beta = a.accelerated ? nesterov_inertia(theta_spec, 0.) : 0.0;
    const int ia = (cur + 1) % 3, ip = a.accelerated ? (cur + 2) % 3 : (cur + 1) % 3;
    double* r_acc = rb[ia];
    double* r_plain = rb[ip];
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      double ev = 0.0, gap = 0.0;
      if (i < a.n) {
        double ut[3], r[3], z[3];
        contact_velocity<D>(a, i, ut);
        store3(a.ut, i, ut);
        load3(rc, i, r);
        load3(a.z, i, z);
        const double sc = __ldg(a.scaling + i);
        const double lx[3] = {ut[0] * sc, ut[1] * sc, ut[2] * sc};
        const double im = ldcg(a.inv_mu + i);
        ev = law_eval(false, im, lx, r);
        const double d3[3] = {ut[0] - z[0], ut[1] - z[1], ut[2] - z[2]};
        gap = a.use_inf ? dmax(dmax(fabs(d3[0]), fabs(d3[1])), fabs(d3[2])) : sq3(d3);
        // P3
        double zn[3];
        for (int k = 0; k < 3; ++k) zn[k] = ut[k] - inv_gamma * r[k];
        project_cone(im, zn);
        if (a.accelerated) {
          double yp[3], y[3], rn[3], za[3];
          if (plain) {
            for (int k = 0; k < 3; ++k) yp[k] = -inv_gamma * r[k];
          } else {
            load3(a.yprev, i, yp);
          }
          for (int k = 0; k < 3; ++k) {
            y[k] = (ut[k] - zn[k]) - inv_gamma * r[k];
            rn[k] = -gamma * fma(beta, y[k] - yp[k], y[k]);
            za[k] = fma(beta, zn[k] - z[k], zn[k]);
          }
          store3(r_acc, i, rn);
          store3(a.yprev, i, y);
          store3(a.zacc, i, za);
        }
        double rn[3];
        for (int k = 0; k < 3; ++k) rn[k] = fma(gamma, zn[k] - ut[k], r[k]);
        store3(r_plain, i, rn);
        store3(a.z, i, zn);
      }
      put(0, c, ev, a.use_inf != 0);
      put(1, c, gap, a.use_inf != 0);
    }
    if (!ctx.sync_reduce2(a.use_inf ? 3u : 0u)) return;
    {
      const double e0 = ldcg(a.scal), g0 = ldcg(a.scal + 1);
      res = a.use_inf ? e0 + g0 : e0 / (double)(1 + a.n) + g0 / (double)(1 + 3 * (size_t)a.n);
    }
    if (a.trace && writer) a.trace[it] = res;
    if (res < a.tol) break;
    const bool acc_branch = a.accelerated && res < res_prev;
    if (acc_branch) {
      theta_prev = theta_spec;
      cur = ia;
      plain = false;
    } else {
      theta_prev = 1.;
      cur = ip;
      plain = true;
    }
    res_prev = res;
  }
  // the final r in the caller's buffer (nothing reads the spare buffers after the last barrier)
  if (cur != 0) {
    for (int c = ctx.next(); c < C; c = ctx.next()) {
      const int i = 32 * c + lane;
      if (i < a.n) {
        double r[3];
        load3(rb[cur], i, r);
        store3(a.r, i, r);
      }
    }
  }
  if (writer) {
    a.out->res = res;
    a.out->iters = it;
    a.out->converged = res >= 0 && res < a.tol;
  }
}

template <int D>
__global__ void __launch_bounds__(256) k_admm_persistent(ADMMArgs a) {
  __shared__ double smem8[8];
  AdmmCtx ctx{a, smem8, (a.n + 31) / 32};
  admm_body<D>(a, ctx);
}


// ---- DualAMA --------------------------------------------------------------------------------------------
// PrimalFrictionProblem::solveWith(DualAMAType&, v, r, staticProblem) (PrimalFrictionProblem.cpp:78-99).
// Phases of one iteration (one lane per body in body phases, 32-contact chunks in contact phases):
//   Q1 bodies + contacts  x = f + M v, z = H^T r - x and its norms; u = w + H v, law error at (r, u) .... reduce
//   Q2 contacts + bodies  g = u + COV(u) + gamma H z; the best (r, v) kept; the first trial's Q3 on the
//                         contact's own g ............................................................. barrier
//   line search, trial by trial:
//     Q3 contacts         r_s = P(r - lambda g), from the second trial on ................................ barrier
//     Q4 bodies           H^T r_s, y = v + gamma (H^T r_s - x) over-relaxed, |(H^T r_s - f) - M y|^2 .. reduce
//   (no line search: Q3 writes r = P(r - lambda g), Q5 forms H^T r)
//   Q5 bodies             z = H^T r - x, y = v + gamma z, v = y + beta (y - y_prev) ..................... barrier
//                         (with a line search Q4 already forms these for its trial: the last trial's become
//                         the current v and y_prev by a pointer swap, and Q5 and its barrier are skipped)
// Orders: M v chains over the dofs from 0 and is added to f (subtracted from H^T r - f); H^T r per dof over the
// body's contacts in increasing order, rows inner; H z and H v as the ADMM kernel's products; dof norms each body's
// dofs left to right, then the canonical sum over bodies.
template <int D>
__device__ void dama_body(const DamaArgs& a, double* smem8) {
  constexpr int DM = D > 0 ? D : kMaxDof;
  const int d = D > 0 ? D : a.d;
  const int lane = threadIdx.x & 31;
  const int C = (a.n + 31) / 32, CB = (a.nbodies + 31) / 32;
  const int CC = C > CB ? C : CB;
  const bool inf = a.use_inf != 0, desaxce = a.desaxce != 0;
  const bool writer = blockIdx.x == 0 && threadIdx.x == 0;
  auto put = [&](int q, int c, double v, bool is_max) {
    v = is_max ? warp_max_butterfly(v) : warp_sum_butterfly(v);
    if (lane == 0) a.csum[q * CC + c] = v;
  };
  Tickets tk{a.tickets};
  auto next = [&]() { return tk.next(); };
  auto sync = [&]() {
    const bool ok = grid_barrier(a.gb, [&] { tk.clear(); });
    ++tk.phase;
    return ok;
  };
  // value 0 over count0 chunks, values 1.. over count1 chunks
  auto sync_reduce = [&](int K, int count0, int count1, unsigned maxmask) {
    const bool ok = grid_barrier_combine(a.gb, a.combine_count, a.csum, (size_t)CC, count0, count1, K, maxmask,
                                         a.stripes, a.scal, [&] { tk.clear(); });
    ++tk.phase;
    return ok;
  };
  // H^T src for body b (d values): per dof, contacts in increasing order, rows inner
  auto body_HT = [&](int b, const double* src, double* out) {
#pragma unroll
    for (int q = 0; q < DM; ++q)
      if (q < d) out[q] = 0.0;
    const int e0 = __ldg(a.bptr + b), e1 = __ldg(a.bptr + b + 1);
    for (int e = e0; e < e1; ++e) {
      const int ent = __ldg(a.bent + e);
      const int i = ent >> 1;
      const double* Hb = a.H + (size_t)ent * 3 * d;
      const double rv[3] = {ldcg(src + 3 * i), ldcg(src + 3 * i + 1), ldcg(src + 3 * i + 2)};
#pragma unroll
      for (int q = 0; q < DM; ++q)
        if (q < d) {
          double s = out[q];
          for (int rr = 0; rr < 3; ++rr) s = fma(__ldg(Hb + rr * d + q), rv[rr], s);
          out[q] = s;
        }
    }
  };
  // (M_b src)_a: fma chain over the dofs from 0
  auto body_M = [&](int b, const double* src, int row) {
    const double* Mb = a.M + (size_t)b * d * d;
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < DM; ++q)
      if (q < d) t = fma(__ldg(Mb + row * d + q), src[q], t);
    return t;
  };
  // contact velocity-like product: init + H src (src per body)
  auto contact_H = [&](int i, const double* init, const double* src, double* out) {
#pragma unroll
    for (int r = 0; r < 3; ++r) out[r] = init ? __ldg(init + 3 * i + r) : 0.0;
    for (int t = 0; t < 2; ++t) {
      const int body = __ldg(a.cb + 2 * i + t);
      if (body < 0) continue;
      const double* Hb = a.H + (2 * (size_t)i + t) * 3 * d;
      double sv[DM];
#pragma unroll
      for (int m = 0; m < DM; ++m)
        if (m < d) sv[m] = ldcg(src + (size_t)body * d + m);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        double acc = out[r];
#pragma unroll
        for (int m = 0; m < DM; ++m)
          if (m < d) acc = fma(__ldg(Hb + r * d + m), sv[m], acc);
        out[r] = acc;
      }
    }
  };

  double* r = a.r;
  double* rs = a.rs;
  // v and y_prev, and the line search's candidates for them (swapped in when a trial ends the search)
  double* vc = a.v;
  double* ypc = a.y_prev;
  double* vn = a.v_spare;
  double* ypn = a.yp_spare;
  // H^T r once
  for (int c = next(); c < CB; c = next()) {
    const int b = 32 * c + lane;
    if (b < a.nbodies) {
      double h[DM];
      body_HT(b, r, h);
#pragma unroll
      for (int q = 0; q < DM; ++q)
        if (q < d) a.HrBp[(size_t)b * d + q] = h[q];
    }
  }
  if (!sync()) return;
  double lambda = a.lambda0, theta_prev = 1., res_prev = -1., min_res = -1., res = -1.;
  unsigned it = 0, trials = 0;
  int stopped = 0;
  for (; it < a.max_iters; ++it) {
    // Q1: tickets [0, CB) take body chunks, [CB, CB + C) contact chunks
    for (int t = next(); t < CB + C; t = next()) {
      if (t >= CB) {
        const int c = t - CB;
        const int i = 32 * c + lane;
        double ev = 0.0;
        if (i < a.n) {
          double u[3];
          contact_H(i, a.w, vc, u);
          a.ut[3 * i] = u[0];
          a.ut[3 * i + 1] = u[1];
          a.ut[3 * i + 2] = u[2];
          const double sc = __ldg(a.scaling + i);
          const double lx[3] = {ldcg(r + 3 * i) * sc, ldcg(r + 3 * i + 1) * sc, ldcg(r + 3 * i + 2) * sc};
          ev = law_eval(desaxce, __ldg(a.mu + i), lx, u);
        }
        put(0, c, ev, inf);
        continue;
      }
      const int c = t;
      const int b = 32 * c + lane;
      double pz = 0.0, pz2 = 0.0;
      if (b < a.nbodies) {
        double vb[DM];
#pragma unroll
        for (int q = 0; q < DM; ++q)
          if (q < d) vb[q] = ldcg(vc + (size_t)b * d + q);
#pragma unroll
        for (int q = 0; q < DM; ++q)
          if (q < d) {
            const double xq = __ldg(a.f + (size_t)b * d + q) + body_M(b, vb, q);
            a.x[(size_t)b * d + q] = xq;
            const double z = ldcg(a.HrBp + (size_t)b * d + q) - xq;
            pz = inf ? dmax(fabs(z), pz) : pz + z * z;
            pz2 = pz2 + z * z;
          }
      }
      put(1, c, pz, inf);
      put(2, c, pz2, false);
    }
    if (!sync_reduce(3, C, CB, inf ? 3u : 0u)) return;
    {
      const double e0 = ldcg(a.scal), z0 = ldcg(a.scal + 1);
      res = (inf ? e0 : e0 / (double)(1 + a.n)) + (inf ? z0 : z0 / (1.0 + a.m_true));
    }
    const double h0 = ldcg(a.scal + 2);
    if (a.trace && writer) a.trace[it] = res;
    const bool best = res < min_res || it == 0;
    if (best) min_res = res;
    const bool done = best && res < a.tol;
    if (!best && res > 1.e50) {
      stopped = 1;
      break;
    }
    double beta = 0.0;
    if (a.accelerated && res < res_prev) beta = nesterov_inertia(theta_prev, 0.);
    else theta_prev = 1.;
    // Q2: g (unless done) and the best (r, v): tickets [0, C) take contact chunks, [C, C + CB) body chunks
    // (these only when the iterate is the best so far). Q3 of the first trial, r_s = P(r - lambda g), needs only
    // the contact's own g, so it runs here on the g just computed (in place, r = P(r - lambda g), without a
    // line search).
    if (!done && a.ls_iters != 0) lambda *= a.opt;
    double* q3_out = a.ls_iters == 0 ? r : rs;
    const int q2_end = C + (best ? CB : 0);
    for (int t = next(); t < q2_end; t = next()) {
      if (t >= C) {
        const int b = 32 * (t - C) + lane;
        if (b < a.nbodies)
          for (int q = 0; q < d; ++q) a.v_best[(size_t)b * d + q] = ldcg(vc + (size_t)b * d + q);
        continue;
      }
      const int c = t;
      const int i = 32 * c + lane;
      if (i < a.n) {
        double rc[3];
        for (int k = 0; k < 3; ++k) rc[k] = ldcg(r + 3 * i + k);
        if (best)
          for (int k = 0; k < 3; ++k) a.r_best[3 * i + k] = rc[k];
        if (!done) {
          double u[3], hz[3];
          for (int k = 0; k < 3; ++k) u[k] = ldcg(a.ut + 3 * i + k);
          // H z with z = H^T r - x per body
          hz[0] = hz[1] = hz[2] = 0.0;
          for (int t = 0; t < 2; ++t) {
            const int body = __ldg(a.cb + 2 * i + t);
            if (body < 0) continue;
            const double* Hb = a.H + (2 * (size_t)i + t) * 3 * d;
            double zb[DM];
#pragma unroll
            for (int m = 0; m < DM; ++m)
              if (m < d) zb[m] = ldcg(a.HrBp + (size_t)body * d + m) - ldcg(a.x + (size_t)body * d + m);
#pragma unroll
            for (int rr = 0; rr < 3; ++rr) {
              double acc = hz[rr];
#pragma unroll
              for (int m = 0; m < DM; ++m)
                if (m < d) acc = fma(__ldg(Hb + rr * d + m), zb[m], acc);
              hz[rr] = acc;
            }
          }
          const double s0 = duality_cov(desaxce, __ldg(a.mu + i), u);
          const double g[3] = {fma(a.gamma, hz[0], u[0] + s0), fma(a.gamma, hz[1], u[1] + 0.0),
                               fma(a.gamma, hz[2], u[2] + 0.0)};
          a.g[3 * i] = g[0];
          a.g[3 * i + 1] = g[1];
          a.g[3 * i + 2] = g[2];
          double rr[3];
          for (int k = 0; k < 3; ++k) rr[k] = rc[k] - lambda * g[k];
          project_cone(__ldg(a.mu + i), rr);
          for (int k = 0; k < 3; ++k) q3_out[3 * i + k] = rr[k];
        }
      }
    }
    if (a.ls_iters != 0 && !done) ++trials;
    if (!sync()) return;
    if (done) {
      stopped = 1;
      break;
    }
    if (a.ls_iters != 0) {
      for (unsigned ls = 0; ls < a.ls_iters; ++ls) {
        if (ls > 0) {
          ++trials;
          // Q3: r_s = P(r - lambda g) for a later trial
          for (int c = next(); c < C; c = next()) {
            const int i = 32 * c + lane;
            if (i < a.n) {
              double rr[3];
              for (int k = 0; k < 3; ++k) rr[k] = ldcg(r + 3 * i + k) - lambda * ldcg(a.g + 3 * i + k);
              project_cone(__ldg(a.mu + i), rr);
              for (int k = 0; k < 3; ++k) rs[3 * i + k] = rr[k];
            }
          }
          if (!sync()) return;
        }
        // Q4
        for (int c = next(); c < CB; c = next()) {
          const int b = 32 * c + lane;
          double ph = 0.0;
          if (b < a.nbodies) {
            double hr[DM], y[DM];
            body_HT(b, rs, hr);
#pragma unroll
            for (int q = 0; q < DM; ++q)
              if (q < d) {
                a.HrBp[(size_t)b * d + q] = hr[q];
                const double zq = hr[q] - ldcg(a.x + (size_t)b * d + q);
                const double yk = ldcg(vc + (size_t)b * d + q) + a.gamma * zq;
                y[q] = yk + beta * (yk - ldcg(ypc + (size_t)b * d + q));
                // the velocity update of this trial (Q5's values, should the trial be the last)
                vn[(size_t)b * d + q] = y[q];
                ypn[(size_t)b * d + q] = yk;
              }
#pragma unroll
            for (int q = 0; q < DM; ++q)
              if (q < d) {
                const double gq = (hr[q] - __ldg(a.f + (size_t)b * d + q)) - body_M(b, y, q);
                ph = ph + gq * gq;
              }
          }
          put(0, c, ph, false);
        }
        if (!sync_reduce(1, CB, CB, 0u)) return;
        const double hh = ldcg(a.scal);
        if (hh < h0) break;
        lambda *= a.pess;
      }
      double* t = r;  // r = r_s
      r = rs;
      rs = t;
      // Q5 with a line search: its v = yk + beta (yk - y_prev) and y_prev = yk are the last trial's, already
      // formed by Q4 with the same operations; they become the current ones
      t = vc;
      vc = vn;
      vn = t;
      t = ypc;
      ypc = ypn;
      ypn = t;
    }
    // Q5 (no line search): z = H^T r - x, y = v + gamma z, v = y + beta (y - y_prev)
    if (a.ls_iters == 0) {
      for (int c = next(); c < CB; c = next()) {
        const int b = 32 * c + lane;
        if (b < a.nbodies) {
          double hr[DM];
          body_HT(b, r, hr);
#pragma unroll
          for (int q = 0; q < DM; ++q)
            if (q < d) {
              a.HrBp[(size_t)b * d + q] = hr[q];
              const double zq = hr[q] - ldcg(a.x + (size_t)b * d + q);
              const double yk = ldcg(vc + (size_t)b * d + q) + a.gamma * zq;
              const double yp = ldcg(ypc + (size_t)b * d + q);
              vc[(size_t)b * d + q] = yk + beta * (yk - yp);
              ypc[(size_t)b * d + q] = yk;
            }
        }
      }
    }
    res_prev = res;
    if (a.ls_iters == 0 && !sync()) return;
  }
  if (writer) {
    a.out->min_res = min_res;
    a.out->iters = it;
    a.out->stopped = stopped;
    a.out->trials = trials;
  }
}

template <int D>
__global__ void __launch_bounds__(256) k_dama_persistent(DamaArgs a) {
  __shared__ double smem8[8];
  dama_body<D>(a, smem8);
}

}  // namespace

cudaError_t launch_admm(const ADMMArgs& a, int grid, cudaStream_t s) {
  ADMMArgs copy = a;
  void* args[] = {&copy};
  const void* fn = a.d == 6 ? (const void*)k_admm_persistent<6> : (const void*)k_admm_persistent<0>;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s);
}

int admm_max_grid(int device, int d) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  const cudaError_t e = d == 6 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_admm_persistent<6>, 256, 0)
                               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_admm_persistent<0>, 256, 0);
  if (e != cudaSuccess) return 0;
  if (per > 2) per = 2;
  return per * sms;
}

}  // namespace bogus_gpu

namespace bogus_gpu {

cudaError_t launch_dama(const DamaArgs& a, int grid, cudaStream_t s) {
  DamaArgs copy = a;
  void* args[] = {&copy};
  const void* fn = a.d == 6 ? (const void*)k_dama_persistent<6> : (const void*)k_dama_persistent<0>;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s);
}

int dama_max_grid(int device, int d) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  const cudaError_t e = d == 6 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dama_persistent<6>, 256, 0)
                               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dama_persistent<0>, 256, 0);
  if (e != cudaSuccess) return 0;
  if (per > 2) per = 2;
  return per * sms;
}

// Sets this file's copy of the device-side wait limit on the current device.
BOGUS_GPU_WAIT_LIMIT_SETTER(set_wait_limit_admm)

}  // namespace bogus_gpu
