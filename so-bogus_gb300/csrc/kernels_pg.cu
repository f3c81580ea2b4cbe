// Persistent projected-gradient solvers: the whole solve of PgMethod<APGD / Descent / SPG>
// (Core/BlockSolvers/ProjectedGradient.impl.hpp:74-155, 288-351) runs in one cooperative launch.
//
// Work split: warp w of the grid owns the 32-contact chunks w, w + W, w + 2W, ... in every phase, lane l
// contact 32c + l. A phase is one pass over the contacts (row-local vector work) or over W (SpMV with the
// row-local work fused into its epilogue). Global dot products are reduced in the canonical order: a
// butterfly per chunk inside the warp, then the 8-stripe combination run by the last CTA to reach the
// grid barrier, which publishes the scalars; every CTA then takes the same line-search / momentum
// decisions on identical values. Waits are bounded (grid_barrier), so a fault elsewhere ends the kernel
// with BOGUS_GPU_TIMEOUT instead of a hang.
//
// Phases of one APGD iteration (reference line numbers in ProjectedGradient.impl.hpp):
//   A   y = Mx + b, residual (:110-111), s = COV(y), y += s, J (:113-115), xs = P(x - a y) (:123-125)
//   C   Mxs = W xs; Js, y.(xs-x), |xs-x|^2 (:127-132), (xs-prev).y (:135); APGD also writes the
//       momentum point x = xs + beta (xs - prev) (:137-139) to a spare buffer ........... barrier+reduce
//   B   line-search retry: xs = P(x - a y) ............................................ barrier
//   E+A Mx = W x (:141) fused with A of the next iteration ............................. barrier+reduce
// With momentum, the spare buffer becomes x (a buffer swap); without, x = xs and Mx = Mxs are swaps and A
// runs as its own pass. Phase counter 5 (a separate momentum pass) is no longer used.
#include "internal.h"
#include "soc_device.cuh"
#include "soc_ops.cuh"
#include "spmv_chunk.cuh"

namespace bogus_gpu {

namespace {

template <class T>
__device__ __forceinline__ void load3cg(const T* p, int i, T* v) {
  v[0] = ldcg(p + 3 * i);
  v[1] = ldcg(p + 3 * i + 1);
  v[2] = ldcg(p + 3 * i + 2);
}
template <class T>
__device__ __forceinline__ void store3(T* p, int i, const T* v) {
  p[3 * i] = v[0];
  p[3 * i + 1] = v[1];
  p[3 * i + 2] = v[2];
}

// Position buffers 0, 1, 2 (X0..X2) and 4 (Wv, free in APGD / Descent: the speculative momentum point);
// 3 names the x_best buffer in PGOut::best_buf.
template <class T>
struct Bufs {
  const PGArgsT<T>& a;
  __device__ T* X(int k) const { return k == 0 ? a.X0 : (k == 1 ? a.X1 : (k == 2 ? a.X2 : a.Wv)); }
  __device__ T* MX(int k) const { return k == 0 ? a.MX0 : (k == 1 ? a.MX1 : (k == 2 ? a.MX2 : a.MX3)); }
};

__device__ __forceinline__ int third(int p, int q) {
  for (int k = 0; k < 3; ++k)
    if (k != p && k != q) return k;
  return 0;
}

// The first two of the product buffers {0, 1, 2, 3} other than p and q (p == q allowed).
__device__ __forceinline__ void two_free_mx(int p, int q, int& f0, int& f1) {
  f0 = -1;
  f1 = -1;
  for (int v = 0; v < 4; ++v) {
    if (v == p || v == q) continue;
    if (f0 < 0) f0 = v;
    else if (f1 < 0) f1 = v;
  }
}

// The first two of the position buffers {0, 1, 2, 4} other than p and q (p == q allowed).
__device__ __forceinline__ void two_free(int p, int q, int& f0, int& f1) {
  const int ids[4] = {0, 1, 2, 4};
  f0 = -1;
  f1 = -1;
  for (int k = 0; k < 4; ++k) {
    const int v = ids[k];
    if (v == p || v == q) continue;
    if (f0 < 0) f0 = v;
    else if (f1 < 0) f1 = v;
  }
}

}  // namespace

// Per-warp scratch of the FP32 correction products, allocated only in the kernel that uses them (HY).
template <bool HY>
__device__ __forceinline__ ChunkScratchT<float>* hy_scratch() { return nullptr; }
template <>
__device__ __forceinline__ ChunkScratchT<float>* hy_scratch<true>() {
  __shared__ ChunkScratchT<float> s[8];
  return s;
}

// W v for row 32c + lane as W x_ref + W32 (v - x_ref)_32, d = (v - x_ref)_32: FP32 chains over the FP32 copy of
// W (interleaved, or the plain BSR values of the batched solves) in the chunk-segmented order, then added to the
// FP64 W x_ref.
template <class T, bool IL>
__device__ __forceinline__ void hy_product(const PGArgsT<T>& a, int c, const float* __restrict__ d,
                                           ChunkScratchT<float>& sh32, T* acc) {
  float acc32[3] = {0.f, 0.f, 0.f};
  if constexpr (IL) {
    const InterleavedBlocks<float> b32{a.icol, a.hy_ival, a.slot0};
    spmv_chunk<1, true>(a.rowptr, b32, a.n, c, sh32, [&](int j, float* x) { load3cg(d, j, x); }, acc32);
  } else {
    const PlainBlocks<float> b32{a.col, a.hy_ival};
    spmv_chunk<1, true>(a.rowptr, b32, a.n, c, sh32, [&](int j, float* x) { load3cg(d, j, x); }, acc32);
  }
  const int i = 32 * c + (threadIdx.x & 31);
  if (i < a.n) {
    acc[0] = ldcg(a.hy_wxref + 3 * i) + (double)acc32[0];
    acc[1] = ldcg(a.hy_wxref + 3 * i + 1) + (double)acc32[1];
    acc[2] = ldcg(a.hy_wxref + 3 * i + 2) + (double)acc32[2];
  }
}

template <class T, bool IL>
struct BlocksOf;
template <class T>
struct BlocksOf<T, false> {
  static __device__ __forceinline__ PlainBlocks<T> make(const PGArgsT<T>& a) { return PlainBlocks<T>{a.col, a.val}; }
};
template <class T>
struct BlocksOf<T, true> {
  static __device__ __forceinline__ InterleavedBlocks<T> make(const PGArgsT<T>& a) {
    return InterleavedBlocks<T>{a.icol, a.ival, a.slot0};
  }
};

// IL: read W through its interleaved copy (single-problem solves) or the plain BSR arrays (batched and
// allocation-free solves). The arithmetic is the same.
// SC: the Standard and Conjugated variants (their own kernel instantiation, so that their code does not change the
// register allocation of the APGD / Descent / SPG kernels).
// HY: APGD with FP32 correction products (FP64 iterates, law and reductions; its own instantiation as well):
// W v = W x_ref + W32 (v - x_ref)_32, x_ref and W x_ref refreshed in FP64 every hy_refresh iterations.
template <class T, bool IL, bool SC = false, bool HY = false, class Ctx>
__device__ __forceinline__ int pg_body_inl(const PGArgsT<T>& a, Ctx& ctx) {
  using Ops = SocOps<T>;
  const Bufs<T> B{a};
  ChunkScratchT<T>& sh = ctx.cs[threadIdx.x >> 5];
  const auto blocks = BlocksOf<T, IL>::make(a);
  // y = W x of chunk c for every lane (row 32c + lane), x gathered from a buffer written earlier in the kernel
  auto product = [&](int c, const T* __restrict__ xsrc, T* acc) {
    spmv_chunk<1, true>(a.rowptr, blocks, a.n, c, sh, [&](int j, T* x) { load3cg(xsrc, j, x); }, acc);
  };
  const int lane = threadIdx.x & 31;
  // HY: the FP32 correction v - x_ref of position buffer k (0, 1, 2 or 4), written beside every position that a
  // later product multiplies
  auto hy_d = [&](int k) -> float* { return a.hy_d + (size_t)(k == 4 ? 3 : k) * a.hy_stride; };
  auto store_corr = [&](int k, int i, const T* v) {
    if constexpr (HY) {
      T xr[3];
      load3cg(a.hy_xref, i, xr);
      float* d = hy_d(k);
      d[3 * i] = (float)(v[0] - xr[0]);
      d[3 * i + 1] = (float)(v[1] - xr[1]);
      d[3 * i + 2] = (float)(v[2] - xr[2]);
    }
  };
  // W X(k) for row 32c + lane: the FP64 product or, HY, W x_ref + W32 (X(k) - x_ref)_32 (FP32 FMA chains in the
  // chunk-segmented order over the FP32 interleaved copy of W)
  auto product_k = [&](int c, int k, T* acc) {
    if constexpr (HY) {
      hy_product<T, IL>(a, c, hy_d(k), hy_scratch<HY>()[threadIdx.x >> 5], acc);
    } else {
      product(c, B.X(k), acc);
    }
  };
  const bool desaxce = a.desaxce != 0;
  const bool spg = a.variant == 4;
  const bool apgd = a.variant == 3;
  const int C = a.nchunks;
  const unsigned res_mask = a.use_inf ? 1u : 0u;

  auto put = [&](int q, int c, double v, bool is_max) {
    v = is_max ? warp_max_butterfly(v) : warp_sum_butterfly(v);
    if (lane == 0) a.csum[q * C + c] = v;
  };
  // chunk sums of values 0 and 1 (value 0 the maximum when max0)
  auto put2 = [&](int c, double v0, double v1, bool max0) {
    if (max0) {
      put(0, c, v0, true);
      put(1, c, v1, false);
      return;
    }
    const double v = warp_sum2_butterfly(v0, v1);
    if ((lane & 15) == 0) a.csum[(lane >> 4) * C + c] = v;
  };
  auto put4 = [&](int c, double v0, double v1, double v2, double v3) {
    const double v = warp_sum4_butterfly(v0, v1, v2, v3);
    if ((lane & 7) == 0) a.csum[(lane >> 3) * C + c] = v;
  };
  auto sync = [&]() -> bool { return ctx.sync(); };
  auto sync_reduce = [&](int K, unsigned maxmask) -> bool { return ctx.sync_reduce(K, maxmask); };
  // split: the CTAs may go on before the scalars are published; read them after ctx.await_scalars()
  auto sync_reduce_split = [&](int K, unsigned maxmask) -> bool { return ctx.sync_reduce_split(K, maxmask); };
  auto scal = [&](int q) { return ctx.scal(q); };
  // ConstrainedSolverBase::eval: sum / (1 + n), or the maximum with the infinity norm
  auto residual_of = [&](double reduced) { return a.use_inf ? reduced : reduced / (double)(1 + a.n); };
  unsigned ph[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  unsigned n_refresh = 0;  // HY: refreshes of x_ref
  auto finish = [&](double min_res, unsigned iters, int best_buf, int converged) -> int {
    if (ctx.writer()) {
      a.out->min_res = min_res;
      a.out->iters = iters;
      a.out->best_buf = best_buf;
      a.out->converged = converged;
#pragma unroll
      for (int k = 0; k < 9; ++k) a.out->phases[k] = ph[k];
      a.out->hy_refreshes = n_refresh;
    }
    return best_buf;
  };

  int ix = 0, iprev = 0, ixs = 1, imx = 0;

  // projectOnConstraints(x) (:90)
  ph[0]++;
  for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
    const int i = 32 * c + lane;
    if (i < a.n) {
      T x[3];
      load3cg(a.X0, i, x);
      Ops::project(__ldg(a.mu + i), x);
      store3(a.X0, i, x);
    }
  }
  if (!sync()) return -1;

  // Mx = W x (:93) and guess_alpha (:21-28): |W (x - 1)|^2, |x - 1|^2
  ph[1]++;
  for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
    const int i = 32 * c + lane;
    double v0 = 0.0, v1 = 0.0;
    T acc[3] = {T(0), T(0), T(0)}, accd[3] = {T(0), T(0), T(0)};
    spmv_chunk<2, true>(a.rowptr, blocks, a.n, c, sh, [&](int j, T* x) { load3cg(a.X0, j, x); }, acc, accd);
    if (i < a.n) {
      store3(a.MX0, i, acc);
      v0 = Ops::sq3(accd);
      T x[3];
      load3cg(a.X0, i, x);
      const T d[3] = {x[0] - T(1), x[1] - T(1), x[2] - T(1)};
      v1 = Ops::sq3(d);
      if constexpr (HY) {
        store3(a.hy_wxref, i, acc);
        store3(a.hy_xref, i, x);
      }
    }
    put2(c, v0, v1, false);
  }
  if (!sync_reduce(2, 0u)) return -1;
  double alpha = 1.0;
  {
    const double nMx = scal(0);
    if (nMx > 1.e-16) alpha = dmin(1., scal(1) / nMx);
  }
  if (a.max_iters == 0) {
    return finish(-1.0, 0, 0, 0);
  }

  // Row-local part A, given Mx_i: writes y, s0 and xs = P(x - alpha_t y) (APGD) and returns the residual
  // and objective terms; SPG additionally needs (xs - prev).y.
  auto phaseA = [&](int i, const T* Mx, double alpha_t, double& res_i, double& second_i) {
    T x[3], bb[3];
    load3cg(B.X(ix), i, x);
    bb[0] = __ldg(a.b + 3 * i);
    bb[1] = __ldg(a.b + 3 * i + 1);
    bb[2] = __ldg(a.b + 3 * i + 2);
    const T mu = __ldg(a.mu + i), sc = __ldg(a.scaling + i);
    T y[3] = {Mx[0] + bb[0], Mx[1] + bb[1], Mx[2] + bb[2]};
    const T lx[3] = {x[0] * sc, x[1] * sc, x[2] * sc};
    res_i = Ops::law_eval(desaxce, mu, lx, y);
    const T s0 = Ops::cov(desaxce, mu, y);
    y[0] = y[0] + s0;
    y[1] = Ops::plus0(y[1]);
    y[2] = Ops::plus0(y[2]);
    const T na = T(-alpha_t);
    T xs[3] = {fma(na, y[0], x[0]), fma(na, y[1], x[1]), fma(na, y[2], x[2])};
    Ops::project(mu, xs);
    store3(a.Y, i, y);
    a.S0[i] = s0;
    store3(B.X(ixs), i, xs);
    store_corr(ixs, i, xs);
    if (spg) {
      T pv[3];
      load3cg(B.X(iprev), i, pv);
      const T d[3] = {xs[0] - pv[0], xs[1] - pv[1], xs[2] - pv[2]};
      second_i = Ops::dot3(d, y);
    } else {
      const T t[3] = {(Ops::half(Mx[0]) + bb[0]) + s0, Ops::plus0(Ops::half(Mx[1]) + bb[1]),
                      Ops::plus0(Ops::half(Mx[2]) + bb[2])};
      second_i = Ops::dot3(x, t);
    }
  };

  auto runA = [&](double alpha_t, bool split) -> bool {  // A as its own pass (Mx already in MX(imx))
    ph[2]++;
    for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
      const int i = 32 * c + lane;
      double r = 0.0, q = 0.0;
      if (i < a.n) {
        T Mx[3];
        load3cg(B.MX(imx), i, Mx);
        phaseA(i, Mx, alpha_t, r, q);
      }
      put2(c, r, q, res_mask != 0);
    }
    return split ? sync_reduce_split(2, res_mask) : sync_reduce(2, res_mask);
  };

  double min_res = -1.0, theta = 1.0;
  bool best_pending = false;
  unsigned it = 0;

  if constexpr (SC) {
    // ------------------------------------------------ Standard (:157-209) and Conjugated (:211-286)
    // Single-problem solves only (the host rejects them elsewhere): the Conjugated variant's first reduction
    // has 5 quantities. x = X(ix), the line search's trial point X(ixs) (the two swap when a search ends),
    // Mx = MX(imx), its product MX(1 - imx). Standard: pg = X(2), W pg = MX(2). Conjugated: prev_pg = X(2),
    // prev_dir = MX(2) (formed in A as (x - x_old) / alpha of the last search, x_old still in X(ixs)),
    // dir = X(4).
    const bool conj = a.variant == 2;
    double alpha_s = 1.0, alpha_prev = 1.0, prev_n2 = 0.0;
    bool have_prev = false;
    for (;;) {
      // A: y = Mx + b, the residual, s = COV(y), y += s, J; xs = P(x - y), pg = x - xs (:164-176, :218-231)
      ph[2]++;
      for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
        const int i = 32 * c + lane;
        double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        if (i < a.n) {
          T x[3], Mx[3], bb[3];
          load3cg(B.X(ix), i, x);
          load3cg(B.MX(imx), i, Mx);
          bb[0] = __ldg(a.b + 3 * i);
          bb[1] = __ldg(a.b + 3 * i + 1);
          bb[2] = __ldg(a.b + 3 * i + 2);
          const T mu = __ldg(a.mu + i), sc = __ldg(a.scaling + i);
          T y[3] = {Mx[0] + bb[0], Mx[1] + bb[1], Mx[2] + bb[2]};
          const T lx[3] = {x[0] * sc, x[1] * sc, x[2] * sc};
          v[0] = Ops::law_eval(desaxce, mu, lx, y);
          const T s0 = Ops::cov(desaxce, mu, y);
          y[0] = y[0] + s0;
          y[1] = Ops::plus0(y[1]);
          y[2] = Ops::plus0(y[2]);
          const T t[3] = {(Ops::half(Mx[0]) + bb[0]) + s0, Ops::plus0(Ops::half(Mx[1]) + bb[1]),
                          Ops::plus0(Ops::half(Mx[2]) + bb[2])};
          v[1] = Ops::dot3(x, t);
          T xs[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
          Ops::project(mu, xs);
          const T pg[3] = {x[0] - xs[0], x[1] - xs[1], x[2] - xs[2]};
          store3(a.Y, i, y);
          a.S0[i] = s0;
          if (!conj) {
            v[2] = Ops::dot3(y, pg);
          } else {
            v[2] = Ops::sq3(pg);
            if (have_prev) {
              T xo[3], ppg[3];
              load3cg(B.X(ixs), i, xo);
              load3cg(B.X(2), i, ppg);
              const T pd[3] = {(x[0] - xo[0]) / T(alpha_prev), (x[1] - xo[1]) / T(alpha_prev),
                               (x[2] - xo[2]) / T(alpha_prev)};
              store3(B.MX(2), i, pd);
              const T dg[3] = {pg[0] - ppg[0], pg[1] - ppg[1], pg[2] - ppg[2]};
              v[3] = Ops::dot3(pd, dg);
              v[4] = Ops::dot3(pg, ppg);
            }
          }
          store3(B.X(2), i, pg);
        }
        put(0, c, v[0], res_mask != 0);
        put(1, c, v[1], false);
        put(2, c, v[2], false);
        if (conj) {
          put(3, c, v[3], false);
          put(4, c, v[4], false);
        }
      }
      if (!sync_reduce(conj ? 5 : 3, res_mask)) return -1;
      const double res = residual_of(scal(0)), J = scal(1), s2 = scal(2);
      const double den_c = conj ? scal(3) : 0.0, xp = conj ? scal(4) : 0.0;
      if (a.trace && ctx.writer()) a.trace[it] = res;
      if (it == 0 || res < min_res) {
        min_res = res;
        best_pending = true;
      }
      if (res < a.tol) return finish(min_res, it, ix, 1);
      // the step direction
      double beta = 0.0;
      bool neg_y = false;
      if (!conj) {
        // Mpg = W pg, pg.Mpg (:177-181); pg *= beta with beta = -y.pg / pg.Mpg
        ph[3]++;
        for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
          const int i = 32 * c + lane;
          double v0 = 0.0;
          T acc[3] = {T(0), T(0), T(0)};
          product(c, B.X(2), acc);
          if (i < a.n) {
            T pg[3];
            load3cg(B.X(2), i, pg);
            store3(B.MX(2), i, acc);
            v0 = Ops::dot3(pg, acc);
          }
          put(0, c, v0, false);
        }
        if (!sync_reduce(1, 0u)) return -1;
        beta = -s2 / scal(0);
      } else if (prev_n2 == 0.) {
        neg_y = true;  // dir = -y (:232-233)
      } else {
        // dir = beta prev_dir - y, with dir = -y when it is not a descent direction (:235-245)
        beta = (den_c < 1.e-12) ? dmax(0., (s2 - xp)) / prev_n2 : dmax(0., (s2 - xp)) / den_c;
        const T bc = T(beta);
        ph[7]++;
        for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
          const int i = 32 * c + lane;
          double v0 = 0.0;
          if (i < a.n) {
            T pd[3], y[3];
            load3cg(B.MX(2), i, pd);
            load3cg(a.Y, i, y);
            const T dir[3] = {bc * pd[0] - y[0], bc * pd[1] - y[1], bc * pd[2] - y[2]};
            store3(B.X(4), i, dir);
            v0 = Ops::dot3(dir, y);
          }
          put(0, c, v0, false);
        }
        if (!sync_reduce(1, 0u)) return -1;
        neg_y = scal(0) >= 0.;
      }
      if (conj) prev_n2 = s2;
      // Armijo line search (:93-107 of the same file's line-search helper): xs = P(x + alpha dir), W xs,
      // Js = xs.((W xs / 2 + (b + s)) + 0) against J + armijo (y.(xs - x))
      alpha_s = conj ? alpha_s * a.opt : dmin(1., alpha_s * a.opt);
      const T bt = T(beta);
      for (unsigned ls = 0; ls < a.ls_iters; ++ls) {
        const T al = T(alpha_s);
        ph[4]++;
        for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
          const int i = 32 * c + lane;
          if (i < a.n) {
            T x[3], d[3];
            load3cg(B.X(ix), i, x);
            if (!conj) {
              T pg[3];
              load3cg(B.X(2), i, pg);
              d[0] = pg[0] * bt; d[1] = pg[1] * bt; d[2] = pg[2] * bt;
            } else if (neg_y) {
              T y[3];
              load3cg(a.Y, i, y);
              d[0] = -y[0]; d[1] = -y[1]; d[2] = -y[2];
            } else {
              load3cg(B.X(4), i, d);
            }
            T xs[3] = {fma(al, d[0], x[0]), fma(al, d[1], x[1]), fma(al, d[2], x[2])};
            Ops::project(__ldg(a.mu + i), xs);
            store3(B.X(ixs), i, xs);
            if (best_pending) store3(a.XB, i, x);
          }
        }
        best_pending = false;
        if (!sync()) return -1;
        ph[3]++;
        for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
          const int i = 32 * c + lane;
          double v0 = 0.0, v1 = 0.0;
          T acc[3] = {T(0), T(0), T(0)};
          product(c, B.X(ixs), acc);
          if (i < a.n) {
            store3(B.MX(1 - imx), i, acc);
            T x[3], xs[3], y[3];
            load3cg(B.X(ix), i, x);
            load3cg(B.X(ixs), i, xs);
            load3cg(a.Y, i, y);
            const T s0 = ldcg(a.S0 + i);
            const T bs[3] = {__ldg(a.b + 3 * i) + s0, Ops::plus0(__ldg(a.b + 3 * i + 1)),
                             Ops::plus0(__ldg(a.b + 3 * i + 2))};
            const T t[3] = {Ops::plus0(Ops::half(acc[0]) + bs[0]), Ops::plus0(Ops::half(acc[1]) + bs[1]),
                            Ops::plus0(Ops::half(acc[2]) + bs[2])};
            v0 = Ops::dot3(xs, t);
            const T dd[3] = {xs[0] - x[0], xs[1] - x[1], xs[2] - x[2]};
            v1 = Ops::dot3(y, dd);
          }
          put2(c, v0, v1, false);
        }
        if (!sync_reduce(2, 0u)) return -1;
        if (scal(0) < J + a.armijo * scal(1)) break;
        alpha_s *= a.pess;
      }
      // x = xs, Mx = W xs
      const int t2 = ix;
      ix = ixs;
      ixs = t2;
      imx = 1 - imx;
      alpha_prev = alpha_s;
      have_prev = true;
      ++it;
      if (it >= a.max_iters) break;
    }
    return finish(min_res, it, 3, 0);
  }

  if (!spg) {
    // ---------------------------------------------------------------- APGD / Descent
    // APGD's momentum point x = xs + beta (xs - prev) (:137-139) is formed speculatively by every trial
    // product (C) into the spare buffer ispec, with beta from the Nesterov sequence (it needs no reduction);
    // when the line search ends with momentum, that buffer becomes x without a pass of its own.
    // A (alone or fused with E) ends with a split reduction: the trial product of the next C phase does not
    // need the residual and objective, so a warp reads them (iteration top: trace, best iterate, convergence)
    // after the product of its first chunk, or after the phase when it gets no chunk.
    int ispec = 4;
    // momentum product by linearity: imp holds W prev (prev = x after the projection: MX(imx)); each trial
    // product goes to ims and the momentum product fma(beta, W xs - W prev, W xs) to imn
    const bool lin = apgd && a.lin_momentum != 0;
    int imp = imx, ims = 1, imn = 2;
    unsigned next_refresh = HY ? a.hy_refresh : 0u;  // HY: the first iteration whose momentum step refreshes x_ref
    double alpha_t = alpha * a.opt;
    // stall test of the FP32 part (stall_iters > 0; compiled into the FP32 kernels only): consecutive iterations
    // whose residual repeats the previous one bit for bit or whose line search ran out of trials
    // HY: the part ends (for the plain FP64 solve to take over) when the best residual has not improved by 1 %
    // in 10 refresh intervals, the noise of the FP32 corrections having become the limit
    constexpr bool kStallTest = sizeof(T) == 4 || HY;
    unsigned stall_run = 0;
    bool exhausted = false;
    double prev_res = 0.0;
    double hy_best = 0.0;
    unsigned hy_best_it = 0;
    if (!runA(alpha_t, true)) return -1;
    for (;;) {
      double res = 0.0, J = 0.0;
      bool top_done = false, converged = false, stalled = false;
      auto top = [&]() -> bool {
        if (top_done) return true;
        if (!ctx.await_scalars()) return false;
        res = residual_of(scal(0));
        J = scal(1);
        if (a.trace && ctx.writer()) a.trace[it] = res;
        if (it == 0 || res < min_res) {
          min_res = res;
          best_pending = true;
        }
        converged = res < a.tol;
        if (sizeof(T) == 4 && a.stall_iters) {
          stall_run = ((it > 0 && res == prev_res) || exhausted) ? stall_run + 1 : 0;
          prev_res = res;
          stalled = !converged && stall_run >= a.stall_iters;
        }
        if constexpr (HY) {
          if (it == 0 || res < 0.99 * hy_best) {
            hy_best = res;
            hy_best_it = it;
          }
          stalled = !converged && it - hy_best_it >= 10u * a.hy_refresh;
        }
        top_done = true;
        return true;
      };
      alpha = alpha_t;
      unsigned ls = 0;
      double decr2 = 0.0;
      double theta_spec = theta;
      const double beta_spec = apgd ? nesterov_inertia(theta_spec, 0.0) : 0.0;
      const T bt = T(beta_spec);
      if (lin) two_free_mx(imx, imp, ims, imn);
      const int ims_t = lin ? ims : 1 - imx;
      for (;;) {
        // C: Mxs = W xs, the line-search terms and the speculative momentum point (and its product, lin)
        for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
          const int i = 32 * c + lane;
          double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
          T acc[3] = {T(0), T(0), T(0)};
          product_k(c, ixs, acc);
          if (!top()) return -1;
          if (converged || (kStallTest && stalled)) break;
          if (i < a.n) {
            store3(B.MX(ims_t), i, acc);
            T x[3], xs[3], pv[3], y[3];
            load3cg(B.X(ix), i, x);
            load3cg(B.X(ixs), i, xs);
            load3cg(B.X(iprev), i, pv);
            load3cg(a.Y, i, y);
            const T s0 = ldcg(a.S0 + i);
            const T t[3] = {(Ops::half(acc[0]) + __ldg(a.b + 3 * i)) + s0, Ops::plus0(Ops::half(acc[1]) + __ldg(a.b + 3 * i + 1)),
                            Ops::plus0(Ops::half(acc[2]) + __ldg(a.b + 3 * i + 2))};
            v0 = Ops::dot3(xs, t);
            const T d[3] = {xs[0] - x[0], xs[1] - x[1], xs[2] - x[2]};
            v1 = Ops::dot3(y, d);
            v2 = Ops::sq3(d);
            const T d2[3] = {xs[0] - pv[0], xs[1] - pv[1], xs[2] - pv[2]};
            v3 = Ops::dot3(d2, y);
            if (best_pending) store3(a.XB, i, x);
            if (apgd) {
              const T xn[3] = {fma(bt, xs[0] - pv[0], xs[0]), fma(bt, xs[1] - pv[1], xs[1]), fma(bt, xs[2] - pv[2], xs[2])};
              store3(B.X(ispec), i, xn);
              store_corr(ispec, i, xn);
              if (lin) {
                T mp[3];
                load3cg(B.MX(imp), i, mp);
                const T mn[3] = {fma(bt, acc[0] - mp[0], acc[0]), fma(bt, acc[1] - mp[1], acc[1]),
                                 fma(bt, acc[2] - mp[2], acc[2])};
                store3(B.MX(imn), i, mn);
              }
            }
          }
          put4(c, v0, v1, v2, v3);
        }
        if (!top()) return -1;
        if (converged) return finish(min_res, it, best_pending ? ix : 3, 1);
        if (kStallTest && stalled) return finish(min_res, it, best_pending ? ix : 3, 0);
        ph[3]++;
        best_pending = false;
        if (!sync_reduce(4, 0u)) return -1;
        const double Js = scal(0), decr = scal(1), nrm = scal(2);
        decr2 = scal(3);
        if (Js < (J + decr) + (.5 / alpha) * nrm) break;
        ++ls;
        alpha *= a.pess;
        if (ls >= a.ls_iters) break;
        // B: retry with a smaller step
        ph[4]++;
        for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
          const int i = 32 * c + lane;
          if (i < a.n) {
            T x[3], y[3];
            load3cg(B.X(ix), i, x);
            load3cg(a.Y, i, y);
            const T na = T(-alpha);
            T xs[3] = {fma(na, y[0], x[0]), fma(na, y[1], x[1]), fma(na, y[2], x[2])};
            Ops::project(__ldg(a.mu + i), xs);
            store3(B.X(ixs), i, xs);
            store_corr(ixs, i, xs);
          }
        }
        if (!sync()) return -1;
      }
      if (sizeof(T) == 4) exhausted = ls > 0 && ls >= a.ls_iters;
      ++it;
      const bool more = it < a.max_iters;
      if (apgd && decr2 < 0) {
        theta = theta_spec;  // nesterov_inertia(theta, 0) (:137), whose value beta_spec already holds
        const int nix = ispec, nprev = ixs;
        ix = nix;
        iprev = nprev;
        two_free(ix, iprev, ixs, ispec);
        if (!more) break;
        alpha_t = alpha * a.opt;
        if (lin) {
          // W x formed in C: A alone
          imx = imn;
          imp = ims;
          if (!runA(alpha_t, true)) return -1;
          continue;
        }
        // E + A: Mx = W x, then A of the next iteration on the same rows (HY: at a refresh the FP64 product,
        // which becomes W x_ref, with x_ref = x)
        const bool refresh = HY && it >= next_refresh;
        ph[6]++;
        for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
          const int i = 32 * c + lane;
          double r = 0.0, q = 0.0;
          T acc[3] = {T(0), T(0), T(0)};
          if constexpr (HY) {
            if (refresh) {
              product(c, B.X(ix), acc);
              if (i < a.n) {
                T xr[3];
                load3cg(B.X(ix), i, xr);
                store3(a.hy_xref, i, xr);
                store3(a.hy_wxref, i, acc);
              }
            } else {
              product_k(c, ix, acc);
            }
          } else {
            product(c, B.X(ix), acc);
          }
          if (i < a.n) {
            store3(B.MX(imx), i, acc);
            phaseA(i, acc, alpha_t, r, q);
          }
          put2(c, r, q, res_mask != 0);
        }
        if (refresh) {
          next_refresh = it + a.hy_refresh;
          ++n_refresh;
        }
        if (!sync_reduce_split(2, res_mask)) return -1;
      } else {
        theta = 1.;
        ix = ixs;
        iprev = ixs;
        if (lin) {
          imx = ims;
          imp = ims;
        } else {
          imx = 1 - imx;
        }
        two_free(ix, iprev, ixs, ispec);
        if (!more) break;
        alpha_t = alpha * a.opt;
        if (!runA(alpha_t, true)) return -1;
      }
    }
    return finish(min_res, it, 3, 0);
  }

  // ------------------------------------------------------------------ SPG (:288-351)
  const double a_min = 1.e-6, a_max = 1.e6;
  unsigned repeats = 0;  // stall test of the FP32 part (stall_iters > 0; FP32 kernels): the residual repeats in a row
  double prev_res = 0.0;
  for (;;) {
    if (!runA(alpha, false)) return -1;  // y, residual, s, xs = P(x - alpha y), (xs - prev).y
    const double res = residual_of(scal(0)), decr = scal(1);
    if (a.trace && ctx.writer()) a.trace[it] = res;
    if (it == 0 || res < min_res) {
      min_res = res;
      best_pending = true;
    }
    if (res < a.tol) {
      return finish(min_res, it, best_pending ? ix : 3, 1);
    }
    if (sizeof(T) == 4 && a.stall_iters) {
      repeats = (it > 0 && res == prev_res) ? repeats + 1 : 0;
      prev_res = res;
      if (repeats >= a.stall_iters) return finish(min_res, it, best_pending ? ix : 3, 0);
    }
    const bool mom = decr < 0.;
    const double beta = mom ? nesterov_inertia(theta, 0.0) : 0.0;
    if (!mom) theta = 1.;
    // D: w and the new x (over the old x); keep the best iterate first
    ph[7]++;
    for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
      const int i = 32 * c + lane;
      if (i < a.n) {
        T x[3], xs[3], pv[3], w[3], xn[3];
        load3cg(B.X(ix), i, x);
        load3cg(B.X(ixs), i, xs);
        load3cg(B.X(iprev), i, pv);
        if (best_pending) store3(a.XB, i, x);
        const T bt = T(beta);
        for (int k = 0; k < 3; ++k) {
          if (mom) {
            w[k] = fma(bt, xs[k] - pv[k], xs[k]) - x[k];
            xn[k] = x[k] + w[k];
          } else {
            w[k] = xs[k] - x[k];
            xn[k] = xs[k];
          }
        }
        store3(a.Wv, i, w);
        store3(B.X(ix), i, xn);
      }
    }
    best_pending = false;
    if (!sync()) return -1;
    // E: Mx_new = W x; z = -Mx_old + Mx_new; w.z, |z|^2
    ph[8]++;
    for (int c = ctx.first_chunk(); c < C; c = ctx.next_chunk(c)) {
      const int i = 32 * c + lane;
      double v0 = 0.0, v1 = 0.0;
      T acc[3] = {T(0), T(0), T(0)};
      product(c, B.X(ix), acc);
      if (i < a.n) {
        T mo[3], w[3];
        store3(B.MX(1 - imx), i, acc);
        load3cg(B.MX(imx), i, mo);
        load3cg(a.Wv, i, w);
        const T z[3] = {-mo[0] + acc[0], -mo[1] + acc[1], -mo[2] + acc[2]};
        v0 = Ops::dot3(w, z);
        v1 = Ops::sq3(z);
      }
      put2(c, v0, v1, false);
    }
    if (!sync_reduce(2, 0u)) return -1;
    imx = 1 - imx;
    iprev = ixs;
    ixs = third(ix, iprev);
    alpha = scal(0) / scal(1);
    alpha = dmin(a_max, dmax(a_min, alpha));
    ++it;
    if (it >= a.max_iters) break;
  }
  return finish(min_res, it, 3, 0);
}


// Single problem: the whole GPU, phases separated by bounded grid barriers on monotonic counters
// (mono_barrier); at a reducing barrier the last CTAs to arrive combine the chunk sums, one stripe each, and
// the last of them publishes the scalars in global memory. After a split reduction the CTAs go on once every
// CTA has arrived, and each warp waits for the publication only where it reads the scalars. Each CTA takes
// its 32-contact chunks from its own list (cta_ptr / cta_list: the chunks dealt largest first to the CTAs in
// serpentine rounds, so every SM's total is the same to within about one chunk), its warps sharing the list
// through a shared-memory counter per phase parity; without lists (the allocation-free entry point) warps
// take chunks from a global ticket counter per phase parity, cleared by the last CTA of the barrier that ends
// the phase, in largest-first order (chunk_order). Every cross-phase dependency goes through a barrier, and
// the reduction order does not depend on which warp handles a chunk.
template <class T>
struct GridCtx {
  const PGArgsT<T>& a;
  double* smem8;
  ChunkScratchT<T>* cs;
  unsigned* s_cnt;     // 2 shared-memory counters (phase parity) over the CTA's chunk list
  unsigned phase = 0;  // barriers passed (identical in every CTA)
  __device__ int ticket() {
    int c = 0;
    if ((threadIdx.x & 31) == 0) {
      if (a.cta_ptr) {
        const int k = (int)atomicAdd(s_cnt + (phase & 1u), 1u);
        const int b0 = __ldg(a.cta_ptr + blockIdx.x), b1 = __ldg(a.cta_ptr + blockIdx.x + 1);
        c = b0 + k < b1 ? __ldg(a.cta_list + b0 + k) : a.nchunks;
      } else {
        c = (int)atomicAdd(a.tickets + (phase & 1u), 1u);
        if (a.chunk_order) c = c < a.nchunks ? __ldg(a.chunk_order + c) : a.nchunks;
      }
    }
    return __shfl_sync(0xffffffffu, c, 0);
  }
  // after a barrier (every warp of the CTA is past its draws of this phase): the counter of this phase's
  // parity is free for the phase after next
  __device__ void reset_cta_counter() {
    if (a.cta_ptr && threadIdx.x == 0) s_cnt[phase & 1u] = 0u;
  }
  __device__ int first_chunk() { return ticket(); }
  __device__ int next_chunk(int) { return ticket(); }
  __device__ bool writer() const { return blockIdx.x == 0 && threadIdx.x == 0; }
  __device__ void clear_tickets() {
    if (threadIdx.x == 0) a.tickets[phase & 1u] = 0u;
  }
  unsigned reductions = 0;  // reductions published or pending (identical in every CTA)
  bool pending = false;     // this warp has not yet waited for the last (split) reduction
  __device__ MonoBarrier mb() const { return MonoBarrier{a.mono, a.gb.status, gridDim.x + a.phantom_ctas}; }
  __device__ bool sync() {
    const bool ok = mono_barrier(mb(), phase, [&] { clear_tickets(); });
    reset_cta_counter();
    ++phase;
    return ok;
  }
  __device__ bool reduce(int K, unsigned maxmask, bool split) {
    const bool ok = mono_barrier_combine(mb(), phase, reductions, split, a.csum, (size_t)a.nchunks, a.nchunks,
                                         a.nchunks, K, maxmask, a.stripes, a.scal, [&] { clear_tickets(); });
    reset_cta_counter();
    ++phase;
    ++reductions;
    pending = split;
    return ok;
  }
  __device__ bool sync_reduce(int K, unsigned maxmask) { return reduce(K, maxmask, false); }
  __device__ bool sync_reduce_split(int K, unsigned maxmask) { return reduce(K, maxmask, true); }
  __device__ bool await_scalars() {
    if (!pending) return true;
    pending = false;
    return mono_await(mb(), reductions);
  }
  __device__ double scal(int q) const { return ldcg(a.scal + q); }
};

// The solver body; the hybrid instantiation is inlined by force (the compiler's own choice outlines it, with
// 500-odd bytes of spills), the others as the compiler decides.
template <class T, bool IL, bool SC = false, bool HY = false, class Ctx>
__device__ int pg_body(const PGArgsT<T>& a, Ctx& ctx) {
  return pg_body_inl<T, IL, SC, HY>(a, ctx);
}

// Occupancy target: 3 resident CTAs per SM (see pg_max_grid).
template <class T, bool IL, bool SC = false, bool HY = false>
__global__ void __launch_bounds__(256, 3) k_pg_persistent(PGArgsT<T> a) {
  __shared__ double smem8[32];
  __shared__ ChunkScratchT<T> cs[8];
  __shared__ unsigned s_cnt[2];
  if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0u;
  __syncthreads();
  GridCtx<T> ctx{a, smem8, cs, s_cnt};
  if constexpr (HY) {
    pg_body_inl<T, IL, SC, HY>(a, ctx);
  } else {
    pg_body<T, IL, SC, HY>(a, ctx);
  }
}

// One problem per CTA (batched solves): phases separated by __syncthreads, scalars reduced by the CTA's
// 8 warps (the same 8-stripe combination) and kept in shared memory.
template <class T>
struct BlockCtx {
  const PGArgsT<T>& a;
  double* smem8;
  double* sscal;
  ChunkScratchT<T>* cs;
  __device__ int first_chunk() const { return threadIdx.x >> 5; }
  __device__ int next_chunk(int c) const { return c + 8; }
  __device__ bool writer() const { return threadIdx.x == 0; }
  __device__ bool sync() {
    __syncthreads();
    return true;
  }
  __device__ bool sync_reduce(int K, unsigned maxmask) {
    __syncthreads();
    block8_combine_k(a.csum, a.nchunks, K, maxmask, smem8, sscal);
    return true;
  }
  __device__ bool sync_reduce_split(int K, unsigned maxmask) { return sync_reduce(K, maxmask); }
  __device__ bool await_scalars() const { return true; }
  __device__ double scal(int q) const { return sscal[q]; }
};

// Batched solves: CTAs take problems from a queue (largest first); each runs the complete solve of its
// problem with the same arithmetic as the single-problem kernel, then writes the best iterate to r.
template <class T, bool HY = false>
__global__ void __launch_bounds__(256) k_pg_batched(PGBatchArgsT<T> ba) {
  __shared__ double smem8[32], sscal[8];
  __shared__ ChunkScratchT<T> cs[8];
  __shared__ int s_job;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_job = atomicAdd(ba.next, 1);
    __syncthreads();
    const int job = s_job;
    if (job >= ba.nproblems) return;
    const int p = ba.queue[job];
    const int c0 = ba.contact_ptr[p];
    const int n = ba.contact_ptr[p + 1] - c0;
    PGArgsT<T> a = ba.base;
    a.n = n;
    a.nchunks = (n + 31) / 32;
    a.rowptr = ba.base.rowptr + c0;
    a.b = ba.base.b + 3 * (size_t)c0;
    a.mu = ba.base.mu + c0;
    a.scaling = ba.base.scaling + c0;
    a.X0 = ba.base.X0 + 3 * (size_t)c0;
    a.X1 = ba.base.X1 + 3 * (size_t)c0;
    a.X2 = ba.base.X2 + 3 * (size_t)c0;
    a.MX0 = ba.base.MX0 + 3 * (size_t)c0;
    a.MX1 = ba.base.MX1 + 3 * (size_t)c0;
    if (ba.base.lin_momentum) {
      a.MX2 = ba.base.MX2 + 3 * (size_t)c0;
      a.MX3 = ba.base.MX3 + 3 * (size_t)c0;
    }
    a.Y = ba.base.Y + 3 * (size_t)c0;
    a.S0 = ba.base.S0 + c0;
    a.XB = ba.base.XB + 3 * (size_t)c0;
    a.Wv = ba.base.Wv + 3 * (size_t)c0;
    a.csum = ba.base.csum + 4 * (size_t)ba.chunk_ptr[p];
    a.trace = nullptr;
    a.out = ba.base.out + p;
    if constexpr (HY) {
      a.hy_d = ba.base.hy_d + 3 * (size_t)c0;
      a.hy_xref = ba.base.hy_xref + 3 * (size_t)c0;
      a.hy_wxref = ba.base.hy_wxref + 3 * (size_t)c0;
    }
    BlockCtx<T> ctx{a, smem8, sscal, cs};
    int best;
    if constexpr (HY) {
      best = pg_body_inl<T, false, false, true>(a, ctx);
    } else {
      best = pg_body<T, false>(a, ctx);
    }
    __syncthreads();
    if (n == 0) continue;
    const T* src = best == 3 ? a.XB : (best == 4 ? a.Wv : (best == 0 ? a.X0 : (best == 1 ? a.X1 : a.X2)));
    T* dst = ba.r + 3 * (size_t)c0;
    for (int k = threadIdx.x; k < 3 * n; k += blockDim.x) dst[k] = ldcg(src + k);
  }
}

// Team schedule: CTAs [team * size, team * size + size) solve one problem at a time with the single-problem
// context (dynamic chunk tickets, bounded barrier, chunk sums combined by the team's last CTAs to arrive
// (grid_barrier_combine), scalars published in the team's slot), on counters of their own. The last CTA to reach the barrier before a job takes the next problem from the queue. The
// arithmetic is that of the other schedules, so each problem's result is the same bit for bit.
template <class T>
struct TeamCtx {
  const PGArgsT<T>& a;
  double* smem8;
  ChunkScratchT<T>* cs;
  unsigned* tickets;        // 2
  unsigned* combine_count;  // 1
  double* sc;               // 8 scalars, then 32 stripe sums
  GridBarrier gb;
  int rank;
  unsigned phase = 0;
  __device__ int ticket() {
    int c = 0;
    if ((threadIdx.x & 31) == 0) c = (int)atomicAdd(tickets + (phase & 1u), 1u);
    return __shfl_sync(0xffffffffu, c, 0);
  }
  __device__ int first_chunk() { return ticket(); }
  __device__ int next_chunk(int) { return ticket(); }
  __device__ bool writer() const { return rank == 0 && threadIdx.x == 0; }
  __device__ void clear_tickets() {
    if (threadIdx.x == 0) tickets[phase & 1u] = 0u;
  }
  __device__ bool sync() {
    const bool ok = grid_barrier(gb, [&] { clear_tickets(); });
    ++phase;
    return ok;
  }
  __device__ bool sync_reduce(int K, unsigned maxmask) {
    const bool ok = grid_barrier_combine(gb, combine_count, a.csum, (size_t)a.nchunks, a.nchunks, a.nchunks, K, maxmask,
                                         sc + 8, sc, [&] { clear_tickets(); });
    ++phase;
    return ok;
  }
  __device__ bool sync_reduce_split(int K, unsigned maxmask) { return sync_reduce(K, maxmask); }
  __device__ bool await_scalars() const { return true; }
  __device__ double scal(int q) const { return ldcg(sc + q); }
};

template <class T, bool HY = false>
__global__ void __launch_bounds__(256, 3) k_pg_team(PGBatchArgsT<T> ba, PGTeamArgs ta) {
  __shared__ double smem8[32];
  __shared__ ChunkScratchT<T> cs[8];
  const int team = blockIdx.x / ta.size, rank = blockIdx.x - team * ta.size;
  unsigned* cnt = ta.counters + 8 * (size_t)team;
  const GridBarrier gb{cnt, cnt + 1, ta.status, (unsigned)ta.size};
  for (;;) {
    // the last CTA to arrive takes the next problem and clears the team's chunk tickets: the final phase of the
    // previous problem (a converged solve leaves its last product phase without a closing barrier) may have
    // drawn tickets that no barrier cleared
    if (!grid_barrier(gb, [&] {
          if (threadIdx.x == 0) {
            ta.job[team] = (int)atomicAdd((unsigned*)ba.next, 1u);
            cnt[2] = 0u;
            cnt[3] = 0u;
          }
        }))
      return;
    const int job = *(volatile int*)(ta.job + team);
    if (job >= ba.nproblems) return;
    const int p = ba.queue[job];
    const int c0 = ba.contact_ptr[p];
    const int n = ba.contact_ptr[p + 1] - c0;
    PGArgsT<T> a = ba.base;
    a.n = n;
    a.nchunks = (n + 31) / 32;
    a.rowptr = ba.base.rowptr + c0;
    a.b = ba.base.b + 3 * (size_t)c0;
    a.mu = ba.base.mu + c0;
    a.scaling = ba.base.scaling + c0;
    a.X0 = ba.base.X0 + 3 * (size_t)c0;
    a.X1 = ba.base.X1 + 3 * (size_t)c0;
    a.X2 = ba.base.X2 + 3 * (size_t)c0;
    a.MX0 = ba.base.MX0 + 3 * (size_t)c0;
    a.MX1 = ba.base.MX1 + 3 * (size_t)c0;
    if (ba.base.lin_momentum) {
      a.MX2 = ba.base.MX2 + 3 * (size_t)c0;
      a.MX3 = ba.base.MX3 + 3 * (size_t)c0;
    }
    a.Y = ba.base.Y + 3 * (size_t)c0;
    a.S0 = ba.base.S0 + c0;
    a.XB = ba.base.XB + 3 * (size_t)c0;
    a.Wv = ba.base.Wv + 3 * (size_t)c0;
    a.csum = ba.base.csum + 4 * (size_t)ba.chunk_ptr[p];
    a.trace = nullptr;
    a.out = ba.base.out + p;
    if constexpr (HY) {
      a.hy_d = ba.base.hy_d + 3 * (size_t)c0;
      a.hy_xref = ba.base.hy_xref + 3 * (size_t)c0;
      a.hy_wxref = ba.base.hy_wxref + 3 * (size_t)c0;
    }
    TeamCtx<T> ctx{a, smem8, cs, cnt + 2, cnt + 4, ta.scal + 40 * (size_t)team, gb, rank};
    int best;
    if constexpr (HY) {
      best = pg_body_inl<T, false, false, true>(a, ctx);
    } else {
      best = pg_body<T, false>(a, ctx);
    }
    if (best < 0) return;  // a wait ran out (status recorded)
    if (n == 0) continue;
    const T* src = best == 3 ? a.XB : (best == 4 ? a.Wv : (best == 0 ? a.X0 : (best == 1 ? a.X1 : a.X2)));
    T* dst = ba.r + 3 * (size_t)c0;
    for (int k = rank * (int)blockDim.x + (int)threadIdx.x; k < 3 * n; k += ta.size * (int)blockDim.x)
      dst[k] = ldcg(src + k);
  }
}

// Resident 256-thread CTAs per SM that both kernels reach (the FP64 batched kernels and their instantiations with
// FP32 correction products share launch shapes).
template <class K1, class K2>
cudaError_t occupancy_min(int* per, K1 k1, K2 k2) {
  int a = 0, b = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k1, 256, 0);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k2, 256, 0);
  *per = a < b ? a : b;
  return e;
}

template <class T>
cudaError_t launch_team_t(const PGBatchArgsT<T>& b, const PGTeamArgs& t, int grid, cudaStream_t s) {
  PGBatchArgsT<T> bc = b;
  PGTeamArgs tc = t;
  void* args[] = {&bc, &tc};
  const void* fn = (const void*)k_pg_team<T>;
  if constexpr (sizeof(T) == 8) {
    if (b.base.hy_refresh) {
      if (b.base.variant != 3 || b.base.lin_momentum || !b.base.hy_ival || !b.base.hy_d || !b.base.hy_xref ||
          !b.base.hy_wxref)
        return cudaErrorInvalidValue;
      fn = (const void*)k_pg_team<T, true>;
    }
  }
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s);
}

cudaError_t launch_pg_team(const PGBatchArgs& b, const PGTeamArgs& t, int grid, cudaStream_t s) {
  return launch_team_t(b, t, grid, s);
}

cudaError_t launch_pg_team(const PGBatchArgs32& b, const PGTeamArgs& t, int grid, cudaStream_t s) {
  return launch_team_t(b, t, grid, s);
}

int pg_team_per_sm(int device, bool fp32) {
  int per = 0;
  (void)device;
  const cudaError_t e = fp32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pg_team<float>, 256, 0)
                             : occupancy_min(&per, k_pg_team<double>, k_pg_team<double, true>);
  return e == cudaSuccess ? per : 0;
}

int pg_batched_per_sm(int device, bool fp32) {
  int per = 0;
  (void)device;
  const cudaError_t e = fp32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pg_batched<float>, 256, 0)
                             : occupancy_min(&per, k_pg_batched<double>, k_pg_batched<double, true>);
  return e == cudaSuccess ? per : 0;
}

int pg_team_grid(int device, bool fp32) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  const cudaError_t e = fp32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pg_team<float>, 256, 0)
                             : occupancy_min(&per, k_pg_team<double>, k_pg_team<double, true>);
  if (e != cudaSuccess) return 0;
  const int cap = 3;
  if (per > cap) per = cap;
  return per * sms;
}

cudaError_t launch_pg_batched(const PGBatchArgs& b, int grid, cudaStream_t s) {
  if (b.base.hy_refresh) {
    if (b.base.variant != 3 || b.base.lin_momentum || !b.base.hy_ival || !b.base.hy_d || !b.base.hy_xref ||
        !b.base.hy_wxref)
      return cudaErrorInvalidValue;
    k_pg_batched<double, true><<<grid, 256, 0, s>>>(b);
  } else {
    k_pg_batched<double><<<grid, 256, 0, s>>>(b);
  }
  return cudaGetLastError();
}

cudaError_t launch_pg_batched(const PGBatchArgs32& b, int grid, cudaStream_t s) {
  k_pg_batched<float><<<grid, 256, 0, s>>>(b);
  return cudaGetLastError();
}

int pg_batched_grid(int device, bool fp32) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  const cudaError_t e = fp32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pg_batched<float>, 256, 0)
                             : occupancy_min(&per, k_pg_batched<double>, k_pg_batched<double, true>);
  if (e != cudaSuccess) return 0;
  return per * sms;
}

cudaError_t launch_pg_persistent(const PGArgs& a, int grid, cudaStream_t s) {
  PGArgs copy = a;
  void* args[] = {&copy};
  const bool sc = a.variant == 0 || a.variant == 2;  // Standard, Conjugated
  const bool hy = a.hy_refresh != 0;                 // FP32 correction products (APGD)
  if ((sc || hy) && !a.slot0) return cudaErrorInvalidValue;  // they run on the interleaved copy only
  if (hy && (a.variant != 3 || a.lin_momentum || !a.hy_ival || !a.hy_d || !a.hy_xref || !a.hy_wxref))
    return cudaErrorInvalidValue;
  const void* fn = sc ? (const void*)k_pg_persistent<double, true, true>
                      : (hy ? (const void*)k_pg_persistent<double, true, false, true>
                            : (a.slot0 ? (const void*)k_pg_persistent<double, true>
                                       : (const void*)k_pg_persistent<double, false>));
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s);
}

cudaError_t launch_pg_persistent(const PGArgs32& a, int grid, cudaStream_t s) {
  if (!a.slot0) return cudaErrorInvalidValue;  // the FP32 solve reads the interleaved copy only
  PGArgs32 copy = a;
  void* args[] = {&copy};
  return cudaLaunchCooperativeKernel((const void*)k_pg_persistent<float, true>, dim3(grid), dim3(256), args, 0, s);
}

int pg_max_grid(int device, bool fp32, bool interleaved) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  const void* fn = fp32 ? (const void*)k_pg_persistent<float, true>
                        : (interleaved ? (const void*)k_pg_persistent<double, true>
                                       : (const void*)k_pg_persistent<double, false>);
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, 0);
  if (e != cudaSuccess) return 0;
  // Measured on the 200 000-contact problem: 3 resident CTAs per SM for FP64 (0.388 ms per APGD iteration
  // against 0.411 with 2 and 0.502 with 1; later 0.215 ms against 0.249 with 4 CTAs at 64 registers). FP32:
  // 3 CTAs at 80 registers with the block values and x loaded two blocks ahead, 0.120 ms per iteration, against
  // 0.126 at 4 CTAs (64 registers, one block ahead), 0.137 at 4 CTAs with only x ahead, 0.141 with 5 at 48
  // registers and 0.232 with 2.
  const int cap = 3;
  if (per > cap) per = cap;
  return per * sms;
}

// Sets this file's copy of the device-side wait limit on the current device.
BOGUS_GPU_WAIT_LIMIT_SETTER(set_wait_limit_pg)

}  // namespace bogus_gpu
