// Projected Gauss-Seidel sweep (Core/BlockSolvers/GaussSeidel.impl.hpp:62-124), level by level.
//
// The sweep order is the contacts' own order or, with coloring, the order of Coloring::compute after the
// contact permutation (MecheInterface.cpp:330-337); the problem is renumbered so that the sweep visits
// contacts 0, 1, 2, ... In the sequential sweep, contact i reads the new value of every neighbour visited
// before it and the old value of every neighbour visited after it. Give each contact the level
// 1 + max(level of its earlier neighbours): contacts of one level share no block of W, and processing the
// levels in increasing order gives every contact exactly the values the sequential sweep gives it. So one
// launch per level reproduces the sequential result bit for bit: thread i gathers its split row
// b_i - reg_i x_i + sum_{j != i} W_ij x_j (columns in increasing order, canonical chain), runs the local
// Coulomb / SOC solver and applies the (possibly halved) update.
//
// The skip heuristic (:107-117) depends on ndxRef, a running maximum over the contacts already visited in
// the sweep. It is reproduced exactly after each sweep: the level kernels record every solved contact's
// step norm and a per-tile maximum (max is order-independent), and k_gs_skip turns them into the
// sequential prefix maximum and the skip counters.
#include "internal.h"
#include "soc_device.cuh"

namespace bogus_gpu {

__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// One warp per CTA: a level is latency bound (long dependent FP64 chains per contact), so its contacts are
// spread over as many SMs as possible.
__global__ void __launch_bounds__(32) k_gs_level(GSArgs a, int l0, int l1, int parity) {
  const int t = l0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= l1) return;
  const int i = a.order[t];
  if (a.skip[i]) {
    a.skip[i] = (unsigned char)(a.skip[i] - 1);
    a.processed[i] = 0;
    return;
  }
  double lx[3] = {a.x[3 * i], a.x[3 * i + 1], a.x[3 * i + 2]};
  const double reg = a.reg[i];
  double lb[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) lb[k] = a.b[3 * i + k] - reg * lx[k];
  const int k1 = a.rowptr[i + 1];
  for (int k = a.rowptr[i]; k < k1; ++k) {
    const int j = a.col[k];
    if (j == i) continue;
    const double* B = a.val + 9 * (size_t)k;
    const double x0 = a.x[3 * j], x1 = a.x[3 * j + 1], x2 = a.x[3 * j + 2];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double s = lb[r];
      s = fma(B[3 * r + 0], x0, s);
      s = fma(B[3 * r + 1], x1, s);
      s = fma(B[3 * r + 2], x2, s);
      lb[r] = s;
    }
  }
  double A[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) A[e] = a.local[9 * (size_t)i + e];
  double ldx[3] = {-lx[0], -lx[1], -lx[2]};
  const double sc = a.scaling[i];
  const bool ok = law_solve_local(a.desaxce != 0, a.strat, A, lb, lx, a.mu[i], sc);
#pragma unroll
  for (int k = 0; k < 3; ++k) ldx[k] = ldx[k] + lx[k];
  if (!ok) {
    ldx[0] *= .5;
    ldx[1] *= .5;
    ldx[2] *= .5;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) a.x[3 * i + k] = a.x[3 * i + k] + ldx[k];
  const double s2 = sc * sc;
  const double nx2 = s2 * sq3(lx);
  const double ndx2 = s2 * sq3(ldx);
  a.nx2[i] = nx2;
  a.ndx2[i] = ndx2;
  a.processed[i] = 1;
  // ndxRef only grows through "if (ndx2 > ndxRef)": NaN never enters; non-negative doubles order as their bits
  if (ndx2 > 0.0) {
    const int ntiles = (a.n + kGSTile - 1) / kGSTile;
    atomicMax(a.tile_max + parity * ntiles + i / kGSTile, dbits(ndx2));
  }
}

cudaError_t launch_gs_level(const GSArgs& a, int l0, int l1, int parity, cudaStream_t s) {
  if (l1 <= l0) return cudaSuccess;
  k_gs_level<<<(l1 - l0 + 31) / 32, 32, 0, s>>>(a, l0, l1, parity);
  return cudaGetLastError();
}

// One CTA per tile of kGSTile contacts (sweep order). ndxRef entering the tile is the maximum of the
// value at the start of the sweep and of every earlier tile's maximum; inside the tile an inclusive
// prefix maximum over the solved contacts gives each contact's ndxRef, then the skip rule (:115-117).
// The tile maxima of the next sweep (other parity) are cleared here; CTA 0 stores the ndxRef at the end
// of the sweep in the other parity slot.
__global__ void __launch_bounds__(kGSTile) k_gs_skip(GSArgs a, int parity, double abs_skip_tol, double skip_tol,
                                                     int abs_skip_iters) {
  __shared__ double warp_max[kGSTile / 32];
  __shared__ double s_prefix;
  const int ntiles = (a.n + kGSTile - 1) / kGSTile;
  const int t = blockIdx.x;
  const unsigned long long* tm = a.tile_max + parity * ntiles;
  const double start = a.ndx_ref[parity];
  if (threadIdx.x < 32) {
    double m = start;
    for (int k = threadIdx.x; k < t; k += 32) {
      const double v = __longlong_as_double((long long)tm[k]);
      m = (v > m) ? v : m;
    }
    m = warp_max_butterfly(m);
    if (threadIdx.x == 0) s_prefix = m;
  }
  if (t == 0 && threadIdx.x < 32) {
    double m = start;
    for (int k = threadIdx.x; k < ntiles; k += 32) {
      const double v = __longlong_as_double((long long)tm[k]);
      m = (v > m) ? v : m;
    }
    m = warp_max_butterfly(m);
    if (threadIdx.x == 0) a.ndx_ref[1 - parity] = m;
  }
  const int i = t * kGSTile + threadIdx.x;
  const bool live = i < a.n && a.processed[i];
  const double nd = live ? a.ndx2[i] : 0.0;
  // inclusive prefix max inside the tile
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double v = nd;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double o = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v = (o > v) ? o : v;
  }
  if (lane == 31) warp_max[warp] = v;
  __syncthreads();
  double before = s_prefix;
  for (int w = 0; w < warp; ++w) before = (warp_max[w] > before) ? warp_max[w] : before;
  const double ref = (v > before) ? v : before;
  if (live) {
    const double nx2 = a.nx2[i];
    if (dmin(nx2, nd) < abs_skip_tol || nd < skip_tol * dmin(nx2, ref)) a.skip[i] = (unsigned char)abs_skip_iters;
  }
  if (threadIdx.x == 0) a.tile_max[(1 - parity) * ntiles + t] = 0ull;
}

cudaError_t launch_gs_skip(const GSArgs& a, int parity, double abs_skip_tol, double skip_tol, int abs_skip_iters,
                           cudaStream_t s) {
  const int ntiles = (a.n + kGSTile - 1) / kGSTile;
  if (ntiles == 0) return cudaSuccess;
  k_gs_skip<<<ntiles, kGSTile, 0, s>>>(a, parity, abs_skip_tol, skip_tol, abs_skip_iters);
  return cudaGetLastError();
}

}  // namespace bogus_gpu
