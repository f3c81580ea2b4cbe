// Projected Gauss-Seidel sweep (Core/BlockSolvers/GaussSeidel.impl.hpp:62-124).
//
// The sweep order is the contacts' own order or, with coloring, the order of Coloring::compute after the
// contact permutation (MecheInterface.cpp:330-337); the problem is renumbered so that the sweep visits
// contacts 0, 1, 2, ... In the sequential sweep, contact i reads the new value of every neighbour visited
// before it and the old value of every neighbour visited after it. Give each contact the level
// 1 + max(level of its earlier neighbours): contacts of one level share no block of W, and any schedule that
// visits a contact after its earlier neighbours and before its later ones gives every contact exactly the
// values the sequential sweep gives it, so the result is the same bit for bit. Visiting contact i: gather its
// split row b_i - reg_i x_i + sum_{j != i} W_ij x_j (columns in increasing order, canonical chain), run the
// local Coulomb / SOC solver and apply the (possibly halved) update.
//
// The skip heuristic (:107-117) depends on ndxRef, a running maximum over the contacts already visited in
// the sweep. It is reproduced exactly after each sweep: the sweep records every solved contact's step norm
// and a per-tile maximum (max is order-independent), and k_gs_skip turns them into the sequential prefix
// maximum and the skip counters.
#include "internal.h"
#include "soc_device.cuh"

namespace bogus_gpu {

__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// Dataflow sweep: one launch visits every contact. Each warp takes the next contact in level order from a
// counter and waits only for the earlier neighbours of its contact (flags set when they are visited): a
// contact starts as soon as its own earlier neighbours are done, not when the slowest contact of the previous
// level is (a launch per level would wait for it; the sweep is latency bound, the local solves being long
// dependent FP64 chains). Level order rather than sweep order keeps the contacts in flight mostly independent
// (consecutive contacts of the sweep often share a body). An earlier neighbour has been visited (its flag was
// set after its x was written), a later neighbour has not (it waits for this contact's flag), so every contact
// sees the values of the sequential sweep. A warp waits only for contacts of lower levels, handed out before its own and so already taken by
// running warps: the sweep always progresses. Every wait is bounded (wait_limit_ns()); a wait that runs
// out records BOGUS_GPU_TIMEOUT and the warp stops.
__device__ __forceinline__ bool gs_wait_done(const unsigned* f, unsigned tag, const int* status) {
  if (ld_acquire_u32(f) == tag) return true;
  const unsigned long long t0 = global_timer_ns();
  unsigned spins = 0;
  for (;;) {
    __nanosleep(64);
    if (ld_acquire_u32(f) == tag) return true;
    if ((++spins & 63u) == 0) {
      if (ld_relaxed_i32(status) != 0) return false;
      if (global_timer_ns() - t0 > wait_limit_ns()) {
        atomicCAS(const_cast<int*>(status), 0, (int)BOGUS_GPU_TIMEOUT);
        return false;
      }
    }
  }
}

// The whole warp works on its contact: lanes stage the row's blocks (before waiting, they do not change) and the
// neighbours' x (after); lanes 0-2 accumulate one component of the split row each (the three chains of the
// scalar loop); every lane then runs the same local solve, whose eigenvalue step is shared across the lanes
// (local_solve<true>), and lane 0 writes the result.
__global__ void __launch_bounds__(32 * kGSFlowWarps) k_gs_flow(GSArgs a, int parity) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ double sB[kGSFlowWarps][32][12];
  __shared__ int sJ[kGSFlowWarps][32];
  __shared__ double sHq[kGSFlowWarps][16];
  const unsigned tag = ld_acquire_u32(a.flow + 1);
  const int ntiles = (a.n + kGSTile - 1) / kGSTile;
  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(a.flow, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= (unsigned)a.n) return;
    const int i = a.order[t];
    const unsigned char sk = a.skip[i];
    __syncwarp();  // every lane has read the counter before lane 0 changes it: the branch below is warp-uniform
    if (sk) {
      if (lane == 0) {
        a.skip[i] = (unsigned char)(sk - 1);
        a.processed[i] = 0;
        st_release_u32(a.done + i, tag);
      }
      continue;
    }
    double lx[3] = {ldcg(a.x + 3 * i), ldcg(a.x + 3 * i + 1), ldcg(a.x + 3 * i + 2)};
    const double reg = a.reg[i];
    const int rc = lane < 3 ? lane : 0;  // the component lanes 0-2 accumulate
    double lbr = a.b[3 * i + rc] - reg * lx[rc];
    const int k0 = a.rowptr[i], k1 = a.rowptr[i + 1];
    bool ok_wait = true;
    for (int base = k0; base < k1; base += 32) {
      const int k = base + lane;
      int j = i;
      if (k < k1) {
        j = a.col[k];
        sJ[w][lane] = j;
        const double* B = a.val + 9 * (size_t)k;
#pragma unroll
        for (int e = 0; e < 9; ++e) sB[w][lane][e] = B[e];
        if (j < i && !gs_wait_done(a.done + j, tag, a.status)) ok_wait = false;
        sB[w][lane][9] = ldcg(a.x + 3 * j);
        sB[w][lane][10] = ldcg(a.x + 3 * j + 1);
        sB[w][lane][11] = ldcg(a.x + 3 * j + 2);
      }
      if (!__all_sync(0xffffffffu, ok_wait)) return;
      if (lane < 3) {
        const int cnt = min(32, k1 - base);
        double s = lbr;
        for (int q = 0; q < cnt; ++q) {
          if (sJ[w][q] == i) continue;
          const double* B = sB[w][q];
          s = fma(B[3 * rc + 0], B[9], s);
          s = fma(B[3 * rc + 1], B[10], s);
          s = fma(B[3 * rc + 2], B[11], s);
        }
        lbr = s;
      }
      __syncwarp();
    }
    const double lb[3] = {__shfl_sync(0xffffffffu, lbr, 0), __shfl_sync(0xffffffffu, lbr, 1),
                          __shfl_sync(0xffffffffu, lbr, 2)};
    double A[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) A[e] = a.local[9 * (size_t)i + e];
    double ldx[3] = {-lx[0], -lx[1], -lx[2]};
    const double sc = a.scaling[i];
    const bool ok = law_solve_local<true>(a.desaxce != 0, a.strat, A, lb, lx, a.mu[i], sc, sHq[w]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) ldx[k] = ldx[k] + lx[k];
      if (!ok) {
        ldx[0] *= .5;
        ldx[1] *= .5;
        ldx[2] *= .5;
      }
      double xn[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) xn[k] = ldcg(a.x + 3 * i + k) + ldx[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) a.x[3 * i + k] = xn[k];
      const double s2 = sc * sc;
      const double nx2 = s2 * sq3(lx);
      const double ndx2 = s2 * sq3(ldx);
      a.nx2[i] = nx2;
      a.ndx2[i] = ndx2;
      a.processed[i] = 1;
      if (ndx2 > 0.0) atomicMax(a.tile_max + parity * ntiles + i / kGSTile, dbits(ndx2));
      __threadfence();
      st_release_u32(a.done + i, tag);
    }
    __syncwarp();
  }
}

cudaError_t launch_gs_flow(const GSArgs& a, int grid, int parity, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  k_gs_flow<<<grid, 32 * kGSFlowWarps, 0, s>>>(a, parity);
  return cudaGetLastError();
}

int gs_flow_grid(int device) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_gs_flow, 32 * kGSFlowWarps, 0) != cudaSuccess) return 0;
  return per * sms;
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
  // the next dataflow sweep hands out positions from 0 under a new tag
  if (t == 0 && threadIdx.x == 0 && a.flow) {
    a.flow[0] = 0u;
    a.flow[1] = a.flow[1] + 1u;
  }
}

cudaError_t launch_gs_skip(const GSArgs& a, int parity, double abs_skip_tol, double skip_tol, int abs_skip_iters,
                           cudaStream_t s) {
  const int ntiles = (a.n + kGSTile - 1) / kGSTile;
  if (ntiles == 0) return cudaSuccess;
  k_gs_skip<<<ntiles, kGSTile, 0, s>>>(a, parity, abs_skip_tol, skip_tol, abs_skip_iters);
  return cudaGetLastError();
}

// ---- matrix-free sweep (ProductGaussSeidel<HType, MInvType, true>, ProductGaussSeidel.impl.hpp:108-296) -----
// Levels from the shared bodies (contacts sharing a body never share a level); every body's Mx = M^-1 H^T x is
// read and updated by one contact at a time, in sweep order:
//   lb = b_i - local_i x_i + sum_t H_t Mx_(body t)  (rowMultiply), local solve, x_i += dx,
//   Mx_(body t) += T_t dx  (colMultiply, T = M^-1 H^T).
// Orders: local_i x_i per row with the dot3 chain, subtracted from b_i; each slot's H_t Mx row as a chain over the
// dofs from 0, added to lb; T_t dx with the dot3 chain, added to Mx.
// Same dataflow schedule as k_gs_flow. Two contacts depend on each other when they share a body, and the
// updates of Mx_b by the contacts on body b form a chain in sweep order, so contact i waits only for the
// previous contact on each of its bodies (pdep, -1 when none): when that one is done, every earlier update of
// Mx_b is in. A later contact on the body waits (directly or along the chain) for this one.
__global__ void __launch_bounds__(32 * kGSFlowWarps) k_pgs_flow(GSArgs a, int parity) {
  // the whole warp works on its contact, as in k_gs_flow: lanes 0-2 form one component of lb each, every lane
  // runs the same local solve, lanes 0..d-1 update one dof of Mx each
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ double sHq[kGSFlowWarps][16];
  const unsigned tag = ld_acquire_u32(a.flow + 1);
  const int ntiles = (a.n + kGSTile - 1) / kGSTile;
  const int d = a.d;
  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(a.flow, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= (unsigned)a.n) return;
    const int i = a.order[t];
    bool ok_wait = true;
    if (lane < 2) {
      const int j = a.pdep[2 * i + lane];
      if (j >= 0 && !gs_wait_done(a.done + j, tag, a.status)) ok_wait = false;
    }
    if (!__all_sync(0xffffffffu, ok_wait)) return;
    const unsigned char sk = a.skip[i];
    __syncwarp();  // every lane has read the counter before lane 0 changes it: the branch below is warp-uniform
    if (sk) {
      if (lane == 0) {
        a.skip[i] = (unsigned char)(sk - 1);
        a.processed[i] = 0;
        st_release_u32(a.done + i, tag);
      }
      continue;
    }
    double lx[3] = {ldcg(a.x + 3 * i), ldcg(a.x + 3 * i + 1), ldcg(a.x + 3 * i + 2)};
    double A[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) A[e] = a.local[9 * (size_t)i + e];
    const int rc = lane < 3 ? lane : 0;
    double lbr = a.b[3 * i + rc] - dot3(&A[3 * rc], lx);
    for (int sl = 0; sl < 2; ++sl) {
      const int body = a.cb[2 * i + sl];
      if (body < 0) continue;
      const double* Hs = a.H + (2 * (size_t)i + sl) * 3 * d;
      const double* mx = a.Mx + (size_t)body * d;
      double s = 0.0;
      for (int m = 0; m < d; ++m) s = fma(Hs[rc * d + m], ldcg(mx + m), s);
      lbr = lbr + s;
    }
    const double lb[3] = {__shfl_sync(0xffffffffu, lbr, 0), __shfl_sync(0xffffffffu, lbr, 1),
                          __shfl_sync(0xffffffffu, lbr, 2)};
    double ldx[3] = {-lx[0], -lx[1], -lx[2]};
    const double sc = a.scaling[i];
    const bool ok = law_solve_local<true>(a.desaxce != 0, a.strat, A, lb, lx, a.mu[i], sc, sHq[w]);
#pragma unroll
    for (int k = 0; k < 3; ++k) ldx[k] = ldx[k] + lx[k];
    if (!ok) {
      ldx[0] *= .5;
      ldx[1] *= .5;
      ldx[2] *= .5;
    }
    for (int sl = 0; sl < 2; ++sl) {
      const int body = a.cb[2 * i + sl];
      if (body < 0 || lane >= d) continue;
      const double* Ts = a.T + (2 * (size_t)i + sl) * d * 3;
      double* mx = a.Mx + (size_t)body * d;
      const int m = lane;
      mx[m] = ldcg(mx + m) + fma(Ts[m * 3 + 2], ldx[2], fma(Ts[m * 3 + 1], ldx[1], Ts[m * 3] * ldx[0]));
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) {
      double xn[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) xn[k] = ldcg(a.x + 3 * i + k) + ldx[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) a.x[3 * i + k] = xn[k];
      const double s2 = sc * sc;
      const double nx2 = s2 * sq3(lx);
      const double ndx2 = s2 * sq3(ldx);
      a.nx2[i] = nx2;
      a.ndx2[i] = ndx2;
      a.processed[i] = 1;
      if (ndx2 > 0.0) atomicMax(a.tile_max + parity * ntiles + i / kGSTile, dbits(ndx2));
      __threadfence();
      st_release_u32(a.done + i, tag);
    }
    __syncwarp();
  }
}

cudaError_t launch_pgs_flow(const GSArgs& a, int grid, int parity, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  k_pgs_flow<<<grid, 32 * kGSFlowWarps, 0, s>>>(a, parity);
  return cudaGetLastError();
}

int pgs_flow_grid(int device) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pgs_flow, 32 * kGSFlowWarps, 0) != cudaSuccess) return 0;
  return per * sms;
}

// local_i = sum_t H_t T_t: W's diagonal block in the order of the assembly (slots in body order, dofs inner)
__global__ void k_pgs_local(int n, int d, const int* __restrict__ cb, const double* __restrict__ H,
                            const double* __restrict__ T, double* __restrict__ local) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double acc = 0.0;
      for (int sl = 0; sl < 2; ++sl) {
        if (cb[2 * i + sl] < 0) continue;
        const double* Hs = H + (2 * (size_t)i + sl) * 3 * d;
        const double* Ts = T + (2 * (size_t)i + sl) * d * 3;
        for (int m = 0; m < d; ++m) acc = fma(Hs[r * d + m], Ts[m * 3 + c], acc);
      }
      local[9 * (size_t)i + 3 * r + c] = acc;
    }
}

cudaError_t launch_pgs_local(int n, int d, const int* cb, const double* H, const double* T, double* local,
                             cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_pgs_local<<<(n + 127) / 128, 128, 0, s>>>(n, d, cb, H, T, local);
  return cudaGetLastError();
}

// Mx_b = sum over b's incidences (increasing contact) of T x_i, one fma chain per dof
__global__ void k_pgs_mx(int nbodies, int d, const int* __restrict__ bptr, const int* __restrict__ bent,
                         const double* __restrict__ T, const double* __restrict__ x, double* __restrict__ Mx) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbodies) return;
  for (int m = 0; m < d; ++m) {
    double acc = 0.0;
    for (int e = bptr[b]; e < bptr[b + 1]; ++e) {
      const int ent = bent[e];
      const int i = ent >> 1;
      const double* Ts = T + (size_t)ent * d * 3;
      acc = fma(Ts[m * 3], x[3 * i], acc);
      acc = fma(Ts[m * 3 + 1], x[3 * i + 1], acc);
      acc = fma(Ts[m * 3 + 2], x[3 * i + 2], acc);
    }
    Mx[(size_t)b * d + m] = acc;
  }
}

cudaError_t launch_pgs_mx(int nbodies, int d, const int* bptr, const int* bent, const double* T, const double* x,
                          double* Mx, cudaStream_t s) {
  if (nbodies <= 0) return cudaSuccess;
  k_pgs_mx<<<(nbodies + 127) / 128, 128, 0, s>>>(nbodies, d, bptr, bent, T, x, Mx);
  return cudaGetLastError();
}

// y = b + H Mx, each slot's row chain added to y_i
__global__ void k_pgs_y(int n, int d, const int* __restrict__ cb, const double* __restrict__ H,
                        const double* __restrict__ Mx, const double* __restrict__ b, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[3] = {b[3 * i], b[3 * i + 1], b[3 * i + 2]};
  for (int sl = 0; sl < 2; ++sl) {
    const int body = cb[2 * i + sl];
    if (body < 0) continue;
    const double* Hs = H + (2 * (size_t)i + sl) * 3 * d;
    for (int r = 0; r < 3; ++r) {
      double s = 0.0;
      for (int m = 0; m < d; ++m) s = fma(Hs[r * d + m], Mx[(size_t)body * d + m], s);
      v[r] = v[r] + s;
    }
  }
  y[3 * i] = v[0];
  y[3 * i + 1] = v[1];
  y[3 * i + 2] = v[2];
}

cudaError_t launch_pgs_y(int n, int d, const int* cb, const double* H, const double* Mx, const double* b, double* y,
                         cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_pgs_y<<<(n + 127) / 128, 128, 0, s>>>(n, d, cb, H, Mx, b, y);
  return cudaGetLastError();
}

// Sets this file's copy of the device-side wait limit on the current device.
BOGUS_GPU_WAIT_LIMIT_SETTER(set_wait_limit_gs)

}  // namespace bogus_gpu
