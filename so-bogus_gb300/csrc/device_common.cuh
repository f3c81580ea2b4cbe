// Device building blocks shared by the solver kernels: cache-hinted loads, the canonical reduction of
// per-contact values, and a bounded grid barrier for the persistent (cooperative) solver kernels.
#pragma once

#include <cstdint>

#include "bogus_gpu.h"

namespace bogus_gpu {

constexpr int kWarp = 32;

// Loads of data written earlier in the same kernel by other CTAs must bypass L1 (it is not coherent).
__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }
// W streams through once per pass; keep it from evicting the L2-resident vectors.
__device__ __forceinline__ double ldcs(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ldcs(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int ldcs(const int* p) { return __ldcs(p); }

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long atom_add_acq_rel_u64(unsigned long long* p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.add.acq_rel.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Canonical chunk reduction: lane l of a warp holds value l of a 32-contact chunk; xor butterfly.
__device__ __forceinline__ double warp_sum_butterfly(double v) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
// Two or four warp sums at once, each with exactly the tree of warp_sum_butterfly (at every step a lane adds
// its partner's partial to its own, partners at distances 16, 8, 4, 2, 1), but sharing the first steps: at
// distance 16 the lower half keeps the first value(s) and the upper half the others, each lane receiving
// its partner's copy of the value it keeps; at distance 8 (four values) each half splits again. Two values
// cost 5 adds instead of 10, four values 6 instead of 20. Results: warp_sum2 leaves sum(a) in lanes 0-15 and
// sum(b) in lanes 16-31; warp_sum4 leaves sum(a), sum(b), sum(c), sum(d) in lanes 0-7, 8-15, 16-23, 24-31.
__device__ __forceinline__ double warp_sum2_butterfly(double a, double b) {
  const bool hi = (threadIdx.x & 16) != 0;
  double v = (hi ? b : a) + __shfl_xor_sync(0xffffffffu, hi ? a : b, 16);
#pragma unroll
  for (int off = 8; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
__device__ __forceinline__ double warp_sum4_butterfly(double a, double b, double c, double d) {
  const bool hi = (threadIdx.x & 16) != 0;
  const double x = (hi ? c : a) + __shfl_xor_sync(0xffffffffu, hi ? a : c, 16);
  const double y = (hi ? d : b) + __shfl_xor_sync(0xffffffffu, hi ? b : d, 16);
  const bool h8 = (threadIdx.x & 8) != 0;
  double v = (h8 ? y : x) + __shfl_xor_sync(0xffffffffu, h8 ? x : y, 8);
#pragma unroll
  for (int off = 4; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

__device__ __forceinline__ double warp_max_butterfly(double v) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, v, off);
    v = (v < o) ? o : v;
  }
  return v;
}

// Second stage of the canonical reduction, executed by one CTA of exactly 8 warps: chunk sums are
// split into 8 stripes of ceil(C/8) chunks; warp k reduces stripe k (lane l sums chunks start+l,
// start+l+32, ... sequentially, then a butterfly), and the 8 stripe sums are added left to right.
// is_max selects the max-combination (infinity norm). Every thread returns the total.
__device__ __forceinline__ double block8_combine(const double* s, int C, bool is_max, double* smem8) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int per = (C + 7) / 8;
  const int b = warp * per;
  const int e = min(C, b + per);
  double p = 0.0;
  if (is_max) {
    for (int c = b + lane; c < e; c += 32) {
      const double v = ldcg(s + c);
      p = (v < p) ? p : v;
    }
    p = warp_max_butterfly(p);
  } else {
    for (int c = b + lane; c < e; c += 32) p = p + ldcg(s + c);
    p = warp_sum_butterfly(p);
  }
  if (lane == 0) smem8[warp] = p;
  __syncthreads();
  double total = smem8[0];
  for (int k = 1; k < 8; ++k) {
    const double q = smem8[k];
    total = is_max ? ((q < total) ? total : q) : total + q;
  }
  __syncthreads();
  return total;
}

// block8_combine for K <= 4 quantities at once (value q's chunk sums at s + q * C; bit q of maxmask selects
// the max-combination for it), with the same order per quantity. The loads of 4 chunks x K quantities are
// issued before their adds, so one CTA reduces all the scalars of a phase in a few L2 round trips instead of
// one round trip per chunk and quantity. Thread 0 receives the totals in out[0..K).
__device__ __forceinline__ void block8_combine_k(const double* s, int C, int K, unsigned maxmask, double* smem32,
                                                 double* out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int per = (C + 7) / 8;
  const int b = warp * per;
  const int e = min(C, b + per);
  double p[4] = {0.0, 0.0, 0.0, 0.0};
  int c = b + lane;
  for (; c + 96 < e; c += 128) {
    double v[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int u = 0; u < 4; ++u) v[q][u] = q < K ? ldcg(s + (size_t)q * C + c + 32 * u) : 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if ((maxmask >> q) & 1u) p[q] = (v[q][u] < p[q]) ? p[q] : v[q][u];
        else p[q] = p[q] + v[q][u];
      }
  }
  for (; c < e; c += 32)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (q >= K) continue;
      const double v = ldcg(s + (size_t)q * C + c);
      if ((maxmask >> q) & 1u) p[q] = (v < p[q]) ? p[q] : v;
      else p[q] = p[q] + v;
    }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (q >= K) continue;
    const double v = ((maxmask >> q) & 1u) ? warp_max_butterfly(p[q]) : warp_sum_butterfly(p[q]);
    if (lane == 0) smem32[8 * q + warp] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < K; ++q) {
      const bool mx = (maxmask >> q) & 1u;
      double total = smem32[8 * q];
      for (int k = 1; k < 8; ++k) {
        const double v = smem32[8 * q + k];
        total = mx ? ((v < total) ? total : v) : total + v;
      }
      out[q] = total;
    }
  }
  __syncthreads();
}

// Limit of every device-side wait (grid barriers, flag waits), in nanoseconds of %globaltimer. Each
// translation unit holds its own copy in its module; the host sets them all, per device, through
// bogus_gpu_set_wait_limit (the setters are defined by BOGUS_GPU_WAIT_LIMIT_SETTER in the kernel files).
constexpr unsigned long long kDefaultWaitLimitNs = 4000000000ull;
static __device__ unsigned long long g_wait_limit_ns = kDefaultWaitLimitNs;
__device__ __forceinline__ unsigned long long wait_limit_ns() {
  return *reinterpret_cast<const volatile unsigned long long*>(&g_wait_limit_ns);
}
#define BOGUS_GPU_WAIT_LIMIT_SETTER(name)                                 \
  cudaError_t name(unsigned long long ns) {                               \
    return cudaMemcpyToSymbol(g_wait_limit_ns, &ns, sizeof(ns));          \
  }

// Bounded grid barrier for cooperative launches. The last CTA to arrive runs `last_fn` (with all its
// threads) before releasing the others, so final reductions cost one CTA's work, not a second barrier.
// Every wait is bounded: after wait_limit_ns() the waiting CTA records BOGUS_GPU_TIMEOUT in *status and
// returns false; a CTA that sees a non-zero status also returns false. All threads of a CTA get the
// same return value.

struct GridBarrier {
  unsigned* count;
  unsigned* gen;
  int* status;
  unsigned parties;  // CTAs taking part (0: the whole grid)
};

template <class LastFn>
__device__ __forceinline__ bool grid_barrier(const GridBarrier& gb, LastFn&& last_fn) {
  __shared__ int s_last, s_ok;
  __shared__ unsigned s_gen;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned my_gen = ld_acquire_u32(gb.gen);
    s_gen = my_gen;
    const unsigned prev = atom_add_acq_rel_u32(gb.count, 1u);
    s_last = (prev == (gb.parties ? gb.parties : gridDim.x) - 1) ? 1 : 0;
    s_ok = 1;
    if (!s_last) {
      const unsigned long long t0 = global_timer_ns();
      unsigned spins = 0;
      while (ld_acquire_u32(gb.gen) == my_gen) {
        if (ld_relaxed_i32(gb.status) != 0) { s_ok = 0; break; }
        if ((++spins & 255u) == 0 && global_timer_ns() - t0 > wait_limit_ns()) {
          atomicCAS(gb.status, 0, (int)BOGUS_GPU_TIMEOUT);
          s_ok = 0;
          break;
        }
        __nanosleep(40);
      }
    }
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    last_fn();
    __syncthreads();
    if (threadIdx.x == 0) {
      *gb.count = 0u;
      __threadfence();
      st_release_u32(gb.gen, s_gen + 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) s_ok = (s_ok != 0 && ld_relaxed_i32(gb.status) == 0) ? 1 : 0;
  __syncthreads();
  const bool ok = s_ok != 0;
  __syncthreads();
  return ok;
}

// The stripe stage of the canonical reduction, for a CTA that combines stripes role, role + m, ... < 8:
// warp q < K reduces quantity q (chunk sums at s + q * stride; count0 chunks for q = 0, count1 for q > 0),
// stripes of ceil(count / 8) chunks, lane l adding chunks start + l, start + l + 32, ... in turn from 0
// (sum, or maximum where bit q of maxmask is set), then a butterfly; the stripe sum goes to
// stripes[8 q + stripe]. Loads are issued 8 (then 4) per lane ahead of their additions, which keep the order.
__device__ __forceinline__ void combine_stripes(const double* s, size_t stride, int count0, int count1, int K,
                                                unsigned maxmask, int role, int m, double* stripes) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp >= K) return;
  const int C = warp == 0 ? count0 : count1;
  const int per = (C + 7) / 8;
  const bool mx = (maxmask >> warp) & 1u;
  const double* q = s + (size_t)warp * stride;
  for (int st = role; st < 8; st += m) {
    const int e = min(C, st * per + per);
    double p = 0.0;
    int c = st * per + lane;
    for (; c + 224 < e; c += 256) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = ldcg(q + c + 32 * u);
#pragma unroll
      for (int u = 0; u < 8; ++u) p = mx ? ((v[u] < p) ? p : v[u]) : p + v[u];
    }
    for (; c + 96 < e; c += 128) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = ldcg(q + c + 32 * u);
#pragma unroll
      for (int u = 0; u < 4; ++u) p = mx ? ((v[u] < p) ? p : v[u]) : p + v[u];
    }
    for (; c < e; c += 32) {
      const double v = ldcg(q + c);
      p = mx ? ((v < p) ? p : v) : p + v;
    }
    p = mx ? warp_max_butterfly(p) : warp_sum_butterfly(p);
    if (lane == 0) stripes[8 * warp + st] = p;
  }
}

// Bounded grid barrier that also reduces K <= 4 quantities of chunk sums into out[0..K) in the canonical
// order of block8_combine / block8_combine_k. Quantity q's sums are at s + q * stride, over count0 chunks for
// q = 0 and count1 chunks for q > 0. Each is split into 8 stripes of ceil(count / 8) chunks, lane l of a stripe
// summing chunks start + l, start + l + 32, ... in turn, a butterfly per stripe, the 8 stripe sums left to
// right. The combination is spread over the last m = min(8, parties) CTAs to arrive: each waits until every
// CTA has arrived, then reduces stripes role, role + m, ... with one warp per quantity (the chains of a
// stripe run on different SM sub-partitions, and the 8 stripes on different SMs), and writes the stripe sums
// to stripes[8 q + k]. The last of them to finish adds the stripe sums, runs `last_fn` and releases the
// grid. The order of every addition is the one block8_combine_k uses, so the totals are identical. Every
// wait is bounded as in grid_barrier.
template <class LastFn>
__device__ __forceinline__ bool grid_barrier_combine(const GridBarrier& gb, unsigned* combine_count, const double* s,
                                                     size_t stride, int count0, int count1, int K, unsigned maxmask,
                                                     double* stripes, double* out, LastFn&& last_fn) {
  __shared__ int s_role, s_ok, s_final;
  __shared__ unsigned s_gen;
  const unsigned P = gb.parties ? gb.parties : gridDim.x;
  const unsigned m = P < 8u ? P : 8u;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned my_gen = ld_acquire_u32(gb.gen);
    s_gen = my_gen;
    const unsigned prev = atom_add_acq_rel_u32(gb.count, 1u);
    s_role = prev >= P - m ? (int)(prev - (P - m)) : -1;
    s_ok = 1;
    s_final = 0;
    if (s_role >= 0) {  // wait for every CTA's chunk sums
      const unsigned long long t0 = global_timer_ns();
      unsigned spins = 0;
      while (ld_acquire_u32(gb.count) < P) {
        if (ld_relaxed_i32(gb.status) != 0) { s_ok = 0; break; }
        if ((++spins & 255u) == 0 && global_timer_ns() - t0 > wait_limit_ns()) {
          atomicCAS(gb.status, 0, (int)BOGUS_GPU_TIMEOUT);
          s_ok = 0;
          break;
        }
        __nanosleep(20);
      }
      __threadfence();
    }
  }
  __syncthreads();
  if (s_role >= 0 && s_ok) {
    combine_stripes(s, stride, count0, count1, K, maxmask, s_role, (int)m, stripes);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      s_final = atom_add_acq_rel_u32(combine_count, 1u) == m - 1u ? 1 : 0;
      if (s_final) __threadfence();
    }
    __syncthreads();
    if (s_final) {
      if ((int)threadIdx.x < K) {
        const int q = threadIdx.x;
        const bool mx = (maxmask >> q) & 1u;
        double total = ldcg(stripes + 8 * q);
        for (int k = 1; k < 8; ++k) {
          const double v = ldcg(stripes + 8 * q + k);
          total = mx ? ((v < total) ? total : v) : total + v;
        }
        out[q] = total;
      }
      last_fn();
      __syncthreads();
      if (threadIdx.x == 0) {
        *gb.count = 0u;
        *combine_count = 0u;
        __threadfence();
        st_release_u32(gb.gen, s_gen + 1u);
      }
    }
  }
  if (threadIdx.x == 0 && !s_final && s_ok) {
    const unsigned long long t0 = global_timer_ns();
    unsigned spins = 0;
    while (ld_acquire_u32(gb.gen) == s_gen) {
      if (ld_relaxed_i32(gb.status) != 0) { s_ok = 0; break; }
      if ((++spins & 255u) == 0 && global_timer_ns() - t0 > wait_limit_ns()) {
        atomicCAS(gb.status, 0, (int)BOGUS_GPU_TIMEOUT);
        s_ok = 0;
        break;
      }
      __nanosleep(40);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) s_ok = (s_ok != 0 && ld_relaxed_i32(gb.status) == 0) ? 1 : 0;
  __syncthreads();
  const bool ok = s_ok != 0;
  __syncthreads();
  return ok;
}

// Dynamic work split: warps take 32-contact (or 32-body) chunks from a ticket counter, one per phase parity,
// cleared by the last CTA of the barrier that ends the phase (every draw of the phase is done by then), so SMs
// whose sub-partitions finish early take more chunks. Chunk sums are stored by chunk index, so the reduction
// order does not depend on which warp handled a chunk.
struct Tickets {
  unsigned* t;         // 2 counters, zero at launch
  unsigned phase = 0;  // barriers passed (identical in every CTA)
  __device__ int next() {
    int c = 0;
    if ((threadIdx.x & 31) == 0) c = (int)atomicAdd(t + (phase & 1u), 1u);
    return __shfl_sync(0xffffffffu, c, 0);
  }
  // run by every thread of the barrier's last CTA
  __device__ void clear() {
    if (threadIdx.x == 0) t[phase & 1u] = 0u;
  }
};

// ---- grid barrier on monotonic counters (single-problem persistent solvers) ------------------------------
// mono[0] counts CTA arrivals, mono[1] finished stripe combinations, mono[2] published reductions; all start
// at zero at launch and only grow. Barrier k of a launch is complete when mono[0] reaches parties (k + 1),
// reduction r is published when mono[2] reaches r + 1. Since no counter is ever reset, a CTA may leave a
// barrier as soon as every CTA has arrived, while the reduction of that barrier is still being combined (a
// split reduction): the next phase's work that does not need the scalars overlaps the combination, and a warp
// waits for the publication (mono_await) only where it needs them. Every wait is bounded as in grid_barrier.
struct MonoBarrier {
  unsigned long long* mono;
  int* status;
  unsigned parties;
};

// one thread: wait until *p >= target; false (and status set on a timeout) when the wait ends otherwise
__device__ __forceinline__ bool spin_until_geq(const unsigned long long* p, unsigned long long target, int* status,
                                               unsigned sleep_ns) {
  const unsigned long long t0 = global_timer_ns();
  unsigned spins = 0;
  while (ld_acquire_u64(p) < target) {
    if (ld_relaxed_i32(status) != 0) return false;
    if ((++spins & 255u) == 0 && global_timer_ns() - t0 > wait_limit_ns()) {
      atomicCAS(status, 0, (int)BOGUS_GPU_TIMEOUT);
      return false;
    }
    __nanosleep(sleep_ns);
  }
  return true;
}

// Barrier k without a reduction; the last CTA to arrive runs `last_fn` (all its threads), which must not be
// needed by the other CTAs before the next barrier.
template <class LastFn>
__device__ __forceinline__ bool mono_barrier(const MonoBarrier& mb, unsigned k, LastFn&& last_fn) {
  __shared__ int s_ok, s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long target = (unsigned long long)mb.parties * (k + 1ull);
    const unsigned long long prev = atom_add_acq_rel_u64(mb.mono, 1ull);
    s_last = prev == target - 1 ? 1 : 0;
    s_ok = s_last ? 1 : (spin_until_geq(mb.mono, target, mb.status, 20) ? 1 : 0);
  }
  __syncthreads();
  if (s_last) last_fn();
  if (threadIdx.x == 0) s_ok = (s_ok != 0 && ld_relaxed_i32(mb.status) == 0) ? 1 : 0;
  __syncthreads();
  const bool ok = s_ok != 0;
  __syncthreads();
  return ok;
}

// Barrier k with reduction r of K <= 4 quantities, in the canonical order of grid_barrier_combine (the last
// min(8, parties) CTAs to arrive combine one stripe each; the last of them to finish adds the stripe sums into
// out[0..K) and publishes). split = false: every CTA leaves after the publication. split = true: a CTA leaves
// once every CTA has arrived (the combining CTAs after their stripe), and reads out[] after mono_await(r + 1).
template <class LastFn>
__device__ __forceinline__ bool mono_barrier_combine(const MonoBarrier& mb, unsigned k, unsigned r, bool split,
                                                     const double* s, size_t stride, int count0, int count1, int K,
                                                     unsigned maxmask, double* stripes, double* out, LastFn&& last_fn) {
  __shared__ int s_role, s_ok, s_final, s_last;
  const unsigned P = mb.parties;
  const unsigned m = P < 8u ? P : 8u;
  const unsigned long long target = (unsigned long long)P * (k + 1ull);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long prev = atom_add_acq_rel_u64(mb.mono, 1ull);
    s_last = prev == target - 1 ? 1 : 0;
    s_role = prev >= target - m ? (int)(prev - (target - m)) : -1;
    s_ok = 1;
    s_final = 0;
    if (s_role >= 0) {  // every CTA's chunk sums are needed
      if (!s_last) s_ok = spin_until_geq(mb.mono, target, mb.status, 20) ? 1 : 0;
      __threadfence();
    }
  }
  __syncthreads();
  if (s_last) last_fn();
  if (s_role >= 0 && s_ok) {
    combine_stripes(s, stride, count0, count1, K, maxmask, s_role, (int)m, stripes);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      s_final = atom_add_acq_rel_u64(mb.mono + 1, 1ull) == (unsigned long long)m * (r + 1ull) - 1 ? 1 : 0;
      if (s_final) __threadfence();
    }
    __syncthreads();
    if (s_final) {
      if ((int)threadIdx.x < K) {
        const int q = threadIdx.x;
        const bool mx = (maxmask >> q) & 1u;
        double total = ldcg(stripes + 8 * q);
        for (int j = 1; j < 8; ++j) {
          const double v = ldcg(stripes + 8 * q + j);
          total = mx ? ((v < total) ? total : v) : total + v;
        }
        out[q] = total;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        st_release_u64(mb.mono + 2, r + 1ull);
      }
    }
  }
  if (threadIdx.x == 0 && s_ok) {
    if (!split) s_ok = spin_until_geq(mb.mono + 2, r + 1ull, mb.status, 40) ? 1 : 0;
    else if (s_role < 0) s_ok = spin_until_geq(mb.mono, target, mb.status, 20) ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) s_ok = (s_ok != 0 && ld_relaxed_i32(mb.status) == 0) ? 1 : 0;
  __syncthreads();
  const bool ok = s_ok != 0;
  __syncthreads();
  return ok;
}

// One warp: wait until reduction `published` - 1 is published (mono[2] >= published). Every lane of the warp
// must call it; the lanes read the scalars after it returns.
__device__ __forceinline__ bool mono_await(const MonoBarrier& mb, unsigned long long published) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) ok = spin_until_geq(mb.mono + 2, published, mb.status, 40) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

}  // namespace bogus_gpu
