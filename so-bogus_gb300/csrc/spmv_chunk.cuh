// Warp-cooperative 3x3-block product of one 32-row chunk in the canonical chunk-segmented order.
//
// The chunk's blocks [B0, B1) (rows 32c .. 32c+31, contiguous in the BSR arrays) are cut into 32 consecutive
// segments of S = ceil((B1 - B0) / 32) blocks, one per lane, so every lane runs the same number of FP64 FMAs
// whatever the row lengths (GB300 charges a masked-off lane the same FP64 pipe time as an active one). A
// lane walks its segment and, for each row the segment meets, accumulates a piece: the chain
// acc_r = fma(B[r][0], x0, acc_r); fma(B[r][1], x1, .); fma(B[r][2], x2, .) over the row's blocks inside the
// segment, from 0. Segments and rows are two partitions of [B0, B1) into consecutive intervals, so the
// pieces are at most 63 and piece (row t, lane l) can live in slot t + l of a small shared array. The lane
// owning row t then adds its pieces to the initial value in segment order:
//   y_t = ((init_t + piece(t, l_first)) + piece(t, l_first + 1)) + ...
// This is the order the CPU oracle's spmv() follows.
#pragma once

#include "device_common.cuh"
#include "fp64_int.cuh"

namespace bogus_gpu {

template <class T>
struct ChunkScratchT {
  int st[33];       // row starts of the chunk (rows past n start at B1)
  T part[63][6];    // pieces (up to two products)
};
using ChunkScratch = ChunkScratchT<double>;

// Where the blocks live. Both sources give block k (original BSR index), met by a lane at step s of its
// segment (k = B0 + lane S + s).
//
// PlainBlocks: the BSR arrays themselves, column col[k], values val[9k .. 9k+8]. A warp's 32 lanes read
// 32 segments S blocks apart, so each load instruction touches 32 separate sectors.
template <class T>
struct PlainBlocks {
  const int* __restrict__ col;
  const T* __restrict__ val;
  __device__ __forceinline__ void chunk(int) {}
  __device__ __forceinline__ int column(int k, int) const { return ldcs(col + k); }
  __device__ __forceinline__ T value(int k, int, int e) const { return ldcs(val + 9 * (size_t)k + e); }
};

// InterleavedBlocks: each chunk stored step-major for coalesced loads. Chunk c owns slots
// [slot0[c], slot0[c] + 32 S); the block of lane l at step s is slot slot0[c] + 32 s + l, its column is
// icol[slot] and its value e is ival[9 slot0[c] + 32 (9 s + e) + l]. At a given step the 32 lanes read
// consecutive words: one 128-byte (int, float) or 256-byte (double) access per load instruction. Slots
// past the chunk's last block are padding and never read. Built by launch_interleave (kernels_basic.cu).
template <class T>
struct InterleavedBlocks {
  const int* __restrict__ icol;
  const T* __restrict__ ival;
  const long long* __restrict__ slot0;
  long long base = 0;
  __device__ __forceinline__ void chunk(int c) { base = __ldg(slot0 + c); }
  __device__ __forceinline__ int column(int, int s) const {
    return ldcs(icol + base + 32 * (long long)s + (threadIdx.x & 31));
  }
  __device__ __forceinline__ T value(int, int s, int e) const {
    return ldcs(ival + 9 * base + 32 * (long long)(9 * s + e) + (threadIdx.x & 31));
  }
};

// 0 + v for the first piece of a row when the initial value is +0: v itself with -0 turned into +0, as a bit
// operation for FP64 (off the FP64 unit), the plain addition for FP32.
__device__ __forceinline__ double zero_plus(double v) { return ipipe::plus_zero(v); }
__device__ __forceinline__ float zero_plus(float v) { return 0.f + v; }

// NP = 1: y = init + W x. NP = 2: additionally y2 = init2 + W (x - 1) (both from the same pass over W).
// Every lane of the warp must call it (warp-uniform c). acc (and acc2) hold init on entry, the result on
// exit, for row 32c + lane (lanes past n get unspecified values). ZeroInit: every init is +0, so the first
// piece of a row is placed rather than added (the same value).
template <int NP, bool ZeroInit = false, class T, class Src, class Gather>
__device__ __forceinline__ void spmv_chunk(const int* __restrict__ rowptr, Src src, int n, int c,
                                           ChunkScratchT<T>& sh, Gather&& gather, T* acc, T* acc2 = nullptr) {
  const int lane = threadIdx.x & 31;
  src.chunk(c);
  const int r0 = 32 * c;
  const int r1 = min(r0 + 32, n);
  sh.st[lane] = __ldg(rowptr + min(r0 + lane, r1));
  if (lane == 0) sh.st[32] = __ldg(rowptr + r1);
  __syncwarp();
  const int B0 = sh.st[0], B1 = sh.st[32];
  const int nblk = B1 - B0;
  const int S = nblk > 0 ? (nblk + 31) / 32 : 1;
  const int k0 = B0 + lane * S;
  const int e = min(k0 + S, B1);
  // Every lane runs the same S steps (lanes past the end of their segment, or with none, are predicated
  // off) and the warp reconverges after the per-lane row-boundary flush, so the 9 FMAs of a step issue once
  // per warp: lanes cross row boundaries at different steps, and a divergent flush left to itself would
  // split the warp and issue the FMAs once per divergent group.
  int t = 31;
  if (k0 < e) {
    int lo = 0, hi = 31;  // row containing block k0: last t with st[t] <= k0
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sh.st[mid] <= k0) lo = mid;
      else hi = mid - 1;
    }
    t = lo;
  }
  int next = sh.st[t + 1];
  T p[3] = {T(0), T(0), T(0)}, q[3] = {T(0), T(0), T(0)};
  bool open = false;
  // The next block's column index and gathered x are loaded one block ahead, so the dependent col -> x load
  // chain of block k + 1 overlaps the accumulation of block k (the arithmetic order is unchanged).
  // FP32: the block values and gathered x are loaded two blocks ahead (the FP32 solve is bound by load
  // latency); FP64: x one block ahead (the FP64 solve is bound by its FMA pipe; registers set occupancy)
  constexpr bool kAhead = sizeof(T) == 4;
  T xn[3] = {T(0), T(0), T(0)}, xm[3] = {T(0), T(0), T(0)};
  T bn[9], bm[9];
  if (k0 < e) gather(src.column(k0, 0), xn);
  if (kAhead) {
    if (k0 + 1 < e) gather(src.column(k0 + 1, 1), xm);
#pragma unroll
    for (int e2 = 0; e2 < 9; ++e2) bn[e2] = k0 < e ? src.value(k0, 0, e2) : T(0);
#pragma unroll
    for (int e2 = 0; e2 < 9; ++e2) bm[e2] = k0 + 1 < e ? src.value(k0 + 1, 1, e2) : T(0);
  }
  for (int step = 0; step < S; ++step) {
    const int k = k0 + step;
    const bool valid = k < e;
    const T x[3] = {xn[0], xn[1], xn[2]};
    T b[9];
    if (kAhead) {
#pragma unroll
      for (int e2 = 0; e2 < 9; ++e2) b[e2] = bn[e2];
#pragma unroll
      for (int e2 = 0; e2 < 9; ++e2) bn[e2] = bm[e2];
      xn[0] = xm[0]; xn[1] = xm[1]; xn[2] = xm[2];
      if (k + 2 < e) gather(src.column(k + 2, step + 2), xm);
#pragma unroll
      for (int e2 = 0; e2 < 9; ++e2) bm[e2] = k + 2 < e ? src.value(k + 2, step + 2, e2) : T(0);
    } else {
      if (k + 1 < e) gather(src.column(k + 1, step + 1), xn);
#pragma unroll
      for (int e2 = 0; e2 < 9; ++e2) b[e2] = valid ? src.value(k, step, e2) : T(0);
    }
    if (valid) {
      while (k >= next) {
        if (open) {
          T* s = sh.part[t + lane];
          s[0] = p[0]; s[1] = p[1]; s[2] = p[2];
          if (NP == 2) { s[3] = q[0]; s[4] = q[1]; s[5] = q[2]; }
          p[0] = p[1] = p[2] = T(0);
          q[0] = q[1] = q[2] = T(0);
          open = false;
        }
        ++t;
        next = sh.st[t + 1];
      }
    }
    __syncwarp();
    if (valid) {
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        T s = p[r];
        s = fma(b[3 * r + 0], x[0], s);
        s = fma(b[3 * r + 1], x[1], s);
        s = fma(b[3 * r + 2], x[2], s);
        p[r] = s;
      }
      if (NP == 2) {
        const T d0 = x[0] - T(1), d1 = x[1] - T(1), d2 = x[2] - T(1);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          T s = q[r];
          s = fma(b[3 * r + 0], d0, s);
          s = fma(b[3 * r + 1], d1, s);
          s = fma(b[3 * r + 2], d2, s);
          q[r] = s;
        }
      }
      open = true;
    }
  }
  if (open) {
    T* s = sh.part[t + lane];
    s[0] = p[0]; s[1] = p[1]; s[2] = p[2];
    if (NP == 2) { s[3] = q[0]; s[4] = q[1]; s[5] = q[2]; }
  }
  __syncwarp();
  if (r0 + lane < r1) {
    const int rs = sh.st[lane], re = sh.st[lane + 1];
    if (rs < re) {
      const int lf = (rs - B0) / S, ll = (re - 1 - B0) / S;
      for (int l = lf; l <= ll; ++l) {
        const T* s = sh.part[lane + l];
        if (ZeroInit && l == lf) {
          acc[0] = zero_plus(s[0]);
          acc[1] = zero_plus(s[1]);
          acc[2] = zero_plus(s[2]);
          if (NP == 2) {
            acc2[0] = zero_plus(s[3]);
            acc2[1] = zero_plus(s[4]);
            acc2[2] = zero_plus(s[5]);
          }
          continue;
        }
        acc[0] = acc[0] + s[0];
        acc[1] = acc[1] + s[1];
        acc[2] = acc[2] + s[2];
        if (NP == 2) {
          acc2[0] = acc2[0] + s[3];
          acc2[1] = acc2[1] + s[4];
          acc2[2] = acc2[2] + s[5];
        }
      }
    }
  }
  __syncwarp();
}

}  // namespace bogus_gpu
