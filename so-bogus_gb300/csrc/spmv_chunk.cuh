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

namespace bogus_gpu {

template <class T>
struct ChunkScratchT {
  int st[33];       // row starts of the chunk (rows past n start at B1)
  T part[63][6];    // pieces (up to two products)
};
using ChunkScratch = ChunkScratchT<double>;

// NP = 1: y = init + W x. NP = 2: additionally y2 = init2 + W (x - 1) (both from the same pass over W).
// Every lane of the warp must call it (warp-uniform c). acc (and acc2) hold init on entry, the result on
// exit, for row 32c + lane (lanes past n get unspecified values).
template <int NP, class T, class Gather>
__device__ __forceinline__ void spmv_chunk(const int* __restrict__ rowptr, const int* __restrict__ col,
                                           const T* __restrict__ val, int n, int c, ChunkScratchT<T>& sh,
                                           Gather&& gather, T* acc, T* acc2 = nullptr) {
  const int lane = threadIdx.x & 31;
  const int r0 = 32 * c;
  const int r1 = min(r0 + 32, n);
  sh.st[lane] = __ldg(rowptr + min(r0 + lane, r1));
  if (lane == 0) sh.st[32] = __ldg(rowptr + r1);
  __syncwarp();
  const int B0 = sh.st[0], B1 = sh.st[32];
  const int nblk = B1 - B0;
  const int S = nblk > 0 ? (nblk + 31) / 32 : 1;
  int k = B0 + lane * S;
  const int e = min(k + S, B1);
  if (k < e) {
    int lo = 0, hi = 31;  // row containing block k: last t with st[t] <= k
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sh.st[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    int t = lo;
    int next = sh.st[t + 1];
    T p[3] = {T(0), T(0), T(0)}, q[3] = {T(0), T(0), T(0)};
    bool open = false;
    for (; k < e; ++k) {
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
      const int j = ldcs(col + k);
      T x[3];
      gather(j, x);
      const T* Bk = val + 9 * (size_t)k;
      T b[9];
#pragma unroll
      for (int e2 = 0; e2 < 9; ++e2) b[e2] = ldcs(Bk + e2);
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
    if (open) {
      T* s = sh.part[t + lane];
      s[0] = p[0]; s[1] = p[1]; s[2] = p[2];
      if (NP == 2) { s[3] = q[0]; s[4] = q[1]; s[5] = q[2]; }
    }
  }
  __syncwarp();
  if (r0 + lane < r1) {
    const int rs = sh.st[lane], re = sh.st[lane + 1];
    if (rs < re) {
      const int lf = (rs - B0) / S, ll = (re - 1 - B0) / S;
      for (int l = lf; l <= ll; ++l) {
        const T* s = sh.part[lane + l];
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
