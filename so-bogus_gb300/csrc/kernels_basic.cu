// Stand-alone kernels: 3x3-block SpMV, error function, reductions and small vector helpers.
//
// SpMV order: row i accumulates its blocks in increasing column order, as the reference's symmetric product
// (Core/Block/SparseMatrixVectorProduct.impl.hpp:89-175) does when run sequentially, cut into the
// per-lane pieces of the canonical chunk-segmented order (spmv_chunk.cuh), starting from 0 (y = W x) or from
// init_i (y = init + W x).
#include "internal.h"
#include "fp64_int.cuh"
#include "soc_device.cuh"
#include "spmv_chunk.cuh"

namespace bogus_gpu {

// One warp per 32-row chunk (canonical chunk-segmented order, spmv_chunk.cuh).
__global__ void __launch_bounds__(256) k_spmv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                              const double* __restrict__ val, const double* __restrict__ x,
                                              const double* __restrict__ init, double* __restrict__ y) {
  __shared__ ChunkScratch cs[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * 8 + warp;
  if (32 * c >= n) return;
  const int i = 32 * c + lane;
  double acc[3] = {0.0, 0.0, 0.0};
  if (init && i < n) {
    acc[0] = init[3 * i];
    acc[1] = init[3 * i + 1];
    acc[2] = init[3 * i + 2];
  }
  spmv_chunk<1>(rowptr, PlainBlocks<double>{col, val}, n, c, cs[warp],
                [&](int j, double* v) {
                  v[0] = __ldg(x + 3 * j);
                  v[1] = __ldg(x + 3 * j + 1);
                  v[2] = __ldg(x + 3 * j + 2);
                },
                acc);
  if (i < n) {
    y[3 * i] = acc[0];
    y[3 * i + 1] = acc[1];
    y[3 * i + 2] = acc[2];
  }
}

// Interleaved copy of W (InterleavedBlocks, spmv_chunk.cuh): one warp per 32-row chunk; slot (s, lane) takes
// block B0 + lane S + s when it lies in the chunk, else padding (column 0, zero values, never read).
__global__ void k_interleave(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const double* __restrict__ val, const long long* __restrict__ slot0,
                             int* __restrict__ icol, double* __restrict__ ival) {
  const int c = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (32 * c >= n) return;
  const int r1 = min(32 * c + 32, n);
  const int B0 = rowptr[32 * c], B1 = rowptr[r1];
  const int T = B1 - B0;
  const int S = T > 0 ? (T + 31) / 32 : 1;
  const long long base = slot0[c];
  for (int st = 0; st < S; ++st) {
    const int k = B0 + lane * S + st;
    const bool ok = k < B1;
    const long long slot = base + 32 * (long long)st + lane;
    icol[slot] = ok ? col[k] : 0;
    for (int e = 0; e < 9; ++e) ival[9 * base + 32 * (long long)(9 * st + e) + lane] = ok ? val[9 * (size_t)k + e] : 0.0;
  }
}

cudaError_t launch_interleave(const DevBSR& W, const long long* slot0, int* icol, double* ival, cudaStream_t s) {
  if (W.n == 0) return cudaSuccess;
  const int chunks = (W.n + 31) / 32;
  k_interleave<<<(chunks + 7) / 8, 256, 0, s>>>(W.n, W.rowptr, W.col, W.val, slot0, icol, ival);
  return cudaGetLastError();
}

// Right-hand side of an inner solve of the Cadoux fixed point (Interfaces/Cadoux.hpp:73-76): out_i = COV(y_i) + b_i
// with SOCLaw::dualityCOV, COV(y) = (mu |y_T|, 0, 0).
__global__ void k_cadoux_rhs(int n, const double* __restrict__ y, const double* __restrict__ mu,
                             const double* __restrict__ b, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double yy[3] = {y[3 * i], y[3 * i + 1], y[3 * i + 2]};
  const double s0 = duality_cov(true, mu[i], yy);
  out[3 * i] = s0 + b[3 * i];
  out[3 * i + 1] = 0.0 + b[3 * i + 1];
  out[3 * i + 2] = 0.0 + b[3 * i + 2];
}

cudaError_t launch_cadoux_rhs(int n, const double* y, const double* mu, const double* b, double* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_cadoux_rhs<<<(n + 255) / 256, 256, 0, s>>>(n, y, mu, b, out);
  return cudaGetLastError();
}

cudaError_t launch_spmv(const DevBSR& W, const double* x, const double* init, double* y, cudaStream_t s) {
  if (W.n == 0) return cudaSuccess;
  const int chunks = (W.n + 31) / 32;
  k_spmv<<<(chunks + 7) / 8, 256, 0, s>>>(W.n, W.rowptr, W.col, W.val, x, init, y);
  return cudaGetLastError();
}

// First stage of the error function (ConstrainedSolverBase::eval): per-contact law residual at
// (scaling_i x_i, u_i), reduced per 32-contact chunk by the canonical butterfly (or max).
__global__ void k_eval_chunks(int n, const double* __restrict__ x, const double* __restrict__ u,
                              const double* __restrict__ mu, const double* __restrict__ scaling, int desaxce,
                              int use_inf, double* __restrict__ chunk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (i < n) {
    const double s = scaling[i];
    const double lx[3] = {x[3 * i] * s, x[3 * i + 1] * s, x[3 * i + 2] * s};
    const double lu[3] = {u[3 * i], u[3 * i + 1], u[3 * i + 2]};
    v = law_eval(desaxce != 0, mu[i], lx, lu);
  }
  v = use_inf ? warp_max_butterfly(v) : warp_sum_butterfly(v);
  if ((threadIdx.x & 31) == 0 && i - (int)(threadIdx.x & 31) < n) chunk[i >> 5] = v;
}

cudaError_t launch_eval_chunks(int n, const double* x, const double* u, const double* mu, const double* scaling,
                               bool desaxce, bool use_inf, double* chunk, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int nt = ((n + 31) / 32) * 32;
  k_eval_chunks<<<(nt + 255) / 256, 256, 0, s>>>(n, x, u, mu, scaling, desaxce ? 1 : 0, use_inf ? 1 : 0, chunk);
  return cudaGetLastError();
}

// Second stage: one CTA of 8 warps; out = total (or total / scale_div when scale_div > 0).
__global__ void __launch_bounds__(256) k_combine(const double* chunk, int nchunks, int is_max, double scale_div,
                                                 double* out) {
  __shared__ double smem8[8];
  const double t = block8_combine(chunk, nchunks, is_max != 0, smem8);
  if (threadIdx.x == 0) *out = scale_div > 0.0 ? t / scale_div : t;
}

cudaError_t launch_combine(const double* chunk, int nchunks, bool is_max, double scale_div, double* out,
                           cudaStream_t s) {
  k_combine<<<1, 256, 0, s>>>(chunk, nchunks, is_max ? 1 : 0, scale_div, out);
  return cudaGetLastError();
}

// Diagonal block positions and the solver scalings max(1, trace(W_ii)/3)
// (ConstrainedSolverBase.impl.hpp:78-118; 1 when the diagonal block is absent).
__global__ void k_diag_scaling(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                               const double* __restrict__ val, int* __restrict__ diag, double* __restrict__ scaling) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int p = -1;
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
    if (col[k] == i) { p = k; break; }
  diag[i] = p;
  double s = 1.0;
  if (p >= 0) {
    const double* B = val + 9 * (size_t)p;
    s = dmax(1.0, ((B[0] + B[4]) + B[8]) / 3.0);
  }
  scaling[i] = s;
}

// ---- W from its lower triangle: structure checks and the pattern of both triangles on the device ----------
// rowptr has been checked on the host (starts at 0, monotone), so every row's blocks lie in the uploaded col.
// out[0] = the smallest row whose columns are out of range, above the diagonal or not strictly increasing
// (unchanged when none is); out[1] += the number of diagonal blocks.
__global__ void k_check_lower(int n, const int* __restrict__ rowptr, const int* __restrict__ col, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k0 = rowptr[i], k1 = rowptr[i + 1];
  for (int k = k0; k < k1; ++k) {
    const int j = col[k];
    if (j < 0 || j > i || (k > k0 && col[k - 1] >= j)) {
      atomicMin(out, i);
      return;
    }
  }
  if (k1 > k0 && col[k1 - 1] == i) atomicAdd(out + 1, 1);
}

// Structure of a both-triangle BSR handed over in device memory (rowptr: n + 1 entries, col: nnzb): every row
// must have 0 <= rowptr[i] <= rowptr[i + 1] <= nnzb with rowptr[0] = 0 and rowptr[n] = nnzb, strictly increasing
// columns in [0, n) and its diagonal block. out[0] receives the smallest offending row (it must start above
// n, e.g. 0x7f7f7f7f from a byte memset). Columns are read only inside [0, nnzb), whatever rowptr holds.
__global__ void k_check_full(int n, int nnzb, const int* __restrict__ rowptr, const int* __restrict__ col, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k0 = rowptr[i], k1 = rowptr[i + 1];
  bool bad = k0 < 0 || k1 < k0 || k1 > nnzb || (i == 0 && k0 != 0) || (i == n - 1 && k1 != nnzb);
  bool diag = false;
  if (!bad) {
    int prev = -1;
    for (int k = k0; k < k1; ++k) {
      const int j = col[k];
      if (j < 0 || j >= n || j <= prev) {
        bad = true;
        break;
      }
      diag |= j == i;
      prev = j;
    }
  }
  if (bad || !diag) atomicMin(out, i);
}

// upper[j] = number of blocks (i, j), i > j, of the lower triangle (the transposed blocks row j receives)
__global__ void k_count_upper(int n, const int* __restrict__ rowptr, const int* __restrict__ col, int* upper) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
    if (col[k] != i) atomicAdd(upper + col[k], 1);
}

// frowptr = exclusive prefix sum of the full row lengths (lower length + upper[i]), in three coalesced passes:
// the sum of each tile of 1024 rows, an exclusive scan of the tile sums (one CTA), then each tile's scan plus
// its offset. frowptr[n] receives the total.
__device__ __forceinline__ int full_row_length(int i, int n, const int* __restrict__ rowptr, const int* __restrict__ upper) {
  return i < n ? (__ldg(rowptr + i + 1) - __ldg(rowptr + i)) + __ldg(upper + i) : 0;
}
// inclusive scan of v over the 1024 threads of the CTA; warp totals in ws[32]
__device__ __forceinline__ int cta_inclusive_scan(int v, int* ws) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) ws[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int w = ws[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    ws[lane] = w;
  }
  __syncthreads();
  return v + (warp > 0 ? ws[warp - 1] : 0);
}
__global__ void __launch_bounds__(1024) k_rowlen_tiles(int n, const int* __restrict__ rowptr,
                                                       const int* __restrict__ upper, int* tile_sum) {
  __shared__ int ws[32];
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const int v = cta_inclusive_scan(full_row_length(i, n, rowptr, upper), ws);
  if (threadIdx.x == 1023) tile_sum[blockIdx.x] = v;
}
__global__ void __launch_bounds__(1024) k_scan_tiles(int ntiles, int* tile_sum) {
  __shared__ int ws[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < ntiles; base += 1024) {
    const int k = base + threadIdx.x;
    const int v = k < ntiles ? tile_sum[k] : 0;
    const int inc = cta_inclusive_scan(v, ws);
    const int c = carry;
    if (k < ntiles) tile_sum[k] = c + inc - v;  // exclusive
    __syncthreads();
    if (threadIdx.x == 1023) carry = c + inc;
    __syncthreads();
  }
}
__global__ void __launch_bounds__(1024) k_rowptr_tiles(int n, const int* __restrict__ rowptr,
                                                       const int* __restrict__ upper, const int* __restrict__ tile_off,
                                                       int* frowptr) {
  __shared__ int ws[32];
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const int v = full_row_length(i, n, rowptr, upper);
  const int inc = cta_inclusive_scan(v, ws) + tile_off[blockIdx.x];
  if (i < n) frowptr[i] = inc - v;
  if (i == n - 1) frowptr[n] = inc;
}

// Row i of the full matrix: its lower blocks (columns <= i, in order), then the transposed blocks (i, j) of
// rows j > i in increasing j. The lower part is placed directly; the upper part by a cursor per row, then
// sorted by column (rows of the upper part are short), so the layout is that of the host's expansion.
__global__ void k_place_lower(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                              const int* __restrict__ frowptr, int* fcol, int* src, int* cursor) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k0 = rowptr[i], k1 = rowptr[i + 1];
  for (int k = k0; k < k1; ++k) {
    const int p = frowptr[i] + (k - k0);
    fcol[p] = col[k];
    src[p] = k;
    const int j = col[k];
    if (j != i) {
      const int q = frowptr[j] + (rowptr[j + 1] - rowptr[j]) + atomicAdd(cursor + j, 1);
      fcol[q] = i;
      src[q] = ~k;
    }
  }
}

__global__ void k_sort_upper(int n, const int* __restrict__ rowptr, const int* __restrict__ frowptr, int* fcol,
                             int* src) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int b = frowptr[j] + (rowptr[j + 1] - rowptr[j]), e = frowptr[j + 1];
  for (int p = b + 1; p < e; ++p) {
    const int c = fcol[p], s = src[p];
    int q = p - 1;
    while (q >= b && fcol[q] > c) {
      fcol[q + 1] = fcol[q];
      src[q + 1] = src[q];
      --q;
    }
    fcol[q + 1] = c;
    src[q + 1] = s;
  }
}

cudaError_t launch_check_lower(int n, const int* rowptr, const int* col, int* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_check_lower<<<(n + 255) / 256, 256, 0, s>>>(n, rowptr, col, out);
  return cudaGetLastError();
}

cudaError_t launch_check_full(int n, int nnzb, const int* rowptr, const int* col, int* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0x7f, sizeof(int), s);
  if (e != cudaSuccess || n <= 0) return e;
  k_check_full<<<(n + 255) / 256, 256, 0, s>>>(n, nnzb, rowptr, col, out);
  return cudaGetLastError();
}

cudaError_t launch_full_pattern(int n, const int* rowptr, const int* col, int* upper, int* cursor, int* frowptr,
                                int* fcol, int* src, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(upper, 0, sizeof(int) * n, s);
  if (e != cudaSuccess) return e;
  const int g = (n + 255) / 256;
  k_count_upper<<<g, 256, 0, s>>>(n, rowptr, col, upper);
  // the tile sums use `cursor` (n ints; ceil(n / 1024) <= n), zeroed afterwards for k_place_lower
  const int ntiles = (n + 1023) / 1024;
  k_rowlen_tiles<<<ntiles, 1024, 0, s>>>(n, rowptr, upper, cursor);
  k_scan_tiles<<<1, 1024, 0, s>>>(ntiles, cursor);
  k_rowptr_tiles<<<ntiles, 1024, 0, s>>>(n, rowptr, upper, cursor, frowptr);
  if ((e = cudaMemsetAsync(cursor, 0, sizeof(int) * n, s)) != cudaSuccess) return e;
  k_place_lower<<<g, 256, 0, s>>>(n, rowptr, col, frowptr, fcol, src, cursor);
  k_sort_upper<<<g, 256, 0, s>>>(n, rowptr, frowptr, fcol, src);
  return cudaGetLastError();
}

// 3-vectors between the caller's contact order and a permuted one: dst_k = src_perm[k] (or dst_perm[k] = src_k)
__global__ void k_permute3(int n, const int* __restrict__ perm, const double* __restrict__ src, double* dst,
                           int inverse) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int p = perm[k];
  for (int c = 0; c < 3; ++c) {
    if (inverse) dst[3 * (size_t)p + c] = src[3 * (size_t)k + c];
    else dst[3 * (size_t)k + c] = src[3 * (size_t)p + c];
  }
}

cudaError_t launch_permute3(int n, const int* perm, const double* src, double* dst, bool inverse, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_permute3<<<(n + 255) / 256, 256, 0, s>>>(n, perm, src, dst, inverse ? 1 : 0);
  return cudaGetLastError();
}

// *flag = 1 when some value is NaN or infinite (exponent field all ones).
__global__ void k_any_nonfinite(size_t m, const double* __restrict__ v, int* flag) {
  bool bad = false;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m; k += (size_t)gridDim.x * blockDim.x)
    bad |= ((__double_as_longlong(v[k]) >> 52) & 0x7ff) == 0x7ff;
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *flag = 1;
}

cudaError_t launch_any_nonfinite(size_t m, const double* v, int* flag, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  const size_t blocks = (m + 255) / 256;
  k_any_nonfinite<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, s>>>(m, v, flag);
  return cudaGetLastError();
}

// Both triangles from the lower one: block p is lower block src[p], or lower block ~src[p] transposed when
// src[p] < 0 (the placement of the host's symmetric expansion: rows sorted by column).
__global__ void k_expand_lower(int nnz, const int* __restrict__ src, const double* __restrict__ low,
                               double* __restrict__ full) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nnz) return;
  const int q = src[p];
  const double* B = low + 9 * (size_t)(q >= 0 ? q : ~q);
  double* F = full + 9 * (size_t)p;
  if (q >= 0) {
#pragma unroll
    for (int e = 0; e < 9; ++e) F[e] = B[e];
  } else {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) F[3 * r + c] = B[3 * c + r];
  }
}

cudaError_t launch_expand_lower(int nnz, const int* src, const double* low, double* full, cudaStream_t s) {
  if (nnz <= 0) return cudaSuccess;
  k_expand_lower<<<(nnz + 255) / 256, 256, 0, s>>>(nnz, src, low, full);
  return cudaGetLastError();
}

cudaError_t launch_diag_and_scaling(const DevBSR& W, double* scaling, cudaStream_t s) {
  if (W.n == 0) return cudaSuccess;
  k_diag_scaling<<<(W.n + 255) / 256, 256, 0, s>>>(W.n, W.rowptr, W.col, W.val, W.diag, scaling);
  return cudaGetLastError();
}

__global__ void k_add(int m, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) y[k] = a[k] + b[k];
}

cudaError_t launch_add(int m, const double* a, const double* b, double* y, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  k_add<<<(m + 255) / 256, 256, 0, s>>>(m, a, b, y);
  return cudaGetLastError();
}

__global__ void k_scale_scalar(double* p, double divisor) { *p = *p / divisor; }

cudaError_t launch_scale_scalar(double* p, double divisor, cudaStream_t s) {
  k_scale_scalar<<<1, 1, 0, s>>>(p, divisor);
  return cudaGetLastError();
}

template <class S, class D>
__global__ void k_convert(size_t m, const S* __restrict__ src, D* __restrict__ dst) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) dst[k] = (D)src[k];
}

cudaError_t launch_convert(size_t m, const double* src, float* dst, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  k_convert<double, float><<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_convert(size_t m, const float* src, double* dst, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  k_convert<float, double><<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, src, dst);
  return cudaGetLastError();
}

// FP64 FMA throughput: eight independent chains per thread, enough warps to fill every SM.
__global__ void k_fp64_peak(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t measure_fp64_peak(int device, double* tflops) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int nb = sms * 8, nt = 256, iters = 2048;
  double* out = nullptr;
  if ((e = cudaMalloc(&out, sizeof(double) * nb * nt)) != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    k_fp64_peak<<<nb, nt>>>(out, iters, 0.999, 1e-3);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *tflops = 2.0 * 8.0 * iters * (double)nb * nt / (best * 1e-3) / 1e12;
  return e;
}

// Integer-pipe division, square root and exact scalings (fp64_int.cuh) against the hardware operations on
// n generated operands: uniformly random bit patterns, exponents near 1, extreme mantissas, and quotients and
// roots close to exact. out[0], out[1], out[2] count the mismatches of division, square root and scalings.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void k_check_fp64_ops(long long n, unsigned long long seed, unsigned long long* out) {
  using namespace ipipe;
  unsigned long long bad[3] = {0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const uint64_t r = seed + 8 * (uint64_t)i;
    uint64_t ua = mix64(r), ub = mix64(r + 1);
    const int mode = (int)(i & 7);
    if (mode == 1 || mode == 2) {
      ua = (ua & ~(0x7FFull << 52)) | ((uint64_t)(923 + mix64(r + 2) % 200) << 52);
      ub = (ub & ~(0x7FFull << 52)) | ((uint64_t)(923 + mix64(r + 3) % 200) << 52);
    } else if (mode == 3) {
      const uint64_t pat[6] = {0, kMant, kMant - 1, 1, kMant >> 1, (kMant >> 1) + 1};
      ua = (ua & ~kMant & ~(0x7FFull << 52)) | ((uint64_t)(1000 + mix64(r + 2) % 48) << 52) | pat[mix64(r + 3) % 6];
      ub = (ub & ~kMant & ~(0x7FFull << 52)) | ((uint64_t)(1000 + mix64(r + 4) % 48) << 52) | pat[mix64(r + 5) % 6];
    } else if (mode == 4) {
      const double b = from_bits((ub & kMant) | (1023ull << 52));
      const double q = (double)(long long)(mix64(r + 2) >> 40) + 0.5 * (double)(mix64(r + 3) & 1);
      ua = to_bits(__dmul_rn(q, b)) + mix64(r + 4) % 3 - 1;
      ub = to_bits(b);
    }
    const double a = from_bits(ua), b = from_bits(ub);
    const double q0 = a / b, q1 = div_rn(a, b);
    if (to_bits(q0) != to_bits(q1) && q0 == q0) ++bad[0];
    uint64_t ux = ua & ~(1ull << 63);
    if (mode == 5) {
      const double t = (double)(long long)(mix64(r + 5) >> 37);
      ux = to_bits(__dmul_rn(t, t)) + mix64(r + 6) % 3 - 1;
    }
    const double x = from_bits(ux);
    const double s0 = sqrt(x), s1 = sqrt_rn(x);
    if (to_bits(s0) != to_bits(s1) && s0 == s0) ++bad[1];
    if (a == a) {
      if (to_bits(scale2<-1>(a)) != to_bits(__dmul_rn(a, 0.5))) ++bad[2];
      if (to_bits(scale2<1>(a)) != to_bits(__dmul_rn(a, 2.0))) ++bad[2];
      if (__dadd_rn(a, -a) == 0.0 && to_bits(plus_zero(a)) != to_bits(__dadd_rn(a, 0.0))) ++bad[2];
    }
  }
  for (int k = 0; k < 3; ++k)
    if (bad[k]) atomicAdd(out + k, bad[k]);
}

cudaError_t check_fp64_ops(int device, long long n, unsigned long long seed, long long* mismatches) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  unsigned long long* out = nullptr;
  if ((e = cudaMalloc(&out, 3 * sizeof(unsigned long long))) != cudaSuccess) return e;
  cudaMemset(out, 0, 3 * sizeof(unsigned long long));
  k_check_fp64_ops<<<sms * 8, 256>>>(n, seed, out);
  unsigned long long h[3] = {0, 0, 0};
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(h, out, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(out);
  for (int k = 0; k < 3; ++k) mismatches[k] = (long long)h[k];
  return e;
}

}  // namespace bogus_gpu
