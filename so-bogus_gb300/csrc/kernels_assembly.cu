// Delassus assembly W = H M^-1 H^T and b = w - H M^-1 f on the device
// (DualFrictionProblem::computeFrom, Interfaces/FrictionProblem.cpp:30-40; block products of
// Core/Block/SparseMatrixMatrixProduct.impl.hpp:295-349).
//
// Each contact has at most two body slots ordered by body index, with a 3 x ndof Jacobian block per slot.
// Order of evaluation (shared with the CPU oracle):
//   T_(j,t)[m][c]  = chain over q of fma(Minv_k[m][q], H_(j,t)[c][q])            (M^-1 H^T first)
//   W_ij[r][c]     = chain over the shared bodies (increasing), then m, of fma(H_(i,ti)[r][m], T_(j,tj)[m][c])
// The host builds the pattern (which lower blocks exist, which slot pairs share a body, and where each
// block and its transpose sit in the both-triangle BSR); one thread computes one lower block and writes
// it and its transpose.
#include "internal.h"

namespace bogus_gpu {

__global__ void k_assembly_T(int n, int d, const double* __restrict__ minv, const int* __restrict__ cb,
                             const double* __restrict__ H, double* __restrict__ T) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;  // 2 * contact + t
  if (slot >= 2 * n) return;
  const int k = cb[slot];
  if (k < 0) return;
  const double* Mi = minv + (size_t)k * d * d;
  const double* Hs = H + (size_t)slot * 3 * d;
  double* Ts = T + (size_t)slot * d * 3;
  for (int m = 0; m < d; ++m)
    for (int c = 0; c < 3; ++c) {
      double a = 0.0;
      for (int q = 0; q < d; ++q) a = fma(Mi[m * d + q], Hs[c * d + q], a);
      Ts[m * 3 + c] = a;
    }
}

cudaError_t launch_assembly_T(int n, int d, const double* minv, const int* cb, const double* H, double* T,
                              cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_assembly_T<<<(2 * n + 127) / 128, 128, 0, s>>>(n, d, minv, cb, H, T);
  return cudaGetLastError();
}

__global__ void k_assembly_W(int nlow, int d, const int* __restrict__ li, const int* __restrict__ lj,
                             const int* __restrict__ off, const int* __restrict__ pti, const int* __restrict__ ptj,
                             const double* __restrict__ H, const double* __restrict__ T, const int* __restrict__ pij,
                             const int* __restrict__ pji, double* __restrict__ val) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nlow) return;
  const int i = li[k], j = lj[k];
  double B[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double a = 0.0;
      for (int p = off[k]; p < off[k + 1]; ++p) {
        const double* Hi = H + (size_t)(2 * i + pti[p]) * 3 * d;
        const double* Tj = T + (size_t)(2 * j + ptj[p]) * d * 3;
        for (int m = 0; m < d; ++m) a = fma(Hi[r * d + m], Tj[m * 3 + c], a);
      }
      B[3 * r + c] = a;
    }
  double* D = val + 9 * (size_t)pij[k];
#pragma unroll
  for (int e = 0; e < 9; ++e) D[e] = B[e];
  if (pji[k] >= 0) {
    double* Dt = val + 9 * (size_t)pji[k];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) Dt[3 * r + c] = B[3 * c + r];
  }
}

cudaError_t launch_assembly_W(int nlow, int ndof, const int* li, const int* lj, const int* pair_off,
                              const int* pair_ti, const int* pair_tj, const double* H, const double* T,
                              const int* pos_ij, const int* pos_ji, double* val, cudaStream_t s) {
  if (nlow == 0) return cudaSuccess;
  k_assembly_W<<<(nlow + 127) / 128, 128, 0, s>>>(nlow, ndof, li, lj, pair_off, pair_ti, pair_tj, H, T, pos_ij,
                                                  pos_ji, val);
  return cudaGetLastError();
}

__global__ void k_assembly_mf(int nb, int d, const double* __restrict__ minv, const double* __restrict__ f,
                              double* __restrict__ mf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nb * d) return;
  const int k = t / d, m = t % d;
  double a = 0.0;
  for (int q = 0; q < d; ++q) a = fma(minv[(size_t)k * d * d + m * d + q], f ? f[(size_t)k * d + q] : 0.0, a);
  mf[t] = a;
}

__global__ void k_assembly_b(int n, int d, const int* __restrict__ cb, const double* __restrict__ H,
                             const double* __restrict__ mf, const double* __restrict__ w, double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int r = 0; r < 3; ++r) {
    double a = 0.0;
    for (int t = 0; t < 2; ++t) {
      const int k = cb[2 * i + t];
      if (k < 0) continue;
      const double* Hs = H + (size_t)(2 * i + t) * 3 * d;
      for (int m = 0; m < d; ++m) a = fma(Hs[r * d + m], mf[(size_t)k * d + m], a);
    }
    b[3 * i + r] = w[3 * i + r] - a;
  }
}

cudaError_t launch_assembly_b(int n, int nbodies, int ndof, const double* minv, const double* f, const int* cb,
                              const double* H, const double* w, double* mf, double* b, cudaStream_t s) {
  if (nbodies > 0) k_assembly_mf<<<(nbodies * ndof + 127) / 128, 128, 0, s>>>(nbodies, ndof, minv, f, mf);
  if (n > 0) k_assembly_b<<<(n + 127) / 128, 128, 0, s>>>(n, ndof, cb, H, mf, w, b);
  return cudaGetLastError();
}

}  // namespace bogus_gpu
