// Helpers of the adjoint's primal gradients and of the compliance term.
//
// Through W = H M^-1 H^T (+ a constant diagonal) and b = w - H M^-1 f, the gradients with respect to the
// primal data follow from s = dL/db and the solution r (v_r = M^-1 (H^T r - f), v_s = M^-1 H^T s):
//   dL/dH_ik = s_i (v_r)_k^T + r_i (v_s)_k^T,   dL/dw = s,   dL/df = -v_s.
#include "internal.h"

namespace bogus_gpu {

namespace {

constexpr int kMaxDofG = 12;

// out_b = M^-1_b ((H^T vec)_b - f_b), the H^T accumulation over the body's incidences in contact order
__global__ void k_body_transpose(int nbodies, int d, const int* __restrict__ bptr, const int* __restrict__ bent,
                                 const double* __restrict__ H, const double* __restrict__ minv,
                                 const double* __restrict__ vec, const double* __restrict__ f,
                                 double* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbodies) return;
  double acc[kMaxDofG];
  for (int q = 0; q < d; ++q) acc[q] = 0.0;
  for (int e = bptr[b]; e < bptr[b + 1]; ++e) {
    const int ent = bent[e];
    const int i = ent >> 1;
    const double* Hb = H + (size_t)ent * 3 * d;
    for (int q = 0; q < d; ++q) {
      double s = acc[q];
      for (int r = 0; r < 3; ++r) s = fma(Hb[r * d + q], vec[3 * i + r], s);
      acc[q] = s;
    }
  }
  if (f)
    for (int q = 0; q < d; ++q) acc[q] = acc[q] - f[(size_t)b * d + q];
  const double* Mb = minv + (size_t)b * d * d;
  for (int m = 0; m < d; ++m) {
    double s = 0.0;
    for (int q = 0; q < d; ++q) s = fma(Mb[m * d + q], acc[q], s);
    out[(size_t)b * d + m] = s;
  }
}

// dH slot (contact i, slot t) = s_i (v_r)_k^T + r_i (v_s)_k^T; zero for an empty slot
__global__ void k_h_gradient(int n, int d, const int* __restrict__ cb, const double* __restrict__ s,
                             const double* __restrict__ r, const double* __restrict__ vr,
                             const double* __restrict__ vs, double* __restrict__ dH) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= 2 * n) return;
  const int i = slot >> 1;
  const int k = cb[slot];
  double* out = dH + (size_t)slot * 3 * d;
  for (int row = 0; row < 3; ++row)
    for (int m = 0; m < d; ++m)
      out[row * d + m] = k < 0 ? 0.0
                               : s[3 * i + row] * vr[(size_t)k * d + m] + r[3 * i + row] * vs[(size_t)k * d + m];
}

__global__ void k_add_diagonal(int n, const int* __restrict__ diag, double* __restrict__ val,
                               const double* __restrict__ c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = diag[i];
  if (k < 0) return;
  double* B = val + 9 * (size_t)k;
  B[0] = B[0] + c[i];
  B[4] = B[4] + c[i];
  B[8] = B[8] + c[i];
}

}  // namespace

cudaError_t launch_body_transpose(int nbodies, int d, const int* bptr, const int* bent, const double* H,
                                  const double* minv, const double* vec, const double* f, double* out,
                                  cudaStream_t s) {
  if (nbodies <= 0) return cudaSuccess;
  if (d > kMaxDofG) return cudaErrorInvalidValue;
  k_body_transpose<<<(nbodies + 127) / 128, 128, 0, s>>>(nbodies, d, bptr, bent, H, minv, vec, f, out);
  return cudaGetLastError();
}

cudaError_t launch_h_gradient(int n, int d, const int* cb, const double* s, const double* r, const double* vr,
                              const double* vs, double* dH, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_h_gradient<<<(2 * n + 127) / 128, 128, 0, st>>>(n, d, cb, s, r, vr, vs, dH);
  return cudaGetLastError();
}

cudaError_t launch_add_diagonal(const DevBSR& W, const double* c, cudaStream_t s) {
  if (W.n <= 0) return cudaSuccess;
  k_add_diagonal<<<(W.n + 255) / 256, 256, 0, s>>>(W.n, W.diag, W.val, c);
  return cudaGetLastError();
}

}  // namespace bogus_gpu
