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

// ---- MecheFrictionProblem (Interfaces/MecheInterface.cpp) -----------------------------------------------
namespace bogus_gpu {

namespace {

// y_i = E_i^T x_i (transpose) or E_i x_i, E_i row-major 3x3, with the dot3 chain
__global__ void k_frame(int n, const double* __restrict__ E, const double* __restrict__ x, double* __restrict__ y,
                        int transpose) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* e = E + 9 * (size_t)i;
  const double v[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
  for (int a = 0; a < 3; ++a)
    y[3 * i + a] = transpose ? fma(e[6 + a], v[2], fma(e[3 + a], v[1], e[a] * v[0]))
                             : fma(e[3 * a + 2], v[2], fma(e[3 * a + 1], v[1], e[3 * a] * v[0]));
}

// Local-basis Jacobian slots of contact i (MecheInterface.cpp:161-176): H_A = E^T HA, H_B = -E^T HB, or
// E^T (HA - HB) when both objects are the same; slot 0 / 1 ordered by body index as in the primal layout.
// HAw / HBw: world blocks, row-major 3 x d (padded), per contact.
__global__ void k_meche_h(int n, int d, const double* __restrict__ E, const double* __restrict__ HAw,
                          const double* __restrict__ HBw, const int* __restrict__ objA, const int* __restrict__ objB,
                          double* __restrict__ H) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* e = E + 9 * (size_t)i;
  const int A = objA[i], B = objB[i];
  const bool two = B >= 0 && B != A;
  const int sA = (two && B < A) ? 1 : 0;  // slot of body A
  const size_t hs = 3 * (size_t)d;
  double* outA = H + (2 * (size_t)i + sA) * hs;
  double* outB = H + (2 * (size_t)i + (1 - sA)) * hs;
  for (int c = 0; c < d; ++c) {
    double h[3];
    for (int k = 0; k < 3; ++k) {
      h[k] = HAw[(size_t)i * hs + k * d + c];
      if (B == A) h[k] = h[k] - HBw[(size_t)i * hs + k * d + c];
    }
    for (int a = 0; a < 3; ++a) outA[a * d + c] = fma(e[6 + a], h[2], fma(e[3 + a], h[1], e[a] * h[0]));
    for (int a = 0; a < 3; ++a) {
      if (two) {
        const double hb[3] = {HBw[(size_t)i * hs + c], HBw[(size_t)i * hs + d + c], HBw[(size_t)i * hs + 2 * d + c]};
        outB[a * d + c] = -fma(e[6 + a], hb[2], fma(e[3 + a], hb[1], e[a] * hb[0]));
      } else {
        outB[a * d + c] = 0.0;
      }
    }
  }
}

}  // namespace

cudaError_t launch_frame(int n, const double* E, const double* x, double* y, bool transpose, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_frame<<<(n + 255) / 256, 256, 0, s>>>(n, E, x, y, transpose ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_meche_h(int n, int d, const double* E, const double* HAw, const double* HBw, const int* objA,
                           const int* objB, double* H, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_meche_h<<<(n + 127) / 128, 128, 0, s>>>(n, d, E, HAw, HBw, objA, objB, H);
  return cudaGetLastError();
}

}  // namespace bogus_gpu
