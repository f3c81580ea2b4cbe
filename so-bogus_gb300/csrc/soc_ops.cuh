// Per-contact operations of the projected-gradient kernels, by value type.
//
// SocOps<double> forwards to the FP64 functions of soc_device.cuh (the bit-exact drop-in). SocOps<float> is
// the same law in single precision for the FP32 part of the mixed-precision solve: the Fischer-Burmeister
// residual of SOCLaw::eval, the De Saxce change of variable and the projection on the cone, with float
// epsilon in the NumTraits::isZero tests (NumTraits<float>::epsilon(), Core/Utils/NumTraits.hpp:19-24).
#pragma once

#include <cfloat>

#include "soc_device.cuh"

namespace bogus_gpu {

template <class T>
struct SocOps;

template <>
struct SocOps<double> {
  static __device__ __forceinline__ double law_eval(bool desaxce, double mu, const double* x, const double* y) {
    return bogus_gpu::law_eval(desaxce, mu, x, y);
  }
  static __device__ __forceinline__ double cov(bool desaxce, double mu, const double* y) {
    return duality_cov(desaxce, mu, y);
  }
  static __device__ __forceinline__ void project(double mu, double* x) { project_cone(mu, x); }
  static __device__ __forceinline__ double dot3(const double* a, const double* b) { return bogus_gpu::dot3(a, b); }
  static __device__ __forceinline__ double sq3(const double* a) { return bogus_gpu::sq3(a); }
  // 0.5 v and v + 0.0, exact bit operations off the FP64 pipe
  static __device__ __forceinline__ double half(double v) { return ipipe::scale2<-1>(v); }
  static __device__ __forceinline__ double plus0(double v) { return ipipe::plus_zero(v); }
};

template <>
struct SocOps<float> {
  static __device__ __forceinline__ bool is_zero(float s) { return fabsf(s) < FLT_EPSILON; }
  static __device__ __forceinline__ float dot3(const float* a, const float* b) {
    return fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0]));
  }
  static __device__ __forceinline__ float sq3(const float* a) { return dot3(a, a); }
  static __device__ __forceinline__ float half(float v) { return 0.5f * v; }
  static __device__ __forceinline__ float plus0(float v) { return v + 0.f; }
  static __device__ __forceinline__ float norm2(float a0, float a1) { return sqrtf(fmaf(a1, a1, a0 * a0)); }

  static __device__ __forceinline__ void fb_canonical(const float* x, const float* y, float* fb) {
    float z2[3];
    z2[0] = sq3(x) + sq3(y);
    z2[1] = fmaf(x[0], x[1], y[0] * y[1]);
    z2[2] = fmaf(x[0], x[2], y[0] * y[2]);
    const float nz2t = norm2(z2[1], z2[2]);
    float om1[3], om2[3];
    om1[0] = om2[0] = 0.5f;
    if (is_zero(nz2t)) {
      om1[1] = -0.5f; om1[2] = 0.f;
      om2[1] = 0.5f;  om2[2] = 0.f;
    } else {
      const float inv = 1.f / nz2t;
      const float t1 = z2[1] * inv, t2 = z2[2] * inv;
      om1[1] = -0.5f * t1; om1[2] = -0.5f * t2;
      om2[1] = 0.5f * t1;  om2[2] = 0.5f * t2;
    }
    const float l1 = z2[0] - 2.f * nz2t;
    const float rl1 = sqrtf(l1 > 0.f ? l1 : 0.f);
    const float rl2 = sqrtf(z2[0] + 2.f * nz2t);
#pragma unroll
    for (int k = 0; k < 3; ++k) fb[k] = (x[k] + y[k]) - fmaf(rl2, om2[k], rl1 * om1[k]);
  }

  static __device__ __forceinline__ float law_eval(bool desaxce, float mu, const float* x, const float* y) {
    if (mu < 0.f) return sq3(y);
    float yy[3] = {y[0], y[1], y[2]};
    if (desaxce) yy[0] = fmaf(mu, norm2(y[1], y[2]), y[0]);
    float fb[3];
    if (is_zero(mu)) {
      fb[0] = (x[0] + yy[0]) - sqrtf(fmaf(yy[0], yy[0], x[0] * x[0]));
      fb[1] = x[1];
      fb[2] = x[2];
    } else {
      const float xh[3] = {mu * x[0], x[1], x[2]};
      const float yh[3] = {yy[0], mu * yy[1], mu * yy[2]};
      fb_canonical(xh, yh, fb);
    }
    return sq3(fb);
  }
  static __device__ __forceinline__ float cov(bool desaxce, float mu, const float* y) {
    return desaxce ? mu * norm2(y[1], y[2]) : 0.f;
  }
  static __device__ __forceinline__ void project(float mu, float* x) {
    const float nxt = norm2(x[1], x[2]);
    const float xn = x[0];
    if (mu < 0.f) { x[0] = x[1] = x[2] = 0.f; return; }
    if (nxt <= mu * xn) return;
    if (mu * nxt <= -xn) { x[0] = x[1] = x[2] = 0.f; return; }
    const float proj = fmaf(mu, nxt, xn) / fmaf(mu, mu, 1.f);
    x[0] = proj;
    const float f = (proj * mu) / nxt;
    x[1] *= f;
    x[2] *= f;
  }
};

}  // namespace bogus_gpu
