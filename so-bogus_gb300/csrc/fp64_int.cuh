// IEEE binary64 division and square root (round to nearest even) computed on the integer pipe.
//
// On GB300 the FP64 unit of an SM sub-partition takes about 64 cycles per warp instruction, and the IEEE
// division and square root are sequences of several such instructions. The integer pipe issues a warp
// instruction every cycle or two. These functions produce the same correctly rounded result with 64-bit
// integer arithmetic and one single-precision approximation instruction, leaving the FP64 unit to the
// products of the solvers.
//
// Method (Newton's iteration in fixed point followed by an exact remainder correction, as in Brent and
// Zimmermann, "Modern Computer Arithmetic" (2010), sections 3.4 and 3.5):
//   division a / b: with mantissas A, B (53-bit integers, A scaled so that B <= A < 2B), R ~ 2^61 / b for
//     b = B / 2^53 in [1/2, 1) from the single-precision reciprocal, refined by two Newton steps
//     R <- R + R (1 - b R); the estimate Q = A R / 2^61 of floor(A 2^53 / B) is within 2 units, and the
//     remainder A 2^53 - Q B, exact in 64-bit two's complement because it is small, corrects it. The
//     last bit of Q and whether the remainder vanishes give the rounding.
//   square root of x: with the mantissa M (53-bit integer, doubled when the exponent is odd) and
//     m = M / 2^52 in [1, 4), Y ~ 2^62 / sqrt(m) from the single-precision reciprocal square root, refined by
//     two Newton steps Y <- Y + Y (1 - m Y^2) / 2; S = M Y / 2^61 estimates floor(sqrt(M 2^54)) within 2
//     units and the remainder M 2^54 - S^2 corrects it. A square root never falls halfway between two
//     doubles, so the last bit of S alone decides the rounding.
// Zeros, infinities, NaNs, subnormal operands and results outside the normal range are passed to the
// hardware operation, which handles them by definition; ordinary operands never take that branch.
//
// Every function is __host__ __device__: on the host the single-precision approximation is the exact
// reciprocal (optionally perturbed by a test), so the same integer steps can be compared against the host's
// IEEE operations.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef BG_HD
#ifdef __CUDACC__
#define BG_HD __host__ __device__ __forceinline__
#else
#define BG_HD inline
#endif
#endif

namespace bogus_gpu {
namespace ipipe {

constexpr uint64_t kMant = (uint64_t(1) << 52) - 1;
constexpr uint64_t kHidden = uint64_t(1) << 52;

BG_HD uint64_t to_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
BG_HD double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
BG_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
BG_HD float bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
// high 64 bits of the 128-bit products
BG_HD uint64_t umulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
BG_HD int64_t smulhi(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
  return __mul64hi(a, b);
#else
  return (int64_t)(((__int128)a * b) >> 64);
#endif
}

// Single-precision approximations of 1/x and 1/sqrt(x) for x in [1/2, 4]. On the device: the approximate
// reciprocal and reciprocal square root instructions (rcp.approx.ftz.f32, rsqrt.approx.ftz.f32). On the
// host: the correctly rounded values moved by `host_ulps` units in the last place (a test sets it to show
// that the iteration tolerates approximations much worse than the hardware's).
#ifndef __CUDA_ARCH__
inline int& host_ulps() {
  static thread_local int u = 0;
  return u;
}
#endif
BG_HD float rcp_approx(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return bitsf(fbits(1.0f / x) + host_ulps());
#endif
}
BG_HD float rsqrt_approx(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return bitsf(fbits(1.0f / std::sqrt(x)) + host_ulps());
#endif
}

// v * 2^s as an integer, for a float v in [1/4, 4) and s >= 26 (v's 24-bit significand shifted into place)
BG_HD uint64_t fixed_of(float v, int s) {
  const uint32_t u = fbits(v);
  const uint64_t sig = (uint64_t)((u & 0x7FFFFFu) | 0x800000u);
  return sig << (int)(((u >> 23) & 0xFFu) - 150u + (uint32_t)s);
}

// Correctly rounded a / b when a, b are normal and the quotient is normal; `ok` false otherwise (the
// returned value is then meaningless).
BG_HD double div_core(uint64_t ua, uint64_t ub, bool& ok) {
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7FFu, eb = (uint32_t)(ub >> 52) & 0x7FFu;
  uint64_t A = (ua & kMant) | kHidden;
  const uint64_t B = (ub & kMant) | kHidden;
  int e = (int)ea - (int)eb + 1023;
  const bool lt = A < B;
  A <<= lt ? 1 : 0;
  e -= lt ? 1 : 0;
  ok = (ea - 1u < 2046u) && (eb - 1u < 2046u) && (e >= 1) && (e <= 2045);
  // b = B / 2^53 in [1/2, 1), truncated to 24 bits as a float
  const float bf = bitsf(0x3F000000u | (uint32_t)((B >> 29) & 0x7FFFFFu));
  uint64_t R = fixed_of(rcp_approx(bf), 61);  // ~ 2^61 / b, in (2^60, 2^62]
  const uint64_t Bs = B << 11;                 // b 2^64
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int64_t E = (int64_t)((uint64_t(1) << 61) - umulhi(Bs, R));  // 2^61 (1 - b R / 2^61)
    R = (uint64_t)((int64_t)R + smulhi((int64_t)R, E * 8));
  }
  uint64_t Q = umulhi(A << 3, R);  // ~ floor(A 2^53 / B), in [2^53, 2^54)
  int64_t rem = (int64_t)((A << 53) - Q * B);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool lo = rem < 0;
    Q -= lo ? 1 : 0;
    rem += lo ? (int64_t)B : 0;
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool hi = rem >= (int64_t)B;
    Q += hi ? 1 : 0;
    rem -= hi ? (int64_t)B : 0;
  }
  uint64_t mant = Q >> 1;
  const bool up = (Q & 1) && (rem != 0 || (mant & 1));
  mant += up ? 1 : 0;
  const bool carry = mant >> 53;
  mant >>= carry ? 1 : 0;
  e += carry ? 1 : 0;
  return from_bits(((ua ^ ub) & (uint64_t(1) << 63)) | ((uint64_t)e << 52) | (mant & kMant));
}

// Correctly rounded sqrt(x) for a positive normal x; `ok` false otherwise.
BG_HD double sqrt_core(uint64_t ux, bool& ok) {
  const uint32_t ex = (uint32_t)(ux >> 52);  // sign included: negative x fails the range test
  ok = ex - 1u < 2046u;
  int u = (int)ex - 1023;
  const bool odd = u & 1;
  const uint64_t M = ((ux & kMant) | kHidden) << (odd ? 1 : 0);  // [2^52, 2^54)
  u -= odd ? 1 : 0;
  // m = M / 2^52 in [1, 4), truncated to 24 bits as a float
  const float mf = odd ? bitsf(0x40000000u | (uint32_t)((M >> 30) & 0x7FFFFFu))
                       : bitsf(0x3F800000u | (uint32_t)((M >> 29) & 0x7FFFFFu));
  uint64_t Y = fixed_of(rsqrt_approx(mf), 62);  // ~ 2^62 / sqrt(m), in (2^60, 2^62]
  const uint64_t Ms = M << 10;                   // m 2^62
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const uint64_t Y2 = umulhi(Y, Y);                                   // y^2 2^60
    const int64_t E = (int64_t)((uint64_t(1) << 58) - umulhi(Ms, Y2));  // 2^58 (1 - m y^2)
    Y = (uint64_t)((int64_t)Y + smulhi((int64_t)Y, E * 32));
  }
  uint64_t S = umulhi(M << 3, Y);  // ~ floor(sqrt(M 2^54)), in [2^53, 2^54)
  int64_t rem = (int64_t)((M << 54) - S * S);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool lo = rem < 0;
    S -= lo ? 1 : 0;
    rem += lo ? (int64_t)(2 * S + 1) : 0;
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool hi = rem > (int64_t)(2 * S);
    rem -= hi ? (int64_t)(2 * S + 1) : 0;
    S += hi ? 1 : 0;
  }
  uint64_t mant = (S >> 1) + (S & 1);
  const bool carry = mant >> 53;
  mant >>= carry ? 1 : 0;
  u += carry ? 2 : 0;
  return from_bits((uint64_t)(u / 2 + 1023) << 52 | (mant & kMant));
}

// The hardware operations for the operands outside the fast domain, behind a call that the compiler cannot
// evaluate speculatively next to the integer path.
#ifdef __CUDA_ARCH__
__device__ __noinline__ double div_slow(double a, double b) { return a / b; }
__device__ __noinline__ double sqrt_slow(double x) { return sqrt(x); }
#else
inline double div_slow(double a, double b) { return a / b; }
inline double sqrt_slow(double x) { return std::sqrt(x); }
#endif

BG_HD double div_rn(double a, double b) {
  bool ok;
  double q = div_core(to_bits(a), to_bits(b), ok);
  if (!ok) q = div_slow(a, b);
  return q;
}
BG_HD double sqrt_rn(double x) {
  bool ok;
  double s = sqrt_core(to_bits(x), ok);
  if (!ok) s = sqrt_slow(x);
  return s;
}

// x * 2^k (k = -1 or 1 in the solvers): a change of the exponent field when x and the product are normal,
// the hardware product otherwise (zero, subnormal, infinite, NaN or out-of-range results).
#ifdef __CUDA_ARCH__
__device__ __noinline__ double mul_slow(double a, double b) { return a * b; }
#else
inline double mul_slow(double a, double b) { return a * b; }
#endif
template <int K>
BG_HD double scale2(double x) {
  const uint64_t u = to_bits(x);
  const int e = (int)((u >> 52) & 0x7FFu);
  double r = from_bits(u + (uint64_t)((int64_t)K << 52));
  if (!(e >= 1 && e <= 2046 && e + K >= 1 && e + K <= 2046)) r = mul_slow(x, K > 0 ? double(1 << K) : 1.0 / double(1 << -K));
  return r;
}

// x + 0.0: x itself, except -0.0, which becomes +0.0 (x finite)
BG_HD double plus_zero(double x) {
  const uint64_t u = to_bits(x);
  return from_bits(u == (uint64_t(1) << 63) ? 0 : u);
}

}  // namespace ipipe
}  // namespace bogus_gpu
