"""The integer-pipe IEEE division, square root and exact scalings of fp64_int.cuh, compiled for the host.

The header's functions are __host__ __device__. On the host the single-precision starting approximation is
the exact reciprocal moved by a chosen number of units in the last place, so the test also shows that the
Newton steps and the remainder correction tolerate starting points far worse than the hardware's
approximations. Every result is compared bit for bit with the host's IEEE operations (which round
correctly, as the GPU's do); the GPU comparison runs in test_gpu_fp64_int.py.
"""
import ctypes
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "so-bogus_gb300", "csrc")

SRC = r"""
#include "fp64_int.cuh"
#include <random>
using namespace bogus_gpu::ipipe;
static uint64_t pick(std::mt19937_64& rng, long i, uint64_t u) {
  switch (i % 4) {
    case 1: return (u & ~(0x7FFull << 52)) | ((uint64_t)(923 + rng() % 200) << 52);
    case 2: return (u & ~(0x7FFull << 52)) | ((uint64_t)(rng() % 2048) << 52);
    case 3: {
      const uint64_t pat[6] = {0, kMant, kMant - 1, 1, kMant >> 1, (kMant >> 1) + 1};
      return (u & ~kMant & ~(0x7FFull << 52)) | ((uint64_t)(1000 + rng() % 48) << 52) | pat[rng() % 6];
    }
    default: return u;
  }
}
extern "C" long check(long n, unsigned long long seed, int ulps, long* fast) {
  std::mt19937_64 rng(seed);
  host_ulps() = ulps;
  long bad = 0, nf = 0;
  for (long i = 0; i < n; ++i) {
    uint64_t ua = pick(rng, i, rng()), ub = pick(rng, i, rng());
    if (i % 8 == 5) {  // quotients and roots close to exact
      const double b = from_bits((ub & kMant) | (1023ull << 52));
      const double q = (double)(long long)(rng() >> 40) + 0.5 * (double)(rng() & 1);
      ua = to_bits(q * b) + (uint64_t)(rng() % 3) - 1;
      ub = to_bits(b);
    }
    const double a = from_bits(ua), b = from_bits(ub);
    bool ok;
    const double q = div_core(ua, ub, ok);
    if (ok) { ++nf; if (to_bits(q) != to_bits(a / b)) ++bad; }
    if (to_bits(div_rn(a, b)) != to_bits(a / b) && a / b == a / b) ++bad;
    uint64_t ux = ua & ~(1ull << 63);
    if (i % 8 == 7) { const double t = (double)(long long)(rng() >> 37); ux = to_bits(t * t) + (uint64_t)(rng() % 3) - 1; }
    const double x = from_bits(ux);
    const double s = sqrt_core(ux, ok);
    if (ok) { ++nf; if (to_bits(s) != to_bits(std::sqrt(x))) ++bad; }
    if (to_bits(sqrt_rn(x)) != to_bits(std::sqrt(x)) && x == x) ++bad;
    if (a == a) {
      if (to_bits(scale2<-1>(a)) != to_bits(a * 0.5)) ++bad;
      if (to_bits(scale2<1>(a)) != to_bits(a * 2.0)) ++bad;
      if (a - a == 0.0 && to_bits(plus_zero(a)) != to_bits(a + 0.0)) ++bad;
    }
  }
  if (to_bits(plus_zero(-0.0)) != to_bits(-0.0 + 0.0)) ++bad;
  if (to_bits(scale2<-1>(-0.0)) != to_bits(-0.0 * 0.5)) ++bad;
  *fast = nf;
  return bad;
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("fp64_int")
    src = d / "check.cpp"
    src.write_text(SRC)
    so = d / "libcheck.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, "-o", str(so),
                    str(src)], check=True)
    L = ctypes.CDLL(str(so))
    L.check.restype = ctypes.c_long
    L.check.argtypes = [ctypes.c_long, ctypes.c_ulonglong, ctypes.c_int, ctypes.POINTER(ctypes.c_long)]
    return L


@pytest.mark.parametrize("ulps", [0, 1, -1, 3, -3, 12, -12, 40, -40])
def test_division_and_sqrt_bitwise(lib, ulps):
    fast = ctypes.c_long(0)
    bad = lib.check(400_000, 1000 + ulps, ulps, ctypes.byref(fast))
    assert bad == 0
    assert fast.value > 400_000  # most cases take the integer path
