// Projected-gradient solve that allocates no memory.
//
// Some callers cannot allocate device memory at solve time: a physics step running under a fixed memory
// budget, a real-time loop where cudaMalloc's implicit device synchronisation would stall the frame, or a
// host that hands this library only the buffers it owns. bogus_gpu_solve_pg_noalloc serves them: the
// caller passes W, b, mu and r already in device memory, and every temporary of the persistent APGD /
// Descent / SPG kernel lives in one fixed array compiled into the library (g_noalloc_scratch below).
//
// The array is a host-side symbol: host code must never hand &g_noalloc_scratch to a kernel (that address
// means nothing on the GPU). Instead, the first call on each device, with that device current, asks the
// runtime for its device address with cudaGetSymbolAddress and remembers it; later calls on that device
// reuse it. Because that first call does this set-up, it should come before any stream capture.
//
// Every call on a device shares the same array. Its contents persist from one call to the next, so each
// call clears the parts that must start at zero (the grid-barrier words, the chunk counters, the error status
// and the words of the input check) before launching; two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the array and must not be issued.
//
// The remembered address belongs to the device's current CUDA context: cudaDeviceReset destroys that context
// and with it the array, so a process that resets a device must not call this entry point on it afterwards.
//
// The caller's W is checked on the device before it is used (row pointers in order and in range, columns in
// range and increasing, a diagonal block in every row, finite values in W, b and mu); the check's results go
// to words of the same fixed array, so a malformed problem is rejected with BOGUS_GPU_BAD_INPUT (or NONFINITE)
// before any kernel reads out of bounds, still without allocating. The entry point makes `device` current
// for its work and restores the caller's current device before it returns.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "bogus_gpu.h"
#include "internal.h"

namespace bogus_gpu {

namespace {

constexpr int kMaxContacts = BOGUS_GPU_NOALLOC_MAX_CONTACTS;
constexpr int kMaxIters = BOGUS_GPU_NOALLOC_MAX_ITERS;
constexpr int kMaxChunks = (kMaxContacts + 31) / 32;

// Region sizes in doubles, each rounded up to 256 bytes (32 doubles).
constexpr size_t round32(size_t v) { return (v + 31) / 32 * 32; }
constexpr size_t kVec3 = round32(3 * (size_t)kMaxContacts);
constexpr size_t kVec1 = round32((size_t)kMaxContacts);
constexpr size_t kOffX = 0;                          // 3 position buffers
constexpr size_t kOffMX = kOffX + 3 * kVec3;         // 2 product buffers
constexpr size_t kOffY = kOffMX + 2 * kVec3;
constexpr size_t kOffS0 = kOffY + kVec3;
constexpr size_t kOffXB = kOffS0 + kVec1;
constexpr size_t kOffWv = kOffXB + kVec3;
constexpr size_t kOffScaling = kOffWv + kVec3;
constexpr size_t kOffDiag = kOffScaling + kVec1;     // int32 per contact (stored in double slots)
constexpr size_t kOffCsum = kOffDiag + round32((size_t)kMaxContacts / 2 + 1);
constexpr size_t kOffScal = kOffCsum + round32(4 * (size_t)kMaxChunks);
constexpr size_t kOffTrace = kOffScal + 64;  // 8 scalars, 32 stripe sums
constexpr size_t kOffOut = kOffTrace + round32((size_t)kMaxIters + 1);
constexpr size_t kOffWords = kOffOut + round32(sizeof(PGOut) / sizeof(double) + 1);  // barrier count, gen, status
constexpr size_t kScratchDoubles = kOffWords + 32;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

int fail(int status, const std::string& msg) {
  set_last_error(msg);  // reported by bogus_gpu_last_error()
  return status;
}

// Device address of g_noalloc_scratch, looked up once per device (with that device current).
double* scratch_for_device(int device, int* status) {
  static std::mutex mu;
  static double* table[64] = {nullptr};
  static bool done[64] = {false};
  *status = BOGUS_GPU_OK;
  if (device < 0 || device >= 64) {
    *status = fail(BOGUS_GPU_NO_DEVICE, "device index out of range");
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!done[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      *status = fail(BOGUS_GPU_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return nullptr;
    }
    table[device] = static_cast<double*>(p);
    done[device] = true;
  }
  return table[device];
}

}  // namespace

}  // namespace bogus_gpu

using namespace bogus_gpu;

namespace {
int solve_on_current_device(int device, int n, int nnzb, const int* d_rowptr, const int* d_colidx,
                            const double* d_blocks, const double* d_b, const double* d_mu, const bogus_gpu_pg_options* o,
                            double* d_r, double* residual, unsigned* iters, void* stream);
}  // namespace

#define NA_CUDA(call)                                                                            \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail(BOGUS_GPU_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

extern "C" int bogus_gpu_solve_pg_noalloc(int device, int n, int nnzb, const int* d_rowptr, const int* d_colidx,
                                          const double* d_blocks, const double* d_b, const double* d_mu,
                                          const bogus_gpu_pg_options* o, double* d_r, double* residual,
                                          unsigned* iters, void* stream) {
  if (!o) return fail(BOGUS_GPU_BAD_INPUT, "null options");
  if (n < 0 || nnzb < 0) return fail(BOGUS_GPU_BAD_INPUT, "negative size");
  if (n > kMaxContacts)
    return fail(BOGUS_GPU_BAD_INPUT, "bogus_gpu_solve_pg_noalloc: " + std::to_string(n) + " contacts exceed the fixed "
                "scratch capacity of " + std::to_string(kMaxContacts) + " (use bogus_gpu_solve_pg_device)");
  if (o->max_iters > (unsigned)kMaxIters)
    return fail(BOGUS_GPU_BAD_INPUT, "bogus_gpu_solve_pg_noalloc: max_iters exceeds " + std::to_string(kMaxIters));
  if (o->variant != BOGUS_GPU_PG_APGD && o->variant != BOGUS_GPU_PG_DESCENT && o->variant != BOGUS_GPU_PG_SPG)
    return fail(BOGUS_GPU_BAD_INPUT, "projected-gradient variant not available on the GPU (APGD, Descent, SPG)");
  if (o->ls_iters == 0 && o->variant != BOGUS_GPU_PG_SPG) return fail(BOGUS_GPU_BAD_INPUT, "ls_iters must be >= 1");
  if (o->momentum_by_linearity && o->variant == BOGUS_GPU_PG_APGD)
    return fail(BOGUS_GPU_BAD_INPUT, "momentum_by_linearity needs two more product buffers than the fixed array holds");
  if (o->mixed_precision) return fail(BOGUS_GPU_BAD_INPUT, "the allocation-free entry point solves in FP64 only");
  if (!(o->tol >= 0) || !(o->ls_optimistic_factor > 0) || !(o->ls_pessimistic_factor > 0))
    return fail(BOGUS_GPU_BAD_INPUT, "invalid projected-gradient factors");
  if (n > 0 && (!d_rowptr || !d_b || !d_mu || !d_r || (nnzb > 0 && (!d_colidx || !d_blocks))))
    return fail(BOGUS_GPU_BAD_INPUT, "null device pointer");
  int prev_device = -1;
  NA_CUDA(cudaGetDevice(&prev_device));
  NA_CUDA(cudaSetDevice(device));
  const int st = solve_on_current_device(device, n, nnzb, d_rowptr, d_colidx, d_blocks, d_b, d_mu, o, d_r, residual,
                                         iters, stream);
  cudaSetDevice(prev_device);
  return st;
}

namespace {

int solve_on_current_device(int device, int n, int nnzb, const int* d_rowptr, const int* d_colidx,
                            const double* d_blocks, const double* d_b, const double* d_mu, const bogus_gpu_pg_options* o,
                            double* d_r, double* residual, unsigned* iters, void* stream) {
  int st = 0;
  double* s = scratch_for_device(device, &st);
  if (!s) return st;
  if (n == 0) {
    if (residual) *residual = 0.0;
    if (iters) *iters = 0;
    return BOGUS_GPU_OK;
  }
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const size_t n3 = 3 * (size_t)n;
  // [0] count, [1] gen, [2] status, [3..4] tickets, [8..13] 3 monotonic u64, [16] the first malformed row of W,
  // [17] the non-finite flag of the input check
  unsigned* words = reinterpret_cast<unsigned*>(s + kOffWords);
  {
    int* chk = reinterpret_cast<int*>(words + 16);
    NA_CUDA(launch_check_full(n, nnzb, d_rowptr, d_colidx, chk, cs));
    NA_CUDA(cudaMemsetAsync(chk + 1, 0, sizeof(int), cs));
    NA_CUDA(launch_any_nonfinite(9 * (size_t)nnzb, d_blocks, chk + 1, cs));
    NA_CUDA(launch_any_nonfinite(n3, d_b, chk + 1, cs));
    NA_CUDA(launch_any_nonfinite((size_t)n, d_mu, chk + 1, cs));
    NA_CUDA(launch_any_nonfinite(n3, d_r, chk + 1, cs));
    int check[2] = {0, 0};
    NA_CUDA(cudaMemcpyAsync(check, chk, sizeof(check), cudaMemcpyDeviceToHost, cs));
    NA_CUDA(cudaStreamSynchronize(cs));
    if (check[0] < n)
      return fail(BOGUS_GPU_BAD_INPUT, "bogus_gpu_solve_pg_noalloc: row " + std::to_string(check[0]) + " of W is "
                  "malformed (row pointers out of order or range, a column out of range or not increasing, or no "
                  "diagonal block)");
    if (check[1]) return fail(BOGUS_GPU_NONFINITE, "bogus_gpu_solve_pg_noalloc: non-finite value in W, b, mu or r");
  }
  // diagonal positions and scalings into the scratch
  DevBSR W;
  W.n = n;
  W.nnzb = nnzb;
  W.rowptr = const_cast<int*>(d_rowptr);
  W.col = const_cast<int*>(d_colidx);
  W.val = const_cast<double*>(d_blocks);
  W.diag = reinterpret_cast<int*>(s + kOffDiag);
  NA_CUDA(launch_diag_and_scaling(W, s + kOffScaling, cs));
  NA_CUDA(cudaMemcpyAsync(s + kOffX, d_r, sizeof(double) * n3, cudaMemcpyDeviceToDevice, cs));
  NA_CUDA(cudaMemsetAsync(words, 0, 14 * sizeof(unsigned), cs));
  PGArgs a{};
  a.n = n;
  a.nchunks = (n + 31) / 32;
  a.rowptr = d_rowptr;
  a.col = d_colidx;
  a.val = d_blocks;
  a.b = d_b;
  a.mu = d_mu;
  a.scaling = s + kOffScaling;
  a.X0 = s + kOffX;
  a.X1 = s + kOffX + kVec3;
  a.X2 = s + kOffX + 2 * kVec3;
  a.MX0 = s + kOffMX;
  a.MX1 = s + kOffMX + kVec3;
  a.Y = s + kOffY;
  a.S0 = s + kOffS0;
  a.XB = s + kOffXB;
  a.Wv = s + kOffWv;
  a.csum = s + kOffCsum;
  a.scal = s + kOffScal;
  a.trace = s + kOffTrace;
  a.out = reinterpret_cast<PGOut*>(s + kOffOut);
  a.gb = GridBarrier{words, words + 1, reinterpret_cast<int*>(words + 2)};
  a.tickets = words + 3;
  a.mono = reinterpret_cast<unsigned long long*>(words + 8);
  a.stripes = s + kOffScal + 8;
  a.desaxce = o->static_problem ? 0 : 1;
  a.variant = o->variant;
  a.use_inf = o->use_infinity_norm ? 1 : 0;
  a.tol = o->tol;
  a.opt = o->ls_optimistic_factor;
  a.pess = o->ls_pessimistic_factor;
  a.max_iters = o->max_iters;
  a.ls_iters = o->ls_iters;
  int grid = pg_max_grid(device);
  if (grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "cooperative occupancy query failed");
  const int want = (a.nchunks + 7) / 8;
  if (want < grid) grid = want < 1 ? 1 : want;
  NA_CUDA(launch_pg_persistent(a, grid, cs));
  PGOut out{};
  int dev_status = 0;
  NA_CUDA(cudaMemcpyAsync(&out, a.out, sizeof(PGOut), cudaMemcpyDeviceToHost, cs));
  NA_CUDA(cudaMemcpyAsync(&dev_status, words + 2, sizeof(int), cudaMemcpyDeviceToHost, cs));
  NA_CUDA(cudaStreamSynchronize(cs));
  if (dev_status != 0) return fail(dev_status, "device-side wait timed out in the projected-gradient kernel");
  const double* best =
      out.best_buf == 3 ? a.XB
                        : (out.best_buf == 4 ? a.Wv : (out.best_buf == 0 ? a.X0 : (out.best_buf == 1 ? a.X1 : a.X2)));
  NA_CUDA(cudaMemcpyAsync(d_r, best, sizeof(double) * n3, cudaMemcpyDeviceToDevice, cs));
  NA_CUDA(cudaStreamSynchronize(cs));
  if (residual) *residual = out.min_res;
  if (iters) *iters = out.iters;
  return out.converged ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

}  // namespace
