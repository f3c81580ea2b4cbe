// Internal declarations shared by the host API and the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "device_common.cuh"

namespace bogus_gpu {

// Both-triangle 3x3-block BSR of W resident in HBM: rows sorted by column, 9 doubles per block
// (row-major), int32 indices. Rows are contacts; vectors are contact-major (3 doubles per contact).
struct DevBSR {
  int n = 0;
  int nnzb = 0;
  int* rowptr = nullptr;  // n + 1
  int* col = nullptr;     // nnzb
  double* val = nullptr;  // 9 nnzb
  int* diag = nullptr;    // n: position of the diagonal block, -1 when absent
};

// Arguments of the persistent projected-gradient kernels (APGD / Descent / SPG).
struct PGOut {
  double min_res;
  unsigned iters;
  int best_buf;   // 0..2: position buffer holding the best iterate; 3: the x_best buffer
  int converged;
  // passes made by the solve, by kind (for the algorithmic-bytes accounting of the roofline):
  // 0 projection, 1 guess product, 2 A, 3 C (trial product), 4 B (retry), 5 D (momentum), 6 E+A,
  // 7 SPG D, 8 SPG E
  unsigned phases[9];
};

struct PGArgs {
  int n, nchunks;
  const int* rowptr;
  const int* col;
  const double* val;
  const double* b;
  const double* mu;
  const double* scaling;
  double* X0;
  double* X1;
  double* X2;
  double* MX0;
  double* MX1;
  double* Y;
  double* S0;
  double* XB;
  double* Wv;     // SPG step w
  double* csum;   // 4 * nchunks chunk sums
  double* scal;   // published scalars
  double* trace;  // residual per iteration
  PGOut* out;
  GridBarrier gb;
  unsigned* tickets;  // 2 chunk counters (phase parity) for dynamic work distribution; zero at launch
  int desaxce, variant, use_inf;
  double tol, opt, pess;
  unsigned max_iters, ls_iters;
};

// Batched solves: problem p owns contacts [contact_ptr[p], contact_ptr[p+1]) of every per-contact array of
// `base` and chunk sums from 4 * chunk_ptr[p]; W rows are global, column indices local to the problem.
struct PGBatchArgs {
  PGArgs base;
  int nproblems;
  const int* contact_ptr;
  const int* chunk_ptr;
  const int* queue;  // problem order (largest first)
  int* next;         // queue position counter (zeroed before the launch)
  double* r;         // results, contact-major over all problems
};

// Launchers (kernels_basic.cu)
cudaError_t launch_spmv(const DevBSR& W, const double* x, const double* init, double* y, cudaStream_t s);
cudaError_t launch_eval_chunks(int n, const double* x, const double* u, const double* mu, const double* scaling,
                               bool desaxce, bool use_inf, double* chunk, cudaStream_t s);
cudaError_t launch_combine(const double* chunk, int nchunks, bool is_max, double scale_div, double* out,
                           cudaStream_t s);
cudaError_t launch_diag_and_scaling(const DevBSR& W, double* scaling, cudaStream_t s);
cudaError_t launch_add(int m, const double* a, const double* b, double* y, cudaStream_t s);

// Persistent solvers (kernels_pg.cu)
cudaError_t launch_pg_persistent(const PGArgs& a, int grid, cudaStream_t s);
int pg_max_grid(int device);
cudaError_t launch_pg_batched(const PGBatchArgs& b, int grid, cudaStream_t s);
int pg_batched_grid(int device);

// Gauss-Seidel (kernels_gs.cu)
struct GSArgs {
  int n;
  const int* rowptr;
  const int* col;
  const double* val;
  const double* local;    // 9 n: diagonal block + regularization
  const double* reg;      // n
  const double* scaling;  // n
  const double* b;
  const double* mu;
  double* x;
  double* nx2;
  double* ndx2;
  unsigned char* skip;
  unsigned char* processed;
  unsigned long long* tile_max;  // 2 * ntiles (sweep parity)
  double* ndx_ref;               // 2 (sweep parity)
  const int* order;              // contacts grouped by level (sweep positions)
  int desaxce, strat;
};
constexpr int kGSTile = 1024;
cudaError_t launch_gs_level(const GSArgs& a, int l0, int l1, int parity, cudaStream_t s);
cudaError_t launch_gs_skip(const GSArgs& a, int parity, double abs_skip_tol, double skip_tol, int abs_skip_iters,
                           cudaStream_t s);
cudaError_t launch_scale_scalar(double* p, double divisor, cudaStream_t s);
cudaError_t measure_fp64_peak(int device, double* tflops);

// Records the message returned by bogus_gpu_last_error() on this thread.
void set_last_error(const std::string& msg);

}  // namespace bogus_gpu
