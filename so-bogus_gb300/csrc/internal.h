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

// Result of a persistent projected-gradient solve (APGD / Descent / SPG).
struct PGOut {
  double min_res;
  unsigned iters;
  int best_buf;   // 0..2: position buffer X0..X2 holding the best iterate; 3: the x_best buffer; 4: Wv
  int converged;
  // passes made by the solve, by kind (for the algorithmic-bytes accounting of the roofline):
  // 0 projection, 1 guess product, 2 A, 3 C (trial product), 4 B (retry), 5 D (momentum), 6 E+A,
  // 7 SPG D, 8 SPG E
  unsigned phases[9];
  unsigned hy_refreshes;  // FP32 correction products: momentum steps that took the FP64 product (x_ref refreshed)
};

// T: storage and per-contact arithmetic type (double: the FP64 drop-in; float: the FP32 part of the
// mixed-precision solve). Reductions (chunk sums, published scalars, residual trace) are always FP64.
template <class T>
struct PGArgsT {
  int n, nchunks;
  const int* rowptr;
  const int* col;
  const T* val;
  // the interleaved copy of W (InterleavedBlocks, spmv_chunk.cuh); null: the plain BSR arrays are read
  const int* icol;
  const T* ival;
  const long long* slot0;
  const int* chunk_order;  // chunks in the order the tickets hand them out (largest first); null: natural
  // per-CTA chunk lists of the single-problem kernel (CTA b takes cta_list[cta_ptr[b] .. cta_ptr[b+1]), its
  // warps sharing them through a counter in shared memory); null: one global ticket counter
  const int* cta_ptr;
  const int* cta_list;
  const T* b;
  const T* mu;
  const T* scaling;
  T* X0;
  T* X1;
  T* X2;
  T* MX0;
  T* MX1;
  T* MX2;  // MX2, MX3: the kept W prev and the momentum product when lin_momentum (else unused, may be null)
  T* MX3;
  T* Y;
  T* S0;
  T* XB;
  T* Wv;          // SPG step w
  double* csum;   // 4 * nchunks chunk sums
  double* scal;   // published scalars
  double* trace;  // residual per iteration (may be null)
  PGOut* out;
  GridBarrier gb;
  unsigned* tickets;  // 2 chunk counters (phase parity) for dynamic work distribution; zero at launch
  double* stripes;          // 8 stripe sums per reduced quantity (32 doubles)
  unsigned long long* mono; // 3 monotonic counters of the single-problem kernel's barriers (MonoBarrier); zero at launch
  int desaxce, variant, use_inf;
  int lin_momentum;  // APGD's momentum product by linearity (needs MX2, MX3)
  double tol, opt, pess;
  double armijo;     // the Armijo coefficient of the Standard and Conjugated variants' line search
  unsigned max_iters, ls_iters;
  // FP32 part of the FP32-refined solves (0 elsewhere): stop once the residual has repeated bit for bit on this
  // many consecutive iterations, or the line search has run out of trials this many times in a row
  unsigned stall_iters;
  // FP64 iterations with FP32 correction products (the HY instantiations of the FP64 kernels): W v = W x_ref +
  // W32 (v - x_ref)_32, with x_ref and W x_ref (FP64) refreshed at the first momentum step on or after every
  // hy_refresh iterations. hy_ival: FP32 values of W in the layout the kernel reads (interleaved: icol and slot0
  // shared; plain: col); hy_d: v - x_ref in FP32 for the position buffers 0, 1, 2 and 4 (buffer 4 last), the
  // buffers hy_stride floats apart (3 n of the whole problem or batch)
  const float* hy_ival;
  float* hy_d;
  size_t hy_stride;
  double* hy_xref;
  double* hy_wxref;
  unsigned hy_refresh;
  // test of the timeout path (single-problem kernel): the barriers count this many CTAs more than the launch
  // has, so the first one never completes and its bounded wait runs out; 0 in every solve
  unsigned phantom_ctas;
};
using PGArgs = PGArgsT<double>;
using PGArgs32 = PGArgsT<float>;

// Batched solves: problem p owns contacts [contact_ptr[p], contact_ptr[p+1]) of every per-contact array of
// `base` and chunk sums from 4 * chunk_ptr[p]; W rows are global, column indices local to the problem.
template <class T>
struct PGBatchArgsT {
  PGArgsT<T> base;
  int nproblems;
  const int* contact_ptr;
  const int* chunk_ptr;
  const int* queue;  // problem order (largest first)
  int* next;         // queue position counter (zeroed before the launch)
  T* r;              // results, contact-major over all problems
};
using PGBatchArgs = PGBatchArgsT<double>;
using PGBatchArgs32 = PGBatchArgsT<float>;

// Team schedule of the batched solve, for batches with fewer problems than resident CTAs: `size` CTAs of one
// cooperative launch solve one problem at a time, with a barrier, ticket counters and published scalars per
// team (the single-problem schedule on a slice of the GPU).
struct PGTeamArgs {
  int size;            // CTAs per team
  unsigned* counters;  // 8 per team: barrier count, barrier generation, tickets of phase parity 0 and 1, combine count
  int* job;            // 1 per team: the problem the team solves
  double* scal;        // 40 per team: the scalars published by the team's last barrier, then 32 stripe sums
  int* status;
};
// Launch shape of a batched solve. schedule 0: one CTA per problem (k_pg_batched), at most ctas_per_sm resident
// CTAs per SM; schedule 1: teams of team_size CTAs per problem (k_pg_team), at most ctas_per_sm CTAs per SM. Every
// shape gives the same results bit for bit (the chunk order of each problem's reductions is fixed).
struct BatchShape {
  int schedule = -1;  // -1: none
  int ctas_per_sm = 0;
  int team_size = 0;
  bool operator==(const BatchShape& o) const {
    return schedule == o.schedule && ctas_per_sm == o.ctas_per_sm && team_size == o.team_size;
  }
};
int pg_batched_per_sm(int device, bool fp32);  // occupancy of k_pg_batched (CTAs per SM)
int pg_team_per_sm(int device, bool fp32);     // occupancy of k_pg_team (CTAs per SM)
cudaError_t launch_pg_team(const PGBatchArgs& b, const PGTeamArgs& t, int grid, cudaStream_t s);
cudaError_t launch_pg_team(const PGBatchArgs32& b, const PGTeamArgs& t, int grid, cudaStream_t s);
int pg_team_grid(int device, bool fp32);

// Launchers (kernels_basic.cu)
cudaError_t launch_spmv(const DevBSR& W, const double* x, const double* init, double* y, cudaStream_t s);
cudaError_t launch_eval_chunks(int n, const double* x, const double* u, const double* mu, const double* scaling,
                               bool desaxce, bool use_inf, double* chunk, cudaStream_t s);
cudaError_t launch_combine(const double* chunk, int nchunks, bool is_max, double scale_div, double* out,
                           cudaStream_t s);
cudaError_t launch_diag_and_scaling(const DevBSR& W, double* scaling, cudaStream_t s);
cudaError_t launch_any_nonfinite(size_t m, const double* v, int* flag, cudaStream_t s);
cudaError_t launch_permute3(int n, const int* perm, const double* src, double* dst, bool inverse, cudaStream_t s);
cudaError_t launch_check_lower(int n, const int* rowptr, const int* col, int* out, cudaStream_t s);
// Structure check of a both-triangle BSR in device memory (k_check_full): *out = the smallest malformed row, or a
// value above n when every row is well formed (rows in range and sorted, columns in [0, n), diagonal present).
cudaError_t launch_check_full(int n, int nnzb, const int* rowptr, const int* col, int* out, cudaStream_t s);
cudaError_t launch_full_pattern(int n, const int* rowptr, const int* col, int* upper, int* cursor, int* frowptr,
                                int* fcol, int* src, cudaStream_t s);
cudaError_t launch_expand_lower(int nnz, const int* src, const double* low, double* full, cudaStream_t s);
cudaError_t launch_add(int m, const double* a, const double* b, double* y, cudaStream_t s);
cudaError_t launch_cadoux_rhs(int n, const double* y, const double* mu, const double* b, double* out, cudaStream_t s);

// Persistent solvers (kernels_pg.cu)
cudaError_t launch_pg_persistent(const PGArgs& a, int grid, cudaStream_t s);
cudaError_t launch_pg_persistent(const PGArgs32& a, int grid, cudaStream_t s);
int pg_max_grid(int device, bool fp32 = false, bool interleaved = false);
cudaError_t launch_pg_batched(const PGBatchArgs& b, int grid, cudaStream_t s);
cudaError_t launch_pg_batched(const PGBatchArgs32& b, int grid, cudaStream_t s);
int pg_batched_grid(int device, bool fp32 = false);
cudaError_t launch_convert(size_t m, const double* src, float* dst, cudaStream_t s);
// Interleaved copy of a both-triangle BSR (InterleavedBlocks): slot0 has nchunks + 1 entries (device).
cudaError_t launch_interleave(const DevBSR& W, const long long* slot0, int* icol, double* ival, cudaStream_t s);
cudaError_t launch_convert(size_t m, const float* src, double* dst, cudaStream_t s);

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
  const int* order;              // contacts grouped by level (sweep positions): the order contacts are handed out
  int desaxce, strat;
  // matrix-free sweep (ProductGaussSeidel): slot Jacobians H (3 x d), T = M^-1 H^T (d x 3), slot bodies cb,
  // Mx = M^-1 H^T x per body (nbodies x d)
  const double* H;
  const double* T;
  const int* cb;
  double* Mx;
  int d;
  // dataflow sweep: flow[0] = next sweep position to hand out, flow[1] = the sweep's tag; done[i] = tag once
  // contact i has been visited in this sweep; status records a wait that ran out
  unsigned* flow;
  unsigned* done;
  int* status;
  const int* pdep;  // matrix-free sweep: per contact slot, the previous contact on that body (-1: none)
};
constexpr int kGSTile = 1024;
constexpr int kGSFlowWarps = 4;  // warps per CTA of the dataflow sweep
cudaError_t launch_gs_flow(const GSArgs& a, int grid, int parity, cudaStream_t s);
int gs_flow_grid(int device);
cudaError_t launch_gs_skip(const GSArgs& a, int parity, double abs_skip_tol, double skip_tol, int abs_skip_iters,
                           cudaStream_t s);
cudaError_t launch_scale_scalar(double* p, double divisor, cudaStream_t s);
// matrix-free Gauss-Seidel (kernels_gs.cu)
cudaError_t launch_pgs_flow(const GSArgs& a, int grid, int parity, cudaStream_t s);
int pgs_flow_grid(int device);
cudaError_t launch_pgs_local(int n, int d, const int* cb, const double* H, const double* T, double* local,
                             cudaStream_t s);
cudaError_t launch_pgs_mx(int nbodies, int d, const int* bptr, const int* bent, const double* T, const double* x,
                          double* Mx, cudaStream_t s);
cudaError_t launch_pgs_y(int n, int d, const int* cb, const double* H, const double* Mx, const double* b, double* y,
                         cudaStream_t s);
cudaError_t measure_fp64_peak(int device, double* tflops);
cudaError_t check_fp64_ops(int device, long long n, unsigned long long seed, long long* mismatches);

// Primal ADMM / AMA (kernels_admm.cu): Core/BlockSolvers/ADMM.impl.hpp:54-127 with QuadraticProxOp
// (:29-38) as PrimalFrictionProblem::solveWith(ADMM&, lambda, v, r) calls it (PrimalFrictionProblem.cpp:61-73).
struct ADMMOut {
  double res;
  unsigned iters;
  int converged;
};
struct ADMMArgs {
  int n, nbodies, d;
  const int* cb;       // 2 n: bodies of the contact's two H slots, ordered by body index (-1: none)
  const double* H;     // 2 n x 3 x d: slot blocks, row-major
  const int* bptr;     // nbodies + 1
  const int* bent;     // incidences of each body, increasing contact index: 2 i + slot
  const int* border;   // nbodies: the order in which the body phase takes the bodies (null: natural)
  const double* prox;  // nbodies x d x d: the prox operator's blocks (M^-1)
  const double* f;     // nbodies x d, or null (f = 0)
  const double* w;     // 3 n
  const double* mu;    // n
  double* inv_mu;      // n (written)
  double *x, *r, *ut, *z, *zacc, *yprev;
  double* r_spare[2];  // 3 n each: the two candidate updates of r (r, r_spare[0], r_spare[1] rotate)
  double* csum;        // 2 x nchunks
  double* scal;        // published scalars
  unsigned* combine_count;  // grid_barrier_combine's counter; zero at launch
  unsigned* tickets;        // 2 chunk-ticket counters (one per phase parity); zero at launch
  double* stripes;          // 8 stripe sums per reduced quantity
  double* trace;       // max_iters entries, or null
  ADMMOut* out;
  GridBarrier gb;
  double lambda, gamma, tol;
  unsigned max_iters;
  int accelerated, use_inf;
  const double* scaling;  // n: the error function's scalings (1 unless H is square at the block level)
};
cudaError_t launch_admm(const ADMMArgs& a, int grid, cudaStream_t s);
int admm_max_grid(int device, int d);

// DualAMA (kernels_admm.cu): Core/BlockSolvers/ADMM.impl.hpp:128-303 with A = M, B = 0, trivial preconditioner.
struct DamaOut {
  double min_res;
  unsigned iters;
  int stopped;     // the loop ended before max_iters (tolerance reached or divergence)
  unsigned trials; // line-search trials over all iterations
};
struct DamaArgs {
  int n, nbodies, d;
  const int* cb;
  const double* H;
  const int* bptr;
  const int* bent;
  const double* M;        // nbodies x d x d mass blocks
  const double* f;        // nbodies x d
  const double* w;        // 3 n
  const double* mu;       // n
  const double* scaling;  // n
  double *v, *r, *rs, *x, *HrBp, *ut, *g, *y_prev, *r_best, *v_best;
  double *v_spare, *yp_spare;  // nbodies x d each: the line search's candidate v and y_prev
  double* csum;           // 3 x max(contact chunks, body chunks)
  double* scal;
  unsigned* combine_count;  // grid_barrier_combine's counter; zero at launch
  unsigned* tickets;        // 2 chunk-ticket counters (one per phase parity); zero at launch
  double* stripes;          // 8 stripe sums per reduced quantity
  double* trace;          // max_iters
  DamaOut* out;
  GridBarrier gb;
  double tol, gamma, lambda0, opt, pess, m_true;
  unsigned max_iters, ls_iters;
  int accelerated, use_inf, desaxce;
};
cudaError_t launch_dama(const DamaArgs& a, int grid, cudaStream_t s);
int dama_max_grid(int device, int d);

// Adjoint of the SOC solve (kernels_adjoint.cu).
struct AdjOut {
  unsigned iters;
  double rel_res;
};
struct AdjArgs {
  int n, nchunks;
  const int* rowptr;
  const int* icol;     // W, both triangles, interleaved (InterleavedBlocks)
  const double* ival;
  const long long* slot0;
  const double* val;   // W, plain BSR (diagonal blocks)
  const double* b;
  const double* mu;
  const double* scaling;  // per-contact fixed-point step 1 / scaling_i
  const double* r;     // the solution
  const double* g;     // dL/dr
  const int* diag;     // position of each diagonal block
  double *V, *D, *K;   // per contact basis (9), diagonal term (3, negative: masked), dP/dmu (3)
  double* Pc;          // per contact inverse of the preconditioner block (9)
  double *P, *R, *Z, *Dir, *Y, *Q;  // conjugate-gradient vectors (3 per contact)
  double* S;           // out: dL/db
  double* dmu;         // out: dL/dmu
  double* csum;
  double* scal;
  unsigned* combine_count;  // grid_barrier_combine's counter; zero at launch
  unsigned* tickets;        // 2 chunk-ticket counters (one per phase parity); zero at launch
  double* stripes;          // 8 stripe sums per reduced quantity
  AdjOut* out;
  GridBarrier gb;
  double tol;
  unsigned max_iters;
  // Coulomb law (De Saxce change of variable, bi-conjugate gradients stabilised): per contact (|u_T|, tau) with
  // tau = mu u_T / |u_T|, and five more work vectors (3 per contact)
  double* Tc;
  double *Rh, *Ph, *Sv, *Sh, *Tv;
};
cudaError_t launch_adjoint(const AdjArgs& a, int grid, cudaStream_t s);
cudaError_t launch_adjoint_coulomb(const AdjArgs& a, int grid, cudaStream_t s);
int adjoint_max_grid(int device);
// Helpers of the primal gradients and of the compliance term (kernels_grad.cu)
cudaError_t launch_body_transpose(int nbodies, int d, const int* bptr, const int* bent, const double* H,
                                  const double* minv, const double* vec, const double* f, double* out,
                                  cudaStream_t s);
cudaError_t launch_h_gradient(int n, int d, const int* cb, const double* s, const double* r, const double* vr,
                              const double* vs, double* dH, cudaStream_t st);
cudaError_t launch_add_diagonal(const DevBSR& W, const double* c, cudaStream_t s);
// MecheFrictionProblem frames (kernels_grad.cu): y_i = E_i^T x_i or E_i x_i; H slots from world Jacobians
cudaError_t launch_frame(int n, const double* E, const double* x, double* y, bool transpose, cudaStream_t s);
cudaError_t launch_meche_h(int n, int d, const double* E, const double* HAw, const double* HBw, const int* objA,
                           const int* objB, double* H, cudaStream_t s);

// Device-side wait limits (nanoseconds) of the kernel files, set on the current device.
cudaError_t set_wait_limit_pg(unsigned long long ns);
cudaError_t set_wait_limit_gs(unsigned long long ns);
cudaError_t set_wait_limit_admm(unsigned long long ns);
cudaError_t set_wait_limit_adjoint(unsigned long long ns);

// Records the message returned by bogus_gpu_last_error() on this thread.
void set_last_error(const std::string& msg);

}  // namespace bogus_gpu
