// Host side of the C ABI declared in include/bogus_gpu.h: problem upload and validation, the solve drivers
// (persistent projected gradient, colored Gauss-Seidel), the error function and the Delassus assembly.
// Host work is limited to one-off structure preparation (symmetric expansion, coloring, permutation,
// assembly pattern); every iteration runs on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "bogus_gpu.h"
#include "host_sparse.h"
#include "internal.h"
#include "soc_device.cuh"

namespace bogus_gpu {

// assembly kernels (kernels_assembly.cu)
struct AssemblyPlan {
  int n = 0, nbodies = 0, ndof = 0;
  int nlow = 0;  // lower blocks to compute
};
cudaError_t launch_assembly_T(int n, int ndof, const double* minv, const int* cb, const double* H, double* T,
                              cudaStream_t s);
cudaError_t launch_assembly_W(int nlow, int ndof, const int* li, const int* lj, const int* pair_off,
                              const int* pair_ti, const int* pair_tj, const double* H, const double* T,
                              const int* pos_ij, const int* pos_ji, double* val, cudaStream_t s);
cudaError_t launch_assembly_b(int n, int nbodies, int ndof, const double* minv, const double* f, const int* cb,
                              const double* H, const double* w, double* mf, double* b, cudaStream_t s);

namespace {

thread_local std::string g_last_error;

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

#define BG_CUDA(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return fail(BOGUS_GPU_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// A device array owned by a handle: grown on demand, freed by release() or when the handle is deleted (on
// the handle's device, which bogus_gpu_destroy makes current first). Not copyable: one owner per allocation.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

struct GSCache {
  bool valid = false;
  std::vector<int> perm, colors;
  std::vector<int> level_off;  // contacts of level L: order[level_off[L] .. level_off[L+1])
  DevBuf<int> order;
  DevBuf<int> rowptr, col;
  DevBuf<double> val, local, reg, scaling, b, mu;
  DevBuf<double> x, nx2, ndx2, y, chunk, scalar, xbest;
  DevBuf<unsigned char> skip, processed;
  DevBuf<unsigned long long> tile_max;
  DevBuf<double> ndx_ref;
  DevBuf<unsigned> flow, done;  // dataflow sweep: position counter and tag, per-contact visit tags
  DevBuf<int> pdep;             // matrix-free sweep: previous contact on each slot's body
  int flow_grid = 0;
  double auto_reg = -1.0;
  int use_coloring = -1;
  // one captured sweep per ndxRef parity, keyed by the law / strategy / skip settings baked into it
  cudaGraphExec_t sweep[2] = {nullptr, nullptr};
  long long sweep_key = -1;
  void drop_graphs() {
    for (auto& g : sweep)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    sweep_key = -1;
  }
  void release() {
    drop_graphs();
    order.release();
    rowptr.release(); col.release(); val.release(); local.release(); reg.release(); scaling.release();
    b.release(); mu.release(); x.release(); nx2.release(); ndx2.release(); y.release(); chunk.release();
    scalar.release(); xbest.release(); skip.release(); processed.release(); tile_max.release(); ndx_ref.release();
    flow.release(); done.release(); pdep.release();
    valid = false;
  }
};

}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }

}  // namespace bogus_gpu

using namespace bogus_gpu;

struct bogus_gpu_problem {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // dual problem (both triangles on the device)
  DevBSR W;
  DevBuf<int> rowptr, col, diag;
  DevBuf<double> val, b, mu, scaling;
  bool has_dual = false;
  bool host_lower_valid = false;
  HostBSR host_lower;  // lower triangle (for the coloring); kept when W came from host arrays or assembly
  // lower triangle as uploaded by bogus_gpu_set_dual (two sets: the next upload is checked in the other one),
  // copied to host_lower when first needed; work of the device-side expansion
  bool low_pending = false;
  int low_cur = 0;
  // DualFrictionProblem::applyPermutation: contact k of the stored problem is contact perm[k] of the caller's
  bool permuted = false;
  std::vector<int> perm, inv_perm;
  DevBuf<int> d_perm, d_inv_perm;
  DevBuf<double> perm_r;
  DevBuf<int> low_rowptr[2], low_col[2];
  DevBuf<double> low_val[2];
  DevBuf<int> full_src, pat_upper, pat_cursor, pat_check;
  std::vector<double> host_b, host_mu;
  // projected-gradient work
  DevBuf<double> X, MX, Y, S0, XB, Wv, csum, scal, trace;
  // interleaved copy of W (coalesced chunk layout read by the single-problem solvers), valid while W is unchanged
  bool il_valid = false;
  DevBuf<long long> slot0;
  DevBuf<int> chunk_order;  // chunks by decreasing segment length (ticket order of the persistent solvers)
  std::vector<int> h_chunk_order;  // the same on the host
  // per-CTA chunk lists of the single-problem kernel for a grid of cta_grid CTAs (0: none built)
  DevBuf<int> cta_ptr, cta_list;
  int cta_grid = 0;
  DevBuf<int> icol;
  DevBuf<double> ival;
  // FP32 copies of W (interleaved), b, mu, scalings and FP32 work (mixed precision), valid while W is unchanged
  bool fp32_valid = false;
  DevBuf<float> val32, b32, mu32, sc32, X32, MX32, Y32, S032, XB32, Wv32;
  DevBuf<float> val32p;  // FP32 copy of W's plain BSR values (batched FP32 solves)
  // FP32 correction products of the FP64 refinement: v - x_ref for 4 position buffers, x_ref, W x_ref
  DevBuf<float> hy_d;
  DevBuf<double> hy_xref, hy_wxref;
  bool fp32p_valid = false;
  DevBuf<PGOut> pgout;
  DevBuf<unsigned> barrier;
  DevBuf<int> status;
  // misc work
  DevBuf<double> vx, vy, chunk, scalar;
  GSCache gs;
  GSCache pgs;          // matrix-free Gauss-Seidel (levels from shared bodies, local matrices from H and M^-1)
  DevBuf<double> pgs_Mx;
  // primal data for the assembly
  int nbodies = 0, ndof = 0, ncontacts = 0;
  DevBuf<double> minv, H, T, mf;
  DevBuf<int> cb;  // per contact: body of slot 0, body of slot 1 (-1), slot order by body index
  std::vector<int> h_cb, h_objA;
  // ADMM: body -> (contact, slot) incidences in increasing contact order, per-call data and work
  bool admm_incidence_valid = false;
  size_t admm_ninc = 0;
  DevBuf<int> bptr, bent;
  DevBuf<int> border;  // bodies by decreasing contact count (the ADMM body phase's lane order)
  DevBuf<double> a_prox, a_f, a_w, a_mu, a_invmu, a_x, a_r, a_ut, a_z, a_zacc, a_rs1, a_rs2, a_yprev;
  DevBuf<ADMMOut> admm_out;
  // error-function scalings of ADMM / DualAMA (ConstrainedSolverBase::updateScalings), per contact, and the
  // bodies' own dof count (padding excluded), both set with the incidences
  DevBuf<double> a_sc;
  long long true_dofs = 0;
  std::vector<int> body_dofs;  // the bodies' own dof counts (d each unless set otherwise)
  // PrimalFrictionProblem::E: per-contact frames (local to world, row-major 3 x 3); w is given in world
  // coordinates and taken to the local basis (E^T w) by the primal solves and the assembly
  bool frames_valid = false;
  DevBuf<double> frames;
  // DualAMA: mass blocks, affine part and work
  DevBuf<double> dm_M, dm_f, dm_v, dm_rs, dm_x, dm_hr, dm_g, dm_yp, dm_rb, dm_vb, dm_v2, dm_yp2;
  DevBuf<DamaOut> dama_out;
  // Cadoux fixed point: the original right-hand side while the inner solves use COV(u) + b
  DevBuf<double> cad_b;
  // MecheFrictionProblem facade: frames, world w (then local), padded f, per-body dofs; dual built at first use
  bool meche_valid = false, meche_dual = false;
  DevBuf<double> meche_E, meche_w, meche_r, meche_v, meche_fd;
  std::vector<double> meche_wloc, meche_f, meche_mu;
  std::vector<double> meche_mass;  // mass blocks, row-major, padded to d dofs with zeros
  std::vector<unsigned> meche_ndof;
  // adjoint: per-contact basis, CG vectors, the last solution r and s = dL/db (device and host copies)
  DevBuf<double> adj_V, adj_Pc, adj_D, adj_K, adj_P, adj_R, adj_Z, adj_Dir, adj_Y, adj_Q, adj_S, adj_dmu, adj_r, adj_g;
  DevBuf<double> adj_Tc, adj_Rh, adj_Ph, adj_Sv, adj_Sh, adj_Tv;  // Coulomb law: |u_T| and tau, BiCGSTAB vectors
  DevBuf<AdjOut> adj_out;
  bool adj_valid = false;
  std::vector<double> h_adj_s, h_adj_r;
  // batch partition (block-diagonal W)
  int nproblems = 0;
  std::vector<int> h_contact_ptr, h_problem_nnz;
  DevBuf<int> contact_ptr, chunk_ptr, queue, col_local, next;
  DevBuf<PGOut> batch_out;
  DevBuf<unsigned> team_cnt;  // team schedule of the batched solve: counters, jobs, published scalars
  DevBuf<int> team_job;
  DevBuf<double> team_scal;
  // launch shape of the batched solves: forced by the caller, or tuned on the device (per precision) and cached
  // until the next bogus_gpu_set_batch; the shape of the last batched launch
  bool batch_tuning = false;
  BatchShape forced_shape, tuned_shape[2], last_shape;
  DevBuf<double> tune_x;  // the batch's starting iterate, kept while the tuner tries shapes
  std::vector<BatchShape> tune_cand;  // the shapes the tuner measured last, and their times (ms)
  std::vector<double> tune_ms;
  // the batched solve captured in a CUDA graph (bogus_gpu_solve_pg_batch_graph) and what it was captured with
  cudaGraphExec_t batch_graph = nullptr;
  PGBatchArgs graph_args{};
  PGTeamArgs graph_team{};
  BatchShape graph_shape;
  const double* graph_r = nullptr;
  PGOut* pinned_out = nullptr;  // page-locked copies of the per-problem results and the status word
  int* pinned_status = nullptr;
  int pinned_np = 0;
  bogus_gpu_callback callback = nullptr;
  void* callback_user = nullptr;
  bool test_wait_timeout = false;  // bogus_gpu_test_wait_timeout
  float last_ms = 0.f;
  unsigned last_launches = 0;
  bogus_gpu_solve_stats last_stats{};
};

namespace {

int check_handle(const bogus_gpu_problem* h) {
  if (!h) return fail(BOGUS_GPU_BAD_INPUT, "null handle");
  return BOGUS_GPU_OK;
}

int set_device(const bogus_gpu_problem* h) {
  const cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return fail(BOGUS_GPU_CUDA_ERROR, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  return BOGUS_GPU_OK;
}

// Uploads a both-triangle host BSR and b, mu; computes diagonal positions and scalings on the device.
int upload_full(bogus_gpu_problem* h, const HostBSR& f, const double* b, const double* mu) {
  const int n = f.n;
  const int nnz = f.nnzb();
  BG_CUDA(h->rowptr.ensure(n + 1));
  BG_CUDA(h->col.ensure(nnz));
  BG_CUDA(h->val.ensure(9 * (size_t)nnz));
  BG_CUDA(h->diag.ensure(n));
  BG_CUDA(h->b.ensure(3 * (size_t)n));
  BG_CUDA(h->mu.ensure(n));
  BG_CUDA(h->scaling.ensure(n));
  BG_CUDA(cudaMemcpyAsync(h->rowptr.p, f.rowptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, h->stream));
  if (nnz) {
    BG_CUDA(cudaMemcpyAsync(h->col.p, f.col.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, h->stream));
    BG_CUDA(cudaMemcpyAsync(h->val.p, f.val.data(), sizeof(double) * 9 * (size_t)nnz, cudaMemcpyHostToDevice, h->stream));
  }
  if (n) {
    BG_CUDA(cudaMemcpyAsync(h->b.p, b, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, h->stream));
    BG_CUDA(cudaMemcpyAsync(h->mu.p, mu, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  }
  h->W.n = n;
  h->W.nnzb = nnz;
  h->W.rowptr = h->rowptr.p;
  h->W.col = h->col.p;
  h->W.val = h->val.p;
  h->W.diag = h->diag.p;
  BG_CUDA(launch_diag_and_scaling(h->W, h->scaling.p, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  h->has_dual = true;
  h->gs.valid = false;
  h->nproblems = 0;
  h->fp32_valid = false;
  h->fp32p_valid = false;
  h->il_valid = false;
  h->adj_valid = false;
  return BOGUS_GPU_OK;
}

int check_finite(const double* v, size_t m, const char* what);

// bogus_gpu_set_dual from the lower triangle. The host checks rowptr (n + 1 integers) and b, mu; the blocks
// cross to the device once, into the staging set of the lower-triangle buffers, where their columns (range,
// lower triangle, strictly increasing) and values (finite) are checked. On an error the handle keeps its
// problem (the exact message comes from the host check of the structure). Then the device builds the pattern
// of both triangles and expands the values. The host copy of the lower triangle (coloring, Gauss-Seidel,
// adjoint) is downloaded when first needed (ensure_host_lower).
int set_dual_lower(bogus_gpu_problem* h, int n, const int* rowptr, const int* colidx, const double* blocks,
                   const double* b, const double* mu) {
  if (rowptr[0] != 0) return fail(BOGUS_GPU_BAD_INPUT, "rowptr[0] must be 0");
  for (int i = 0; i < n; ++i)
    if (rowptr[i + 1] < rowptr[i]) return fail(BOGUS_GPU_BAD_INPUT, "rowptr not monotone at row " + std::to_string(i));
  if (int e = check_finite(b, 3 * (size_t)n, "b")) return e;
  if (int e = check_finite(mu, n, "mu")) return e;
  if (int e = set_device(h)) return e;
  cudaStream_t s = h->stream;
  const int nlow = rowptr[n];
  const int nx = 1 - h->low_cur;
  BG_CUDA(h->low_rowptr[nx].ensure(n + 1));
  BG_CUDA(h->low_col[nx].ensure(nlow > 0 ? nlow : 1));
  BG_CUDA(h->low_val[nx].ensure(9 * (size_t)(nlow > 0 ? nlow : 1)));
  BG_CUDA(h->status.ensure(1));
  BG_CUDA(h->pat_check.ensure(2));
  const int check0[2] = {INT_MAX, 0};
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  BG_CUDA(cudaMemcpyAsync(h->pat_check.p, check0, sizeof(check0), cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(h->low_rowptr[nx].p, rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
  if (nlow) {
    BG_CUDA(cudaMemcpyAsync(h->low_col[nx].p, colidx, sizeof(int) * nlow, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->low_val[nx].p, blocks, sizeof(double) * 9 * (size_t)nlow, cudaMemcpyHostToDevice, s));
  }
  BG_CUDA(launch_check_lower(n, h->low_rowptr[nx].p, h->low_col[nx].p, h->pat_check.p, s));
  BG_CUDA(launch_any_nonfinite(9 * (size_t)nlow, h->low_val[nx].p, h->status.p, s));
  int check[2] = {0, 0}, bad = 0;
  BG_CUDA(cudaMemcpyAsync(check, h->pat_check.p, sizeof(check), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaMemcpyAsync(&bad, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  if (check[0] != INT_MAX) {
    const std::string err = validate_bsr_structure(n, rowptr, colidx, true);
    return fail(BOGUS_GPU_BAD_INPUT, err.empty() ? "invalid lower-triangle structure" : err);
  }
  if (bad) return fail(BOGUS_GPU_NONFINITE, "non-finite block value");
  // the staged upload becomes the problem
  h->low_cur = nx;
  const int nnz = 2 * nlow - check[1];
  BG_CUDA(h->rowptr.ensure(n + 1));
  BG_CUDA(h->col.ensure(nnz));
  BG_CUDA(h->val.ensure(9 * (size_t)nnz));
  BG_CUDA(h->full_src.ensure(nnz > 0 ? nnz : 1));
  BG_CUDA(h->pat_upper.ensure(n > 0 ? n : 1));
  BG_CUDA(h->pat_cursor.ensure(n > 0 ? n : 1));
  BG_CUDA(h->diag.ensure(n));
  BG_CUDA(h->b.ensure(3 * (size_t)n));
  BG_CUDA(h->mu.ensure(n));
  BG_CUDA(h->scaling.ensure(n));
  if (n == 0) BG_CUDA(cudaMemsetAsync(h->rowptr.p, 0, sizeof(int), s));
  BG_CUDA(launch_full_pattern(n, h->low_rowptr[nx].p, h->low_col[nx].p, h->pat_upper.p, h->pat_cursor.p, h->rowptr.p,
                              h->col.p, h->full_src.p, s));
  BG_CUDA(launch_expand_lower(nnz, h->full_src.p, h->low_val[nx].p, h->val.p, s));
  if (n) {
    BG_CUDA(cudaMemcpyAsync(h->b.p, b, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->mu.p, mu, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  }
  h->W.n = n;
  h->W.nnzb = nnz;
  h->W.rowptr = h->rowptr.p;
  h->W.col = h->col.p;
  h->W.val = h->val.p;
  h->W.diag = h->diag.p;
  BG_CUDA(launch_diag_and_scaling(h->W, h->scaling.p, s));
  h->host_b.assign(b, b + 3 * (size_t)n);
  h->host_mu.assign(mu, mu + n);
  BG_CUDA(cudaStreamSynchronize(s));
  h->host_lower_valid = false;
  h->low_pending = true;
  h->host_lower.n = n;
  h->has_dual = true;
  h->gs.valid = false;
  h->nproblems = 0;
  h->fp32_valid = false;
  h->fp32p_valid = false;
  h->il_valid = false;
  h->adj_valid = false;
  return BOGUS_GPU_OK;
}

// The host copy of W's lower triangle, downloaded after bogus_gpu_set_dual at first use.
int ensure_host_lower(bogus_gpu_problem* h) {
  if (h->host_lower_valid) return BOGUS_GPU_OK;
  if (!h->low_pending) return fail(BOGUS_GPU_NO_PROBLEM, "no host copy of W (set W from host arrays or by assembly)");
  if (int e = set_device(h)) return e;
  HostBSR& l = h->host_lower;
  const int n = l.n;
  cudaStream_t s = h->stream;
  l.rowptr.resize(n + 1);
  BG_CUDA(cudaMemcpyAsync(l.rowptr.data(), h->low_rowptr[h->low_cur].p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  const int nlow = l.rowptr[n];
  l.col.resize(nlow);
  l.val.resize(9 * (size_t)nlow);
  if (nlow) {
    BG_CUDA(cudaMemcpyAsync(l.col.data(), h->low_col[h->low_cur].p, sizeof(int) * nlow, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(l.val.data(), h->low_val[h->low_cur].p, sizeof(double) * 9 * (size_t)nlow,
                            cudaMemcpyDeviceToHost, s));
  }
  BG_CUDA(cudaStreamSynchronize(s));
  h->host_lower_valid = true;
  h->low_pending = false;
  return BOGUS_GPU_OK;
}

// APGD's momentum product by linearity (bogus_gpu_pg_options::momentum_by_linearity; no effect on the other
// variants, which have no momentum product)
int lin_momentum(const bogus_gpu_pg_options* o) {
  return o->momentum_by_linearity && o->variant == BOGUS_GPU_PG_APGD ? 1 : 0;
}

int check_finite(const double* v, size_t m, const char* what) {
  for (size_t k = 0; k < m; ++k)
    if (!std::isfinite(v[k])) return fail(BOGUS_GPU_NONFINITE, std::string("non-finite value in ") + what);
  return BOGUS_GPU_OK;
}

int ensure_pg_work(bogus_gpu_problem* h, unsigned max_iters) {
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  const int C = (n + 31) / 32;
  BG_CUDA(h->X.ensure(3 * n3));
  BG_CUDA(h->MX.ensure(4 * n3));
  BG_CUDA(h->Y.ensure(n3));
  BG_CUDA(h->S0.ensure(n));
  BG_CUDA(h->XB.ensure(n3));
  BG_CUDA(h->Wv.ensure(n3));
  BG_CUDA(h->csum.ensure(5 * (size_t)C));  // up to 5 reduced quantities (the Conjugated variant)
  BG_CUDA(h->scal.ensure(8 + 40));         // scalars, then the stripe sums of grid_barrier_combine
  BG_CUDA(h->trace.ensure((size_t)max_iters + 1));
  BG_CUDA(h->pgout.ensure(1));
  BG_CUDA(h->barrier.ensure(16));  // [0..7] barrier words, [8..13] three 64-bit monotonic counters
  BG_CUDA(h->status.ensure(1));
  return BOGUS_GPU_OK;
}

int ensure_interleaved(bogus_gpu_problem* h);
int ensure_cta_lists(bogus_gpu_problem* h, int G);
int ensure_incidence(bogus_gpu_problem* h);

// Algorithmic bytes and W passes of one persistent solve from its phase counters. A W pass reads nnzb blocks
// (9 values + a column index) and the n + 1 row pointers; the per-contact vector bytes of each pass kind
// follow PGOut::phases (3-vectors 3 values, scalars 1 value). elem = bytes per value (8 FP64, 4 FP32).
struct PGTraffic {
  double bytes = 0, fma = 0;
  unsigned passes = 0;
};
PGTraffic pg_traffic(const PGOut& out, int n, long long nnzb, int variant, double elem, bool lin = false,
                     double welem = 0.0) {
  const bool spg = variant == BOGUS_GPU_PG_SPG, apgd = variant == BOGUS_GPU_PG_APGD;
  const double wpass = (double)nnzb * (9.0 * (welem > 0.0 ? welem : elem) + 4.0) + 4.0 * (n + 1);
  // values per contact; APGD's trial product also writes the momentum point (and, by linearity, reads the kept
  // product of prev and writes the momentum product)
  const double per_contact[9] = {7, 6, spg ? 21.0 : 18.0, apgd ? (lin ? 28.0 : 22.0) : 19.0, 10, 9, 18, 15, 12};
  const bool has_w[9] = {false, true, false, true, false, false, true, false, true};
  PGTraffic t;
  for (int k = 0; k < 9; ++k) {
    t.bytes += out.phases[k] * (per_contact[k] * elem * n + (has_w[k] ? wpass : 0.0));
    if (has_w[k]) {
      t.passes += out.phases[k];
      t.fma += out.phases[k] * 9.0 * (double)nnzb * (k == 1 ? 2.0 : 1.0);
    }
  }
  return t;
}

// FP32 correction products of an FP64 refinement (k_pg_persistent<double, true, false, true>).
struct HyArgs {
  const float* ival;
  float* d;
  double* xref;
  double* wxref;
  unsigned refresh;
  size_t stride;  // floats between the position buffers' corrections in d
};

// Runs the persistent solver with r already in X[0]; returns the buffer holding the result. hy: FP64 iterations
// with FP32 correction products (APGD; no callback: their residuals are those of the corrected products).
int run_pg(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* residual, unsigned* iters, const double** best,
           const HyArgs* hy = nullptr) {
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  if (int e = ensure_interleaved(h)) return e;
  PGArgs a{};
  a.n = n;
  a.nchunks = (n + 31) / 32;
  a.rowptr = h->W.rowptr;
  a.col = h->W.col;
  a.val = h->W.val;
  a.icol = h->icol.p;
  a.ival = h->ival.p;
  a.slot0 = h->slot0.p;
  a.chunk_order = h->chunk_order.p;
  a.b = h->b.p;
  a.mu = h->mu.p;
  a.scaling = h->scaling.p;
  a.X0 = h->X.p;
  a.X1 = h->X.p + n3;
  a.X2 = h->X.p + 2 * n3;
  a.MX0 = h->MX.p;
  a.MX1 = h->MX.p + n3;
  a.MX2 = h->MX.p + 2 * n3;
  a.MX3 = h->MX.p + 3 * n3;
  a.Y = h->Y.p;
  a.S0 = h->S0.p;
  a.XB = h->XB.p;
  a.Wv = h->Wv.p;
  a.csum = h->csum.p;
  a.scal = h->scal.p;
  a.trace = h->trace.p;
  a.out = h->pgout.p;
  a.gb = GridBarrier{h->barrier.p, h->barrier.p + 1, h->status.p};
  a.tickets = h->barrier.p + 2;
  a.stripes = h->scal.p + 8;
  a.mono = reinterpret_cast<unsigned long long*>(h->barrier.p + 8);
  a.desaxce = o->static_problem ? 0 : 1;
  a.variant = o->variant;
  a.use_inf = o->use_infinity_norm ? 1 : 0;
  a.tol = o->tol;
  a.opt = o->ls_optimistic_factor;
  a.pess = o->ls_pessimistic_factor;
  a.max_iters = o->max_iters;
  a.ls_iters = o->ls_iters;
  a.lin_momentum = lin_momentum(o);
  a.armijo = o->ls_armijo_coefficient;
  a.phantom_ctas = h->test_wait_timeout ? 1u : 0u;
  if (hy) {
    a.hy_ival = hy->ival;
    a.hy_d = hy->d;
    a.hy_xref = hy->xref;
    a.hy_wxref = hy->wxref;
    a.hy_refresh = hy->refresh;
    a.hy_stride = hy->stride;
    a.lin_momentum = 0;
  }
  BG_CUDA(cudaMemsetAsync(h->barrier.p, 0, 16 * sizeof(unsigned), h->stream));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), h->stream));
  int grid = pg_max_grid(h->device, false, true);
  if (grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "cooperative occupancy query failed");
  const int want = (a.nchunks + 7) / 8;
  if (want < grid) grid = want < 1 ? 1 : want;
  if (int e = ensure_cta_lists(h, grid)) return e;
  a.cta_ptr = h->cta_ptr.p;
  a.cta_list = h->cta_list.p;
  BG_CUDA(cudaEventRecord(h->ev0, h->stream));
  BG_CUDA(launch_pg_persistent(a, grid, h->stream));
  BG_CUDA(cudaEventRecord(h->ev1, h->stream));
  PGOut out{};
  int st = 0;
  BG_CUDA(cudaMemcpyAsync(&out, h->pgout.p, sizeof(PGOut), cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->last_launches = 1;
  if (st != 0) return fail(st, "device-side wait timed out in the projected-gradient kernel");
  {
    // hy: the trial and momentum products read FP32 values; the guess product and the refreshes the FP64 ones
    PGTraffic t = pg_traffic(out, n, h->W.nnzb, o->variant, 8.0, lin_momentum(o) != 0 && !hy, hy ? 4.0 : 0.0);
    if (hy) {
      const double fp64_passes = (double)out.phases[1] + (double)out.hy_refreshes;
      t.bytes += fp64_passes * 36.0 * (double)h->W.nnzb;
      t.fma = 9.0 * (double)h->W.nnzb * (2.0 * out.phases[1] + out.hy_refreshes);
    }
    h->last_stats.iterations = out.iters;
    h->last_stats.refine_iterations = 0;
    h->last_stats.fp32_device_ms = 0.0;
    h->last_stats.fp32_product_iterations = 0;
    h->last_stats.w_passes = t.passes;
    h->last_stats.algorithmic_bytes = t.bytes;
    h->last_stats.fp64_fma = t.fma;
  }
  if (residual) *residual = out.min_res;
  if (iters) *iters = out.iters;
  *best = out.best_buf == 3 ? h->XB.p : (out.best_buf == 4 ? h->Wv.p : h->X.p + (size_t)out.best_buf * n3);
  if (h->callback && !hy) {
    const unsigned count = out.converged ? out.iters + 1 : out.iters;
    std::vector<double> tr(count);
    if (count) {
      BG_CUDA(cudaMemcpy(tr.data(), h->trace.p, sizeof(double) * count, cudaMemcpyDeviceToHost));
    }
    for (unsigned k = 0; k < count; ++k) h->callback(k, tr[k], h->callback_user);
  }
  return out.converged ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

// The interleaved copy of W: chunk c (rows 32c .. 32c+31, blocks [B0, B1)) takes 32 S slots, S =
// ceil((B1 - B0) / 32) (1 for an empty chunk), from slot0[c].
// Per-CTA chunk lists for a grid of G CTAs: the chunks in ticket order (largest first) dealt to the CTAs
// in serpentine rounds (0 .. G-1, then G-1 .. 0, ...), so every CTA's total and every SM's (its resident
// CTAs') are equal to within about one chunk; each CTA's warps share its list dynamically. A phase then
// ends with every SM at about the same time instead of each SM finishing the chunks it happened to hold when
// a global ticket pool ran out. Which warp handles a chunk does not change any result.
int ensure_cta_lists(bogus_gpu_problem* h, int G) {
  if (h->cta_grid == G) return BOGUS_GPU_OK;
  const int C = (int)h->h_chunk_order.size();
  std::vector<int> cnt(G + 1, 0), owner(C);
  for (int k = 0; k < C; ++k) {
    const int round = k / G, pos = k % G;
    owner[k] = (round & 1) ? G - 1 - pos : pos;
    ++cnt[owner[k] + 1];
  }
  for (int b = 0; b < G; ++b) cnt[b + 1] += cnt[b];
  std::vector<int> list(C > 0 ? C : 1), fill(cnt.begin(), cnt.end() - 1);
  for (int k = 0; k < C; ++k) list[fill[owner[k]]++] = h->h_chunk_order[k];
  BG_CUDA(h->cta_ptr.ensure(G + 1));
  BG_CUDA(h->cta_list.ensure(C > 0 ? C : 1));
  BG_CUDA(cudaMemcpyAsync(h->cta_ptr.p, cnt.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice, h->stream));
  BG_CUDA(cudaMemcpyAsync(h->cta_list.p, list.data(), sizeof(int) * (C > 0 ? C : 1), cudaMemcpyHostToDevice,
                          h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  h->cta_grid = G;
  return BOGUS_GPU_OK;
}

int ensure_interleaved(bogus_gpu_problem* h) {
  if (h->il_valid) return BOGUS_GPU_OK;
  const int n = h->W.n;
  const int C = (n + 31) / 32;
  std::vector<int> rp(n + 1);
  BG_CUDA(cudaMemcpy(rp.data(), h->W.rowptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
  std::vector<long long> s0(C + 1, 0);
  std::vector<int> seg(C), order(C);
  for (int c = 0; c < C; ++c) {
    const int r1 = std::min(32 * c + 32, n);
    const int T = rp[r1] - rp[32 * c];
    const long long S = T > 0 ? (T + 31) / 32 : 1;
    s0[c + 1] = s0[c] + 32 * S;
    seg[c] = (int)S;
    order[c] = c;
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return seg[x] > seg[y]; });
  h->h_chunk_order = order;
  h->cta_grid = 0;
  BG_CUDA(h->chunk_order.ensure(C > 0 ? C : 1));
  if (C) BG_CUDA(cudaMemcpyAsync(h->chunk_order.p, order.data(), sizeof(int) * C, cudaMemcpyHostToDevice, h->stream));
  const size_t slots = (size_t)s0[C];
  BG_CUDA(h->slot0.ensure(C + 1));
  BG_CUDA(h->icol.ensure(slots > 0 ? slots : 1));
  BG_CUDA(h->ival.ensure(9 * (slots > 0 ? slots : 1)));
  BG_CUDA(cudaMemcpyAsync(h->slot0.p, s0.data(), sizeof(long long) * (C + 1), cudaMemcpyHostToDevice, h->stream));
  BG_CUDA(launch_interleave(h->W, h->slot0.p, h->icol.p, h->ival.p, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  h->il_valid = true;
  h->fp32_valid = false;
  return BOGUS_GPU_OK;
}

// FP32 copies of the problem and FP32 work buffers for the mixed-precision solve.
int ensure_fp32(bogus_gpu_problem* h) {
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  cudaStream_t s = h->stream;
  BG_CUDA(h->X32.ensure(3 * n3));
  BG_CUDA(h->MX32.ensure(4 * n3));
  BG_CUDA(h->Y32.ensure(n3));
  BG_CUDA(h->S032.ensure(n));
  BG_CUDA(h->XB32.ensure(n3));
  BG_CUDA(h->Wv32.ensure(n3));
  if (int e = ensure_interleaved(h)) return e;
  if (h->fp32_valid) return BOGUS_GPU_OK;
  BG_CUDA(h->val32.ensure(h->ival.n));
  BG_CUDA(h->b32.ensure(n3));
  BG_CUDA(h->mu32.ensure(n));
  BG_CUDA(h->sc32.ensure(n));
  BG_CUDA(launch_convert(h->ival.n, h->ival.p, h->val32.p, s));
  BG_CUDA(launch_convert(n3, h->b.p, h->b32.p, s));
  BG_CUDA(launch_convert((size_t)n, h->mu.p, h->mu32.p, s));
  BG_CUDA(launch_convert((size_t)n, h->scaling.p, h->sc32.p, s));
  h->fp32_valid = true;
  return BOGUS_GPU_OK;
}

template <class T>
void fill_args(PGArgsT<T>& a, const bogus_gpu_pg_options* o) {
  a.desaxce = o->static_problem ? 0 : 1;
  a.variant = o->variant;
  a.use_inf = o->use_infinity_norm ? 1 : 0;
  a.tol = o->tol;
  a.opt = o->ls_optimistic_factor;
  a.pess = o->ls_pessimistic_factor;
  a.max_iters = o->max_iters;
  a.ls_iters = o->ls_iters;
  a.lin_momentum = lin_momentum(o);
  a.armijo = o->ls_armijo_coefficient;
}

// Mixed precision: FP32 solve from X[0] (double), its best iterate back into X[0], then the FP64 solve from
// there for at most refine_max_iters iterations.
int run_pg_mixed(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* residual, unsigned* iters,
                 const double** best) {
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  if (int e = ensure_fp32(h)) return e;
  if (int e = ensure_pg_work(h, o->max_iters > o->refine_max_iters ? o->max_iters : o->refine_max_iters)) return e;
  cudaStream_t s = h->stream;
  PGArgs32 a{};
  a.n = n;
  a.nchunks = (n + 31) / 32;
  a.rowptr = h->W.rowptr;
  a.col = nullptr;
  a.val = nullptr;
  a.icol = h->icol.p;
  a.ival = h->val32.p;
  a.slot0 = h->slot0.p;
  a.chunk_order = h->chunk_order.p;
  a.b = h->b32.p;
  a.mu = h->mu32.p;
  a.scaling = h->sc32.p;
  a.X0 = h->X32.p;
  a.X1 = h->X32.p + n3;
  a.X2 = h->X32.p + 2 * n3;
  a.MX0 = h->MX32.p;
  a.MX1 = h->MX32.p + n3;
  a.MX2 = h->MX32.p + 2 * n3;
  a.MX3 = h->MX32.p + 3 * n3;
  a.Y = h->Y32.p;
  a.S0 = h->S032.p;
  a.XB = h->XB32.p;
  a.Wv = h->Wv32.p;
  a.csum = h->csum.p;
  a.scal = h->scal.p;
  a.trace = nullptr;
  a.out = h->pgout.p;
  a.gb = GridBarrier{h->barrier.p, h->barrier.p + 1, h->status.p};
  a.tickets = h->barrier.p + 2;
  a.stripes = h->scal.p + 8;
  a.mono = reinterpret_cast<unsigned long long*>(h->barrier.p + 8);
  fill_args(a, o);
  // momentum_by_linearity applies to the FP64 iterations only: in FP32 the recombined product's rounding makes
  // the line search retry more often (measured slower, with a worse starting point for the FP64 part)
  a.lin_momentum = 0;
  a.stall_iters = o->fp32_stall_iters;
  BG_CUDA(launch_convert(n3, h->X.p, h->X32.p, s));
  BG_CUDA(cudaMemsetAsync(h->barrier.p, 0, 16 * sizeof(unsigned), s));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  int grid = pg_max_grid(h->device, true, true);
  if (grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "cooperative occupancy query failed");
  const int want = (a.nchunks + 7) / 8;
  if (want < grid) grid = want < 1 ? 1 : want;
  if (int e = ensure_cta_lists(h, grid)) return e;
  a.cta_ptr = h->cta_ptr.p;
  a.cta_list = h->cta_list.p;
  BG_CUDA(cudaEventRecord(h->ev0, s));
  BG_CUDA(launch_pg_persistent(a, grid, s));
  BG_CUDA(cudaEventRecord(h->ev1, s));
  PGOut out{};
  int st = 0;
  BG_CUDA(cudaMemcpyAsync(&out, h->pgout.p, sizeof(PGOut), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  float ms32 = 0.f;
  BG_CUDA(cudaEventElapsedTime(&ms32, h->ev0, h->ev1));
  if (st != 0) return fail(st, "device-side wait timed out in the FP32 projected-gradient kernel");
  const float* b32 =
      out.best_buf == 3 ? h->XB32.p : (out.best_buf == 4 ? h->Wv32.p : h->X32.p + (size_t)out.best_buf * n3);
  BG_CUDA(launch_convert(n3, b32, h->X.p, s));
  const unsigned it32 = out.iters;
  const PGTraffic t32 = pg_traffic(out, n, h->W.nnzb, o->variant, 4.0, lin_momentum(o) != 0);
  bogus_gpu_pg_options o64 = *o;
  o64.max_iters = o->refine_max_iters;
  // FP64 iterations with FP32 correction products, then the plain FP64 check from their best iterate
  unsigned ith = 0;
  float msh = 0.f;
  bogus_gpu_solve_stats sth{};
  if (o->fp32_products_refresh) {
    BG_CUDA(h->hy_d.ensure(4 * n3));
    BG_CUDA(h->hy_xref.ensure(n3));
    BG_CUDA(h->hy_wxref.ensure(n3));
    const HyArgs hy{h->val32.p, h->hy_d.p, h->hy_xref.p, h->hy_wxref.p, o->fp32_products_refresh, n3};
    double resh = 0.0;
    const double* besth = nullptr;
    const int hst = run_pg(h, &o64, &resh, &ith, &besth, &hy);
    if (hst != BOGUS_GPU_OK && hst != BOGUS_GPU_NOT_CONVERGED) return hst;
    if (besth != h->X.p) BG_CUDA(cudaMemcpyAsync(h->X.p, besth, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    sth = h->last_stats;
    msh = h->last_ms;
    o64.max_iters = o->refine_max_iters > ith ? o->refine_max_iters - ith : 1u;
  }
  const int rst = run_pg(h, &o64, residual, iters, best);
  if (rst != BOGUS_GPU_OK && rst != BOGUS_GPU_NOT_CONVERGED) return rst;
  h->last_stats.refine_iterations = h->last_stats.iterations + ith;
  h->last_stats.fp32_product_iterations = ith;
  h->last_stats.iterations = it32 + ith + h->last_stats.iterations;
  h->last_stats.w_passes += t32.passes + sth.w_passes;
  h->last_stats.algorithmic_bytes += t32.bytes + sth.algorithmic_bytes;
  h->last_stats.fp64_fma += sth.fp64_fma;
  h->last_stats.fp32_device_ms = ms32;
  h->last_ms += ms32 + msh;
  h->last_launches += o->fp32_products_refresh ? 2 : 1;
  if (iters) *iters = it32 + ith + *iters;
  return rst;
}

int check_pg_options(const bogus_gpu_pg_options* o) {
  if (!o) return fail(BOGUS_GPU_BAD_INPUT, "null options");
  if (o->variant < BOGUS_GPU_PG_STANDARD || o->variant > BOGUS_GPU_PG_SPG)
    return fail(BOGUS_GPU_BAD_INPUT, "unknown projected-gradient variant");
  const bool std_conj = o->variant == BOGUS_GPU_PG_STANDARD || o->variant == BOGUS_GPU_PG_CONJUGATED;
  if (std_conj && o->mixed_precision)
    return fail(BOGUS_GPU_BAD_INPUT, "the Standard and Conjugated variants run in FP64 only");
  if (o->ls_iters == 0 && o->variant != BOGUS_GPU_PG_SPG)
    return fail(BOGUS_GPU_BAD_INPUT, "ls_iters must be >= 1 (the reference reuses an undefined step otherwise)");
  if (!(o->tol >= 0) || !(o->ls_optimistic_factor > 0) || !(o->ls_pessimistic_factor > 0))
    return fail(BOGUS_GPU_BAD_INPUT, "invalid projected-gradient factors");
  if (o->mixed_precision && o->refine_max_iters == 0)
    return fail(BOGUS_GPU_BAD_INPUT, "mixed precision needs refine_max_iters >= 1 (the FP64 residual)");
  if (o->fp32_products_refresh && (!o->mixed_precision || o->variant != BOGUS_GPU_PG_APGD || o->momentum_by_linearity))
    return fail(BOGUS_GPU_BAD_INPUT,
                "fp32_products_refresh needs mixed_precision and the APGD variant, without momentum_by_linearity");
  return BOGUS_GPU_OK;
}

// ---- Gauss-Seidel ---------------------------------------------------------------------------------
int prepare_gs(bogus_gpu_problem* h, double auto_reg, int use_coloring) {
  GSCache& g = h->gs;
  if (g.valid && g.auto_reg == auto_reg && g.use_coloring == use_coloring) return BOGUS_GPU_OK;
  if (int e = ensure_host_lower(h)) return e;
  g.drop_graphs();
  const HostBSR& low = h->host_lower;
  const int n = low.n;
  if (use_coloring) {
    greedy_coloring(low, g.perm, g.colors);
  } else {
    g.perm.resize(n);
    for (int i = 0; i < n; ++i) g.perm[i] = i;
    g.colors = {0, n};
  }
  const HostBSR plow = permute_lower(low, g.perm);
  const HostBSR pf = expand_lower(n, plow.rowptr.data(), plow.col.data(), plow.val.data());
  std::vector<double> pb(3 * (size_t)n), pmu(n), local(9 * (size_t)n, 0.0), reg(n, 0.0), sc(n, 1.0);
  for (int i = 0; i < n; ++i) {
    const int o = g.perm[i];
    for (int k = 0; k < 3; ++k) pb[3 * (size_t)i + k] = h->host_b[3 * (size_t)o + k];
    pmu[i] = h->host_mu[o];
    for (int k = pf.rowptr[i]; k < pf.rowptr[i + 1]; ++k)
      if (pf.col[k] == i) std::copy(&pf.val[9 * (size_t)k], &pf.val[9 * (size_t)k] + 9, &local[9 * (size_t)i]);
    double* D = &local[9 * (size_t)i];
    sc[i] = dmax(1.0, ((D[0] + D[4]) + D[8]) / 3.0);
    if (auto_reg > 0.) {
      reg[i] = dmax(0.0, auto_reg - min_eigen_symmetric3(D));
      D[0] += reg[i];
      D[4] += reg[i];
      D[8] += reg[i];
    }
  }
  // levels of the sweep (renumbered so that the sweep visits 0, 1, 2, ...): one more than the highest level
  // among the earlier neighbours, i.e. the lower-triangle neighbours of the permuted matrix
  std::vector<int> level(n, 0);
  int nlevels = n > 0 ? 1 : 0;
  for (int i = 0; i < n; ++i) {
    int lv = 0;
    for (int k = plow.rowptr[i]; k < plow.rowptr[i + 1]; ++k) {
      const int j = plow.col[k];
      if (j < i && level[j] + 1 > lv) lv = level[j] + 1;
    }
    level[i] = lv;
    if (lv + 1 > nlevels) nlevels = lv + 1;
  }
  g.level_off.assign(nlevels + 1, 0);
  for (int i = 0; i < n; ++i) ++g.level_off[level[i] + 1];
  for (int L = 0; L < nlevels; ++L) g.level_off[L + 1] += g.level_off[L];
  std::vector<int> order(n), fill(g.level_off.begin(), g.level_off.end() - 1);
  for (int i = 0; i < n; ++i) order[fill[level[i]]++] = i;
  const int nnz = pf.nnzb();
  const int ntiles = (n + kGSTile - 1) / kGSTile;
  BG_CUDA(g.order.ensure(n));
  BG_CUDA(g.rowptr.ensure(n + 1));
  BG_CUDA(g.col.ensure(nnz));
  BG_CUDA(g.val.ensure(9 * (size_t)nnz));
  BG_CUDA(g.local.ensure(9 * (size_t)n));
  BG_CUDA(g.reg.ensure(n));
  BG_CUDA(g.scaling.ensure(n));
  BG_CUDA(g.b.ensure(3 * (size_t)n));
  BG_CUDA(g.mu.ensure(n));
  BG_CUDA(g.x.ensure(3 * (size_t)n));
  BG_CUDA(g.xbest.ensure(3 * (size_t)n));
  BG_CUDA(g.y.ensure(3 * (size_t)n));
  BG_CUDA(g.nx2.ensure(n));
  BG_CUDA(g.ndx2.ensure(n));
  BG_CUDA(g.skip.ensure(n));
  BG_CUDA(g.processed.ensure(n));
  BG_CUDA(g.tile_max.ensure(2 * (size_t)(ntiles > 0 ? ntiles : 1)));
  BG_CUDA(g.ndx_ref.ensure(2));
  BG_CUDA(g.chunk.ensure((n + 31) / 32 + 1));
  BG_CUDA(g.scalar.ensure(2));
  BG_CUDA(g.flow.ensure(2));
  BG_CUDA(g.done.ensure(n > 0 ? n : 1));
  BG_CUDA(h->status.ensure(1));
  g.flow_grid = gs_flow_grid(h->device);
  if (g.flow_grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "occupancy query failed (Gauss-Seidel sweep)");
  cudaStream_t s = h->stream;
  {
    const unsigned f0[2] = {0u, 1u};
    BG_CUDA(cudaMemcpyAsync(g.flow.p, f0, sizeof(f0), cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemsetAsync(g.done.p, 0, sizeof(unsigned) * (n > 0 ? n : 1), s));
  }
  BG_CUDA(cudaMemcpyAsync(g.rowptr.p, pf.rowptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
  if (nnz) {
    BG_CUDA(cudaMemcpyAsync(g.col.p, pf.col.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g.val.p, pf.val.data(), sizeof(double) * 9 * (size_t)nnz, cudaMemcpyHostToDevice, s));
  }
  if (n) {
    BG_CUDA(cudaMemcpyAsync(g.order.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g.local.p, local.data(), sizeof(double) * 9 * (size_t)n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g.reg.p, reg.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g.scaling.p, sc.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g.b.p, pb.data(), sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(g.mu.p, pmu.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
  }
  BG_CUDA(cudaStreamSynchronize(s));
  g.auto_reg = auto_reg;
  g.use_coloring = use_coloring;
  g.valid = true;
  return BOGUS_GPU_OK;
}

// One sweep (the dataflow kernel of the assembled or the matrix-free sweep), then the skip update. Captured once
// per parity into a CUDA graph and replayed (the arguments never change between sweeps of the same settings).
int launch_sweep(bogus_gpu_problem* h, GSCache& g, const GSArgs& a, int parity, double abs_skip_tol,
                 double skip_tol, int abs_skip_iters, long long key, bool product) {
  cudaStream_t s = h->stream;
  const int nlevels = (int)g.level_off.size() - 1;
  if (g.sweep_key != key) g.drop_graphs();
  if (!g.sweep[parity]) {
    cudaGraph_t graph = nullptr;
    BG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    e = product ? launch_pgs_flow(a, g.flow_grid, parity, s) : launch_gs_flow(a, g.flow_grid, parity, s);
    if (e == cudaSuccess) e = launch_gs_skip(a, parity, abs_skip_tol, skip_tol, abs_skip_iters, s);
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(BOGUS_GPU_CUDA_ERROR, std::string("sweep capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    const cudaError_t e3 = cudaGraphInstantiate(&g.sweep[parity], graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) return fail(BOGUS_GPU_CUDA_ERROR, std::string("sweep instantiate: ") + cudaGetErrorString(e3));
    g.sweep_key = key;
  }
  BG_CUDA(cudaGraphLaunch(g.sweep[parity], s));
  h->last_launches += 2;
  return BOGUS_GPU_OK;
}

// error function of the permuted GS problem at g.x: u = init + W x (init = b) as in solveWithLinearConstraints
int gs_eval(bogus_gpu_problem* h, const GSArgs& a, const double* xdev, const double* u_init, bool desaxce, bool use_inf,
            double* err) {
  GSCache& g = h->gs;
  const int n = a.n;
  DevBSR Wp;
  Wp.n = n;
  Wp.rowptr = g.rowptr.p;
  Wp.col = g.col.p;
  Wp.val = g.val.p;
  const double* u = u_init;
  if (xdev) {
    BG_CUDA(launch_spmv(Wp, xdev, u_init, g.y.p, h->stream));
    u = g.y.p;
  }
  const double* xe = xdev ? xdev : g.y.p;  // x = 0 path handled by caller passing a zero vector
  BG_CUDA(launch_eval_chunks(n, xe, u, g.mu.p, g.scaling.p, desaxce, use_inf, g.chunk.p, h->stream));
  BG_CUDA(launch_combine(g.chunk.p, (n + 31) / 32, use_inf, use_inf ? 0.0 : (double)(1 + n), g.scalar.p, h->stream));
  BG_CUDA(cudaMemcpyAsync(err, g.scalar.p, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  h->last_launches += xdev ? 3 : 2;
  return BOGUS_GPU_OK;
}

}  // namespace

// =================================================================================================
extern "C" {

void bogus_gpu_pg_options_default(bogus_gpu_pg_options* o) {
  if (!o) return;
  o->tol = 1.e-6;
  o->max_iters = 300;
  o->ls_iters = 8;
  o->ls_optimistic_factor = 1.25;
  o->ls_pessimistic_factor = .5;
  o->ls_armijo_coefficient = .5;
  o->variant = BOGUS_GPU_PG_APGD;
  o->use_infinity_norm = 0;
  o->static_problem = 1;
  o->mixed_precision = 0;
  o->refine_max_iters = 50;
  o->momentum_by_linearity = 0;
  o->fp32_stall_iters = 4;
  o->fp32_products_refresh = 0;
}

void bogus_gpu_gs_options_default(bogus_gpu_gs_options* o) {
  if (!o) return;
  o->tol = 1.e-6;
  o->max_iters = 250;
  o->eval_every = 25;
  o->skip_tol = 1.e-6;
  o->skip_iters = 10;
  o->auto_regularization = 0.;
  o->try_zero_as_well = 1;
  o->use_infinity_norm = 0;
  o->static_problem = 0;
  o->local_strategy = BOGUS_GPU_LOCAL_REV_HYBRID;
  o->use_coloring = 0;
}

const char* bogus_gpu_status_string(int s) {
  switch (s) {
    case BOGUS_GPU_OK: return "ok";
    case BOGUS_GPU_NOT_CONVERGED: return "not converged";
    case BOGUS_GPU_BAD_INPUT: return "bad input";
    case BOGUS_GPU_NONFINITE: return "non-finite input";
    case BOGUS_GPU_CUDA_ERROR: return "CUDA error";
    case BOGUS_GPU_TIMEOUT: return "device wait timed out";
    case BOGUS_GPU_NO_DEVICE: return "no suitable CUDA device";
    case BOGUS_GPU_NO_PROBLEM: return "no problem set";
  }
  return "unknown status";
}

const char* bogus_gpu_last_error(void) { return g_last_error.c_str(); }

int bogus_gpu_create(int device, bogus_gpu_problem** out) {
  if (!out) return fail(BOGUS_GPU_BAD_INPUT, "null output pointer");
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return fail(BOGUS_GPU_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= count) return fail(BOGUS_GPU_NO_DEVICE, "device index out of range");
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return fail(BOGUS_GPU_NO_DEVICE, "device query failed");
  if (prop.major != 10 || prop.minor != 3)
    return fail(BOGUS_GPU_NO_DEVICE, std::string("this library is built for sm_103 (GB300); found ") + prop.name);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) return fail(BOGUS_GPU_NO_DEVICE, "device lacks cooperative launch");
  auto* h = new bogus_gpu_problem;
  h->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) {
    delete h;
    return fail(BOGUS_GPU_CUDA_ERROR, "stream/event creation failed");
  }
  *out = h;
  return BOGUS_GPU_OK;
}

int bogus_gpu_destroy(bogus_gpu_problem* h) {
  if (!h) return BOGUS_GPU_OK;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  if (h->batch_graph) cudaGraphExecDestroy(h->batch_graph);
  if (h->pinned_out) cudaFreeHost(h->pinned_out);
  if (h->pinned_status) cudaFreeHost(h->pinned_status);
  h->tune_x.release();
  for (auto* b : {&h->val, &h->b, &h->mu, &h->scaling, &h->X, &h->MX, &h->Y, &h->S0, &h->XB, &h->Wv, &h->csum,
                  &h->scal, &h->trace, &h->vx, &h->vy, &h->chunk, &h->scalar, &h->minv, &h->H, &h->T, &h->mf})
    b->release();
  for (auto* b : {&h->val32, &h->b32, &h->mu32, &h->sc32, &h->X32, &h->MX32, &h->Y32, &h->S032, &h->XB32, &h->Wv32,
                  &h->val32p})
    b->release();
  h->slot0.release();
  h->chunk_order.release();
  h->cta_ptr.release();
  h->cta_list.release();
  h->icol.release();
  h->ival.release();
  for (auto* b : {&h->a_prox, &h->a_f, &h->a_w, &h->a_mu, &h->a_invmu, &h->a_x, &h->a_r, &h->a_ut, &h->a_z, &h->a_zacc,
                  &h->a_rs1, &h->a_rs2, &h->a_yprev})
    b->release();
  h->bptr.release();
  h->bent.release();
  h->border.release();
  h->admm_out.release();
  h->cad_b.release();
  for (auto* b : {&h->meche_E, &h->meche_w, &h->meche_r, &h->meche_v, &h->meche_fd}) b->release();
  for (auto* b : {&h->adj_V, &h->adj_Pc, &h->adj_D, &h->adj_K, &h->adj_P, &h->adj_R, &h->adj_Z, &h->adj_Dir,
                  &h->adj_Y, &h->adj_Q, &h->adj_S, &h->adj_dmu, &h->adj_r, &h->adj_g, &h->adj_Tc, &h->adj_Rh,
                  &h->adj_Ph, &h->adj_Sv, &h->adj_Sh, &h->adj_Tv})
    b->release();
  h->adj_out.release();
  h->rowptr.release();
  h->col.release();
  h->diag.release();
  h->contact_ptr.release();
  h->chunk_ptr.release();
  h->queue.release();
  h->col_local.release();
  h->next.release();
  h->batch_out.release();
  h->cb.release();
  h->pgout.release();
  h->barrier.release();
  h->status.release();
  h->gs.release();
  h->pgs.release();
  h->pgs_Mx.release();
  cudaEventDestroy(h->ev0);
  cudaEventDestroy(h->ev1);
  cudaStreamDestroy(h->stream);
  delete h;
  return BOGUS_GPU_OK;
}

static int set_dual_any(bogus_gpu_problem* h, int n, const int* rowptr, const int* colidx, const double* blocks,
                        int symmetric_lower, const double* b, const double* mu);

int bogus_gpu_set_dual(bogus_gpu_problem* h, int n, const int* rowptr, const int* colidx, const double* blocks,
                       int symmetric_lower, const double* b, const double* mu) {
  if (int e = check_handle(h)) return e;
  const int st = set_dual_any(h, n, rowptr, colidx, blocks, symmetric_lower, b, mu);
  if (st == BOGUS_GPU_OK) {
    h->permuted = false;
    h->perm.clear();
    h->inv_perm.clear();
  }
  return st;
}

static int set_dual_any(bogus_gpu_problem* h, int n, const int* rowptr, const int* colidx, const double* blocks,
                        int symmetric_lower, const double* b, const double* mu) {
  if (n < 0 || (n > 0 && (!rowptr || !b || !mu))) return fail(BOGUS_GPU_BAD_INPUT, "null input array");
  if (n > 0 && rowptr[n] > 0 && (!colidx || !blocks)) return fail(BOGUS_GPU_BAD_INPUT, "null block arrays");
  if (!rowptr) return fail(BOGUS_GPU_BAD_INPUT, "null row pointer");
  if (symmetric_lower) return set_dual_lower(h, n, rowptr, colidx, blocks, b, mu);
  const std::string err = validate_bsr(n, rowptr, colidx, blocks, false);
  if (!err.empty()) return fail(err.find("non-finite") != std::string::npos ? BOGUS_GPU_NONFINITE : BOGUS_GPU_BAD_INPUT, err);
  if (int e = check_finite(b, 3 * (size_t)n, "b")) return e;
  if (int e = check_finite(mu, n, "mu")) return e;
  if (int e = set_device(h)) return e;
  HostBSR full;
  {
    full.n = n;
    full.rowptr.assign(rowptr, rowptr + n + 1);
    full.col.assign(colidx, colidx + rowptr[n]);
    full.val.assign(blocks, blocks + 9 * (size_t)rowptr[n]);
    h->host_lower = lower_of(full);
  }
  h->host_lower_valid = true;
  h->low_pending = false;
  h->host_b.assign(b, b + 3 * (size_t)n);
  h->host_mu.assign(mu, mu + n);
  return upload_full(h, full, b, mu);
}

int bogus_gpu_set_dual_device(bogus_gpu_problem* h, int n, int nnzb, const int* d_rowptr, const int* d_colidx,
                              const double* d_blocks, const double* d_b, const double* d_mu) {
  if (int e = check_handle(h)) return e;
  if (n < 0 || nnzb < 0) return fail(BOGUS_GPU_BAD_INPUT, "negative size");
  if (n > 0 && (!d_rowptr || !d_b || !d_mu || (nnzb > 0 && (!d_colidx || !d_blocks))))
    return fail(BOGUS_GPU_BAD_INPUT, "null device pointer");
  if (int e = set_device(h)) return e;
  {
    // the caller's arrays are checked where they lie, before anything is copied: a rejected problem leaves the
    // handle's problem in place
    cudaStream_t s = h->stream;
    BG_CUDA(h->pat_check.ensure(2));
    BG_CUDA(launch_check_full(n, nnzb, d_rowptr, d_colidx, h->pat_check.p, s));
    BG_CUDA(cudaMemsetAsync(h->pat_check.p + 1, 0, sizeof(int), s));
    BG_CUDA(launch_any_nonfinite(9 * (size_t)nnzb, d_blocks, h->pat_check.p + 1, s));
    BG_CUDA(launch_any_nonfinite(3 * (size_t)n, d_b, h->pat_check.p + 1, s));
    BG_CUDA(launch_any_nonfinite((size_t)n, d_mu, h->pat_check.p + 1, s));
    int check[2] = {0, 0};
    BG_CUDA(cudaMemcpyAsync(check, h->pat_check.p, sizeof(check), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    if (n > 0 && check[0] < n)
      return fail(BOGUS_GPU_BAD_INPUT, "row " + std::to_string(check[0]) + " of W is malformed (row pointers out of "
                  "order or range, a column out of range or not increasing, or no diagonal block)");
    if (check[1]) return fail(BOGUS_GPU_NONFINITE, "non-finite value in W, b or mu");
  }
  BG_CUDA(h->rowptr.ensure(n + 1));
  BG_CUDA(h->col.ensure(nnzb));
  BG_CUDA(h->val.ensure(9 * (size_t)nnzb));
  BG_CUDA(h->diag.ensure(n));
  BG_CUDA(h->b.ensure(3 * (size_t)n));
  BG_CUDA(h->mu.ensure(n));
  BG_CUDA(h->scaling.ensure(n));
  cudaStream_t s = h->stream;
  BG_CUDA(cudaMemcpyAsync(h->rowptr.p, d_rowptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice, s));
  if (nnzb) {
    BG_CUDA(cudaMemcpyAsync(h->col.p, d_colidx, sizeof(int) * nnzb, cudaMemcpyDeviceToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->val.p, d_blocks, sizeof(double) * 9 * (size_t)nnzb, cudaMemcpyDeviceToDevice, s));
  }
  if (n) {
    BG_CUDA(cudaMemcpyAsync(h->b.p, d_b, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->mu.p, d_mu, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  }
  h->W.n = n;
  h->W.nnzb = nnzb;
  h->W.rowptr = h->rowptr.p;
  h->W.col = h->col.p;
  h->W.val = h->val.p;
  h->W.diag = h->diag.p;
  BG_CUDA(launch_diag_and_scaling(h->W, h->scaling.p, s));
  BG_CUDA(cudaStreamSynchronize(s));
  h->has_dual = true;
  h->permuted = false;
  h->host_lower_valid = false;
  h->low_pending = false;
  h->gs.valid = false;
  h->nproblems = 0;
  h->fp32_valid = false;
  h->fp32p_valid = false;
  h->il_valid = false;
  h->adj_valid = false;
  return BOGUS_GPU_OK;
}

int bogus_gpu_nnzb(const bogus_gpu_problem* h, int* nnzb) {
  if (int e = check_handle(h)) return e;
  if (nnzb) *nnzb = h->W.nnzb;
  return BOGUS_GPU_OK;
}

int bogus_gpu_set_callback(bogus_gpu_problem* h, bogus_gpu_callback cb, void* user) {
  if (int e = check_handle(h)) return e;
  h->callback = cb;
  h->callback_user = user;
  return BOGUS_GPU_OK;
}

int bogus_gpu_spmv(bogus_gpu_problem* h, const double* x, double* y) {
  if (int e = check_handle(h)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (int e = set_device(h)) return e;
  const size_t n3 = 3 * (size_t)h->W.n;
  if (n3 == 0) return BOGUS_GPU_OK;
  BG_CUDA(h->vx.ensure(n3));
  BG_CUDA(h->vy.ensure(n3));
  BG_CUDA(cudaMemcpyAsync(h->vx.p, x, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream));
  BG_CUDA(launch_spmv(h->W, h->vx.p, nullptr, h->vy.p, h->stream));
  BG_CUDA(cudaMemcpyAsync(y, h->vy.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return BOGUS_GPU_OK;
}

static int eval_stored(bogus_gpu_problem* h, const double* r, int static_problem, int use_inf, double* residual) {
  if (int e = check_handle(h)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (int e = set_device(h)) return e;
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  if (n == 0) {
    if (residual) *residual = 0.0;
    return BOGUS_GPU_OK;
  }
  BG_CUDA(h->vx.ensure(n3));
  BG_CUDA(h->vy.ensure(n3));
  BG_CUDA(h->chunk.ensure((n + 31) / 32));
  BG_CUDA(h->scalar.ensure(2));
  BG_CUDA(cudaMemcpyAsync(h->vx.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream));
  BG_CUDA(launch_spmv(h->W, h->vx.p, nullptr, h->vy.p, h->stream));
  BG_CUDA(launch_add((int)n3, h->vy.p, h->b.p, h->vy.p, h->stream));
  BG_CUDA(launch_eval_chunks(n, h->vx.p, h->vy.p, h->mu.p, h->scaling.p, !static_problem, use_inf != 0, h->chunk.p,
                             h->stream));
  BG_CUDA(launch_combine(h->chunk.p, (n + 31) / 32, use_inf != 0, use_inf ? 0.0 : (double)(1 + n), h->scalar.p,
                         h->stream));
  double v = 0;
  BG_CUDA(cudaMemcpyAsync(&v, h->scalar.p, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  if (residual) *residual = v;
  return BOGUS_GPU_OK;
}

static int solve_pg_device_stored(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* d_r, double* residual,
                                  unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (int e = check_pg_options(o)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (int e = set_device(h)) return e;
  const size_t n3 = 3 * (size_t)h->W.n;
  if (n3 == 0) {
    if (residual) *residual = 0.0;
    if (iters) *iters = 0;
    return BOGUS_GPU_OK;
  }
  if (int e = ensure_pg_work(h, o->max_iters)) return e;
  BG_CUDA(cudaMemcpyAsync(h->X.p, d_r, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
  const double* best = nullptr;
  const int st = o->mixed_precision ? run_pg_mixed(h, o, residual, iters, &best) : run_pg(h, o, residual, iters, &best);
  if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
  BG_CUDA(cudaMemcpyAsync(d_r, best, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return st;
}

static int solve_pg_stored(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* r, double* residual,
                           unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (int e = check_pg_options(o)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (int e = set_device(h)) return e;
  const size_t n3 = 3 * (size_t)h->W.n;
  if (n3 == 0) {
    if (residual) *residual = 0.0;
    if (iters) *iters = 0;
    return BOGUS_GPU_OK;
  }
  if (int e = check_finite(r, n3, "r")) return e;
  if (int e = ensure_pg_work(h, o->max_iters)) return e;
  BG_CUDA(cudaMemcpyAsync(h->X.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream));
  const double* best = nullptr;
  const int st = o->mixed_precision ? run_pg_mixed(h, o, residual, iters, &best) : run_pg(h, o, residual, iters, &best);
  if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
  BG_CUDA(cudaMemcpyAsync(r, best, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return st;
}

int bogus_gpu_coloring(bogus_gpu_problem* h, int* perm, int* colors, int* ncolors) {
  if (int e = check_handle(h)) return e;
  if (int e = ensure_host_lower(h)) return e;
  std::vector<int> p, c;
  greedy_coloring(h->host_lower, p, c);
  if (perm) std::memcpy(perm, p.data(), sizeof(int) * p.size());
  if (colors) std::memcpy(colors, c.data(), sizeof(int) * c.size());
  if (ncolors) *ncolors = (int)c.size() - 1;
  return BOGUS_GPU_OK;
}

}  // extern "C"

namespace {

int check_gs_options(const bogus_gpu_gs_options* o) {
  if (!o) return fail(BOGUS_GPU_BAD_INPUT, "null options");
  if (o->eval_every == 0) return fail(BOGUS_GPU_BAD_INPUT, "eval_every must be >= 1");
  if (o->local_strategy < 0 || o->local_strategy > 3) return fail(BOGUS_GPU_BAD_INPUT, "unknown local strategy");
  return BOGUS_GPU_OK;
}

GSArgs gs_args(bogus_gpu_problem* h, const bogus_gpu_gs_options* o) {
  GSCache& g = h->gs;
  GSArgs a{};
  a.n = h->W.n;
  a.rowptr = g.rowptr.p;
  a.col = g.col.p;
  a.val = g.val.p;
  a.local = g.local.p;
  a.reg = g.reg.p;
  a.scaling = g.scaling.p;
  a.b = g.b.p;
  a.mu = g.mu.p;
  a.x = g.x.p;
  a.nx2 = g.nx2.p;
  a.ndx2 = g.ndx2.p;
  a.skip = g.skip.p;
  a.processed = g.processed.p;
  a.tile_max = g.tile_max.p;
  a.ndx_ref = g.ndx_ref.p;
  a.order = g.order.p;
  a.desaxce = o->static_problem ? 0 : 1;
  a.strat = o->local_strategy;
  a.flow = g.flow.p;
  a.done = g.done.p;
  a.status = h->status.p;
  return a;
}

// GaussSeidel::solve (GaussSeidel.impl.hpp:144-205) on the prepared (permuted) problem, rhs g.b, from g.x;
// leaves the result in g.x and the (iteration, error) pairs in *trace.
int run_gs_core(bogus_gpu_problem* h, const bogus_gpu_gs_options* o, double* residual, unsigned* iters,
                std::vector<std::pair<unsigned, double>>* trace, bool* converged_out) {
  GSCache& g = h->gs;
  cudaStream_t s = h->stream;
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  const int ntiles = (n + kGSTile - 1) / kGSTile;
  BG_CUDA(cudaMemsetAsync(g.tile_max.p, 0, sizeof(unsigned long long) * 2 * ntiles, s));
  BG_CUDA(cudaMemsetAsync(g.ndx_ref.p, 0, sizeof(double) * 2, s));
  BG_CUDA(cudaMemsetAsync(g.skip.p, 0, n, s));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  const GSArgs a = gs_args(h, o);
  // a wait of the dataflow sweep that ran out (BOGUS_GPU_TIMEOUT), read when the host synchronises anyway
  auto sweep_status = [&]() -> int {
    int st = 0;
    BG_CUDA(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    if (st != 0) return fail(st, "device-side wait timed out in the Gauss-Seidel sweep");
    return BOGUS_GPU_OK;
  };
  const bool desaxce = !o->static_problem;
  const bool use_inf = o->use_infinity_norm != 0;
  // initial evaluation and tryZero (GaussSeidel.impl.hpp:152-167)
  double err_best = DBL_MAX;
  bool has_best = false;
  double err = 0;
  if (int e = gs_eval(h, a, g.x.p, g.b.p, desaxce, use_inf, &err)) return e;
  if (err < err_best) {
    BG_CUDA(cudaMemcpyAsync(g.xbest.p, g.x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    err_best = err;
    has_best = true;
  }
  if (o->try_zero_as_well) {
    // eval(law, b, 0): u = b, x = 0
    BG_CUDA(cudaMemsetAsync(g.y.p, 0, sizeof(double) * n3, s));
    BG_CUDA(launch_eval_chunks(n, g.y.p, g.b.p, g.mu.p, g.scaling.p, desaxce, use_inf, g.chunk.p, s));
    BG_CUDA(launch_combine(g.chunk.p, (n + 31) / 32, use_inf, use_inf ? 0.0 : (double)(1 + n), g.scalar.p, s));
    double err_zero = 0;
    BG_CUDA(cudaMemcpyAsync(&err_zero, g.scalar.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    h->last_launches += 2;
    if (err_zero < err_best) {
      err_best = err_zero;
      BG_CUDA(cudaMemsetAsync(g.xbest.p, 0, sizeof(double) * n3, s));
      BG_CUDA(cudaMemsetAsync(g.x.p, 0, sizeof(double) * n3, s));
      has_best = true;
    } else if (has_best) {
      BG_CUDA(cudaMemcpyAsync(g.x.p, g.xbest.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    }
  }
  if (trace) trace->push_back({0u, err_best});
  const double abs_skip_tol = dmin(o->skip_tol, o->tol);
  const int abs_skip_iters = (int)dmin((double)o->skip_iters, (double)(unsigned)std::sqrt((double)n));
  // settings baked into the captured sweeps
  long long key = 0;
  {
    double st = o->skip_tol, ast = abs_skip_tol;
    unsigned long long b1, b2;
    std::memcpy(&b1, &st, 8);
    std::memcpy(&b2, &ast, 8);
    key = (long long)((b1 * 1000003ull) ^ (b2 * 10007ull) ^ ((unsigned long long)abs_skip_iters << 8) ^
                      ((unsigned long long)a.desaxce << 4) ^ (unsigned long long)a.strat);
    if (key < 0) key = -key - 1;
  }
  unsigned it;
  int parity = 0;
  bool converged = false;
  for (it = 1; it <= o->max_iters; ++it) {
    if (int e = launch_sweep(h, h->gs, a, parity, abs_skip_tol, o->skip_tol, abs_skip_iters, key, false)) return e;
    parity ^= 1;
    if (0 == (it % o->eval_every)) {
      if (int e = gs_eval(h, a, g.x.p, g.b.p, desaxce, use_inf, &err)) return e;
      if (int e = sweep_status()) return e;
      if (err < err_best) {
        BG_CUDA(cudaMemcpyAsync(g.xbest.p, g.x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
        err_best = err;
        has_best = true;
      }
      if (trace) trace->push_back({it, err});
      if (err < o->tol) {
        converged = true;
        break;
      }
      BG_CUDA(launch_scale_scalar(g.ndx_ref.p + parity, (double)o->eval_every, s));
      h->last_launches += 1;
    }
  }
  if (int e = sweep_status()) return e;
  if (it > o->max_iters && has_best)
    BG_CUDA(cudaMemcpyAsync(g.x.p, g.xbest.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
  if (residual) *residual = err_best;
  if (iters) *iters = it > o->max_iters ? o->max_iters : it;
  if (converged_out) *converged_out = converged;
  return BOGUS_GPU_OK;
}

// r (caller's order, host) <-> g.x (sweep order, device)
int gs_load_x(bogus_gpu_problem* h, const double* r) {
  GSCache& g = h->gs;
  const int n = h->W.n;
  std::vector<double> pr(3 * (size_t)n);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) pr[3 * (size_t)i + k] = r[3 * (size_t)g.perm[i] + k];
  BG_CUDA(cudaMemcpyAsync(g.x.p, pr.data(), sizeof(double) * pr.size(), cudaMemcpyHostToDevice, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return BOGUS_GPU_OK;
}
int gs_store_x(bogus_gpu_problem* h, double* r) {
  GSCache& g = h->gs;
  const int n = h->W.n;
  std::vector<double> pr(3 * (size_t)n);
  BG_CUDA(cudaMemcpyAsync(pr.data(), g.x.p, sizeof(double) * pr.size(), cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) r[3 * (size_t)g.perm[i] + k] = pr[3 * (size_t)i + k];
  return BOGUS_GPU_OK;
}

}  // namespace

extern "C" {

static int solve_gs_stored(bogus_gpu_problem* h, const bogus_gpu_gs_options* o, double* r, double* residual,
                           unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (int e = check_gs_options(o)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (int e = set_device(h)) return e;
  const int n = h->W.n;
  if (n == 0) {
    if (residual) *residual = 0.0;
    if (iters) *iters = 0;
    return BOGUS_GPU_OK;
  }
  if (int e = check_finite(r, 3 * (size_t)n, "r")) return e;
  if (int e = prepare_gs(h, o->auto_regularization, o->use_coloring ? 1 : 0)) return e;
  h->last_launches = 0;
  if (int e = gs_load_x(h, r)) return e;
  BG_CUDA(cudaEventRecord(h->ev0, h->stream));
  std::vector<std::pair<unsigned, double>> trace;
  bool converged = false;
  if (int e = run_gs_core(h, o, residual, iters, &trace, &converged)) return e;
  BG_CUDA(cudaEventRecord(h->ev1, h->stream));
  if (int e = gs_store_x(h, r)) return e;
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  if (h->callback)
    for (auto& t : trace) h->callback(t.first, t.second, h->callback_user);
  return converged ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

// ---- matrix-free Gauss-Seidel (ProductGaussSeidel<HType, MInvType, true>; PrimalFrictionProblem::solveWith,
//      PrimalFrictionProblem.cpp:41-59) ------------------------------------------------------------------------
}  // extern "C"

namespace {

// Levels from the contacts' bodies (two contacts depend on each other when they share a body), T = M^-1 H^T per
// slot, local matrices sum_t H_t T_t with their scalings and regularisation.
int prepare_pgs(bogus_gpu_problem* h, double auto_reg) {
  GSCache& g = h->pgs;
  if (g.valid && g.auto_reg == auto_reg) return BOGUS_GPU_OK;
  g.drop_graphs();
  const int n = h->ncontacts, nb = h->nbodies, d = h->ndof;
  const size_t n3 = 3 * (size_t)n;
  cudaStream_t s = h->stream;
  if (int e = ensure_incidence(h)) return e;
  BG_CUDA(h->T.ensure(2 * (size_t)n * d * 3));
  BG_CUDA(launch_assembly_T(n, d, h->minv.p, h->cb.p, h->H.p, h->T.p, s));
  BG_CUDA(g.local.ensure(9 * (size_t)n));
  BG_CUDA(launch_pgs_local(n, d, h->cb.p, h->H.p, h->T.p, g.local.p, s));
  std::vector<double> local(9 * (size_t)n), reg(n, 0.0), sc(n, 1.0);
  BG_CUDA(cudaMemcpyAsync(local.data(), g.local.p, sizeof(double) * local.size(), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i) {
    double* D = &local[9 * (size_t)i];
    sc[i] = dmax(1.0, ((D[0] + D[4]) + D[8]) / 3.0);
    if (auto_reg > 0.) {
      reg[i] = dmax(0.0, auto_reg - min_eigen_symmetric3(D));
      D[0] += reg[i];
      D[4] += reg[i];
      D[8] += reg[i];
    }
  }
  // levels (the order contacts are handed out) and, per slot, the previous contact on the slot's body
  std::vector<int> last(nb, -1), prev(nb, -1), level(n, 0), pdep(2 * (size_t)(n > 0 ? n : 1), -1);
  int nlevels = n > 0 ? 1 : 0;
  for (int i = 0; i < n; ++i) {
    int lv = 0;
    for (int t = 0; t < 2; ++t) {
      const int b = h->h_cb[2 * (size_t)i + t];
      if (b >= 0 && last[b] + 1 > lv) lv = last[b] + 1;
      if (b >= 0) pdep[2 * (size_t)i + t] = prev[b];
    }
    level[i] = lv;
    for (int t = 0; t < 2; ++t) {
      const int b = h->h_cb[2 * (size_t)i + t];
      if (b >= 0 && lv > last[b]) last[b] = lv;
      if (b >= 0) prev[b] = i;
    }
    if (lv + 1 > nlevels) nlevels = lv + 1;
  }
  g.level_off.assign(nlevels + 1, 0);
  for (int i = 0; i < n; ++i) ++g.level_off[level[i] + 1];
  for (int L = 0; L < nlevels; ++L) g.level_off[L + 1] += g.level_off[L];
  std::vector<int> order(n), fill(g.level_off.begin(), g.level_off.end() - 1);
  for (int i = 0; i < n; ++i) order[fill[level[i]]++] = i;
  const int ntiles = (n + kGSTile - 1) / kGSTile;
  BG_CUDA(g.order.ensure(n));
  BG_CUDA(g.reg.ensure(n));
  BG_CUDA(g.scaling.ensure(n));
  BG_CUDA(g.b.ensure(n3));
  BG_CUDA(g.mu.ensure(n));
  BG_CUDA(g.x.ensure(n3));
  BG_CUDA(g.xbest.ensure(n3));
  BG_CUDA(g.y.ensure(n3));
  BG_CUDA(g.nx2.ensure(n));
  BG_CUDA(g.ndx2.ensure(n));
  BG_CUDA(g.skip.ensure(n));
  BG_CUDA(g.processed.ensure(n));
  BG_CUDA(g.tile_max.ensure(2 * (size_t)(ntiles > 0 ? ntiles : 1)));
  BG_CUDA(g.ndx_ref.ensure(2));
  BG_CUDA(g.chunk.ensure((n + 31) / 32 + 1));
  BG_CUDA(g.scalar.ensure(2));
  BG_CUDA(h->pgs_Mx.ensure((size_t)nb * d));
  BG_CUDA(h->mf.ensure((size_t)nb * d));
  BG_CUDA(g.flow.ensure(2));
  BG_CUDA(g.done.ensure(n > 0 ? n : 1));
  BG_CUDA(g.pdep.ensure(pdep.size()));
  BG_CUDA(h->status.ensure(1));
  g.flow_grid = pgs_flow_grid(h->device);
  if (g.flow_grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "occupancy query failed (matrix-free sweep)");
  {
    const unsigned f0[2] = {0u, 1u};
    BG_CUDA(cudaMemcpyAsync(g.flow.p, f0, sizeof(f0), cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemsetAsync(g.done.p, 0, sizeof(unsigned) * (n > 0 ? n : 1), s));
  }
  BG_CUDA(cudaMemcpyAsync(g.pdep.p, pdep.data(), sizeof(int) * pdep.size(), cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(g.order.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(g.local.p, local.data(), sizeof(double) * local.size(), cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(g.reg.p, reg.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(g.scaling.p, sc.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaStreamSynchronize(s));
  g.auto_reg = auto_reg;
  g.use_coloring = 0;
  g.valid = true;
  return BOGUS_GPU_OK;
}

// error at x with y = b + H Mx after recomputing Mx = M^-1 H^T x (ProductGaussSeidel.impl.hpp:249-252, 283-285)
int pgs_eval(bogus_gpu_problem* h, bool desaxce, bool use_inf, double* err) {
  GSCache& g = h->pgs;
  const int n = h->ncontacts;
  cudaStream_t s = h->stream;
  BG_CUDA(launch_pgs_mx(h->nbodies, h->ndof, h->bptr.p, h->bent.p, h->T.p, g.x.p, h->pgs_Mx.p, s));
  BG_CUDA(launch_pgs_y(n, h->ndof, h->cb.p, h->H.p, h->pgs_Mx.p, g.b.p, g.y.p, s));
  BG_CUDA(launch_eval_chunks(n, g.x.p, g.y.p, g.mu.p, g.scaling.p, desaxce, use_inf, g.chunk.p, s));
  BG_CUDA(launch_combine(g.chunk.p, (n + 31) / 32, use_inf, use_inf ? 0.0 : (double)(1 + n), g.scalar.p, s));
  BG_CUDA(cudaMemcpyAsync(err, g.scalar.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  h->last_launches += 4;
  return BOGUS_GPU_OK;
}

}  // namespace

extern "C" {

int bogus_gpu_solve_product_gs(bogus_gpu_problem* h, const bogus_gpu_gs_options* o, const double* f,
                               const double* w, const double* mu, double* r, double* residual, unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (int e = check_gs_options(o)) return e;
  if (o->use_coloring)
    return fail(BOGUS_GPU_BAD_INPUT, "the matrix-free sweep visits the contacts in their own order (no coloring)");
  if (h->nbodies == 0) return fail(BOGUS_GPU_NO_PROBLEM, "no primal problem set (bogus_gpu_set_primal)");
  const int n = h->ncontacts, nb = h->nbodies, d = h->ndof;
  const size_t n3 = 3 * (size_t)n, m = (size_t)nb * d;
  if (n == 0) {
    if (residual) *residual = 0.0;
    if (iters) *iters = 0;
    return BOGUS_GPU_OK;
  }
  if (!w || !mu || !r) return fail(BOGUS_GPU_BAD_INPUT, "null w, mu or r");
  if (int e = check_finite(w, n3, "w")) return e;
  if (int e = check_finite(mu, n, "mu")) return e;
  if (int e = check_finite(r, n3, "r")) return e;
  if (f)
    if (int e = check_finite(f, m, "f")) return e;
  if (int e = set_device(h)) return e;
  if (int e = prepare_pgs(h, o->auto_regularization)) return e;
  GSCache& g = h->pgs;
  cudaStream_t s = h->stream;
  h->last_launches = 0;
  // b = w - H M^-1 f (the dual's right-hand side, PrimalFrictionProblem.cpp:44-45)
  DevBuf<double> dw, df;
  BG_CUDA(dw.ensure(n3));
  BG_CUDA(cudaMemcpyAsync(dw.p, w, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  if (h->frames_valid) BG_CUDA(launch_frame(n, h->frames.p, dw.p, dw.p, true, s));
  if (f) {
    BG_CUDA(df.ensure(m));
    BG_CUDA(cudaMemcpyAsync(df.p, f, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  BG_CUDA(launch_assembly_b(n, nb, d, h->minv.p, f ? df.p : nullptr, h->cb.p, h->H.p, dw.p, h->mf.p, g.b.p, s));
  BG_CUDA(cudaMemcpyAsync(g.mu.p, mu, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(g.x.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  const int ntiles = (n + kGSTile - 1) / kGSTile;
  BG_CUDA(cudaMemsetAsync(g.tile_max.p, 0, sizeof(unsigned long long) * 2 * ntiles, s));
  BG_CUDA(cudaMemsetAsync(g.ndx_ref.p, 0, sizeof(double) * 2, s));
  BG_CUDA(cudaMemsetAsync(g.skip.p, 0, n, s));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  BG_CUDA(cudaEventRecord(h->ev0, s));
  auto sweep_status = [&]() -> int {
    int st = 0;
    BG_CUDA(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    if (st != 0) return fail(st, "device-side wait timed out in the matrix-free sweep");
    return BOGUS_GPU_OK;
  };
  GSArgs a{};
  a.n = n;
  a.local = g.local.p;
  a.reg = g.reg.p;
  a.scaling = g.scaling.p;
  a.b = g.b.p;
  a.mu = g.mu.p;
  a.x = g.x.p;
  a.nx2 = g.nx2.p;
  a.ndx2 = g.ndx2.p;
  a.skip = g.skip.p;
  a.processed = g.processed.p;
  a.tile_max = g.tile_max.p;
  a.ndx_ref = g.ndx_ref.p;
  a.order = g.order.p;
  a.desaxce = o->static_problem ? 0 : 1;
  a.strat = o->local_strategy;
  a.H = h->H.p;
  a.T = h->T.p;
  a.cb = h->cb.p;
  a.Mx = h->pgs_Mx.p;
  a.d = d;
  a.flow = g.flow.p;
  a.done = g.done.p;
  a.status = h->status.p;
  a.pdep = g.pdep.p;
  const bool desaxce = !o->static_problem;
  const bool use_inf = o->use_infinity_norm != 0;
  double err_best = DBL_MAX, err = 0;
  bool has_best = false;
  if (int e = pgs_eval(h, desaxce, use_inf, &err)) return e;
  if (err < err_best) {
    BG_CUDA(cudaMemcpyAsync(g.xbest.p, g.x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    err_best = err;
    has_best = true;
  }
  if (o->try_zero_as_well) {
    BG_CUDA(cudaMemsetAsync(g.y.p, 0, sizeof(double) * n3, s));
    BG_CUDA(launch_eval_chunks(n, g.y.p, g.b.p, g.mu.p, g.scaling.p, desaxce, use_inf, g.chunk.p, s));
    BG_CUDA(launch_combine(g.chunk.p, (n + 31) / 32, use_inf, use_inf ? 0.0 : (double)(1 + n), g.scalar.p, s));
    double err_zero = 0;
    BG_CUDA(cudaMemcpyAsync(&err_zero, g.scalar.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    h->last_launches += 2;
    if (err_zero < err_best) {
      err_best = err_zero;
      BG_CUDA(cudaMemsetAsync(g.xbest.p, 0, sizeof(double) * n3, s));
      BG_CUDA(cudaMemsetAsync(g.x.p, 0, sizeof(double) * n3, s));
      BG_CUDA(cudaMemsetAsync(h->pgs_Mx.p, 0, sizeof(double) * m, s));
      has_best = true;
    } else if (has_best) {
      BG_CUDA(cudaMemcpyAsync(g.x.p, g.xbest.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    }
  }
  std::vector<std::pair<unsigned, double>> trace;
  trace.push_back({0u, err_best});
  const double abs_skip_tol = dmin(o->skip_tol, o->tol);
  const int abs_skip_iters = (int)dmin((double)o->skip_iters, (double)(unsigned)std::sqrt((double)n));
  long long key = 0;
  {
    double st = o->skip_tol, ast = abs_skip_tol;
    unsigned long long b1, b2;
    std::memcpy(&b1, &st, 8);
    std::memcpy(&b2, &ast, 8);
    key = (long long)((b1 * 1000003ull) ^ (b2 * 10007ull) ^ ((unsigned long long)abs_skip_iters << 8) ^
                      ((unsigned long long)a.desaxce << 4) ^ (unsigned long long)a.strat);
    if (key < 0) key = -key - 1;
  }
  unsigned it;
  int parity = 0;
  bool converged = false;
  for (it = 1; it <= o->max_iters; ++it) {
    if (int e = launch_sweep(h, g, a, parity, abs_skip_tol, o->skip_tol, abs_skip_iters, key, true)) return e;
    parity ^= 1;
    if (0 == (it % o->eval_every)) {
      if (int e = pgs_eval(h, desaxce, use_inf, &err)) return e;
      if (int e = sweep_status()) return e;
      if (err < err_best) {
        BG_CUDA(cudaMemcpyAsync(g.xbest.p, g.x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
        err_best = err;
        has_best = true;
      }
      trace.push_back({it, err});
      if (err < o->tol) {
        converged = true;
        break;
      }
      BG_CUDA(launch_scale_scalar(g.ndx_ref.p + parity, (double)o->eval_every, s));
      h->last_launches += 1;
    }
  }
  if (int e = sweep_status()) return e;
  const double* result = (it > o->max_iters && has_best) ? g.xbest.p : g.x.p;
  BG_CUDA(cudaEventRecord(h->ev1, s));
  BG_CUDA(cudaMemcpyAsync(r, result, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  if (residual) *residual = err_best;
  if (iters) *iters = it > o->max_iters ? o->max_iters : it;
  if (h->callback)
    for (auto& t : trace) h->callback(t.first, t.second, h->callback_user);
  return converged ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

// ---- Cadoux fixed point (Interfaces/Cadoux.hpp:44-91, DualFrictionProblem::solveCadoux,
//      FrictionProblem.impl.hpp:76-92) -----------------------------------------------------------------
static int solve_cadoux_gs_stored(bogus_gpu_problem* h, const bogus_gpu_gs_options* o, double* r, unsigned cadoux_iters,
                                  double* residual, unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (int e = check_gs_options(o)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (int e = set_device(h)) return e;
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  if (n == 0) {
    if (residual) *residual = 0.0;
    if (iters) *iters = 0;
    return BOGUS_GPU_OK;
  }
  if (int e = check_finite(r, n3, "r")) return e;
  if (int e = prepare_gs(h, o->auto_regularization, o->use_coloring ? 1 : 0)) return e;
  GSCache& g = h->gs;
  cudaStream_t s = h->stream;
  h->last_launches = 0;
  if (int e = gs_load_x(h, r)) return e;
  BG_CUDA(h->cad_b.ensure(n3));
  BG_CUDA(cudaMemcpyAsync(h->cad_b.p, g.b.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
  BG_CUDA(cudaEventRecord(h->ev0, s));
  bogus_gpu_gs_options oi = *o;
  oi.static_problem = 1;  // inner problems: SOCLaw<3, false>
  const GSArgs a = gs_args(h, &oi);
  const bool use_inf = o->use_infinity_norm != 0;
  std::vector<std::pair<unsigned, double>> trace;
  double res = 0;
  int st = gs_eval(h, a, g.x.p, h->cad_b.p, true, use_inf, &res);  // Coulomb error at (r, W r + b)
  trace.push_back({0u, res});
  const double tol = o->tol;
  unsigned it = 0;
  for (; st == BOGUS_GPU_OK && it < cadoux_iters; ++it) {
    oi.tol = 1.e-1 * dmax(tol, dmin(res, 1.));
    if (launch_cadoux_rhs(n, g.y.p, g.mu.p, h->cad_b.p, g.b.p, s) != cudaSuccess) {
      st = fail(BOGUS_GPU_CUDA_ERROR, "Cadoux right-hand side");
      break;
    }
    h->last_launches += 1;
    st = run_gs_core(h, &oi, nullptr, nullptr, nullptr, nullptr);
    if (st != BOGUS_GPU_OK) break;
    st = gs_eval(h, a, g.x.p, h->cad_b.p, true, use_inf, &res);
    trace.push_back({it + 1, res});
    if (res < tol) {
      ++it;
      break;
    }
  }
  BG_CUDA(cudaMemcpyAsync(g.b.p, h->cad_b.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
  if (st != BOGUS_GPU_OK) return st;
  BG_CUDA(cudaEventRecord(h->ev1, s));
  if (int e = gs_store_x(h, r)) return e;
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  if (residual) *residual = res;
  if (iters) *iters = it;
  if (h->callback)
    for (auto& t : trace) h->callback(t.first, t.second, h->callback_user);
  return res < tol ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

static int solve_cadoux_pg_stored(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* r, unsigned cadoux_iters,
                                  double* residual, unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (int e = check_pg_options(o)) return e;
  if (o->mixed_precision) return fail(BOGUS_GPU_BAD_INPUT, "the Cadoux fixed point runs its inner solves in FP64");
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (int e = set_device(h)) return e;
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  if (n == 0) {
    if (residual) *residual = 0.0;
    if (iters) *iters = 0;
    return BOGUS_GPU_OK;
  }
  if (int e = check_finite(r, n3, "r")) return e;
  if (int e = ensure_pg_work(h, o->max_iters)) return e;
  cudaStream_t s = h->stream;
  const int C = (n + 31) / 32;
  BG_CUDA(h->cad_b.ensure(n3));
  BG_CUDA(h->vx.ensure(n3));
  BG_CUDA(h->vy.ensure(n3));
  BG_CUDA(h->chunk.ensure(C + 1));
  BG_CUDA(h->scalar.ensure(2));
  BG_CUDA(cudaMemcpyAsync(h->cad_b.p, h->b.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
  BG_CUDA(cudaMemcpyAsync(h->vx.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  const bool use_inf = o->use_infinity_norm != 0;
  // Coulomb error at (x, W x + b) with the solver's scalings
  auto coulomb_error = [&](double* err) -> int {
    BG_CUDA(launch_spmv(h->W, h->vx.p, h->cad_b.p, h->vy.p, s));
    BG_CUDA(launch_eval_chunks(n, h->vx.p, h->vy.p, h->mu.p, h->scaling.p, true, use_inf, h->chunk.p, s));
    BG_CUDA(launch_combine(h->chunk.p, C, use_inf, use_inf ? 0.0 : (double)(1 + n), h->scalar.p, s));
    BG_CUDA(cudaMemcpyAsync(err, h->scalar.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    return BOGUS_GPU_OK;
  };
  const bogus_gpu_callback cb = h->callback;
  h->callback = nullptr;  // the inner solves report nothing; the fixed point reports its own iterations
  std::vector<std::pair<unsigned, double>> trace;
  double res = 0;
  float total_ms = 0.f;
  unsigned launches = 3;
  int st = coulomb_error(&res);
  trace.push_back({0u, res});
  bogus_gpu_pg_options oi = *o;
  oi.static_problem = 1;  // inner problems: SOCLaw<3, false>
  const double tol = o->tol;
  unsigned it = 0;
  for (; st == BOGUS_GPU_OK && it < cadoux_iters; ++it) {
    oi.tol = 1.e-1 * dmax(tol, dmin(res, 1.));
    if (launch_cadoux_rhs(n, h->vy.p, h->mu.p, h->cad_b.p, h->b.p, s) != cudaSuccess ||
        cudaMemcpyAsync(h->X.p, h->vx.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      st = fail(BOGUS_GPU_CUDA_ERROR, "Cadoux right-hand side");
      break;
    }
    const double* best = nullptr;
    const int ps = run_pg(h, &oi, nullptr, nullptr, &best);
    if (ps != BOGUS_GPU_OK && ps != BOGUS_GPU_NOT_CONVERGED) {
      st = ps;
      break;
    }
    total_ms += h->last_ms;
    launches += h->last_launches + 4;
    if (cudaMemcpyAsync(h->vx.p, best, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      st = fail(BOGUS_GPU_CUDA_ERROR, "Cadoux iterate copy");
      break;
    }
    st = coulomb_error(&res);
    trace.push_back({it + 1, res});
    if (res < tol) {
      ++it;
      break;
    }
  }
  h->callback = cb;
  BG_CUDA(cudaMemcpyAsync(h->b.p, h->cad_b.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
  if (st != BOGUS_GPU_OK) return st;
  BG_CUDA(cudaMemcpyAsync(r, h->vx.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  h->last_ms = total_ms;
  h->last_launches = launches;
  if (residual) *residual = res;
  if (iters) *iters = it;
  if (h->callback)
    for (auto& t : trace) h->callback(t.first, t.second, h->callback_user);
  return res < tol ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

// ---- MecheFrictionProblem facade (Interfaces/MecheInterface.hpp:40-170, MecheInterface.cpp:97-367) ----------
void bogus_gpu_meche_options_default(bogus_gpu_meche_options* o) {
  if (!o) return;
  o->max_threads = 0;
  o->max_iters = 0;
  o->cadoux_iters = 0;
  o->tolerance = 0.0;
  o->use_infinity_norm = 0;
  o->algorithm = BOGUS_GPU_MECHE_GAUSS_SEIDEL;
  o->gs_regularization = 0.0;
  o->gs_coloring = 0;
  o->gs_skip_iters = -1;
  o->try_zero_as_well = 1;
  o->pg_variant = BOGUS_GPU_PG_SPG;
  o->admm_proj_step_size = 1.0;
  o->admm_fp_step_size = 1.e-3;
}

int bogus_gpu_meche_from_primal(bogus_gpu_problem* h, unsigned nobj, const unsigned* ndof,
                                const double* const* mass, const double* f, unsigned n, const double* mu,
                                const double* E, const double* w, const int* objA, const int* objB,
                                const double* const* HA, const double* const* HB) {
  if (int e = check_handle(h)) return e;
  if (nobj == 0 || !ndof || !mass) return fail(BOGUS_GPU_BAD_INPUT, "no objects");
  if (n > 0 && (!mu || !E || !w || !objA || !objB || !HA || !HB)) return fail(BOGUS_GPU_BAD_INPUT, "null contact array");
  unsigned d = 1;
  size_t m = 0;
  for (unsigned k = 0; k < nobj; ++k) {
    if (ndof[k] == 0 || ndof[k] > 12 || !mass[k]) return fail(BOGUS_GPU_BAD_INPUT, "object dofs must be in 1..12");
    d = std::max(d, ndof[k]);
    m += ndof[k];
  }
  for (unsigned i = 0; i < n; ++i) {
    if (objA[i] < 0 || objA[i] >= (int)nobj || objB[i] < -1 || objB[i] >= (int)nobj)
      return fail(BOGUS_GPU_BAD_INPUT, "object index out of range");
    if (!HA[i] || (objB[i] >= 0 && !HB[i])) return fail(BOGUS_GPU_BAD_INPUT, "null Jacobian block");
  }
  if (int e = check_finite(E, 9 * (size_t)n, "E")) return e;
  if (int e = check_finite(w, 3 * (size_t)n, "w")) return e;
  if (int e = check_finite(mu, n, "mu")) return e;
  if (f)
    if (int e = check_finite(f, m, "f")) return e;
  // inverse mass blocks (PrimalFrictionProblem::computeMInv), padded to d dofs with inert (zero) entries
  std::vector<double> minv((size_t)nobj * d * d, 0.0), mpad((size_t)nobj * d * d, 0.0), fpad((size_t)nobj * d, 0.0);
  {
    size_t off = 0;
    for (unsigned k = 0; k < nobj; ++k) {
      const int dk = (int)ndof[k];
      if (int e = check_finite(mass[k], (size_t)dk * dk, "mass")) return e;
      std::vector<double> Mk((size_t)dk * dk), inv((size_t)dk * dk);
      for (int a = 0; a < dk; ++a)
        for (int c = 0; c < dk; ++c) Mk[(size_t)a * dk + c] = mass[k][(size_t)c * dk + a];
      if (!invert_gauss_jordan(dk, Mk.data(), inv.data())) return fail(BOGUS_GPU_BAD_INPUT, "singular mass block");
      for (int a = 0; a < dk; ++a) {
        for (int c = 0; c < dk; ++c) {
          minv[(size_t)k * d * d + a * d + c] = inv[(size_t)a * dk + c];
          mpad[(size_t)k * d * d + a * d + c] = Mk[(size_t)a * dk + c];
        }
        if (f) fpad[(size_t)k * d + a] = f[off + a];
      }
      off += ndof[k];
    }
  }
  // frames (row-major per contact) and padded row-major world Jacobian blocks
  const size_t hs = 3 * (size_t)d;
  std::vector<double> Er(9 * (size_t)n), HAw(n * hs, 0.0), HBw(n * hs, 0.0);
  std::vector<int> cbh(2 * (size_t)n), oA(objA, objA + n), oB(objB, objB + n);
  for (unsigned i = 0; i < n; ++i) {
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) Er[9 * (size_t)i + 3 * a + c] = E[(size_t)c * 3 * n + 3 * i + a];
    const int A = objA[i], B = objB[i];
    for (unsigned c = 0; c < ndof[A]; ++c)
      for (int k = 0; k < 3; ++k) HAw[i * hs + k * d + c] = HA[i][(size_t)c * 3 + k];
    if (B >= 0) {
      const unsigned dB = ndof[B == A ? A : B];
      for (unsigned c = 0; c < dB; ++c)
        for (int k = 0; k < 3; ++k) HBw[i * hs + k * d + c] = HB[i][(size_t)c * 3 + k];
    }
    const bool two = B >= 0 && B != A;
    cbh[2 * (size_t)i] = two ? std::min(A, B) : A;
    cbh[2 * (size_t)i + 1] = two ? std::max(A, B) : -1;
  }
  if (int e = check_finite(HAw.data(), HAw.size(), "HA")) return e;
  if (int e = check_finite(HBw.data(), HBw.size(), "HB")) return e;
  if (int e = set_device(h)) return e;
  cudaStream_t s = h->stream;
  DevBuf<double> dHA, dHB;
  DevBuf<int> dA, dB;
  const size_t nn = n > 0 ? n : 1;
  BG_CUDA(h->meche_E.ensure(9 * nn));
  BG_CUDA(h->minv.ensure((size_t)nobj * d * d));
  BG_CUDA(h->H.ensure(2 * nn * hs));
  BG_CUDA(h->cb.ensure(2 * nn));
  BG_CUDA(dHA.ensure(nn * hs));
  BG_CUDA(dHB.ensure(nn * hs));
  BG_CUDA(dA.ensure(nn));
  BG_CUDA(dB.ensure(nn));
  BG_CUDA(h->meche_w.ensure(3 * nn));
  BG_CUDA(cudaMemcpyAsync(h->minv.p, minv.data(), sizeof(double) * minv.size(), cudaMemcpyHostToDevice, s));
  if (n > 0) {
    BG_CUDA(cudaMemcpyAsync(h->meche_E.p, Er.data(), sizeof(double) * Er.size(), cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(dHA.p, HAw.data(), sizeof(double) * HAw.size(), cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(dHB.p, HBw.data(), sizeof(double) * HBw.size(), cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(dA.p, objA, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(dB.p, objB, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->cb.p, cbh.data(), sizeof(int) * cbh.size(), cudaMemcpyHostToDevice, s));
    BG_CUDA(launch_meche_h((int)n, (int)d, h->meche_E.p, dHA.p, dHB.p, dA.p, dB.p, h->H.p, s));
    // w to the local basis once: E^T w
    BG_CUDA(cudaMemcpyAsync(h->meche_w.p, w, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(launch_frame((int)n, h->meche_E.p, h->meche_w.p, h->meche_w.p, true, s));
  }
  h->meche_wloc.assign(3 * (size_t)n, 0.0);
  if (n > 0)
    BG_CUDA(cudaMemcpyAsync(h->meche_wloc.data(), h->meche_w.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  h->nbodies = (int)nobj;
  h->ndof = (int)d;
  h->ncontacts = (int)n;
  h->h_cb = std::move(cbh);
  h->pgs.valid = false;
  h->h_objA = std::move(oA);
  h->admm_incidence_valid = false;
  h->meche_ndof.assign(ndof, ndof + nobj);
  h->body_dofs.assign(ndof, ndof + nobj);
  h->meche_f = std::move(fpad);
  h->meche_mass = std::move(mpad);
  h->meche_mu.assign(mu, mu + n);
  h->meche_valid = true;
  h->permuted = false;
  h->frames_valid = false;
  h->meche_dual = false;
  return BOGUS_GPU_OK;
}

int bogus_gpu_meche_solve(bogus_gpu_problem* h, double* r, double* v, const bogus_gpu_meche_options* o,
                          int static_problem, double problem_regularization, double* residual) {
  if (int e = check_handle(h)) return e;
  if (!o) return fail(BOGUS_GPU_BAD_INPUT, "null options");
  if (!h->meche_valid) return fail(BOGUS_GPU_NO_PROBLEM, "no problem set (bogus_gpu_meche_from_primal)");
  if (o->algorithm != BOGUS_GPU_MECHE_GAUSS_SEIDEL && o->algorithm != BOGUS_GPU_MECHE_PROJECTED_GRADIENT &&
      o->algorithm != BOGUS_GPU_MECHE_ADMM && o->algorithm != BOGUS_GPU_MECHE_MATRIX_FREE_GAUSS_SEIDEL &&
      o->algorithm != BOGUS_GPU_MECHE_DUAL_AMA)
    return fail(BOGUS_GPU_BAD_INPUT, "unknown algorithm");
  const int n = h->ncontacts, nb = h->nbodies, d = h->ndof;
  const size_t n3 = 3 * (size_t)n, md = (size_t)nb * d;
  if (n > 0 && !r) return fail(BOGUS_GPU_BAD_INPUT, "null r");
  if (int e = check_finite(r, n3, "r")) return e;
  if (int e = set_device(h)) return e;
  cudaStream_t s = h->stream;
  BG_CUDA(h->meche_r.ensure(n3 > 0 ? n3 : 1));
  BG_CUDA(h->meche_v.ensure(md));
  BG_CUDA(h->meche_fd.ensure(md));
  BG_CUDA(cudaMemcpyAsync(h->meche_fd.p, h->meche_f.data(), sizeof(double) * md, cudaMemcpyHostToDevice, s));
  std::vector<double> rl(n3), vp(md, 0.0);
  // r to local coordinates: E^T r
  if (n > 0) {
    BG_CUDA(cudaMemcpyAsync(h->meche_r.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
    BG_CUDA(launch_frame(n, h->meche_E.p, h->meche_r.p, h->meche_r.p, true, s));
    BG_CUDA(cudaMemcpyAsync(rl.data(), h->meche_r.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
  }
  BG_CUDA(cudaStreamSynchronize(s));
  auto velocity = [&]() -> int {  // v = M^-1 (H^T r_loc - f) into vp
    if (int e = ensure_incidence(h)) return e;
    BG_CUDA(launch_body_transpose(nb, d, h->bptr.p, h->bent.p, h->H.p, h->minv.p, h->meche_r.p, h->meche_fd.p,
                                  h->meche_v.p, s));
    BG_CUDA(cudaMemcpyAsync(vp.data(), h->meche_v.p, sizeof(double) * md, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    return BOGUS_GPU_OK;
  };
  auto pad_v = [&]() {
    size_t off = 0;
    for (int k = 0; k < nb; ++k) {
      for (unsigned a = 0; a < h->meche_ndof[k]; ++a) vp[(size_t)k * d + a] = v[off + a];
      off += h->meche_ndof[k];
    }
  };
  int st = BOGUS_GPU_OK;
  double res = -1.0;
  if (o->algorithm == BOGUS_GPU_MECHE_DUAL_AMA) {
    // MecheInterface.cpp:237-261: v given or M^-1 (H^T r - f); no line search, the facade's step sizes
    if (v) pad_v();
    else if (int e = velocity()) return e;
    bogus_gpu_dual_ama_options da;
    bogus_gpu_dual_ama_options_default(&da);
    if (o->tolerance != 0.) da.tol = o->tolerance;
    if (o->max_iters != 0) da.max_iters = o->max_iters;
    da.use_infinity_norm = o->use_infinity_norm;
    da.ls_iters = 0;
    da.fp_step_size = o->admm_fp_step_size;
    da.proj_step_size = o->admm_proj_step_size;
    st = bogus_gpu_solve_dual_ama(h, &da, h->meche_mass.data(), h->meche_f.data(), h->meche_wloc.data(),
                                  h->meche_mu.data(), static_problem, vp.data(), rl.data(), &res, nullptr);
    if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
    if (n > 0) BG_CUDA(cudaMemcpyAsync(h->meche_r.p, rl.data(), sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  } else if (o->algorithm == BOGUS_GPU_MECHE_ADMM) {
    if (v) pad_v();
    else if (int e = velocity()) return e;
    bogus_gpu_admm_options ao;
    bogus_gpu_admm_options_default(&ao);
    ao.step_size = o->admm_proj_step_size;
    if (o->tolerance != 0.) ao.tol = o->tolerance;
    if (o->max_iters != 0) ao.max_iters = o->max_iters;
    ao.use_infinity_norm = o->use_infinity_norm;
    st = bogus_gpu_solve_admm(h, &ao, 0.0, nullptr, h->meche_f.data(), h->meche_wloc.data(), h->meche_mu.data(),
                              vp.data(), rl.data(), &res, nullptr);
    if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
    if (n > 0) BG_CUDA(cudaMemcpyAsync(h->meche_r.p, rl.data(), sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  } else if (o->algorithm == BOGUS_GPU_MECHE_MATRIX_FREE_GAUSS_SEIDEL) {
    // PrimalFrictionProblem::solveWith(ProductGaussSeidelType&, r_loc, staticProblem) (MecheInterface.cpp:290-302)
    bogus_gpu_gs_options go;
    bogus_gpu_gs_options_default(&go);
    if (o->tolerance != 0.) go.tol = o->tolerance;
    if (o->max_iters != 0) go.max_iters = o->max_iters;
    if (o->gs_skip_iters >= 0) go.skip_iters = (unsigned)o->gs_skip_iters;
    go.use_infinity_norm = o->use_infinity_norm;
    go.auto_regularization = o->gs_regularization;
    go.try_zero_as_well = o->try_zero_as_well;
    go.static_problem = static_problem ? 1 : 0;
    st = bogus_gpu_solve_product_gs(h, &go, h->meche_f.data(), h->meche_wloc.data(), h->meche_mu.data(), rl.data(),
                                    &res, nullptr);
    if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
    if (n > 0) {
      BG_CUDA(cudaMemcpyAsync(h->meche_r.p, rl.data(), sizeof(double) * n3, cudaMemcpyHostToDevice, s));
      BG_CUDA(cudaStreamSynchronize(s));
    }
    if (v)
      if (int e = velocity()) return e;
  } else {
    if (!h->meche_dual) {
      if (int e = bogus_gpu_assemble_dual(h, h->meche_f.data(), h->meche_wloc.data(), h->meche_mu.data())) return e;
      if (problem_regularization > 0. && n > 0) {
        std::vector<double> c(n, problem_regularization);
        if (int e = bogus_gpu_add_compliance(h, c.data())) return e;
      }
      h->meche_dual = true;
    }
    const bool cadoux = !static_problem && o->cadoux_iters > 0;
    if (o->algorithm == BOGUS_GPU_MECHE_PROJECTED_GRADIENT) {
      bogus_gpu_pg_options po;
      bogus_gpu_pg_options_default(&po);
      if (o->tolerance != 0.) po.tol = o->tolerance;
      if (o->max_iters != 0) po.max_iters = o->max_iters;
      po.use_infinity_norm = o->use_infinity_norm;
      po.variant = o->pg_variant;
      po.static_problem = static_problem ? 1 : 0;
      st = cadoux ? solve_cadoux_pg_stored(h, &po, rl.data(), o->cadoux_iters, &res, nullptr)
                  : solve_pg_stored(h, &po, rl.data(), &res, nullptr);
    } else {
      bogus_gpu_gs_options go;
      bogus_gpu_gs_options_default(&go);
      if (o->tolerance != 0.) go.tol = o->tolerance;
      if (o->max_iters != 0) go.max_iters = o->max_iters;
      if (o->gs_skip_iters >= 0) go.skip_iters = (unsigned)o->gs_skip_iters;
      go.auto_regularization = o->gs_regularization;
      go.use_infinity_norm = o->use_infinity_norm;
      go.use_coloring = (o->max_threads != 1 && o->gs_coloring) ? 1 : 0;
      go.static_problem = static_problem ? 1 : 0;
      go.try_zero_as_well = cadoux ? 0 : o->try_zero_as_well;
      st = cadoux ? solve_cadoux_gs_stored(h, &go, rl.data(), o->cadoux_iters, &res, nullptr)
                  : solve_gs_stored(h, &go, rl.data(), &res, nullptr);
    }
    if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
    if (n > 0) {
      BG_CUDA(cudaMemcpyAsync(h->meche_r.p, rl.data(), sizeof(double) * n3, cudaMemcpyHostToDevice, s));
      BG_CUDA(cudaStreamSynchronize(s));
    }
    if (v)
      if (int e = velocity()) return e;
  }
  if (v) {
    size_t off = 0;
    for (int k = 0; k < nb; ++k) {
      for (unsigned a = 0; a < h->meche_ndof[k]; ++a) v[off + a] = vp[(size_t)k * d + a];
      off += h->meche_ndof[k];
    }
  }
  // r back to world coordinates: E r_loc
  if (n > 0) {
    BG_CUDA(launch_frame(n, h->meche_E.p, h->meche_r.p, h->meche_r.p, false, s));
    BG_CUDA(cudaMemcpyAsync(r, h->meche_r.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
  }
  if (residual) *residual = res;
  return st;
}

// ---- primal data and Delassus assembly ---------------------------------------------------------------
int bogus_gpu_set_primal(bogus_gpu_problem* h, int nbodies, int ndof, const double* minv, int ncontacts, const int* objA,
                         const int* objB, const double* HA, const double* HB) {
  if (int e = check_handle(h)) return e;
  if (nbodies <= 0 || ndof <= 0 || ndof > 12 || ncontacts < 0) return fail(BOGUS_GPU_BAD_INPUT, "invalid primal sizes");
  if (!minv || (ncontacts > 0 && (!objA || !objB || !HA || !HB))) return fail(BOGUS_GPU_BAD_INPUT, "null primal array");
  if (int e = check_finite(minv, (size_t)nbodies * ndof * ndof, "minv")) return e;
  if (int e = check_finite(HA, (size_t)ncontacts * 3 * ndof, "HA")) return e;
  if (int e = check_finite(HB, (size_t)ncontacts * 3 * ndof, "HB")) return e;
  std::vector<int> cbh(2 * (size_t)ncontacts);
  std::vector<double> Hh(2 * (size_t)ncontacts * 3 * ndof, 0.0);
  const size_t hs = 3 * (size_t)ndof;
  for (int i = 0; i < ncontacts; ++i) {
    const int a = objA[i], b = objB[i];
    if (a < 0 || a >= nbodies || b < -1 || b >= nbodies) return fail(BOGUS_GPU_BAD_INPUT, "body index out of range");
    // slots ordered by body index; a repeated body counts once (slot A)
    int s0 = a, s1 = -1;
    const double* h0 = HA + i * hs;
    const double* h1 = nullptr;
    if (b >= 0 && b != a) {
      if (b < a) {
        s0 = b; s1 = a; h0 = HB + i * hs; h1 = HA + i * hs;
      } else {
        s1 = b; h1 = HB + i * hs;
      }
    }
    cbh[2 * (size_t)i] = s0;
    cbh[2 * (size_t)i + 1] = s1;
    std::copy(h0, h0 + hs, &Hh[(2 * (size_t)i) * hs]);
    if (h1) std::copy(h1, h1 + hs, &Hh[(2 * (size_t)i + 1) * hs]);
  }
  if (int e = set_device(h)) return e;
  BG_CUDA(h->minv.ensure((size_t)nbodies * ndof * ndof));
  BG_CUDA(h->H.ensure(Hh.size()));
  BG_CUDA(h->cb.ensure(cbh.size()));
  BG_CUDA(cudaMemcpyAsync(h->minv.p, minv, sizeof(double) * nbodies * ndof * ndof, cudaMemcpyHostToDevice, h->stream));
  if (ncontacts) {
    BG_CUDA(cudaMemcpyAsync(h->H.p, Hh.data(), sizeof(double) * Hh.size(), cudaMemcpyHostToDevice, h->stream));
    BG_CUDA(cudaMemcpyAsync(h->cb.p, cbh.data(), sizeof(int) * cbh.size(), cudaMemcpyHostToDevice, h->stream));
  }
  BG_CUDA(cudaStreamSynchronize(h->stream));
  h->nbodies = nbodies;
  h->ndof = ndof;
  h->ncontacts = ncontacts;
  h->h_cb = std::move(cbh);
  h->pgs.valid = false;
  h->h_objA.assign(objA, objA + ncontacts);
  h->admm_incidence_valid = false;
  h->body_dofs.assign(nbodies, ndof);
  h->frames_valid = false;
  h->meche_valid = false;
  h->meche_dual = false;
  return BOGUS_GPU_OK;
}

int bogus_gpu_set_body_dofs(bogus_gpu_problem* h, const int* ndof) {
  if (int e = check_handle(h)) return e;
  if (h->nbodies == 0) return fail(BOGUS_GPU_NO_PROBLEM, "no primal problem set (bogus_gpu_set_primal)");
  if (!ndof) return fail(BOGUS_GPU_BAD_INPUT, "null ndof");
  for (int k = 0; k < h->nbodies; ++k)
    if (ndof[k] < 1 || ndof[k] > h->ndof) return fail(BOGUS_GPU_BAD_INPUT, "body dof count out of range");
  h->body_dofs.assign(ndof, ndof + h->nbodies);
  h->admm_incidence_valid = false;
  return BOGUS_GPU_OK;
}

int bogus_gpu_set_frames(bogus_gpu_problem* h, const double* E) {
  if (int e = check_handle(h)) return e;
  if (h->nbodies == 0) return fail(BOGUS_GPU_NO_PROBLEM, "no primal problem set (bogus_gpu_set_primal)");
  const int n = h->ncontacts;
  if (!E) {
    h->frames_valid = false;
    return BOGUS_GPU_OK;
  }
  if (int e = check_finite(E, 9 * (size_t)n, "E")) return e;
  if (int e = set_device(h)) return e;
  BG_CUDA(h->frames.ensure(9 * (size_t)(n > 0 ? n : 1)));
  if (n) BG_CUDA(cudaMemcpyAsync(h->frames.p, E, sizeof(double) * 9 * n, cudaMemcpyHostToDevice, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  h->frames_valid = true;
  return BOGUS_GPU_OK;
}

}  // extern "C"

namespace {

// Body -> (contact, slot) incidences in increasing contact order (ADMM's H^T products, the adjoint's
// primal gradients), built once per primal problem.
int ensure_incidence(bogus_gpu_problem* h) {
  if (h->admm_incidence_valid) return BOGUS_GPU_OK;
  const int n = h->ncontacts, nb = h->nbodies;
  cudaStream_t s = h->stream;
  std::vector<int> bp(nb + 1, 0), be;
  for (int i = 0; i < n; ++i)
    for (int t = 0; t < 2; ++t)
      if (h->h_cb[2 * (size_t)i + t] >= 0) ++bp[h->h_cb[2 * (size_t)i + t] + 1];
  for (int k = 0; k < nb; ++k) bp[k + 1] += bp[k];
  be.resize(bp[nb] > 0 ? bp[nb] : 1);
  std::vector<int> fill(bp.begin(), bp.end() - 1);
  for (int i = 0; i < n; ++i)  // increasing contact index within each body
    for (int t = 0; t < 2; ++t) {
      const int k = h->h_cb[2 * (size_t)i + t];
      if (k >= 0) be[fill[k]++] = 2 * i + t;
    }
  BG_CUDA(h->bptr.ensure(nb + 1));
  BG_CUDA(h->bent.ensure(be.size()));
  BG_CUDA(cudaMemcpyAsync(h->bptr.p, bp.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(h->bent.p, be.data(), sizeof(int) * be.size(), cudaMemcpyHostToDevice, s));
  // bodies by decreasing contact count, stable: a warp's 32 bodies then loop over about as many contacts
  // each, so the lanes of the H^T r loop stay busy (a body's own arithmetic does not depend on the order)
  {
    int maxdeg = 0;
    for (int k = 0; k < nb; ++k) maxdeg = std::max(maxdeg, bp[k + 1] - bp[k]);
    std::vector<int> cnt(maxdeg + 2, 0), ord(nb > 0 ? nb : 1);
    for (int k = 0; k < nb; ++k) ++cnt[maxdeg - (bp[k + 1] - bp[k]) + 1];
    for (int q = 0; q <= maxdeg; ++q) cnt[q + 1] += cnt[q];
    for (int k = 0; k < nb; ++k) ord[cnt[maxdeg - (bp[k + 1] - bp[k])]++] = k;
    BG_CUDA(h->border.ensure(ord.size()));
    BG_CUDA(cudaMemcpyAsync(h->border.p, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice, s));
  }
  // scalings (ConstrainedSolverBase.impl.hpp:84-118): 1, unless H is square at the block level (3 n rows ==
  // the bodies' dofs, n == nbodies), where contact i with a block on body i takes max(1, trace / 3) of it
  const int d = h->ndof;
  const bool own = h->body_dofs.size() == (size_t)nb;
  long long m = 0;
  for (int k = 0; k < nb; ++k) m += own ? h->body_dofs[k] : d;
  std::vector<double> sc(n > 0 ? n : 1, 1.0);
  if (n > 0 && 3LL * n == m && n == nb) {
    std::vector<double> Hh(2 * (size_t)n * 3 * d);
    BG_CUDA(cudaMemcpyAsync(Hh.data(), h->H.p, sizeof(double) * Hh.size(), cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i)
      for (int t = 0; t < 2; ++t)
        if (h->h_cb[2 * (size_t)i + t] == i) {
          const int dk = own ? h->body_dofs[i] : d;
          const int kk = dk < 3 ? dk : 3;
          const double* Hb = &Hh[(2 * (size_t)i + t) * 3 * d];
          double tr = 0.0;
          for (int k = 0; k < kk; ++k) tr = tr + Hb[k * d + k];
          sc[i] = std::max(1.0, tr / 3.0);
        }
  }
  BG_CUDA(h->a_sc.ensure(sc.size()));
  BG_CUDA(cudaMemcpyAsync(h->a_sc.p, sc.data(), sizeof(double) * sc.size(), cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaStreamSynchronize(s));
  h->true_dofs = m;
  h->admm_ninc = (size_t)bp[nb];
  h->admm_incidence_valid = true;
  return BOGUS_GPU_OK;
}

// Runs the adjoint kernel with r and g already in adj_r / adj_g; leaves s and dL/dmu in adj_S / adj_dmu.
int run_adjoint(bogus_gpu_problem* h, const bogus_gpu_adjoint_options* o, double* residual, unsigned* iters) {
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n > 0 ? 3 * (size_t)n : 1;
  cudaStream_t s = h->stream;
  BG_CUDA(h->adj_V.ensure(3 * n3));
  BG_CUDA(h->adj_Pc.ensure(3 * n3));
  for (auto* b : {&h->adj_D, &h->adj_K, &h->adj_P, &h->adj_R, &h->adj_Z, &h->adj_Dir, &h->adj_Y, &h->adj_Q,
                  &h->adj_S})
    BG_CUDA(b->ensure(n3));
  if (o->coulomb)
    for (auto* b : {&h->adj_Tc, &h->adj_Rh, &h->adj_Ph, &h->adj_Sv, &h->adj_Sh, &h->adj_Tv}) BG_CUDA(b->ensure(n3));
  BG_CUDA(h->adj_dmu.ensure(n > 0 ? n : 1));
  BG_CUDA(h->adj_out.ensure(1));
  const int C = (n + 31) / 32;
  BG_CUDA(h->csum.ensure(4 * (size_t)(C > 0 ? C : 1)));
  BG_CUDA(h->scal.ensure(8 + 32));  // scalars, then the stripe sums of grid_barrier_combine
  BG_CUDA(h->barrier.ensure(8));
  BG_CUDA(h->status.ensure(1));
  if (int e = ensure_interleaved(h)) return e;
  AdjArgs a{};
  a.n = n;
  a.nchunks = C;
  a.rowptr = h->W.rowptr;
  a.icol = h->icol.p;
  a.ival = h->ival.p;
  a.slot0 = h->slot0.p;
  a.val = h->W.val;
  a.b = h->b.p;
  a.mu = h->mu.p;
  a.scaling = h->scaling.p;
  a.r = h->adj_r.p;
  a.g = h->adj_g.p;
  a.diag = h->W.diag;
  a.V = h->adj_V.p;
  a.Pc = h->adj_Pc.p;
  a.Z = h->adj_Z.p;
  a.D = h->adj_D.p;
  a.K = h->adj_K.p;
  a.P = h->adj_P.p;
  a.R = h->adj_R.p;
  a.Dir = h->adj_Dir.p;
  a.Y = h->adj_Y.p;
  a.Q = h->adj_Q.p;
  a.S = h->adj_S.p;
  a.dmu = h->adj_dmu.p;
  a.csum = h->csum.p;
  a.scal = h->scal.p;
  a.out = h->adj_out.p;
  a.gb = GridBarrier{h->barrier.p, h->barrier.p + 1, h->status.p};
  a.tickets = h->barrier.p + 2;
  a.combine_count = h->barrier.p + 4;
  a.stripes = h->scal.p + 8;
  a.tol = o->tol;
  a.max_iters = o->max_iters;
  if (o->coulomb) {
    a.Tc = h->adj_Tc.p;
    a.Rh = h->adj_Rh.p;
    a.Ph = h->adj_Ph.p;
    a.Sv = h->adj_Sv.p;
    a.Sh = h->adj_Sh.p;
    a.Tv = h->adj_Tv.p;
  }
  BG_CUDA(cudaMemsetAsync(h->barrier.p, 0, 8 * sizeof(unsigned), s));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  int grid = adjoint_max_grid(h->device);
  if (grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "cooperative occupancy query failed");
  const int want = (C + 7) / 8;
  if (want < grid) grid = want < 1 ? 1 : want;
  BG_CUDA(cudaEventRecord(h->ev0, s));
  BG_CUDA(o->coulomb ? launch_adjoint_coulomb(a, grid, s) : launch_adjoint(a, grid, s));
  BG_CUDA(cudaEventRecord(h->ev1, s));
  AdjOut out{};
  int st = 0;
  BG_CUDA(cudaMemcpyAsync(&out, h->adj_out.p, sizeof(AdjOut), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->last_launches = 1;
  if (st != 0) return fail(st, "device-side wait timed out in the adjoint kernel");
  // per CG iteration: one W pass, the basis (9 values), D, dir, Q, P, R, Y streams
  const double wpass = (double)h->W.nnzb * 76.0 + 4.0 * (n + 1);
  h->last_stats.iterations = out.iters;
  h->last_stats.refine_iterations = 0;
  h->last_stats.fp32_device_ms = 0.0;
  if (o->coulomb) {
    // per BiCGSTAB iteration: two W passes; per contact the basis (9) x 4, D and tau (6) x 4, the preconditioner
    // (9) x 2 and 27 streams of 3 values over the five phases (6, 4, 5, 4 and 8, the products' gathers counted once)
    h->last_stats.w_passes = 2 * out.iters + 2;
    h->last_stats.algorithmic_bytes =
        (2.0 * out.iters + 2) * wpass + (double)out.iters * n * 8.0 * (36 + 24 + 18 + 3 * 27);
    h->last_stats.fp64_fma = (2.0 * out.iters + 2) * 9.0 * (double)h->W.nnzb;
  } else {
    h->last_stats.w_passes = out.iters + 2;
    // per iteration per contact: basis 9 x 2, preconditioner 9, D 3 x 2, and 14 streams of 3 values as the phases
    // read and write them: dir 4, Q 2, P 2, R 2, Z 2, Y 2 (its gather in the product counted once)
    h->last_stats.algorithmic_bytes = (out.iters + 2) * wpass + (double)out.iters * n * 8.0 * (18 + 9 + 6 + 3 * 14);
    h->last_stats.fp64_fma = (out.iters + 2) * 9.0 * (double)h->W.nnzb;
  }
  h->adj_valid = true;
  if (residual) *residual = out.rel_res;
  if (iters) *iters = out.iters;
  const bool ok = n == 0 || out.rel_res <= o->tol;
  return ok ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

int adjoint_checks(bogus_gpu_problem* h, const bogus_gpu_adjoint_options* o) {
  if (int e = check_handle(h)) return e;
  if (!o) return fail(BOGUS_GPU_BAD_INPUT, "null options");
  if (!(o->tol >= 0)) return fail(BOGUS_GPU_BAD_INPUT, "invalid tolerance");
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (h->permuted) return fail(BOGUS_GPU_BAD_INPUT, "the adjoint needs the contacts in their own order (undo the permutation)");
  return set_device(h);
}

}  // namespace

extern "C" {

void bogus_gpu_adjoint_options_default(bogus_gpu_adjoint_options* o) {
  if (!o) return;
  o->tol = 1e-10;
  o->max_iters = 5000;
  o->coulomb = 0;
}

int bogus_gpu_adjoint(bogus_gpu_problem* h, const bogus_gpu_adjoint_options* o, const double* r,
                      const double* dL_dr, double* dL_db, double* dL_dmu, double* residual, unsigned* iters) {
  if (int e = adjoint_checks(h, o)) return e;
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  if (n > 0 && (!r || !dL_dr)) return fail(BOGUS_GPU_BAD_INPUT, "null r or dL_dr");
  if (int e = check_finite(r, n3, "r")) return e;
  if (int e = check_finite(dL_dr, n3, "dL_dr")) return e;
  BG_CUDA(h->adj_r.ensure(n3 > 0 ? n3 : 1));
  BG_CUDA(h->adj_g.ensure(n3 > 0 ? n3 : 1));
  if (n > 0) {
    BG_CUDA(cudaMemcpyAsync(h->adj_r.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream));
    BG_CUDA(cudaMemcpyAsync(h->adj_g.p, dL_dr, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream));
  }
  const int st = run_adjoint(h, o, residual, iters);
  if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
  h->h_adj_s.resize(n3);
  h->h_adj_r.assign(r, r + n3);
  if (n > 0) {
    BG_CUDA(cudaMemcpy(h->h_adj_s.data(), h->adj_S.p, sizeof(double) * n3, cudaMemcpyDeviceToHost));
    if (dL_dmu) BG_CUDA(cudaMemcpy(dL_dmu, h->adj_dmu.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (dL_db) std::memcpy(dL_db, h->h_adj_s.data(), sizeof(double) * n3);
  }
  return st;
}

int bogus_gpu_adjoint_device(bogus_gpu_problem* h, const bogus_gpu_adjoint_options* o, const double* d_r,
                             const double* d_g, double* d_dL_db, double* d_dL_dmu, double* residual,
                             unsigned* iters) {
  if (int e = adjoint_checks(h, o)) return e;
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  if (n > 0 && (!d_r || !d_g)) return fail(BOGUS_GPU_BAD_INPUT, "null r or dL_dr");
  BG_CUDA(h->adj_r.ensure(n3 > 0 ? n3 : 1));
  BG_CUDA(h->adj_g.ensure(n3 > 0 ? n3 : 1));
  if (n > 0) {
    BG_CUDA(cudaMemcpyAsync(h->adj_r.p, d_r, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    BG_CUDA(cudaMemcpyAsync(h->adj_g.p, d_g, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
  }
  const int st = run_adjoint(h, o, residual, iters);
  if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
  h->h_adj_s.clear();
  h->h_adj_r.clear();
  if (n > 0) {
    if (d_dL_db)
      BG_CUDA(cudaMemcpyAsync(d_dL_db, h->adj_S.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
    if (d_dL_dmu)
      BG_CUDA(cudaMemcpyAsync(d_dL_dmu, h->adj_dmu.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    BG_CUDA(cudaStreamSynchronize(h->stream));
  }
  return st;
}

int bogus_gpu_adjoint_dual_lower(bogus_gpu_problem* h, double* dW) {
  if (int e = check_handle(h)) return e;
  if (!h->adj_valid) return fail(BOGUS_GPU_NO_PROBLEM, "no adjoint computed (bogus_gpu_adjoint)");
  if (int e = ensure_host_lower(h)) return e;
  if (!dW) return fail(BOGUS_GPU_BAD_INPUT, "null output");
  const HostBSR& l = h->host_lower;
  const size_t n3 = 3 * (size_t)l.n;
  if (h->h_adj_s.size() != n3 || h->h_adj_r.size() != n3) {
    if (int e = set_device(h)) return e;
    h->h_adj_s.resize(n3);
    h->h_adj_r.resize(n3);
    if (n3) {
      BG_CUDA(cudaMemcpy(h->h_adj_s.data(), h->adj_S.p, sizeof(double) * n3, cudaMemcpyDeviceToHost));
      BG_CUDA(cudaMemcpy(h->h_adj_r.data(), h->adj_r.p, sizeof(double) * n3, cudaMemcpyDeviceToHost));
    }
  }
  const double* sv = h->h_adj_s.data();
  const double* rv = h->h_adj_r.data();
  for (int i = 0; i < l.n; ++i)
    for (int k = l.rowptr[i]; k < l.rowptr[i + 1]; ++k) {
      const int j = l.col[k];
      double* G = dW + 9 * (size_t)k;
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c)
          G[3 * a + c] = sv[3 * i + a] * rv[3 * j + c] + (i != j ? rv[3 * i + a] * sv[3 * j + c] : 0.0);
    }
  return BOGUS_GPU_OK;
}

int bogus_gpu_adjoint_primal(bogus_gpu_problem* h, const double* f, double* dHA, double* dHB, double* dw,
                             double* df) {
  if (int e = check_handle(h)) return e;
  if (!h->adj_valid) return fail(BOGUS_GPU_NO_PROBLEM, "no adjoint computed (bogus_gpu_adjoint)");
  if (h->nbodies == 0 || h->ncontacts != h->W.n)
    return fail(BOGUS_GPU_NO_PROBLEM, "the dual problem was not assembled from the handle's primal data");
  if (int e = set_device(h)) return e;
  const int n = h->ncontacts, nb = h->nbodies, d = h->ndof;
  const size_t m = (size_t)nb * d, n3 = 3 * (size_t)n, hs = 3 * (size_t)d;
  if (f)
    if (int e = check_finite(f, m, "f")) return e;
  if (int e = ensure_incidence(h)) return e;
  cudaStream_t s = h->stream;
  DevBuf<double> fd, vr, vs, dH;
  BG_CUDA(vr.ensure(m));
  BG_CUDA(vs.ensure(m));
  BG_CUDA(dH.ensure(2 * n3 * d > 0 ? 2 * n3 * d : 1));
  if (f) {
    BG_CUDA(fd.ensure(m));
    BG_CUDA(cudaMemcpyAsync(fd.p, f, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  BG_CUDA(launch_body_transpose(nb, d, h->bptr.p, h->bent.p, h->H.p, h->minv.p, h->adj_r.p, f ? fd.p : nullptr,
                                vr.p, s));
  BG_CUDA(launch_body_transpose(nb, d, h->bptr.p, h->bent.p, h->H.p, h->minv.p, h->adj_S.p, nullptr, vs.p, s));
  BG_CUDA(launch_h_gradient(n, d, h->cb.p, h->adj_S.p, h->adj_r.p, vr.p, vs.p, dH.p, s));
  std::vector<double> slots(2 * n3 * d);
  std::vector<double> vsh(m);
  if (n) BG_CUDA(cudaMemcpyAsync(slots.data(), dH.p, sizeof(double) * slots.size(), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaMemcpyAsync(vsh.data(), vs.p, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
  std::vector<double> sh(n3);
  if (n) BG_CUDA(cudaMemcpyAsync(sh.data(), h->adj_S.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i) {
    // slots are ordered by body index; map them back to A and B
    const int s0 = h->h_cb[2 * (size_t)i], s1 = h->h_cb[2 * (size_t)i + 1];
    const double* g0 = &slots[(2 * (size_t)i) * hs];
    const double* g1 = &slots[(2 * (size_t)i + 1) * hs];
    const bool b_first = s1 >= 0 && s0 != h->h_objA[i];
    double* A = dHA ? dHA + (size_t)i * hs : nullptr;
    double* B = dHB ? dHB + (size_t)i * hs : nullptr;
    for (size_t k = 0; k < hs; ++k) {
      if (A) A[k] = b_first ? g1[k] : g0[k];
      if (B) B[k] = s1 < 0 ? 0.0 : (b_first ? g0[k] : g1[k]);
    }
  }
  if (dw) std::memcpy(dw, sh.data(), sizeof(double) * n3);
  if (df)
    for (size_t k = 0; k < m; ++k) df[k] = -vsh[k];
  return BOGUS_GPU_OK;
}

int bogus_gpu_add_compliance(bogus_gpu_problem* h, const double* c) {
  if (int e = check_handle(h)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  const int n = h->W.n;
  if (n > 0 && !c) return fail(BOGUS_GPU_BAD_INPUT, "null compliance");
  for (int i = 0; i < n; ++i)
    if (!(c[i] >= 0) || !std::isfinite(c[i])) return fail(BOGUS_GPU_BAD_INPUT, "compliance must be finite and >= 0");
  if (int e = set_device(h)) return e;
  {
    std::vector<int> dg(n);
    if (n) BG_CUDA(cudaMemcpy(dg.data(), h->W.diag, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i)
      if (dg[i] < 0) return fail(BOGUS_GPU_BAD_INPUT, "W has no diagonal block at some contact");
  }
  DevBuf<double> dc;
  BG_CUDA(dc.ensure(n > 0 ? n : 1));
  if (n) BG_CUDA(cudaMemcpyAsync(dc.p, c, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  if (h->low_pending)  // the host copy of the lower triangle takes the same diagonal terms
    if (int e = ensure_host_lower(h)) return e;
  BG_CUDA(launch_add_diagonal(h->W, dc.p, h->stream));
  BG_CUDA(launch_diag_and_scaling(h->W, h->scaling.p, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  if (h->host_lower_valid) {
    HostBSR& l = h->host_lower;
    for (int i = 0; i < n; ++i) {
      const int k = l.rowptr[i + 1] - 1;  // the diagonal block ends a lower row
      double* B = &l.val[9 * (size_t)k];
      B[0] = B[0] + c[i];
      B[4] = B[4] + c[i];
      B[8] = B[8] + c[i];
    }
  }
  h->gs.valid = false;
  h->fp32_valid = false;
  h->fp32p_valid = false;
  h->il_valid = false;
  h->adj_valid = false;
  return BOGUS_GPU_OK;
}

void bogus_gpu_admm_options_default(bogus_gpu_admm_options* o) {
  if (!o) return;
  o->tol = 1e-6;
  o->max_iters = 300;
  o->step_size = 1e-2;
  o->variant = BOGUS_GPU_ADMM_ACCELERATED;
  o->use_infinity_norm = 0;
}

int bogus_gpu_solve_admm(bogus_gpu_problem* h, const bogus_gpu_admm_options* o, double lambda,
                         const double* prox, const double* f, const double* w, const double* mu, double* v,
                         double* r, double* residual, unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (!o) return fail(BOGUS_GPU_BAD_INPUT, "null options");
  if (h->nbodies == 0) return fail(BOGUS_GPU_NO_PROBLEM, "no primal problem set (bogus_gpu_set_primal)");
  if (o->variant != BOGUS_GPU_ADMM_STANDARD && o->variant != BOGUS_GPU_ADMM_ACCELERATED)
    return fail(BOGUS_GPU_BAD_INPUT, "unknown ADMM variant");
  if (!(o->step_size > 0) || !(o->tol >= 0) || !std::isfinite(lambda) || lambda < 0)
    return fail(BOGUS_GPU_BAD_INPUT, "invalid ADMM step size, tolerance or lambda");
  const int n = h->ncontacts, nb = h->nbodies, d = h->ndof;
  const size_t n3 = 3 * (size_t)n, m = (size_t)nb * d;
  if ((n > 0 && (!w || !mu || !r)) || !v) return fail(BOGUS_GPU_BAD_INPUT, "null w, mu, v or r");
  if (int e = check_finite(w, n3, "w")) return e;
  if (int e = check_finite(mu, n, "mu")) return e;
  if (int e = check_finite(v, m, "v")) return e;
  if (int e = check_finite(r, n3, "r")) return e;
  if (f)
    if (int e = check_finite(f, m, "f")) return e;
  if (prox)
    if (int e = check_finite(prox, m * d, "prox")) return e;
  if (int e = set_device(h)) return e;
  cudaStream_t s = h->stream;
  if (int e = ensure_incidence(h)) return e;
  const size_t nv = n3 > 0 ? n3 : 1;
  for (auto* b : {&h->a_w, &h->a_r, &h->a_ut, &h->a_z, &h->a_zacc, &h->a_rs1, &h->a_rs2, &h->a_yprev})
    BG_CUDA(b->ensure(nv));
  BG_CUDA(h->a_mu.ensure(n > 0 ? n : 1));
  BG_CUDA(h->a_invmu.ensure(n > 0 ? n : 1));
  BG_CUDA(h->a_x.ensure(m));
  if (f) BG_CUDA(h->a_f.ensure(m));
  if (prox) BG_CUDA(h->a_prox.ensure(m * d));
  const int C = (n + 31) / 32;
  BG_CUDA(h->csum.ensure(2 * (size_t)(C > 0 ? C : 1)));
  BG_CUDA(h->scal.ensure(8 + 32));  // scalars, then the stripe sums of grid_barrier_combine
  BG_CUDA(h->trace.ensure((size_t)o->max_iters + 1));
  BG_CUDA(h->admm_out.ensure(1));
  BG_CUDA(h->barrier.ensure(8));
  BG_CUDA(h->status.ensure(1));
  if (n > 0) {
    BG_CUDA(cudaMemcpyAsync(h->a_w.p, w, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
    if (h->frames_valid) BG_CUDA(launch_frame(n, h->frames.p, h->a_w.p, h->a_w.p, true, s));
    BG_CUDA(cudaMemcpyAsync(h->a_mu.p, mu, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->a_r.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  }
  BG_CUDA(cudaMemcpyAsync(h->a_x.p, v, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (f) BG_CUDA(cudaMemcpyAsync(h->a_f.p, f, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (prox) BG_CUDA(cudaMemcpyAsync(h->a_prox.p, prox, sizeof(double) * m * d, cudaMemcpyHostToDevice, s));
  ADMMArgs a{};
  a.n = n;
  a.nbodies = nb;
  a.d = d;
  a.cb = h->cb.p;
  a.H = h->H.p;
  a.bptr = h->bptr.p;
  a.bent = h->bent.p;
  a.border = h->border.p;
  a.prox = prox ? h->a_prox.p : h->minv.p;
  a.f = f ? h->a_f.p : nullptr;
  a.w = h->a_w.p;
  a.mu = h->a_mu.p;
  a.inv_mu = h->a_invmu.p;
  a.x = h->a_x.p;
  a.r = h->a_r.p;
  a.ut = h->a_ut.p;
  a.z = h->a_z.p;
  a.zacc = h->a_zacc.p;
  a.yprev = h->a_yprev.p;
  a.r_spare[0] = h->a_rs1.p;
  a.r_spare[1] = h->a_rs2.p;
  a.csum = h->csum.p;
  a.scal = h->scal.p;
  a.trace = h->trace.p;
  a.out = h->admm_out.p;
  a.gb = GridBarrier{h->barrier.p, h->barrier.p + 1, h->status.p};
  a.tickets = h->barrier.p + 2;
  a.combine_count = h->barrier.p + 4;
  a.stripes = h->scal.p + 8;
  a.lambda = lambda;
  a.gamma = o->step_size;
  a.tol = o->tol;
  a.max_iters = o->max_iters;
  a.accelerated = o->variant == BOGUS_GPU_ADMM_ACCELERATED;
  a.use_inf = o->use_infinity_norm ? 1 : 0;
  a.scaling = h->a_sc.p;
  BG_CUDA(cudaMemsetAsync(h->barrier.p, 0, 8 * sizeof(unsigned), s));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  int grid = admm_max_grid(h->device, d);
  if (grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "cooperative occupancy query failed");
  const int units = ((n > nb ? n : nb) + 31) / 32;
  const int want = (units + 7) / 8;
  if (want < grid) grid = want < 1 ? 1 : want;
  BG_CUDA(cudaEventRecord(h->ev0, s));
  BG_CUDA(launch_admm(a, grid, s));
  BG_CUDA(cudaEventRecord(h->ev1, s));
  ADMMOut out{};
  int st = 0;
  BG_CUDA(cudaMemcpyAsync(&out, h->admm_out.p, sizeof(ADMMOut), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->last_launches = 1;
  if (st != 0) return fail(st, "device-side wait timed out in the ADMM kernel");
  BG_CUDA(cudaMemcpy(v, h->a_x.p, sizeof(double) * m, cudaMemcpyDeviceToHost));
  if (n > 0) BG_CUDA(cudaMemcpy(r, h->a_r.p, sizeof(double) * n3, cudaMemcpyDeviceToHost));
  {
    // per iteration: P1 reads the incidences, 3 x d H rows, r (and zacc, ut with lambda) per incidence,
    // the d x d prox block, f and x per body and writes x; P2 reads H, x of the bodies, w, r, z, 1/mu and
    // writes ut per contact; its P3 part writes z and the plain branch's r, and in the accelerated variant
    // reads y_prev and writes the accelerated branch's r, y_prev and zacc
    const double inc = (double)h->admm_ninc;
    const double p1 = inc * (4.0 + 24.0 * d + 24.0 + (lambda < 2.220446049250313e-16 ? 0.0 : 48.0)) +
                      (double)nb * (8.0 * d * d + (f ? 16.0 : 8.0) * d + 4.0);
    const double p2 = inc * (24.0 * d + 8.0 * d + 4.0) + (double)n * (24.0 * 4 + 8.0);
    const double p3 = (double)n * (24.0 * 2 + (o->variant == BOGUS_GPU_ADMM_ACCELERATED ? 24.0 * 4 : 0.0));
    h->last_stats.iterations = out.iters;
    h->last_stats.refine_iterations = 0;
    h->last_stats.fp32_device_ms = 0.0;
    h->last_stats.w_passes = 0;
    h->last_stats.algorithmic_bytes = out.iters * (p1 + p2 + p3) + (p2 + p3);
    h->last_stats.fp64_fma = (double)out.iters * inc * 3.0 * d * 2.0;
  }
  if (residual) *residual = out.res;
  if (iters) *iters = out.iters;
  if (h->callback) {
    const unsigned count = out.converged ? out.iters + 1 : out.iters;
    std::vector<double> tr(count);
    if (count) BG_CUDA(cudaMemcpy(tr.data(), h->trace.p, sizeof(double) * count, cudaMemcpyDeviceToHost));
    for (unsigned k = 0; k < count; ++k) h->callback(k, tr[k], h->callback_user);
  }
  return out.converged ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

void bogus_gpu_dual_ama_options_default(bogus_gpu_dual_ama_options* o) {
  if (!o) return;
  o->tol = 1e-6;
  o->max_iters = 300;
  o->fp_step_size = 1.e-1;
  o->proj_step_size = 1.e-1;
  o->ls_iters = 6;
  o->ls_optimistic_factor = 1.25;
  o->ls_pessimistic_factor = .5;
  o->variant = BOGUS_GPU_ADMM_ACCELERATED;
  o->use_infinity_norm = 0;
}

int bogus_gpu_solve_dual_ama(bogus_gpu_problem* h, const bogus_gpu_dual_ama_options* o, const double* mass,
                             const double* f, const double* w, const double* mu, int static_problem, double* v,
                             double* r, double* residual, unsigned* iters) {
  if (int e = check_handle(h)) return e;
  if (!o) return fail(BOGUS_GPU_BAD_INPUT, "null options");
  if (h->nbodies == 0) return fail(BOGUS_GPU_NO_PROBLEM, "no primal problem set (bogus_gpu_set_primal)");
  if (o->variant != BOGUS_GPU_ADMM_STANDARD && o->variant != BOGUS_GPU_ADMM_ACCELERATED)
    return fail(BOGUS_GPU_BAD_INPUT, "unknown DualAMA variant");
  if (!(o->fp_step_size > 0) || !(o->proj_step_size > 0) || !(o->tol >= 0) || !(o->ls_optimistic_factor > 0) ||
      !(o->ls_pessimistic_factor > 0) || !std::isfinite(o->fp_step_size) || !std::isfinite(o->proj_step_size))
    return fail(BOGUS_GPU_BAD_INPUT, "invalid DualAMA step sizes, factors or tolerance");
  const int n = h->ncontacts, nb = h->nbodies, d = h->ndof;
  const size_t n3 = 3 * (size_t)n, m = (size_t)nb * d;
  if ((n > 0 && (!w || !mu || !r)) || !v || !mass) return fail(BOGUS_GPU_BAD_INPUT, "null mass, w, mu, v or r");
  if (int e = check_finite(mass, m * d, "mass")) return e;
  if (int e = check_finite(w, n3, "w")) return e;
  if (int e = check_finite(mu, n, "mu")) return e;
  if (int e = check_finite(v, m, "v")) return e;
  if (int e = check_finite(r, n3, "r")) return e;
  if (f)
    if (int e = check_finite(f, m, "f")) return e;
  if (int e = set_device(h)) return e;
  cudaStream_t s = h->stream;
  if (int e = ensure_incidence(h)) return e;
  const size_t nv = n3 > 0 ? n3 : 1;
  for (auto* b : {&h->a_w, &h->a_r, &h->a_ut, &h->dm_rs, &h->dm_g, &h->dm_rb}) BG_CUDA(b->ensure(nv));
  for (auto* b : {&h->dm_f, &h->dm_v, &h->dm_x, &h->dm_hr, &h->dm_yp, &h->dm_vb, &h->dm_v2, &h->dm_yp2})
    BG_CUDA(b->ensure(m));
  BG_CUDA(h->dm_M.ensure(m * d));
  BG_CUDA(h->a_mu.ensure(n > 0 ? n : 1));
  const int C = (n + 31) / 32, CB = (nb + 31) / 32;
  const int CC = C > CB ? C : CB;
  BG_CUDA(h->csum.ensure(3 * (size_t)(CC > 0 ? CC : 1)));
  BG_CUDA(h->scal.ensure(8 + 32));  // scalars, then the stripe sums of grid_barrier_combine
  BG_CUDA(h->trace.ensure((size_t)o->max_iters + 1));
  BG_CUDA(h->dama_out.ensure(1));
  BG_CUDA(h->barrier.ensure(8));
  BG_CUDA(h->status.ensure(1));
  if (n > 0) {
    BG_CUDA(cudaMemcpyAsync(h->a_w.p, w, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
    if (h->frames_valid) BG_CUDA(launch_frame(n, h->frames.p, h->a_w.p, h->a_w.p, true, s));
    BG_CUDA(cudaMemcpyAsync(h->a_mu.p, mu, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->a_r.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
    BG_CUDA(cudaMemcpyAsync(h->dm_rb.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  }
  BG_CUDA(cudaMemcpyAsync(h->dm_v.p, v, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(h->dm_vb.p, v, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(h->dm_yp.p, v, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(h->dm_M.p, mass, sizeof(double) * m * d, cudaMemcpyHostToDevice, s));
  if (f) BG_CUDA(cudaMemcpyAsync(h->dm_f.p, f, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  else BG_CUDA(cudaMemsetAsync(h->dm_f.p, 0, sizeof(double) * m, s));
  DamaArgs a{};
  a.n = n;
  a.nbodies = nb;
  a.d = d;
  a.cb = h->cb.p;
  a.H = h->H.p;
  a.bptr = h->bptr.p;
  a.bent = h->bent.p;
  a.M = h->dm_M.p;
  a.f = h->dm_f.p;
  a.w = h->a_w.p;
  a.mu = h->a_mu.p;
  a.scaling = h->a_sc.p;
  a.v = h->dm_v.p;
  a.r = h->a_r.p;
  a.rs = h->dm_rs.p;
  a.x = h->dm_x.p;
  a.HrBp = h->dm_hr.p;
  a.ut = h->a_ut.p;
  a.g = h->dm_g.p;
  a.y_prev = h->dm_yp.p;
  a.v_spare = h->dm_v2.p;
  a.yp_spare = h->dm_yp2.p;
  a.r_best = h->dm_rb.p;
  a.v_best = h->dm_vb.p;
  a.csum = h->csum.p;
  a.scal = h->scal.p;
  a.trace = h->trace.p;
  a.out = h->dama_out.p;
  a.gb = GridBarrier{h->barrier.p, h->barrier.p + 1, h->status.p};
  a.tickets = h->barrier.p + 2;
  a.combine_count = h->barrier.p + 4;
  a.stripes = h->scal.p + 8;
  a.tol = o->tol;
  a.gamma = o->fp_step_size;
  a.lambda0 = o->proj_step_size;
  a.opt = o->ls_optimistic_factor;
  a.pess = o->ls_pessimistic_factor;
  a.m_true = (double)h->true_dofs;
  a.max_iters = o->max_iters;
  a.ls_iters = o->ls_iters;
  a.accelerated = o->variant == BOGUS_GPU_ADMM_ACCELERATED;
  a.use_inf = o->use_infinity_norm ? 1 : 0;
  a.desaxce = static_problem ? 0 : 1;
  BG_CUDA(cudaMemsetAsync(h->barrier.p, 0, 8 * sizeof(unsigned), s));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  int grid = dama_max_grid(h->device, d);
  if (grid <= 0) return fail(BOGUS_GPU_CUDA_ERROR, "cooperative occupancy query failed");
  const int want = (CC + 7) / 8;
  if (want < grid) grid = want < 1 ? 1 : want;
  BG_CUDA(cudaEventRecord(h->ev0, s));
  BG_CUDA(launch_dama(a, grid, s));
  BG_CUDA(cudaEventRecord(h->ev1, s));
  DamaOut out{};
  int st = 0;
  BG_CUDA(cudaMemcpyAsync(&out, h->dama_out.p, sizeof(DamaOut), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->last_launches = 1;
  if (st != 0) return fail(st, "device-side wait timed out in the DualAMA kernel");
  BG_CUDA(cudaMemcpy(v, h->dm_vb.p, sizeof(double) * m, cudaMemcpyDeviceToHost));
  if (n > 0) BG_CUDA(cudaMemcpy(r, h->dm_rb.p, sizeof(double) * n3, cudaMemcpyDeviceToHost));
  {
    // per iteration: Q1 reads M, f, v, H^T r per body and writes x; reads w, H and v of the bodies, r, mu and
    // the scaling and writes u per contact; Q2 reads u, mu, H and (H^T r, x) of the bodies, writes g; per
    // line-search trial Q3 reads r, g, mu and writes r_s, Q4 reads the incidences, H rows and r_s per
    // incidence, x, v, y_prev, f and M per body and writes H^T r_s and the candidate v, y_prev; without a line
    // search Q5 reads the incidences, H rows and r per incidence, x, v, y_prev and writes H^T r, v, y_prev
    const double inc = (double)h->admm_ninc, dd = (double)d, nn = (double)n, bb = (double)nb;
    const bool ls = o->ls_iters != 0;
    const double q1 = bb * (8.0 * dd * dd + 32.0 * dd) + inc * (24.0 * dd + 8.0 * dd) + nn * (24.0 * 3 + 16.0);
    const double q2 = inc * (24.0 * dd + 16.0 * dd) + nn * (24.0 + 8.0 + 24.0);
    const double q34 =
        nn * (24.0 * 3 + 8.0) + inc * (4.0 + 24.0 * dd + 24.0) + bb * (8.0 * dd * dd + 48.0 * dd + 16.0 * dd);
    const double q5 = ls ? 0.0 : inc * (4.0 + 24.0 * dd + 24.0) + bb * 48.0 * dd;
    h->last_stats.iterations = out.iters;
    h->last_stats.refine_iterations = 0;
    h->last_stats.fp32_device_ms = 0.0;
    h->last_stats.w_passes = 0;
    h->last_stats.algorithmic_bytes = out.iters * (q1 + q2 + q5) + (double)out.trials * q34 + q1;
    h->last_stats.fp64_fma = (double)out.iters * inc * 3.0 * dd * 3.0 + (double)out.trials * inc * 3.0 * dd;
  }
  if (residual) *residual = out.min_res;
  if (iters) *iters = out.iters;
  if (h->callback) {
    const unsigned count = out.iters < o->max_iters ? out.iters + 1 : out.iters;
    std::vector<double> tr(count);
    if (count) BG_CUDA(cudaMemcpy(tr.data(), h->trace.p, sizeof(double) * count, cudaMemcpyDeviceToHost));
    for (unsigned k = 0; k < count; ++k) h->callback(k, tr[k], h->callback_user);
  }
  return out.min_res >= 0 && out.min_res < o->tol ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

int bogus_gpu_assemble_dual(bogus_gpu_problem* h, const double* f, const double* w, const double* mu) {
  if (int e = check_handle(h)) return e;
  if (h->ncontacts == 0 && h->nbodies == 0) return fail(BOGUS_GPU_NO_PROBLEM, "no primal problem set");
  if (h->ncontacts > 0 && (!w || !mu)) return fail(BOGUS_GPU_BAD_INPUT, "null w or mu");
  if (int e = set_device(h)) return e;
  const int n = h->ncontacts, nb = h->nbodies, d = h->ndof;
  if (int e = check_finite(w, 3 * (size_t)n, "w")) return e;
  if (int e = check_finite(mu, n, "mu")) return e;
  if (f)
    if (int e = check_finite(f, (size_t)nb * d, "f")) return e;
  // symbolic part: lower blocks (i, j <= i) of contacts sharing a body, shared (slot_i, slot_j) pairs
  std::vector<std::vector<int>> by_body(nb);
  for (int i = 0; i < n; ++i)
    for (int t = 0; t < 2; ++t)
      if (h->h_cb[2 * (size_t)i + t] >= 0) by_body[h->h_cb[2 * (size_t)i + t]].push_back(i);
  HostBSR low;
  low.n = n;
  low.rowptr.assign(n + 1, 0);
  std::vector<int> li, lj, pair_off(1, 0), pair_ti, pair_tj, cols;
  for (int i = 0; i < n; ++i) {
    cols.clear();
    for (int t = 0; t < 2; ++t) {
      const int k = h->h_cb[2 * (size_t)i + t];
      if (k < 0) continue;
      for (int j : by_body[k])
        if (j <= i) cols.push_back(j);
    }
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    for (int j : cols) {
      li.push_back(i);
      lj.push_back(j);
      for (int ti = 0; ti < 2; ++ti)
        for (int tj = 0; tj < 2; ++tj) {
          const int bi = h->h_cb[2 * (size_t)i + ti], bj = h->h_cb[2 * (size_t)j + tj];
          if (bi >= 0 && bi == bj) {
            pair_ti.push_back(ti);
            pair_tj.push_back(tj);
          }
        }
      pair_off.push_back((int)pair_ti.size());
      low.col.push_back(j);
    }
    low.rowptr[i + 1] = (int)low.col.size();
  }
  const int nlow = (int)li.size();
  // full-structure positions of every lower block and of its transpose
  HostBSR fullpat;
  fullpat.n = n;
  {
    std::vector<int> cnt(n + 1, 0);
    for (int k = 0; k < nlow; ++k) {
      ++cnt[li[k] + 1];
      if (lj[k] != li[k]) ++cnt[lj[k] + 1];
    }
    fullpat.rowptr.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) fullpat.rowptr[i + 1] = fullpat.rowptr[i] + cnt[i + 1];
  }
  std::vector<int> pos_ij(nlow), pos_ji(nlow, -1);
  fullpat.col.assign(fullpat.rowptr[n], 0);
  {
    std::vector<int> pos(fullpat.rowptr.begin(), fullpat.rowptr.end() - 1);
    for (int k = 0; k < nlow; ++k) {  // lower blocks come row by row, columns increasing
      pos_ij[k] = pos[li[k]]++;
      fullpat.col[pos_ij[k]] = lj[k];
      if (lj[k] != li[k]) {
        pos_ji[k] = pos[lj[k]]++;
        fullpat.col[pos_ji[k]] = li[k];
      }
    }
  }
  const int nnz = fullpat.rowptr[n];
  DevBuf<int> d_li, d_lj, d_off, d_ti, d_tj, d_pij, d_pji;
  BG_CUDA(d_li.ensure(nlow)); BG_CUDA(d_lj.ensure(nlow)); BG_CUDA(d_off.ensure(nlow + 1));
  BG_CUDA(d_ti.ensure(pair_ti.size())); BG_CUDA(d_tj.ensure(pair_tj.size()));
  BG_CUDA(d_pij.ensure(nlow)); BG_CUDA(d_pji.ensure(nlow));
  cudaStream_t s = h->stream;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
  };
  BG_CUDA(up(d_li.p, li.data(), sizeof(int) * nlow));
  BG_CUDA(up(d_lj.p, lj.data(), sizeof(int) * nlow));
  BG_CUDA(up(d_off.p, pair_off.data(), sizeof(int) * (nlow + 1)));
  BG_CUDA(up(d_ti.p, pair_ti.data(), sizeof(int) * pair_ti.size()));
  BG_CUDA(up(d_tj.p, pair_tj.data(), sizeof(int) * pair_tj.size()));
  BG_CUDA(up(d_pij.p, pos_ij.data(), sizeof(int) * nlow));
  BG_CUDA(up(d_pji.p, pos_ji.data(), sizeof(int) * nlow));
  BG_CUDA(h->rowptr.ensure(n + 1));
  BG_CUDA(h->col.ensure(nnz));
  BG_CUDA(h->val.ensure(9 * (size_t)nnz));
  BG_CUDA(h->diag.ensure(n));
  BG_CUDA(h->b.ensure(3 * (size_t)n));
  BG_CUDA(h->mu.ensure(n));
  BG_CUDA(h->scaling.ensure(n));
  BG_CUDA(h->T.ensure(2 * (size_t)n * d * 3));
  BG_CUDA(h->mf.ensure((size_t)nb * d));
  BG_CUDA(up(h->rowptr.p, fullpat.rowptr.data(), sizeof(int) * (n + 1)));
  BG_CUDA(up(h->col.p, fullpat.col.data(), sizeof(int) * nnz));
  BG_CUDA(up(h->mu.p, mu, sizeof(double) * n));
  DevBuf<double> d_w, d_f;
  BG_CUDA(d_w.ensure(3 * (size_t)n));
  BG_CUDA(up(d_w.p, w, sizeof(double) * 3 * n));
  if (h->frames_valid) BG_CUDA(launch_frame(n, h->frames.p, d_w.p, d_w.p, true, s));
  if (f) {
    BG_CUDA(d_f.ensure((size_t)nb * d));
    BG_CUDA(up(d_f.p, f, sizeof(double) * nb * d));
  }
  BG_CUDA(cudaEventRecord(h->ev0, s));
  BG_CUDA(launch_assembly_T(n, d, h->minv.p, h->cb.p, h->H.p, h->T.p, s));
  BG_CUDA(launch_assembly_W(nlow, d, d_li.p, d_lj.p, d_off.p, d_ti.p, d_tj.p, h->H.p, h->T.p, d_pij.p, d_pji.p,
                            h->val.p, s));
  BG_CUDA(launch_assembly_b(n, nb, d, h->minv.p, f ? d_f.p : nullptr, h->cb.p, h->H.p, d_w.p, h->mf.p, h->b.p, s));
  BG_CUDA(cudaEventRecord(h->ev1, s));
  h->W.n = n;
  h->W.nnzb = nnz;
  h->W.rowptr = h->rowptr.p;
  h->W.col = h->col.p;
  h->W.val = h->val.p;
  h->W.diag = h->diag.p;
  BG_CUDA(launch_diag_and_scaling(h->W, h->scaling.p, s));
  // host copies for the Gauss-Seidel coloring / permutation
  low.val.resize(9 * (size_t)nlow);
  std::vector<double> fullval(9 * (size_t)nnz);
  if (nnz) BG_CUDA(cudaMemcpyAsync(fullval.data(), h->val.p, sizeof(double) * 9 * (size_t)nnz, cudaMemcpyDeviceToHost, s));
  h->host_b.resize(3 * (size_t)n);
  if (n) BG_CUDA(cudaMemcpyAsync(h->host_b.data(), h->b.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  BG_CUDA(cudaStreamSynchronize(s));
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->last_launches = 3;
  for (int k = 0; k < nlow; ++k) std::copy(&fullval[9 * (size_t)pos_ij[k]], &fullval[9 * (size_t)pos_ij[k]] + 9, &low.val[9 * (size_t)k]);
  h->host_lower = std::move(low);
  h->host_lower_valid = true;
  h->low_pending = false;
  h->permuted = false;
  h->host_mu.assign(mu, mu + n);
  d_li.release(); d_lj.release(); d_off.release(); d_ti.release(); d_tj.release(); d_pij.release(); d_pji.release();
  d_w.release(); d_f.release();
  h->has_dual = true;
  h->gs.valid = false;
  h->nproblems = 0;
  h->fp32_valid = false;
  h->fp32p_valid = false;
  h->il_valid = false;
  h->adj_valid = false;
  return BOGUS_GPU_OK;
}

int bogus_gpu_set_batch(bogus_gpu_problem* h, int nproblems, const int* cptr) {
  if (int e = check_handle(h)) return e;
  if (h->permuted) return fail(BOGUS_GPU_BAD_INPUT, "batched solves need the contacts in their own order (undo the permutation)");
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (nproblems < 0 || (nproblems > 0 && !cptr)) return fail(BOGUS_GPU_BAD_INPUT, "invalid batch partition");
  const int n = h->W.n;
  if (nproblems == 0 ? n != 0 : (cptr[0] != 0 || cptr[nproblems] != n))
    return fail(BOGUS_GPU_BAD_INPUT, "contact_ptr must run from 0 to the number of contacts");
  for (int p = 0; p < nproblems; ++p)
    if (cptr[p + 1] < cptr[p]) return fail(BOGUS_GPU_BAD_INPUT, "contact_ptr not monotone");
  if (int e = set_device(h)) return e;
  // structure of the both-triangle W, to check block-diagonality and localise the column indices
  std::vector<int> rp(n + 1), cl(h->W.nnzb);
  BG_CUDA(cudaMemcpyAsync(rp.data(), h->W.rowptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, h->stream));
  if (h->W.nnzb) BG_CUDA(cudaMemcpyAsync(cl.data(), h->W.col, sizeof(int) * h->W.nnzb, cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  std::vector<int> chunk(nproblems + 1, 0), nnz(nproblems, 0);
  for (int p = 0; p < nproblems; ++p) {
    const int c0 = cptr[p], c1 = cptr[p + 1];
    for (int i = c0; i < c1; ++i)
      for (int k = rp[i]; k < rp[i + 1]; ++k) {
        if (cl[k] < c0 || cl[k] >= c1)
          return fail(BOGUS_GPU_BAD_INPUT, "W is not block diagonal for this partition (row " + std::to_string(i) + ")");
        cl[k] -= c0;
      }
    nnz[p] = rp[c1] - rp[c0];
    chunk[p + 1] = chunk[p] + (c1 - c0 + 31) / 32;
  }
  std::vector<int> queue(nproblems);
  for (int p = 0; p < nproblems; ++p) queue[p] = p;
  std::stable_sort(queue.begin(), queue.end(),
                   [&](int a, int b) { return cptr[a + 1] - cptr[a] > cptr[b + 1] - cptr[b]; });
  BG_CUDA(h->contact_ptr.ensure(nproblems + 1));
  BG_CUDA(h->chunk_ptr.ensure(nproblems + 1));
  BG_CUDA(h->queue.ensure(nproblems > 0 ? nproblems : 1));
  BG_CUDA(h->col_local.ensure(h->W.nnzb));
  BG_CUDA(h->next.ensure(1));
  BG_CUDA(h->batch_out.ensure(nproblems > 0 ? nproblems : 1));
  cudaStream_t s = h->stream;
  BG_CUDA(cudaMemcpyAsync(h->contact_ptr.p, cptr, sizeof(int) * (nproblems + 1), cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaMemcpyAsync(h->chunk_ptr.p, chunk.data(), sizeof(int) * (nproblems + 1), cudaMemcpyHostToDevice, s));
  if (nproblems) BG_CUDA(cudaMemcpyAsync(h->queue.p, queue.data(), sizeof(int) * nproblems, cudaMemcpyHostToDevice, s));
  if (h->W.nnzb) BG_CUDA(cudaMemcpyAsync(h->col_local.p, cl.data(), sizeof(int) * h->W.nnzb, cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaStreamSynchronize(s));
  h->nproblems = nproblems;
  h->h_contact_ptr.assign(cptr, cptr + nproblems + 1);
  h->h_problem_nnz = nnz;
  h->tuned_shape[0] = h->tuned_shape[1] = BatchShape{};
  h->tune_ms.clear();
  h->tune_cand.clear();
  if (h->batch_graph) {
    cudaGraphExecDestroy(h->batch_graph);
    h->batch_graph = nullptr;
  }
  return BOGUS_GPU_OK;
}

}  // extern "C"

namespace {

// ---- launch shape of a batched solve ------------------------------------------------------------------
int batch_max_chunks(const bogus_gpu_problem* h) {
  int maxchunks = 0;
  for (int p = 0; p < h->nproblems; ++p)
    maxchunks = std::max(maxchunks, (h->h_contact_ptr[p + 1] - h->h_contact_ptr[p] + 31) / 32);
  return maxchunks;
}

// The default rule: one CTA per problem (k_pg_batched, as many resident CTAs as fit) when there are at least as
// many problems as half the resident team CTAs (3 per SM), else teams sized so that they fill the GPU and each
// CTA's warps still have a chunk of the largest problem each.
BatchShape rule_shape(const bogus_gpu_problem* h, bool fp32) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  const int np = h->nproblems;
  const int team_per = std::min(3, pg_team_per_sm(h->device, fp32));
  const int gmax = team_per * sms;
  int size = np > 0 ? gmax / np : 0;
  size = std::min(size, std::min(16, std::max(1, batch_max_chunks(h) / 8)));
  BatchShape sh;
  if (size < 2) {
    sh.schedule = 0;
    sh.ctas_per_sm = pg_batched_per_sm(h->device, fp32);
    sh.team_size = 1;
  } else {
    sh.schedule = 1;
    sh.ctas_per_sm = team_per;
    sh.team_size = size;
  }
  return sh;
}

int check_shape(const bogus_gpu_problem* h, const BatchShape& sh, bool fp32) {
  const int per = sh.schedule == 0 ? pg_batched_per_sm(h->device, fp32) : pg_team_per_sm(h->device, fp32);
  if (sh.schedule != 0 && sh.schedule != 1) return fail(BOGUS_GPU_BAD_INPUT, "batch schedule must be 0 or 1");
  if (sh.ctas_per_sm < 1 || sh.ctas_per_sm > per)
    return fail(BOGUS_GPU_BAD_INPUT, "ctas_per_sm must lie in [1, " + std::to_string(per) + "] for this kernel");
  if (sh.schedule == 1 && (sh.team_size < 1 || sh.team_size > 64)) return fail(BOGUS_GPU_BAD_INPUT, "team_size must lie in [1, 64]");
  return BOGUS_GPU_OK;
}

// Team arguments and grid of a shape (schedule 1); allocates the team counters.
int team_setup(bogus_gpu_problem* h, const BatchShape& sh, PGTeamArgs* ta, int* grid) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
  const int np = h->nproblems;
  const int teams = std::max(1, std::min(np, sh.ctas_per_sm * sms / sh.team_size));
  BG_CUDA(h->team_cnt.ensure(8 * (size_t)teams));
  BG_CUDA(h->team_job.ensure(teams));
  BG_CUDA(h->team_scal.ensure(40 * (size_t)teams));
  *ta = PGTeamArgs{sh.team_size, h->team_cnt.p, h->team_job.p, h->team_scal.p, h->status.p};
  *grid = teams * sh.team_size;
  return BOGUS_GPU_OK;
}

// Enqueues one batched launch with the given shape (counters cleared first; nothing waits for it). The status word
// (a wait of the team schedule that ran out) is read by the caller after the stream is synchronised.
int launch_shape(bogus_gpu_problem* h, const BatchShape& sh, const PGBatchArgs* ba64, const PGBatchArgs32* ba32,
                 bool events) {
  const bool fp32 = ba32 != nullptr;
  const int np = h->nproblems;
  cudaStream_t s = h->stream;
  BG_CUDA(h->status.ensure(1));
  BG_CUDA(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
  BG_CUDA(cudaMemsetAsync(h->next.p, 0, sizeof(int), s));
  if (sh.schedule == 0) {
    int sms = 0;
    BG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
    int grid = sh.ctas_per_sm * sms;
    if (np < grid) grid = np > 0 ? np : 1;
    if (events) BG_CUDA(cudaEventRecord(h->ev0, s));
    BG_CUDA(fp32 ? launch_pg_batched(*ba32, grid, s) : launch_pg_batched(*ba64, grid, s));
    if (events) BG_CUDA(cudaEventRecord(h->ev1, s));
  } else {
    PGTeamArgs ta{};
    int grid = 0;
    if (int e = team_setup(h, sh, &ta, &grid)) return e;
    BG_CUDA(cudaMemsetAsync(h->team_cnt.p, 0, sizeof(unsigned) * 8 * (size_t)(grid / sh.team_size), s));
    if (events) BG_CUDA(cudaEventRecord(h->ev0, s));
    BG_CUDA(fp32 ? launch_pg_team(*ba32, ta, grid, s) : launch_pg_team(*ba64, ta, grid, s));
    if (events) BG_CUDA(cudaEventRecord(h->ev1, s));
  }
  h->last_shape = sh;
  return BOGUS_GPU_OK;
}

int read_status(bogus_gpu_problem* h) {
  int st = 0;
  BG_CUDA(cudaMemcpy(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (st != 0) return fail(st, "device-side wait timed out in the batched solve");
  return BOGUS_GPU_OK;
}

// The candidate shapes the tuner measures: one CTA per problem at 1..occupancy CTAs per SM (up to 4), and teams of
// 2, 4, 8, 16 CTAs (no larger than a quarter of the largest problem's chunks allows) at 2 and 3 CTAs per SM.
std::vector<BatchShape> tune_candidates(const bogus_gpu_problem* h, bool fp32) {
  std::vector<BatchShape> c;
  const int pb = std::min(4, pg_batched_per_sm(h->device, fp32));
  for (int k = 1; k <= pb; ++k) c.push_back(BatchShape{0, k, 1});
  const int pt = std::min(3, pg_team_per_sm(h->device, fp32));
  const int tmax = std::max(2, batch_max_chunks(h) / 4);
  for (int t = 2; t <= 16 && t <= tmax; t *= 2)
    for (int k = 2; k <= pt; ++k) c.push_back(BatchShape{1, k, t});
  return c;
}

// Process-wide cache of tuned shapes by device, precision and batch size class (problems, largest problem's and
// total chunks), so that another handle with a batch of the same make-up reuses the choice.
struct TuneKey {
  int device, fp32, np, maxchunks;
  long long chunks;
  bool operator<(const TuneKey& o) const {
    return std::tie(device, fp32, np, maxchunks, chunks) < std::tie(o.device, o.fp32, o.np, o.maxchunks, o.chunks);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, BatchShape> g_tune_cache;

TuneKey tune_key(const bogus_gpu_problem* h, bool fp32) {
  long long chunks = 0;
  for (int p = 0; p < h->nproblems; ++p) chunks += (h->h_contact_ptr[p + 1] - h->h_contact_ptr[p] + 31) / 32;
  return TuneKey{h->device, fp32 ? 1 : 0, h->nproblems, batch_max_chunks(h), chunks};
}

constexpr unsigned kTuneIters = 30;

int launch_args(bogus_gpu_problem* h, const BatchShape& sh, const PGBatchArgs& ba) {
  return launch_shape(h, sh, &ba, nullptr, true);
}
int launch_args(bogus_gpu_problem* h, const BatchShape& sh, const PGBatchArgs32& ba) {
  return launch_shape(h, sh, nullptr, &ba, true);
}

// Measures every candidate shape on the batch itself (each run from the same starting iterate, capped at
// kTuneIters iterations, timed with CUDA events) and keeps the fastest. The starting iterate (x0, 3 n values of
// type T) is restored afterwards.
template <class BA>
int tune_shape(bogus_gpu_problem* h, BA ba, bool fp32, size_t bytes_x0, void* x0) {
  cudaStream_t s = h->stream;
  BG_CUDA(h->tune_x.ensure((bytes_x0 + 7) / 8));
  BG_CUDA(cudaMemcpyAsync(h->tune_x.p, x0, bytes_x0, cudaMemcpyDeviceToDevice, s));
  ba.base.max_iters = std::min(ba.base.max_iters, kTuneIters);
  const std::vector<BatchShape> cand = tune_candidates(h, fp32);
  h->tune_cand = cand;
  h->tune_ms.assign(cand.size(), 0.0);
  int best = -1;
  for (size_t k = 0; k < cand.size(); ++k) {
    BG_CUDA(cudaMemcpyAsync(x0, h->tune_x.p, bytes_x0, cudaMemcpyDeviceToDevice, s));
    if (int e = launch_args(h, cand[k], ba)) return e;
    BG_CUDA(cudaStreamSynchronize(s));
    if (int st = read_status(h)) return st;
    float ms = 0.f;
    BG_CUDA(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->tune_ms[k] = ms;
    if (best < 0 || ms < h->tune_ms[best]) best = (int)k;
  }
  BG_CUDA(cudaMemcpyAsync(x0, h->tune_x.p, bytes_x0, cudaMemcpyDeviceToDevice, s));
  h->tuned_shape[fp32 ? 1 : 0] = cand[best];
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache[tune_key(h, fp32)] = cand[best];
  return BOGUS_GPU_OK;
}

// The shape of the next batched launch: the caller's, else the tuned one (tuning first when enabled and not yet
// done for this batch and precision, or taken from the process-wide cache), else the rule.
template <class BA>
int choose_shape(bogus_gpu_problem* h, const BA& ba, bool fp32, size_t bytes_x0, void* x0, BatchShape* out) {
  if (h->forced_shape.schedule >= 0) {
    if (int e = check_shape(h, h->forced_shape, fp32)) return e;
    *out = h->forced_shape;
    return BOGUS_GPU_OK;
  }
  if (h->batch_tuning) {
    BatchShape& t = h->tuned_shape[fp32 ? 1 : 0];
    if (t.schedule < 0) {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = g_tune_cache.find(tune_key(h, fp32));
      if (it != g_tune_cache.end()) t = it->second;
    }
    if (t.schedule < 0)
      if (int e = tune_shape(h, ba, fp32, bytes_x0, x0)) return e;
    *out = t;
    return BOGUS_GPU_OK;
  }
  *out = rule_shape(h, fp32);
  return BOGUS_GPU_OK;
}

PGBatchArgs batch_args64(bogus_gpu_problem* h, const bogus_gpu_pg_options* o) {
  const size_t n3 = 3 * (size_t)h->W.n;
  PGBatchArgs ba{};
  PGArgs& a = ba.base;
  a.rowptr = h->W.rowptr;
  a.col = h->col_local.p;
  a.val = h->W.val;
  a.b = h->b.p;
  a.mu = h->mu.p;
  a.scaling = h->scaling.p;
  a.X0 = h->X.p;
  a.X1 = h->X.p + n3;
  a.X2 = h->X.p + 2 * n3;
  a.MX0 = h->MX.p;
  a.MX1 = h->MX.p + n3;
  a.MX2 = h->MX.p + 2 * n3;
  a.MX3 = h->MX.p + 3 * n3;
  a.Y = h->Y.p;
  a.S0 = h->S0.p;
  a.XB = h->XB.p;
  a.Wv = h->Wv.p;
  a.csum = h->csum.p;
  a.out = h->batch_out.p;
  a.lin_momentum = lin_momentum(o);
  a.desaxce = o->static_problem ? 0 : 1;
  a.variant = o->variant;
  a.use_inf = o->use_infinity_norm ? 1 : 0;
  a.tol = o->tol;
  a.opt = o->ls_optimistic_factor;
  a.pess = o->ls_pessimistic_factor;
  a.max_iters = o->max_iters;
  a.ls_iters = o->ls_iters;
  ba.nproblems = h->nproblems;
  ba.contact_ptr = h->contact_ptr.p;
  ba.chunk_ptr = h->chunk_ptr.p;
  ba.queue = h->queue.p;
  ba.next = h->next.p;
  ba.r = h->X.p;  // each problem's best iterate is copied over its initial iterate
  return ba;
}

// Per-problem outputs and the solve statistics from the per-problem results.
int finish_batch(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, const PGOut* out, double* residuals,
                 unsigned* iters, bool hy = false) {
  const int np = h->nproblems;
  bool all = true;
  PGTraffic sum;
  unsigned maxit = 0;
  for (int p = 0; p < np; ++p) {
    if (residuals) residuals[p] = out[p].min_res;
    if (iters) iters[p] = out[p].iters;
    all = all && (out[p].converged || h->h_contact_ptr[p + 1] == h->h_contact_ptr[p]);
    const int np_c = h->h_contact_ptr[p + 1] - h->h_contact_ptr[p];
    PGTraffic t = pg_traffic(out[p], np_c, h->h_problem_nnz[p], o->variant, 8.0, lin_momentum(o) != 0 && !hy,
                             hy ? 4.0 : 0.0);
    if (hy) {  // the guess product and the refreshes read the FP64 values
      const double nnz = (double)h->h_problem_nnz[p];
      t.bytes += ((double)out[p].phases[1] + (double)out[p].hy_refreshes) * 36.0 * nnz;
      t.fma = 9.0 * nnz * (2.0 * out[p].phases[1] + out[p].hy_refreshes);
    }
    sum.bytes += t.bytes;
    sum.fma += t.fma;
    sum.passes += t.passes;
    if (out[p].iters > maxit) maxit = out[p].iters;
  }
  h->last_stats.iterations = maxit;
  h->last_stats.refine_iterations = 0;
  h->last_stats.fp32_device_ms = 0.0;
  h->last_stats.fp32_product_iterations = 0;
  h->last_stats.w_passes = sum.passes;
  h->last_stats.algorithmic_bytes = sum.bytes;
  h->last_stats.fp64_fma = sum.fma;
  return all ? BOGUS_GPU_OK : BOGUS_GPU_NOT_CONVERGED;
}

// hy: the FP64 iterations with FP32 correction products (the plain FP32 copy of W's values)
int run_pg_batch(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* residuals, unsigned* iters,
                 const HyArgs* hy = nullptr) {
  const int np = h->nproblems;
  PGBatchArgs ba = batch_args64(h, o);
  if (hy) {
    ba.base.hy_ival = hy->ival;
    ba.base.hy_d = hy->d;
    ba.base.hy_xref = hy->xref;
    ba.base.hy_wxref = hy->wxref;
    ba.base.hy_refresh = hy->refresh;
    ba.base.hy_stride = hy->stride;
    ba.base.lin_momentum = 0;
  }
  BatchShape sh;
  if (int e = choose_shape(h, ba, false, sizeof(double) * 3 * (size_t)h->W.n, h->X.p, &sh)) return e;
  if (int e = launch_shape(h, sh, &ba, nullptr, true)) return e;
  std::vector<PGOut> out(np);
  if (np) BG_CUDA(cudaMemcpyAsync(out.data(), h->batch_out.p, sizeof(PGOut) * np, cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  if (int e = read_status(h)) return e;
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->last_launches = 1;
  return finish_batch(h, o, out.data(), residuals, iters, hy != nullptr);
}

int batch_checks(bogus_gpu_problem* h, const bogus_gpu_pg_options* o) {
  if (int e = check_handle(h)) return e;
  if (int e = check_pg_options(o)) return e;
  if (o->variant == BOGUS_GPU_PG_STANDARD || o->variant == BOGUS_GPU_PG_CONJUGATED)
    return fail(BOGUS_GPU_BAD_INPUT, "batched solves run APGD, Descent or SPG");
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (h->nproblems == 0 && h->W.n > 0) return fail(BOGUS_GPU_NO_PROBLEM, "no batch partition set (bogus_gpu_set_batch)");

  if (int e = set_device(h)) return e;
  const int n = h->W.n;
  BG_CUDA(h->X.ensure(3 * 3 * (size_t)n));
  BG_CUDA(h->MX.ensure(4 * 3 * (size_t)n));
  BG_CUDA(h->Y.ensure(3 * (size_t)n));
  BG_CUDA(h->S0.ensure(n));
  BG_CUDA(h->XB.ensure(3 * (size_t)n));
  BG_CUDA(h->Wv.ensure(3 * (size_t)n));
  size_t tot_chunks = 0;
  for (int p = 0; p < h->nproblems; ++p) tot_chunks += (h->h_contact_ptr[p + 1] - h->h_contact_ptr[p] + 31) / 32;
  BG_CUDA(h->csum.ensure(4 * tot_chunks + 4));
  return BOGUS_GPU_OK;
}

}  // namespace



namespace {

// FP32-refined batched solve: every problem first runs up to max_iters FP32 iterations (one CTA per problem, W,
// iterates and per-contact law in FP32, reductions and decisions in FP64), then up to refine_max_iters FP64
// iterations from its FP32 result. Per-problem iteration counts add both parts; residuals are FP64.
int run_pg_batch_mixed(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* residuals, unsigned* iters) {
  const int n = h->W.n;
  const size_t n3 = 3 * (size_t)n;
  const int np = h->nproblems;
  cudaStream_t s = h->stream;
  BG_CUDA(h->X32.ensure(3 * n3));
  BG_CUDA(h->MX32.ensure(4 * n3));
  BG_CUDA(h->Y32.ensure(n3));
  BG_CUDA(h->S032.ensure(n));
  BG_CUDA(h->XB32.ensure(n3));
  BG_CUDA(h->Wv32.ensure(n3));
  if (!h->fp32p_valid) {
    BG_CUDA(h->val32p.ensure(9 * (size_t)h->W.nnzb));
    BG_CUDA(h->b32.ensure(n3));
    BG_CUDA(h->mu32.ensure(n));
    BG_CUDA(h->sc32.ensure(n));
    BG_CUDA(launch_convert(9 * (size_t)h->W.nnzb, h->W.val, h->val32p.p, s));
    BG_CUDA(launch_convert(n3, h->b.p, h->b32.p, s));
    BG_CUDA(launch_convert((size_t)n, h->mu.p, h->mu32.p, s));
    BG_CUDA(launch_convert((size_t)n, h->scaling.p, h->sc32.p, s));
    h->fp32p_valid = true;
    h->fp32_valid = false;  // b32 / mu32 / sc32 are shared with the interleaved FP32 copy: rebuild it when needed
  }
  PGBatchArgs32 ba{};
  PGArgs32& a = ba.base;
  a.rowptr = h->W.rowptr;
  a.col = h->col_local.p;
  a.val = h->val32p.p;
  a.b = h->b32.p;
  a.mu = h->mu32.p;
  a.scaling = h->sc32.p;
  a.X0 = h->X32.p;
  a.X1 = h->X32.p + n3;
  a.X2 = h->X32.p + 2 * n3;
  a.MX0 = h->MX32.p;
  a.MX1 = h->MX32.p + n3;
  a.MX2 = h->MX32.p + 2 * n3;
  a.MX3 = h->MX32.p + 3 * n3;
  a.Y = h->Y32.p;
  a.S0 = h->S032.p;
  a.XB = h->XB32.p;
  a.Wv = h->Wv32.p;
  a.csum = h->csum.p;
  a.out = h->batch_out.p;
  a.lin_momentum = 0;  // FP64 iterations only, as in run_pg_mixed
  a.desaxce = o->static_problem ? 0 : 1;
  a.variant = o->variant;
  a.use_inf = o->use_infinity_norm ? 1 : 0;
  a.tol = o->tol;
  a.opt = o->ls_optimistic_factor;
  a.pess = o->ls_pessimistic_factor;
  a.max_iters = o->max_iters;
  a.ls_iters = o->ls_iters;
  a.stall_iters = o->fp32_stall_iters;
  ba.nproblems = np;
  ba.contact_ptr = h->contact_ptr.p;
  ba.chunk_ptr = h->chunk_ptr.p;
  ba.queue = h->queue.p;
  ba.next = h->next.p;
  ba.r = h->X32.p;
  BG_CUDA(launch_convert(n3, h->X.p, h->X32.p, s));
  BatchShape sh;
  if (int e = choose_shape(h, ba, true, sizeof(float) * n3, h->X32.p, &sh)) return e;
  if (int e = launch_shape(h, sh, nullptr, &ba, true)) return e;
  std::vector<PGOut> out32(np);
  if (np) BG_CUDA(cudaMemcpyAsync(out32.data(), h->batch_out.p, sizeof(PGOut) * np, cudaMemcpyDeviceToHost, s));
  BG_CUDA(launch_convert(n3, h->X32.p, h->X.p, s));
  BG_CUDA(cudaStreamSynchronize(s));
  if (int e = read_status(h)) return e;
  float ms32 = 0.f;
  BG_CUDA(cudaEventElapsedTime(&ms32, h->ev0, h->ev1));
  bogus_gpu_pg_options o64 = *o;
  o64.max_iters = o->refine_max_iters;
  o64.mixed_precision = 0;
  o64.fp32_products_refresh = 0;
  // FP64 iterations with FP32 correction products, then the plain FP64 check from each problem's best iterate
  std::vector<unsigned> ith(np, 0u);
  unsigned maxh = 0;
  float msh = 0.f;
  bogus_gpu_solve_stats sth{};
  if (o->fp32_products_refresh) {
    BG_CUDA(h->hy_d.ensure(4 * n3));
    BG_CUDA(h->hy_xref.ensure(n3));
    BG_CUDA(h->hy_wxref.ensure(n3));
    const HyArgs hy{h->val32p.p, h->hy_d.p, h->hy_xref.p, h->hy_wxref.p, o->fp32_products_refresh, n3};
    std::vector<double> resh(np);
    bogus_gpu_pg_options oh = o64;
    oh.fp32_products_refresh = o->fp32_products_refresh;
    oh.mixed_precision = 1;
    const int hst = run_pg_batch(h, &oh, resh.data(), ith.data(), &hy);
    if (hst != BOGUS_GPU_OK && hst != BOGUS_GPU_NOT_CONVERGED) return hst;
    for (int p = 0; p < np; ++p) maxh = std::max(maxh, ith[p]);
    sth = h->last_stats;
    msh = h->last_ms;
    o64.max_iters = o->refine_max_iters > maxh ? o->refine_max_iters - maxh : 1u;
  }
  const int st = run_pg_batch(h, &o64, residuals, iters);
  if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
  unsigned maxit = 0;
  for (int p = 0; p < np; ++p) {
    if (iters) iters[p] += out32[p].iters + ith[p];
    maxit = std::max(maxit, out32[p].iters);
  }
  h->last_stats.refine_iterations = h->last_stats.iterations + maxh;
  h->last_stats.fp32_product_iterations = maxh;
  h->last_stats.iterations += maxit + maxh;
  h->last_stats.w_passes += sth.w_passes;
  h->last_stats.algorithmic_bytes += sth.algorithmic_bytes;
  h->last_stats.fp64_fma += sth.fp64_fma;
  h->last_stats.fp32_device_ms = ms32;
  h->last_ms += ms32 + msh;
  h->last_launches += o->fp32_products_refresh ? 2 : 1;
  return st;
}

}  // namespace

extern "C" {

int bogus_gpu_solve_pg_batch(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* r, double* residuals,
                             unsigned* iters) {
  if (int e = batch_checks(h, o)) return e;
  const size_t n3 = 3 * (size_t)h->W.n;
  if (n3 == 0) return BOGUS_GPU_OK;
  if (int e = check_finite(r, n3, "r")) return e;
  BG_CUDA(cudaMemcpyAsync(h->X.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream));
  const int st = o->mixed_precision ? run_pg_batch_mixed(h, o, residuals, iters) : run_pg_batch(h, o, residuals, iters);
  if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
  BG_CUDA(cudaMemcpyAsync(r, h->X.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return st;
}

int bogus_gpu_solve_pg_batch_device(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* d_r, double* residuals,
                                    unsigned* iters) {
  if (int e = batch_checks(h, o)) return e;
  const size_t n3 = 3 * (size_t)h->W.n;
  if (n3 == 0) return BOGUS_GPU_OK;
  BG_CUDA(cudaMemcpyAsync(h->X.p, d_r, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
  const int st = o->mixed_precision ? run_pg_batch_mixed(h, o, residuals, iters) : run_pg_batch(h, o, residuals, iters);
  if (st != BOGUS_GPU_OK && st != BOGUS_GPU_NOT_CONVERGED) return st;
  BG_CUDA(cudaMemcpyAsync(d_r, h->X.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return st;
}

int bogus_gpu_solve_pg_batch_graph(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* r, double* residuals,
                                   unsigned* iters) {
  if (int e = batch_checks(h, o)) return e;
  if (o->mixed_precision) return fail(BOGUS_GPU_BAD_INPUT, "the captured batched solve is FP64 only");
  const size_t n3 = 3 * (size_t)h->W.n;
  const int np = h->nproblems;
  if (n3 == 0) return BOGUS_GPU_OK;
  {
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, r) != cudaSuccess || attr.type != cudaMemoryTypeHost) {
      cudaGetLastError();
      return fail(BOGUS_GPU_BAD_INPUT, "r must be page-locked host memory (cudaHostAlloc or cudaHostRegister)");
    }
  }
  cudaStream_t s = h->stream;
  if (h->pinned_np < np) {
    if (h->pinned_out) cudaFreeHost(h->pinned_out);
    h->pinned_out = nullptr;
    h->pinned_np = 0;
    BG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&h->pinned_out), sizeof(PGOut) * np, cudaHostAllocDefault));
    h->pinned_np = np;
  }
  if (!h->pinned_status) BG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&h->pinned_status), sizeof(int), cudaHostAllocDefault));
  BG_CUDA(h->status.ensure(1));
  const PGBatchArgs ba = batch_args64(h, o);
  // the shape is chosen (and tuned, when enabled) before any capture: tuning synchronises and needs the starting
  // iterate on the device
  if (h->forced_shape.schedule < 0 && h->batch_tuning && h->tuned_shape[0].schedule < 0)
    BG_CUDA(cudaMemcpyAsync(h->X.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s));
  BatchShape sh;
  if (int e = choose_shape(h, ba, false, sizeof(double) * n3, h->X.p, &sh)) return e;
  PGTeamArgs ta{};
  int tgrid = 0;
  if (sh.schedule == 1)
    if (int e = team_setup(h, sh, &ta, &tgrid)) return e;
  const bool same = h->batch_graph && std::memcmp(&h->graph_args, &ba, sizeof(ba)) == 0 &&
                    std::memcmp(&h->graph_team, &ta, sizeof(ta)) == 0 && h->graph_shape == sh && h->graph_r == r;
  if (!same) {
    if (h->batch_graph) {
      cudaGraphExecDestroy(h->batch_graph);
      h->batch_graph = nullptr;
    }
    BG_CUDA(cudaStreamSynchronize(s));
    BG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int e = BOGUS_GPU_OK;
    {
      const cudaError_t c = cudaMemcpyAsync(h->X.p, r, sizeof(double) * n3, cudaMemcpyHostToDevice, s);
      if (c != cudaSuccess) e = fail(BOGUS_GPU_CUDA_ERROR, std::string("capture: ") + cudaGetErrorString(c));
    }
    if (!e) e = launch_shape(h, sh, &ba, nullptr, false);
    if (!e && np) {
      const cudaError_t c = cudaMemcpyAsync(h->pinned_out, h->batch_out.p, sizeof(PGOut) * np, cudaMemcpyDeviceToHost, s);
      if (c != cudaSuccess) e = fail(BOGUS_GPU_CUDA_ERROR, std::string("capture: ") + cudaGetErrorString(c));
    }
    if (!e) {
      cudaError_t c = cudaMemcpyAsync(h->pinned_status, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (c == cudaSuccess) c = cudaMemcpyAsync(r, h->X.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, s);
      if (c != cudaSuccess) e = fail(BOGUS_GPU_CUDA_ERROR, std::string("capture: ") + cudaGetErrorString(c));
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (e) {
      if (graph) cudaGraphDestroy(graph);
      return e;
    }
    if (ce != cudaSuccess) return fail(BOGUS_GPU_CUDA_ERROR, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    const cudaError_t ie = cudaGraphInstantiate(&h->batch_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      h->batch_graph = nullptr;
      return fail(BOGUS_GPU_CUDA_ERROR, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
    }
    h->graph_args = ba;
    h->graph_team = ta;
    h->graph_shape = sh;
    h->graph_r = r;
  }
  BG_CUDA(cudaEventRecord(h->ev0, s));
  BG_CUDA(cudaGraphLaunch(h->batch_graph, s));
  BG_CUDA(cudaEventRecord(h->ev1, s));
  BG_CUDA(cudaStreamSynchronize(s));
  if (*h->pinned_status != 0) return fail(*h->pinned_status, "device-side wait timed out in the batched solve");
  BG_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->last_launches = 1;
  h->last_shape = sh;
  return finish_batch(h, o, h->pinned_out, residuals, iters);
}

int bogus_gpu_set_batch_tuning(bogus_gpu_problem* h, int on) {
  if (int e = check_handle(h)) return e;
  h->batch_tuning = on != 0;
  return BOGUS_GPU_OK;
}

int bogus_gpu_set_batch_shape(bogus_gpu_problem* h, const bogus_gpu_batch_shape* shape) {
  if (int e = check_handle(h)) return e;
  if (!shape) {
    h->forced_shape = BatchShape{};
    return BOGUS_GPU_OK;
  }
  const BatchShape sh{shape->schedule, shape->ctas_per_sm, shape->team_size};
  if (int e = set_device(h)) return e;
  if (int e = check_shape(h, sh, false)) return e;
  if (int e = check_shape(h, sh, true)) return e;
  h->forced_shape = sh;
  return BOGUS_GPU_OK;
}

int bogus_gpu_get_batch_shape(const bogus_gpu_problem* h, bogus_gpu_batch_shape* shape) {
  if (int e = check_handle(h)) return e;
  if (!shape) return fail(BOGUS_GPU_BAD_INPUT, "null output");
  shape->schedule = h->last_shape.schedule;
  shape->ctas_per_sm = h->last_shape.ctas_per_sm;
  shape->team_size = h->last_shape.team_size;
  return BOGUS_GPU_OK;
}

int bogus_gpu_get_batch_tuning_log(const bogus_gpu_problem* h, bogus_gpu_batch_shape* shapes, double* ms, int* count) {
  if (int e = check_handle(h)) return e;
  if (!count) return fail(BOGUS_GPU_BAD_INPUT, "null output");
  const int k = (int)h->tune_ms.size();
  if (shapes || ms) {
    if (*count < k) return fail(BOGUS_GPU_BAD_INPUT, "output arrays too short");
    const std::vector<BatchShape>& cand = h->tune_cand;
    for (int i = 0; i < k && i < (int)cand.size(); ++i) {
      if (shapes) shapes[i] = bogus_gpu_batch_shape{cand[i].schedule, cand[i].ctas_per_sm, cand[i].team_size};
      if (ms) ms[i] = h->tune_ms[i];
    }
  }
  *count = k;
  return BOGUS_GPU_OK;
}

int bogus_gpu_get_dual_lower(bogus_gpu_problem* h, int* rowptr, int* colidx, double* blocks, int* nnzb_lower) {
  if (int e = check_handle(h)) return e;
  if (int e = ensure_host_lower(h)) return e;
  const HostBSR& l = h->host_lower;
  if (nnzb_lower) *nnzb_lower = l.nnzb();
  if (rowptr) std::memcpy(rowptr, l.rowptr.data(), sizeof(int) * (l.n + 1));
  if (colidx) std::memcpy(colidx, l.col.data(), sizeof(int) * l.nnzb());
  if (blocks) std::memcpy(blocks, l.val.data(), sizeof(double) * 9 * (size_t)l.nnzb());
  return BOGUS_GPU_OK;
}

int bogus_gpu_get_dual_rhs(bogus_gpu_problem* h, double* b, double* mu) {
  if (int e = check_handle(h)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  const int n = h->W.n;
  if (n == 0) return BOGUS_GPU_OK;
  if (int e = set_device(h)) return e;
  if (b) BG_CUDA(cudaMemcpyAsync(b, h->b.p, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
  if (mu) BG_CUDA(cudaMemcpyAsync(mu, h->mu.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return BOGUS_GPU_OK;
}

int bogus_gpu_get_solve_stats(const bogus_gpu_problem* h, bogus_gpu_solve_stats* out) {
  if (int e = check_handle(h)) return e;
  if (!out) return fail(BOGUS_GPU_BAD_INPUT, "null output");
  *out = h->last_stats;
  out->device_ms = h->last_ms;
  out->kernel_launches = h->last_launches;
  return BOGUS_GPU_OK;
}

int bogus_gpu_get_stream(const bogus_gpu_problem* h, void** stream) {
  if (int e = check_handle(h)) return e;
  if (!stream) return fail(BOGUS_GPU_BAD_INPUT, "null output");
  *stream = (void*)h->stream;
  return BOGUS_GPU_OK;
}

int bogus_gpu_set_wait_limit(int device, double seconds) {
  if (!(seconds >= 1e-6 && seconds <= 3600.0))
    return fail(BOGUS_GPU_BAD_INPUT, "wait limit must lie in [1e-6, 3600] seconds");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
    return fail(BOGUS_GPU_NO_DEVICE, "no such CUDA device");
  int prev = -1;
  BG_CUDA(cudaGetDevice(&prev));
  BG_CUDA(cudaSetDevice(device));
  const unsigned long long ns = (unsigned long long)(seconds * 1e9);
  cudaError_t e = set_wait_limit_pg(ns);
  if (e == cudaSuccess) e = set_wait_limit_gs(ns);
  if (e == cudaSuccess) e = set_wait_limit_admm(ns);
  if (e == cudaSuccess) e = set_wait_limit_adjoint(ns);
  cudaSetDevice(prev);
  if (e != cudaSuccess) return fail(BOGUS_GPU_CUDA_ERROR, std::string("setting the wait limit: ") + cudaGetErrorString(e));
  return BOGUS_GPU_OK;
}

int bogus_gpu_test_wait_timeout(bogus_gpu_problem* h, int on) {
  if (int e = check_handle(h)) return e;
  h->test_wait_timeout = on != 0;
  return BOGUS_GPU_OK;
}

int bogus_gpu_measure_fp64_peak(int device, double* tflops) {
  if (!tflops) return fail(BOGUS_GPU_BAD_INPUT, "null output");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
    return fail(BOGUS_GPU_NO_DEVICE, "no such CUDA device");
  BG_CUDA(measure_fp64_peak(device, tflops));
  return BOGUS_GPU_OK;
}

int bogus_gpu_check_fp64_ops(int device, long long n, unsigned long long seed, long long* mismatches) {
  if (!mismatches || n < 0) return fail(BOGUS_GPU_BAD_INPUT, "null output or negative count");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
    return fail(BOGUS_GPU_NO_DEVICE, "no such CUDA device");
  BG_CUDA(check_fp64_ops(device, n, seed, mismatches));
  return BOGUS_GPU_OK;
}

// ---- contact permutation (DualFrictionProblem::applyPermutation / undoPermutation, FrictionProblem.cpp:102-125)
// The stored problem becomes W' = P W P^T, b' = P b, mu' = P mu with contact k of the stored problem being
// contact perm[k] of the caller's (the layout of SparseBlockMatrixBase::applyPermutation: blocks moved above the
// diagonal are stored transposed in the lower triangle). While permuted, the solves and the error evaluation
// take and return r in the caller's order (FrictionProblem.impl.hpp:38-91).
namespace {
int permute_stored(bogus_gpu_problem* h, const std::vector<int>& p) {
  if (int e = ensure_host_lower(h)) return e;
  const int n = h->W.n;
  const HostBSR plow = permute_lower(h->host_lower, p);
  std::vector<double> pb(3 * (size_t)n), pmu(n);
  for (int k = 0; k < n; ++k) {
    for (int c = 0; c < 3; ++c) pb[3 * (size_t)k + c] = h->host_b[3 * (size_t)p[k] + c];
    pmu[k] = h->host_mu[p[k]];
  }
  return set_dual_lower(h, n, plow.rowptr.data(), plow.col.data(), plow.val.data(), pb.data(), pmu.data());
}

// r (3 n, caller's order) <-> the stored order
void to_stored(const bogus_gpu_problem* h, const double* r, double* out) {
  const int n = h->W.n;
  for (int k = 0; k < n; ++k)
    for (int c = 0; c < 3; ++c) out[3 * (size_t)k + c] = r[3 * (size_t)h->perm[k] + c];
}
void from_stored(const bogus_gpu_problem* h, const double* in, double* r) {
  const int n = h->W.n;
  for (int k = 0; k < n; ++k)
    for (int c = 0; c < 3; ++c) r[3 * (size_t)h->perm[k] + c] = in[3 * (size_t)k + c];
}
bool solved(int st) { return st == BOGUS_GPU_OK || st == BOGUS_GPU_NOT_CONVERGED; }
}  // namespace

int bogus_gpu_apply_permutation(bogus_gpu_problem* h, const int* perm) {
  if (int e = check_handle(h)) return e;
  if (!h->has_dual) return fail(BOGUS_GPU_NO_PROBLEM, "no dual problem set");
  if (h->permuted) return fail(BOGUS_GPU_BAD_INPUT, "the problem is already permuted (undo the permutation first)");
  const int n = h->W.n;
  if (n > 0 && !perm) return fail(BOGUS_GPU_BAD_INPUT, "null permutation");
  std::vector<int> p(perm, perm + n), inv(n, -1);
  for (int k = 0; k < n; ++k) {
    if (p[k] < 0 || p[k] >= n || inv[p[k]] >= 0) return fail(BOGUS_GPU_BAD_INPUT, "not a permutation of the contacts");
    inv[p[k]] = k;
  }
  if (int e = permute_stored(h, p)) return e;
  h->permuted = true;
  h->perm = std::move(p);
  h->inv_perm = std::move(inv);
  BG_CUDA(h->d_perm.ensure(n > 0 ? n : 1));
  if (n) BG_CUDA(cudaMemcpyAsync(h->d_perm.p, h->perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->stream));
  BG_CUDA(cudaStreamSynchronize(h->stream));
  return BOGUS_GPU_OK;
}

int bogus_gpu_undo_permutation(bogus_gpu_problem* h) {
  if (int e = check_handle(h)) return e;
  if (!h->permuted) return BOGUS_GPU_OK;
  if (int e = permute_stored(h, h->inv_perm)) return e;
  h->permuted = false;
  h->perm.clear();
  h->inv_perm.clear();
  return BOGUS_GPU_OK;
}

int bogus_gpu_permuted(const bogus_gpu_problem* h, int* permuted) {
  if (int e = check_handle(h)) return e;
  if (!permuted) return fail(BOGUS_GPU_BAD_INPUT, "null output");
  *permuted = h->permuted ? 1 : 0;
  return BOGUS_GPU_OK;
}

int bogus_gpu_eval(bogus_gpu_problem* h, const double* r, int static_problem, int use_inf, double* residual) {
  if (!h || !h->permuted || !r) return eval_stored(h, r, static_problem, use_inf, residual);
  std::vector<double> rs(3 * (size_t)h->W.n);
  to_stored(h, r, rs.data());
  return eval_stored(h, rs.data(), static_problem, use_inf, residual);
}

int bogus_gpu_solve_pg(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* r, double* residual,
                       unsigned* iters) {
  if (!h || !h->permuted || !r) return solve_pg_stored(h, o, r, residual, iters);
  std::vector<double> rs(3 * (size_t)h->W.n);
  to_stored(h, r, rs.data());
  const int st = solve_pg_stored(h, o, rs.data(), residual, iters);
  if (solved(st)) from_stored(h, rs.data(), r);
  return st;
}

int bogus_gpu_solve_gs(bogus_gpu_problem* h, const bogus_gpu_gs_options* o, double* r, double* residual,
                       unsigned* iters) {
  if (!h || !h->permuted || !r) return solve_gs_stored(h, o, r, residual, iters);
  std::vector<double> rs(3 * (size_t)h->W.n);
  to_stored(h, r, rs.data());
  const int st = solve_gs_stored(h, o, rs.data(), residual, iters);
  if (solved(st)) from_stored(h, rs.data(), r);
  return st;
}

int bogus_gpu_solve_cadoux_gs(bogus_gpu_problem* h, const bogus_gpu_gs_options* o, double* r, unsigned cadoux_iters,
                              double* residual, unsigned* iters) {
  if (!h || !h->permuted || !r) return solve_cadoux_gs_stored(h, o, r, cadoux_iters, residual, iters);
  std::vector<double> rs(3 * (size_t)h->W.n);
  to_stored(h, r, rs.data());
  const int st = solve_cadoux_gs_stored(h, o, rs.data(), cadoux_iters, residual, iters);
  if (solved(st)) from_stored(h, rs.data(), r);
  return st;
}

int bogus_gpu_solve_cadoux_pg(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* r, unsigned cadoux_iters,
                              double* residual, unsigned* iters) {
  if (!h || !h->permuted || !r) return solve_cadoux_pg_stored(h, o, r, cadoux_iters, residual, iters);
  std::vector<double> rs(3 * (size_t)h->W.n);
  to_stored(h, r, rs.data());
  const int st = solve_cadoux_pg_stored(h, o, rs.data(), cadoux_iters, residual, iters);
  if (solved(st)) from_stored(h, rs.data(), r);
  return st;
}

int bogus_gpu_solve_pg_device(bogus_gpu_problem* h, const bogus_gpu_pg_options* o, double* d_r, double* residual,
                              unsigned* iters) {
  if (!h || !h->permuted || !d_r) return solve_pg_device_stored(h, o, d_r, residual, iters);
  const int n = h->W.n;
  BG_CUDA(h->perm_r.ensure(3 * (size_t)(n > 0 ? n : 1)));
  BG_CUDA(launch_permute3(n, h->d_perm.p, d_r, h->perm_r.p, false, h->stream));
  const int st = solve_pg_device_stored(h, o, h->perm_r.p, residual, iters);
  if (solved(st)) {
    BG_CUDA(launch_permute3(n, h->d_perm.p, h->perm_r.p, d_r, true, h->stream));
    BG_CUDA(cudaStreamSynchronize(h->stream));
  }
  return st;
}

}  // extern "C"
