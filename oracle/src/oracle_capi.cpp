// ORACLE — test infrastructure only (see oracle_math.hpp). C entry points for the Python tests and for
// the CPU-baseline leg of bench.py (ctypes). Mirrors the reference's dual-problem calls:
// DualFrictionProblem::solveWith / evalWith (Interfaces/FrictionProblem.cpp:42-66), including the
// coloring + permutation wiring of MecheFrictionProblem::solve (Interfaces/MecheInterface.cpp:326-337).
#include <cstring>
#include <memory>
#include <vector>

#include "oracle_fp32.hpp"
#include "oracle_math.hpp"
#include "oracle_meche.hpp"
#include "oracle_solvers.hpp"
#include "oracle_sparse.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace oracle;

namespace {

struct DualProblem {
  BSR low;   // stored lower triangle, as given
  BSR full;  // both triangles
  std::vector<double> b, mu;
};

typedef void (*oracle_callback)(unsigned, double, void*);

Callback wrap(oracle_callback cb, void* user) {
  if (!cb) return Callback();
  return [cb, user](unsigned it, double r) { cb(it, r, user); };
}

BSR makeBSR(int n, const int* rowptr, const int* col, const double* val) {
  BSR m;
  m.n = n;
  m.rowptr.assign(rowptr, rowptr + n + 1);
  const int nnz = rowptr[n];
  m.col.assign(col, col + nnz);
  m.val.assign(val, val + 9 * (size_t)nnz);
  return m;
}

}  // namespace

extern "C" {

int oracle_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Threads of the colored Gauss-Seidel sweeps that follow (1, the default: the sequential sweep the parity
// tests compare against; more: the reference's per-color OpenMP loop, for CPU timing only).
static int g_gs_threads = 1;
void oracle_set_gs_threads(int t) { g_gs_threads = t > 1 ? t : 1; }
// Wall time (ms) of the sweeps and evaluations of the last Gauss-Seidel solve, without its setup.
static double g_gs_sweep_ms = 0.0;
double oracle_last_gs_sweep_ms() { return g_gs_sweep_ms; }

void oracle_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

void* oracle_dual_create(int n, const int* rowptr, const int* col, const double* val, const double* b,
                         const double* mu) {
  auto* p = new DualProblem;
  p->low = makeBSR(n, rowptr, col, val);
  p->full = expandSymmetric(p->low);
  p->b.assign(b, b + 3 * (size_t)n);
  p->mu.assign(mu, mu + n);
  return p;
}

void oracle_dual_destroy(void* h) { delete static_cast<DualProblem*>(h); }

int oracle_dual_nnz_full(void* h) { return static_cast<DualProblem*>(h)->full.nnzb(); }

void oracle_dual_full(void* h, int* rowptr, int* col, double* val) {
  const BSR& f = static_cast<DualProblem*>(h)->full;
  std::memcpy(rowptr, f.rowptr.data(), sizeof(int) * (f.n + 1));
  std::memcpy(col, f.col.data(), sizeof(int) * f.nnzb());
  std::memcpy(val, f.val.data(), sizeof(double) * 9 * (size_t)f.nnzb());
}

// y = W x (init null) or y = init + W x
void oracle_dual_spmv(void* h, const double* x, double* y, const double* init) {
  spmv(static_cast<DualProblem*>(h)->full, x, y, init);
}

void oracle_dual_split_row(void* h, int row, const double* x, double* res) {
  splitRowMultiply(static_cast<DualProblem*>(h)->full, row, x, res);
}

// evalWith (FrictionProblem.impl.hpp:58-74): u = W r + b, scalings of the solver's matrix
double oracle_dual_eval(void* h, int desaxce, const double* r, int useInfinityNorm) {
  auto* p = static_cast<DualProblem*>(h);
  SolverBase s;
  s.setMatrix(p->full);
  s.useInfinityNorm = useInfinityNorm != 0;
  std::vector<double> u(p->b.size());
  spmv(p->full, r, u.data());
  for (size_t k = 0; k < u.size(); ++k) u[k] = u[k] + p->b[k];
  Law law{desaxce != 0, RevHybrid, p->mu.data()};
  return s.eval(law, u.data(), r);
}

double oracle_dual_solve_pg(void* h, int variant, int desaxce, double tol, unsigned maxIters, unsigned lsIters,
                            double optimistic, double pessimistic, double armijo, int useInfinityNorm, int linMomentum,
                            unsigned hyRefresh, double* r, unsigned* iters, oracle_callback cb, void* user) {
  auto* p = static_cast<DualProblem*>(h);
  ProjectedGradient pg;
  pg.setMatrix(p->full);
  pg.variant = variant;
  pg.linMomentum = linMomentum != 0;
  pg.hyRefresh = hyRefresh;
  pg.tol = tol;
  pg.maxIters = maxIters;
  pg.lsIters = lsIters;
  pg.lsOptimisticFactor = optimistic;
  pg.lsPessimisticFactor = pessimistic;
  pg.lsArmijoCoefficient = armijo;
  pg.useInfinityNorm = useInfinityNorm != 0;
  pg.callback = wrap(cb, user);
  Law law{desaxce != 0, RevHybrid, p->mu.data()};
  return pg.solve(law, p->b.data(), r, iters);
}

// The FP32 part of the FP32-refined solve (APGD when apgd, else Descent): r is rounded to float, solved in
// single precision with the stall test, and the best iterate is written back widened to double.
double oracle_dual_solve_pg_fp32(void* h, int apgd, int desaxce, double tol, unsigned maxIters, unsigned lsIters,
                                 double optimistic, double pessimistic, int useInfinityNorm, unsigned stallIters,
                                 double* r, unsigned* iters) {
  auto* p = static_cast<DualProblem*>(h);
  ProjectedGradient pg;
  pg.setMatrix(p->full);
  pg.tol = tol;
  pg.maxIters = maxIters;
  pg.lsIters = lsIters;
  pg.lsOptimisticFactor = optimistic;
  pg.lsPessimisticFactor = pessimistic;
  pg.useInfinityNorm = useInfinityNorm != 0;
  const size_t n3 = 3 * (size_t)p->full.n;
  std::vector<float> x(n3);
  for (size_t k = 0; k < n3; ++k) x[k] = (float)r[k];
  const double res = fp32::solveAPGD32(pg, p->full, desaxce != 0, p->mu.data(), p->b.data(), x.data(), apgd != 0,
                                       stallIters, iters);
  for (size_t k = 0; k < n3; ++k) r[k] = (double)x[k];
  return res;
}

// Greedy coloring of the stored lower triangle; returns the number of colors (perm: n, colors: ncolors+1).
int oracle_dual_coloring(void* h, int* perm, int* colors) {
  auto* p = static_cast<DualProblem*>(h);
  std::vector<int> pm, cl;
  greedyColoring(p->low, pm, cl);
  std::memcpy(perm, pm.data(), sizeof(int) * pm.size());
  std::memcpy(colors, cl.data(), sizeof(int) * cl.size());
  return (int)cl.size() - 1;
}

// GaussSeidel through solveWith: with use_coloring the problem is permuted so that colors are contiguous
// (applyPermutation), solved color by color, and r is permuted back.
double oracle_dual_solve_gs(void* h, int desaxce, int strat, double tol, unsigned maxIters, unsigned evalEvery,
                            double skipTol, unsigned skipIters, double autoReg, int tryZero, int useInfinityNorm,
                            int useColoring, double* r, unsigned* iters, oracle_callback cb, void* user) {
  auto* p = static_cast<DualProblem*>(h);
  const int n = p->low.n;
  GaussSeidel gs;
  gs.tol = tol;
  gs.maxIters = maxIters;
  gs.evalEvery = evalEvery;
  gs.skipTol = skipTol;
  gs.skipIters = skipIters;
  gs.autoRegularization = autoReg;
  gs.tryZeroAsWell = tryZero != 0;
  gs.useInfinityNorm = useInfinityNorm != 0;
  gs.callback = wrap(cb, user);
  gs.threads = g_gs_threads;
  if (!useColoring) {
    gs.setMatrix(p->full);
    Law law{desaxce != 0, strat, p->mu.data()};
    const double res = gs.solve(law, p->b.data(), r, iters);
    g_gs_sweep_ms = gs.sweepSeconds * 1e3;
    return res;
  }
  std::vector<int> perm, colors;
  greedyColoring(p->low, perm, colors);
  const BSR plow = permuteSymmetric(p->low, perm);
  const BSR pfull = expandSymmetric(plow);
  const std::vector<double> pb = permuteSegments(p->b, perm, 3);
  const std::vector<double> pmu = permuteSegments(p->mu, perm, 1);
  std::vector<double> rv(r, r + 3 * (size_t)n);
  std::vector<double> pr = permuteSegments(rv, perm, 3);
  gs.perm.resize(n);
  for (int i = 0; i < n; ++i) gs.perm[i] = i;
  gs.colors = colors;
  gs.setMatrix(pfull);
  Law law{desaxce != 0, strat, pmu.data()};
  const double res = gs.solve(law, pb.data(), pr.data(), iters);
  g_gs_sweep_ms = gs.sweepSeconds * 1e3;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) r[3 * (size_t)perm[i] + k] = pr[3 * (size_t)i + k];
  return res;
}

// DualFrictionProblem::solveCadoux (Interfaces/FrictionProblem.impl.hpp:76-92) with a GaussSeidel minimizer
// (the coloring permutation applied around the whole fixed point, as the reference does for a permuted problem).
double oracle_dual_solve_cadoux_gs(void* h, int strat, double tol, unsigned maxIters, unsigned evalEvery,
                                   double skipTol, unsigned skipIters, double autoReg, int tryZero,
                                   int useInfinityNorm, int useColoring, unsigned cadouxIters, double* r,
                                   unsigned* iters, oracle_callback cb, void* user) {
  auto* p = static_cast<DualProblem*>(h);
  const int n = p->low.n;
  GaussSeidel gs;
  gs.tol = tol;
  gs.maxIters = maxIters;
  gs.evalEvery = evalEvery;
  gs.skipTol = skipTol;
  gs.skipIters = skipIters;
  gs.autoRegularization = autoReg;
  gs.tryZeroAsWell = tryZero != 0;
  gs.useInfinityNorm = useInfinityNorm != 0;
  std::vector<int> perm(n), colors{0, n};
  for (int i = 0; i < n; ++i) perm[i] = i;
  if (useColoring) greedyColoring(p->low, perm, colors);
  const BSR plow = permuteSymmetric(p->low, perm);
  const BSR pfull = expandSymmetric(plow);
  const std::vector<double> pb = permuteSegments(p->b, perm, 3);
  const std::vector<double> pmu = permuteSegments(p->mu, perm, 1);
  std::vector<double> rv(r, r + 3 * (size_t)n);
  std::vector<double> pr = permuteSegments(rv, perm, 3);
  gs.perm.resize(n);
  for (int i = 0; i < n; ++i) gs.perm[i] = i;
  gs.colors = colors;
  gs.setMatrix(pfull);
  const double res = solveCadoux(gs, pfull, pb.data(), pmu.data(), strat, pr.data(), cadouxIters, wrap(cb, user), iters);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) r[3 * (size_t)perm[i] + k] = pr[3 * (size_t)i + k];
  return res;
}

// DualFrictionProblem::solveCadoux with a ProjectedGradient minimizer.
double oracle_dual_solve_cadoux_pg(void* h, int variant, double tol, unsigned maxIters, unsigned lsIters,
                                   double optimistic, double pessimistic, double armijo, int useInfinityNorm,
                                   unsigned cadouxIters, double* r, unsigned* iters, oracle_callback cb, void* user) {
  auto* p = static_cast<DualProblem*>(h);
  ProjectedGradient pg;
  pg.setMatrix(p->full);
  pg.variant = variant;
  pg.tol = tol;
  pg.maxIters = maxIters;
  pg.lsIters = lsIters;
  pg.lsOptimisticFactor = optimistic;
  pg.lsPessimisticFactor = pessimistic;
  pg.lsArmijoCoefficient = armijo;
  pg.useInfinityNorm = useInfinityNorm != 0;
  return solveCadoux(pg, p->full, p->b.data(), p->mu.data(), RevHybrid, r, cadouxIters, wrap(cb, user), iters);
}

// ---- MecheFrictionProblem (Interfaces/MecheInterface.cpp) -------------------------------------------
// mass: the bodies' column-major blocks one after the other; HA / HB: the contacts' column-major 3 x ndof blocks
// one after the other (HB: none for objB == -1, 3 x ndof[objA] when objB == objA). Returns null on a singular
// mass block.
void* oracle_meche_create(int nobj, const unsigned* ndof, const double* mass, const double* f, int n,
                          const double* mu, const double* E, const double* w, const int* objA, const int* objB,
                          const double* HA, const double* HB) {
  std::vector<const double*> mp(nobj), hap(n), hbp(n);
  size_t off = 0;
  for (int k = 0; k < nobj; ++k) {
    mp[k] = mass + off;
    off += (size_t)ndof[k] * ndof[k];
  }
  size_t oa = 0, ob = 0;
  for (int i = 0; i < n; ++i) {
    hap[i] = HA + oa;
    oa += 3 * (size_t)ndof[objA[i]];
    hbp[i] = HB + ob;
    if (objB[i] >= 0) ob += 3 * (size_t)ndof[objB[i] == objA[i] ? objA[i] : objB[i]];
  }
  auto* m = new Meche();
  if (!mecheFromPrimal(*m, nobj, ndof, mp.data(), f, n, mu, E, w, objA, objB, hap.data(), hbp.data())) {
    delete m;
    return nullptr;
  }
  return m;
}
void oracle_meche_destroy(void* h) { delete static_cast<Meche*>(h); }

// y = E^T x per contact (E: n x 3 x 3 row-major), the frame chain of the facade (oracle_meche.hpp: frameT)
void oracle_frame_t(int n, const double* E, const double* x, double* y) {
  for (int i = 0; i < n; ++i) frameT(E + 9 * (size_t)i, x + 3 * (size_t)i, y + 3 * (size_t)i);
}

// MecheFrictionProblem::solve(r, v, options, staticProblem, problemRegularization) (:226-367); algorithm 0 GS,
// 1 PG, 2 matrix-free GS, 3 ADMM, 4 DualAMA. v: unpadded (sum of ndof), may be null. Returns the solver's
// residual.
double oracle_meche_solve(void* h, double* r, double* v, int maxThreads, unsigned maxIters, unsigned cadouxIters,
                          double tolerance, int useInfinityNorm, int algorithm, double gsRegularization,
                          int gsColoring, int gsSkipIters, int tryZeroAsWell, int pgVariant, double admmProjStepSize,
                          double admmFpStepSize, int staticProblem, double problemRegularization, oracle_callback cb,
                          void* user) {
  auto* m = static_cast<Meche*>(h);
  const Primal& P = m->P;
  const int n = P.ncontacts, d = P.ndof;
  const size_t n3 = 3 * (size_t)n, md = (size_t)P.nbodies * d;
  std::vector<double> rl(n3), wl(n3);
  for (int i = 0; i < n; ++i) {
    frameT(&m->E[9 * (size_t)i], r + 3 * i, &rl[3 * (size_t)i]);
    frameT(&m->E[9 * (size_t)i], &m->w[3 * (size_t)i], &wl[3 * (size_t)i]);
  }
  std::vector<double> vp(md, 0.0);
  double res = -1;
  const Callback callback = wrap(cb, user);
  if (algorithm == 3 || algorithm == 4) {
    // v given (unpadded) or M^-1 (H^T r - f)
    if (v) {
      size_t off = 0;
      for (int k = 0; k < P.nbodies; ++k) {
        for (int a = 0; a < m->ndof[k]; ++a) vp[(size_t)k * d + a] = v[off + a];
        off += m->ndof[k];
      }
    } else {
      mecheVelocity(*m, rl.data(), vp.data());
    }
    ADMMSolver s;
    s.P = &P;
    s.setScalings(m->ndof);
    if (algorithm == 4) {
      // MecheInterface.cpp:249-261: DualAMA without line search, the facade's step sizes
      DualAMASolver dama;
      dama.P = &P;
      if (tolerance != 0.) dama.tol = tolerance;
      if (maxIters != 0) dama.maxIters = maxIters;
      dama.useInfinityNorm = useInfinityNorm != 0;
      dama.lsIters = 0;
      dama.fpStepSize = admmFpStepSize;
      dama.projStepSize = admmProjStepSize;
      dama.callback = callback;
      dama.scalings = s.scalings;
      dama.mTrue = 0;
      for (int k : m->ndof) dama.mTrue += k;
      res = dama.solve(m->mu.data(), staticProblem == 0, m->mass, m->f.data(), wl.data(), vp.data(), rl.data());
    } else {
      s.stepSize = admmProjStepSize;
      if (tolerance != 0.) s.tol = tolerance;
      if (maxIters != 0) s.maxIters = maxIters;
      s.useInfinityNorm = useInfinityNorm != 0;
      s.callback = callback;
      std::vector<double> invMu(n);
      for (int i = 0; i < n; ++i) invMu[i] = 1. / m->mu[i];
      res = s.solve(invMu.data(), P.minv, 0., m->f.data(), wl.data(), vp.data(), rl.data());
    }
  } else if (algorithm == 2) {
    // PrimalFrictionProblem::solveWith(ProductGaussSeidelType&, r_loc, staticProblem)
    ProductGaussSeidel gs;
    if (tolerance != 0.) gs.tol = tolerance;
    if (maxIters != 0) gs.maxIters = maxIters;
    if (gsSkipIters >= 0) gs.skipIters = (unsigned)gsSkipIters;
    gs.useInfinityNorm = useInfinityNorm != 0;
    gs.autoRegularization = gsRegularization;
    gs.tryZeroAsWell = tryZeroAsWell != 0;
    gs.callback = callback;
    gs.setPrimal(P);
    const std::vector<double> b = assembleB(P, m->f.data(), wl.data());
    Law law{staticProblem == 0, RevHybrid, m->mu.data()};
    res = gs.solve(law, b.data(), rl.data());
    if (v) mecheVelocity(*m, rl.data(), vp.data());
  } else {
    if (!m->hasDual) {
      m->low = assembleW(P);
      if (problemRegularization > 0.)
        for (int i = 0; i < n; ++i) {
          double* B = &m->low.val[9 * (size_t)(m->low.rowptr[i + 1] - 1)];
          B[0] = B[0] + problemRegularization;
          B[4] = B[4] + problemRegularization;
          B[8] = B[8] + problemRegularization;
        }
      m->full = expandSymmetric(m->low);
      m->b = assembleB(P, m->f.data(), wl.data());
      m->hasDual = true;
    }
    const bool cadoux = !staticProblem && cadouxIters > 0;
    if (algorithm == 1) {
      ProjectedGradient pg;
      pg.setMatrix(m->full);
      if (tolerance != 0.) pg.tol = tolerance;
      if (maxIters != 0) pg.maxIters = maxIters;
      pg.useInfinityNorm = useInfinityNorm != 0;
      pg.variant = pgVariant;
      if (!cadoux) {
        pg.callback = callback;
        Law law{staticProblem == 0, RevHybrid, m->mu.data()};
        res = pg.solve(law, m->b.data(), rl.data());
      } else {
        res = solveCadoux(pg, m->full, m->b.data(), m->mu.data(), RevHybrid, rl.data(), cadouxIters, callback);
      }
    } else {
      GaussSeidel gs;
      if (tolerance != 0.) gs.tol = tolerance;
      if (maxIters != 0) gs.maxIters = maxIters;
      if (gsSkipIters >= 0) gs.skipIters = (unsigned)gsSkipIters;
      gs.autoRegularization = gsRegularization;
      gs.useInfinityNorm = useInfinityNorm != 0;
      const bool useColoring = maxThreads != 1 && gsColoring;
      std::vector<int> perm(n), colors{0, n};
      for (int i = 0; i < n; ++i) perm[i] = i;
      if (useColoring) greedyColoring(m->low, perm, colors);
      const BSR plow = permuteSymmetric(m->low, perm);
      const BSR pfull = expandSymmetric(plow);
      const std::vector<double> pb = permuteSegments(m->b, perm, 3);
      const std::vector<double> pmu = permuteSegments(m->mu, perm, 1);
      std::vector<double> pr = permuteSegments(rl, perm, 3);
      gs.perm.resize(n);
      for (int i = 0; i < n; ++i) gs.perm[i] = i;
      gs.colors = colors;
      gs.setMatrix(pfull);
      if (!cadoux) {
        gs.tryZeroAsWell = tryZeroAsWell != 0;
        gs.callback = callback;
        Law law{staticProblem == 0, RevHybrid, pmu.data()};
        res = gs.solve(law, pb.data(), pr.data());
      } else {
        gs.tryZeroAsWell = false;
        res = solveCadoux(gs, pfull, pb.data(), pmu.data(), RevHybrid, pr.data(), cadouxIters, callback);
      }
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) rl[3 * (size_t)perm[i] + k] = pr[3 * (size_t)i + k];
    }
    if (v) mecheVelocity(*m, rl.data(), vp.data());
  }
  if (v) {
    size_t off = 0;
    for (int k = 0; k < P.nbodies; ++k) {
      for (int a = 0; a < m->ndof[k]; ++a) v[off + a] = vp[(size_t)k * d + a];
      off += m->ndof[k];
    }
  }
  for (int i = 0; i < n; ++i) frame(&m->E[9 * (size_t)i], &rl[3 * (size_t)i], r + 3 * i);
  return res;
}

// ---- per-contact mathematics -------------------------------------------------------------------
double oracle_local_solve(int desaxce, int strat, const double* A, const double* b, double* x, double mu, double tol,
                          double scaling) {
  return localSolve(desaxce != 0, strat, A, b, x, mu, tol, scaling);
}

int oracle_law_solve_local(int desaxce, int strat, const double* A, const double* b, double* x, double mu,
                           double scaling) {
  return lawSolveLocal(desaxce != 0, strat, A, b, x, mu, scaling) ? 1 : 0;
}

// coeffs: dim entries (monic, degenerate == 0) or dim + 1 entries (degenerate != 0; copied first)
int oracle_real_roots(const double* coeffs, int dim, int degenerate, int filter, double* roots) {
  double c[8];
  for (int k = 0; k < dim + (degenerate ? 1 : 0); ++k) c[k] = coeffs[k];
  if (degenerate) return realRootsDegenerate(c, dim, roots, (RootsFilter)filter);
  return realRootsMonic(c, dim, roots, (RootsFilter)filter);
}

void oracle_project(double mu, double* x) { projectCone(mu, x); }

double oracle_law_eval(int desaxce, double mu, const double* x, const double* y) {
  return lawEval(desaxce != 0, mu, x, y);
}

void oracle_fb_jacobian(int desaxce, double mu, double scaling, const double* A, const double* b, const double* x,
                        double* fb, double* dFdx) {
  LocalFB f{desaxce != 0, mu, scaling, A, b};
  f.computeJacobian(x, fb, dFdx);
}

double oracle_canonical_sum(const double* v, size_t n) { return canonicalSum(v, n); }

// ---- primal problem / Delassus assembly ---------------------------------------------------------
void* oracle_primal_create(int nbodies, int ndof, const double* minv, int ncontacts, const int* objA, const int* objB,
                           const double* HA, const double* HB) {
  auto* P = new Primal;
  P->nbodies = nbodies;
  P->ndof = ndof;
  P->ncontacts = ncontacts;
  P->minv.assign(minv, minv + (size_t)nbodies * ndof * ndof);
  P->objA.assign(objA, objA + ncontacts);
  P->objB.assign(objB, objB + ncontacts);
  P->HA.assign(HA, HA + (size_t)ncontacts * 3 * ndof);
  P->HB.assign(HB, HB + (size_t)ncontacts * 3 * ndof);
  return P;
}

void oracle_primal_destroy(void* h) { delete static_cast<Primal*>(h); }

// Assembles the lower triangle of W; returns nnzb. Call with null outputs first to size them.
int oracle_primal_assemble(void* h, int* rowptr, int* col, double* val) {
  const BSR W = assembleW(*static_cast<Primal*>(h));
  if (rowptr) std::memcpy(rowptr, W.rowptr.data(), sizeof(int) * (W.n + 1));
  if (col) std::memcpy(col, W.col.data(), sizeof(int) * W.nnzb());
  if (val) std::memcpy(val, W.val.data(), sizeof(double) * 9 * (size_t)W.nnzb());
  return W.nnzb();
}

void oracle_primal_rhs(void* h, const double* f, const double* w, double* b) {
  const std::vector<double> bb = assembleB(*static_cast<Primal*>(h), f, w);
  std::memcpy(b, bb.data(), sizeof(double) * bb.size());
}

// PrimalFrictionProblem::solveWith(ProductGaussSeidelType&, r, staticProblem): b = w - H M^-1 f, then the
// matrix-free Gauss-Seidel (desaxce: the Coulomb law, else SOC).
double oracle_primal_solve_product_gs(void* h, const double* f, const double* w, const double* mu, int desaxce,
                                      int strat, double tol, unsigned maxIters, unsigned evalEvery, double skipTol,
                                      unsigned skipIters, double autoReg, int tryZero, int useInfinityNorm, double* r,
                                      unsigned* iters, oracle_callback cb, void* user) {
  auto* P = static_cast<Primal*>(h);
  const std::vector<double> b = assembleB(*P, f, w);
  ProductGaussSeidel gs;
  gs.tol = tol;
  gs.maxIters = maxIters;
  gs.evalEvery = evalEvery;
  gs.skipTol = skipTol;
  gs.skipIters = skipIters;
  gs.autoRegularization = autoReg;
  gs.tryZeroAsWell = tryZero != 0;
  gs.useInfinityNorm = useInfinityNorm != 0;
  gs.callback = wrap(cb, user);
  gs.setPrimal(*P);
  Law law{desaxce != 0, strat, mu};
  return gs.solve(law, b.data(), r, iters);
}

// PrimalFrictionProblem::solveWith(DualAMAType&, v, r, staticProblem): mass blocks M (nbodies x d x d),
// trueDofs: the bodies' own dof counts (for the scalings; null: all d).
double oracle_primal_solve_dual_ama(void* h, const double* mass, const double* mu, const double* f, const double* w,
                                   int staticProblem, double tol, unsigned maxIters, double fpStep, double projStep,
                                   unsigned lsIters, double optimistic, double pessimistic, int accelerated,
                                   int useInfinityNorm, const int* trueDofs, double* v, double* r, unsigned* iters,
                                   oracle_callback cb, void* user) {
  auto* P = static_cast<Primal*>(h);
  DualAMASolver s;
  s.P = P;
  s.tol = tol;
  s.maxIters = maxIters;
  s.fpStepSize = fpStep;
  s.projStepSize = projStep;
  s.lsIters = lsIters;
  s.lsOptimisticFactor = optimistic;
  s.lsPessimisticFactor = pessimistic;
  s.accelerated = accelerated != 0;
  s.useInfinityNorm = useInfinityNorm != 0;
  s.callback = wrap(cb, user);
  ADMMSolver sc;
  sc.P = P;
  std::vector<int> td(P->nbodies, P->ndof);
  if (trueDofs) td.assign(trueDofs, trueDofs + P->nbodies);
  sc.setScalings(td);
  s.scalings = sc.scalings;
  s.mTrue = 0;
  for (int k : td) s.mTrue += k;
  std::vector<double> M(mass, mass + (size_t)P->nbodies * P->ndof * P->ndof);
  return s.solve(mu, staticProblem == 0, M, f, w, v, r, iters);
}

// PrimalFrictionProblem::solveWith(ADMM&, lambda, v, r): proxInv = (M + lambda I)^-1 blocks; trueDofs: the
// bodies' own dof counts (for the scalings; null: all d).
double oracle_primal_solve_admm(void* h, const double* proxInv, double lambda, const double* mu, const double* f,
                                const double* w, double tol, unsigned maxIters, double stepSize, int accelerated,
                                int useInfinityNorm, const int* trueDofs, double* v, double* r, unsigned* iters,
                                oracle_callback cb, void* user) {
  auto* P = static_cast<Primal*>(h);
  ADMMSolver s;
  s.P = P;
  s.tol = tol;
  s.maxIters = maxIters;
  s.stepSize = stepSize;
  s.accelerated = accelerated != 0;
  s.useInfinityNorm = useInfinityNorm != 0;
  s.callback = wrap(cb, user);
  std::vector<double> invMu(P->ncontacts);
  for (int i = 0; i < P->ncontacts; ++i) invMu[i] = 1. / mu[i];
  std::vector<double> pinv(proxInv, proxInv + (size_t)P->nbodies * P->ndof * P->ndof);
  std::vector<int> td(P->nbodies, P->ndof);
  if (trueDofs) td.assign(trueDofs, trueDofs + P->nbodies);
  s.setScalings(td);
  return s.solve(invMu.data(), pinv, lambda, f, w, v, r, iters);
}

}  // extern "C"
