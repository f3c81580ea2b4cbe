// A C++ caller of the library through include/bogus_gpu.hpp, written the way a caller of the reference's
// DualFrictionProblem / GaussSeidel / ProjectedGradient API would write it.
//
//   shim_check defaults            option defaults against the reference's constructors, the host-side
//                                  BAD_INPUT paths, and what a solve reports without a usable GPU
//   shim_check solve IN OUT        reads a primal problem (IN), assembles the dual on the GPU, solves it with
//                                  Gauss-Seidel (Coulomb), APGD (SOC), the Cadoux fixed point and ADMM, and writes
//                                  W, b and the results (OUT) for the test to compare with the oracle
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "bogus_gpu.hpp"

namespace {

int failures = 0;
void expect(bool ok, const char* what) {
  if (!ok) {
    std::cerr << "FAILED: " << what << "\n";
    ++failures;
  }
}

template <class T>
void read_vec(std::ifstream& in, std::vector<T>& v, std::size_t n) {
  v.resize(n);
  in.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
}
template <class T>
void write_vec(std::ofstream& out, const T* p, std::size_t n) {
  out.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(T)));
}

int defaults() {
  bogus_gpu::GaussSeidel gs;
  expect(gs.tol() == 1e-6 && gs.maxIters() == 250, "GaussSeidel tol / maxIters");
  expect(gs.evalEvery() == 25 && gs.skipTol() == 1e-6 && gs.skipIters() == 10, "GaussSeidel evalEvery / skip");
  expect(gs.autoRegularization() == 0.0 && gs.tryZeroAsWell() && !gs.usesInfinityNorm(), "GaussSeidel regularization");
  expect(!gs.coloring().enabled(), "GaussSeidel coloring off");
  bogus_gpu::ProjectedGradient pg;
  expect(pg.tol() == 1e-6 && pg.maxIters() == 300 && pg.lineSearchIterations() == 8, "ProjectedGradient tol / iters");
  expect(pg.lineSearchOptimisticFactor() == 1.25 && pg.lineSearchPessimisticFactor() == 0.5 &&
             pg.lineSearchArmijoCoefficient() == 0.5,
         "ProjectedGradient line search");
  expect(pg.defaultVariant() == bogus_gpu::projected_gradient::APGD, "ProjectedGradient variant");
  bogus_gpu::ADMM admm;
  expect(admm.tol() == 1e-6 && admm.maxIters() == 300 && admm.stepSize() == 1e-2, "ADMM defaults");
  bogus_gpu::DualAMA dama;
  expect(dama.tol() == 1e-6 && dama.maxIters() == 300 && dama.fpStepSize() == 1e-1 && dama.projStepSize() == 1e-1,
         "DualAMA defaults");
  // options built from the setters
  pg.setMaxIters(17);
  pg.setDefaultVariant(bogus_gpu::projected_gradient::SPG);
  expect(pg.options(true).momentum_by_linearity == 0, "ProjectedGradient: the reference's momentum product by default");
  pg.setMomentumByLinearity(true);
  const bogus_gpu_pg_options o = pg.options(false);
  expect(o.max_iters == 17 && o.variant == BOGUS_GPU_PG_SPG && o.static_problem == 0 && o.momentum_by_linearity == 1,
         "ProjectedGradient options");
  expect(o.fp32_stall_iters == 4, "ProjectedGradient: FP32 stall test on by default");
  pg.setFp32StallIterations(0);
  expect(pg.options(true).fp32_stall_iters == 0, "ProjectedGradient: FP32 stall test off");

  // host-side BAD_INPUT paths (no GPU needed)
  bogus_gpu::DualFrictionProblem<3> dual;
  const int outer[3] = {0, 1, 3}, inner[3] = {0, 0, 1};
  const double blocks[27] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  dual.W.setFromLower(2, outer, inner, blocks);
  dual.b.resize(5);  // should be 6
  dual.mu.resize(2);
  std::vector<double> r(6, 0.0);
  try {
    dual.solveWith(pg, r.data());
    expect(false, "b of the wrong size must throw");
  } catch (const bogus_gpu::Error& e) {
    expect(e.status() == BOGUS_GPU_BAD_INPUT, "b of the wrong size: BAD_INPUT");
  }
  bogus_gpu::PrimalFrictionProblem<3> primal;
  primal.objA = {0};
  primal.objB = {-1};
  primal.HA.assign(18, 0.0);
  primal.HB.assign(17, 0.0);  // should be 18
  primal.MInv.assign(36, 0.0);
  try {
    dual.computeFrom(primal);
    expect(false, "inconsistent primal arrays must throw");
  } catch (const bogus_gpu::Error& e) {
    expect(e.status() == BOGUS_GPU_BAD_INPUT, "inconsistent primal arrays: BAD_INPUT");
  }
  // computeMInv on a diagonal and a full block
  primal.M = {2, 0, 0, 0, 0, 0, 0, 2, 0, 0, 0, 0, 0, 0, 2, 0, 0, 0, 0, 0, 0, 4, 0, 0, 0, 0, 0, 0, 4, 0, 0, 0, 0, 0, 0, 4};
  primal.computeMInv();
  expect(primal.MInv[0] == 0.5 && primal.MInv[21] == 0.25 && primal.MInv[1] == 0.0, "computeMInv");
  // a well-formed problem: solves on a GPU, reports NO_DEVICE / CUDA_ERROR without one
  dual.b.resize(6);
  dual.b.setZero();
  dual.mu[0] = dual.mu[1] = 0.5;
  try {
    const double res = dual.solveWith(pg, r.data());
    std::cout << "solved on a GPU, residual " << res << "\n";
  } catch (const bogus_gpu::Error& e) {
    expect(e.status() == BOGUS_GPU_NO_DEVICE || e.status() == BOGUS_GPU_CUDA_ERROR, "no GPU: NO_DEVICE");
    std::cout << "no usable GPU: " << e.what() << "\n";
  }
  if (failures == 0) std::cout << "defaults ok\n";
  return failures ? 1 : 0;
}

int solve(const char* in_path, const char* out_path) {
  std::ifstream in(in_path, std::ios::binary);
  int hdr[3];
  in.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
  const int n = hdr[0], nb = hdr[1], d = hdr[2];
  bogus_gpu::PrimalFrictionProblem<3> primal;
  primal.ndof = (unsigned)d;
  read_vec(in, primal.MInv, (std::size_t)nb * d * d);
  read_vec(in, primal.objA, n);
  read_vec(in, primal.objB, n);
  read_vec(in, primal.HA, (std::size_t)n * 3 * d);
  read_vec(in, primal.HB, (std::size_t)n * 3 * d);
  std::vector<double> w, mu;
  read_vec(in, w, 3 * (std::size_t)n);
  read_vec(in, mu, n);
  if (!in) {
    std::cerr << "short input\n";
    return 2;
  }
  primal.w = w.data();
  primal.mu = mu.data();

  bogus_gpu::DualFrictionProblem<3> dual;
  dual.computeFrom(primal);
  std::ofstream out(out_path, std::ios::binary);
  const int nnz = dual.W.nonZeros();
  write_vec(out, &nnz, 1);
  write_vec(out, dual.W.outerIndexPtr(), n + 1);
  write_vec(out, dual.W.innerIndexPtr(), nnz);
  write_vec(out, dual.W.blockPtr(), 9 * (std::size_t)nnz);
  write_vec(out, dual.b.data(), 3 * (std::size_t)n);

  // Gauss-Seidel, Coulomb law (the solveWith default), with a callback
  bogus_gpu::DualFrictionProblem<3>::GaussSeidelType gs;
  gs.setTol(1e-8);
  unsigned calls = 0;
  gs.callback().connect([&](unsigned, double) { ++calls; });
  std::vector<double> r(3 * (std::size_t)n, 0.0);
  double res = dual.solveWith(gs, r.data());
  write_vec(out, &res, 1);
  write_vec(out, r.data(), r.size());
  const double ev = dual.evalWith(gs, r.data());
  write_vec(out, &ev, 1);
  const double ncalls = (double)calls;
  write_vec(out, &ncalls, 1);

  // APGD, SOC law (the solveWith default)
  bogus_gpu::DualFrictionProblem<3>::ProjectedGradientType pg;
  pg.setTol(1e-8);
  std::fill(r.begin(), r.end(), 0.0);
  res = dual.solveWith(pg, r.data());
  write_vec(out, &res, 1);
  write_vec(out, r.data(), r.size());

  // Cadoux fixed point with projected gradient, 10 iterations
  bogus_gpu::ProjectedGradient pgc;
  pgc.setTol(1e-8);
  std::fill(r.begin(), r.end(), 0.0);
  res = dual.solveCadoux(pgc, r.data(), 10);
  write_vec(out, &res, 1);
  write_vec(out, r.data(), r.size());

  // a changed b is uploaded again before the next solve
  for (int i = 0; i < n; ++i) dual.b[3 * (std::size_t)i] += 0.125;
  std::fill(r.begin(), r.end(), 0.0);
  res = dual.solveWith(pg, r.data());
  write_vec(out, &res, 1);
  write_vec(out, r.data(), r.size());

  // primal ADMM (lambda = 0: AMA), SOC law
  bogus_gpu::PrimalFrictionProblem<3>::ADMMType admm;
  admm.setMaxIters(50);
  std::vector<double> v((std::size_t)nb * d, 0.0);
  std::fill(r.begin(), r.end(), 0.0);
  res = primal.solveWith(admm, 0.0, v.data(), r.data());
  write_vec(out, &res, 1);
  write_vec(out, v.data(), v.size());
  write_vec(out, r.data(), r.size());
  std::cout << "solve ok\n";
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    if (argc >= 2 && std::strcmp(argv[1], "defaults") == 0) return defaults();
    if (argc >= 4 && std::strcmp(argv[1], "solve") == 0) return solve(argv[2], argv[3]);
  } catch (const bogus_gpu::Error& e) {
    std::cerr << "bogus_gpu::Error " << e.status() << ": " << e.what() << "\n";
    return 3;
  }
  std::cerr << "usage: shim_check defaults | solve IN OUT\n";
  return 2;
}
