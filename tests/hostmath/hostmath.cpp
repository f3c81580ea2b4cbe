// Test helper: the library's per-contact device mathematics (so-bogus_gb300/csrc/soc_device.cuh) compiled
// for the host with the same evaluation rules (-ffp-contract=off), exported for ctypes. The CPU tests compare
// it bit for bit with the oracle; the GPU tests then compare the kernels with the oracle.
#include "soc_device.cuh"

using namespace bogus_gpu;

extern "C" {

double hm_local_solve(int desaxce, int strat, const double* A, const double* b, double* x, double mu, double tol,
                      double scaling) {
  return local_solve(desaxce != 0, strat, A, b, x, mu, tol, scaling);
}

int hm_law_solve_local(int desaxce, int strat, const double* A, const double* b, double* x, double mu,
                       double scaling) {
  return law_solve_local(desaxce != 0, strat, A, b, x, mu, scaling) ? 1 : 0;
}

double hm_law_eval(int desaxce, double mu, const double* x, const double* y) { return law_eval(desaxce != 0, mu, x, y); }

void hm_project(double mu, double* x) { project_cone(mu, x); }

int hm_real_roots(const double* coeffs, int dim, int degenerate, int filter, double* roots) {
  double c[8];
  for (int k = 0; k < dim + (degenerate ? 1 : 0); ++k) c[k] = coeffs[k];
  return degenerate ? real_roots_degenerate(c, dim, roots, filter) : real_roots_monic(c, dim, roots, filter);
}

void hm_fb_jacobian(int desaxce, double mu, double scaling, const double* A, const double* b, const double* x,
                    double* fb, double* dFdx) {
  LocalFB f{desaxce != 0, mu, scaling, A, b};
  f.jacobian(x, fb, dFdx);
}

double hm_min_eigen_symmetric3(const double* D) { return min_eigen_symmetric3(D); }

}  // extern "C"
