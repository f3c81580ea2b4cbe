// CPU restatement of MecheFrictionProblem (Interfaces/MecheInterface.cpp:97-187, 226-367). Test infrastructure:
// the checker of the GPU facade, never the product.
//
// fromPrimal (:97-187): the mass blocks are inverted (PrimalFrictionProblem::computeMInv), H is built per
// contact in the local basis, H_A = E^T HA, H_B = -E^T HB, or E^T (HA - HB) when both objects are the same.
// Bodies with fewer degrees of freedom than the largest are padded with inert dofs (zero Jacobian, zero inverse
// mass), which changes nothing in W, b or v.
// solve (:226-367): r to local coordinates (E^T r), the dual computed once per primal (W + reg I when reg > 0),
// the solver chosen by the options (Gauss-Seidel with the coloring order when maxThreads != 1 and gsColoring,
// projected gradient, Cadoux for a non-static problem with cadouxIters > 0, primal ADMM, DualAMA without line
// search), v = M^-1 (H^T r - f), r back to world coordinates (E r). ADMM and DualAMA scale their error function
// as ConstrainedSolverBase::updateScalings does for this H (the bodies' own dofs, padding excluded).
//
// Evaluation order (shared with the GPU facade): a 3x3 frame block is applied row by row with the dot3 chain,
// E^T x: y_a = fma(E[2][a], x2, fma(E[1][a], x1, E[0][a] x0)), E x: y_a = fma(E[a][2], x2, fma(E[a][1], x1,
// E[a][0] x0)); E^T H column by column with the same chain; the inverse by Gauss-Jordan elimination with
// partial pivoting (first largest |pivot| in the column), row operations a_jk = a_jk - f * a_ik.
#pragma once

#include <cmath>
#include <vector>

#include "oracle_math.hpp"
#include "oracle_solvers.hpp"
#include "oracle_sparse.hpp"

namespace oracle {

// Inverse of a d x d matrix (row-major) by Gauss-Jordan elimination with partial pivoting; false if singular.
inline bool invertGaussJordan(int d, const double* M, double* inv) {
  std::vector<double> a(M, M + (size_t)d * d), b((size_t)d * d, 0.0);
  for (int i = 0; i < d; ++i) b[(size_t)i * d + i] = 1.0;
  for (int c = 0; c < d; ++c) {
    int p = c;
    double best = std::fabs(a[(size_t)c * d + c]);
    for (int rr = c + 1; rr < d; ++rr) {
      const double v = std::fabs(a[(size_t)rr * d + c]);
      if (v > best) {
        best = v;
        p = rr;
      }
    }
    if (!(best > 0.0)) return false;
    if (p != c)
      for (int k = 0; k < d; ++k) {
        std::swap(a[(size_t)p * d + k], a[(size_t)c * d + k]);
        std::swap(b[(size_t)p * d + k], b[(size_t)c * d + k]);
      }
    const double ip = 1.0 / a[(size_t)c * d + c];
    for (int k = 0; k < d; ++k) {
      a[(size_t)c * d + k] = a[(size_t)c * d + k] * ip;
      b[(size_t)c * d + k] = b[(size_t)c * d + k] * ip;
    }
    for (int rr = 0; rr < d; ++rr) {
      if (rr == c) continue;
      const double f = a[(size_t)rr * d + c];
      for (int k = 0; k < d; ++k) {
        a[(size_t)rr * d + k] = a[(size_t)rr * d + k] - f * a[(size_t)c * d + k];
        b[(size_t)rr * d + k] = b[(size_t)rr * d + k] - f * b[(size_t)c * d + k];
      }
    }
  }
  std::copy(b.begin(), b.end(), inv);
  return true;
}

inline void frameT(const double* E, const double* x, double* y) {  // y = E^T x
  for (int a = 0; a < 3; ++a) y[a] = std::fma(E[6 + a], x[2], std::fma(E[3 + a], x[1], E[a] * x[0]));
}
inline void frame(const double* E, const double* x, double* y) {  // y = E x
  for (int a = 0; a < 3; ++a) y[a] = std::fma(E[3 * a + 2], x[2], std::fma(E[3 * a + 1], x[1], E[3 * a] * x[0]));
}

struct Meche {
  Primal P;                  // local-basis H slots as (HA, HB) per contact, minv padded to the largest ndof
  std::vector<int> ndof;     // per body
  std::vector<double> E;     // 9 per contact, row-major E_i[a][b]
  std::vector<double> f;     // nbodies x d (padded)
  std::vector<double> mass;  // nbodies x d x d mass blocks, row-major, padded with zeros
  std::vector<double> w;     // world, 3 n
  std::vector<double> mu;
  bool hasDual = false;
  BSR low, full;
  std::vector<double> b;
};

// MecheFrictionProblem::fromPrimal. mass[k]: column-major ndof[k] x ndof[k]; E: (3n x 3) column-major;
// HA[i] / HB[i]: column-major 3 x ndof of the contact's objects (HB[i] unused when objB[i] == -1).
inline bool mecheFromPrimal(Meche& m, int nobj, const unsigned* ndof, const double* const* mass, const double* f,
                            int n, const double* mu, const double* E, const double* w, const int* objA,
                            const int* objB, const double* const* HA, const double* const* HB) {
  int d = 1;
  for (int k = 0; k < nobj; ++k) d = std::max(d, (int)ndof[k]);
  Primal& P = m.P;
  P.nbodies = nobj;
  P.ndof = d;
  P.ncontacts = n;
  m.ndof.assign(ndof, ndof + nobj);
  P.minv.assign((size_t)nobj * d * d, 0.0);
  m.mass.assign((size_t)nobj * d * d, 0.0);
  m.f.assign((size_t)nobj * d, 0.0);
  for (int k = 0; k < nobj; ++k) {
    const int dk = (int)ndof[k];
    std::vector<double> Mk((size_t)dk * dk), inv((size_t)dk * dk);
    for (int a = 0; a < dk; ++a)
      for (int c = 0; c < dk; ++c) Mk[(size_t)a * dk + c] = mass[k][(size_t)c * dk + a];
    if (!invertGaussJordan(dk, Mk.data(), inv.data())) return false;
    for (int a = 0; a < dk; ++a)
      for (int c = 0; c < dk; ++c) {
        P.minv[(size_t)k * d * d + a * d + c] = inv[(size_t)a * dk + c];
        m.mass[(size_t)k * d * d + a * d + c] = Mk[(size_t)a * dk + c];
      }
  }
  // f is given packed by body (ndof[0] + ndof[1] + ... entries); pad it
  if (f) {
    size_t off = 0;
    for (int k = 0; k < nobj; ++k) {
      for (unsigned a = 0; a < ndof[k]; ++a) m.f[(size_t)k * d + a] = f[off + a];
      off += ndof[k];
    }
  }
  m.E.assign(9 * (size_t)n, 0.0);
  P.objA.assign(n, 0);
  P.objB.assign(n, -1);
  P.HA.assign((size_t)n * 3 * d, 0.0);
  P.HB.assign((size_t)n * 3 * d, 0.0);
  for (int i = 0; i < n; ++i) {
    double* Ei = &m.E[9 * (size_t)i];
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) Ei[3 * a + c] = E[(size_t)c * 3 * n + 3 * i + a];
    const int A = objA[i], B = objB[i];
    const int dA = (int)ndof[A];
    P.objA[i] = A;
    for (int c = 0; c < dA; ++c) {
      double h[3], out[3];
      for (int k = 0; k < 3; ++k) {
        h[k] = HA[i][(size_t)c * 3 + k];
        if (B == A) h[k] = h[k] - HB[i][(size_t)c * 3 + k];
      }
      frameT(Ei, h, out);
      for (int rr = 0; rr < 3; ++rr) P.HA[(size_t)i * 3 * d + rr * d + c] = out[rr];
    }
    if (B >= 0 && B != A) {
      P.objB[i] = B;
      const int dB = (int)ndof[B];
      for (int c = 0; c < dB; ++c) {
        double h[3], out[3];
        for (int k = 0; k < 3; ++k) h[k] = HB[i][(size_t)c * 3 + k];
        frameT(Ei, h, out);
        for (int rr = 0; rr < 3; ++rr) P.HB[(size_t)i * 3 * d + rr * d + c] = -out[rr];
      }
    }
  }
  m.w.assign(w, w + 3 * (size_t)n);
  m.mu.assign(mu, mu + n);
  m.hasDual = false;
  return true;
}

// v = M^-1 (H^T r - f), bodies' contributions in contact order (as the ADMM restatement's H^T product)
inline void mecheVelocity(const Meche& m, const double* r_loc, double* v) {
  ADMMSolver s;
  s.P = &m.P;
  const size_t md = (size_t)m.P.nbodies * m.P.ndof;
  std::vector<double> ht(md);
  s.HTmul(r_loc, nullptr, ht.data());
  s.prox(m.P.minv, ht.data(), m.f.data(), v);
}

}  // namespace oracle
