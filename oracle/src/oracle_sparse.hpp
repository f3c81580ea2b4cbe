// ORACLE — test infrastructure only (see oracle_math.hpp).
//
// CPU restatement of the reference's 3x3-block sparse containers and products used on the friction path:
//  * W is SparseBlockMatrix<Matrix3d RowMajor, SYMMETRIC>: block-rows sorted by column, only the lower
//    triangle (col <= row) stored (Core/Block/Constants.hpp:60-65, SparseBlockMatrix.hpp:55-135);
//  * symmetric products y = W x: for row i the stored blocks W_ij (j <= i) act directly and every stored
//    W_ji (j > i) acts transposed (Core/Block/SparseMatrixVectorProduct.impl.hpp:89-175); run
//    sequentially this visits row i's columns in increasing order; the "full" view holds both triangles,
//    each row sorted by column, and spmv() sums each row in that column order, cut into the pieces
//    described at spmv();
//  * splitRowMultiply: the same row sum without the diagonal block (:298-320);
//  * the error function and dot products reduce per-contact values with a fixed tree, canonicalSum().
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "oracle_math.hpp"

namespace oracle {

struct BSR {
  int n = 0;                 // block rows (contacts)
  std::vector<int> rowptr;   // n + 1
  std::vector<int> col;      // nnzb
  std::vector<double> val;   // 9 * nnzb, row-major blocks
  int nnzb() const { return (int)col.size(); }
  const double* block(int k) const { return &val[9 * (size_t)k]; }
  int diagPtr(int i) const {
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (col[k] == i) return k;
    return -1;
  }
};

// Both triangles from the stored lower triangle; W_ij = W_ji^T above the diagonal.
inline BSR expandSymmetric(const BSR& low) {
  const int n = low.n;
  std::vector<int> cnt(n + 1, 0);
  for (int i = 0; i < n; ++i)
    for (int k = low.rowptr[i]; k < low.rowptr[i + 1]; ++k) {
      const int j = low.col[k];
      if (j > i) throw std::runtime_error("expandSymmetric: block above the diagonal");
      ++cnt[i + 1];
      if (j != i) ++cnt[j + 1];
    }
  BSR full;
  full.n = n;
  full.rowptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) full.rowptr[i + 1] = full.rowptr[i] + cnt[i + 1];
  const int nnz = full.rowptr[n];
  full.col.assign(nnz, 0);
  full.val.assign(9 * (size_t)nnz, 0.0);
  std::vector<int> pos(full.rowptr.begin(), full.rowptr.end() - 1);
  // Row i receives, in increasing column order: its own stored blocks (j <= i, already sorted) first, then
  // transposed blocks W_ji for j > i, which are appended while scanning rows j = i+1.. in order.
  for (int i = 0; i < n; ++i)
    for (int k = low.rowptr[i]; k < low.rowptr[i + 1]; ++k) {
      const int j = low.col[k];
      const double* B = low.block(k);
      int p = pos[i]++;
      full.col[p] = j;
      std::copy(B, B + 9, &full.val[9 * (size_t)p]);
      if (j != i) {
        p = pos[j]++;
        full.col[p] = i;
        double* T = &full.val[9 * (size_t)p];
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) T[3 * r + c] = B[3 * c + r];
      }
    }
  // rows built above are sorted when the lower input is sorted: own blocks (cols <= i) precede the
  // transposed ones (cols > i, appended in increasing j); check it.
  for (int i = 0; i < n; ++i)
    for (int k = full.rowptr[i] + 1; k < full.rowptr[i + 1]; ++k)
      if (full.col[k] <= full.col[k - 1]) throw std::runtime_error("expandSymmetric: unsorted or duplicate blocks");
  return full;
}

// acc[r] += sum_c B[r][c] x[c] as the canonical chain of three fused multiply-adds per component
inline void blockAccumulate(const double* B, const double* x, double* acc) {
  for (int r = 0; r < 3; ++r) {
    double a = acc[r];
    a = std::fma(B[3 * r + 0], x[0], a);
    a = std::fma(B[3 * r + 1], x[1], a);
    a = std::fma(B[3 * r + 2], x[2], a);
    acc[r] = a;
  }
}

// y = W x (init == nullptr) or y = init + W x; full view. Canonical chunk-segmented order (the order the GPU
// kernels use to keep their lanes evenly loaded): the blocks [B0, B1) of each 32-row chunk are cut into 32
// consecutive segments of S = ceil((B1 - B0) / 32) blocks; for row i, each segment meeting its blocks gives a
// piece p (the blockAccumulate chain over the blocks of row i inside the segment, from 0), and
// y_i = (((init_i + p_first) + p_next) + ...) in segment order. Columns are still visited in increasing order.
inline void spmv(const BSR& W, const double* x, double* y, const double* init = nullptr) {
  const int C = (W.n + 31) / 32;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < C; ++c) {
    const int r0 = 32 * c, r1 = std::min(W.n, r0 + 32);
    const int B0 = W.rowptr[r0], B1 = W.rowptr[r1];
    const int T = B1 - B0;
    const int S = T > 0 ? (T + 31) / 32 : 1;
    for (int i = r0; i < r1; ++i) {
      double acc[3] = {0.0, 0.0, 0.0};
      if (init) { acc[0] = init[3 * i]; acc[1] = init[3 * i + 1]; acc[2] = init[3 * i + 2]; }
      int k = W.rowptr[i];
      const int hi = W.rowptr[i + 1];
      while (k < hi) {
        const int l = (k - B0) / S;
        const int e = std::min(hi, std::min(B0 + (l + 1) * S, B1));
        double p[3] = {0.0, 0.0, 0.0};
        for (; k < e; ++k) blockAccumulate(W.block(k), &x[3 * (size_t)W.col[k]], p);
        acc[0] = acc[0] + p[0];
        acc[1] = acc[1] + p[1];
        acc[2] = acc[2] + p[2];
      }
      y[3 * i] = acc[0];
      y[3 * i + 1] = acc[1];
      y[3 * i + 2] = acc[2];
    }
  }
}

// y = W32 x in single precision, W32 the float copy of W's values (9 per block, BSR order), in the same canonical
// chunk-segmented order as spmv (pieces from 0 by fmaf chains, the first piece of a row placed as 0 + piece, the
// next ones added). Not in the reference: the FP32 correction products of the FP32-refined solve.
inline void spmv32(const BSR& W, const float* W32, const float* x, float* y) {
  const int C = (W.n + 31) / 32;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < C; ++c) {
    const int r0 = 32 * c, r1 = std::min(W.n, r0 + 32);
    const int B0 = W.rowptr[r0], B1 = W.rowptr[r1];
    const int T = B1 - B0;
    const int S = T > 0 ? (T + 31) / 32 : 1;
    for (int i = r0; i < r1; ++i) {
      float acc[3] = {0.f, 0.f, 0.f};
      int k = W.rowptr[i];
      const int hi = W.rowptr[i + 1];
      while (k < hi) {
        const int l = (k - B0) / S;
        const int e = std::min(hi, std::min(B0 + (l + 1) * S, B1));
        float p[3] = {0.f, 0.f, 0.f};
        for (; k < e; ++k) {
          const float* B = W32 + 9 * (size_t)k;
          const float* xv = x + 3 * (size_t)W.col[k];
          for (int r = 0; r < 3; ++r) {
            float a = p[r];
            a = std::fma(B[3 * r + 0], xv[0], a);
            a = std::fma(B[3 * r + 1], xv[1], a);
            a = std::fma(B[3 * r + 2], xv[2], a);
            p[r] = a;
          }
        }
        acc[0] = acc[0] + p[0];
        acc[1] = acc[1] + p[1];
        acc[2] = acc[2] + p[2];
      }
      y[3 * i] = acc[0];
      y[3 * i + 1] = acc[1];
      y[3 * i + 2] = acc[2];
    }
  }
}

// res += sum_{j != row} W_row,j x_j (splitRowMultiply), full view
inline void splitRowMultiply(const BSR& W, int row, const double* x, double* res) {
  for (int k = W.rowptr[row]; k < W.rowptr[row + 1]; ++k) {
    const int j = W.col[k];
    if (j != row) blockAccumulate(W.block(k), &x[3 * (size_t)j], res);
  }
}

// ---------------------------------------------------------------------------------------------
// Canonical reduction of n per-contact values (the order the GPU kernels use):
//   1. chunk c = values[32c .. 32c+31] (zero padded) is reduced by a xor butterfly: at offsets
//      16, 8, 4, 2, 1 every lane l adds lane l^off; the result is lane 0's value;
//   2. the chunk sums are split into 8 stripes of ceil(C/8) consecutive chunks; in stripe k, lane l
//      sums chunks start+l, start+l+32, ... sequentially from 0, then the 32 lane sums are reduced by
//      the same butterfly;
//   3. the 8 stripe sums are added left to right.
// ---------------------------------------------------------------------------------------------
inline double butterfly32(double* v) {
  for (int off = 16; off >= 1; off >>= 1) {
    double t[32];
    for (int l = 0; l < 32; ++l) t[l] = v[l] + v[l ^ off];
    for (int l = 0; l < 32; ++l) v[l] = t[l];
  }
  return v[0];
}

inline std::vector<double> chunkSums(const double* vals, size_t n) {
  const size_t C = (n + 31) / 32;
  std::vector<double> s(C);
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < (long long)C; ++c) {
    double v[32];
    for (int l = 0; l < 32; ++l) {
      const size_t i = (size_t)c * 32 + l;
      v[l] = i < n ? vals[i] : 0.0;
    }
    s[c] = butterfly32(v);
  }
  return s;
}

inline double combineChunkSums(const double* s, size_t C) {
  const size_t per = (C + 7) / 8;
  double total = 0.0;
  for (int k = 0; k < 8; ++k) {
    const size_t b = k * per, e = std::min(C, (k + 1) * per);
    double lane[32];
    for (int l = 0; l < 32; ++l) {
      double p = 0.0;
      for (size_t c = b + l; c < e; c += 32) p = p + s[c];
      lane[l] = p;
    }
    const double q = butterfly32(lane);
    total = (k == 0) ? q : total + q;
  }
  return total;
}

inline double canonicalSum(const double* vals, size_t n) {
  const std::vector<double> s = chunkSums(vals, n);
  return combineChunkSums(s.data(), s.size());
}

inline double maxOf(const double* vals, size_t n) {
  double m = 0.0;
  for (size_t i = 0; i < n; ++i) m = dmax(vals[i], m);
  return m;
}

// ---------------------------------------------------------------------------------------------
// Greedy coloring (Core/BlockSolvers/Coloring.impl.hpp:20-62): contacts in natural order; for each color c
// and each lower neighbour j of i (stored blocks W_ij, j < i, increasing), the reference tests
// `color.end() != std::lower_bound(color.begin(), color.end(), j)` and rejects c when the test holds, that
// is when c has any member >= j (not only j). Restated literally (binary search over the sorted members).
// ---------------------------------------------------------------------------------------------
inline void greedyColoring(const BSR& low, std::vector<int>& perm, std::vector<int>& colors) {
  const int n = low.n;
  std::vector<std::vector<int>> members;
  for (int i = 0; i < n; ++i) {
    bool ok = false;
    const int nColors = (int)members.size();
    for (int c = 0; c < nColors; ++c) {
      std::vector<int>& color = members[c];
      ok = true;
      for (int k = low.rowptr[i]; k < low.rowptr[i + 1] && low.col[k] < i; ++k) {
        if (color.end() != std::lower_bound(color.begin(), color.end(), low.col[k])) {
          ok = false;
          break;
        }
      }
      if (ok) {
        color.push_back(i);
        break;
      }
    }
    if (!ok) {
      members.emplace_back();
      members.back().push_back(i);
    }
  }
  perm.clear();
  colors.assign(1, 0);
  for (auto& m : members) {
    perm.insert(perm.end(), m.begin(), m.end());
    colors.push_back((int)perm.size());
  }
}

// new[i] = old[perm[i]] (bogus::applyPermutation, Core/Block/SparseBlockMatrixBase.impl.hpp:309-326)
template <typename T>
inline std::vector<T> permuteSegments(const std::vector<T>& v, const std::vector<int>& perm, int dim) {
  std::vector<T> out(v.size());
  for (size_t i = 0; i < perm.size(); ++i)
    for (int d = 0; d < dim; ++d) out[dim * i + d] = v[dim * (size_t)perm[i] + d];
  return out;
}

// P W P^T on the symmetric lower storage: new block (i, j) = old (perm[i], perm[j]); blocks that land
// above the diagonal are stored transposed at (j, i) (SparseBlockMatrixBase.impl.hpp:328-383).
inline BSR permuteSymmetric(const BSR& low, const std::vector<int>& perm) {
  const int n = low.n;
  std::vector<int> inv(n);
  for (int i = 0; i < n; ++i) inv[perm[i]] = i;
  std::vector<std::vector<std::pair<int, int>>> rows(n);  // (col, source block), transpose flag in sign
  for (int oi = 0; oi < n; ++oi)
    for (int k = low.rowptr[oi]; k < low.rowptr[oi + 1]; ++k) {
      const int ni = inv[oi], nj = inv[low.col[k]];
      if (nj > ni)
        rows[nj].push_back({ni, -(k + 1)});
      else
        rows[ni].push_back({nj, k + 1});
    }
  BSR out;
  out.n = n;
  out.rowptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    std::sort(rows[i].begin(), rows[i].end());
    out.rowptr[i + 1] = out.rowptr[i] + (int)rows[i].size();
  }
  out.col.resize(out.rowptr[n]);
  out.val.resize(9 * (size_t)out.rowptr[n]);
  for (int i = 0; i < n; ++i) {
    int p = out.rowptr[i];
    for (auto& e : rows[i]) {
      out.col[p] = e.first;
      const bool tr = e.second < 0;
      const int k = (tr ? -e.second : e.second) - 1;
      const double* B = low.block(k);
      double* D = &out.val[9 * (size_t)p];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) D[3 * r + c] = tr ? B[3 * c + r] : B[3 * r + c];
      ++p;
    }
  }
  return out;
}

// ---------------------------------------------------------------------------------------------
// Delassus assembly W = H M^-1 H^T, b = w - H M^-1 f (Interfaces/FrictionProblem.cpp:30-40 with E = I).
// Contact i touches body objA[i] (always) and objB[i] (or -1); its Jacobian blocks HA[i], HB[i] are 3 x ndof
// row-major. M^-1 is block diagonal, minv[k] an ndof x ndof row-major block.
// Canonical order: T_jk = M^-1_k H_jk^T first (as the reference evaluates M^-1 H^T first), element
// (m, c) = chain over q of fma(Minv[m][q], H_jk[c][q]); W_ij[r][c] = chain over the shared bodies k in
// increasing body index, then over m, of fma(H_ik[r][m], T_jk[m][c]).
// ---------------------------------------------------------------------------------------------
struct Primal {
  int nbodies = 0, ndof = 6, ncontacts = 0;
  std::vector<double> minv;       // nbodies * ndof * ndof
  std::vector<int> objA, objB;    // ncontacts
  std::vector<double> HA, HB;     // ncontacts * 3 * ndof
};

inline void contactBodies(const Primal& P, int i, int* bodies, const double** H, int& nb) {
  nb = 0;
  const int a = P.objA[i], b = P.objB[i];
  const double* ha = &P.HA[(size_t)i * 3 * P.ndof];
  const double* hb = &P.HB[(size_t)i * 3 * P.ndof];
  if (b >= 0 && b < a) {
    bodies[nb] = b; H[nb++] = hb;
    bodies[nb] = a; H[nb++] = ha;
  } else {
    bodies[nb] = a; H[nb++] = ha;
    if (b >= 0 && b != a) { bodies[nb] = b; H[nb++] = hb; }
  }
}

// T = M^-1 H^T for every (contact, slot): d x 3 row-major blocks at (2 j + t) d 3, slots in body order.
inline std::vector<double> slotT(const Primal& P) {
  const int n = P.ncontacts, d = P.ndof;
  std::vector<double> T((size_t)n * 2 * d * 3, 0.0);
  for (int j = 0; j < n; ++j) {
    int bodies[2]; const double* H[2]; int nb;
    contactBodies(P, j, bodies, H, nb);
    for (int t = 0; t < nb; ++t) {
      const double* Mi = &P.minv[(size_t)bodies[t] * d * d];
      double* Tj = &T[((size_t)j * 2 + t) * d * 3];
      for (int m = 0; m < d; ++m)
        for (int c = 0; c < 3; ++c) {
          double a = 0.0;
          for (int q = 0; q < d; ++q) a = std::fma(Mi[m * d + q], H[t][c * d + q], a);
          Tj[m * 3 + c] = a;
        }
    }
  }
  return T;
}

inline BSR assembleW(const Primal& P) {
  const int n = P.ncontacts, d = P.ndof;
  // body -> contacts incidence
  std::vector<std::vector<int>> byBody(P.nbodies);
  for (int i = 0; i < n; ++i) {
    int bodies[2]; const double* H[2]; int nb;
    contactBodies(P, i, bodies, H, nb);
    for (int t = 0; t < nb; ++t) byBody[bodies[t]].push_back(i);
  }
  // T_jk for every (contact, body)
  const std::vector<double> T = slotT(P);
  BSR low;
  low.n = n;
  low.rowptr.assign(n + 1, 0);
  std::vector<int> cols;
  for (int i = 0; i < n; ++i) {
    int bi[2]; const double* Hi[2]; int nbi;
    contactBodies(P, i, bi, Hi, nbi);
    cols.clear();
    for (int t = 0; t < nbi; ++t)
      for (int j : byBody[bi[t]])
        if (j <= i) cols.push_back(j);
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    for (int j : cols) {
      int bj[2]; const double* Hj[2]; int nbj;
      contactBodies(P, j, bj, Hj, nbj);
      double B[9];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          double a = 0.0;
          for (int ti = 0; ti < nbi; ++ti)
            for (int tj = 0; tj < nbj; ++tj) {
              if (bi[ti] != bj[tj]) continue;
              const double* Tj = &T[((size_t)j * 2 + tj) * d * 3];
              for (int m = 0; m < d; ++m) a = std::fma(Hi[ti][r * d + m], Tj[m * 3 + c], a);
            }
          B[3 * r + c] = a;
        }
      low.col.push_back(j);
      low.val.insert(low.val.end(), B, B + 9);
    }
    low.rowptr[i + 1] = (int)low.col.size();
  }
  return low;
}

// b = w - H (M^-1 f)
inline std::vector<double> assembleB(const Primal& P, const double* f, const double* w) {
  const int d = P.ndof;
  std::vector<double> mf((size_t)P.nbodies * d);
  for (int k = 0; k < P.nbodies; ++k)
    for (int m = 0; m < d; ++m) {
      double a = 0.0;
      for (int q = 0; q < d; ++q) a = std::fma(P.minv[(size_t)k * d * d + m * d + q], f[(size_t)k * d + q], a);
      mf[(size_t)k * d + m] = a;
    }
  std::vector<double> b(3 * (size_t)P.ncontacts);
  for (int i = 0; i < P.ncontacts; ++i) {
    int bodies[2]; const double* H[2]; int nb;
    contactBodies(P, i, bodies, H, nb);
    for (int r = 0; r < 3; ++r) {
      double a = 0.0;
      for (int t = 0; t < nb; ++t)
        for (int m = 0; m < d; ++m) a = std::fma(H[t][r * d + m], mf[(size_t)bodies[t] * d + m], a);
      b[3 * i + r] = w[3 * i + r] - a;
    }
  }
  return b;
}

}  // namespace oracle
