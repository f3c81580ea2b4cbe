// Host-side sparse structure work of the library: validation, symmetric expansion, greedy coloring and
// contact permutation of the dual problem (one-off per problem; the iterations run on the GPU).
#pragma once

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace bogus_gpu {

struct HostBSR {
  int n = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
  int nnzb() const { return (int)col.size(); }
};

// Checks rowptr/col (monotone rows, sorted unique columns in range, lower triangle when asked); returns an
// empty string when valid.
inline std::string validate_bsr_structure(int n, const int* rowptr, const int* col, bool lower) {
  if (n < 0) return "negative number of contacts";
  if (!rowptr) return "null row pointer";
  if (rowptr[0] != 0) return "rowptr[0] must be 0";
  for (int i = 0; i < n; ++i) {
    if (rowptr[i + 1] < rowptr[i]) return "rowptr not monotone at row " + std::to_string(i);
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
      if (j < 0 || j >= n) return "column index out of range in row " + std::to_string(i);
      if (lower && j > i) return "block above the diagonal in a symmetric-lower matrix, row " + std::to_string(i);
      if (k > rowptr[i] && col[k - 1] >= j) return "columns not sorted/unique in row " + std::to_string(i);
    }
  }
  return std::string();
}

// Checks rowptr/col (monotone rows, sorted unique columns in range, lower triangle when asked) and finite
// values; returns an empty string when valid.
inline std::string validate_bsr(int n, const int* rowptr, const int* col, const double* val, bool lower) {
  if (n < 0) return "negative number of contacts";
  if (!rowptr) return "null row pointer";
  if (rowptr[0] != 0) return "rowptr[0] must be 0";
  for (int i = 0; i < n; ++i) {
    if (rowptr[i + 1] < rowptr[i]) return "rowptr not monotone at row " + std::to_string(i);
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
      if (j < 0 || j >= n) return "column index out of range in row " + std::to_string(i);
      if (lower && j > i) return "block above the diagonal in a symmetric-lower matrix, row " + std::to_string(i);
      if (k > rowptr[i] && col[k - 1] >= j) return "columns not sorted/unique in row " + std::to_string(i);
    }
  }
  const size_t nv = 9 * (size_t)rowptr[n];
  for (size_t k = 0; k < nv; ++k)
    if (!std::isfinite(val[k])) return "non-finite block value";
  return std::string();
}

// Both triangles from the lower one (W_ij = W_ji^T above the diagonal); rows stay sorted.
inline HostBSR expand_lower(int n, const int* rowptr, const int* col, const double* val) {
  HostBSR f;
  f.n = n;
  std::vector<int> cnt(n + 1, 0);
  for (int i = 0; i < n; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      ++cnt[i + 1];
      if (col[k] != i) ++cnt[col[k] + 1];
    }
  f.rowptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) f.rowptr[i + 1] = f.rowptr[i] + cnt[i + 1];
  const int nnz = f.rowptr[n];
  f.col.resize(nnz);
  f.val.resize(9 * (size_t)nnz);
  std::vector<int> pos(f.rowptr.begin(), f.rowptr.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
      const int j = col[k];
      const double* B = val + 9 * (size_t)k;
      int p = pos[i]++;
      f.col[p] = j;
      std::copy(B, B + 9, &f.val[9 * (size_t)p]);
      if (j != i) {
        p = pos[j]++;
        f.col[p] = i;
        double* T = &f.val[9 * (size_t)p];
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) T[3 * r + c] = B[3 * c + r];
      }
    }
  return f;
}

// Lower triangle of a both-triangle matrix.
inline HostBSR lower_of(const HostBSR& full) {
  HostBSR l;
  l.n = full.n;
  l.rowptr.assign(full.n + 1, 0);
  for (int i = 0; i < full.n; ++i) {
    for (int k = full.rowptr[i]; k < full.rowptr[i + 1]; ++k)
      if (full.col[k] <= i) {
        l.col.push_back(full.col[k]);
        l.val.insert(l.val.end(), &full.val[9 * (size_t)k], &full.val[9 * (size_t)k] + 9);
      }
    l.rowptr[i + 1] = (int)l.col.size();
  }
  return l;
}

// Coloring::compute (Core/BlockSolvers/Coloring.impl.hpp:20-62). The reference rejects color c for contact i
// as soon as lower_bound(c, j) != end for a lower neighbour j, i.e. when c holds any member >= j (not only
// j itself). Members are appended in increasing order, so c is accepted iff its last member is below the
// smallest lower neighbour of i (any color when i has none). perm lists contacts color by color; colors
// holds the offsets.
inline void greedy_coloring(const HostBSR& low, std::vector<int>& perm, std::vector<int>& colors) {
  const int n = low.n;
  std::vector<std::vector<int>> members;
  for (int i = 0; i < n; ++i) {
    const int first = low.rowptr[i] < low.rowptr[i + 1] ? low.col[low.rowptr[i]] : i;
    const bool has_lower = first < i;
    int chosen = -1;
    for (int c = 0; c < (int)members.size(); ++c)
      if (!has_lower || members[c].back() < first) { chosen = c; break; }
    if (chosen < 0) {
      chosen = (int)members.size();
      members.emplace_back();
    }
    members[chosen].push_back(i);
  }
  perm.clear();
  colors.assign(1, 0);
  for (auto& m : members) {
    perm.insert(perm.end(), m.begin(), m.end());
    colors.push_back((int)perm.size());
  }
}

// P W P^T of a lower-stored symmetric matrix: new (i, j) = old (perm[i], perm[j]), blocks landing above the
// diagonal stored transposed (Core/Block/SparseBlockMatrixBase.impl.hpp:328-383).
inline HostBSR permute_lower(const HostBSR& low, const std::vector<int>& perm) {
  const int n = low.n;
  std::vector<int> inv(n);
  for (int i = 0; i < n; ++i) inv[perm[i]] = i;
  std::vector<int> cnt(n + 1, 0);
  for (int oi = 0; oi < n; ++oi)
    for (int k = low.rowptr[oi]; k < low.rowptr[oi + 1]; ++k) {
      const int ni = inv[oi], nj = inv[low.col[k]];
      ++cnt[(nj > ni ? nj : ni) + 1];
    }
  HostBSR out;
  out.n = n;
  out.rowptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) out.rowptr[i + 1] = out.rowptr[i] + cnt[i + 1];
  std::vector<std::pair<int, int>> ent(out.rowptr[n]);  // (new col, signed source block)
  std::vector<int> pos(out.rowptr.begin(), out.rowptr.end() - 1);
  for (int oi = 0; oi < n; ++oi)
    for (int k = low.rowptr[oi]; k < low.rowptr[oi + 1]; ++k) {
      const int ni = inv[oi], nj = inv[low.col[k]];
      if (nj > ni)
        ent[pos[nj]++] = {ni, -(k + 1)};
      else
        ent[pos[ni]++] = {nj, k + 1};
    }
  out.col.resize(out.rowptr[n]);
  out.val.resize(9 * (size_t)out.rowptr[n]);
  for (int i = 0; i < n; ++i) {
    std::sort(ent.begin() + out.rowptr[i], ent.begin() + out.rowptr[i + 1]);
    for (int p = out.rowptr[i]; p < out.rowptr[i + 1]; ++p) {
      out.col[p] = ent[p].first;
      const bool tr = ent[p].second < 0;
      const int k = (tr ? -ent[p].second : ent[p].second) - 1;
      const double* Bsrc = &low.val[9 * (size_t)k];
      double* D = &out.val[9 * (size_t)p];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) D[3 * r + c] = tr ? Bsrc[3 * c + r] : Bsrc[3 * r + c];
    }
  }
  return out;
}

// Inverse of a d x d row-major matrix by Gauss-Jordan elimination with partial pivoting (the first largest
// |pivot| in the column; the pivot row scaled by the pivot's reciprocal; row updates a_jk - f a_ik); false when
// a column has no non-zero pivot. Used for the mass blocks of the MecheFrictionProblem facade.
inline bool invert_gauss_jordan(int d, const double* M, double* inv) {
  std::vector<double> a(M, M + (size_t)d * d), b((size_t)d * d, 0.0);
  for (int i = 0; i < d; ++i) b[(size_t)i * d + i] = 1.0;
  for (int c = 0; c < d; ++c) {
    int piv = c;
    double best = std::fabs(a[(size_t)c * d + c]);
    for (int row = c + 1; row < d; ++row) {
      const double m = std::fabs(a[(size_t)row * d + c]);
      if (m > best) {
        best = m;
        piv = row;
      }
    }
    if (!(best > 0.0)) return false;
    if (piv != c)
      for (int k = 0; k < d; ++k) {
        std::swap(a[(size_t)piv * d + k], a[(size_t)c * d + k]);
        std::swap(b[(size_t)piv * d + k], b[(size_t)c * d + k]);
      }
    const double rp = 1.0 / a[(size_t)c * d + c];
    for (int k = 0; k < d; ++k) {
      a[(size_t)c * d + k] = a[(size_t)c * d + k] * rp;
      b[(size_t)c * d + k] = b[(size_t)c * d + k] * rp;
    }
    for (int row = 0; row < d; ++row) {
      if (row == c) continue;
      const double g = a[(size_t)row * d + c];
      for (int k = 0; k < d; ++k) {
        a[(size_t)row * d + k] = a[(size_t)row * d + k] - g * a[(size_t)c * d + k];
        b[(size_t)row * d + k] = b[(size_t)row * d + k] - g * b[(size_t)c * d + k];
      }
    }
  }
  std::copy(b.begin(), b.end(), inv);
  return true;
}

}  // namespace bogus_gpu
