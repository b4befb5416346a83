// Host side of the AMG setup: the reference's C/F splitting and projection
// (AMGSolver::Project, src/AMGSolver.cpp:18-226) and the greedy colouring
// that orders the GPU smoother.
//
// Project runs on the host by design (it is a sequential greedy sweep over
// the rows).  This implementation keeps the reference's decisions and
// floating-point operations -- the same strength threshold, the same
// row-order greedy passes, the same weight formulas accumulated in the same
// order -- so C/F flags and P are bitwise the reference's.  It replaces the
// reference's linear scans (SparseMatrix::el, std::find, SparsityPattern::add)
// by binary searches on the sorted rows, which return the same entries.
#include <algorithm>
#include <cmath>
#include <queue>
#include <tuple>
#include <cstdlib>
#include <cstring>

#include "common.cuh"
#include "kernels.cuh"

namespace afp {

namespace {

// value of (i, j) in a [diag, ascending others] row, 0 when absent
inline double entry(const HostCSR& M, int i, int j) {
  const int b = M.rowptr[i], e = M.rowptr[i + 1];
  if (b == e) return 0.0;
  if (M.cols[b] == j) return M.vals[b];
  const int* lo = M.cols.data() + b + 1;
  const int* hi = M.cols.data() + e;
  const int* p = std::lower_bound(lo, hi, j);
  return (p != hi && *p == j) ? M.vals[p - M.cols.data()] : 0.0;
}

}  // namespace

void host_project(const HostCSR& M, double alpha, std::vector<int>& flag, HostCSR& P, HostCSR& Pt) {
  const int m = (int)M.m;
  const int* rs = M.rowptr.data();
  const int* cn = M.cols.data();
  const double* v = M.vals.data();
  flag.assign(m, 0);
  std::vector<double> beta(m, 0.0);
  int n_core = 0;
  // first pass: thresholds and greedy C-point choice in row order
  for (int i = 0; i < m; ++i) {
    double b = 0.0;
    for (int j = rs[i] + 1; j < rs[i + 1]; ++j) {
      const double a = std::fabs(v[j]);
      b = (a < b) ? b : a;
    }
    beta[i] = b * alpha;
    if (flag[i] != 0) continue;
    for (int j = rs[i] + 1; j < rs[i + 1]; ++j) {
      const int k = cn[j];
      if (flag[k] == -1) continue;
      if (std::fabs(v[j]) < beta[i]) continue;
      flag[k] = 1;
    }
    flag[i] = -1;
    ++n_core;
  }
  // second pass: F points with a strong F-F connection lacking a common
  // strong C neighbour become C points.  The set of i's strong C neighbours
  // is a marker array (dep_mark[c] == i) instead of the reference's list
  // scan: the same membership answers in O(1), which keeps dense coarse
  // levels (rows of ~10^3 entries) from turning the pass quadratic.
  std::vector<int> dep_mark(m, -1);
  for (int i = 0; i < m; ++i) {
    if (flag[i] != 1) continue;
    for (int j = rs[i] + 1; j < rs[i + 1]; ++j) {
      if (std::fabs(v[j]) < beta[i]) continue;
      if (flag[cn[j]] == -1) dep_mark[cn[j]] = i;
    }
    bool is_FF = false;
    for (int j = rs[i] + 1; j < rs[i + 1]; ++j) {
      const int k = cn[j];
      if (flag[k] == -1 || k < i || std::fabs(v[j]) < beta[i]) continue;
      is_FF = true;
      for (int j1 = rs[k] + 1; j1 < rs[k + 1]; ++j1) {
        const int k1 = cn[j1];
        if (flag[k1] != -1) continue;
        if (dep_mark[k1] == i) {
          is_FF = false;
          break;
        }
      }
      if (is_FF) break;
    }
    if (!is_FF) continue;
    flag[i] = -1;
    ++n_core;
  }
  std::vector<int> core_point(n_core), core_at(m, -1);
  for (int i = 0, n = 0; i < m; ++i)
    if (flag[i] == -1) {
      core_point[n] = i;
      core_at[i] = n++;
    }
  // pattern of P: row c = {core point} U {its non-C neighbours}, ascending
  // (rectangular SparsityPattern rows are fully sorted by compress)
  P.m = n_core;
  P.n = m;
  P.rowptr.assign(n_core + 1, 0);
  for (int c = 0; c < n_core; ++c) {
    const int k = core_point[c];
    int len = 1;
    for (int j = rs[k] + 1; j < rs[k + 1]; ++j) len += (flag[cn[j]] != -1);
    P.rowptr[c + 1] = P.rowptr[c] + len;
  }
  P.cols.resize(P.rowptr[n_core]);
  for (int c = 0; c < n_core; ++c) {
    const int k = core_point[c];
    int* out = P.cols.data() + P.rowptr[c];
    int q = 0;
    bool placed = false;
    for (int j = rs[k] + 1; j < rs[k + 1]; ++j) {
      const int l = cn[j];
      if (flag[l] == -1) continue;
      if (!placed && l > k) {
        out[q++] = k;
        placed = true;
      }
      out[q++] = l;
    }
    if (!placed) out[q++] = k;
  }
  if (n_core == m) {
    // square case: SparsityPattern keeps the diagonal first (all points are C)
    for (int c = 0; c < n_core; ++c) P.cols[P.rowptr[c]] = c;
  }
  // Pt = transpose pattern, rows ascending in the coarse index
  Pt.m = m;
  Pt.n = n_core;
  Pt.rowptr.assign(m + 1, 0);
  for (int q = 0; q < P.rowptr[n_core]; ++q) Pt.rowptr[P.cols[q] + 1]++;
  for (int i = 0; i < m; ++i) Pt.rowptr[i + 1] += Pt.rowptr[i];
  Pt.cols.resize(P.rowptr[n_core]);
  {
    std::vector<int> cur(Pt.rowptr.begin(), Pt.rowptr.end() - 1);
    for (int c = 0; c < n_core; ++c)
      for (int q = P.rowptr[c]; q < P.rowptr[c + 1]; ++q) Pt.cols[cur[P.cols[q]]++] = c;
  }
  // weights, accumulated per fine point in the reference's order.
  // a_lc[q] = M(l, core_point[c]) for the Pt entry q = (l, c): it depends on
  // the entry only, so it is looked up once instead of once per neighbour i.
  // The dependency set of i (its Pt row) is a marker array: dep_at[c] is the
  // position of (i, c) in Pt while dep_row[c] == i.
  const int64_t nnz_p = (int64_t)Pt.cols.size();
  Pt.vals.assign(nnz_p, 0.0);
  std::vector<double> a_lc(nnz_p);
  for (int l = 0; l < m; ++l)
    for (int q = Pt.rowptr[l]; q < Pt.rowptr[l + 1]; ++q) a_lc[q] = entry(M, l, core_point[Pt.cols[q]]);
  std::vector<int> dep_row(n_core, -1), dep_at(n_core, 0);
  for (int i = 0; i < m; ++i) {
    for (int q = Pt.rowptr[i]; q < Pt.rowptr[i + 1]; ++q) {
      dep_row[Pt.cols[q]] = i;
      dep_at[Pt.cols[q]] = q;
    }
    const int k = core_at[i];
    if (k >= 0) {
      Pt.vals[dep_at[k]] += 1.0;
      continue;
    }
    double aii = v[rs[i]];
    for (int j = rs[i] + 1; j < rs[i + 1]; ++j)
      if (std::fabs(v[j]) < beta[i]) aii += v[j];
    for (int j = rs[i] + 1; j < rs[i + 1]; ++j) {
      const int l = cn[j];
      if (std::fabs(v[j]) < beta[i]) continue;
      if (core_at[l] >= 0) {
        if (dep_row[core_at[l]] == i) Pt.vals[dep_at[core_at[l]]] += std::fabs(v[j] / aii);
      } else {
        double d = 0.0;
        for (int i1 = Pt.rowptr[l]; i1 < Pt.rowptr[l + 1]; ++i1)
          if (dep_row[Pt.cols[i1]] == i) d += a_lc[i1];
        if (std::fabs(d * aii) < 1e-16) continue;
        for (int i1 = Pt.rowptr[l]; i1 < Pt.rowptr[l + 1]; ++i1) {
          const int c1 = Pt.cols[i1];
          if (dep_row[c1] == i) Pt.vals[dep_at[c1]] += std::fabs(v[j] * a_lc[i1] / (d * aii));
        }
      }
    }
  }
  // P values: P(c, i) received the same additions as Pt(i, c)
  P.vals.assign(P.cols.size(), 0.0);
  {
    std::vector<int> cur(P.rowptr.begin(), P.rowptr.end() - 1);
    for (int i = 0; i < m; ++i)
      for (int q = Pt.rowptr[i]; q < Pt.rowptr[i + 1]; ++q) {
        const int c = Pt.cols[q];
        // P rows are ascending in the fine index and i ascends here
        P.vals[cur[c]++] = Pt.vals[q];
      }
  }
}

// AMGSolver::lazyProject (src/AMGSolver.cpp:235-284): greedy independent set
// of "core" rows in row order; each core row aggregates itself and its
// neighbours, a neighbour l with weight 1/(number of core rows next to l).
// The reference sizes both patterns with SparsityPattern::max_entries_per_row(),
// which skips the last row (SparsityPattern.h:239-249), and
// SparsityPattern::add silently drops entries of a full row; both are kept so
// that P is the reference's.
void host_lazy_project(const HostCSR& M, HostCSR& P, HostCSR& Pt) {
  const int m = (int)M.m;
  const int* rs = M.rowptr.data();
  const int* cn = M.cols.data();
  std::vector<int> counter(m, 0), core;
  for (int i = 0; i < m; ++i) {
    if (counter[i] > 0) continue;
    for (int j = rs[i] + 1; j < rs[i + 1]; ++j) counter[cn[j]]++;
    core.push_back(i);
  }
  const int nc = (int)core.size();
  int cap = 0;
  for (int i = 1; i < m; ++i) cap = std::max(cap, rs[i] - rs[i - 1]);
  const bool square = (nc == m);
  // slot patterns with capacity `cap` per row (diagonal preset when square)
  std::vector<int> ps((size_t)nc * cap, -1), ts((size_t)m * cap, -1);
  if (square && cap > 0) {
    for (int i = 0; i < nc; ++i) ps[(size_t)i * cap] = i;
    for (int i = 0; i < m; ++i) ts[(size_t)i * cap] = i;
  }
  auto add = [cap](std::vector<int>& slots, int row, int col) {
    int* s = slots.data() + (size_t)row * cap;
    for (int k = 0; k < cap; ++k) {
      if (s[k] == col) return;
      if (s[k] == -1) {
        s[k] = col;
        return;
      }
    }
  };
  for (int i = 0; i < nc; ++i) {
    const int k = core[i];
    add(ps, i, k);
    add(ts, k, i);
    for (int j = rs[k] + 1; j < rs[k + 1]; ++j) {
      add(ps, i, cn[j]);
      add(ts, cn[j], i);
    }
  }
  auto compress = [cap, square](const std::vector<int>& slots, int rows, int ncols, HostCSR& out) {
    out.m = rows;
    out.n = ncols;
    out.rowptr.assign(rows + 1, 0);
    out.cols.clear();
    for (int i = 0; i < rows; ++i) {
      const int* s = slots.data() + (size_t)i * cap;
      int len = 0;
      while (len < cap && s[len] != -1) ++len;
      const size_t b = out.cols.size();
      out.cols.insert(out.cols.end(), s, s + len);
      std::sort(out.cols.begin() + b + (square && len > 0 ? 1 : 0), out.cols.end());
      out.rowptr[i + 1] = (int)out.cols.size();
    }
    out.vals.assign(out.cols.size(), 0.0);
  };
  compress(ps, nc, m, P);
  compress(ts, m, nc, Pt);
  auto madd = [](HostCSR& A, int i, int j, double v) {
    for (int q = A.rowptr[i]; q < A.rowptr[i + 1]; ++q)
      if (A.cols[q] == j) {
        A.vals[q] += v;
        return;
      }
  };
  for (int i = 0; i < nc; ++i) {
    const int k = core[i];
    madd(P, i, k, 1.0);
    madd(Pt, k, i, 1.0);
    for (int j = rs[k] + 1; j < rs[k + 1]; ++j) {
      const int l = cn[j];
      madd(P, i, l, 1.0 / counter[l]);
      madd(Pt, l, i, 1.0 / counter[l]);
    }
  }
}

namespace {

// Greedy colouring in row order: row i takes the smallest colour that none of
// its coupled, already coloured rows has (max_colors: the overflow class).
int greedy_color(const HostCSR& A, int max_colors, std::vector<int>& color) {
  const int m = (int)A.m;
  color.assign(m, -1);
  std::vector<int> mark(max_colors + 1, -1);
  int used = 0;
  bool overflow = false;
  for (int i = 0; i < m; ++i) {
    for (int q = A.rowptr[i] + 1; q < A.rowptr[i + 1]; ++q) {
      const int k = A.cols[q];
      if (color[k] < 0) continue;
      if (A.vals[q] == 0.0 && entry(A, k, i) == 0.0) continue;  // no coupling either way
      mark[color[k]] = i;
    }
    int c = 0;
    while (c < max_colors && mark[c] == i) ++c;
    color[i] = c;  // c == max_colors is the overflow class
    if (c == max_colors) overflow = true;
    else used = std::max(used, c + 1);
  }
  return overflow ? max_colors + 1 : used;
}

// DSATUR (Brelaz): repeatedly colours the uncoloured row whose coupled rows
// already show the most distinct colours (ties: more couplings, then the
// lower row), with the smallest colour they leave free.  On mesh graphs it
// finds colourings close to the fewest classes where row-order greedy
// colouring needs about twice as many (the 3D Kuhn-split lattice: 4 against
// 8).  Returns the colours used, or max_colors + 1 if some row found no free
// colour below max_colors (it is then left in the overflow class).
int dsatur_color(const HostCSR& A, int max_colors, std::vector<int>& color) {
  const int m = (int)A.m;
  // coupled neighbours (a nonzero entry either way), as adjacency lists
  std::vector<int> off(m + 1, 0), adj;
  adj.reserve(A.nnz());
  for (int i = 0; i < m; ++i) {
    for (int q = A.rowptr[i] + 1; q < A.rowptr[i + 1]; ++q) {
      const int k = A.cols[q];
      if (k == i || (A.vals[q] == 0.0 && entry(A, k, i) == 0.0)) continue;
      adj.push_back(k);
    }
    off[i + 1] = (int)adj.size();
  }
  color.assign(m, -1);
  std::vector<uint64_t> seen(m, 0);  // colours present among coupled rows (max_colors <= 63)
  std::vector<int> sat(m, 0);
  using Key = std::tuple<int, int, int>;  // (saturation, couplings, -row)
  std::priority_queue<Key> pq;
  for (int i = 0; i < m; ++i) pq.push(Key(0, off[i + 1] - off[i], -i));
  int used = 0;
  bool overflow = false;
  while (!pq.empty()) {
    const Key top = pq.top();
    pq.pop();
    const int i = -std::get<2>(top);
    if (color[i] >= 0 || std::get<0>(top) != sat[i]) continue;  // stale entry
    int c = 0;
    while (c < max_colors && ((seen[i] >> c) & 1u)) ++c;
    color[i] = c;
    if (c == max_colors) {
      overflow = true;
      continue;
    }
    used = std::max(used, c + 1);
    for (int q = off[i]; q < off[i + 1]; ++q) {
      const int k = adj[q];
      if (color[k] >= 0 || ((seen[k] >> c) & 1u)) continue;
      seen[k] |= uint64_t(1) << c;
      ++sat[k];
      pq.push(Key(sat[k], off[k + 1] - off[k], -k));
    }
  }
  return overflow ? max_colors + 1 : used;
}

}  // namespace

int host_color(const HostCSR& A, int max_colors, std::vector<int>& color) {
  const int greedy = greedy_color(A, max_colors, color);
  // A level that needs the overflow class keeps the row-order classes (each
  // a maximal independent set of the rows left, which keeps the l1-Jacobi
  // remainder small); otherwise DSATUR is tried for fewer classes, i.e. fewer
  // dependent steps per Gauss-Seidel sweep.
  if (greedy > max_colors || greedy <= 2 || max_colors > 63) return greedy;
  std::vector<int> ds;
  const int k = dsatur_color(A, max_colors, ds);
  if (k < greedy) {
    color.swap(ds);
    return k;
  }
  return greedy;
}

}  // namespace afp

using namespace afp;

extern "C" afp_status afp_host_coarsen(int64_t m, const int32_t* rowptr, const int32_t* cols, const double* vals,
                                       double alpha, int32_t* cf, int64_t* n_coarse, int32_t** p_rowptr,
                                       int32_t** p_cols, double** p_vals) {
  return guarded([&] {
    AFP_REQUIRE(m > 0 && rowptr && cols && vals && n_coarse && p_rowptr && p_cols && p_vals, AFP_ERR_INVALID,
                "null argument");
    HostCSR M;
    M.m = M.n = m;
    M.rowptr.assign(rowptr, rowptr + m + 1);
    M.cols.assign(cols, cols + rowptr[m]);
    M.vals.assign(vals, vals + rowptr[m]);
    std::vector<int> flag;
    HostCSR P, Pt;
    host_project(M, alpha, flag, P, Pt);
    if (cf) std::memcpy(cf, flag.data(), sizeof(int) * m);
    *n_coarse = P.m;
    *p_rowptr = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (P.m + 1)));
    *p_cols = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max<size_t>(1, P.cols.size())));
    *p_vals = static_cast<double*>(std::malloc(sizeof(double) * std::max<size_t>(1, P.vals.size())));
    AFP_REQUIRE(*p_rowptr && *p_cols && *p_vals, AFP_ERR_OUT_OF_MEMORY, "host allocation failed");
    std::memcpy(*p_rowptr, P.rowptr.data(), sizeof(int32_t) * (P.m + 1));
    std::memcpy(*p_cols, P.cols.data(), sizeof(int32_t) * P.cols.size());
    std::memcpy(*p_vals, P.vals.data(), sizeof(double) * P.vals.size());
  });
}
