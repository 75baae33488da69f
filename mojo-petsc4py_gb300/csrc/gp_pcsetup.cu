// Host-side set-up analysis for the preconditioners: orderings, the
// incomplete-factor symbolic phase (level of fill), and the dependency levels
// that order the rows of every sync-free device sweep.
//
// The symbolic phase produces the reference's factor layouts:
//   ILU  (src/factor.mojo:31-67, 70-122, 335-381): L rows first in row order,
//        then the U rows in reverse row order, each U row ascending and ending
//        on its diagonal; bdiag[i] is the diagonal slot, bdiag[n] = nnz(L) - 1.
//   IC   (src/factor.mojo:125-273, 384-412): row k holds its strictly upper
//        columns ascending, then the diagonal slot; bdiag[k] = bi[k+1] - 1.
// The level-of-fill rule is the reference's: a fill entry (i, j) reached
// through pivot p gets level lev(i, p) + lev(p, j) + 1, is kept when that is
// at most `levels`, and an entry reached several ways keeps its smallest level.
// Rows are built in flat arrays over a dense level array (ILU: a sorted
// linked list, as the reference's; IC: a sorted list of touched columns);
// the resulting patterns are the same sets in the same (ascending) order.
#include <algorithm>
#include <mutex>
#include <climits>
#include <string>
#include <vector>

#include "gp_pc.h"

namespace gp {

// Reverse Cuthill-McKee as the reference computes it (src/factor.mojo:279-332):
// breadth-first from each unvisited node in index order, neighbours visited in
// ascending index, each component reversed and appended.
int rcm_order(const std::vector<int>& rowptr, const std::vector<int>& colind, int n,
              std::vector<int>& perm) {
  perm.assign(n, 0);
  std::vector<char> seen(n, 0);
  std::vector<int> queue(n);
  int filled = 0;
  for (int start = 0; start < n; start++) {
    if (seen[start]) continue;
    seen[start] = 1;
    int head = 0, tail = 0;
    queue[tail++] = start;
    while (head < tail) {
      int node = queue[head++];
      for (int j = rowptr[node]; j < rowptr[node + 1]; j++) {
        int c = colind[j];
        if (!seen[c]) {
          seen[c] = 1;
          queue[tail++] = c;
        }
      }
    }
    for (int i = 0; i < tail; i++) perm[filled + i] = queue[tail - 1 - i];
    filled += tail;
  }
  return GP_OK;
}

// Multicolour ordering: greedy colouring of the symmetrised graph in index
// order (each row takes the smallest colour none of its neighbours has), then
// the rows colour by colour, ascending within a colour.  A factor in this
// ordering has one dependency level per colour in each triangular solve (two
// for a 5- or 7-point stencil), which is what the mixed-precision form's
// bandwidth-bound triangle passes want: with as many passes as colours they
// apply the triangles exactly.  No counterpart in the reference (it offers
// natural and RCM orderings).
int color_order(const std::vector<int>& rowptr, const std::vector<int>& colind, int n,
                std::vector<int>& perm, int* ncolors) {
  std::vector<int> tp(n + 1, 0), tc(rowptr[n]);
  for (int k = 0; k < rowptr[n]; k++) tp[colind[k] + 1]++;
  for (int i = 0; i < n; i++) tp[i + 1] += tp[i];
  std::vector<int> fill(tp.begin(), tp.end() - 1);
  for (int i = 0; i < n; i++)
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) tc[fill[colind[k]]++] = i;
  std::vector<int> color(n, -1), mark;
  int nc = 0;
  for (int i = 0; i < n; i++) {
    auto see = [&](int j) {
      if (j != i && color[j] >= 0) mark[color[j]] = i;
    };
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) see(colind[k]);
    for (int k = tp[i]; k < tp[i + 1]; k++) see(tc[k]);
    int c = 0;
    while (c < nc && mark[c] == i) c++;
    if (c == nc) {
      nc++;
      mark.push_back(-1);
    }
    color[i] = c;
  }
  std::vector<int> start(nc + 1, 0);
  for (int i = 0; i < n; i++) start[color[i] + 1]++;
  for (int c = 0; c < nc; c++) start[c + 1] += start[c];
  perm.assign(n, 0);
  for (int i = 0; i < n; i++) perm[start[color[i]]++] = i;
  if (ncolors) *ncolors = nc;
  return GP_OK;
}

// Rows of a symbolic factor in flat form: row i is cols[rs[i] .. rs[i+1])
// ascending, with their levels in lv; nL[i] counts the strictly lower ones.
struct SymRows {
  std::vector<int> rs, cols, lv, nL;
};

// The permuted row i of A: ascending distinct columns ic[colind] of row r[i].
static void permuted_row(const Csr* A, const std::vector<int>& r, const std::vector<int>& ic,
                         int i, std::vector<int>& out) {
  out.clear();
  const int ri = r[i];
  for (int j = A->h_rowptr[ri]; j < A->h_rowptr[ri + 1]; j++) out.push_back(ic[A->h_colind[j]]);
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
}

// Level 0: every row is the operator's permuted row, so rows are independent:
// counted on host threads, prefix-summed, then filled on host threads (the
// same rows and levels as the general loop).  `keep(i, c)` selects the
// columns a row keeps; nL (when given) counts each row's columns below i.
template <class Keep>
static int rows_level0(const Csr* A, const std::vector<int>& r, const std::vector<int>& ic,
                       Keep keep, SymRows& R, bool need_diag, const char* who) {
  const int n = A->n;
  R.rs.assign(n + 1, 0);
  R.nL.assign(n, 0);
  std::vector<int> missing(1, -1);
  std::mutex mu;
  host_parallel_for(n, [&](int64_t i0, int64_t i1) {
    std::vector<int> row;
    for (int i = (int)i0; i < (int)i1; i++) {
      permuted_row(A, r, ic, i, row);
      if (need_diag && !std::binary_search(row.begin(), row.end(), i)) {
        // the first such row in the factor's order, as a row-by-row pass finds
        std::lock_guard<std::mutex> g(mu);
        if (missing[0] < 0 || i < missing[0]) missing[0] = i;
      }
      int cnt = 0, low = 0;
      for (int c : row)
        if (keep(i, c)) {
          cnt++;
          low += c < i;
        }
      R.rs[i + 1] = cnt;
      R.nL[i] = low;
    }
  });
  if (missing[0] >= 0) {
    set_error(std::string(who) + ": row " + std::to_string(r[missing[0]]) +
              " has no diagonal entry");
    return GP_ERR_ARG;
  }
  int64_t tot = 0;
  for (int i = 0; i < n; i++) {
    tot += R.rs[i + 1];
    if (tot > INT32_MAX - 1 - (int64_t)n) {
      set_error(std::string(who) + " factor too large for 32-bit indices");
      return GP_ERR_ARG;
    }
    R.rs[i + 1] = (int)tot;
  }
  R.cols.assign(tot, 0);
  R.lv.assign(tot, 0);
  host_parallel_for(n, [&](int64_t i0, int64_t i1) {
    std::vector<int> row;
    for (int i = (int)i0; i < (int)i1; i++) {
      permuted_row(A, r, ic, i, row);
      int q = R.rs[i];
      for (int c : row)
        if (keep(i, c)) R.cols[q++] = c;
    }
  });
  return GP_OK;
}

// Row offsets are int32 (the factor's device indices): the slot count is
// checked in 64 bits before each narrowing, against `limit`.
static bool slots_fit(size_t count, int64_t limit, const char* who) {
  if ((int64_t)count <= limit) return true;
  set_error(std::string(who) + " factor too large for 32-bit indices");
  return false;
}

// ILU(levels) rows.  Row i starts from A's permuted row at level 0; its
// pivots p < i are visited in ascending order, fill included (a fill column
// reached through p is always > p), and each adds U(p, :) past the diagonal
// at level lev(i, p) + lev(p, j) + 1.  The row is a sorted linked list over
// a dense level array, so no per-row allocation is made.
static int ilu_rows_flat(const Csr* A, int levels, const std::vector<int>& r,
                         const std::vector<int>& ic, SymRows& R) {
  const int n = A->n;
  if (levels == 0)
    return rows_level0(A, r, ic, [](int, int) { return true; }, R, true, "ILU");
  R.rs.assign(n + 1, 0);
  R.nL.assign(n, 0);
  R.cols.clear();
  R.lv.clear();
  R.cols.reserve(A->nnz);
  R.lv.reserve(A->nnz);
  std::vector<int> lev(n, -1), nxt(levels > 0 ? n : 0), row;
  for (int i = 0; i < n; i++) {
    permuted_row(A, r, ic, i, row);
    if (!std::binary_search(row.begin(), row.end(), i)) {
      set_error("ILU: row " + std::to_string(r[i]) + " has no diagonal entry");
      return GP_ERR_ARG;
    }
    if (levels == 0) {
      R.nL[i] = (int)(std::lower_bound(row.begin(), row.end(), i) - row.begin());
      R.cols.insert(R.cols.end(), row.begin(), row.end());
      R.lv.insert(R.lv.end(), row.size(), 0);
      if (!slots_fit(R.cols.size(), INT32_MAX - 1, "ILU")) return GP_ERR_ARG;
      R.rs[i + 1] = (int)R.cols.size();
      continue;
    }
    // list end marker: n (above every column)
    const int head = row[0];
    for (size_t q = 0; q < row.size(); q++) {
      lev[row[q]] = 0;
      nxt[row[q]] = q + 1 < row.size() ? row[q + 1] : n;
    }
    for (int p = head; p < i; p = nxt[p]) {
      const int lip = lev[p];
      int cur = p;  // U(p, :) is ascending, so the insertion point only moves on
      for (int q = R.rs[p] + R.nL[p] + 1; q < R.rs[p + 1]; q++) {
        const int j = R.cols[q];
        const int l = R.lv[q] + lip + 1;
        if (l > levels) continue;
        if (lev[j] < 0) {
          while (nxt[cur] < j) cur = nxt[cur];
          nxt[j] = nxt[cur];
          nxt[cur] = j;
          lev[j] = l;
        } else if (lev[j] > l) {
          lev[j] = l;
        }
      }
    }
    int cnt = 0;
    for (int c = head; c != n; c = nxt[c]) {
      R.cols.push_back(c);
      R.lv.push_back(lev[c]);
      if (c < i) cnt++;
      lev[c] = -1;
    }
    R.nL[i] = cnt;
    if (!slots_fit(R.cols.size(), INT32_MAX - 1, "ILU")) return GP_ERR_ARG;
    R.rs[i + 1] = (int)R.cols.size();
  }
  return GP_OK;
}

// IC(levels) rows: the strictly upper part of row k, from A's permuted row at
// level 0 and the fill through every earlier row p holding column k, each
// adding its columns past k at level lev(p, k) + lev(p, j) + 1 (the smallest
// level is kept; the set and the levels do not depend on the order in which
// the rows p are visited).
static int icc_rows_flat(const Csr* A, int levels, const std::vector<int>& r,
                         const std::vector<int>& ic, SymRows& R) {
  const int n = A->n;
  if (levels == 0)
    return rows_level0(A, r, ic, [](int k, int c) { return c > k; }, R, false, "IC");
  R.rs.assign(n + 1, 0);
  R.nL.assign(n, 0);
  R.cols.clear();
  R.lv.clear();
  R.cols.reserve(A->nnz);
  R.lv.reserve(A->nnz);
  std::vector<int> lev(n, -1), row, touched;
  // rows p holding column k: per-column lists of (p, lev(p, k)) entries
  std::vector<int> chead(levels > 0 ? n : 0, -1), enext, erow, elev;
  for (int k = 0; k < n; k++) {
    permuted_row(A, r, ic, k, row);
    touched.clear();
    for (int c : row)
      if (c > k) {
        lev[c] = 0;
        touched.push_back(c);
      }
    if (levels > 0) {
      for (int e = chead[k]; e >= 0; e = enext[e]) {
        const int p = erow[e], lpk = elev[e];
        for (int q = R.rs[p]; q < R.rs[p + 1]; q++) {
          const int j = R.cols[q];
          if (j <= k) continue;
          const int l = R.lv[q] + lpk + 1;
          if (l > levels) continue;
          if (lev[j] < 0) {
            lev[j] = l;
            touched.push_back(j);
          } else if (lev[j] > l) {
            lev[j] = l;
          }
        }
      }
      std::sort(touched.begin(), touched.end());
    }
    for (int c : touched) {
      R.cols.push_back(c);
      R.lv.push_back(lev[c]);
      if (levels > 0) {
        if (!slots_fit(erow.size() + 1, INT32_MAX - 1, "IC")) return GP_ERR_ARG;
        enext.push_back(chead[c]);
        erow.push_back(k);
        elev.push_back(lev[c]);
        chead[c] = (int)erow.size() - 1;
      }
      lev[c] = -1;
    }
    // the diagonal slots (one a row) come on top of the strict rows
    if (!slots_fit(R.cols.size(), (int64_t)INT32_MAX - 1 - n, "IC")) return GP_ERR_ARG;
    R.rs[k + 1] = (int)R.cols.size();
  }
  return GP_OK;
}

static void rows_to_pairs(const SymRows& R, int n,
                          std::vector<std::vector<std::pair<int, int>>>& rows) {
  rows.assign(n, {});
  for (int i = 0; i < n; i++)
    for (int q = R.rs[i]; q < R.rs[i + 1]; q++) rows[i].emplace_back(R.cols[q], R.lv[q]);
}

// Rows of the ILU(levels) pattern: ascending (column, level) pairs of each
// permuted row, and the count of strictly lower entries in nL.
int ilu_symbolic_rows(const Csr* A, int levels, const std::vector<int>& r,
                      const std::vector<int>& ic,
                      std::vector<std::vector<std::pair<int, int>>>& rows, std::vector<int>& nL) {
  SymRows R;
  GP_TRY(ilu_rows_flat(A, levels, r, ic, R));
  rows_to_pairs(R, A->n, rows);
  nL = R.nL;
  return GP_OK;
}

int ilu_symbolic(const Csr* A, int levels, const std::vector<int>& r, const std::vector<int>& ic,
                 FactorPattern& out) {
  const int n = A->n;
  SymRows R;
  GP_TRY(ilu_rows_flat(A, levels, r, ic, R));
  // reference layout
  const int64_t total = R.rs[n];
  if (total > INT32_MAX - 1) {
    set_error("ILU factor too large for 32-bit indices");
    return GP_ERR_ARG;
  }
  out.bi.assign(n + 1, 0);
  for (int i = 0; i < n; i++) out.bi[i + 1] = out.bi[i] + R.nL[i];
  out.nnz = (int)total;
  out.bj.assign(std::max<int64_t>(total, 1), 0);
  out.bdiag.assign(n + 1, 0);
  // L rows ascending, then the U rows from the last row up, each ending on its
  // diagonal: bdiag by a suffix sum, then every row copied on host threads
  const int nLtot = out.bi[n];
  out.bdiag[n] = nLtot - 1;
  for (int i = n - 1; i >= 0; i--)
    out.bdiag[i] = out.bdiag[i + 1] + (R.rs[i + 1] - R.rs[i] - R.nL[i] - 1) + 1;
  host_parallel_for(n, [&](int64_t i0, int64_t i1) {
    for (int i = (int)i0; i < (int)i1; i++) {
      for (int q = 0; q < R.nL[i]; q++) out.bj[out.bi[i] + q] = R.cols[R.rs[i] + q];
      const int nz = R.rs[i + 1] - R.rs[i] - R.nL[i] - 1;
      int k = out.bdiag[i + 1] + 1;  // row i's U block starts right after row i+1's diagonal
      for (int q = 0; q < nz; q++) out.bj[k++] = R.cols[R.rs[i] + R.nL[i] + 1 + q];
      out.bj[k] = i;
    }
  });
  out.r = r;
  out.ic = ic;
  return GP_OK;
}

// Rows of the IC(levels) pattern: the strictly upper (column, level) pairs of
// each permuted row, ascending.
int icc_symbolic_rows(const Csr* A, int levels, const std::vector<int>& r,
                      const std::vector<int>& ic,
                      std::vector<std::vector<std::pair<int, int>>>& rows) {
  SymRows R;
  GP_TRY(icc_rows_flat(A, levels, r, ic, R));
  rows_to_pairs(R, A->n, rows);
  return GP_OK;
}

int icc_symbolic(const Csr* A, int levels, const std::vector<int>& r, const std::vector<int>& ic,
                 FactorPattern& out) {
  const int n = A->n;
  SymRows R;
  GP_TRY(icc_rows_flat(A, levels, r, ic, R));
  const int64_t total = (int64_t)R.rs[n] + n;
  if (total > INT32_MAX - 1) {
    set_error("IC factor too large for 32-bit indices");
    return GP_ERR_ARG;
  }
  out.bi.assign(n + 1, 0);
  out.nnz = (int)total;
  out.bj.assign(std::max<int64_t>(total, 1), 0);
  out.bdiag.assign(n + 1, 0);
  // row k: its strict upper columns, then its diagonal slot (k rows before it)
  host_parallel_for(n, [&](int64_t k0, int64_t k1) {
    for (int k = (int)k0; k < (int)k1; k++) {
      int pos = R.rs[k] + k;
      out.bi[k] = pos;
      for (int q = R.rs[k]; q < R.rs[k + 1]; q++) out.bj[pos++] = R.cols[q];
      out.bdiag[k] = pos;
      out.bj[pos] = k;
    }
  });
  out.bi[n] = (int)total;
  out.bdiag[n] = (int)total;
  out.r = r;
  out.ic = ic;
  return GP_OK;
}

void level_order(int n, const std::vector<int>& dptr, const std::vector<int>& dcol, bool forward,
                 std::vector<int>& order, int* nlevels) {
  std::vector<int> lev(n, 0);
  int maxlev = 0;
  if (forward) {
    for (int i = 0; i < n; i++) {
      int l = 0;
      for (int e = dptr[i]; e < dptr[i + 1]; e++) l = std::max(l, lev[dcol[e]] + 1);
      lev[i] = l;
      maxlev = std::max(maxlev, l);
    }
  } else {
    for (int i = n - 1; i >= 0; i--) {
      int l = 0;
      for (int e = dptr[i]; e < dptr[i + 1]; e++) l = std::max(l, lev[dcol[e]] + 1);
      lev[i] = l;
      maxlev = std::max(maxlev, l);
    }
  }
  std::vector<int> cnt(maxlev + 2, 0);
  for (int i = 0; i < n; i++) cnt[lev[i] + 1]++;
  for (int l = 0; l <= maxlev; l++) cnt[l + 1] += cnt[l];
  order.assign(std::max(n, 1), 0);
  if (forward) {
    for (int i = 0; i < n; i++) order[cnt[lev[i]]++] = i;
  } else {
    for (int i = n - 1; i >= 0; i--) order[cnt[lev[i]]++] = i;
  }
  *nlevels = n ? maxlev + 1 : 0;
}

}  // namespace gp
