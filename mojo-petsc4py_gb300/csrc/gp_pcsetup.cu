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
// Sets of columns are kept in ordered maps rather than the reference's linked
// lists; the resulting patterns are the same sets in the same (ascending)
// order.
#include <algorithm>
#include <map>
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

// Rows of the ILU(levels) pattern: ascending (column, level) pairs of each
// permuted row, and the count of strictly lower entries in nL.
int ilu_symbolic_rows(const Csr* A, int levels, const std::vector<int>& r,
                      const std::vector<int>& ic,
                      std::vector<std::vector<std::pair<int, int>>>& rows, std::vector<int>& nL) {
  const int n = A->n;
  const auto& rp = A->h_rowptr;
  const auto& ci = A->h_colind;
  rows.assign(n, {});
  nL.assign(n, 0);
  for (int i = 0; i < n; i++) {
    std::map<int, int> row;
    const int ri = r[i];
    for (int j = rp[ri]; j < rp[ri + 1]; j++) row.emplace(ic[ci[j]], 0);
    if (!row.count(i)) {
      set_error("ILU: row " + std::to_string(ri) + " has no diagonal entry");
      return GP_ERR_ARG;
    }
    if (levels > 0) {
      for (auto it = row.begin(); it != row.end() && it->first < i; ++it) {
        const int p = it->first, lip = it->second;
        const auto& prow = rows[p];
        for (int q = nL[p] + 1; q < (int)prow.size(); q++) {  // U(p, :) past the diagonal
          const int j = prow[q].first;
          const int lev = prow[q].second + lip + 1;
          if (lev > levels) continue;
          auto f = row.find(j);
          if (f == row.end())
            row.emplace(j, lev);
          else if (f->second > lev)
            f->second = lev;
        }
      }
    }
    rows[i].assign(row.begin(), row.end());
    int cnt = 0;
    while (cnt < (int)rows[i].size() && rows[i][cnt].first < i) cnt++;
    nL[i] = cnt;
  }
  return GP_OK;
}

int ilu_symbolic(const Csr* A, int levels, const std::vector<int>& r, const std::vector<int>& ic,
                 FactorPattern& out) {
  const int n = A->n;
  std::vector<std::vector<std::pair<int, int>>> rows;
  std::vector<int> nL;
  GP_TRY(ilu_symbolic_rows(A, levels, r, ic, rows, nL));
  // reference layout
  out.bi.assign(n + 1, 0);
  int64_t total = 0;
  for (int i = 0; i < n; i++) {
    out.bi[i + 1] = out.bi[i] + nL[i];
    total += rows[i].size();
  }
  if (total > INT32_MAX - 1) {
    set_error("ILU factor too large for 32-bit indices");
    return GP_ERR_ARG;
  }
  out.nnz = (int)total;
  out.bj.assign(std::max<int64_t>(total, 1), 0);
  out.bdiag.assign(n + 1, 0);
  for (int i = 0; i < n; i++)
    for (int q = 0; q < nL[i]; q++) out.bj[out.bi[i] + q] = rows[i][q].first;
  const int nLtot = out.bi[n];
  out.bdiag[n] = nLtot - 1;
  int k = nLtot;
  for (int i = n - 1; i >= 0; i--) {
    const int nz = (int)rows[i].size() - nL[i] - 1;
    for (int q = 0; q < nz; q++) out.bj[k++] = rows[i][nL[i] + 1 + q].first;
    out.bj[k++] = i;
    out.bdiag[i] = out.bdiag[i + 1] + nz + 1;
  }
  out.r = r;
  out.ic = ic;
  return GP_OK;
}

// Rows of the IC(levels) pattern: the strictly upper (column, level) pairs of
// each permuted row, ascending.
int icc_symbolic_rows(const Csr* A, int levels, const std::vector<int>& r,
                      const std::vector<int>& ic,
                      std::vector<std::vector<std::pair<int, int>>>& rows) {
  const int n = A->n;
  const auto& rp = A->h_rowptr;
  const auto& ci = A->h_colind;
  rows.assign(n, {});
  std::vector<std::vector<std::pair<int, int>>> colsrc(n);  // column k <- (prow, level)
  for (int k = 0; k < n; k++) {
    std::map<int, int> row;
    const int rk = r[k];
    for (int j = rp[rk]; j < rp[rk + 1]; j++) {
      const int c = ic[ci[j]];
      if (c > k) row.emplace(c, 0);
    }
    if (levels > 0) {
      for (const auto& src : colsrc[k]) {
        const int p = src.first, lpk = src.second;
        for (const auto& e : rows[p]) {
          if (e.first <= k) continue;
          const int lev = e.second + lpk + 1;
          if (lev > levels) continue;
          auto f = row.find(e.first);
          if (f == row.end())
            row.emplace(e.first, lev);
          else if (f->second > lev)
            f->second = lev;
        }
      }
    }
    rows[k].assign(row.begin(), row.end());
    for (const auto& e : rows[k]) colsrc[e.first].emplace_back(k, e.second);
  }
  return GP_OK;
}

int icc_symbolic(const Csr* A, int levels, const std::vector<int>& r, const std::vector<int>& ic,
                 FactorPattern& out) {
  const int n = A->n;
  std::vector<std::vector<std::pair<int, int>>> rows;
  GP_TRY(icc_symbolic_rows(A, levels, r, ic, rows));
  out.bi.assign(n + 1, 0);
  int64_t total = 0;
  for (int k = 0; k < n; k++) total += rows[k].size() + 1;
  if (total > INT32_MAX - 1) {
    set_error("IC factor too large for 32-bit indices");
    return GP_ERR_ARG;
  }
  out.nnz = (int)total;
  out.bj.assign(std::max<int64_t>(total, 1), 0);
  out.bdiag.assign(n + 1, 0);
  int pos = 0;
  for (int k = 0; k < n; k++) {
    out.bi[k] = pos;
    for (const auto& e : rows[k]) out.bj[pos++] = e.first;
    out.bdiag[k] = pos;
    out.bj[pos++] = k;
  }
  out.bi[n] = pos;
  out.bdiag[n] = pos;
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
