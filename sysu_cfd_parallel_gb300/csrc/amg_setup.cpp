// Aggregation hierarchy for the pressure-correction preconditioner (host, once per mesh).
//
// Plain (unsmoothed) aggregation: every level groups a root row with up to maxsize-1 of its
// most strongly coupled free neighbours (strength = the symmetric weight of the connection,
// here the face coefficient area/|d.n| summed Galerkin-style on coarse levels), left-over
// rows join their strongest aggregated neighbour.  Prolongation is piecewise constant, so
// the Galerkin coarse matrix P^T A P is a plain sum of fine entries; this setup records, for
// every coarse non-zero, the fine non-zeros that add into it (in ascending order), so the
// device rebuilds the coarse values each iteration with deterministic gathers.
#include <algorithm>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "cycas_amg.h"

namespace cycas {

namespace {

void aggregate(const AmgHostLevel& L, const std::vector<double>& w, int maxsize, std::vector<int>& agg, int& na) {
  const int n = L.n;
  agg.assign(n, -1);
  na = 0;
  std::vector<std::pair<double, int>> cand;
  for (int i = 0; i < n; i++) {
    if (agg[i] >= 0) continue;
    bool free_nbhd = true;
    for (int k = L.rowptr[i]; k < L.rowptr[i + 1]; k++)
      if (L.col[k] != i && agg[L.col[k]] >= 0) {
        free_nbhd = false;
        break;
      }
    if (!free_nbhd) continue;
    cand.clear();
    for (int k = L.rowptr[i]; k < L.rowptr[i + 1]; k++)
      if (L.col[k] != i) cand.push_back({-w[k], L.col[k]});
    std::stable_sort(cand.begin(), cand.end(),
                     [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a.first < b.first; });
    agg[i] = na;
    for (int q = 0; q < (int)cand.size() && q < maxsize - 1; q++) agg[cand[q].second] = na;
    na++;
  }
  for (int i = 0; i < n; i++) {
    if (agg[i] >= 0) continue;
    int best = -1;
    double bw = -1.0;
    for (int k = L.rowptr[i]; k < L.rowptr[i + 1]; k++) {
      int j = L.col[k];
      if (j != i && agg[j] >= 0 && w[k] > bw) {
        bw = w[k];
        best = j;
      }
    }
    agg[i] = best >= 0 ? agg[best] : na++;
  }
}

}  // namespace

AmgHostHierarchy amg_build(int n, const int* rowptr, const int* col, const double* weight, int maxsize,
                           int coarse_max, int max_levels) {
  AmgHostHierarchy H;
  AmgHostLevel L0;
  L0.n = n;
  L0.rowptr.assign(rowptr, rowptr + n + 1);
  L0.col.assign(col, col + rowptr[n]);
  L0.nnz = rowptr[n];
  std::vector<double> w(weight, weight + rowptr[n]);
  H.lv.push_back(std::move(L0));
  while (H.lv.back().n > coarse_max && (int)H.lv.size() < max_levels) {
    AmgHostLevel& F = H.lv.back();
    int na = 0;
    aggregate(F, w, maxsize, F.agg, na);
    if (na >= F.n) break;  // no coarsening possible
    // coarse row -> fine rows
    F.ptptr.assign(na + 1, 0);
    for (int i = 0; i < F.n; i++) F.ptptr[F.agg[i] + 1]++;
    for (int a = 0; a < na; a++) F.ptptr[a + 1] += F.ptptr[a];
    F.ptrow.assign(F.n, 0);
    {
      std::vector<int> fill(F.ptptr.begin(), F.ptptr.end() - 1);
      for (int i = 0; i < F.n; i++) F.ptrow[fill[F.agg[i]]++] = i;
    }
    // coarse pattern
    AmgHostLevel C;
    C.n = na;
    C.rowptr.assign(na + 1, 0);
    std::vector<int> cols;
    std::vector<std::vector<int>> rows(na);
    for (int a = 0; a < na; a++) {
      cols.clear();
      for (int q = F.ptptr[a]; q < F.ptptr[a + 1]; q++) {
        int i = F.ptrow[q];
        for (int k = F.rowptr[i]; k < F.rowptr[i + 1]; k++) cols.push_back(F.agg[F.col[k]]);
      }
      std::sort(cols.begin(), cols.end());
      cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
      rows[a] = cols;
      C.rowptr[a + 1] = C.rowptr[a] + (int)cols.size();
    }
    C.nnz = C.rowptr[na];
    C.col.reserve(C.nnz);
    for (int a = 0; a < na; a++) C.col.insert(C.col.end(), rows[a].begin(), rows[a].end());
    // contribution map: fine nnz -> coarse nnz, grouped by coarse nnz (fine order ascending)
    std::vector<int> target(F.nnz);
    for (int i = 0; i < F.n; i++) {
      int a = F.agg[i];
      const int* rb = C.col.data() + C.rowptr[a];
      const int* re = C.col.data() + C.rowptr[a + 1];
      for (int k = F.rowptr[i]; k < F.rowptr[i + 1]; k++)
        target[k] = C.rowptr[a] + (int)(std::lower_bound(rb, re, F.agg[F.col[k]]) - rb);
    }
    F.cptr.assign(C.nnz + 1, 0);
    for (int k = 0; k < F.nnz; k++) F.cptr[target[k] + 1]++;
    for (int c = 0; c < C.nnz; c++) F.cptr[c + 1] += F.cptr[c];
    F.csrc.assign(F.nnz, 0);
    {
      std::vector<int> fill(F.cptr.begin(), F.cptr.end() - 1);
      for (int k = 0; k < F.nnz; k++) F.csrc[fill[target[k]]++] = k;
    }
    // coarse strength weights (off-diagonal sums)
    std::vector<double> wc(C.nnz, 0.0);
    for (int i = 0; i < F.n; i++)
      for (int k = F.rowptr[i]; k < F.rowptr[i + 1]; k++)
        if (F.col[k] != i) wc[target[k]] += w[k];
    w.swap(wc);
    H.lv.push_back(std::move(C));
  }
  for (AmgHostLevel& L : H.lv) {
    L.diag.assign(L.n, -1);
    for (int i = 0; i < L.n; i++)
      for (int k = L.rowptr[i]; k < L.rowptr[i + 1]; k++)
        if (L.col[k] == i) L.diag[i] = k;
    for (int i = 0; i < L.n; i++)
      if (L.diag[i] < 0) throw std::runtime_error("AMG level without a diagonal entry");
  }
  return H;
}

}  // namespace cycas
