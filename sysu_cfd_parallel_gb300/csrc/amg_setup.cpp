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
#include <exception>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "cycas_amg.h"
#include "host_threads.h"

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

// ------------------------------------------------------------------ multi-case upload
namespace cycas {

namespace {

int align16(long b) { return (int)((b + 15) / 16 * 16); }

// SELL-32 copy of a level's pattern (AmgDevLevel::sell_*): rows ordered by length (longest
// first, ties in row order), slices of 32 consecutive positions padded to their longest row
struct Sell {
  std::vector<int> ptr, src;
  std::vector<unsigned short> col, row;
};
Sell sell32(const AmgHostLevel& L) {
  Sell S;
  const int ns = (L.n + 31) / 32;
  auto len = [&](int i) { return L.rowptr[i + 1] - L.rowptr[i]; };
  std::vector<int> order(L.n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return len(a) > len(b); });
  S.row.assign(32L * ns, 0);
  for (int p = 0; p < L.n; p++) S.row[p] = (unsigned short)order[p];
  S.ptr.assign(ns + 1, 0);
  for (int s = 0; s < ns; s++) S.ptr[s + 1] = S.ptr[s] + 32 * len(order[32 * s]);  // the slice's first row is its longest
  S.col.assign(S.ptr[ns], 0);
  S.src.assign(S.ptr[ns], -1);
  for (int s = 0; s < ns; s++) {
    const int w = (S.ptr[s + 1] - S.ptr[s]) / 32;
    for (int lane = 0; lane < 32; lane++) {
      const int p = 32 * s + lane;
      if (p >= L.n) continue;
      const int i = order[p];
      for (int k = 0; k < w; k++) {
        const int e = S.ptr[s] + 32 * k + lane;
        if (k < len(i)) {
          S.col[e] = (unsigned short)L.col[L.rowptr[i] + k];
          S.src[e] = L.rowptr[i] + k;
        } else {
          S.col[e] = (unsigned short)i;  // padding: the row's own column, value 0
        }
      }
    }
  }
  return S;
}

// tail = the shortest suffix of levels ending at the coarsest whose arrays fit the budget;
// columns are stored in 16 bits, so a tail level has fewer than 65536 rows.  sell[l]: entries of
// level l's SELL-32 layout
TailLayout tail_layout(const std::vector<int>& n, const std::vector<int>& sell) {
  TailLayout T{};
  const int L = (int)n.size();
  auto level_bytes = [&](int l) -> long {
    if (l == L - 1) return align16(4L * n[l] * n[l]) + 2L * align16(4L * n[l]);
    const long ns = (n[l] + 31) / 32;
    return align16(4L * (ns + 1)) + align16(2L * sell[l]) + align16(4L * sell[l]) + align16(64L * ns) +
           align16(4L * n[l]) +
           align16(4L * n[l]) + align16(4L * (n[l + 1] + 1)) + align16(4L * n[l]) + 3L * align16(4L * n[l]);
  };
  long total = level_bytes(L - 1);
  int t = L - 1;
  while (t > 0 && n[t - 1] < 65536 && total + level_bytes(t - 1) <= kAmgTailBudget) total += level_bytes(--t);
  T.tail = t;
  int off = 0;
  auto take = [&](long b) {
    int o = off;
    off += align16(b);
    return o;
  };
  for (int l = 0; l < kAmgMaxLevels; l++) T.lv[l] = TailLevelOff{-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
  for (int l = t; l < L; l++) {
    TailLevelOff& o = T.lv[l];
    if (l + 1 < L) {
      o.rowptr = take(4L * ((n[l] + 31) / 32 + 1));
      o.col = take(2L * sell[l]);
      o.val = take(4L * sell[l]);
      o.perm = take(64L * ((n[l] + 31) / 32));
      o.wdinv = take(4L * n[l]);
      o.agg = take(4L * n[l]);
      o.ptptr = take(4L * (n[l + 1] + 1));
      o.ptrow = take(4L * n[l]);
      o.T = take(4L * n[l]);
    } else {
      T.inv = take(4L * n[l] * n[l]);
    }
    o.R = take(4L * n[l]);
    o.X = take(4L * n[l]);
  }
  T.bytes = off;
  return T;
}

// entries of a level's SELL-32 layout (sell32(L).col.size()) without building it: 32 times the
// length of every 32nd row in decreasing row length, from a histogram of the row lengths
long sell_entries(const AmgHostLevel& L) {
  int mx = 0;
  for (int i = 0; i < L.n; i++) mx = std::max(mx, L.rowptr[i + 1] - L.rowptr[i]);
  std::vector<long> cnt(mx + 1, 0);
  for (int i = 0; i < L.n; i++) cnt[L.rowptr[i + 1] - L.rowptr[i]]++;
  long total = 0, p = 0;  // positions [p, p + cnt[v]) of the decreasing order have length v
  for (int v = mx; v >= 0; v--) {
    const long first = (p + 31) / 32 * 32;  // the first slice head at or after p
    if (first < p + cnt[v]) total += 32L * v * ((p + cnt[v] - 1 - first) / 32 + 1);
    p += cnt[v];
  }
  return total;
}

}  // namespace

void amg_setup_cases(AmgHostView& v, int n, const int* rowptr, const int* col, const double* weight,
                     const int* rowptr_dev, const int* col_dev, const int* diag_dev, const double* val64_dev,
                     const std::vector<int>& lo, const std::vector<int>& hi, AmgUploader& up,
                     std::vector<std::shared_ptr<const AmgHostHierarchy>>* cache) {
  const int nc = (int)lo.size();
  if (cache && (int)cache->size() != nc) throw std::runtime_error("AMG: cache size differs from the case count");
  std::vector<std::shared_ptr<const AmgHostHierarchy>> Hp(nc);
  std::vector<int> case_nnz0(nc + 1, 0);  // first level-0 entry of every case (cases are contiguous)
  int D = 0;
  // the hierarchies of the cases not in the cache, built in parallel (they are independent)
  std::vector<long> build_work(nc, 0);
  for (int c = 0; c < nc; c++) {
    const bool in_range = hi[c] - lo[c] >= 1 && hi[c] <= n && lo[c] >= 0;
    if (in_range && !(cache && (*cache)[c]) && rowptr) build_work[c] = rowptr[hi[c]] - rowptr[lo[c]];
  }
  std::vector<std::exception_ptr> build_err = for_each_case(build_work, [&](int c) {
    const int l0 = lo[c], nr = hi[c] - lo[c];
    if (nr < 1 || hi[c] > n || l0 < 0) throw std::runtime_error("AMG: empty or out-of-range case");
    if (cache && (*cache)[c]) {
      Hp[c] = (*cache)[c];
      if (Hp[c]->lv.empty() || Hp[c]->lv[0].n != nr) throw std::runtime_error("AMG: cached hierarchy of another case");
      return;
    }
    if (!rowptr || !col || !weight) throw std::runtime_error("AMG: pattern needed to build a hierarchy");
    const int k0 = rowptr[l0];
    std::vector<int> rp(nr + 1), cl(rowptr[hi[c]] - k0);
    std::vector<double> w(cl.size());
    for (int i = 0; i <= nr; i++) rp[i] = rowptr[l0 + i] - k0;
    for (size_t k = 0; k < cl.size(); k++) {
      const int j = col[k0 + k];
      if (j < l0 || j >= hi[c]) throw std::runtime_error("AMG: the pressure system couples two cases");
      cl[k] = j - l0;
      w[k] = weight[k0 + k];
    }
    auto h = std::make_shared<AmgHostHierarchy>(
        amg_build(nr, rp.data(), cl.data(), w.data(), 4, kAmgCoarseMax, kAmgMaxLevels));
    if (h->lv.back().n > kAmgCoarseMax) throw std::runtime_error("aggregation did not reach a small enough coarsest level");
    Hp[c] = h;
  });
  // case by case, as if built in order: a case's build error comes before its own contiguity check
  for (int c = 0; c < nc; c++) {
    if (build_err[c]) std::rethrow_exception(build_err[c]);
    if (cache) (*cache)[c] = Hp[c];
    case_nnz0[c + 1] = case_nnz0[c] + Hp[c]->lv[0].nnz;
    if (rowptr && rowptr[lo[c]] != case_nnz0[c]) throw std::runtime_error("AMG: cases are not contiguous in the pattern");
    D = std::max(D, (int)Hp[c]->lv.size());
  }
  auto H = [&](int c) -> const AmgHostHierarchy& { return *Hp[c]; };
  v.ncases = nc;
  v.val64 = val64_dev;
  v.dep.assign(D, AmgHostView::Depth{});
  v.levels.assign(nc, std::vector<AmgDevLevel>());
  v.cases.assign(nc, AmgCaseDesc{});
  for (int c = 0; c < nc; c++) v.levels[c].assign(H(c).lv.size(), AmgDevLevel{});

  // offsets of every case's slice per depth (cases without the level get none)
  std::vector<std::vector<int>> row_off(D, std::vector<int>(nc, -1)), nnz_off(D, std::vector<int>(nc, -1)),
      rp_off(D, std::vector<int>(nc, -1)), pt_off(D, std::vector<int>(nc, -1)), ptr_off(D, std::vector<int>(nc, -1)),
      cp_off(D, std::vector<int>(nc, -1));
  std::vector<int> nrows(D, 0), nnzs(D, 0), nrp(D, 0), npt(D, 0), nptr(D, 0), ncp(D, 0);
  for (int l = 0; l < D; l++)
    for (int c = 0; c < nc; c++) {
      if ((int)H(c).lv.size() <= l) continue;
      const AmgHostLevel& L = H(c).lv[l];
      row_off[l][c] = l == 0 ? lo[c] : nrows[l];
      nnz_off[l][c] = l == 0 ? case_nnz0[c] : nnzs[l];
      rp_off[l][c] = nrp[l];
      if (l > 0) {
        nrows[l] += L.n;
        nnzs[l] += L.nnz;
        nrp[l] += L.n + 1;
      }
      if (l + 1 < (int)H(c).lv.size()) {
        pt_off[l][c] = npt[l];
        npt[l] += (int)L.ptptr.size();
        ptr_off[l][c] = nptr[l];
        nptr[l] += L.n;
        cp_off[l][c] = ncp[l];
        ncp[l] += (int)L.csrc.size();
      }
    }
  nrows[0] = n;
  nnzs[0] = case_nnz0[nc];

  // host arrays per depth; every case fills its own slices (in parallel), then they are uploaded
  // in a fixed order
  for (int l = 0; l < D; l++) {
    const bool next = l + 1 < D;
    std::vector<int> rp(l > 0 ? nrp[l] : 0), cl(l > 0 ? nnzs[l] : 0), dg(l > 0 ? nrows[l] : 0);
    std::vector<int> ag(l == 0 ? n : nrows[l], -1), pp(npt[l]), pr(nptr[l]);
    // Galerkin map into depth l+1, in the depth l+1 order of cases: coarse entry e of case c is
    // entry nnz_off[l+1][c] + e of depth l+1 and sums the fine entries csrc[cptr[.]..cptr[.+1])
    std::vector<int> cptr(next ? nnzs[l + 1] + 1 : 0);
    if (next) cptr[0] = 0;
    // The arrays of one entry per entry of the depth are written only by the cases (the cases'
    // entries tile the depth, level 0 included: they are checked contiguous), so they start
    // uninitialised: csrc, the row of every diagonal entry (-1 elsewhere; the setup kernels write
    // w / a_ii where they make a_ii) and agg[col[k]] (cases without a coarser level: unused zeros).
    const long ne = std::max(1, nnzs[l]);
    std::unique_ptr<int[]> csrc(new int[next ? std::max(1, ncp[l]) : 1]);
    std::unique_ptr<int[]> dr(new int[ne]), ac(new int[ne]);
    dr[0] = -1;  // the depth has entries; this only covers an empty one
    ac[0] = 0;
    std::vector<long> fill_work(nc, 0);
    for (int c = 0; c < nc; c++)
      if ((int)H(c).lv.size() > l) fill_work[c] = H(c).lv[l].nnz;
    rethrow_first(for_each_case(fill_work, [&](int c) {
      if ((int)H(c).lv.size() <= l) return;
      const AmgHostLevel& L = H(c).lv[l];
      const int ro = row_off[l][c], no = nnz_off[l][c];
      if (l > 0) {
        std::copy(L.rowptr.begin(), L.rowptr.end(), rp.begin() + rp_off[l][c]);
        std::copy(L.col.begin(), L.col.end(), cl.begin() + no);
        for (int i = 0; i < L.n; i++) dg[ro + i] = L.diag[i] + no;
      }
      std::fill(dr.get() + no, dr.get() + no + L.nnz, -1);
      for (int i = 0; i < L.n; i++) dr[L.diag[i] + no] = ro + i;
      if ((int)H(c).lv.size() <= l + 1) {
        std::fill(ac.get() + no, ac.get() + no + L.nnz, 0);
        return;
      }
      for (int i = 0; i < L.n; i++) ag[ro + i] = L.agg[i];
      std::copy(L.ptptr.begin(), L.ptptr.end(), pp.begin() + pt_off[l][c]);
      const int shift = l == 0 ? lo[c] : 0;
      for (int i = 0; i < L.n; i++) pr[ptr_off[l][c] + i] = L.ptrow[i] + shift;
      const int e0 = nnz_off[l + 1][c], base = cp_off[l][c];
      for (size_t q = 1; q < L.cptr.size(); q++) cptr[e0 + q] = base + L.cptr[q];
      for (size_t k = 0; k < L.csrc.size(); k++) csrc[base + k] = L.csrc[k] + no;
      for (int k = 0; k < L.nnz; k++) ac[no + k] = L.agg[L.col[k]];
    }));
    AmgHostView::Depth& d = v.dep[l];
    d.nrows = nrows[l];
    d.nnz = nnzs[l];
    const int* d_rp = l == 0 ? rowptr_dev : up.upload_int(rp.data(), (long)rp.size());
    const int* d_cl = l == 0 ? col_dev : up.upload_int(cl.data(), (long)cl.size());
    d.diag = l == 0 ? diag_dev : up.upload_int(dg.data(), (long)dg.size());
    d.diag_row = up.upload_int(dr.get(), ne);
    d.val = up.alloc_float(std::max(1, nnzs[l]));
    d.wdinv = up.alloc_float(std::max(1, nrows[l]));
    float* d_r = up.alloc_float(std::max(1, nrows[l]));
    float* d_t = l == 0 ? nullptr : up.alloc_float(std::max(1, nrows[l]));
    float* d_wr = up.alloc_float(std::max(1, nrows[l]));
    float* d_sr = up.alloc_float(std::max(1, nrows[l]));
    const int* d_ac = up.upload_int(ac.get(), ne);
    const int* d_ag = up.upload_int(ag.data(), (long)ag.size());
    const int* d_pp = pp.empty() ? nullptr : up.upload_int(pp.data(), (long)pp.size());
    const int* d_pr = pr.empty() ? nullptr : up.upload_int(pr.data(), (long)pr.size());
    if (l + 1 < D) {
      d.cptr = up.upload_int(cptr.data(), (long)cptr.size());
      d.csrc = up.upload_int(csrc.get(), (long)ncp[l]);
      d.nnz_next = (int)cptr.size() - 1;
    }
    for (int c = 0; c < nc; c++) {
      if ((int)H(c).lv.size() <= l) continue;
      const AmgHostLevel& L = H(c).lv[l];
      AmgDevLevel& e = v.levels[c][l];
      e.n = L.n;
      e.nnz = L.nnz;
      e.maxagg = 0;
      for (size_t I = 0; I + 1 < L.ptptr.size(); I++) e.maxagg = std::max(e.maxagg, L.ptptr[I + 1] - L.ptptr[I]);
      if (l == 0) {
        e.nnz_off = 0;
        e.rowptr = d_rp;
        e.col = d_cl;
        e.diag = d.diag;
        e.val = d.val;
        e.wdinv = d.wdinv;
        e.agg = d_ag;
        e.r = d_r;
        e.t = nullptr;
        e.wr = d_wr;
        e.sr = d_sr;
        e.aggcol = d_ac;
      } else {
        e.nnz_off = nnz_off[l][c];
        e.rowptr = d_rp + rp_off[l][c];
        e.col = d_cl + nnz_off[l][c];
        e.diag = d.diag + row_off[l][c];
        e.val = d.val + nnz_off[l][c];
        e.wdinv = d.wdinv + row_off[l][c];
        e.agg = d_ag + row_off[l][c];
        e.r = d_r + row_off[l][c];
        e.t = d_t + row_off[l][c];
        e.wr = d_wr + row_off[l][c];
        e.sr = d_sr + row_off[l][c];
        e.aggcol = d_ac + nnz_off[l][c];
      }
      e.ptptr = pt_off[l][c] >= 0 ? d_pp + pt_off[l][c] : nullptr;
      e.ptrow = ptr_off[l][c] >= 0 ? d_pr + ptr_off[l][c] : nullptr;
    }
  }

  // dense inverses, per-case descriptors
  long ninv = 0;
  std::vector<long> inv_off(nc);
  for (int c = 0; c < nc; c++) {
    inv_off[c] = ninv;
    const int m = H(c).lv.back().n;
    ninv += (long)m * m;
  }
  v.coarse_inv = up.alloc_float(std::max(1L, ninv));
  int tail_max = 0;
  for (int c = 0; c < nc; c++) {
    std::vector<int> ln, lz, ls;
    for (const AmgHostLevel& L : H(c).lv) {
      ln.push_back(L.n);
      lz.push_back(L.nnz);
      // the SELL copy only matters for levels small enough to be in the tail
      ls.push_back(L.n < 65536 ? (int)sell_entries(L) : L.nnz);
    }
    AmgCaseDesc& cd = v.cases[c];
    cd.lo = lo[c];
    cd.hi = hi[c];
    cd.nlev = (int)H(c).lv.size();
    cd.coarse_inv = v.coarse_inv + inv_off[c];
    cd.tl = tail_layout(ln, ls);
    for (int l = 0; l < cd.nlev; l++) {
      AmgDevLevel& e = v.levels[c][l];
      e.sell_ptr = nullptr;
      e.sell_col = nullptr;
      e.sell_src = nullptr;
      e.sell_row = nullptr;
      e.sell_len = 0;
      if (l < cd.tl.tail || l + 1 >= cd.nlev) continue;
      const Sell S = sell32(H(c).lv[l]);
      e.sell_ptr = up.upload_int(S.ptr.data(), (long)S.ptr.size());
      e.sell_col = (const unsigned short*)up.upload_bytes(S.col.data(), 2L * (long)S.col.size());
      e.sell_src = up.upload_int(S.src.data(), (long)S.src.size());
      e.sell_row = (const unsigned short*)up.upload_bytes(S.row.data(), 2L * (long)S.row.size());
      e.sell_len = (int)S.col.size();
    }
    cd.levels = (const AmgDevLevel*)up.upload_bytes(v.levels[c].data(), sizeof(AmgDevLevel) * cd.nlev);
    cd.gamma = v.gamma > 0 ? v.gamma : (hi[c] - lo[c] >= kAmgWRows ? 2 : 1);
    tail_max = std::max(tail_max, cd.tl.bytes);
    if (c == 0) {
      v.rows0 = ln;
      v.nnz0 = lz;
    }
  }
  v.d_cases = (AmgCaseDesc*)up.upload_bytes(v.cases.data(), sizeof(AmgCaseDesc) * nc);
  v.smem_bytes = tail_max + kAmgDownBuf * (int)sizeof(float);
}

}  // namespace cycas
