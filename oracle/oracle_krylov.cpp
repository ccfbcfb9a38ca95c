// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h; parity unpinned at the PETSc boundary).
//
// The reference hands every system to PETSc KSP (MPIStructure.cpp:234-531):
// GMRES, restart 30, classical (unmodified) Gram-Schmidt without refinement,
// left preconditioning, convergence when the preconditioned residual norm
// drops below max(rtol*rnorm0, abstol) where rnorm0 = ||B b|| (nonzero initial
// guess) or the initial preconditioned residual (zero guess), divergence at
// dtol*rnorm0 or on NaN, DIVERGED_ITS at max_it.  Default preconditioner on one
// rank: ILU(0) in the natural ordering.  This file restates that published
// algorithm (Saad, Iterative Methods for Sparse Linear Systems, 2nd ed., Alg.
// 6.9 and 10.4) together with PETSc's documented default settings.
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "oracle.h"

namespace orc {

namespace {

struct Pc {
  int type = PC_NONE;
  int n = 0;
  std::vector<double> dinv;          // Jacobi: 1/a_ii
  // ILU(0) on the matrix pattern, factor values stored in place of A,
  // with the reciprocal of each U pivot kept separately
  const Csr* A = nullptr;
  std::vector<double> lu, udinv;
  std::vector<int> perm, iperm;      // optional symmetric permutation (new -> old, old -> new)
  std::vector<int> prow, pcol;       // permuted pattern
  std::vector<double> pval;
  std::vector<int> pdiag;

  void setup(const Csr& M, const KspSettings& s) {
    type = s.pc;
    n = M.n;
    A = &M;
    if (type == PC_JACOBI || poly_degree(type) > 0) {
      dinv.resize(n);
      for (int i = 0; i < n; i++) dinv[i] = 1.0 / M.val[M.diag[i]];
    } else if (type == PC_ILU0) {
      // build the (optionally permuted) copy
      bool hasPerm = !s.perm.empty();
      perm.assign(n, 0);
      iperm.assign(n, 0);
      for (int i = 0; i < n; i++) perm[i] = hasPerm ? s.perm[i] : i;
      for (int i = 0; i < n; i++) iperm[perm[i]] = i;
      prow.assign(n + 1, 0);
      pcol.clear();
      pval.clear();
      std::vector<std::pair<int, double>> row;
      for (int i = 0; i < n; i++) {
        int o = perm[i];
        row.clear();
        for (int k = M.rowptr[o]; k < M.rowptr[o + 1]; k++) row.push_back({iperm[M.col[k]], M.val[k]});
        std::sort(row.begin(), row.end(), [](const std::pair<int, double>& a, const std::pair<int, double>& b) { return a.first < b.first; });
        for (auto& e : row) {
          pcol.push_back(e.first);
          pval.push_back(e.second);
        }
        prow[i + 1] = (int)pcol.size();
      }
      pdiag.assign(n, -1);
      for (int i = 0; i < n; i++)
        for (int k = prow[i]; k < prow[i + 1]; k++)
          if (pcol[k] == i) pdiag[i] = k;
      lu = pval;
      udinv.assign(n, 0.0);
      // IKJ ILU(0): multipliers use the reciprocal of the pivot
      std::vector<int> where(n, -1);
      for (int i = 0; i < n; i++) {
        for (int k = prow[i]; k < prow[i + 1]; k++) where[pcol[k]] = k;
        for (int k = prow[i]; k < prow[i + 1] && pcol[k] < i; k++) {
          int kr = pcol[k];
          double mult = lu[k] * udinv[kr];
          lu[k] = mult;
          for (int q = pdiag[kr] + 1; q < prow[kr + 1]; q++) {
            int w = where[pcol[q]];
            if (w >= 0) lu[w] -= mult * lu[q];
          }
        }
        double piv = lu[pdiag[i]];
        if (piv == 0.0) throw std::runtime_error("zero pivot in ILU(0)");
        udinv[i] = 1.0 / piv;
        for (int k = prow[i]; k < prow[i + 1]; k++) where[pcol[k]] = -1;
      }
    }
  }

  void apply(const double* r, double* z) const {
    if (type == PC_NONE) {
      std::copy(r, r + n, z);
    } else if (type == PC_JACOBI) {
      for (int i = 0; i < n; i++) z[i] = r[i] * dinv[i];
    } else if (poly_degree(type) > 0) {
      // y_0 = D^-1 r, y_i = y_0 + y_{i-1} - D^-1 A y_{i-1}
      const int deg = poly_degree(type);
      std::vector<double> z0(n), y(n), ay(n);
      for (int i = 0; i < n; i++) z0[i] = r[i] * dinv[i];
      y = z0;
      for (int d = 0; d < deg; d++) {
        for (int i = 0; i < n; i++) {
          double s = 0.0;
          for (int k = A->rowptr[i]; k < A->rowptr[i + 1]; k++) s += A->val[k] * y[A->col[k]];
          ay[i] = s;
        }
        for (int i = 0; i < n; i++) y[i] = (z0[i] + y[i]) - dinv[i] * ay[i];
      }
      std::copy(y.begin(), y.end(), z);
    } else {
      std::vector<double> y(n);
      for (int i = 0; i < n; i++) {
        double s = r[perm[i]];
        for (int k = prow[i]; k < pdiag[i]; k++) s -= lu[k] * y[pcol[k]];
        y[i] = s;
      }
      for (int i = n - 1; i >= 0; i--) {
        double s = y[i];
        for (int k = pdiag[i] + 1; k < prow[i + 1]; k++) s -= lu[k] * y[pcol[k]];
        y[i] = s * udinv[i];
      }
      for (int i = 0; i < n; i++) z[perm[i]] = y[i];
    }
  }
};

void spmv(const Csr& A, const double* x, double* y) {
  for (int i = 0; i < A.n; i++) {
    double s = 0.0;
    for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; k++) s += A.val[k] * x[A.col[k]];
    y[i] = s;
  }
}

double dot(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

}  // namespace

// PETSc KSPCG (Hestenes-Stiefel form, preconditioned-norm convergence test).  It stops
// only when beta or p'Ap changes sign between iterations, so the negative-definite
// pressure-correction system is accepted as it stands.
static KspResult cg_solve(const Csr& A, const Pc& pc, const KspSettings& s, double rtol, int maxit, bool guess_zero,
                          const double* b, double* x) {
  const int n = A.n;
  std::vector<double> r(n), z(n), p(n), w(n);
  KspResult res;
  if (guess_zero) {
    std::fill(x, x + n, 0.0);
    std::copy(b, b + n, r.begin());
  } else {
    spmv(A, x, w.data());
    for (int i = 0; i < n; i++) r[i] = b[i] - w[i];
  }
  pc.apply(r.data(), z.data());
  double dp = std::sqrt(dot(z.data(), z.data(), n));
  double rnorm0, ttol;
  if (!guess_zero) {
    std::vector<double> t(n);
    pc.apply(b, t.data());
    double snorm = std::sqrt(dot(t.data(), t.data(), n));
    rnorm0 = snorm != 0.0 ? snorm : dp;
  } else {
    rnorm0 = dp;
  }
  ttol = std::max(rtol * rnorm0, s.abstol);
  auto test = [&](double rn) -> int {
    if (std::isnan(rn) || std::isinf(rn)) return KSP_DIVERGED_NANORINF;
    if (rn <= ttol) return rn < s.abstol ? KSP_CONVERGED_ATOL : KSP_CONVERGED_RTOL;
    if (rn >= s.dtol * rnorm0) return KSP_DIVERGED_DTOL;
    return 0;
  };
  res.rnorm = dp;
  res.reason = test(dp);
  if (res.reason) return res;
  double beta = dot(z.data(), r.data(), n), betaold = 0.0, dpi = 0.0, dpiold = 0.0;
  int i = 0;
  do {
    res.its = i + 1;
    if (beta == 0.0) {
      res.reason = KSP_CONVERGED_ATOL;
      break;
    }
    if (i > 0 && beta * betaold < 0.0) {
      res.reason = KSP_DIVERGED_INDEFINITE_PC;
      break;
    }
    if (i == 0) {
      std::copy(z.begin(), z.end(), p.begin());
    } else {
      double bb = beta / betaold;
      for (int k = 0; k < n; k++) p[k] = z[k] + bb * p[k];
    }
    dpiold = dpi;
    spmv(A, p.data(), w.data());
    dpi = dot(p.data(), w.data(), n);
    betaold = beta;
    if (dpi == 0.0 || (i > 0 && ((dpi > 0) - (dpi < 0)) * ((dpiold > 0) - (dpiold < 0)) < 0)) {
      res.reason = KSP_DIVERGED_INDEFINITE_MAT;
      break;
    }
    double a = beta / dpi;
    for (int k = 0; k < n; k++) x[k] += a * p[k];
    for (int k = 0; k < n; k++) r[k] += -a * w[k];
    pc.apply(r.data(), z.data());
    dp = std::sqrt(dot(z.data(), z.data(), n));
    res.rnorm = dp;
    res.reason = test(dp);
    if (res.reason) break;
    beta = dot(z.data(), r.data(), n);
    i++;
  } while (i < maxit);
  if (i >= maxit) res.reason = KSP_DIVERGED_ITS;
  return res;
}

KspResult ksp_solve(const Csr& A, const KspSettings& s, double rtol, int maxit, bool guess_zero,
                    const double* b, double* x) {
  const int n = A.n, m = s.restart;
  Pc pc;
  pc.setup(A, s);
  if (s.type == KSP_CG) return cg_solve(A, pc, s, rtol, maxit, guess_zero, b, x);
  KspResult res;
  std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
  std::vector<double> hh((m + 1) * m, 0.0), cc(m, 0.0), ss(m, 0.0), grs(m + 1, 0.0), nrs(m, 0.0), t(n), w(n);
  auto HH = [&](int r, int c) -> double& { return hh[c * (m + 1) + r]; };
  if (guess_zero) std::fill(x, x + n, 0.0);
  int its = 0, reason = 0;
  double rnorm0 = 0.0, ttol = 0.0, rnorm = 0.0;
  bool first = true;
  auto converged = [&](int k, double rn) -> int {
    if (k == 0) {
      if (!guess_zero && first) {
        pc.apply(b, t.data());
        double snorm = std::sqrt(dot(t.data(), t.data(), n));
        rnorm0 = snorm != 0.0 ? snorm : rn;
      } else if (first) {
        rnorm0 = rn;
      }
      ttol = std::max(rtol * rnorm0, s.abstol);
    }
    if (std::isnan(rn) || std::isinf(rn)) return KSP_DIVERGED_NANORINF;
    if (rn <= ttol) return rn < s.abstol ? KSP_CONVERGED_ATOL : KSP_CONVERGED_RTOL;
    if (rn >= s.dtol * rnorm0) return KSP_DIVERGED_DTOL;
    return 0;
  };
  int itcount = 0;
  while (!reason) {
    // initial (preconditioned) residual
    if (first && guess_zero) {
      pc.apply(b, V[0].data());
    } else {
      spmv(A, x, t.data());
      for (int i = 0; i < n; i++) t[i] = b[i] - t[i];
      pc.apply(t.data(), V[0].data());
    }
    double beta = std::sqrt(dot(V[0].data(), V[0].data(), n));
    grs[0] = beta;
    rnorm = beta;
    int it = 0;
    if (beta == 0.0) {
      reason = KSP_CONVERGED_ATOL;
      if (first && !guess_zero) { /* rnorm0 unset: nothing more to do */ }
      break;
    }
    for (int i = 0; i < n; i++) V[0][i] *= 1.0 / beta;
    reason = converged(its, rnorm);
    first = false;
    while (!reason && it < m && its < maxit) {
      spmv(A, V[it].data(), t.data());
      pc.apply(t.data(), w.data());
      // classical Gram-Schmidt
      for (int j = 0; j <= it; j++) HH(j, it) = dot(w.data(), V[j].data(), n);
      for (int j = 0; j <= it; j++) {
        double h = HH(j, it);
        for (int i = 0; i < n; i++) w[i] -= h * V[j][i];
      }
      double tt = std::sqrt(dot(w.data(), w.data(), n));
      double scale = 1.0 / tt;
      for (int i = 0; i < n; i++) V[it + 1][i] = w[i] * scale;
      HH(it + 1, it) = tt;
      double hapbnd = std::fabs(tt / grs[it]);
      if (hapbnd > s.haptol) hapbnd = s.haptol;
      bool hapend = tt < hapbnd;
      // apply previous rotations, then the new one
      for (int j = 1; j <= it; j++) {
        double tmp = HH(j - 1, it);
        HH(j - 1, it) = cc[j - 1] * tmp + ss[j - 1] * HH(j, it);
        HH(j, it) = cc[j - 1] * HH(j, it) - ss[j - 1] * tmp;
      }
      double r;
      if (!hapend) {
        double d = std::sqrt(HH(it, it) * HH(it, it) + HH(it + 1, it) * HH(it + 1, it));
        if (d == 0.0) {
          reason = KSP_DIVERGED_BREAKDOWN;
          break;
        }
        cc[it] = HH(it, it) / d;
        ss[it] = HH(it + 1, it) / d;
        grs[it + 1] = -(ss[it] * grs[it]);
        grs[it] = cc[it] * grs[it];
        HH(it, it) = cc[it] * HH(it, it) + ss[it] * HH(it + 1, it);
        r = std::fabs(grs[it + 1]);
      } else {
        r = 0.0;
      }
      it++;
      its++;
      rnorm = r;
      reason = converged(its, rnorm);
      if (hapend && !reason) {
        reason = KSP_DIVERGED_BREAKDOWN;
        break;
      }
    }
    // form the solution update from the first `it` Krylov vectors
    if (it > 0) {
      int k = it - 1;
      if (HH(k, k) == 0.0) {
        reason = KSP_DIVERGED_BREAKDOWN;
      } else {
        nrs[k] = grs[k] / HH(k, k);
        for (int ii = 1; ii <= k; ii++) {
          int q = k - ii;
          double tt = grs[q];
          for (int j = q + 1; j <= k; j++) tt = tt - HH(q, j) * nrs[j];
          nrs[q] = tt / HH(q, q);
        }
        std::fill(t.begin(), t.end(), 0.0);
        for (int j = 0; j <= k; j++)
          for (int i = 0; i < n; i++) t[i] += nrs[j] * V[j][i];
        for (int i = 0; i < n; i++) x[i] += t[i];
      }
    }
    itcount += it;
    if (itcount >= maxit) {
      if (!reason) reason = KSP_DIVERGED_ITS;
      break;
    }
  }
  res.its = its;
  res.reason = reason;
  res.rnorm = rnorm;
  return res;
}

}  // namespace orc
