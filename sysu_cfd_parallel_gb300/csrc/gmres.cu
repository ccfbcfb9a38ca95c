// GMRES(m) for one or several systems that share a matrix and preconditioner, as one
// persistent cooperative kernel.
//
// Algorithm per system: PETSc's KSPGMRES as the reference uses it (MPIStructure.cpp:234-531):
// restart m, classical Gram-Schmidt without refinement, left preconditioning, Givens least
// squares, convergence when the preconditioned residual norm drops below
// max(rtol * rnorm0, abstol) with rnorm0 = ||B b|| (nonzero initial guess) or the first
// preconditioned residual (zero guess); DIVERGED_DTOL at dtol * rnorm0, NaN/Inf, breakdown,
// and DIVERGED_ITS when the total iteration count reaches maxit.
//
// The momentum equations solve three right-hand sides with one operator
// (solveVelocity_GMRES, MPIStructure.cpp:268-345); they run here in lockstep: every grid
// phase and barrier is shared, one sweep over a CSR row gathers the operand of every active
// system, and each system keeps its own Krylov basis, Hessenberg matrix and control state,
// so its arithmetic is the same as a solve on its own.
//
// Mixed precision (T = float): the Krylov basis, the Arnoldi SpMV (FP32 matrix copy), the
// Jacobi scaling, the Gram-Schmidt products and the basis updates are FP32, while the
// Hessenberg matrix, the Givens least squares, the cross-CTA sums, x, and every restart's true
// residual z = D^-1 (b - A x) are FP64.  A cycle ends when its residual estimate has dropped
// by inner_rtol (or at the restart length); the restart that follows is the refinement step,
// and the outer convergence test is made on its FP64 residual only.  GB300 runs FP64 at 1/64
// of the FP32 rate, so this moves the arithmetic-bound part of every Arnoldi step to FP32.
//
// Each step is two grid barriers.  Per system the step is one of
//   START / RESTART: (x update of the finished cycle) | residual z = D^-1 (b - A x) | beta, tests
//   ARNOLDI:         w = D^-1 A v_j, partial <w, v_i> | h, w -= sum h_i v_i, ||w|| | Givens, tests
//   FINAL:           x update of the last cycle, then idle
// All CTAs reduce partial sums in the same fixed order, so every CTA takes the same decisions.
#include <cuda_runtime.h>

#include "cycas_device.h"
#include "krylov_common.cuh"

namespace cycas {

namespace {

using namespace kry;

// M_RES2: with the polynomial preconditioner, the (re)start residual's Neumann stages
enum Mode { M_START = 0, M_ARNOLDI = 1, M_RESTART = 2, M_FINAL = 3, M_DONE = 4, M_RES2 = 5 };

template <int NS, class T>
struct GmMsArgs {
  int n, m, maxit, nb;
  const int* __restrict__ rowptr;
  const int* __restrict__ col;
  const double* __restrict__ val;
  const double* __restrict__ dinv;
  const T* __restrict__ valT;   // matrix and Jacobi inverse in the Arnoldi precision
  const T* __restrict__ dinvT;
  double inner_rtol;            // > 0: cycles end at this relative drop (refinement)
  const double* b[NS];
  double* x[NS];
  int guess_zero;
  T* V;   // system s, vector q at (s*(m+1)+q)*ldv
  long ldv;
  double* part;  // [nb][NS][kPartStride]
  unsigned* bar;
  int* err;
  KspOut* out[NS];
  double rtol, abstol, dtol, haptol;
  // batched solves: teams of CTAs, each solving its cases' row ranges in turn (null: one team
  // of the whole grid solving rows [0, n))
  const BatchSchedule* sched;
  // polynomial preconditioner (degree 1 to 5; 0: the Jacobi scaling alone): scratch vectors per
  // system at (s * ldv): Zs and S1, and S2 from degree 3 on
  int poly;
  T* Zs;
  T* S1;
  T* S2;  // second stage scratch (degree 3)
};

// the CTAs that solve one row range together
struct Team {
  int rank, size;  // this CTA's index in the team, CTAs in the team
  unsigned* bar;   // the team's barrier words
  double* part;    // the team's partial sums [size][NS][kPartStride]
};

// sum over CSR row r of val[k] * vec_s[col[k]] for every system s in mask, column order; W
// entries per batch (a tetrahedral row, 5 entries, is one batch for a single system)
template <int NS, class T>
__device__ __forceinline__ void row_gather_ms(const int* __restrict__ rowptr, const int* __restrict__ col,
                                              const T* __restrict__ val, int r, const T* const* vec,
                                              unsigned mask, T* out) {
  constexpr int W = NS == 1 ? 5 : 3;
  const int k0 = __ldg(rowptr + r), k1 = __ldg(rowptr + r + 1);
#pragma unroll
  for (int s = 0; s < NS; s++) out[s] = T(0);
  for (int b = k0; b < k1; b += W) {
    int c[W];
    T v[W], xv[NS][W];
#pragma unroll
    for (int q = 0; q < W; q++) {
      const bool ok = b + q < k1;
      c[q] = ok ? __ldg(col + b + q) : 0;
      v[q] = ok ? __ldg(val + b + q) : T(0);
    }
#pragma unroll
    for (int s = 0; s < NS; s++)
#pragma unroll
      for (int q = 0; q < W; q++) xv[s][q] = ((mask >> s) & 1u) && b + q < k1 ? __ldcg(vec[s] + c[q]) : T(0);
#pragma unroll
    for (int s = 0; s < NS; s++)
#pragma unroll
      for (int q = 0; q < W; q++)
        if (b + q < k1) out[s] += v[q] * xv[s][q];
  }
}

// w + sum_{q < cnt} coef[q] * V[q*ldv + r] in the basis precision, ascending q.  The
// coefficients are already in the basis precision: converting FP64 to FP32 per element would
// run on the FP64 pipe.
template <class T>
__device__ __forceinline__ T basis_axpy(T w, const T* V, long ldv, int r, const T* coef, int cnt) {
  for (int q0 = 0; q0 < cnt; q0 += 8) {
    T v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = (q0 + k < cnt) ? __ldcg(V + (long)(q0 + k) * ldv + r) : T(0);
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (q0 + k < cnt) w = fma(coef[q0 + k], v[k], w);
  }
  return w;
}

// sum of load(blk) over blk = lane, lane + 32, lane + 64, ... < nb, added in that order (the
// order every CTA uses); the loads of up to eight terms are in flight together
template <class F>
__device__ __forceinline__ double lane_sum(int lane, int nb, F load) {
  double sum = 0.0;
  for (int b0 = lane; b0 < nb; b0 += 32 * 8) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = b0 + 32 * k < nb ? load(b0 + 32 * k) : 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (b0 + 32 * k < nb) sum += v[k];
  }
  return sum;
}

template <int NS, class Tv>
__device__ __forceinline__ void gmres_team(const GmMsArgs<NS, Tv>& a, const Team& T, int lo, int hi, KspOut* const* out) {
  constexpr int M = kMaxRestart;
  constexpr int MAXP = NS * (M + 1);
  __shared__ double s_hh[NS][(M + 1) * M];
  __shared__ double s_cc[NS][M], s_ss[NS][M], s_grs[NS][M + 1], s_nrs[NS][M];
  __shared__ double s_scale[NS][M + 1], s_h[NS][M + 1], s_coef[NS][M + 1];
  __shared__ Tv s_coefT[NS][M + 1];  // s_coef in the basis precision
  __shared__ double s_pair[MAXP > 32 ? MAXP : 32];
  __shared__ double s_red[kDotGroup], s_warp[kGmWarps * kDotGroup];
  __shared__ double s_rnorm0[NS], s_ttol[NS], s_rnorm[NS], s_cyc[NS];
  __shared__ int s_mode[NS], s_it[NS], s_its[NS], s_reason[NS], s_first[NS], s_nupd[NS];
  __shared__ unsigned char s_ps[MAXP], s_pq[MAXP];
  __shared__ int s_npairs;

  const int m = a.m, nb = T.size, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int chunk = (hi - lo + nb - 1) / nb;
  const int r0 = min(hi, lo + T.rank * chunk);
  const int r1 = min(hi, r0 + chunk);
  const int kNorm = M + 1, kInit = M + 2;
  auto part_of = [&](int blk, int s) { return T.part + ((long)blk * NS + s) * kPartStride; };
  auto Vv = [&](int s, int q) { return a.V + ((long)s * (m + 1) + q) * a.ldv; };
  const bool mixed = a.inner_rtol > 0.0;
  const int poly = a.poly;
  auto Zv = [&](int s) { return a.Zs + (long)s * a.ldv; };
  auto S1v = [&](int s) { return a.S1 + (long)s * a.ldv; };
  auto S2v = [&](int s) { return a.S2 + (long)s * a.ldv; };

  // w_s = D^-1 A v_{s,it[s]} / |v_{s,it[s]}| into v_{s,it[s]+1} (with the polynomial
  // preconditioner: into z_s, the input of its Neumann stages) for the systems in mask, over this
  // CTA's rows taken by threads t0, t0 + stride, ...; a row's arithmetic does not depend on the
  // thread that computes it
  auto arnoldi_spmv = [&](unsigned mask, const int* it, int t0, int stride) {
    const Tv* vj[NS];
    Tv sj[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) {
      vj[s] = Vv(s, it[s]);
      sj[s] = (Tv)s_scale[s][it[s]];
    }
    for (int r = r0 + t0; r < r1; r += stride) {
      Tv acc[NS];
      row_gather_ms<NS, Tv>(a.rowptr, a.col, a.valT, r, vj, mask, acc);
      const Tv d = a.dinvT ? a.dinvT[r] : Tv(1);
#pragma unroll
      for (int s = 0; s < NS; s++)
        if ((mask >> s) & 1u) (poly ? Zv(s) : Vv(s, it[s] + 1))[r] = (acc[s] * sj[s]) * d;
    }
  };
  // Neumann preconditioner M^-1 = sum_{i<=poly} (I - D^-1 A)^i D^-1, applied to z_s = D^-1 y_s
  // (already in z_s) for the systems in mask: y_0 = z, y_i = z + y_{i-1} - D^-1 A y_{i-1}, the
  // last stage into dst[s].  Each stage follows a barrier (its input must be complete over the
  // team's rows); false after a barrier gave up.
  auto poly_apply = [&](unsigned mask, Tv* const* dst) -> bool {
    for (int st = 1; st <= poly; st++) {
      if (!grid_barrier(T.bar, nb, a.err)) return false;
      const Tv* src[NS];
      Tv* outp[NS];
#pragma unroll
      for (int s = 0; s < NS; s++) {
        // stages alternate between the two scratch vectors, the last one writes dst
        src[s] = st == 1 ? Zv(s) : (st % 2 == 0 ? S1v(s) : S2v(s));
        outp[s] = st == poly ? dst[s] : (st % 2 == 1 ? S1v(s) : S2v(s));
      }
      for (int r = r0 + tid; r < r1; r += kGmThreads) {
        Tv acc[NS];
        row_gather_ms<NS, Tv>(a.rowptr, a.col, a.valT, r, src, mask, acc);
        const Tv d = a.dinvT[r];
#pragma unroll
        for (int s = 0; s < NS; s++)
          if ((mask >> s) & 1u) outp[s][r] = (__ldcg(Zv(s) + r) + __ldcg(src[s] + r)) - d * acc[s];
      }
    }
    __syncthreads();
    return true;
  };
  unsigned spec_prev = 0;  // systems whose next Arnoldi product was computed during the last control phase

  if (tid < NS) {
    s_mode[tid] = M_START;
    s_it[tid] = 0;
    s_its[tid] = 0;
    s_reason[tid] = 0;
    s_first[tid] = 1;
    s_nupd[tid] = 0;
    s_rnorm[tid] = 0.0;
  }
  __syncthreads();
  if (poly && !a.guess_zero) {  // |M^-1 b|, the reference norm of a nonzero initial guess
    for (int r = r0 + tid; r < r1; r += kGmThreads)
#pragma unroll
      for (int s = 0; s < NS; s++) Zv(s)[r] = (Tv)(a.b[s][r] * a.dinv[r]);
    Tv* dst[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) dst[s] = Vv(s, 0);
    if (!poly_apply((1u << NS) - 1u, dst)) return;
    double acc[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) {
      Tv t = Tv(0);
      for (int r = r0 + tid; r < r1; r += kGmThreads) {
        const Tv y = Vv(s, 0)[r];
        t += y * y;
      }
      acc[s] = (double)t;
    }
    block_reduce<NS>(acc, s_warp, s_red);
    if (tid < NS) part_of(T.rank, tid)[kInit + 1] = s_red[tid];
  }

  while (true) {
    int mode[NS], itv[NS];
    bool any = false;
#pragma unroll
    for (int s = 0; s < NS; s++) {
      mode[s] = s_mode[s];
      itv[s] = s_it[s];
      any |= mode[s] != M_DONE;
    }
    if (!any) break;

    // ------------------------------------------------------------ phase X
    unsigned arn = 0, res2 = 0;
#pragma unroll
    for (int s = 0; s < NS; s++) {
      if (mode[s] == M_RES2) res2 |= 1u << s;
      if (mode[s] == M_RESTART || mode[s] == M_FINAL) {
        const int cnt = s_nupd[s];
        for (int r = r0 + tid; r < r1; r += kGmThreads) {
          const Tv t = basis_axpy<Tv>(Tv(0), Vv(s, 0), a.ldv, r, s_coefT[s], cnt);
          a.x[s][r] += (double)t;
        }
      } else if (mode[s] == M_START && a.guess_zero) {
        for (int r = r0 + tid; r < r1; r += kGmThreads) a.x[s][r] = 0.0;
      }
      if (mode[s] == M_ARNOLDI) arn |= 1u << s;
    }
    if (arn) {
      const unsigned todo = arn & ~spec_prev;
      if (todo) arnoldi_spmv(todo, itv, tid, kGmThreads);
    }
    if (poly && (arn | res2)) {
      // Neumann stages: Arnoldi products into v_{it+1}, (re)start residuals into v_0
      Tv* dst[NS];
#pragma unroll
      for (int s = 0; s < NS; s++) dst[s] = ((arn >> s) & 1u) ? Vv(s, itv[s] + 1) : Vv(s, 0);
      if (!poly_apply(arn | res2, dst)) return;
      if (res2) {
        double acc[NS];
#pragma unroll
        for (int s = 0; s < NS; s++) {
          double t = 0.0;
          if ((res2 >> s) & 1u)
            for (int r = r0 + tid; r < r1; r += kGmThreads) {
              const double y = (double)Vv(s, 0)[r];
              t += y * y;
            }
          acc[s] = t;
        }
        block_reduce<NS>(acc, s_warp, s_red);
        if (tid < NS && ((res2 >> tid) & 1u)) part_of(T.rank, tid)[kInit] = s_red[tid];
      }
    }
    if (arn) {
      // pairs (system, basis vector) for the dot products
      if (tid == 0) {
        int p = 0;
        for (int s = 0; s < NS; s++)
          if ((arn >> s) & 1u)
            for (int q = 0; q <= itv[s]; q++) {
              s_ps[p] = (unsigned char)s;
              s_pq[p] = (unsigned char)q;
              p++;
            }
        s_npairs = p;
      }
      __syncthreads();
      // partial dots <w_s, v_{s,q}>, pair-major: one or more warps stream one basis vector
      const int P = s_npairs;
      const int wpp = P >= kGmWarps ? 1 : kGmWarps / P;
      for (int pb = wid / wpp; pb < P; pb += (kGmWarps / wpp)) {
        const int sub = wid % wpp;
        if (wid / wpp >= (kGmWarps / wpp)) break;
        const int s = s_ps[pb], q = s_pq[pb];
        const Tv* vq = Vv(s, q);
        const Tv* w = Vv(s, itv[s] + 1);
        const int step = wpp * 32;
        Tv acct = Tv(0);
        for (int base = r0 + sub * 32 + lane; base < r1; base += 8 * step) {
          Tv wv[8], vv[8];
#pragma unroll
          for (int k = 0; k < 8; k++) {
            const int r = base + k * step;
            wv[k] = r < r1 ? __ldcg(w + r) : Tv(0);
            vv[k] = r < r1 ? __ldcg(vq + r) : Tv(0);
          }
#pragma unroll
          for (int k = 0; k < 8; k++) acct += wv[k] * vv[k];
        }
        double acc = (double)acct;  // lanes, warps and CTAs reduce in FP64
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) s_pair[pb * wpp + sub < (MAXP > 32 ? MAXP : 32) ? pb * wpp + sub : 0] = acc;
      }
      __syncthreads();
      for (int p = tid; p < P; p += kGmThreads) {
        double sum = 0.0;
        for (int k = 0; k < wpp; k++) sum += s_pair[p * wpp + k];
        part_of(T.rank, s_ps[p])[s_pq[p]] = sum;
      }
    }
    if (!grid_barrier(T.bar, nb, a.err)) return;

    // ------------------------------------------------------------ phase Y
    unsigned res_mask = 0;
#pragma unroll
    for (int s = 0; s < NS; s++)
      if (mode[s] == M_START || mode[s] == M_RESTART) res_mask |= 1u << s;
    if (arn) {
      const int P = s_npairs;
      for (int p = wid; p < P; p += kGmWarps) {
        const int s = s_ps[p], q = s_pq[p];
        const double* base = T.part + (long)s * kPartStride + q;
        double sum = lane_sum(lane, nb, [&](int blk) { return ldcg(base + (long)blk * NS * kPartStride); });
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
        if (lane == 0) {
          const double h = sum * s_scale[s][q];
          s_h[s][q] = h;
          s_coef[s][q] = -(h * s_scale[s][q]);  // w -= h v_q / |v_q|
          s_coefT[s][q] = (Tv)s_coef[s][q];
        }
      }
      __syncthreads();
      double nrm[NS];
#pragma unroll
      for (int s = 0; s < NS; s++) {
        nrm[s] = 0.0;
        if (!((arn >> s) & 1u)) continue;
        Tv* w = Vv(s, itv[s] + 1);
        Tv nt = Tv(0);
        for (int r = r0 + tid; r < r1; r += kGmThreads) {
          const Tv wr = basis_axpy<Tv>(__ldcg(w + r), Vv(s, 0), a.ldv, r, s_coefT[s], itv[s] + 1);
          w[r] = wr;
          nt += wr * wr;
        }
        nrm[s] = (double)nt;
      }
      block_reduce<NS>(nrm, s_warp, s_red);
      if (tid < NS && ((arn >> tid) & 1u)) part_of(T.rank, tid)[kNorm] = s_red[tid];
    }
    if (res_mask) {
      const double* xs[NS];
#pragma unroll
      for (int s = 0; s < NS; s++) xs[s] = a.x[s];
      double acc[2 * NS];
#pragma unroll
      for (int k = 0; k < 2 * NS; k++) acc[k] = 0.0;
      for (int r = r0 + tid; r < r1; r += kGmThreads) {
        unsigned gmask = res_mask;
        if (a.guess_zero) {
#pragma unroll
          for (int s = 0; s < NS; s++)
            if (mode[s] == M_START) gmask &= ~(1u << s);  // x = 0: residual is b
        }
        double ax[NS];
        if (gmask) row_gather_ms<NS, double>(a.rowptr, a.col, a.val, r, xs, gmask, ax);
        const double d = a.dinv ? a.dinv[r] : 1.0;
#pragma unroll
        for (int s = 0; s < NS; s++) {
          if (!((res_mask >> s) & 1u)) continue;
          const double br = a.b[s][r];
          const double t = ((gmask >> s) & 1u) ? br - ax[s] : br;
          const double z = t * d;
          (poly ? Zv(s) : Vv(s, 0))[r] = (Tv)z;  // with the polynomial: its stages come next
          acc[2 * s] += z * z;
          if (mode[s] == M_START && !a.guess_zero) {
            const double zb = br * d;
            acc[2 * s + 1] += zb * zb;
          }
        }
      }
      block_reduce<2 * NS>(acc, s_warp, s_red);
      if (!poly && tid < 2 * NS && ((res_mask >> (tid >> 1)) & 1u))
        part_of(T.rank, tid >> 1)[kInit + (tid & 1)] = s_red[tid];
    }
    if (!grid_barrier(T.bar, nb, a.err)) return;

    // ------------------------------------------------------------ phase Z (warp s controls system s)
    // Systems whose cycle goes on unless this step meets the tolerance get their next Arnoldi
    // product now, from the warps that do not control a system, while the control warps apply
    // the Givens rotations (serial FP64 work); a cycle that ends discards that product.
    unsigned spec = 0;
#pragma unroll
    for (int s = 0; s < NS; s++)
      if (mode[s] == M_ARNOLDI && itv[s] + 1 < m && s_its[s] + 1 < a.maxit) spec |= 1u << s;
    double tt = 0.0;  // the new subdiagonal entry, on lane 0 of the control warp
    if (wid < NS && mode[wid] == M_ARNOLDI) {
      const int s = wid;
      double sum = lane_sum(lane, nb, [&](int blk) { return ldcg(part_of(blk, s) + kNorm); });
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
      double* hh = s_hh[s] + itv[s] * (m + 1);  // the new Hessenberg column, copied by the warp
      for (int q = lane; q <= itv[s]; q += 32) hh[q] = s_h[s][q];
      if (lane == 0) {
        tt = sqrt(sum);
        s_scale[s][itv[s] + 1] = __drcp_rn(tt);  // 1 / tt, correctly rounded
      }
    }
    __syncthreads();
    if (wid >= NS && spec) {
      int itn[NS];
#pragma unroll
      for (int s = 0; s < NS; s++) itn[s] = itv[s] + 1;
      arnoldi_spmv(spec, itn, tid - NS * 32, kGmThreads - NS * 32);
    }
    if (wid < NS) {
      const int s = wid;
      const int md = mode[s];
      if (md == M_ARNOLDI) {
        if (lane == 0) {
          const int it = itv[s];
          double* hh = s_hh[s] + it * (m + 1);
          hh[it + 1] = tt;
          // happy breakdown: tt < min(|tt / g_it|, haptol); the division only when tt < haptol
          const bool hapend = tt < a.haptol && tt < fabs(tt / s_grs[s][it]);
          // the previous rotations applied to the new column; the entry carried from one
          // rotation to the next stays in a register
          double carry = hh[0];
          for (int j = 1; j <= it; j++) {
            const double hj = hh[j], c = s_cc[s][j - 1], sn = s_ss[s][j - 1];
            hh[j - 1] = c * carry + sn * hj;
            carry = c * hj - sn * carry;
          }
          hh[it] = carry;
          int rs = 0, used = it;
          bool brk = false;
          double res = s_rnorm[s];
          if (!hapend) {
            const double d = sqrt(hh[it] * hh[it] + hh[it + 1] * hh[it + 1]);
            if (d == 0.0) {
              rs = -5;
              brk = true;
            } else {
              const double rd = __drcp_rn(d);
              s_cc[s][it] = hh[it] * rd;
              s_ss[s][it] = hh[it + 1] * rd;
              s_grs[s][it + 1] = -(s_ss[s][it] * s_grs[s][it]);
              s_grs[s][it] = s_cc[s][it] * s_grs[s][it];
              hh[it] = s_cc[s][it] * hh[it] + s_ss[s][it] * hh[it + 1];
              res = fabs(s_grs[s][it + 1]);
            }
          } else {
            res = 0.0;
          }
          bool inner_done = false;
          if (!brk) {
            used = it + 1;
            s_its[s]++;
            s_rnorm[s] = res;
            if (isnan(res) || isinf(res)) rs = -9;
            else if (mixed) {
              // refinement: the cycle ends at its own relative drop; convergence is decided on
              // the FP64 residual of the restart that follows
              inner_done = res <= fmax(s_ttol[s], a.inner_rtol * s_cyc[s]) || hapend;
            } else if (res <= s_ttol[s]) rs = res < a.abstol ? 3 : 2;
            else if (res >= a.dtol * s_rnorm0[s]) rs = -4;
            if (hapend && !rs && !mixed) rs = -5;
          }
          s_reason[s] = rs;
          const bool end_cycle = brk || rs != 0 || inner_done || used == m || s_its[s] >= a.maxit;
          if (!end_cycle) {
            s_it[s] = used;
          } else {
            // least-squares solution of the cycle (back substitution on the rotated Hessenberg)
            int nup = 0;
            if (used > 0) {
              const int k = used - 1;
              const double* H = s_hh[s];
              auto HH = [&](int row, int c) { return H[c * (m + 1) + row]; };
              if (HH(k, k) == 0.0) {
                s_reason[s] = -5;
              } else {
                s_nrs[s][k] = s_grs[s][k] / HH(k, k);
                for (int ii = 1; ii <= k; ii++) {
                  const int q = k - ii;
                  double t = s_grs[s][q];
                  for (int j = q + 1; j <= k; j++) t = t - HH(q, j) * s_nrs[s][j];
                  s_nrs[s][q] = t / HH(q, q);
                }
                for (int j = 0; j <= k; j++) {
                  s_coef[s][j] = s_nrs[s][j] * s_scale[s][j];
                  s_coefT[s][j] = (Tv)s_coef[s][j];
                }
                nup = used;
              }
            }
            s_nupd[s] = nup;
            if (mixed && s_reason[s] == 0 && nup > 0) {
              s_mode[s] = M_RESTART;  // x update and the FP64 residual decide
            } else {
              if (s_reason[s] == 0 && s_its[s] >= a.maxit) s_reason[s] = -3;
              const bool finished = s_reason[s] != 0;
              s_mode[s] = finished ? (nup > 0 ? M_FINAL : M_DONE) : (nup > 0 ? M_RESTART : M_START);
            }
            s_it[s] = 0;
          }
        }
      } else if (poly && (md == M_START || md == M_RESTART)) {
        if (lane == 0) s_mode[s] = M_RES2;  // the residual's Neumann stages run next
      } else if (md == M_START || md == M_RESTART || md == M_RES2) {
        double s0 = lane_sum(lane, nb, [&](int blk) { return ldcg(part_of(blk, s) + kInit); });
        double s1 = lane_sum(lane, nb, [&](int blk) { return ldcg(part_of(blk, s) + kInit + 1); });
        for (int o = 16; o > 0; o >>= 1) {
          s0 += __shfl_down_sync(0xffffffffu, s0, o);
          s1 += __shfl_down_sync(0xffffffffu, s1, o);
        }
        if (lane == 0) {
          const double beta = sqrt(s0);
          if (s_first[s]) {
            if (a.guess_zero) s_rnorm0[s] = beta;
            else {
              const double snorm = sqrt(s1);
              s_rnorm0[s] = snorm != 0.0 ? snorm : beta;
            }
          }
          s_grs[s][0] = beta;
          s_scale[s][0] = 1.0 / beta;
          s_rnorm[s] = beta;
          s_cyc[s] = beta;
          int rs = 0;
          if (beta == 0.0) {
            rs = 3;
          } else {
            if (s_its[s] == 0) s_ttol[s] = fmax(a.rtol * s_rnorm0[s], a.abstol);
            if (isnan(beta) || isinf(beta)) rs = -9;
            else if (beta <= s_ttol[s]) rs = beta < a.abstol ? 3 : 2;
            else if (beta >= a.dtol * s_rnorm0[s]) rs = -4;
            else if (mixed && s_its[s] >= a.maxit) rs = -3;
          }
          s_reason[s] = rs;
          s_first[s] = 0;
          s_it[s] = 0;
          s_mode[s] = rs ? M_DONE : M_ARNOLDI;
        }
      } else if (md == M_FINAL) {
        if (lane == 0) s_mode[s] = M_DONE;
      }
    }
    __syncthreads();
    spec_prev = spec;
  }
  if (T.rank == 0 && tid < NS) {
    out[tid]->its = s_its[tid];
    out[tid]->reason = s_reason[tid];
    out[tid]->rnorm = s_rnorm[tid];
  }
  __syncthreads();
}

template <int NS, class Tv>
__global__ void __launch_bounds__(kGmThreads, 1) k_gmres_ms(GmMsArgs<NS, Tv> a) {
  if (launch_failed(a.err)) return;
  if (!a.sched) {
    const Team T{(int)blockIdx.x, a.nb, a.bar, a.part};
    gmres_team<NS, Tv>(a, T, 0, a.n, a.out);
    return;
  }
  const BatchSchedule& S = *a.sched;
  const int team = S.cta_team[blockIdx.x];
  const Team T{S.cta_rank[blockIdx.x], S.team_size[team], a.bar + 2L * team,
               a.part + (long)S.team_cta0[team] * NS * kPartStride};
  for (int k = S.team_case0[team]; k < S.team_case0[team + 1]; k++) {
    const int c = S.case_list[k];
    KspOut* out[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) out[s] = a.out[s] + c;
    gmres_team<NS, Tv>(a, T, S.case_lo[c], S.case_hi[c], out);
    if (*(volatile int*)a.err) return;
  }
}

template <int NS, class Tv>
cudaError_t launch_ms(const GmresCall* calls, KrylovWork& w, cudaStream_t s, const BatchSchedule* sched = nullptr,
                      int grid = 0, KspOut* const* outs = nullptr) {
  GmMsArgs<NS, Tv> a;
  const GmresCall& c = calls[0];
  // workspace bounds: basis NS*(m+1) vectors, partials nb*NS*stride
  const int nb = sched ? grid : gmres_grid(c.n, w.nblocks);
  const int extra = c.poly ? (c.poly >= 3 ? 3 : 2) * NS : 0;  // Neumann scratch vectors
  if (c.restart < 1 || c.restart > kMaxRestart || ((long)NS * (c.restart + 1) + extra) * w.ldv > w.v_len ||
      (long)nb * NS * kPartStride > w.part_len || w.ldv < c.n || c.poly < 0 || c.poly > 5 ||
      (c.poly && (!c.dinv || (sizeof(Tv) != sizeof(double) && !c.dinv32))))
    return cudaErrorInvalidValue;
  a.n = c.n;
  a.m = c.restart;
  a.maxit = c.maxit;
  a.nb = nb;
  a.sched = sched;
  a.rowptr = c.rowptr;
  a.col = c.col;
  a.val = c.val;
  a.dinv = c.dinv;
  if constexpr (sizeof(Tv) == sizeof(double)) {
    a.valT = c.val;
    a.dinvT = c.dinv;
    a.inner_rtol = 0.0;
  } else {
    if (!c.val32 || (c.dinv && !c.dinv32) || !(c.inner_rtol > 0.0)) return cudaErrorInvalidValue;
    a.valT = c.val32;
    a.dinvT = c.dinv ? c.dinv32 : nullptr;
    a.inner_rtol = c.inner_rtol;
  }
  for (int k = 0; k < NS; k++) {
    a.b[k] = calls[k].b;
    a.x[k] = calls[k].x;
    a.out[k] = outs ? outs[k] : calls[k].out;
  }
  a.guess_zero = c.guess_zero;
  a.V = reinterpret_cast<Tv*>(w.V);
  a.ldv = w.ldv;
  a.poly = c.poly;
  a.Zs = a.V + (long)NS * (c.restart + 1) * w.ldv;
  a.S1 = a.Zs + (long)NS * w.ldv;
  a.S2 = a.S1 + (long)NS * w.ldv;  // used from degree 3 on (inside the capacity checked above)
  a.part = w.part;
  a.bar = w.bar;
  a.err = c.err;
  a.rtol = c.rtol;
  a.abstol = 1e-50;
  a.dtol = 1e4;
  a.haptol = 1e-30;
  void* args[] = {&a};
  return launch_cooperative((const void*)k_gmres_ms<NS, Tv>, nb, kGmThreads, args, 0, s);
}

}  // namespace

cudaError_t launch_gmres_batch(const GmresCall* calls, int nsys, KrylovWork& w, const BatchSchedule* sched, int grid,
                               KspOut* const* outs, cudaStream_t s) {
  if (!sched || grid < 1 || grid > w.nblocks) return cudaErrorInvalidValue;
  const bool mx = calls[0].val32 != nullptr;
  if (nsys == 1) return mx ? launch_ms<1, float>(calls, w, s, sched, grid, outs) : launch_ms<1, double>(calls, w, s, sched, grid, outs);
  if (nsys == 3) return mx ? launch_ms<3, float>(calls, w, s, sched, grid, outs) : launch_ms<3, double>(calls, w, s, sched, grid, outs);
  return cudaErrorInvalidValue;
}

cudaError_t launch_gmres_multi(const GmresCall* calls, int nsys, KrylovWork& w, cudaStream_t s) {
  const bool mx = calls[0].val32 != nullptr;
  if (nsys == 1) return mx ? launch_ms<1, float>(calls, w, s) : launch_ms<1, double>(calls, w, s);
  if (nsys == 3) return mx ? launch_ms<3, float>(calls, w, s) : launch_ms<3, double>(calls, w, s);
  return cudaErrorInvalidValue;
}

}  // namespace cycas
