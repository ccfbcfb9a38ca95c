// Aggregation-AMG preconditioned CG for the pressure-correction system.
//
// The reference solves the pressure correction with PETSc CG + ILU(0) at rtol 1e-6 and a
// 1000-iteration cap (navier_pressure.cpp:28, MPIStructure.cpp:449-531).  On the 480k-cell
// channel that takes ~390 ILU-CG iterations and Jacobi-CG does not converge within the
// cap; a level-scheduled ILU apply would cost ~70 grid barriers.  Here an FP64 conjugate
// gradient with PETSc's preconditioned-norm test runs with one V-cycle of plain aggregation
// multigrid as the preconditioner:
//   down:   x_l = w D_l^-1 r_l;  r_{l+1} = P^T (r_l - A_l x_l)
//   bottom: x_L = (A_L - s 11^T)^-1 r_L, dense                       (the system is singular:
//           the rank-one shift removes the constant null space without moving the range)
//   up:     t_l = y + w D_l^-1 (r_l - A_l y),  y = x_l + a P t_{l+1}
// Pre- and post-smoothing are transposes of each other and P = R^T, so the cycle is a fixed
// symmetric operator.  All sums are in fixed order (deterministic).
//
// GB300 executes FP64 arithmetic at 1/64 of the FP32 rate (about two FP64 FMAs per clock per
// SM), which makes an FP64 V-cycle arithmetic-bound; the cycle therefore runs in FP32 (values,
// Jacobi weights, residuals and corrections), and only the CG -- SpMV, inner products, vector
// updates -- is FP64.  An FP32 cycle is symmetric only up to rounding, so the CG is the
// flexible variant FCG(1): each direction is A-orthogonalised against the previous one
// (beta = -(u, A p_old) / (p_old, A p_old)), which equals the Hestenes-Stiefel beta when the
// preconditioner is exactly symmetric and stays robust when it is not.
//
// Synchronisation is the cost on a 152-SM grid, so each level above the tail takes one grid
// barrier down (smoothing and restriction fused per coarse row block: x_l is recomputed from
// r_l where it is needed instead of stored) and one up; the coarsest levels (the "tail",
// chosen so that their matrices, with 16-bit columns, fit in shared memory) are loaded into
// every CTA's shared memory once per solve and cycled there by every CTA at once, with block
// barriers only: each CTA then holds the whole coarse correction, so the first prolongation
// follows the tail without a grid barrier and no CTA waits while another works alone.  CG itself is the
// Chronopoulos-Gear form: w = A u and the inner products (r,u), (w,u), (u,u), (u,s) come out
// of one pass and one grid reduction, and p, s = A p, x, r are updated locally, so an
// iteration costs two grid barriers plus the V-cycle's.
#include <cuda_runtime.h>

#include "cycas_amg.h"
#include "cycas_device.h"
#include "krylov_common.cuh"

namespace cycas {

namespace {

using namespace kry;

constexpr int kThreads = 256;

// ---------------------------------------------------------------- per-solve setup
// FP32 copy of the pressure matrix; a diagonal entry also gives its row's smoother weight w / a_ii
__global__ void k_amg_level0(int nnz, const double* __restrict__ val64, float* __restrict__ val,
                             const int* __restrict__ diag_row, float omega, float* __restrict__ wdinv) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const float v = (float)val64[k];
  val[k] = v;
  const int i = diag_row[k];
  if (i >= 0) wdinv[i] = omega / v;
}

// Galerkin sum of one coarse entry (fine entries in ascending order); a diagonal entry also
// gives its row's smoother weight
__global__ void k_amg_galerkin(int nnz_c, const int* __restrict__ cptr, const int* __restrict__ csrc,
                               const float* __restrict__ valf, float* __restrict__ valc,
                               const int* __restrict__ diag_row_c, float omega, float* __restrict__ wdinv_c) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nnz_c) return;
  float s = 0.0f;
  for (int q = cptr[c]; q < cptr[c + 1]; q++) s += valf[csrc[q]];
  valc[c] = s;
  const int i = diag_row_c[c];
  if (i >= 0) wdinv_c[i] = omega / s;
}

// dense inverse of A_L + s 11^T, s = mean(diag)/n, for the coarsest level of case blockIdx.x,
// by in-place Gauss-Jordan in shared memory.  A_L is singular with the constant null vector
// (row sums vanish); the shift has the sign of the diagonal, so the shifted matrix is
// definite and needs no pivoting.  A case with a single level is inverted on its own rows of
// the system (global numbering).
__global__ void k_amg_coarse_inverse(const AmgCaseDesc* __restrict__ cases) {
  __shared__ float M[kAmgCoarseMax * kAmgCoarseMax];
  __shared__ float colk[kAmgCoarseMax];
  __shared__ float s_shift;
  const AmgCaseDesc& cd = cases[blockIdx.x];
  const AmgDevLevel K = cd.levels[cd.nlev - 1];
  const int n = K.n;
  const int row0 = cd.nlev == 1 ? cd.lo : 0;
  float* inv = const_cast<float*>(cd.coarse_inv);
  const int tid = threadIdx.x;
  for (int e = tid; e < n * n; e += blockDim.x) M[e] = 0.0f;
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x)
    for (int k = K.rowptr[row0 + i]; k < K.rowptr[row0 + i + 1]; k++) M[i * n + K.col[k] - row0] = K.val[k];
  if (tid == 0) {
    float d = 0.0f;
    for (int i = 0; i < n; i++) d += K.val[K.diag[row0 + i] - K.nnz_off];
    s_shift = d / ((float)n * (float)n);
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) M[e] += s_shift;
  __syncthreads();
  for (int k = 0; k < n; k++) {
    float piv = M[k * n + k];
    for (int i = tid; i < n; i += blockDim.x) colk[i] = M[i * n + k];
    __syncthreads();
    for (int j = tid; j < n; j += blockDim.x) M[k * n + j] = (j == k ? 1.0f : M[k * n + j]) / piv;
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) {
      int i = e / n, j = e % n;
      if (i == k) continue;
      M[e] = (j == k ? 0.0f : M[e]) - colk[i] * M[k * n + j];
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += blockDim.x) inv[e] = M[e];
}

// ---------------------------------------------------------------- V-cycle
struct CgAmgArgs {
  int n, maxit, guess_zero, nb;
  const int* __restrict__ rowptr;
  const int* __restrict__ col;
  const double* __restrict__ val;
  const double* __restrict__ b;
  double* x;
  double *r, *u, *p, *w, *s;
  double* part;
  unsigned* bar;
  int* err;
  KspOut* out;  // [ncases]
  double rtol, abstol, dtol;
  float alpha;
  const AmgCaseDesc* cases;
  const BatchSchedule* sched;
};

// the CTAs that solve one case together
struct Team {
  int rank, size;
  unsigned* bar;
  double* part;  // [size][kPartStride]
};

struct Rows {
  int r0, r1;
};
// the team member's share of rows [lo, hi)
__device__ __forceinline__ Rows share(int lo, int hi, const Team& T) {
  const int ch = (hi - lo + T.size - 1) / T.size;
  const int r0 = min(hi, lo + T.rank * ch);
  return {r0, min(hi, r0 + ch)};
}

__device__ __forceinline__ float ldcgf(const float* p) { return __ldcg(p); }

// FP32 row sum of val[k] * f(col[k]) in column order, loads issued W entries at a time
template <int W, class F>
__device__ __forceinline__ float row_gather_f(const int* __restrict__ rowptr, const int* __restrict__ col,
                                              const float* __restrict__ val, int r, F f) {
  const int k0 = __ldg(rowptr + r), k1 = __ldg(rowptr + r + 1);
  float s = 0.0f;
  for (int b = k0; b < k1; b += W) {
    int c[W];
    float v[W], xv[W];
#pragma unroll
    for (int q = 0; q < W; q++) {
      const bool ok = b + q < k1;
      c[q] = ok ? __ldg(col + b + q) : 0;
      v[q] = ok ? __ldg(val + b + q) : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < W; q++) xv[q] = (b + q < k1) ? f(c[q]) : 0.0f;
#pragma unroll
    for (int q = 0; q < W; q++)
      if (b + q < k1) s += v[q] * xv[q];
  }
  return s;
}

template <class T>
__device__ __forceinline__ T* at(unsigned char* sb, int off) {
  return reinterpret_cast<T*>(sb + off);
}

// the kernel's dynamic shared memory, named at file scope so that the tail functions address it
// as shared memory rather than through generic pointers
extern __shared__ __align__(16) unsigned char amg_smem[];
template <class T>
__device__ __forceinline__ T* sat(int off) {
  return reinterpret_cast<T*>(amg_smem + off);
}

// every member of a team: the tail levels of its case (matrices with 16-bit columns, transfer
// lists, the coarsest inverse) into its own shared memory; level 0 is renumbered from the
// system's rows to the case's
template <class T>
__device__ __forceinline__ void copy_in(T* dst, const T* src, int cnt, T shift = T(0)) {
  for (int i = threadIdx.x; i < cnt; i += kGmThreads) dst[i] = src[i] - shift;
}

__device__ void tail_load(const AmgDevLevel* L, int nlev, const TailLayout& T, const float* coarse_inv, int lo,
                          unsigned char* sb) {
  for (int l = T.tail; l < nlev; l++) {
    const AmgDevLevel& F = L[l];
    const TailLevelOff& o = T.lv[l];
    const int row0 = l == 0 ? lo : 0;
    if (l + 1 < nlev) {
      // the matrix in SELL-32 layout; values gathered from the level's CSR values (level 0:
      // the case's entries start at the system's row pointer of its first row)
      const int k0 = l == 0 ? __ldg(F.rowptr + lo) : 0;
      const int ns = (F.n + 31) / 32;
      copy_in(sat<int>(o.rowptr), F.sell_ptr, ns + 1);
      copy_in(sat<unsigned short>(o.col), F.sell_col, F.sell_len);
      copy_in(sat<unsigned short>(o.perm), F.sell_row, 32 * ns);
      float* va = sat<float>(o.val);
      for (int e = threadIdx.x; e < F.sell_len; e += kGmThreads) {
        const int src = __ldg(F.sell_src + e);
        va[e] = src >= 0 ? F.val[k0 + src] : 0.0f;
      }
      copy_in(sat<float>(o.wdinv), (const float*)F.wdinv + row0, F.n);
      copy_in(sat<int>(o.agg), F.agg + row0, F.n);
      copy_in(sat<int>(o.ptptr), F.ptptr, L[l + 1].n + 1);
      copy_in(sat<int>(o.ptrow), F.ptrow, F.n, row0);
    } else {
      copy_in(sat<float>(T.inv), coarse_inv, F.n * F.n);
    }
  }
  __syncthreads();
}

// Tail levels in shared memory, cycled by every member of a team.  Per level l: R (residual in),
// X (correction out), T (scratch); R_l is read-only while a cycle runs through level l.

// sum over the row at SELL-32 position p of a shared-memory matrix (slice offsets sp, columns
// cl, values va) of va * f(column), in the row's CSR order followed by its zero padding.  The
// positions of a warp are 32 consecutive positions of one slice, so every load of a column or
// value is one conflict-free shared-memory access; the loads of up to eight entries are issued
// together.
template <class F>
__device__ __forceinline__ float sell_row(const int* sp, const unsigned short* cl, const float* va, int p, F f) {
  const int sl = p >> 5;
  const int b0 = sp[sl] + (p & 31), w = (sp[sl + 1] - sp[sl]) >> 5;
  float s = 0.0f;
  for (int k0 = 0; k0 < w; k0 += 8) {
    int c[8];
    float v[8], x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const bool ok = k0 + q < w;
      c[q] = ok ? (int)cl[b0 + 32 * (k0 + q)] : 0;
      v[q] = ok ? va[b0 + 32 * (k0 + q)] : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = k0 + q < w ? f(c[q]) : 0.0f;
#pragma unroll
    for (int q = 0; q < 8; q++) s += v[q] * x[q];
  }
  return s;
}

// pre-smoothing and restriction: X_l = w D^-1 R_l, T_l = R_l - A_l X_l, R_{l+1} = P^T T_l.  X is
// written in a pass of its own, so the residual gathers one shared-memory value per entry.
__device__ void tail_down(const AmgDevLevel* L, const TailLayout& T, unsigned char* sb, int l) {
  const int tid = threadIdx.x;
  const TailLevelOff& o = T.lv[l];
  const int n = L[l].n, nc = L[l + 1].n;
  const int* rp = sat<int>(o.rowptr);
  const unsigned short* cl = sat<unsigned short>(o.col);
  const float* va = sat<float>(o.val);
  const float* wd = sat<float>(o.wdinv);
  const float* R = sat<float>(o.R);
  float* X = sat<float>(o.X);
  float* Tt = sat<float>(o.T);
  const unsigned short* pm = sat<unsigned short>(o.perm);
  for (int i = tid; i < n; i += kGmThreads) X[i] = wd[i] * R[i];
  __syncthreads();
  for (int p = tid; p < n; p += kGmThreads) {  // one shared-memory gather per entry
    const int i = pm[p];
    Tt[i] = R[i] - sell_row(rp, cl, va, p, [&](int j) { return X[j]; });
  }
  __syncthreads();
  const int* pp = sat<int>(o.ptptr);
  const int* pr = sat<int>(o.ptrow);
  float* Rn = sat<float>(T.lv[l + 1].R);
  for (int I = tid; I < nc; I += kGmThreads) {
    const int q0 = pp[I], q1 = pp[I + 1];
    float s = 0.0f;
    for (int q = q0; q < q1; q += 8) {
      float t[8];
#pragma unroll
      for (int u = 0; u < 8; u++) t[u] = q + u < q1 ? Tt[pr[q + u]] : 0.0f;
#pragma unroll
      for (int u = 0; u < 8; u++) s += t[u];
    }
    Rn[I] = s;
  }
  __syncthreads();
}

// the coarsest level: X = (A + s 11^T)^-1 R, one warp per row
__device__ void tail_coarsest(const AmgDevLevel* L, int nlev, const TailLayout& T, unsigned char* sb) {
  const int tid = threadIdx.x;
  const int n = L[nlev - 1].n;
  const float* inv = sat<float>(T.inv);
  const float* R = sat<float>(T.lv[nlev - 1].R);
  float* X = sat<float>(T.lv[nlev - 1].X);
  const int lane = tid & 31, wid = tid >> 5;
  for (int i = wid; i < n; i += kGmWarps) {
    float s = 0.0f;
    for (int j = lane; j < n; j += 32) s += inv[i * n + j] * R[j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) X[i] = s;
  }
  __syncthreads();
}

// prolongation and post-smoothing: Y = X_l + alpha P X_{l+1}, X_l = Y + w D^-1 (R_l - A_l Y)
__device__ void tail_up(const AmgDevLevel* L, const TailLayout& T, float alpha, unsigned char* sb, int l) {
  const int tid = threadIdx.x;
  const TailLevelOff& o = T.lv[l];
  const int n = L[l].n;
  const int* rp = sat<int>(o.rowptr);
  const unsigned short* cl = sat<unsigned short>(o.col);
  const float* va = sat<float>(o.val);
  const float* wd = sat<float>(o.wdinv);
  const int* ag = sat<int>(o.agg);
  const float* R = sat<float>(o.R);
  float* X = sat<float>(o.X);
  float* Y = sat<float>(o.T);
  const float* Xc = sat<float>(T.lv[l + 1].X);
  for (int i = tid; i < n; i += kGmThreads) Y[i] = X[i] + alpha * Xc[ag[i]];
  __syncthreads();
  const unsigned short* pm = sat<unsigned short>(o.perm);
  for (int p = tid; p < n; p += kGmThreads) {
    const int i = pm[p];
    const float acc = sell_row(rp, cl, va, p, [&](int j) { return Y[j]; });
    X[i] = Y[i] + wd[i] * (R[i] - acc);
  }
  __syncthreads();
}

// V-cycle from tail level s to the coarsest: R_s in, X_s out
__device__ void tail_v(const AmgDevLevel* L, int nlev, const TailLayout& T, float alpha, unsigned char* sb, int s) {
  for (int l = s; l + 1 < nlev; l++) tail_down(L, T, sb, l);
  tail_coarsest(L, nlev, T, sb);
  for (int l = nlev - 2; l >= s; l--) tail_up(L, T, alpha, sb, l);
}

// every member of a team: the cycle from level T.tail down, in its own shared memory (the
// members compute the same values in the same order, so each holds the whole coarse correction
// and the prolongation below needs no barrier).  The input residual is the tail level's r; the
// correction stays in shared memory (X of the tail level) or, when the tail is the whole
// hierarchy, the member's share of rows [lo, hi) goes to the FP64 vector z.  The first coarse
// level of the tail (g = max(tail, 1)) is solved by gamma cycles, x <- x + V(r_g - A_g x) (a
// W-cycle for gamma 2): the tail levels are cheap, with no grid barrier, and a more accurate
// coarse correction cuts the outer CG iterations; g moves further down while its level has
// more than kAmgWLevelRows rows.  `buf` holds the accumulated x and the original r_g (2 n_g
// floats).
__device__ void tail_cycle(const AmgDevLevel* L, int nlev, const TailLayout& T, float alpha, int gamma,
                                        unsigned char* sb, float* buf, int r0, int r1, int lo, double* z) {
  const int tid = threadIdx.x;
  const int t0 = T.tail;
  {
    float* R = sat<float>(T.lv[t0].R);
    const float* rin = t0 == 0 ? L[0].r + lo : L[t0].r;
    for (int i = tid; i < L[t0].n; i += kGmThreads) R[i] = ldcgf(rin + i);
  }
  __syncthreads();
  // the W-cycle's level: the first tail level below level 0 small enough for the second cycle
  // to be cheap (each tail pass runs on one SM's shared memory)
  int g = t0 > 1 ? t0 : 1;
  while (g < nlev - 1 && L[g].n > kAmgWLevelRows) g++;
  if (gamma > 1 && g < nlev - 1 && 2 * L[g].n <= kAmgDownBuf) {
    for (int l = t0; l < g; l++) tail_down(L, T, sb, l);
    const TailLevelOff& o = T.lv[g];
    const int n = L[g].n;
    const int* rp = sat<int>(o.rowptr);
    const unsigned short* cl = sat<unsigned short>(o.col);
    const float* va = sat<float>(o.val);
    float* R = sat<float>(o.R);
    float* X = sat<float>(o.X);
    float* S = sat<float>(T.bytes);  // accumulated correction (the restriction buffer)
    float* Q = S + n;                // the level's original residual
    const unsigned short* pm = sat<unsigned short>(o.perm);
    tail_v(L, nlev, T, alpha, sb, g);
    for (int rep = 1; rep < gamma; rep++) {
      for (int i = tid; i < n; i += kGmThreads) {
        S[i] = rep == 1 ? X[i] : S[i] + X[i];
        if (rep == 1) Q[i] = R[i];
      }
      __syncthreads();
      for (int p = tid; p < n; p += kGmThreads) {
        const int i = pm[p];
        R[i] = Q[i] - sell_row(rp, cl, va, p, [&](int j) { return S[j]; });
      }
      __syncthreads();
      tail_v(L, nlev, T, alpha, sb, g);
    }
    for (int i = tid; i < n; i += kGmThreads) X[i] = S[i] + X[i];
    __syncthreads();
    for (int l = g - 1; l >= t0; l--) tail_up(L, T, alpha, sb, l);
  } else {
    tail_v(L, nlev, T, alpha, sb, t0);
  }
  if (t0 == 0) {
    const float* X = sat<float>(T.lv[0].X);
    for (int r = r0 + tid; r < r1; r += kGmThreads) z[r] = (double)X[r - lo];
  }
}

// level l -> l+1 on the team: each member takes a block of coarse rows, computes the smoothed
// residual t_i = r_i - A_i (w D^-1 r) of their fine rows (in aggregate order; w D^-1 r is kept
// per row, so an entry gathers one value) into shared memory and into F.sr (for the way up), and
// sums each aggregate: r_{l+1} = P^T t, with w D^-1 r_{l+1} when level l+1 is cycled by the grid
// too (c_grid).  Only r_l is read, so no barrier separates smoothing from restriction.
__device__ __forceinline__ void grid_down(const AmgDevLevel& F, const AmgDevLevel& C, bool c_grid, const Team& Tm,
                                          float* buf) {
  const Rows cr = share(0, C.n, Tm);
  const int G = max(1, kAmgDownBuf / max(1, F.maxagg));
  const float* rl = F.r;
  const float* wr = F.wr;
  for (int I0 = cr.r0; I0 < cr.r1; I0 += G) {
    const int I1 = min(I0 + G, cr.r1);
    const int k0 = __ldg(F.ptptr + I0), k1 = __ldg(F.ptptr + I1);
    for (int k = k0 + threadIdx.x; k < k1; k += kGmThreads) {
      const int i = __ldg(F.ptrow + k);
      const float ri = ldcgf(rl + i);
      const float acc = row_gather_f<8>(F.rowptr, F.col, F.val, i, [&](int j) { return ldcgf(wr + j); });
      buf[k - k0] = ri - acc;
      F.sr[i] = ri - acc;
    }
    __syncthreads();
    for (int I = I0 + threadIdx.x; I < I1; I += kGmThreads) {
      const int q0 = __ldg(F.ptptr + I), q1 = __ldg(F.ptptr + I + 1);
      float s = 0.0f;
      for (int q = q0; q < q1; q++) s += buf[q - k0];
      C.r[I] = s;
      if (c_grid) C.wr[I] = __ldg(C.wdinv + I) * s;
    }
    __syncthreads();
  }
}

// prolongation of the coarse correction and post-smoothing on rows rw of a level:
// out = y + w D^-1 (r - A y),  y = w D^-1 r + a P x_C; level 0 writes the FP64 z.  With
// t = r - A w D^-1 r kept from the way down (F.sr), r - A y = t - a A P x_C, so an entry gathers
// only the coarse correction of its column's aggregate (F.aggcol).  xc(I) reads the coarse
// correction of coarse row I (from global memory, or from the tail in shared memory)
template <class XC>
__device__ __forceinline__ void grid_up(const AmgDevLevel& F, XC xc, float alpha, Rows rw, float* outf,
                                        double* outd) {
  const int* agg = F.agg;
  for (int i = rw.r0 + threadIdx.x; i < rw.r1; i += kGmThreads) {
    const float wi = __ldg(F.wdinv + i);
    const float y = ldcgf(F.wr + i) + alpha * xc(__ldg(agg + i));
    const float acc = row_gather_f<8>(F.rowptr, F.aggcol, F.val, i, [&](int J) { return xc(J); });
    const float o = y + wi * (ldcgf(F.sr + i) - alpha * acc);
    if (outd) outd[i] = (double)o;
    else outf[i] = o;
  }
}

// z = M r for the case's rows [lo, hi) of the residual held in L[0].r; false after a barrier
// timeout.  Barriers: one per grid level down, none between the tail and the first level up
// (every member holds the tail's correction), one per grid level up.
__device__ bool vcycle(const AmgDevLevel* L, int nlev, const TailLayout& T, float alpha, int gamma, unsigned char* sb,
                       float* buf, int lo, int hi, double* z, const Team& Tm, int* err) {
  const int t0 = T.tail;
  for (int l = 0; l < t0; l++) {
    grid_down(L[l], L[l + 1], l + 1 < t0, Tm, buf);
    if (!grid_barrier(Tm.bar, Tm.size, err)) return false;
  }
  const Rows own = share(lo, hi, Tm);
  tail_cycle(L, nlev, T, alpha, gamma, sb, buf, own.r0, own.r1, lo, z);
  if (t0 == 0) return grid_barrier(Tm.bar, Tm.size, err);
  const float* Xs = sat<float>(T.lv[t0].X);
  for (int l = t0 - 1; l >= 0; l--) {
    const Rows rw = l == 0 ? own : share(0, L[l].n, Tm);
    float* outf = l == 0 ? nullptr : L[l].t;
    double* outd = l == 0 ? z : nullptr;
    if (l == t0 - 1) {
      grid_up(L[l], [&](int I) { return Xs[I]; }, alpha, rw, outf, outd);
    } else {
      const float* xc = L[l + 1].t;
      grid_up(L[l], [&](int I) { return ldcgf(xc + I); }, alpha, rw, outf, outd);
    }
    if (!grid_barrier(Tm.bar, Tm.size, err)) return false;
  }
  return true;
}

__device__ __forceinline__ int sgn(double v) { return (v > 0) - (v < 0); }

// FCG(1) in Chronopoulos-Gear form on rows [lo, hi) of case c by team Tm
__device__ void cg_amg_team(const CgAmgArgs& a, const Team& Tm, int c) {
  extern __shared__ __align__(16) unsigned char s_dyn[];
  __shared__ double s_warp[kGmWarps * kDotGroup];
  __shared__ double s_red[kDotGroup];
  __shared__ double s_g[5];
  __shared__ AmgDevLevel s_lv[kAmgMaxLevels];
  __shared__ TailLayout s_tl;
  __shared__ int s_case[4];  // lo, hi, nlev, gamma
  const int tid = threadIdx.x;
  const AmgCaseDesc* cd = a.cases + c;
  if (tid == 0) {
    s_case[0] = cd->lo;
    s_case[1] = cd->hi;
    s_case[2] = cd->nlev;
    s_case[3] = cd->gamma;
  }
  for (int k = tid; k < (int)(sizeof(TailLayout) / sizeof(int)); k += kGmThreads)
    reinterpret_cast<int*>(&s_tl)[k] = reinterpret_cast<const int*>(&cd->tl)[k];
  __syncthreads();
  const int lo = s_case[0], hi = s_case[1], nlev = s_case[2], gamma = s_case[3];
  for (int l = tid; l < nlev; l += kGmThreads) s_lv[l] = cd->levels[l];
  __syncthreads();
  unsigned char* sb = s_dyn;
  float* buf = reinterpret_cast<float*>(s_dyn + s_tl.bytes);
  tail_load(s_lv, nlev, s_tl, cd->coarse_inv, lo, sb);
  const Rows own = share(lo, hi, Tm);
  const int stride = kPartStride;
  double* mypart = Tm.part + (long)Tm.rank * stride;
  const float alc = a.alpha;
  float* r32 = s_lv[0].r;
  float* wr32 = s_lv[0].wr;
  const float* wd32 = s_lv[0].wdinv;

  // initial residual r = b - A x (or b); the V-cycle input is its FP32 copy
  for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
    const double br = a.b[r];
    double t;
    if (a.guess_zero) {
      a.x[r] = 0.0;
      t = br;
    } else {
      const double* vv_ = a.x;
      double s = row_gather<5>(a.rowptr, a.col, a.val, r, [&](int cc) { return ldcg(vv_ + cc); });
      t = br - s;
    }
    a.r[r] = t;
    r32[r] = (float)br;
    wr32[r] = wd32[r] * (float)br;
  }
  if (!grid_barrier(Tm.bar, Tm.size, a.err)) return;
  if (!a.guess_zero) {  // |M b| is the reference norm of a nonzero initial guess
    if (!vcycle(s_lv, nlev, s_tl, alc, gamma, sb, buf, lo, hi, a.u, Tm, a.err)) return;
    double acc[1] = {0.0};
    for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
      const double zb = ldcg(a.u + r);
      acc[0] += zb * zb;
      r32[r] = (float)ldcg(a.r + r);
      wr32[r] = wd32[r] * r32[r];
    }
    block_reduce<1>(acc, s_warp, s_red);
    if (tid == 0) mypart[kMaxRestart + 3] = s_red[0];
    if (!grid_barrier(Tm.bar, Tm.size, a.err)) return;
  }
  if (!vcycle(s_lv, nlev, s_tl, alc, gamma, sb, buf, lo, hi, a.u, Tm, a.err)) return;

  // CG scalars are uniform over the CTA: thread 0 keeps them in shared memory
  __shared__ double s_sc[8];  // rnorm0, ttol, dp, gam_old, dpi_old, alpha, beta
  __shared__ int s_st[3];     // reason, its, stop
  for (int i = 0;; i++) {
    // w = A u and the inner products (r,u), (w,u), (u,u), (u, s_old) of u = M r
    {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      const double* uu = a.u;
      for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
        const double s = row_gather<5>(a.rowptr, a.col, a.val, r, [&](int cc) { return ldcg(uu + cc); });
        a.w[r] = s;
        const double ur = ldcg(uu + r);
        acc[0] += ur * ldcg(a.r + r);
        acc[1] += s * ur;
        acc[2] += ur * ur;
        if (i > 0) acc[3] += ur * ldcg(a.s + r);
      }
      block_reduce<4>(acc, s_warp, s_red);
      if (tid < 4) mypart[tid] = s_red[tid];
    }
    if (!grid_barrier(Tm.bar, Tm.size, a.err)) return;
    if (tid < 160) {
      const int q = tid >> 5;
      if (q < 4 || (i == 0 && !a.guess_zero)) {
        double s = warp_sum_blocks(Tm.part, stride, q < 4 ? q : kMaxRestart + 3, Tm.size);
        if ((tid & 31) == 0) s_g[q] = s;
      }
    }
    __syncthreads();
    if (tid == 0) {
      const double gam = s_g[0], del = s_g[1], mu = s_g[3];
      const double dp = sqrt(s_g[2]);
      if (i == 0) {
        s_sc[0] = a.guess_zero ? dp : (s_g[4] != 0.0 ? sqrt(s_g[4]) : dp);
        s_sc[1] = fmax(a.rtol * s_sc[0], a.abstol);
      }
      const double rnorm0 = s_sc[0], ttol = s_sc[1], gam_old = s_sc[3], dpi_old = s_sc[4];
      s_sc[2] = dp;
      int reason = 0, its = i + 1, stop = 1;
      if (isnan(dp) || isinf(dp)) reason = -9;
      else if (dp <= ttol) reason = dp < a.abstol ? 3 : 2;
      else if (dp >= a.dtol * rnorm0) reason = -4;
      if (reason) its = i;
      else if (i >= a.maxit) {
        reason = -3;
        its = i;
      } else if (gam == 0.0) {
        reason = 3;
      } else if (i > 0 && gam * gam_old < 0.0) {
        reason = -8;
      } else {
        const double beta = i == 0 ? 0.0 : -mu / dpi_old;
        const double dpi = i == 0 ? del : del + beta * mu;  // (p, A p)
        if (dpi == 0.0 || (i > 0 && sgn(dpi) * sgn(dpi_old) < 0)) {
          reason = -10;
        } else {
          stop = 0;
          s_sc[3] = gam;
          s_sc[4] = dpi;
          s_sc[5] = gam / dpi;
          s_sc[6] = beta;
        }
      }
      s_st[0] = reason;
      s_st[1] = its;
      s_st[2] = stop;
    }
    __syncthreads();
    if (s_st[2]) break;
    const double alpha = s_sc[5], beta = s_sc[6];
    {
      const double* __restrict__ U = a.u;
      const double* __restrict__ Wv = a.w;
      double* __restrict__ P = a.p;
      double* __restrict__ S = a.s;
      double* __restrict__ X = a.x;
      double* __restrict__ R = a.r;
      for (int r0 = own.r0 + tid; r0 < own.r1; r0 += 2 * kGmThreads) {
        const int r1 = r0 + kGmThreads;
        const bool h1 = r1 < own.r1;
        const double u0 = ldcg(U + r0), w0 = ldcg(Wv + r0), x0 = ldcg(X + r0), q0 = ldcg(R + r0);
        const double p0 = i == 0 ? 0.0 : ldcg(P + r0), s0 = i == 0 ? 0.0 : ldcg(S + r0);
        double u1 = 0.0, w1 = 0.0, x1 = 0.0, q1 = 0.0, p1 = 0.0, s1 = 0.0;
        if (h1) {
          u1 = ldcg(U + r1);
          w1 = ldcg(Wv + r1);
          x1 = ldcg(X + r1);
          q1 = ldcg(R + r1);
          if (i > 0) {
            p1 = ldcg(P + r1);
            s1 = ldcg(S + r1);
          }
        }
        const double pn0 = u0 + beta * p0, sn0 = w0 + beta * s0, rn0 = q0 - alpha * sn0;
        P[r0] = pn0;
        S[r0] = sn0;
        X[r0] = x0 + alpha * pn0;
        R[r0] = rn0;
        r32[r0] = (float)rn0;
        wr32[r0] = wd32[r0] * (float)rn0;
        if (h1) {
          const double pn1 = u1 + beta * p1, sn1 = w1 + beta * s1, rn1 = q1 - alpha * sn1;
          P[r1] = pn1;
          S[r1] = sn1;
          X[r1] = x1 + alpha * pn1;
          R[r1] = rn1;
          r32[r1] = (float)rn1;
          wr32[r1] = wd32[r1] * (float)rn1;
        }
      }
    }
    if (!grid_barrier(Tm.bar, Tm.size, a.err)) return;
    if (!vcycle(s_lv, nlev, s_tl, alc, gamma, sb, buf, lo, hi, a.u, Tm, a.err)) return;
  }
  if (Tm.rank == 0 && tid == 0) {
    a.out[c].its = s_st[1];
    a.out[c].reason = s_st[0];
    a.out[c].rnorm = s_sc[2];
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kGmThreads, 1) k_cg_amg(CgAmgArgs a) {
  if (launch_failed(a.err)) return;
  if (!a.sched) {
    const Team T{(int)blockIdx.x, a.nb, a.bar, a.part};
    cg_amg_team(a, T, 0);
    return;
  }
  const BatchSchedule& S = *a.sched;
  const int team = S.cta_team[blockIdx.x];
  const Team T{S.cta_rank[blockIdx.x], S.team_size[team], a.bar + 2L * team,
               a.part + (long)S.team_cta0[team] * kPartStride};
  for (int k = S.team_case0[team]; k < S.team_case0[team + 1]; k++) {
    cg_amg_team(a, T, S.case_list[k]);
    if (*(volatile int*)a.err) return;
  }
}

}  // namespace

void launch_amg_setup_values(const AmgHostView& h, cudaStream_t s) {
  // FP32 copy of the pressure matrix, Galerkin sums down every hierarchy, Jacobi weights, and
  // the dense inverse of every case's coarsest level
  const int D = (int)h.dep.size();
  const AmgHostView::Depth& d0 = h.dep[0];
  ++g_launch_count, k_amg_level0<<<(d0.nnz + kThreads - 1) / kThreads, kThreads, 0, s>>>(
                        d0.nnz, h.val64, d0.val, d0.diag_row, h.omega, d0.wdinv);
  for (int l = 0; l + 1 < D; l++) {
    const AmgHostView::Depth& F = h.dep[l];
    const AmgHostView::Depth& C = h.dep[l + 1];
    ++g_launch_count, k_amg_galerkin<<<(C.nnz + kThreads - 1) / kThreads, kThreads, 0, s>>>(
                          C.nnz, F.cptr, F.csrc, F.val, C.val, C.diag_row, h.omega, C.wdinv);
  }
  ++g_launch_count, k_amg_coarse_inverse<<<h.ncases, 1024, 0, s>>>(h.d_cases);
}

cudaError_t launch_cg_amg(const GmresCall& c, const AmgHostView& h, KrylovWork& w, const BatchSchedule* sched,
                          int grid, KspOut* out, cudaStream_t s) {
  if (5L * w.ldv > w.v_len || (long)grid * kPartStride > w.part_len || w.ldv < c.n || h.ncases < 1 ||
      grid < 1 || (!sched && h.ncases != 1))
    return cudaErrorInvalidValue;
  for (int k = 0; k < h.ncases; k++) {
    const AmgCaseDesc& cd = h.cases[k];
    if (cd.nlev < 1 || cd.nlev > kAmgMaxLevels || h.levels[k][cd.nlev - 1].n > kAmgCoarseMax || cd.lo < 0 ||
        cd.hi > c.n || cd.lo >= cd.hi)
      return cudaErrorInvalidValue;
    for (int l = 0; l + 1 < cd.nlev; l++)
      if (h.levels[k][l].maxagg > kAmgDownBuf) return cudaErrorInvalidValue;
  }
  CgAmgArgs a;
  a.n = c.n;
  a.maxit = c.maxit;
  a.guess_zero = c.guess_zero;
  a.nb = grid;
  a.rowptr = c.rowptr;
  a.col = c.col;
  a.val = c.val;
  a.b = c.b;
  a.x = c.x;
  a.r = w.V;
  a.u = w.V + w.ldv;
  a.p = w.V + 2 * w.ldv;
  a.w = w.V + 3 * w.ldv;
  a.s = w.V + 4 * w.ldv;
  a.part = w.part;
  a.bar = w.bar;
  a.err = c.err;
  a.out = out;
  a.rtol = c.rtol;
  a.abstol = 1e-50;
  a.dtol = 1e4;
  a.alpha = h.alpha;
  a.cases = h.d_cases;
  a.sched = sched;
  const int smem = h.smem_bytes;
  cudaError_t e = cudaFuncSetAttribute((const void*)k_cg_amg, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  void* args[] = {&a};
  return launch_cooperative((const void*)k_cg_amg, grid, kGmThreads, args, smem, s);
}

}  // namespace cycas
