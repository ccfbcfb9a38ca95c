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
// chosen so that their matrices fit in shared memory) are loaded into CTA 0's shared memory
// once per solve and cycled there with block barriers only.  CG itself is the
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
constexpr int kDownBuf = 8192;             // floats of the per-CTA restriction buffer
constexpr int kTailBudget = 160 * 1024;    // shared-memory bytes for the tail levels

// ---------------------------------------------------------------- per-solve setup
__global__ void k_amg_level0(int nnz, const double* __restrict__ val64, float* __restrict__ val) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nnz) val[k] = (float)val64[k];
}

__global__ void k_amg_galerkin(int nnz_c, const int* __restrict__ cptr, const int* __restrict__ csrc,
                               const float* __restrict__ valf, float* __restrict__ valc) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nnz_c) return;
  float s = 0.0f;
  for (int q = cptr[c]; q < cptr[c + 1]; q++) s += valf[csrc[q]];
  valc[c] = s;
}

__global__ void k_amg_wdinv(int n, float omega, const int* __restrict__ diag, const float* __restrict__ val,
                            float* __restrict__ wdinv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wdinv[i] = omega / val[diag[i]];
}

// dense inverse of A_L + s 11^T, s = mean(diag)/n, by in-place Gauss-Jordan in shared memory.
// A_L is singular with the constant null vector (row sums vanish); the shift has the sign of
// the diagonal, so the shifted matrix is definite.  Pivoting is not needed for a definite matrix.
__global__ void k_amg_coarse_inverse(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                     const int* __restrict__ diag, const float* __restrict__ val,
                                     float* __restrict__ inv) {
  __shared__ float M[kAmgCoarseMax * kAmgCoarseMax];
  __shared__ float colk[kAmgCoarseMax];
  __shared__ float s_shift;
  const int tid = threadIdx.x;
  for (int e = tid; e < n * n; e += blockDim.x) M[e] = 0.0f;
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x)
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) M[i * n + col[k]] = val[k];
  if (tid == 0) {
    float d = 0.0f;
    for (int i = 0; i < n; i++) d += val[diag[i]];
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
struct TailLevelOff {  // byte offsets of one tail level's arrays in dynamic shared memory
  int rowptr, col, val, wdinv, agg, ptptr, ptrow, R, X, T;
};

struct TailLayout {
  int tail;   // first level cycled by CTA 0 from shared memory (levels tail..nlev-1)
  int bytes;  // dynamic shared memory taken by the tail (multiple of 16)
  int inv;    // offset of the coarsest level's dense inverse
  TailLevelOff lv[kAmgMaxLevels];
};

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
  KspOut* out;
  double rtol, abstol, dtol;
  AmgDev amg;
  TailLayout tl;
};

struct Rows {
  int r0, r1;
};
__device__ __forceinline__ Rows own_rows(int n, int nb) {
  int ch = (n + nb - 1) / nb;
  int r0 = blockIdx.x * ch;
  return {min(r0, n), min(n, r0 + ch)};
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

template <class T>
__device__ __forceinline__ void copy_in(T* dst, const T* src, int cnt) {
  for (int i = threadIdx.x; i < cnt; i += kGmThreads) dst[i] = src[i];
}

// CTA 0: the tail levels' matrices, transfer lists and the coarsest inverse into shared memory
__device__ void tail_load(const AmgDevLevel* L, int nlev, const TailLayout& T, const float* coarse_inv,
                          unsigned char* sb) {
  for (int l = T.tail; l < nlev; l++) {
    const AmgDevLevel& F = L[l];
    const TailLevelOff& o = T.lv[l];
    if (l + 1 < nlev) {
      copy_in(at<int>(sb, o.rowptr), F.rowptr, F.n + 1);
      copy_in(at<int>(sb, o.col), F.col, F.nnz);
      copy_in(at<float>(sb, o.val), (const float*)F.val, F.nnz);
      copy_in(at<float>(sb, o.wdinv), (const float*)F.wdinv, F.n);
      copy_in(at<int>(sb, o.agg), F.agg, F.n);
      copy_in(at<int>(sb, o.ptptr), F.ptptr, L[l + 1].n + 1);
      copy_in(at<int>(sb, o.ptrow), F.ptrow, F.n);
    } else {
      copy_in(at<float>(sb, T.inv), coarse_inv, F.n * F.n);
    }
  }
  __syncthreads();
}

// CTA 0: the V-cycle from level T.tail down, in shared memory; its input residual is
// L[tail].r and its correction goes to L[tail].t (or, when the tail is the whole hierarchy,
// to the FP64 vector z)
__device__ void tail_cycle(const AmgDevLevel* L, int nlev, const TailLayout& T, float alpha, unsigned char* sb,
                           double* z) {
  const int tid = threadIdx.x;
  const int t0 = T.tail;
  {
    float* R = at<float>(sb, T.lv[t0].R);
    const float* rin = L[t0].r;
    for (int i = tid; i < L[t0].n; i += kGmThreads) R[i] = ldcgf(rin + i);
  }
  __syncthreads();
  for (int l = t0; l + 1 < nlev; l++) {
    const TailLevelOff& o = T.lv[l];
    const int n = L[l].n, nc = L[l + 1].n;
    const int* rp = at<int>(sb, o.rowptr);
    const int* cl = at<int>(sb, o.col);
    const float* va = at<float>(sb, o.val);
    const float* wd = at<float>(sb, o.wdinv);
    const float* R = at<float>(sb, o.R);
    float* X = at<float>(sb, o.X);
    float* Tt = at<float>(sb, o.T);
    for (int i = tid; i < n; i += kGmThreads) X[i] = wd[i] * R[i];
    __syncthreads();
    for (int i = tid; i < n; i += kGmThreads) {
      float acc = 0.0f;
      for (int k = rp[i]; k < rp[i + 1]; k++) acc += va[k] * X[cl[k]];
      Tt[i] = R[i] - acc;
    }
    __syncthreads();
    const int* pp = at<int>(sb, o.ptptr);
    const int* pr = at<int>(sb, o.ptrow);
    float* Rn = at<float>(sb, T.lv[l + 1].R);
    for (int I = tid; I < nc; I += kGmThreads) {
      float s = 0.0f;
      for (int q = pp[I]; q < pp[I + 1]; q++) s += Tt[pr[q]];
      Rn[I] = s;
    }
    __syncthreads();
  }
  {
    const int n = L[nlev - 1].n;
    const float* inv = at<float>(sb, T.inv);
    const float* R = at<float>(sb, T.lv[nlev - 1].R);
    float* X = at<float>(sb, T.lv[nlev - 1].X);
    const int lane = tid & 31, wid = tid >> 5;
    for (int i = wid; i < n; i += kGmWarps) {
      float s = 0.0f;
      for (int j = lane; j < n; j += 32) s += inv[i * n + j] * R[j];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) X[i] = s;
    }
  }
  __syncthreads();
  for (int l = nlev - 2; l >= t0; l--) {
    const TailLevelOff& o = T.lv[l];
    const int n = L[l].n;
    const int* rp = at<int>(sb, o.rowptr);
    const int* cl = at<int>(sb, o.col);
    const float* va = at<float>(sb, o.val);
    const float* wd = at<float>(sb, o.wdinv);
    const int* ag = at<int>(sb, o.agg);
    const float* R = at<float>(sb, o.R);
    float* X = at<float>(sb, o.X);
    float* Y = at<float>(sb, o.T);
    const float* Xc = at<float>(sb, T.lv[l + 1].X);
    for (int i = tid; i < n; i += kGmThreads) Y[i] = X[i] + alpha * Xc[ag[i]];
    __syncthreads();
    for (int i = tid; i < n; i += kGmThreads) {
      float acc = 0.0f;
      for (int k = rp[i]; k < rp[i + 1]; k++) acc += va[k] * Y[cl[k]];
      X[i] = Y[i] + wd[i] * (R[i] - acc);
    }
    __syncthreads();
  }
  {
    const float* X = at<float>(sb, T.lv[t0].X);
    if (t0 == 0) {
      for (int i = tid; i < L[0].n; i += kGmThreads) z[i] = (double)X[i];
    } else {
      float* out = L[t0].t;
      for (int i = tid; i < L[t0].n; i += kGmThreads) out[i] = X[i];
    }
  }
}

// grid level l -> l+1: each CTA takes a block of coarse rows, computes the smoothed residual
// t_i = r_i - A_i (w D^-1 r) of their fine rows (in aggregate order) into shared memory and
// sums each aggregate: r_{l+1} = P^T t.  Only r_l is read, so no barrier separates smoothing
// from restriction.
__device__ __forceinline__ void grid_down(const AmgDevLevel& F, const AmgDevLevel& C, int nb, float* buf) {
  const Rows cr = own_rows(C.n, nb);
  const int G = max(1, kDownBuf / max(1, F.maxagg));
  const float* rl = F.r;
  const float* wd = F.wdinv;
  for (int I0 = cr.r0; I0 < cr.r1; I0 += G) {
    const int I1 = min(I0 + G, cr.r1);
    const int k0 = __ldg(F.ptptr + I0), k1 = __ldg(F.ptptr + I1);
    for (int k = k0 + threadIdx.x; k < k1; k += kGmThreads) {
      const int i = __ldg(F.ptrow + k);
      const float ri = ldcgf(rl + i);
      float acc = row_gather_f<8>(F.rowptr, F.col, F.val, i, [&](int j) { return __ldg(wd + j) * ldcgf(rl + j); });
      buf[k - k0] = ri - acc;
    }
    __syncthreads();
    for (int I = I0 + threadIdx.x; I < I1; I += kGmThreads) {
      const int q0 = __ldg(F.ptptr + I), q1 = __ldg(F.ptptr + I + 1);
      float s = 0.0f;
      for (int q = q0; q < q1; q++) s += buf[q - k0];
      C.r[I] = s;
    }
    __syncthreads();
  }
}

// prolongation of the coarse correction and post-smoothing on the CTA's rows of grid level
// l: out = y + w D^-1 (r - A y),  y = w D^-1 r + a P x_C; level 0 writes the FP64 z
__device__ __forceinline__ void grid_up(const AmgDevLevel& F, const float* xc, float alpha, Rows rw, float* outf,
                                        double* outd) {
  const float* rl = F.r;
  const float* wd = F.wdinv;
  const int* agg = F.agg;
  for (int i = rw.r0 + threadIdx.x; i < rw.r1; i += kGmThreads) {
    const float ri = ldcgf(rl + i);
    const float wi = __ldg(wd + i);
    const float y = wi * ri + alpha * ldcgf(xc + __ldg(agg + i));
    float acc = row_gather_f<8>(F.rowptr, F.col, F.val, i, [&](int j) {
      return __ldg(wd + j) * ldcgf(rl + j) + alpha * ldcgf(xc + __ldg(agg + j));
    });
    const float o = y + wi * (ri - acc);
    if (outd) outd[i] = (double)o;
    else outf[i] = o;
  }
}

// z = M r for the residual held in L[0].r; every CTA participates; false after a barrier timeout
__device__ bool vcycle(const AmgDevLevel* L, int nlev, const TailLayout& T, float alpha, unsigned char* sb,
                       float* buf, double* z, unsigned* bar, unsigned nb, int* err) {
  const int t0 = T.tail;
  for (int l = 0; l < t0; l++) {
    grid_down(L[l], L[l + 1], nb, buf);
    if (!grid_barrier(bar, nb, err)) return false;
  }
  if (blockIdx.x == 0) tail_cycle(L, nlev, T, alpha, sb, z);
  if (!grid_barrier(bar, nb, err)) return false;
  for (int l = t0 - 1; l >= 0; l--) {
    grid_up(L[l], L[l + 1].t, alpha, own_rows(L[l].n, nb), l == 0 ? nullptr : L[l].t, l == 0 ? z : nullptr);
    if (!grid_barrier(bar, nb, err)) return false;
  }
  return true;
}

__device__ __forceinline__ int sgn(double v) { return (v > 0) - (v < 0); }

__global__ void __launch_bounds__(kGmThreads, 1) k_cg_amg(CgAmgArgs a) {
  extern __shared__ __align__(16) unsigned char s_dyn[];
  __shared__ double s_warp[kGmWarps * kDotGroup];
  __shared__ double s_red[kDotGroup];
  __shared__ double s_g[5];
  __shared__ AmgDevLevel s_lv[kAmgMaxLevels];
  const int nb = a.nb, tid = threadIdx.x;
  const int nlev = a.amg.nlev;
  for (int l = tid; l < nlev; l += kGmThreads) s_lv[l] = a.amg.levels[l];
  __syncthreads();
  unsigned char* sb = s_dyn;
  float* buf = reinterpret_cast<float*>(s_dyn + a.tl.bytes);
  if (blockIdx.x == 0) tail_load(s_lv, nlev, a.tl, a.amg.coarse_inv, sb);
  const Rows own = own_rows(a.n, nb);
  const int stride = kPartStride;
  double* mypart = a.part + (long)blockIdx.x * stride;
  const float alc = a.amg.alpha;
  float* r32 = s_lv[0].r;

  // initial residual r = b - A x (or b); the V-cycle input is its FP32 copy
  for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
    const double br = a.b[r];
    double t;
    if (a.guess_zero) {
      a.x[r] = 0.0;
      t = br;
    } else {
      const double* vv_ = a.x;
      double s = row_gather<5>(a.rowptr, a.col, a.val, r, [&](int c) { return ldcg(vv_ + c); });
      t = br - s;
    }
    a.r[r] = t;
    r32[r] = (float)br;
  }
  if (!grid_barrier(a.bar, nb, a.err)) return;
  if (!a.guess_zero) {  // |M b| is the reference norm of a nonzero initial guess
    if (!vcycle(s_lv, nlev, a.tl, alc, sb, buf, a.u, a.bar, nb, a.err)) return;
    double acc[1] = {0.0};
    for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
      const double zb = ldcg(a.u + r);
      acc[0] += zb * zb;
      r32[r] = (float)ldcg(a.r + r);
    }
    block_reduce<1>(acc, s_warp, s_red);
    if (tid == 0) mypart[kMaxRestart + 3] = s_red[0];
    if (!grid_barrier(a.bar, nb, a.err)) return;
  }
  if (!vcycle(s_lv, nlev, a.tl, alc, sb, buf, a.u, a.bar, nb, a.err)) return;

  double rnorm0 = 0.0, ttol = 0.0, dp = 0.0;
  double gam_old = 0.0, dpi_old = 0.0;
  int reason = 0, its = 0;
  auto test = [&](double rn) -> int {
    if (isnan(rn) || isinf(rn)) return -9;
    if (rn <= ttol) return rn < a.abstol ? 3 : 2;
    if (rn >= a.dtol * rnorm0) return -4;
    return 0;
  };
  for (int i = 0;; i++) {
    // w = A u and the inner products (r,u), (w,u), (u,u), (u, s_old) of u = M r
    {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      const double* uu = a.u;
      for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
        const double s = row_gather<5>(a.rowptr, a.col, a.val, r, [&](int c) { return ldcg(uu + c); });
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
    if (!grid_barrier(a.bar, nb, a.err)) return;
    if (tid < 160) {
      const int q = tid >> 5;
      if (q < 4 || (i == 0 && !a.guess_zero)) {
        double s = warp_sum_blocks(a.part, stride, q < 4 ? q : kMaxRestart + 3, nb);
        if ((tid & 31) == 0) s_g[q] = s;
      }
    }
    __syncthreads();
    const double gam = s_g[0], del = s_g[1], mu = s_g[3];
    dp = sqrt(s_g[2]);
    if (i == 0) {
      rnorm0 = a.guess_zero ? dp : (s_g[4] != 0.0 ? sqrt(s_g[4]) : dp);
      ttol = fmax(a.rtol * rnorm0, a.abstol);
    }
    reason = test(dp);
    if (reason) {
      its = i;
      break;
    }
    if (i >= a.maxit) {
      reason = -3;
      its = i;
      break;
    }
    its = i + 1;
    if (gam == 0.0) {
      reason = 3;
      break;
    }
    if (i > 0 && gam * gam_old < 0.0) {
      reason = -8;
      break;
    }
    const double beta = i == 0 ? 0.0 : -mu / dpi_old;
    const double dpi = i == 0 ? del : del + beta * mu;  // (p, A p)
    if (dpi == 0.0 || (i > 0 && sgn(dpi) * sgn(dpi_old) < 0)) {
      reason = -10;
      break;
    }
    const double alpha = gam / dpi;
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
        if (h1) {
          const double pn1 = u1 + beta * p1, sn1 = w1 + beta * s1, rn1 = q1 - alpha * sn1;
          P[r1] = pn1;
          S[r1] = sn1;
          X[r1] = x1 + alpha * pn1;
          R[r1] = rn1;
          r32[r1] = (float)rn1;
        }
      }
    }
    gam_old = gam;
    dpi_old = dpi;
    if (!grid_barrier(a.bar, nb, a.err)) return;
    if (!vcycle(s_lv, nlev, a.tl, alc, sb, buf, a.u, a.bar, nb, a.err)) return;
  }
  if (blockIdx.x == 0 && tid == 0) {
    a.out->its = its;
    a.out->reason = reason;
    a.out->rnorm = dp;
  }
}

constexpr int align16(long b) { return (int)((b + 15) / 16 * 16); }

// tail = the shortest suffix of levels ending at the coarsest whose arrays fit kTailBudget
TailLayout tail_layout(const AmgHostView& h) {
  TailLayout T{};
  const int L = h.nlev;
  auto level_bytes = [&](int l) -> long {
    const AmgDevLevel& F = h.lv[l];
    if (l == L - 1) return align16(4L * F.n * F.n) + 2L * align16(4L * F.n);
    const int nc = h.lv[l + 1].n;
    return align16(4L * (F.n + 1)) + align16(4L * F.nnz) + align16(4L * F.nnz) + align16(4L * F.n) +
           align16(4L * F.n) + align16(4L * (nc + 1)) + align16(4L * F.n) + 3L * align16(4L * F.n);
  };
  long total = level_bytes(L - 1);
  int t = L - 1;
  while (t > 0 && total + level_bytes(t - 1) <= kTailBudget) total += level_bytes(--t);
  T.tail = t;
  int off = 0;
  auto take = [&](long b) {
    int o = off;
    off += align16(b);
    return o;
  };
  for (int l = 0; l < kAmgMaxLevels; l++) T.lv[l] = TailLevelOff{-1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
  for (int l = t; l < L; l++) {
    const AmgDevLevel& F = h.lv[l];
    TailLevelOff& o = T.lv[l];
    if (l + 1 < L) {
      o.rowptr = take(4L * (F.n + 1));
      o.col = take(4L * F.nnz);
      o.val = take(4L * F.nnz);
      o.wdinv = take(4L * F.n);
      o.agg = take(4L * F.n);
      o.ptptr = take(4L * (h.lv[l + 1].n + 1));
      o.ptrow = take(4L * F.n);
      o.T = take(4L * F.n);
    } else {
      T.inv = take(4L * F.n * F.n);
    }
    o.R = take(4L * F.n);
    o.X = take(4L * F.n);
  }
  T.bytes = off;
  return T;
}

}  // namespace

void launch_amg_setup_values(const AmgHostView& h, cudaStream_t s) {
  // FP32 copy of the pressure matrix, Galerkin sums down the hierarchy, Jacobi weights, and
  // the dense inverse of the coarsest level
  const AmgDevLevel& F0 = h.lv[0];
  ++g_launch_count, k_amg_level0<<<(F0.nnz + kThreads - 1) / kThreads, kThreads, 0, s>>>(F0.nnz, F0.val64, F0.val);
  ++g_launch_count, k_amg_wdinv<<<(F0.n + kThreads - 1) / kThreads, kThreads, 0, s>>>(F0.n, h.omega, F0.diag, F0.val,
                                                                                     F0.wdinv);
  for (int l = 0; l + 1 < h.nlev; l++) {
    const AmgDevLevel& F = h.lv[l];
    const AmgDevLevel& C = h.lv[l + 1];
    ++g_launch_count, k_amg_galerkin<<<(C.nnz + kThreads - 1) / kThreads, kThreads, 0, s>>>(C.nnz, F.cptr, F.csrc,
                                                                                           F.val, C.val);
    ++g_launch_count, k_amg_wdinv<<<(C.n + kThreads - 1) / kThreads, kThreads, 0, s>>>(C.n, h.omega, C.diag, C.val,
                                                                                      C.wdinv);
  }
  const AmgDevLevel& K = h.lv[h.nlev - 1];
  ++g_launch_count, k_amg_coarse_inverse<<<1, 1024, 0, s>>>(K.n, K.rowptr, K.col, K.diag, K.val, h.coarse_inv);
}

cudaError_t launch_cg_amg(const GmresCall& c, const AmgHostView& h, KrylovWork& w, cudaStream_t s) {
  if (5L * w.ldv > w.v_len || (long)gmres_grid(c.n, w.nblocks) * kPartStride > w.part_len || w.ldv < c.n ||
      h.nlev < 1 || h.nlev > kAmgMaxLevels || h.lv[h.nlev - 1].n > kAmgCoarseMax || h.lv[0].n != c.n)
    return cudaErrorInvalidValue;
  for (int l = 0; l + 1 < h.nlev; l++)
    if (h.lv[l].maxagg > kDownBuf) return cudaErrorInvalidValue;
  CgAmgArgs a;
  a.n = c.n;
  a.maxit = c.maxit;
  a.guess_zero = c.guess_zero;
  a.nb = gmres_grid(c.n, w.nblocks);
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
  a.out = c.out;
  a.rtol = c.rtol;
  a.abstol = 1e-50;
  a.dtol = 1e4;
  a.amg.nlev = h.nlev;
  a.amg.omega = h.omega;
  a.amg.alpha = h.alpha;
  a.amg.coarse_inv = h.coarse_inv;
  a.amg.levels = h.d_levels;
  a.tl = tail_layout(h);
  const int smem = a.tl.bytes + kDownBuf * (int)sizeof(float);
  cudaError_t e = cudaFuncSetAttribute((const void*)k_cg_amg, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)k_cg_amg, dim3(a.nb), dim3(kGmThreads), args, smem, s);
}

}  // namespace cycas
