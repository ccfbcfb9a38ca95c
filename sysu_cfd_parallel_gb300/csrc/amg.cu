// Aggregation-AMG preconditioned CG for the pressure-correction system.
//
// The reference solves the pressure correction with PETSc CG + ILU(0) at rtol 1e-6 and a
// 1000-iteration cap (navier_pressure.cpp:28, MPIStructure.cpp:449-531).  On the 480k-cell
// channel that takes ~390 ILU-CG iterations and Jacobi-CG does not converge within the
// cap; a level-scheduled ILU apply would cost ~70 grid barriers.  Here the same CG (PETSc's
// Hestenes-Stiefel form and preconditioned-norm test) runs with one V-cycle of plain
// aggregation multigrid as the preconditioner:
//   down:   x_l = w D_l^-1 r_l;  r_{l+1} = P^T (r_l - A_l x_l)     (one grid barrier per level)
//   bottom: x_L = (A_L - s 11^T)^-1 r_L, dense, by CTA 0            (the system is singular:
//           the rank-one shift removes the constant null space without moving the range)
//   up:     t_l = y + w D_l^-1 (r_l - A_l y),  y = x_l + a P t_{l+1} (one barrier per level)
// Pre- and post-smoothing are transposes of each other and P = R^T, so the cycle is a fixed
// symmetric operator and plain CG applies.  All sums are in fixed order (deterministic).
#include <cuda_runtime.h>

#include "cycas_amg.h"
#include "cycas_device.h"
#include "krylov_common.cuh"

namespace cycas {

namespace {

using namespace kry;

constexpr int kThreads = 256;

__global__ void k_amg_galerkin(int nnz_c, const int* __restrict__ cptr, const int* __restrict__ csrc,
                               const double* __restrict__ valf, double* __restrict__ valc) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nnz_c) return;
  double s = 0.0;
  for (int q = cptr[c]; q < cptr[c + 1]; q++) s += valf[csrc[q]];
  valc[c] = s;
}

__global__ void k_amg_dinv(int n, const int* __restrict__ diag, const double* __restrict__ val,
                           double* __restrict__ dinv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dinv[i] = 1.0 / val[diag[i]];
}

// dense inverse of A_L + s 11^T, s = mean(diag)/n, by in-place Gauss-Jordan in shared memory.
// A_L is singular with the constant null vector (row sums vanish); the shift has the sign of
// the diagonal, so the shifted matrix is definite.  Pivoting is not needed for a definite matrix.
__global__ void k_amg_coarse_inverse(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                     const int* __restrict__ diag, const double* __restrict__ val,
                                     double* __restrict__ inv) {
  __shared__ double M[kAmgCoarseMax * kAmgCoarseMax];
  __shared__ double colk[kAmgCoarseMax];
  __shared__ double s_shift;
  const int tid = threadIdx.x;
  for (int e = tid; e < n * n; e += blockDim.x) M[e] = 0.0;
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x)
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) M[i * n + col[k]] = val[k];
  if (tid == 0) {
    double d = 0.0;
    for (int i = 0; i < n; i++) d += val[diag[i]];
    s_shift = d / ((double)n * (double)n);
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) M[e] += s_shift;
  __syncthreads();
  for (int k = 0; k < n; k++) {
    double piv = M[k * n + k];
    for (int i = tid; i < n; i += blockDim.x) colk[i] = M[i * n + k];
    __syncthreads();
    for (int j = tid; j < n; j += blockDim.x) M[k * n + j] = (j == k ? 1.0 : M[k * n + j]) / piv;
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) {
      int i = e / n, j = e % n;
      if (i == k) continue;
      M[e] = (j == k ? 0.0 : M[e]) - colk[i] * M[k * n + j];
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += blockDim.x) inv[e] = M[e];
}

struct CgAmgArgs {
  int n, maxit, guess_zero, nb;
  const int* __restrict__ rowptr;
  const int* __restrict__ col;
  const double* __restrict__ val;
  const double* __restrict__ b;
  double* x;
  double *r, *z, *p, *w;
  double* part;
  unsigned* bar;
  int* err;
  KspOut* out;
  double rtol, abstol, dtol;
  AmgDev amg;
};

struct Rows {
  int r0, r1;
};
__device__ __forceinline__ Rows own_rows(int n, int nb) {
  int ch = (n + nb - 1) / nb;
  int r0 = blockIdx.x * ch;
  return {min(r0, n), min(n, r0 + ch)};
}

// Levels with at most this many rows are cycled by CTA 0 alone with block-level
// synchronisation instead of grid barriers.
constexpr int kTailRows = 2048;

// pre-smoothing from zero (x = w D^-1 r) and its residual r - A x on rows [rw.r0, rw.r1);
// the residual goes to F.t, which is free until the up pass
__device__ __forceinline__ void down_smooth(const AmgDevLevel& F, const double* rl, double omega, Rows rw) {
  const double* dinv = F.dinv;
  for (int i = rw.r0 + threadIdx.x; i < rw.r1; i += kGmThreads) {
    double ri = ldcg(rl + i);
    F.x[i] = omega * dinv[i] * ri;
    double acc = row_gather(F.rowptr, F.col, F.val, i, [&](int j) { return omega * __ldg(dinv + j) * ldcg(rl + j); });
    F.t[i] = ri - acc;
  }
}

// restriction r_C = P^T res_F on coarse rows [rw.r0, rw.r1)
__device__ __forceinline__ void restrict_rows(const AmgDevLevel& F, const AmgDevLevel& C, Rows rw) {
  for (int I = rw.r0 + threadIdx.x; I < rw.r1; I += kGmThreads) {
    const int q0 = __ldg(F.ptptr + I), q1 = __ldg(F.ptptr + I + 1);
    double s = 0.0;
    for (int b = q0; b < q1; b += 8) {
      int fi[8];
      double rv[8];
#pragma unroll
      for (int q = 0; q < 8; q++) fi[q] = b + q < q1 ? __ldg(F.ptrow + b + q) : 0;
#pragma unroll
      for (int q = 0; q < 8; q++) rv[q] = b + q < q1 ? ldcg(F.t + fi[q]) : 0.0;
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (b + q < q1) s += rv[q];
    }
    C.r[I] = s;
  }
}

// prolongation of the coarse correction and post-smoothing:
// out = y + w D^-1 (r - A y),  y = x + a P x_C
__device__ __forceinline__ void up_smooth(const AmgDevLevel& F, const double* xc, const double* rl, double* out,
                                          double omega, double alpha, Rows rw) {
  const double* xl = F.x;
  const int* agg = F.agg;
  for (int i = rw.r0 + threadIdx.x; i < rw.r1; i += kGmThreads) {
    double y = ldcg(xl + i) + alpha * ldcg(xc + __ldg(agg + i));
    double acc = row_gather(F.rowptr, F.col, F.val, i,
                            [&](int j) { return ldcg(xl + j) + alpha * ldcg(xc + __ldg(agg + j)); });
    out[i] = y + omega * F.dinv[i] * (ldcg(rl + i) - acc);
  }
}

// dense coarsest solve x = inv r, one warp per row (CTA 0 only)
__device__ __forceinline__ void coarse_solve(int n, const double* inv, const double* r, double* x) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = wid; i < n; i += kGmWarps) {
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s += inv[i * n + j] * ldcg(r + j);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) x[i] = s;
  }
}

// z = M r by one V-cycle; every CTA participates; returns false after a barrier timeout
__device__ bool vcycle(const AmgDevLevel* L, int nlev, double omega, double alpha, const double* coarse_inv,
                       const double* rin, double* zout, unsigned* bar, unsigned nb, int* err) {
  // levels [tail, nlev) are small enough for CTA 0 alone
  int tail = nlev - 1;
  while (tail > 0 && L[tail - 1].n <= kTailRows) tail--;
  for (int l = 0; l < tail; l++) {
    const AmgDevLevel& F = L[l];
    down_smooth(F, l == 0 ? rin : F.r, omega, own_rows(F.n, nb));
    if (!grid_barrier(bar, nb, err)) return false;
    restrict_rows(F, L[l + 1], own_rows(L[l + 1].n, nb));
    if (!grid_barrier(bar, nb, err)) return false;
  }
  if (blockIdx.x == 0) {
    for (int l = tail; l + 1 < nlev; l++) {
      const AmgDevLevel& F = L[l];
      down_smooth(F, l == 0 ? rin : F.r, omega, Rows{0, F.n});
      __syncthreads();
      restrict_rows(F, L[l + 1], Rows{0, L[l + 1].n});
      __syncthreads();
    }
    const AmgDevLevel& K = L[nlev - 1];
    coarse_solve(K.n, coarse_inv, nlev == 1 ? rin : K.r, nlev == 1 ? zout : K.t);
    __syncthreads();
    for (int l = nlev - 2; l >= tail; l--) {
      const AmgDevLevel& F = L[l];
      up_smooth(F, L[l + 1].t, l == 0 ? rin : F.r, l == 0 ? zout : F.t, omega, alpha, Rows{0, F.n});
      __syncthreads();
    }
  }
  if (!grid_barrier(bar, nb, err)) return false;
  for (int l = tail - 1; l >= 0; l--) {
    const AmgDevLevel& F = L[l];
    up_smooth(F, L[l + 1].t, l == 0 ? rin : F.r, l == 0 ? zout : F.t, omega, alpha, own_rows(F.n, nb));
    if (!grid_barrier(bar, nb, err)) return false;
  }
  return true;
}

__global__ void __launch_bounds__(kGmThreads, 1) k_cg_amg(CgAmgArgs a) {
  __shared__ double s_warp[kGmWarps * kDotGroup];
  __shared__ double s_red[kDotGroup];
  __shared__ double s_g[4];
  __shared__ AmgDevLevel s_lv[kAmgMaxLevels];
  const int nb = a.nb, tid = threadIdx.x;
  const int nlev = a.amg.nlev;
  for (int l = tid; l < nlev; l += kGmThreads) s_lv[l] = a.amg.levels[l];
  __syncthreads();
  Rows own = own_rows(a.n, nb);
  const int stride = kPartStride;
  double* mypart = a.part + (long)blockIdx.x * stride;
  const double om = a.amg.omega, al_c = a.amg.alpha;

  // initial residual r = b - A x (or b), then z = M r (and M b for a nonzero guess)
  for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
    double br = a.b[r];
    double t;
    if (a.guess_zero) {
      a.x[r] = 0.0;
      t = br;
    } else {
      const double* vv_ = a.x;
      double s = row_gather(a.rowptr, a.col, a.val, r, [&](int c) { return ldcg(vv_ + c); });
      t = br - s;
    }
    a.r[r] = t;
  }
  if (!grid_barrier(a.bar, nb, a.err)) return;
  double snorm2 = 0.0;
  if (!a.guess_zero) {
    if (!vcycle(s_lv, nlev, om, al_c, a.amg.coarse_inv, a.b, a.z, a.bar, nb, a.err)) return;
    double acc[1] = {0.0};
    for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
      double zb = ldcg(a.z + r);
      acc[0] += zb * zb;
    }
    block_reduce<1>(acc, s_warp, s_red);
    if (tid == 0) mypart[kMaxRestart + 3] = s_red[0];
  }
  if (!vcycle(s_lv, nlev, om, al_c, a.amg.coarse_inv, a.r, a.z, a.bar, nb, a.err)) return;
  {
    double acc[2] = {0.0, 0.0};
    for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
      double zz = ldcg(a.z + r);
      acc[0] += zz * zz;
      acc[1] += zz * ldcg(a.r + r);
    }
    block_reduce<2>(acc, s_warp, s_red);
    if (tid < 2) mypart[kMaxRestart + 1 + tid] = s_red[tid];
  }
  if (!grid_barrier(a.bar, nb, a.err)) return;
  if (tid < 96) {
    int q = tid >> 5;
    double s = warp_sum_blocks(a.part, stride, kMaxRestart + 1 + q, nb);
    if ((tid & 31) == 0) s_g[q] = s;
  }
  __syncthreads();
  double dp = sqrt(s_g[0]);
  double beta = s_g[1];
  if (!a.guess_zero) snorm2 = s_g[2];
  double rnorm0 = a.guess_zero ? dp : (snorm2 != 0.0 ? sqrt(snorm2) : dp);
  const double ttol = fmax(a.rtol * rnorm0, a.abstol);
  auto test = [&](double rn) -> int {
    if (isnan(rn) || isinf(rn)) return -9;
    if (rn <= ttol) return rn < a.abstol ? 3 : 2;
    if (rn >= a.dtol * rnorm0) return -4;
    return 0;
  };
  int reason = test(dp);
  int its = 0;
  double betaold = 0.0, dpi = 0.0, dpiold = 0.0;
  int i = 0;
  if (!reason) {
    do {
      its = i + 1;
      if (beta == 0.0) {
        reason = 3;
        break;
      }
      if (i > 0 && beta * betaold < 0.0) {
        reason = -8;
        break;
      }
      double bb = i == 0 ? 0.0 : beta / betaold;
      for (int r = own.r0 + tid; r < own.r1; r += kGmThreads)
        a.p[r] = i == 0 ? ldcg(a.z + r) : ldcg(a.z + r) + bb * ldcg(a.p + r);
      if (!grid_barrier(a.bar, nb, a.err)) return;
      {
        double acc[1] = {0.0};
        for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
          const double* vv_ = a.p;
          double s = row_gather(a.rowptr, a.col, a.val, r, [&](int c) { return ldcg(vv_ + c); });
          a.w[r] = s;
          acc[0] += ldcg(a.p + r) * s;
        }
        block_reduce<1>(acc, s_warp, s_red);
        if (tid == 0) mypart[0] = s_red[0];
      }
      if (!grid_barrier(a.bar, nb, a.err)) return;
      if (tid < 32) {
        double s = warp_sum_blocks(a.part, stride, 0, nb);
        if (tid == 0) s_g[3] = s;
      }
      __syncthreads();
      dpiold = dpi;
      dpi = s_g[3];
      betaold = beta;
      if (dpi == 0.0 || (i > 0 && ((dpi > 0) - (dpi < 0)) * ((dpiold > 0) - (dpiold < 0)) < 0)) {
        reason = -10;
        break;
      }
      double alpha = beta / dpi;
      for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
        a.x[r] += alpha * ldcg(a.p + r);
        a.r[r] = ldcg(a.r + r) + (-alpha) * ldcg(a.w + r);
      }
      if (!grid_barrier(a.bar, nb, a.err)) return;
      if (!vcycle(s_lv, nlev, om, al_c, a.amg.coarse_inv, a.r, a.z, a.bar, nb, a.err)) return;
      {
        double acc[2] = {0.0, 0.0};
        for (int r = own.r0 + tid; r < own.r1; r += kGmThreads) {
          double zz = ldcg(a.z + r);
          acc[0] += zz * zz;
          acc[1] += zz * ldcg(a.r + r);
        }
        block_reduce<2>(acc, s_warp, s_red);
        if (tid < 2) mypart[1 + tid] = s_red[tid];
      }
      if (!grid_barrier(a.bar, nb, a.err)) return;
      if (tid < 64) {
        int q = tid >> 5;
        double s = warp_sum_blocks(a.part, stride, 1 + q, nb);
        if ((tid & 31) == 0) s_g[q] = s;
      }
      __syncthreads();
      dp = sqrt(s_g[0]);
      reason = test(dp);
      if (reason) break;
      beta = s_g[1];
      i++;
    } while (i < a.maxit);
    if (i >= a.maxit && !reason) reason = -3;
  }
  if (blockIdx.x == 0 && tid == 0) {
    a.out->its = its;
    a.out->reason = reason;
    a.out->rnorm = dp;
  }
}

}  // namespace

void launch_amg_setup_values(const AmgHostView& h, cudaStream_t s) {
  // levels 1.. from their finer level, then every diagonal inverse beyond level 0
  for (int l = 0; l + 1 < h.nlev; l++) {
    const AmgDevLevel& F = h.lv[l];
    const AmgDevLevel& C = h.lv[l + 1];
    ++g_launch_count, k_amg_galerkin<<<(C.nnz + kThreads - 1) / kThreads, kThreads, 0, s>>>(C.nnz, F.cptr, F.csrc,
                                                                                           F.val, C.val);
    ++g_launch_count, k_amg_dinv<<<(C.n + kThreads - 1) / kThreads, kThreads, 0, s>>>(C.n, C.diag, C.val, C.dinv);
  }
  const AmgDevLevel& K = h.lv[h.nlev - 1];
  ++g_launch_count, k_amg_coarse_inverse<<<1, 1024, 0, s>>>(K.n, K.rowptr, K.col, K.diag, K.val, h.coarse_inv);
}

cudaError_t launch_cg_amg(const GmresCall& c, const AmgHostView& h, KrylovWork& w, cudaStream_t s) {
  if (4L * w.ldv > w.v_len || (long)gmres_grid(c.n, w.nblocks) * kPartStride > w.part_len || w.ldv < c.n ||
      h.nlev < 1 || h.nlev > kAmgMaxLevels)
    return cudaErrorInvalidValue;
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
  a.z = w.V + w.ldv;
  a.p = w.V + 2 * w.ldv;
  a.w = w.V + 3 * w.ldv;
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
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)k_cg_amg, dim3(a.nb), dim3(kGmThreads), args, 0, s);
}

}  // namespace cycas
