// CG for the pressure correction and the residual reductions of the SIMPLE iteration;
// GMRES lives in gmres.cu.  Original GMRES notes kept for the shared design:
//
// The algorithm is the one the reference gets from PETSc KSP (MPIStructure.cpp:234-531 with
// KSPGMRES defaults): restart m, classical Gram-Schmidt without refinement, left
// preconditioning, Givens least squares, convergence when the preconditioned residual norm
// falls below max(rtol*rnorm0, abstol), rnorm0 = ||B b|| for a nonzero initial guess and
// the first preconditioned residual otherwise; divergence at dtol*rnorm0 or NaN, and
// DIVERGED_ITS at maxit (the reference turns any negative reason into ConvergeError).
//
// GB300 mapping: one CTA per SM, each owning a contiguous slice of rows; all vectors stay
// resident in HBM/L2.  An Arnoldi step is two grid-wide phases:
//   A: w = D^-1 (A v_j) for my rows, then block partial dots <w, v_i>, i <= j
//   B: every CTA reduces the partials in the same fixed order (identical h in every CTA),
//      w -= sum h_i v_i for my rows, block partial of ||w||^2
// after which every CTA reduces the norm identically and runs the (tiny) Givens update
// redundantly, so control flow needs no further synchronisation.  Krylov vectors are
// stored unnormalised with a per-vector scale folded into the coefficients.  Grid barriers
// are bounded: on timeout the kernel records an error and returns.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "cycas_device.h"
#include "krylov_common.cuh"

namespace cycas {

namespace {

using namespace kry;

// ------------------------------------------------------------------ CG
// PETSc KSPCG (Hestenes-Stiefel, left preconditioning, preconditioned-norm test) as one
// persistent kernel.  Per iteration three grid phases:
//   P1 (p complete):  w = A p for my rows, partial p'w
//   P2 (dpi known):   x += a p, r -= a w, z = D^-1 r, partials z'z and z'r
//   P3 (beta known):  convergence test, p = z + (beta/betaold) p for my rows
// It stops with DIVERGED_INDEFINITE_PC / _MAT only when beta or p'Ap changes sign, so the
// negative-definite pressure-correction system is accepted as the reference's PETSc call is.
struct CgArgs {
  int n, maxit, guess_zero, nb, chunk;
  const int* __restrict__ rowptr;
  const int* __restrict__ col;
  const double* __restrict__ val;
  const double* __restrict__ dinv;
  const double* __restrict__ b;
  double* x;
  double *r, *z, *p, *w;
  double* part;
  unsigned* bar;
  int* err;
  KspOut* out;
  double rtol, abstol, dtol;
};

__global__ void __launch_bounds__(kGmThreads, 1) k_cg(CgArgs a) {
  __shared__ double s_warp[kGmWarps * kDotGroup];
  __shared__ double s_red[kDotGroup];
  __shared__ double s_g[4];
  if (launch_failed(a.err)) return;
  const int nb = a.nb, tid = threadIdx.x;
  const int r0 = blockIdx.x * a.chunk;
  const int r1 = min(a.n, r0 + a.chunk);
  const int stride = kPartStride;
  double* mypart = a.part + (long)blockIdx.x * stride;
  // slots: 0/1 initial norms, 2 p'w, 3/4 z'z and z'r  (each written once per phase)
  {
    double acc[3] = {0.0, 0.0, 0.0};
    for (int r = r0 + tid; r < r1; r += kGmThreads) {
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
      double d = a.dinv ? a.dinv[r] : 1.0;
      double z = t * d;
      a.r[r] = t;
      a.z[r] = z;
      acc[0] += z * z;
      acc[1] += z * t;
      if (!a.guess_zero) {
        double zb = br * d;
        acc[2] += zb * zb;
      }
    }
    block_reduce<3>(acc, s_warp, s_red);
    if (tid < 3) mypart[kMaxRestart + 1 + tid] = s_red[tid];
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
  double rnorm0 = a.guess_zero ? dp : (s_g[2] != 0.0 ? sqrt(s_g[2]) : dp);
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
      // p = z (+ b p); my rows only, then every CTA needs all of p
      double bb = i == 0 ? 0.0 : beta / betaold;
      for (int r = r0 + tid; r < r1; r += kGmThreads) a.p[r] = i == 0 ? ldcg(a.z + r) : ldcg(a.z + r) + bb * ldcg(a.p + r);
      if (!grid_barrier(a.bar, nb, a.err)) return;
      // P1: w = A p, partial p'w
      {
        double acc[1] = {0.0};
        for (int r = r0 + tid; r < r1; r += kGmThreads) {
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
      double al = beta / dpi;
      // P2: x += a p, r -= a w, z = D^-1 r, partials
      {
        double acc[2] = {0.0, 0.0};
        for (int r = r0 + tid; r < r1; r += kGmThreads) {
          double pr = ldcg(a.p + r);
          a.x[r] += al * pr;
          double rr = ldcg(a.r + r) + (-al) * ldcg(a.w + r);
          a.r[r] = rr;
          double d = a.dinv ? a.dinv[r] : 1.0;
          double zz = rr * d;
          a.z[r] = zz;
          acc[0] += zz * zz;
          acc[1] += zz * rr;
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

// ------------------------------------------------------------------ residual reductions
constexpr int kRedThreads = 256;

// localRes[0..2] += sum |old - new| * vol (navier_velocity.cpp:48-52); block partials
__global__ void k_residual_uvw(int n, const double* __restrict__ vol, const double* __restrict__ old,
                               const double* __restrict__ U, const double* __restrict__ V,
                               const double* __restrict__ W, double* __restrict__ red) {
  __shared__ double sw[kRedThreads / 32][3];
  double r[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = vol[i];
    r[0] += fabs(old[i] - U[i]) * v;
    r[1] += fabs(old[(long)n + i] - V[i]) * v;
    r[2] += fabs(old[2 * (long)n + i] - W[i]) * v;
  }
  for (int k = 0; k < 3; k++) {
    double t = r[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5][k] = t;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int w = 0; w < kRedThreads / 32; w++) s += sw[w][threadIdx.x];
    red[(long)threadIdx.x * gridDim.x + blockIdx.x] = s;
  }
}

// sums `nparts` partials (stored contiguously) into localRes[slot] in a fixed order
__global__ void k_finalize(const double* __restrict__ red, int nparts, int nslots, int slot0, DevStatus* st) {
  __shared__ double sw[kRedThreads / 32];
  for (int q = 0; q < nslots; q++) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += red[(long)q * nparts + i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kRedThreads / 32; w++) t += sw[w];
      st->localRes[slot0 + q] += t;
    }
    __syncthreads();
  }
}

// per-case residual sums for batches: block b covers rows [blk_lo[b], blk_hi[b]) of one case
__global__ void k_residual_uvw_batch(const int* __restrict__ blk_lo, const int* __restrict__ blk_hi, int nblk,
                                     const double* __restrict__ vol, const double* __restrict__ old, long n,
                                     const double* __restrict__ U, const double* __restrict__ V,
                                     const double* __restrict__ W, double* __restrict__ red) {
  __shared__ double sw[kRedThreads / 32][3];
  double r[3] = {0.0, 0.0, 0.0};
  const int i = blk_lo[blockIdx.x] + threadIdx.x;
  if (i < blk_hi[blockIdx.x]) {
    double v = vol[i];
    r[0] = fabs(old[i] - U[i]) * v;
    r[1] = fabs(old[n + i] - V[i]) * v;
    r[2] = fabs(old[2 * n + i] - W[i]) * v;
  }
  for (int k = 0; k < 3; k++) {
    double t = r[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5][k] = t;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int w = 0; w < kRedThreads / 32; w++) s += sw[w][threadIdx.x];
    red[(long)threadIdx.x * nblk + blockIdx.x] = s;
  }
}

// case c (block c) adds the partials of its blocks [case_blk0[c], case_blk0[c+1]) to res[c][slot]
__global__ void k_finalize_cases(const double* __restrict__ red, int nblk, const int* __restrict__ case_blk0,
                                 int nslots, int slot0, double* __restrict__ res) {
  __shared__ double sw[kRedThreads / 32];
  const int b0 = case_blk0[blockIdx.x], b1 = case_blk0[blockIdx.x + 1];
  for (int q = 0; q < nslots; q++) {
    double s = 0.0;
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) s += red[(long)q * nblk + i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kRedThreads / 32; w++) t += sw[w];
      res[(long)blockIdx.x * 10 + slot0 + q] += t;
    }
    __syncthreads();
  }
}

__global__ void k_to_float(long n, const double* __restrict__ src, float* __restrict__ dst) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

}  // namespace

void launch_to_float(const double* src, float* dst, long n, cudaStream_t s) {
  if (n > 0) ++g_launch_count, k_to_float<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, src, dst);
}

int residual_blocks(int n) {
  int b = (n + kRedThreads - 1) / kRedThreads;
  return b < 1 ? 1 : b;
}

void launch_residual_uvw(const DevMesh& m, const DevFields& f, double* red, DevStatus* st, cudaStream_t s,
                         const DevBatch* b) {
  if (b) {
    ++g_launch_count, k_residual_uvw_batch<<<b->nblk, kRedThreads, 0, s>>>(b->blk_lo, b->blk_hi, b->nblk, m.c_vol,
                                                                            f.old, m.ncel, f.U, f.V, f.W, red);
    ++g_launch_count, k_finalize_cases<<<b->ncases, kRedThreads, 0, s>>>(red, b->nblk, b->case_blk0, 3, 0, b->res);
    return;
  }
  int nb = residual_blocks(m.ncel);
  if (nb > 1024) nb = 1024;
  ++g_launch_count, k_residual_uvw<<<nb, kRedThreads, 0, s>>>(m.ncel, m.c_vol, f.old, f.U, f.V, f.W, red);
  ++g_launch_count, k_finalize<<<1, kRedThreads, 0, s>>>(red, nb, 3, 0, st);
}

void launch_finalize_residual(const double* red, int nparts, int slot, DevStatus* st, cudaStream_t s,
                              const DevBatch* b) {
  if (b) {
    ++g_launch_count, k_finalize_cases<<<b->ncases, kRedThreads, 0, s>>>(red, b->nblk, b->case_blk0, 1, slot, b->res);
    return;
  }
  ++g_launch_count, k_finalize<<<1, kRedThreads, 0, s>>>(red, nparts, 1, slot, st);
}

int gmres_grid(int n, int device_blocks) {
  // at least ~256 rows per CTA so barriers stay cheap on small systems
  int want = (n + 255) / 256;
  if (want < 1) want = 1;
  return want < device_blocks ? want : device_blocks;
}

cudaError_t launch_gmres(const GmresCall& c, KrylovWork& w, cudaStream_t s) {
  return launch_gmres_multi(&c, 1, w, s);
}

cudaError_t launch_cg(const GmresCall& c, KrylovWork& w, cudaStream_t s) {
  if (4L * w.ldv > w.v_len || (long)gmres_grid(c.n, w.nblocks) * kPartStride > w.part_len || w.ldv < c.n)
    return cudaErrorInvalidValue;
  CgArgs a;
  a.n = c.n;
  a.maxit = c.maxit;
  a.guess_zero = c.guess_zero;
  a.nb = gmres_grid(c.n, w.nblocks);
  a.chunk = (c.n + a.nb - 1) / a.nb;
  a.rowptr = c.rowptr;
  a.col = c.col;
  a.val = c.val;
  a.dinv = c.dinv;
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
  void* args[] = {&a};
  return launch_cooperative((const void*)k_cg, a.nb, kGmThreads, args, 0, s);
}

int gmres_max_blocks(int device) {
  int nsm = 0, per = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cg, kGmThreads, 0);
  if (per < 1) per = 1;
  return nsm * per;
}

}  // namespace cycas
