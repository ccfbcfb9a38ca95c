// GMRES(m) for the SIMPLE systems as one persistent cooperative kernel per solve.
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

namespace cycas {

namespace {

constexpr int kGmThreads = 1024;
constexpr int kGmWarps = kGmThreads / 32;
constexpr int kDotGroup = 8;
constexpr long long kSpinLimit = 4000000000LL;  // ~2 s of SM clock before a barrier gives up
constexpr int kPartStride = kMaxRestart + 4;

struct GmArgs {
  int n, m, maxit, guess_zero, nb, chunk;
  const int* __restrict__ rowptr;
  const int* __restrict__ col;
  const double* __restrict__ val;
  const double* __restrict__ dinv;
  const double* __restrict__ b;
  double* x;
  double* V;
  long ldv;
  double* part;  // [nb][kPartStride]
  unsigned* bar;
  int* err;
  KspOut* out;
  double rtol, abstol, dtol, haptol;
};

__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }

// bounded grid barrier for a cooperative launch
__device__ bool grid_barrier(unsigned* bar, unsigned nb, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = bar + 1;
    unsigned g = *gen;
    __threadfence();
    unsigned arrived = atomicAdd(bar, 1u);
    int ok = 1;
    if (arrived == nb - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long t0 = clock64();
      while (*gen == g) {
        if (clock64() - t0 > kSpinLimit) {
          atomicOr(err, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (*(volatile int*)err) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// reduce K per-thread values over the block; result valid in s_out[0..K) after the call
template <int K>
__device__ void block_reduce(double (&v)[K], double* s_warp /*[kGmWarps*K]*/, double* s_out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double t = v[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) s_warp[wid * K + k] = t;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int w = 0; w < kGmWarps; w++) s += s_warp[w * K + threadIdx.x];
    s_out[threadIdx.x] = s;
  }
  __syncthreads();
}

// sum part[b*stride + q] over b = 0..nb-1 in a fixed order; executed by one warp
__device__ __forceinline__ double warp_sum_blocks(const double* part, int stride, int q, int nb) {
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  for (int b = lane; b < nb; b += 32) s += ldcg(part + (long)b * stride + q);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  return __shfl_sync(0xffffffffu, s, 0);
}

__global__ void __launch_bounds__(kGmThreads, 1) k_gmres(GmArgs a) {
  __shared__ double s_warp[kGmWarps * kDotGroup];
  __shared__ double s_red[kDotGroup];
  __shared__ double s_h[kMaxRestart + 1];     // current column, unrotated
  __shared__ double s_coef[kMaxRestart + 1];  // h_i * scale_i
  __shared__ double s_scale[kMaxRestart + 1];
  __shared__ double s_hh[(kMaxRestart + 1) * kMaxRestart];  // rotated Hessenberg, column-major
  __shared__ double s_cc[kMaxRestart], s_ss[kMaxRestart], s_grs[kMaxRestart + 1], s_nrs[kMaxRestart];
  __shared__ int s_ctl[4];      // [0] reason, [1] continue-arnoldi, [2] breakdown
  __shared__ double s_dbl[4];   // [0] rnorm0 [1] ttol [2] rnorm

  const int m = a.m, nb = a.nb, tid = threadIdx.x;
  const int r0 = blockIdx.x * a.chunk;
  const int r1 = min(a.n, r0 + a.chunk);
  // partial-sum slots per CTA: dots [0, kMaxRestart], norm kMaxRestart+1, initial residual
  // kMaxRestart+2 / +3.  Slots written in one phase are read only after the next barrier and
  // rewritten only after every CTA has passed a further barrier.
  const int stride = kPartStride;
  const int kNorm = kMaxRestart + 1, kInit = kMaxRestart + 2;
  double* mypart = a.part + (long)blockIdx.x * stride;

  int its = 0, reason = 0;
  bool first = true;
  double rnorm = 0.0;
  if (tid == 0) {
    s_dbl[0] = s_dbl[1] = s_dbl[2] = 0.0;
  }

  int itcount = 0;
  while (true) {
    // ---------------- initial preconditioned residual, stored unnormalised in V[0]
    double acc[2] = {0.0, 0.0};
    const bool zero_start = first && a.guess_zero;
    const bool need_bnorm = first && !a.guess_zero;
    for (int r = r0 + tid; r < r1; r += kGmThreads) {
      double br = a.b[r];
      double t;
      if (zero_start) {
        a.x[r] = 0.0;
        t = br;
      } else {
        double s = 0.0;
        for (int k = a.rowptr[r]; k < a.rowptr[r + 1]; k++) s += a.val[k] * ldcg(a.x + a.col[k]);
        t = br - s;
      }
      double d = a.dinv ? a.dinv[r] : 1.0;
      double z = t * d;
      a.V[r] = z;
      acc[0] += z * z;
      if (need_bnorm) {
        double zb = br * d;
        acc[1] += zb * zb;
      }
    }
    block_reduce<2>(acc, s_warp, s_red);
    if (tid < 2) mypart[kInit + tid] = s_red[tid];
    if (!grid_barrier(a.bar, nb, a.err)) return;
    if (tid < 64) {
      int q = tid >> 5;
      double s = warp_sum_blocks(a.part, stride, kInit + q, nb);
      if ((tid & 31) == 0) s_red[q] = s;
    }
    __syncthreads();
    double beta = sqrt(s_red[0]);
    if (tid == 0) {
      if (first) {
        if (a.guess_zero) s_dbl[0] = beta;
        else {
          double snorm = sqrt(s_red[1]);
          s_dbl[0] = snorm != 0.0 ? snorm : beta;
        }
      }
      s_grs[0] = beta;
      s_scale[0] = 1.0 / beta;
      int rs = 0;
      if (beta == 0.0) {
        rs = 3;  // KSP_CONVERGED_ATOL: exact initial residual
      } else {
        if (its == 0) s_dbl[1] = fmax(a.rtol * s_dbl[0], a.abstol);
        if (isnan(beta) || isinf(beta)) rs = -9;
        else if (beta <= s_dbl[1]) rs = beta < a.abstol ? 3 : 2;
        else if (beta >= a.dtol * s_dbl[0]) rs = -4;
      }
      s_ctl[0] = rs;
      s_dbl[2] = beta;
    }
    __syncthreads();
    reason = s_ctl[0];
    rnorm = s_dbl[2];
    first = false;
    if (beta == 0.0) break;

    // ---------------- Arnoldi
    int it = 0;
    while (!reason && it < m && its < a.maxit) {
      const double* vj = a.V + (long)it * a.ldv;
      double* w = a.V + (long)(it + 1) * a.ldv;
      const double sj = s_scale[it];
      // phase A1: w = D^-1 A v_j (v_j = V[j] * scale_j)
      for (int r = r0 + tid; r < r1; r += kGmThreads) {
        double s = 0.0;
        for (int k = a.rowptr[r]; k < a.rowptr[r + 1]; k++) s += a.val[k] * ldcg(vj + a.col[k]);
        double d = a.dinv ? a.dinv[r] : 1.0;
        w[r] = (s * sj) * d;
      }
      __syncthreads();
      // phase A2: partial dots <w, V[i]> in groups of kDotGroup
      for (int q0 = 0; q0 <= it; q0 += kDotGroup) {
        double d8[kDotGroup];
#pragma unroll
        for (int k = 0; k < kDotGroup; k++) d8[k] = 0.0;
        for (int r = r0 + tid; r < r1; r += kGmThreads) {
          double wr = ldcg(w + r);
#pragma unroll
          for (int k = 0; k < kDotGroup; k++)
            if (q0 + k <= it) d8[k] += wr * ldcg(a.V + (long)(q0 + k) * a.ldv + r);
        }
        block_reduce<kDotGroup>(d8, s_warp, s_red);
        if (tid < kDotGroup && q0 + tid <= it) mypart[q0 + tid] = s_red[tid];
      }
      if (!grid_barrier(a.bar, nb, a.err)) return;
      // phase B: identical reduction in every CTA, then w -= sum h_i v_i
      {
        const int wid = tid >> 5;
        for (int q = wid; q <= it; q += kGmWarps) {
          double s = warp_sum_blocks(a.part, stride, q, nb);
          if ((tid & 31) == 0) {
            double h = s * s_scale[q];
            s_h[q] = h;
            s_coef[q] = h * s_scale[q];
          }
        }
      }
      __syncthreads();
      double nrm[1] = {0.0};
      for (int r = r0 + tid; r < r1; r += kGmThreads) {
        double wr = ldcg(w + r);
        for (int q = 0; q <= it; q++) wr -= s_coef[q] * ldcg(a.V + (long)q * a.ldv + r);
        w[r] = wr;
        nrm[0] += wr * wr;
      }
      block_reduce<1>(nrm, s_warp, s_red);
      if (tid == 0) mypart[kNorm] = s_red[0];
      if (!grid_barrier(a.bar, nb, a.err)) return;
      if (tid < 32) {
        double s = warp_sum_blocks(a.part, stride, kNorm, nb);
        if (tid == 0) s_red[0] = s;
      }
      __syncthreads();
      // phase C: Hessenberg column, happy-breakdown test and Givens update (thread 0)
      if (tid == 0) {
        double tt = sqrt(s_red[0]);
        double* hh = s_hh + it * (m + 1);
        for (int q = 0; q <= it; q++) hh[q] = s_h[q];
        hh[it + 1] = tt;
        s_scale[it + 1] = 1.0 / tt;
        double hapbnd = fabs(tt / s_grs[it]);
        if (hapbnd > a.haptol) hapbnd = a.haptol;
        bool hapend = tt < hapbnd;
        for (int j = 1; j <= it; j++) {
          double t0 = hh[j - 1];
          hh[j - 1] = s_cc[j - 1] * t0 + s_ss[j - 1] * hh[j];
          hh[j] = s_cc[j - 1] * hh[j] - s_ss[j - 1] * t0;
        }
        double res;
        int rs = 0;
        if (!hapend) {
          double d = sqrt(hh[it] * hh[it] + hh[it + 1] * hh[it + 1]);
          if (d == 0.0) {
            rs = -5;
            res = s_dbl[2];
          } else {
            s_cc[it] = hh[it] / d;
            s_ss[it] = hh[it + 1] / d;
            s_grs[it + 1] = -(s_ss[it] * s_grs[it]);
            s_grs[it] = s_cc[it] * s_grs[it];
            hh[it] = s_cc[it] * hh[it] + s_ss[it] * hh[it + 1];
            res = fabs(s_grs[it + 1]);
          }
        } else {
          res = 0.0;
        }
        int brk = rs != 0;
        if (!brk) {
          if (isnan(res) || isinf(res)) rs = -9;
          else if (res <= s_dbl[1]) rs = res < a.abstol ? 3 : 2;
          else if (res >= a.dtol * s_dbl[0]) rs = -4;
          if (hapend && !rs) rs = -5;
          s_dbl[2] = res;
        }
        s_ctl[0] = rs;
        s_ctl[2] = brk;
      }
      __syncthreads();
      reason = s_ctl[0];
      rnorm = s_dbl[2];
      if (s_ctl[2]) break;  // zero rotation: no step taken
      it++;
      its++;
    }
    // ---------------- solution update x += sum y_k v_k (k < it)
    if (it > 0) {
      if (tid == 0) {
        int k = it - 1;
        const double* H = s_hh;
        auto HH = [&](int r, int c) { return H[c * (m + 1) + r]; };
        if (HH(k, k) == 0.0) {
          s_ctl[0] = -5;
          s_ctl[1] = 0;
        } else {
          s_nrs[k] = s_grs[k] / HH(k, k);
          for (int ii = 1; ii <= k; ii++) {
            int q = k - ii;
            double tt = s_grs[q];
            for (int j = q + 1; j <= k; j++) tt = tt - HH(q, j) * s_nrs[j];
            s_nrs[q] = tt / HH(q, q);
          }
          for (int j = 0; j <= k; j++) s_coef[j] = s_nrs[j] * s_scale[j];
          s_ctl[1] = 1;
        }
      }
      __syncthreads();
      if (s_ctl[1]) {
        for (int r = r0 + tid; r < r1; r += kGmThreads) {
          double t = 0.0;
          for (int j = 0; j < it; j++) t += s_coef[j] * ldcg(a.V + (long)j * a.ldv + r);
          a.x[r] += t;
        }
      }
      reason = s_ctl[0];
    }
    itcount += it;
    if (itcount >= a.maxit) {
      if (!reason) reason = -3;
      break;
    }
    if (reason) break;
    // next cycle reads x of other CTAs
    if (!grid_barrier(a.bar, nb, a.err)) return;
  }
  if (blockIdx.x == 0 && tid == 0) {
    a.out->its = its;
    a.out->reason = reason;
    a.out->rnorm = rnorm;
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

}  // namespace

int residual_blocks(int n) {
  int b = (n + kRedThreads - 1) / kRedThreads;
  return b < 1 ? 1 : b;
}

void launch_residual_uvw(const DevMesh& m, const DevFields& f, double* red, DevStatus* st, cudaStream_t s) {
  int nb = residual_blocks(m.ncel);
  if (nb > 1024) nb = 1024;
  k_residual_uvw<<<nb, kRedThreads, 0, s>>>(m.ncel, m.c_vol, f.old, f.U, f.V, f.W, red);
  k_finalize<<<1, kRedThreads, 0, s>>>(red, nb, 3, 0, st);
}

void launch_finalize_residual(const double* red, int nparts, int slot, DevStatus* st, cudaStream_t s) {
  k_finalize<<<1, kRedThreads, 0, s>>>(red, nparts, 1, slot, st);
}

int gmres_grid(int n, int device_blocks) {
  // at least ~256 rows per CTA so barriers stay cheap on small systems
  int want = (n + 255) / 256;
  if (want < 1) want = 1;
  return want < device_blocks ? want : device_blocks;
}

cudaError_t launch_gmres(const GmresCall& c, KrylovWork& w, cudaStream_t s) {
  GmArgs a;
  a.n = c.n;
  a.m = c.restart;
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
  a.V = w.V;
  a.ldv = w.ldv;
  a.part = w.part;
  a.bar = w.bar;
  a.err = c.err;
  a.out = c.out;
  a.rtol = c.rtol;
  a.abstol = 1e-50;
  a.dtol = 1e4;
  a.haptol = 1e-30;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)k_gmres, dim3(a.nb), dim3(kGmThreads), args, 0, s);
}

int gmres_max_blocks(int device) {
  int nsm = 0, per = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_gmres, kGmThreads, 0);
  if (per < 1) per = 1;
  return nsm * per;
}

}  // namespace cycas
