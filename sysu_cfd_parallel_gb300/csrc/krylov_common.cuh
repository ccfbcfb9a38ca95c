// Device helpers shared by the persistent Krylov kernels: bounded grid barrier and
// deterministic block / grid reductions.
#pragma once
#include <cuda_runtime.h>

#include "cycas_device.h"

namespace cycas {
namespace kry {

constexpr int kGmThreads = 1024;
constexpr int kGmWarps = kGmThreads / 32;
constexpr int kDotGroup = 8;
constexpr long long kSpinLimit = 4000000000LL;  // ~2 s of SM clock before a barrier gives up
constexpr int kPartStride = kMaxRestart + 4;



__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }

// cooperative launch (all CTAs co-resident) through the extensible launch API, which stream
// capture records into a CUDA graph
inline cudaError_t launch_cooperative(const void* fn, int grid, int block, void** args, size_t smem, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, fn, args);
}

// gpu-scope acquire load (PTX memory model): what the releasing CTAs wrote before the barrier
// word changed is visible after it
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// true when an earlier kernel or stage recorded an error: every CTA of a persistent Krylov
// kernel reads the same value at its start (nothing writes it during the launch but a barrier
// that gave up), so either all CTAs run or none does
__device__ __forceinline__ bool launch_failed(const int* err) { return *(const volatile int*)err != 0; }

// gpu-scope release increment of the barrier counter; returns the value before it
__device__ __forceinline__ unsigned atom_add_release_gpu(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.release.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// bounded grid barrier for a cooperative launch: a counting barrier on bar[0], zeroed before
// the launch.  Thread 0 of each CTA adds one with release semantics; the k-th barrier of the
// launch is complete when the counter reaches k * nb, which the value returned by the CTA's own
// increment gives (old / nb + 1) * nb, so no CTA keeps state between barriers.  Waiting is a
// poll with acquire loads.  A wait that outlasts kSpinLimit, or that sees another CTA give up,
// records bit 0 in *err and returns false (the kernel then returns).
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nb, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned old = atom_add_release_gpu(bar, 1u);
    const unsigned target = (old / nb + 1u) * nb;
    int ok = 1;
    if (old + 1u != target) {
      const long long t0 = clock64();
      unsigned spins = 0;
      while ((int)(ld_acquire_gpu(bar) - target) < 0) {
        if ((++spins & 63u) == 0 && (*(volatile int*)err & 1)) {  // another CTA gave up
          ok = 0;
          break;
        }
        if (clock64() - t0 > kSpinLimit) {
          atomicOr(err, 1);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    } else {
      __threadfence();  // the last arrival acquires every other CTA's writes
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// reduce K per-thread values over the block in a fixed order; result valid in s_out[0..K)
// after the call.
//
// A warp-wide FP64 addition occupies GB300's FP64 pipe for about 19 SM cycles, so the cost of
// a block reduction is its count of warp-wide additions.  One shuffle tree per quantity spends
// 5 per quantity in every warp; here the lane stage is a reduce-scatter butterfly: the K
// quantities (padded to P, a power of two) are halved at each of the first log2 P xor levels
// (a lane keeps one half and adds the partner's copy of it), so after P - 1 additions every
// lane carries one quantity, and two plain xor levels leave 8 / P distinct partial sums of it
// per warp -- P + 1 additions per lane in all.  The 8 partials per warp go to s_warp; warp k
// then sums quantity k's 32 * 8 / P partials (a chain of 8 / P per lane, then a tree).
template <int K>
__device__ __forceinline__ void block_reduce(double (&v)[K], double* s_warp /*[kGmWarps*kDotGroup]*/,
                                             double* s_out) {
  static_assert(K >= 1 && K <= kDotGroup, "block_reduce: at most kDotGroup quantities");
  constexpr int P = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : 8;
  constexpr int G = kDotGroup / P;                   // partials per quantity per warp
  constexpr int LOGP = P == 1 ? 0 : P == 2 ? 1 : P == 4 ? 2 : 3;
  constexpr int MP = 16 >> LOGP;                     // first plain xor level
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double a[P];
#pragma unroll
  for (int k = 0; k < P; k++) a[k] = k < K ? v[k] : 0.0;
  int q = 0;  // quantity held in a[0] once the scatter levels are done
#pragma unroll
  for (int h = P / 2, m = 16; h >= 1; h >>= 1, m >>= 1) {
    const bool up = (lane & m) != 0;
#pragma unroll
    for (int j = 0; j < h; j++) {
      const double send = up ? a[j] : a[j + h];
      const double keep = up ? a[j + h] : a[j];
      a[j] = keep + __shfl_xor_sync(0xffffffffu, send, m);
    }
    if (up) q += h;
  }
  a[0] += __shfl_xor_sync(0xffffffffu, a[0], MP);
  a[0] += __shfl_xor_sync(0xffffffffu, a[0], MP >> 1);
  if ((lane & (MP | (MP >> 1))) == 0 && q < K) s_warp[wid * kDotGroup + q * G + (lane & (G - 1))] = a[0];
  __syncthreads();
  if (wid < K) {
    const double* src = s_warp + lane * kDotGroup + wid * G;  // lane l takes warp l's partials
    double t = src[0];
#pragma unroll
    for (int g = 1; g < G; g++) t += src[g];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) s_out[wid] = t;
  }
  __syncthreads();
}

// sum part[b*stride + q] over b = 0..nb-1 in a fixed order; executed by one warp
__device__ __forceinline__ double warp_sum_blocks(const double* part, int stride, int q, int nb) {
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  for (int b0 = lane; b0 < nb; b0 += 32 * 8) {  // same order, up to eight loads in flight
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = b0 + 32 * k < nb ? ldcg(part + (long)(b0 + 32 * k) * stride + q) : 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (b0 + 32 * k < nb) s += v[k];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  return __shfl_sync(0xffffffffu, s, 0);
}

// sum over the CSR row r of val[k] * f(col[k]), accumulated in column order.  The loads of up
// to W entries are issued together (predicated), so a row costs three dependent memory round
// trips (row pointers, column/value, gathered operand) instead of one per entry.
template <int W = 8, class F>
__device__ __forceinline__ double row_gather(const int* __restrict__ rowptr, const int* __restrict__ col,
                                             const double* __restrict__ val, int r, F f) {
  const int k0 = __ldg(rowptr + r), k1 = __ldg(rowptr + r + 1);
  double s = 0.0;
  for (int b = k0; b < k1; b += W) {
    int c[W];
    double v[W], xv[W];
#pragma unroll
    for (int q = 0; q < W; q++) {
      const bool ok = b + q < k1;
      c[q] = ok ? __ldg(col + b + q) : 0;
      v[q] = ok ? __ldg(val + b + q) : 0.0;
    }
#pragma unroll
    for (int q = 0; q < W; q++) xv[q] = (b + q < k1) ? f(c[q]) : 0.0;
#pragma unroll
    for (int q = 0; q < W; q++)
      if (b + q < k1) s += v[q] * xv[q];
  }
  return s;
}

// w + sum_{q < cnt} coef[q] * V[q*ldv + r], terms applied in ascending q; the vector loads are
// issued 8 at a time.  Callers pass coefficients with their sign folded in, so each term is a
// single FP64 FMA.
__device__ __forceinline__ double vec_axpy(double w, const double* V, long ldv, int r, const double* coef, int cnt) {
  for (int q0 = 0; q0 < cnt; q0 += 8) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = (q0 + k < cnt) ? ldcg(V + (long)(q0 + k) * ldv + r) : 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (q0 + k < cnt) w = fma(coef[q0 + k], v[k], w);
  }
  return w;
}


}  // namespace kry
}  // namespace cycas
