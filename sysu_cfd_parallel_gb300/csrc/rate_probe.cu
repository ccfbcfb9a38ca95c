// Bench-only measurement probe (built as libcycas_rate_probe.so, not part of libcycasgpu.so):
// the FP64 and FP32 FMA throughput of the current device.
//
// The SIMPLE path's FP64 loops are bounded by the FP64 issue rate on GB300 (a small fraction of
// the FP32 rate), so the bench reports their arithmetic against this measured peak beside the
// HBM roofline.  One CTA of 1024 threads per SM, eight independent FMA chains per thread.
#include <cuda_runtime.h>

#include "../../include/cycasgpu.h"

namespace {

template <class T>
__global__ void __launch_bounds__(1024, 1) k_fma_rate(int iters, T a, T b, T* sink) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == (T)12345.678) sink[0] = s;  // keeps the chains live; never true for these inputs
}

template <class T>
double rate(int sms, int iters, T* sink) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_rate<T><<<sms, 1024>>>(iters / 4, (T)0.999999, (T)1e-7, sink);
  cudaEventRecord(e0);
  k_fma_rate<T><<<sms, 1024>>>(iters, (T)0.999999, (T)1e-7, sink);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 2.0 * 8 * (double)iters * sms * 1024 / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int cycas_measure_fp_rates(double* fp64_tflops, double* fp32_tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return CYCAS_ERR_CUDA;
  double* sink = nullptr;
  if (cudaMalloc(&sink, 64) != cudaSuccess) return CYCAS_ERR_ALLOC;
  const double r64 = rate<double>(sms, 2048, sink);
  const double r32 = rate<float>(sms, 65536, (float*)sink);
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(sink);
  if (e != cudaSuccess) return CYCAS_ERR_CUDA;
  if (fp64_tflops) *fp64_tflops = r64;
  if (fp32_tflops) *fp32_tflops = r32;
  return CYCAS_OK;
}
