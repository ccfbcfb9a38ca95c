// cycas_csr_solve_noalloc: the standalone GMRES solve without any device allocation.
//
// Some callers cannot call cudaMalloc: their device memory is already reserved by another
// allocator (a framework that pre-reserves HBM for its own pool), or they must not add the
// device-wide synchronisation that cudaMalloc/cudaFree imply in the middle of a stream of
// work.  For them this entry point takes the matrix, right-hand side and solution as device
// pointers the caller owns and takes every scratch buffer -- Krylov basis, Jacobi inverse,
// per-CTA partial sums, grid-barrier counters and the status block -- from one file-scope
// static device array of fixed size (kScratchBytes = 8,987,136 bytes, about 8.6 MiB), which
// every GPU that loads the library holds until the process exits.
//
// Limits: n <= kMaxRows (32768) rows, restart <= kMaxRestart (32).  Larger systems are
// rejected with CYCAS_ERR_INVALID.  The device CSR must be well formed (rowptr ascending from
// 0, columns in [0, n)): it is the caller's device memory and is not checked here.  All calls share the one array: calls whose work overlaps on the GPU
// (different streams or host threads at the same time) race on it and must be serialised by
// the caller.  The barrier counters and the status block are cleared at the start of every
// call; the basis and partial sums are fully rewritten before they are read.
//
// The first call on a device looks up the array's device address (cudaGetSymbolAddress)
// with that device current and caches it; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/cycasgpu.h"
#include "cycas_device.h"

namespace cycas {

extern thread_local std::string g_last_error;

namespace {

constexpr int kMaxRows = 32768;
constexpr long kLdv = kMaxRows;  // multiple of 32
constexpr int kMaxBlocks = 256;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kBasisBytes = align_up(sizeof(double) * (size_t)(kMaxRestart + 1) * kLdv);
constexpr size_t kDinvBytes = align_up(sizeof(double) * (size_t)kMaxRows);
constexpr size_t kPartBytes = align_up(sizeof(double) * (size_t)kMaxBlocks * kGmresPartStride);
constexpr size_t kStatusBytes = align_up(sizeof(DevStatus));
constexpr size_t kBarBytes = align_up(2 * sizeof(unsigned));
constexpr size_t kScratchBytes = kBasisBytes + kDinvBytes + kPartBytes + kStatusBytes + kBarBytes;
static_assert(kScratchBytes == 8987136, "scratch size differs from the documented limit");

// the scratch of every call on this device; host code uses it only through its device address
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

// Jacobi inverse from the caller's device CSR: 1/a_ii (a missing diagonal gives 1/0, as the
// host-array entry point computes it)
__global__ void k_noalloc_dinv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                               const double* __restrict__ val, double* __restrict__ dinv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int k = rowptr[i]; k < rowptr[i + 1]; k++)
    if (col[k] == i) d = val[k];
  dinv[i] = 1.0 / d;
}

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

}  // namespace

}  // namespace cycas

using namespace cycas;

extern "C" int cycas_csr_solve_noalloc(int32_t n, const int32_t* d_rowptr, const int32_t* d_col,
                                       const double* d_val, const double* d_b, double* d_x,
                                       const cycas_ksp_options* ksp, double rtol, int32_t maxit,
                                       int32_t guess_zero, void* stream, cycas_solve_stats* stats) {
  if (!d_rowptr || !d_col || !d_val || !d_b || !d_x || !ksp) return fail(CYCAS_ERR_INVALID, "null argument");
  if (n < 1) return fail(CYCAS_ERR_INVALID, "n must be positive");
  if (n > kMaxRows)
    return fail(CYCAS_ERR_INVALID, "n = " + std::to_string(n) + " exceeds the no-allocation limit of " +
                                       std::to_string(kMaxRows) + " rows");
  if (ksp->restart < 1 || ksp->restart > kMaxRestart)
    return fail(CYCAS_ERR_INVALID, "restart must be in [1, " + std::to_string(kMaxRestart) + "]");
  if (ksp->pc != CYCAS_PC_NONE && ksp->pc != CYCAS_PC_JACOBI)
    return fail(CYCAS_ERR_INVALID, "the no-allocation solve supports the Jacobi preconditioner or none");
  if (ksp->type != CYCAS_KSP_DEFAULT && ksp->type != CYCAS_KSP_GMRES)
    return fail(CYCAS_ERR_INVALID, "the no-allocation solve is GMRES");
  if (maxit < 1) return fail(CYCAS_ERR_INVALID, "maxit must be positive");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(CYCAS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(CYCAS_ERR_INVALID, "device ordinal out of range");
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return fail(CYCAS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_addr[dev] = (unsigned char*)p;
    }
    base = g_addr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* V = (double*)base;
  double* dinv = (double*)(base + kBasisBytes);
  double* part = (double*)(base + kBasisBytes + kDinvBytes);
  DevStatus* st = (DevStatus*)(base + kBasisBytes + kDinvBytes + kPartBytes);
  unsigned* bar = (unsigned*)(base + kBasisBytes + kDinvBytes + kPartBytes + kStatusBytes);

  KrylovWork w;
  w.V = V;
  w.ldv = kLdv;
  w.v_len = (long)(kMaxRestart + 1) * kLdv;
  w.part = part;
  w.part_len = (long)kMaxBlocks * kGmresPartStride;
  w.bar = bar;
  w.nblocks = gmres_max_blocks(dev);
  if (w.nblocks > kMaxBlocks) w.nblocks = kMaxBlocks;
  w.m = ksp->restart;

  e = cudaMemsetAsync(st, 0, sizeof(DevStatus), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return fail(CYCAS_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  if (ksp->pc == CYCAS_PC_JACOBI) {
    ++g_launch_count, k_noalloc_dinv<<<(n + 255) / 256, 256, 0, s>>>(n, d_rowptr, d_col, d_val, dinv);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CYCAS_ERR_CUDA, std::string("Jacobi setup: ") + cudaGetErrorString(e));
  }
  GmresCall g;
  g.n = n;
  g.rowptr = d_rowptr;
  g.col = d_col;
  g.val = d_val;
  g.dinv = ksp->pc == CYCAS_PC_JACOBI ? dinv : nullptr;
  g.b = d_b;
  g.x = d_x;
  g.guess_zero = guess_zero ? 1 : 0;
  g.rtol = rtol;
  g.maxit = maxit;
  g.restart = ksp->restart;
  g.out = &st->ksp[0];
  g.err = &st->err;
  e = launch_gmres_multi(&g, 1, w, s);
  if (e != cudaSuccess) return fail(CYCAS_ERR_CUDA, std::string("GMRES launch: ") + cudaGetErrorString(e));
  DevStatus hs;
  e = cudaMemcpyAsync(&hs, st, sizeof hs, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(CYCAS_ERR_CUDA, std::string("GMRES solve: ") + cudaGetErrorString(e));
  if (stats) {
    stats->its = hs.ksp[0].its;
    stats->reason = hs.ksp[0].reason;
    stats->rnorm = hs.ksp[0].rnorm;
  }
  if (hs.err & 1) return fail(CYCAS_ERR_TIMEOUT, "a device-side grid barrier timed out");
  if (hs.ksp[0].reason == CYCAS_KSP_DIVERGED_NANORINF) return fail(CYCAS_NAN_DETECTED, "NaN or Inf residual norm");
  if (hs.ksp[0].reason < 0) return fail(CYCAS_NOT_CONVERGED, "GMRES did not converge");
  return CYCAS_OK;
}
