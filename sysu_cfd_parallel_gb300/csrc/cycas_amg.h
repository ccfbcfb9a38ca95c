// Aggregation multigrid for the pressure-correction system: host hierarchy and device levels.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace cycas {

constexpr int kAmgMaxLevels = 12;
constexpr int kAmgCoarseMax = 64;  // the coarsest level is inverted densely by one CTA

struct AmgHostLevel {
  int n = 0, nnz = 0;
  std::vector<int> rowptr, col, diag;
  std::vector<int> agg;           // row -> coarse row (all levels but the coarsest)
  std::vector<int> ptptr, ptrow;  // coarse row -> rows of this level
  std::vector<int> cptr, csrc;    // coarse nnz -> contributing nnz of this level
};

struct AmgHostHierarchy {
  std::vector<AmgHostLevel> lv;
};

AmgHostHierarchy amg_build(int n, const int* rowptr, const int* col, const double* weight, int maxsize,
                           int coarse_max, int max_levels);

struct AmgDevLevel {
  int n, nnz, chunk;
  const int* rowptr;
  const int* col;
  const int* diag;
  double* val;
  double* dinv;
  const int* agg;
  const int* ptptr;
  const int* ptrow;
  const int* cptr;
  const int* csrc;
  double* x;  // smoothed correction
  double* t;  // post-smoothed correction
  double* r;  // residual (level 0: the caller's vector)
};

// host-side record of the device hierarchy
struct AmgHostView {
  int nlev = 0;
  double omega = 2.0 / 3.0, alpha = 2.0;
  double* coarse_inv = nullptr;
  AmgDevLevel* d_levels = nullptr;
  AmgDevLevel lv[kAmgMaxLevels];
};

struct AmgDev {
  int nlev;
  double omega;   // Jacobi weight
  double alpha;   // coarse-correction scaling
  double* coarse_inv;  // dense inverse of the (regularised) coarsest matrix, row-major
  AmgDevLevel* levels;  // device array [nlev]
};

struct GmresCall;
struct KrylovWork;
// Galerkin values and diagonal inverses of levels 1.., dense inverse of the coarsest level
void launch_amg_setup_values(const AmgHostView& h, cudaStream_t s);
// PETSc-style CG preconditioned by one V-cycle (persistent cooperative kernel)
cudaError_t launch_cg_amg(const GmresCall& c, const AmgHostView& h, KrylovWork& w, cudaStream_t s);

}  // namespace cycas
