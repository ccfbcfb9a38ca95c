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

// One level of the device hierarchy.  The V-cycle runs in FP32 (it is only a preconditioner;
// the CG around it is FP64), so every level keeps FP32 values; level 0 also points at the
// FP64 pressure matrix the FP32 copy is made from.
struct AmgDevLevel {
  int n, nnz;
  int maxagg;  // largest aggregate (fine rows per coarse row); 0 on the coarsest level
  const int* rowptr;
  const int* col;
  const int* diag;     // position of the diagonal in each row
  const double* val64; // level 0 only: the FP64 system matrix
  float* val;          // FP32 matrix values (level 0: rounded copy; coarser: Galerkin sums)
  float* wdinv;        // w / a_ii
  const int* agg;
  const int* ptptr;
  const int* ptrow;
  const int* cptr;
  const int* csrc;
  float* r;  // residual on this level (level 0: FP32 copy of the CG residual)
  float* t;  // correction returned to the finer level
};

// host-side record of the device hierarchy
struct AmgHostView {
  int nlev = 0;
  float omega = 2.0f / 3.0f, alpha = 2.0f;
  float* coarse_inv = nullptr;
  AmgDevLevel* d_levels = nullptr;
  AmgDevLevel lv[kAmgMaxLevels];
};

struct AmgDev {
  int nlev;
  float omega;          // Jacobi weight
  float alpha;          // coarse-correction scaling
  float* coarse_inv;    // dense inverse of the (regularised) coarsest matrix, row-major
  AmgDevLevel* levels;  // device array [nlev]
};

struct GmresCall;
struct KrylovWork;
// Galerkin values and diagonal inverses of levels 1.., dense inverse of the coarsest level
void launch_amg_setup_values(const AmgHostView& h, cudaStream_t s);
// PETSc-style CG preconditioned by one V-cycle (persistent cooperative kernel)
cudaError_t launch_cg_amg(const GmresCall& c, const AmgHostView& h, KrylovWork& w, cudaStream_t s);

}  // namespace cycas
