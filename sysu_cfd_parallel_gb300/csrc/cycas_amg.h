// Aggregation multigrid for the pressure-correction system: host hierarchy and device levels.
//
// Several independent cases (the members of a batch, or the single case of a context) each
// get their own hierarchy.  On the device, level l of every case that has one is stored in
// one concatenated array per level depth (so the per-solve setup is one launch per depth),
// and every case carries a descriptor with pointers to its slices.  Level 0 is the pressure
// system itself, in the system's global row numbering; coarser levels are numbered locally
// within their case.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <vector>

namespace cycas {

constexpr int kAmgMaxLevels = 12;
constexpr int kAmgCoarseMax = 64;            // the coarsest level is inverted densely by one CTA
constexpr int kAmgDownBuf = 8192;            // floats of the per-CTA restriction buffer
// shared-memory bytes for a case's tail levels: with the restriction buffer and the kernel's
// static shared memory this stays within the 227 KB a CTA can have
constexpr int kAmgTailBudget = 188 * 1024;
// Cases with at least this many pressure rows solve the tail's first level by two cycles (a
// W-cycle there).  The second cycle is a fixed cost per CG iteration (in shared memory, no grid
// barrier) that the saved iterations repay only on large cases: measured on GB300 per 10 SIMPLE
// iterations, 480k-tet channel -7.5 %, 104k -4 %, 60k +8 %, 4k-cell cavity +5 %.
constexpr int kAmgWRows = 80000;
// The second cycle runs on the first tail level (below level 0) with at most this many rows:
// every tail pass streams the level's matrix through one SM's shared memory, so a second cycle
// on a level of ~1000 rows costs more than the CG iterations it saves (48^3 cavity: 20 CG
// iterations of 67 us with the W-cycle on its 1244-row level against 23 of 58 us without).
constexpr int kAmgWLevelRows = 512;

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

// One level of one case, as the V-cycle sees it.
struct AmgDevLevel {
  int n, nnz;
  int maxagg;         // largest aggregate (rows per coarse row); 0 on the coarsest level
  int nnz_off;        // position of this case's first entry in the depth's concatenated values
  const int* rowptr;  // level 0: the system's row pointers (global positions); else local
  const int* col;     // level 0: global columns; else local
  const int* diag;    // global position of each row's diagonal in the depth's values
  float* val;         // FP32 values (level 0: all rows of the system, global positions)
  float* wdinv;       // w / a_ii (level 0: indexed by global row)
  const int* agg;     // row -> coarse row (level 0: indexed by global row)
  const int* ptptr;   // coarse row -> range in ptrow (local)
  const int* ptrow;   // rows of each aggregate (level 0: global rows)
  float* r;           // residual (level 0: FP32 copy of the CG residual, global rows)
  float* t;           // correction returned to the finer level (levels >= 1)
  // levels cycled by the grid (above the shared-memory tail): w D^-1 r of every row, the
  // smoothed residual r - A w D^-1 r kept from the way down for the way up, and the next level's
  // row of each entry's column (agg[col[k]]), so that each pass gathers one value per entry
  float* wr;
  float* sr;
  const int* aggcol;  // level 0: by the system's entry positions
  // levels of the shared-memory tail (else null): the pattern in SELL-32 layout -- rows ordered
  // by length (longest first) and cut into slices of 32 positions, a slice column-major and
  // padded to its longest row, so the 32 lanes of a warp read entry k of 32 rows from
  // consecutive addresses (no bank conflicts) and the ordering keeps the padding small.  Padding
  // entries have the row's own column and take the value 0; the real entries keep the CSR
  // order, so a row sums in the same order as in CSR.
  const int* sell_ptr;             // [ceil(n/32)+1] first entry of each slice
  const unsigned short* sell_col;  // [sell_len] local columns
  const int* sell_src;             // [sell_len] the entry's position in this level's CSR values, -1 for padding
  const unsigned short* sell_row;  // [32 ceil(n/32)] the row at each position
  int sell_len;
};

// byte offsets of one tail level's arrays in dynamic shared memory: rowptr/col/val hold the
// SELL-32 slice offsets, 16-bit columns and values of the level's matrix
struct TailLevelOff {
  int rowptr, col, val, wdinv, agg, ptptr, ptrow, R, X, T, perm;  // perm: the row at each SELL position
};

// the coarsest levels of a case, cycled out of shared memory by every CTA that solves the case
struct TailLayout {
  int tail;   // first level of the tail (levels tail..nlev-1)
  int bytes;  // dynamic shared memory taken by the tail (multiple of 16)
  int inv;    // offset of the coarsest level's dense inverse
  TailLevelOff lv[kAmgMaxLevels];
};

struct AmgCaseDesc {
  int lo, hi;                 // rows of the case in the pressure system
  int nlev;
  const float* coarse_inv;    // dense inverse of the (regularised) coarsest level, row-major
  const AmgDevLevel* levels;  // device array [nlev]
  TailLayout tl;
  int gamma;                  // cycles at the first level of the shared-memory tail
};

// host-side record of the device hierarchies of all cases
struct AmgHostView {
  int ncases = 0;
  // Jacobi weight of the smoother, coarse-correction scale, and cycles at the first coarse
  // level of the shared-memory tail (0: by case size, kAmgWRows).  A scale above 2 puts an
  // eigenvalue 1 - alpha below -1 on the coarse space once the coarse solve is accurate (the
  // W-cycle makes it so), and the cycle stops being a definite preconditioner; 2 is the
  // largest safe value.
  float omega = 0.9f, alpha = 2.0f;
  int gamma = 0;
  std::vector<AmgCaseDesc> cases;                // host copies (level pointers are device arrays)
  std::vector<std::vector<AmgDevLevel>> levels;  // [case][level] host copies
  AmgCaseDesc* d_cases = nullptr;                // device [ncases]
  int smem_bytes = 0;                            // dynamic shared memory of the solver kernel
  // per-depth concatenated arrays, for the per-solve setup launches
  struct Depth {
    int nrows = 0, nnz = 0;
    const int* diag = nullptr;  // [nrows] global positions of the diagonals
    const int* diag_row = nullptr;  // [nnz] the row of a diagonal entry, -1 off the diagonal
    float* val = nullptr;       // [nnz]
    float* wdinv = nullptr;     // [nrows]
    const int* cptr = nullptr;  // depth+1 nnz -> range in csrc (null for the deepest depth)
    const int* csrc = nullptr;  // positions in this depth's values
    int nnz_next = 0;           // entries of depth+1
  };
  std::vector<Depth> dep;
  const double* val64 = nullptr;  // FP64 pressure matrix (depth 0 source)
  float* coarse_inv = nullptr;    // all cases' inverses
  std::vector<int> rows0, nnz0;   // level sizes of case 0, for reporting
};

// Device memory for the hierarchy (implemented by the owner of the device allocations).
struct AmgUploader {
  virtual const int* upload_int(const int* h, long n) = 0;
  virtual float* alloc_float(long n) = 0;
  virtual void* upload_bytes(const void* h, long bytes) = 0;
  virtual ~AmgUploader() = default;
};

// Builds and uploads the hierarchies of the cases [lo[c], hi[c]) of one pattern: rowptr/col
// (host, all rows, global columns) with strength weights per entry; the *_dev pointers are the
// same pattern on the device, diag_dev its diagonal positions and val64_dev the FP64 values.
// cache (optional, one entry per case): a non-null entry is that case's hierarchy, used as it
// is; null entries are built and stored.  With every entry given, rowptr/col/weight may be null.
void amg_setup_cases(AmgHostView& v, int n, const int* rowptr, const int* col, const double* weight,
                     const int* rowptr_dev, const int* col_dev, const int* diag_dev, const double* val64_dev,
                     const std::vector<int>& lo, const std::vector<int>& hi, AmgUploader& up,
                     std::vector<std::shared_ptr<const AmgHostHierarchy>>* cache = nullptr);

struct GmresCall;
struct KrylovWork;
struct BatchSchedule;
struct KspOut;
// FP32 values of every level (Galerkin sums down each hierarchy), Jacobi weights, and the
// dense inverse of every case's coarsest level
void launch_amg_setup_values(const AmgHostView& h, cudaStream_t s);
// CG preconditioned by one V-cycle (persistent cooperative kernel of `grid` CTAs); case 0 over
// the whole grid when sched is null, else the teams of sched solve their cases.  Case c
// reports to out[c].
cudaError_t launch_cg_amg(const GmresCall& c, const AmgHostView& h, KrylovWork& w, const BatchSchedule* sched,
                          int grid, KspOut* out, cudaStream_t s);

}  // namespace cycas
