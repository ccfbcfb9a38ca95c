// Device-resident state of one case and the kernel entry points of libcycasgpu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace cycas {

constexpr int kMaxRestart = 32;  // largest GMRES restart length supported

// kernels launched by this library on the calling thread (measurement only)
extern thread_local long long g_launch_count;

// ---- mesh (structure of arrays; per-cell slot arrays are slot-major [6][ncel]) --------
struct DevMesh {
  int ncel = 0, nfac = 0, nbnd = 0, nnz = 0, nvrt = 0;
  // faces
  int* f_c1 = nullptr;
  int* f_c2 = nullptr;
  int* f_bnd = nullptr;
  int* f_vert = nullptr;   // [4*nfac]
  double* f_x = nullptr;   // [3*nfac]
  double* f_n = nullptr;   // [3*nfac]
  double* f_area = nullptr;
  double* f_lambda = nullptr;
  double* f_rlencos = nullptr;
  double* f_xpac = nullptr;  // [3*nfac]
  double* f_xnac = nullptr;  // [3*nfac]
  // cells
  int* c_nface = nullptr;
  int* c_face = nullptr;   // [6][ncel]  Cell[i].face[j] at j*ncel+i (assembly order)
  int* c_gface = nullptr;  // [6][ncel]  same faces sorted by face index (gradient order)
  int* c_slot = nullptr;   // [6][ncel]  CSR position of the off-diagonal of face slot j, -1 on boundary
  int* c_diag = nullptr;   // [ncel]     CSR position of the diagonal
  int* c_vert = nullptr;   // [8*ncel]
  double* c_vol = nullptr;
  double* c_x = nullptr;   // [3*ncel]
  double* vert = nullptr;  // [3*nvrt]
  // boundary
  int* b_face = nullptr;
  int* b_type = nullptr;
  double* b_dist = nullptr;
  // boundary index lists (reference loop order)
  int n_inlet = 0, n_outlet = 0, n_sym = 0, n_wallcell = 0;
  int* inlet_list = nullptr;
  int* outlet_list = nullptr;
  int* sym_list = nullptr;
  int* wc_cell = nullptr;   // cells that own at least one wall face
  int* wc_start = nullptr;  // [n_wallcell+1] into wc_bnd
  int* wc_bnd = nullptr;    // wall boundary indices of each wall cell, ascending
  // CSR pattern of every system (diagonal + face neighbours, columns ascending)
  int* rowptr = nullptr;
  int* col = nullptr;
};

struct DevFields {
  double *U, *V, *W, *P, *R, *T, *TE, *ED, *dp, *VisLam, *VisTur, *Apr, *RUFace;
  double *BRo, *BU, *BV, *BW, *BPre, *BTE, *BED, *BTem;
  double *dUdX, *dVdX, *dWdX, *dPdX, *dPhidX;  // [3*ncel]
  double* shear;                                // [3*nbnd] wall shear (Bnd[].shear)
  double* old;                                  // [3*ncel] U,V,W before the velocity solve
  double *Prod, *TES, *EDS, *ApTE, *ApED, *VisTE, *VisED;
  double *Au, *Ap, *As;                         // values on the shared pattern
  double *bu, *bv, *bw, *bp, *bs;
  double *dinv_u, *dinv_p, *dinv_s;             // Jacobi: reciprocal of the diagonal
  // transient runs: the previous time level (null when steady).  The reference's second-order
  // save assigns both previous levels from the current one, so one level serves both schemes.
  double *Rnp, *Unp, *Vnp, *Wnp, *Tnp, *TEp, *EDp;
  // energy equation (null when it is not solved)
  double *kcond, *ES, *ApE;
};

// time discretisation of a transient run (scheme 0: steady)
struct TimeConf {
  int scheme = 0;  // 1 Euler, 2 the reference's second-order ("Dual") form
  double dt = 1.0;
};

// perfect-gas constants of the reference (navier.cpp:486-493)
constexpr double kCp = 1006.;
constexpr double kGama = 1.4;
constexpr double kPrl = 0.72;
constexpr double kPrte = 0.9;
constexpr double kRcpcv = kCp - kCp / kGama;

// per-solve report written by the Krylov kernel
struct KspOut {
  int its;
  int reason;
  double rnorm;
};

// one status block per context, read back once per iteration
struct DevStatus {
  double localRes[10];
  KspOut ksp[8];
  int nsolve;
  int err;          // bit 0 barrier timeout, bit 1 mesh check failed, bit 2 reverse inlet flow (scalar)
  int warn_inlet;   // reverse-flow-at-inlet warnings (momentum)
  int pad;
};

struct KrylovWork {
  double* V = nullptr;       // Krylov / work vectors of length ldv
  long ldv = 0;
  long v_len = 0;            // doubles available at V
  long part_len = 0;         // doubles available at part
  double* part = nullptr;    // block partial sums
  unsigned* bar = nullptr;   // grid barrier [count, generation]
  double* red = nullptr;     // residual reduction partials
  int nblocks = 0;           // persistent grid size
  int threads = 0;
  int m = 0;
};

struct KspConf {
  int type;  // CYCAS_KSP_GMRES / CYCAS_KSP_CG
  int restart;
  int pc;
  double rtol;
  int maxit;
};

// ---------------------------------------------------------------- launches
// geometry (CellFaceInfo, NS/geometry.cpp:391-752)
void launch_geometry(const DevMesh& m, int* d_err, cudaStream_t s);

// boundary conditions, gradients, assembly, corrections (NS/navier_*.cpp)
// Case metadata of a batch context (several independent cases in one union mesh).
struct DevBatch {
  int ncases = 0;
  int nblk = 0;                  // case-aligned blocks of at most 256 rows
  const int* blk_lo = nullptr;   // [nblk] first row
  const int* blk_hi = nullptr;   // [nblk] one past the last row
  const int* blk_case = nullptr; // [nblk] case of the block
  const int* case_blk0 = nullptr;// [ncases + 1] blocks of each case
  const int* case_pref = nullptr;// [ncases] global pressure-reference cell
  const int* in0 = nullptr;      // [ncases + 1] inlet boundaries of each case in inlet_list
  const int* out0 = nullptr;     // [ncases + 1] outlet boundaries of each case in outlet_list
  double* res = nullptr;         // [ncases][10] residuals of the iteration
};

// b: the batch metadata of a batch context, nullptr for a single case
void launch_bc_velocity(const DevMesh& m, const DevFields& f, int density_model, bool set_pressure,
                        cudaStream_t s, const DevBatch* b = nullptr);
void launch_bc_deltap(const DevMesh& m, const DevFields& f, cudaStream_t s);
// fp32: the arithmetic in FP32 (mixed-precision contexts; storage stays FP64), else FP64 and
// bit-exact with the reference
void launch_gradient(const DevMesh& m, int nfield, const double* const* phi, const double* const* bphi,
                     double* const* grad, cudaStream_t s, bool fp32 = false);
void launch_momentum(const DevMesh& m, const DevFields& f, const double* urf, const double* gravity,
                     DevStatus* st, cudaStream_t s, const TimeConf& tc = TimeConf(), bool fp32 = false);
void launch_ruface2(const DevMesh& m, const DevFields& f, cudaStream_t s, bool fp32 = false);
void launch_pressure(const DevMesh& m, const DevFields& f, cudaStream_t s);
// compressible (perfect-gas) pressure-correction rows (navier_pressure.cpp:106-224, DensityModel 1)
void launch_pressure_gas(const DevMesh& m, const DevFields& f, const TimeConf& tc, cudaStream_t s);
void launch_correct_cells(const DevMesh& m, const DevFields& f, int cell_pref, double urf_p, double* red,
                          cudaStream_t s, const DevBatch* b = nullptr, int density_model = 0);
void launch_correct_ruface(const DevMesh& m, const DevFields& f, double urf_p, cudaStream_t s,
                           int density_model = 0);
// unsteady terms of a scalar equation: Ap += c (1.5 c), src += c * phi_old (c * (2 phi_old -
// 0.5 phi_old)) with c = R / dt * vol
void launch_scalar_time(const DevMesh& m, const DevFields& f, const TimeConf& tc, const double* phi_old,
                        double* ap, double* src, cudaStream_t s);
// UpdateEnergy sources (navier_scalar.cpp:209-281) and SetBCTemperature (navier_bc.cpp:183-213)
void launch_energy_sources(const DevMesh& m, const DevFields& f, int density_model, cudaStream_t s);
void launch_bc_temperature(const DevMesh& m, const DevFields& f, cudaStream_t s);
void launch_keps_sources(const DevMesh& m, const DevFields& f, cudaStream_t s);
void launch_keps_wall(const DevMesh& m, const DevFields& f, cudaStream_t s);
void launch_scalar(const DevMesh& m, const DevFields& f, const double* phi, const double* bphi,
                   const double* diff, const double* src, const double* app, double urf_s, DevStatus* st,
                   cudaStream_t s);
void launch_clip_te(const DevMesh& m, const DevFields& f, cudaStream_t s);
void launch_eps_wall_rows(const DevMesh& m, const DevFields& f, cudaStream_t s);
void launch_finish_keps(const DevMesh& m, const DevFields& f, cudaStream_t s);

// reductions (krylov.cu)
void launch_residual_uvw(const DevMesh& m, const DevFields& f, double* red, DevStatus* st, cudaStream_t s,
                         const DevBatch* b = nullptr);
void launch_finalize_residual(const double* red, int nparts, int slot, DevStatus* st, cudaStream_t s,
                              const DevBatch* b = nullptr);
int residual_blocks(int n);
void launch_to_float(const double* src, float* dst, long n, cudaStream_t s);

// Krylov
// Batched Krylov solves: the CTAs of one cooperative launch are split into teams; each team
// solves the row ranges of its cases one after another, synchronising only its own CTAs.
struct BatchSchedule {
  const int* cta_team;    // [grid] team of each CTA
  const int* cta_rank;    // [grid] rank of each CTA in its team
  const int* team_size;   // [nteams] CTAs per team
  const int* team_cta0;   // [nteams] first CTA of the team (its partial-sum slots)
  const int* team_case0;  // [nteams + 1] the team's cases are case_list[team_case0[t] .. team_case0[t+1])
  const int* case_list;   // case indices in team order
  const int* case_lo;     // [ncases] first row of each case
  const int* case_hi;     // [ncases] one past its last row
};

struct GmresCall {
  int n;
  const int* rowptr;
  const int* col;
  const double* val;
  const double* dinv;  // nullptr -> no preconditioner
  const double* b;
  double* x;
  int guess_zero;
  double rtol;
  int maxit;
  int restart;
  KspOut* out;
  int* err;
  // mixed precision (GMRES only): FP32 copies of the matrix values and of the Jacobi inverse
  // set => the Arnoldi cycles run in FP32 and each ends when its own residual estimate has
  // dropped by inner_rtol; every restart recomputes the true residual in FP64 (iterative
  // refinement), and convergence is tested on that FP64 residual
  const float* val32 = nullptr;
  const float* dinv32 = nullptr;
  double inner_rtol = 0.0;
  // Jacobi-Neumann polynomial preconditioner of this degree (1 or 2; needs dinv, and dinv32 in
  // mixed precision, where its stages run in FP32 like the Arnoldi cycles and on the FP64
  // residual stored in FP32); takes two more vectors per system in the Krylov workspace
  int poly = 0;
};
int gmres_grid(int n, int device_blocks);
int gmres_max_blocks(int device);
constexpr int kGmresPartStride = kMaxRestart + 4;
cudaError_t launch_gmres(const GmresCall& c, KrylovWork& w, cudaStream_t s);
// nsys (1 or 3) systems sharing rowptr/col/val/dinv/tolerances, solved in lockstep; the
// Krylov basis of system k starts at w.V + k*(restart+1)*w.ldv
cudaError_t launch_gmres_multi(const GmresCall* calls, int nsys, KrylovWork& w, cudaStream_t s);
// the same solves for every case of a batch: the teams of sched (device pointer) over `grid`
// CTAs; system q of case c reports to outs[q][c]
cudaError_t launch_gmres_batch(const GmresCall* calls, int nsys, KrylovWork& w, const BatchSchedule* sched, int grid,
                               KspOut* const* outs, cudaStream_t s);
// PETSc-style CG; needs at least four work vectors in w.V
cudaError_t launch_cg(const GmresCall& c, KrylovWork& w, cudaStream_t s);

}  // namespace cycas
