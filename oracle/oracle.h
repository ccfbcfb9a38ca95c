// CPU ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A single-rank C++ restatement of the Cycas2Parallel (Meiyim/SYSU_CFD_Parallel)
// SIMPLE solve (steady and transient, constant density or perfect gas, k-epsilon and
// energy), written from the reference's behaviour, used only by
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm
// as the checker.  Nothing in the product links or calls it.
//
// Parity status: UNPINNED at the PETSc boundary.  The reference cannot be built
// here (it needs MPI, PETSc, METIS and CGNS, none of which exist on either
// machine) and ships no tests, fixtures or golden vectors.  The linear-solve
// arithmetic lives in PETSc (version unpinned by the reference's makefile);
// this file restates PETSc's documented GMRES(m) (classical Gram-Schmidt,
// left preconditioning, preconditioned-norm convergence test) and ILU(0) /
// Jacobi from the published algorithms.  Everything outside the Krylov solve
// follows the reference's source line by line (file:line cited at each
// function) and is checked by known-answer tests (Green-Gauss exact on linear
// fields, closed-surface normals sum to zero, volumes sum to the box volume,
// pressure-matrix row sums vanish).
//
// Compiled with -ffp-contract=off so every product and sum rounds exactly as
// the source text orders it.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace orc {

constexpr double SMALL = 1.e-16;                       // BasicType.h:12
constexpr int VOID_CELL_ON_BOUNDARY = -10;              // navier.h:17
constexpr int VOID_CELL_ON_INTERFACE = -20;             // navier.h:18
constexpr int INNER_FACE_BOUNDARY = -10;                // navier.h:19
constexpr int RESIDUAL_LEN = 10;                        // navier.h:16

struct Region {            // BdRegion, BasicType.h:247-310
  std::string name;
  int type1 = -1, type2 = -1;
  double fixedValue = 2147483647.0;
  double initvalues[10] = {0};
};

struct Face {              // FaceData, BasicType.h:151-174
  int bnd = 0, vertices[4] = {0, 0, 0, 0}, cell1 = 0, cell2 = 0;
  double x[3], n[3], area, lambda, rlencos, Xpac[3], Xnac[3];
};

struct Cell {              // CellData, BasicType.h:177-221
  int nface = 0, rid = 0, face[6], cell[6], vertices[8], globalIdx = 0;
  double vol, x[3];
};

struct Bnd {               // BoundaryData, BasicType.h:226-243
  int face = 0, vertices[4], rid = 0;
  double distance = 0, yplus = 0, uplus = 0, shear[3] = {0, 0, 0}, h = 0, q = 0, T = 0;
};

// AIJ-like sparse matrix: fixed pattern (diagonal + face neighbours, columns
// sorted as PETSc's AIJ stores them), values inserted with INSERT semantics.
struct Csr {
  int n = 0;
  std::vector<int> rowptr, col, diag;
  std::vector<double> val;
  void insert(int row, int c, double v);
  void zero() { std::fill(val.begin(), val.end(), 0.0); }
};

// PC_POLY1..5: Jacobi-Neumann polynomials sum_{i<=d} (I - D^-1 A)^i D^-1 of degree d = 1..5
// (the GPU path's optional preconditioner for the GMRES systems)
enum PcType { PC_NONE = 0, PC_JACOBI = 1, PC_ILU0 = 2, PC_POLY1 = 3, PC_POLY2 = 4, PC_POLY3 = 5, PC_POLY4 = 6,
              PC_POLY5 = 7 };
inline int poly_degree(int pc) { return pc >= PC_POLY1 && pc <= PC_POLY5 ? pc - PC_POLY1 + 1 : 0; }

enum KspType { KSP_GMRES = 0, KSP_CG = 1 };

struct KspSettings {       // one per system: velocity, pressure, scalar
  int type = KSP_GMRES;    // the pressure system defaults to CG (see Case)
  int restart = 30;
  int pc = PC_ILU0;
  double rtol_override = -1.0;  // <0: use the caller's tol (the reference's per-solve value)
  double abstol = 1e-50, dtol = 1e4, haptol = 1e-30;
  int maxit_override = -1;
  std::vector<int> perm;   // optional symmetric permutation applied before ILU(0)
};

struct KspResult { int its = 0; int reason = 0; double rnorm = 0; };

// KSPConvergedReason values used here (PETSc public enum values)
enum { KSP_CONVERGED_RTOL = 2, KSP_CONVERGED_ATOL = 3, KSP_DIVERGED_ITS = -3, KSP_DIVERGED_DTOL = -4,
       KSP_DIVERGED_BREAKDOWN = -5, KSP_DIVERGED_INDEFINITE_PC = -8, KSP_DIVERGED_NANORINF = -9,
       KSP_DIVERGED_INDEFINITE_MAT = -10 };

struct Case {
  // options pool, navier.cpp:749-791 and defaults navier.cpp:475-516
  int IfReadBackup = 0, IfSteady = 1, SolveEnergy = 0, SolveSpecies = 0, shouldOutputBinary = 0;
  int MaxOuterStep = 50, TurModel = 0, DensityModel = 0, limiter = 0, TimeScheme = 1;
  int noutput = 1, outputFormat = 0, Nspecies = 0, cellPressureRef = 0, MaxStep = 10000;
  double PressureReference = 1.01325e5, gama = 1.4, ga1 = 0.4, cp = 1006., cv = 1006. / 1.4, prl = 0.72, prte = 0.9;
  double Rcpcv = 1006. - 1006. / 1.4, TempRef = 273.15, total_time = 0., dt = 1.0;
  double gravity[3] = {0, 0, 0};
  double URF[8] = {0.6, 0.6, 0.6, 0.5, 0.8, 0.8, 0.8, 0.8};
  double ResidualSteady = 1.e-6;
  std::string GridFileName;
  std::map<int, Region> regionMap;

  // mesh
  int Nvrt = 0, Ncel = 0, Nfac = 0, Nbnd = 0;
  std::vector<double> Vert;          // 3*Nvrt
  std::vector<Face> F;
  std::vector<Cell> C;
  std::vector<Bnd> B;

  // fields (navier.h:110-130)
  std::vector<double> Rn, Un, Vn, Wn, Pn, Tn, TE, ED, deltaP, VisLam, VisTur, Apr, RUFace;
  std::vector<double> dPdX, dUdX, dVdX, dWdX, dPhidX;   // 3*Ncel, row-major [cell][3]
  std::vector<double> BRo, BU, BV, BW, BPre, BTem, BTE, BED;
  double localRes[RESIDUAL_LEN], Residual[RESIDUAL_LEN];
  int step = 0;

  // linear systems (DataPartition Au/Ap/As + bu,bv,bw,bp,bs)
  Csr Au, Ap, As;
  std::vector<double> bu, bv, bw, bp, bs;
  // 0 velocity, 1 pressure, 2 scalar.  solvePressureCorrection selects CG when the density
  // is constant (MPIStructure.cpp:462-464), GMRES otherwise.
  KspSettings ksp[3] = {KspSettings(), KspSettings{KSP_CG}, KspSettings()};
  std::vector<KspResult> kspLog;     // every solve of the last iteration, in call order
  int kspFailures = 0;

  // k-epsilon work arrays kept for inspection (navier_scalar.cpp:21-27)
  std::vector<double> Prod, TESource, EDSource, ApTE, ApED;
  std::vector<double> VisTE, VisED;  // effective diffusivities of the k and epsilon rows
  // energy work arrays kept for inspection (navier_scalar.cpp:209-217)
  std::vector<double> kcond, ESource, ApE;
  int reverseInletWarnings = 0;

  // transient runs (navier.h:136-150): previous time levels and the clock
  std::vector<double> Rnp, Unp, Vnp, Wnp, Tnp, TEp, EDp;
  std::vector<double> Rnp2, Unp2, Vnp2, Wnp2, Tnp2, TEp2, EDp2;
  double cur_time = 0.;

  // TE^1.5 of the wall function: 0 = the mathematical value rounded once (pow15, what the GPU
  // computes), 1 = the C library's std::pow, as the reference's own build calls it
  // (navier_bc.cpp:279); the two differ by one ulp on a small share of arguments.
  int libm_pow = 0;
};

// setup (mesh + params + init), following main.cpp:38-65 at one rank
void read_param_file(Case& cs, const std::string& path);
void read_grid_and_build(Case& cs, const std::string& meshPath);
void init_flow_field(Case& cs);
void build_pattern(Case& cs);

// one SIMPLE iteration of NSSolve (navier.cpp:60-111); returns ResMax
double simple_iteration(Case& cs);
// one physical time step of a transient run (navier.cpp:52-111): SaveTransientOldData, then
// outer iterations until the residual has dropped by a factor 100 or MaxOuterStep - 1 of them
// ran; resmax[k] is the ResMax of outer iteration k.  Returns the number of outer iterations.
int time_step(Case& cs, std::vector<double>* resmax, std::vector<double>* residuals,
              std::vector<KspResult>* ksp);
void save_transient_old_data(Case& cs);
void set_bc_temperature(Case& cs);
void update_energy(Case& cs);
void build_energy(Case& cs);

// stages
void set_bc_velocity(Case& cs);
void set_bc_pressure(Case& cs);
void set_bc_deltap(Case& cs);
void gradient(Case& cs, const double* phi, const double* Bphi, double* grad);
void build_velocity_matrix(Case& cs);
void cal_ruface2(Case& cs);
void build_pressure_matrix(Case& cs);
void correct_ruface2(Case& cs);
void correct_cells(Case& cs);
int calculate_velocity(Case& cs);
int calculate_pressure(Case& cs);
void update_tur_kepsilon(Case& cs);
// the two assembly halves of update_tur_kepsilon: the k rows (sources, wall functions, boundary
// values, unsteady terms) and, on the solved k, the epsilon rows (k clipped, epsilon sources,
// wall-cell rows) -- each ends with the system in As / bs
void keps_build_te(Case& cs);
void keps_build_ed(Case& cs);
void build_scalar_matrix(Case& cs, int iSca, double* Phi, double* BPhi, double* DiffCoef, double* source, double* App);

// linear algebra
KspResult ksp_solve(const Csr& A, const KspSettings& s, double rtol, int maxit, bool guess_zero,
                    const double* b, double* x);

}  // namespace orc
