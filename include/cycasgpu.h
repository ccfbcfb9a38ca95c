/*
 * cycasgpu.h -- C ABI of the GB300 SIMPLE solve (libcycasgpu.so).
 *
 * Drop-in boundary for the reference's per-rank solver seams:
 *   NavierStokesSolver  (NS/navier.h:30-226)   -- CalculateVelocity / CalculatePressure /
 *                                                UpdateTurKEpsilon / NSSolve
 *   DataPartition::solve* (NS/MPIStructure.h:224-228, MPIStructure.cpp:234-531)
 *
 * Plain C types only: pointers + sizes, no C++ or torch types.  Every call returns an
 * int status (CYCAS_OK = 0) and never throws; the text of the last error of the calling
 * thread is available from cycas_last_error().  A context owns all device state of one
 * case and one CUDA stream; its calls must come from one host thread at a time.
 */
#ifndef CYCASGPU_H
#define CYCASGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
enum {
  CYCAS_OK = 0,
  CYCAS_NOT_CONVERGED = 1,  /* a Krylov solve ended with a negative KSP reason; the reference
                               throws ConvergeError{iter,residual,varname} here
                               (BasicType.h:62-68, MPIStructure.cpp:279-282) */
  CYCAS_NAN_DETECTED = 2,   /* NaN/Inf residual norm (KSP_DIVERGED_NANORINF) */
  CYCAS_ERR_INVALID = 3,    /* bad argument / unknown name / size mismatch */
  CYCAS_ERR_CUDA = 4,       /* CUDA runtime error */
  CYCAS_ERR_ALLOC = 5,      /* device or host allocation failed */
  CYCAS_ERR_IO = 6,         /* param or mesh file unreadable */
  CYCAS_ERR_TIMEOUT = 7,    /* a bounded device-side wait ran out (kernel returned early) */
  CYCAS_ERR_MESH = 8,       /* mesh rejected by the reference's own checks */
  CYCAS_ERR_UNSUPPORTED = 9 /* option outside the steady, constant-density path */
};

/* KSP converged reasons reported in cycas_solve_stats.reason (PETSc enum values) */
enum {
  CYCAS_KSP_CONVERGED_RTOL = 2,
  CYCAS_KSP_CONVERGED_ATOL = 3,
  CYCAS_KSP_DIVERGED_ITS = -3,
  CYCAS_KSP_DIVERGED_DTOL = -4,
  CYCAS_KSP_DIVERGED_BREAKDOWN = -5,
  CYCAS_KSP_DIVERGED_NANORINF = -9
};

/* preconditioners */
enum {
  CYCAS_PC_NONE = 0,
  CYCAS_PC_JACOBI = 1,   /* PCJACOBI: z = r / diag(A) */
  CYCAS_PC_ILU0 = 2,     /* ILU(0) in the natural (reference) cell order -- PETSc's
                            one-rank default PC (not available in this build) */
  CYCAS_PC_AMG = 3,      /* one cycle of plain aggregation multigrid (pressure system, CG
                            only): aggregates of <= 4 cells, weighted Jacobi (w 0.9), coarse
                            correction scaled by 2, dense coarsest level (<= 64 rows); see
                            cycas_options.amg_* */
  CYCAS_PC_POLY1 = 4,    /* Jacobi-Neumann polynomial of degree 1: M^-1 = (2I - D^-1 A) D^-1,
                            GMRES systems only (one more matrix product and grid barrier per
                            Krylov iteration, about half the iterations of Jacobi); in mixed
                            precision its stages run in FP32; no counterpart in the reference,
                            which uses PETSc's ILU(0) */
  CYCAS_PC_POLY2 = 5,    /* the same of degree 2: sum_{i<=2} (I - D^-1 A)^i D^-1 */
  CYCAS_PC_POLY3 = 6,    /* ... of degree 3 */
  CYCAS_PC_POLY4 = 7,    /* ... of degree 4 */
  CYCAS_PC_POLY5 = 8     /* ... of degree 5 (the fastest on the 480k-tet channel: each degree
                            costs one matrix product and barrier per iteration and saves
                            iterations up to about here) */
};

/* Krylov methods */
enum {
  CYCAS_KSP_DEFAULT = 0, /* the reference's choice: GMRES, except CG for the constant-density
                            pressure correction (MPIStructure.cpp:462-464) */
  CYCAS_KSP_GMRES = 1,
  CYCAS_KSP_CG = 2       /* PETSc KSPCG algorithm (Hestenes-Stiefel, preconditioned norm) */
};

/* systems, in the order of the reference's three solve wrappers */
enum { CYCAS_SYS_VELOCITY = 0, CYCAS_SYS_PRESSURE = 1, CYCAS_SYS_SCALAR = 2 };

/* Text of the last error on the calling thread (the message the reference prints before
 * MPI_Abort in ErrorHandler::fatalRuntimeError, NS/BasicType.h:23-55); valid until the next
 * failing call on that thread. */
const char* cycas_last_error(void);

/* ---- host-side case (param.in + gmsh v2 ASCII mesh) ------------------------------- */
typedef struct cycas_case cycas_case;

/* Reads a param.in (NS/readparamfile.cpp:10-344) and the gmsh mesh it names
 * (RootProcess::read, NS/RootStructure.cpp:428-487), numbers elements as the reference
 * does at one rank (RootStructure.cpp:797-816), builds the face list in the reference's
 * discovery order (CreateFaces/FindFace, NS/geometry.cpp:222-358) and the initial fields
 * (InitFlowField, NS/navier.cpp:588-697).  A relative gridfile is resolved against the
 * directory of param_path. */
int cycas_case_load(const char* param_path, cycas_case** out);
/* Same with flags: CYCAS_LOAD_MSH_BINARY reads the gridfile as the compressed binary gmsh form
 * (RootProcess::readBin, NS/RootStructure.cpp:61-116; the -mshBinary switch, NS/main.cpp:27,48):
 * uint64 vertex count, {int32 id, 3 doubles} per vertex, uint64 element count, {int32 id, int32
 * type, int32 ntag, ntag int32 tags, one-based int32 vertex ids} per element. */
#define CYCAS_LOAD_MSH_BINARY 1
int cycas_case_load_ex(const char* param_path, int32_t flags, cycas_case** out);
/* releases a loaded case (no counterpart: the reference keeps its mesh until the process exits) */
void cycas_case_free(cycas_case* c);
/* dims: [0] Ncel [1] Nfac [2] Nbnd [3] Nvrt (the solver's mesh sizes, NS/navier.h:104) [4] TurModel
 * [5] MaxStep [6] cellPressureRef (the options pool, NS/navier.cpp:475-516) [7] nnz */
int cycas_case_dims(const cycas_case* c, int64_t dims[8]);
/* residual stop value and relaxation factors of the case (dbOptions, NS/navier.cpp:777-791) */
int cycas_case_params(const cycas_case* c, double* residual_steady, double urf[8], double gravity[3]);
/* time and physics switches of the case: iopt = {IfSteady, TimeScheme, MaxOuterStep, SolveEnergy,
 * DensityModel, MaxStep}, dopt = {dt, total_time, PressureReference} (the "steady"/"transient",
 * "energy", "density" and "PressureRef" keys, NS/readparamfile.cpp:76-140) */
int cycas_case_physics(const cycas_case* c, int32_t iopt[6], double dopt[3]);
/* integer topology arrays by name (face_cell1, face_cell2, face_bnd, face_vertices, cell_nface,
 * cell_face, cell_cell, cell_vertices, cell_rid, bnd_face, bnd_rid, bnd_type, bnd_vertices) */
int cycas_case_get_int(const cycas_case* c, const char* name, int32_t* dst, int64_t n);
/* output cadence (the "output" key, noutput; NS/readparamfile.cpp:317-319) and the "restart"
 * key (IfReadBackup, readparamfile.cpp:168-178).  With restart yes the initial cell fields are
 * read from res.sav in the directory of param_path (ReadBackupFile, NS/navierIO.cpp:389-404,
 * which reads it from the working directory). */
int cycas_case_output(const cycas_case* c, int32_t* noutput, int32_t* restart);
/* host arrays of a loaded case: vert [3*Nvrt] and the initial cell fields U V W P R T VisLam
 * VisTur TE ED [Ncel] */
int cycas_case_get_field(const cycas_case* c, const char* name, double* dst, int64_t n);
/* Grid files of one partition holding the whole mesh: binary = 0 writes the ASCII Tecplot grid
 * (tec/grid.dat of OutputGrid, NS/navierIO.cpp:58-128), binary = 1 the binary geometry
 * (tec/geo of OutputGridBinary, navierIO.cpp:29-55: int32 {rank 0, 1 partition, Ncel, Nvrt},
 * Nvrt x 3 doubles, Ncel x 8 one-based int32 vertex numbers). */
int cycas_write_grid(const cycas_case* c, const char* path, int32_t binary);

/* ---- mesh view for callers that already hold the reference's Face/Cell/Bnd arrays --- */
typedef struct {
  int32_t ncel, nfac, nbnd, nvrt;
  /* topology, reference order (FaceData/CellData/BoundaryData, NS/BasicType.h:151-243) */
  const int32_t* face_cell1;    /* [nfac] */
  const int32_t* face_cell2;    /* [nfac]  < 0 on boundary faces */
  const int32_t* face_bnd;      /* [nfac]  boundary index, < 0 on interior faces */
  const int32_t* face_vertices; /* [4*nfac] (needed only when geometry is computed here) */
  const int32_t* cell_nface;    /* [ncel] */
  const int32_t* cell_face;     /* [6*ncel] row-major, cell_face[6*i+j] = Cell[i].face[j] */
  const int32_t* cell_cell;     /* [6*ncel] row-major, neighbour or < 0 */
  const int32_t* cell_vertices; /* [8*ncel] hex-form vertex list (needed only for geometry) */
  const int32_t* bnd_face;      /* [nbnd] */
  const int32_t* bnd_type;      /* [nbnd] regionMap[Bnd[i].rid].type1: 1 wall 2 inlet 3 outlet 4 sym */
  const double* vert;           /* [3*nvrt] (needed only for geometry) */
  /* geometry (CellFaceInfo, NS/geometry.cpp:391-752).  If face_x is NULL, all geometry is
   * computed on the device from vert/face_vertices/cell_vertices, bit-identical to the
   * reference's formulas evaluated without contraction. */
  const double* face_x;         /* [3*nfac] */
  const double* face_n;         /* [3*nfac] */
  const double* face_area;      /* [nfac] */
  const double* face_lambda;    /* [nfac] */
  const double* face_rlencos;   /* [nfac] */
  const double* face_xpac;      /* [3*nfac] */
  const double* face_xnac;      /* [3*nfac] */
  const double* cell_vol;       /* [ncel] */
  const double* cell_x;         /* [3*ncel] */
  const double* bnd_distance;   /* [nbnd] */
} cycas_mesh_view;

typedef struct {
  int32_t turb_model;        /* TurModel: 0 laminar, 1 k-epsilon */
  int32_t density_model;     /* DensityModel: 0 constant density, 1 perfect gas (energy is then solved) */
  int32_t cell_pressure_ref; /* cellPressureRef */
  double urf[8];             /* URF[0..7] */
  double gravity[3];
  /* fields below: zero selects the steady, isothermal defaults */
  int32_t transient;          /* 0 steady (IfSteady); 1 transient (the "transient" key) */
  int32_t time_scheme;        /* TimeScheme: 1 Euler, 2 the reference's "Dual" second-order form */
  double dt;                  /* time step */
  int32_t max_outer;          /* MaxOuterStep: a time step runs at most max_outer - 1 outer iterations */
  int32_t solve_energy;       /* SolveEnergy */
  double pressure_reference;  /* PressureReference (perfect gas; <= 0: 1.01325e5) */
} cycas_params;

typedef struct {
  int32_t type;      /* CYCAS_KSP_* */
  int32_t restart;   /* GMRES(m), default 30 */
  int32_t pc;        /* CYCAS_PC_* */
  double rtol;       /* <= 0: the reference's per-call value (1e-8 velocity/scalar, 1e-6 pressure) */
  int32_t maxit;     /* <= 0: the reference's per-call value (1000 velocity/pressure, 500 scalar) */
} cycas_ksp_options;

typedef struct {
  cycas_ksp_options ksp[3]; /* indexed by CYCAS_SYS_* */
  int32_t device;           /* CUDA device ordinal */
  int32_t mixed;            /* 0: FP64 Krylov (the reference's arithmetic).  1: mixed precision
                               for the GMRES systems (momentum, k, epsilon): FP32 Arnoldi cycles
                               wrapped in FP64 iterative refinement, each cycle ending at a
                               relative drop of inner_rtol, convergence tested on the FP64 true
                               residual to the system's rtol (no counterpart in the reference).
                               2: as 1, and the gradients, momentum rows and Rhie-Chow face flux
                               computed in FP32 (FP64 storage; the pressure-correction rows, their
                               FP64 mass-imbalance sum, the corrections and the residuals stay
                               FP64).  Level 2 shifts the discrete solution by about 1e-5
                               relative (48^3 cavity at ResMax 1e-6: u 4.5e-6, v 1.6e-5, w 6.5e-6,
                               p 4.9e-6 against FP64) and floors the residual between 1e-6 and
                               1e-8; level 1 stays within 1e-8 of FP64. */
  double inner_rtol;        /* <= 0: 1e-4 */
  /* pressure AMG cycle (CYCAS_PC_AMG; no counterpart in the reference, whose pressure PC is
   * PETSc's ILU(0)); 0 selects the default */
  float amg_omega;          /* Jacobi weight of the smoother, in (0, 1]; default 0.9 */
  float amg_alpha;          /* coarse-correction scale, in (0, 2]; default 2 (above 2 the cycle
                               can stop being a definite preconditioner) */
  int32_t amg_gamma;        /* cycles at the first level held in shared memory, 1..4 (1: a
                               V-cycle throughout, 2: a W-cycle at that level); default 2 for
                               cases of at least 80000 pressure rows, 1 below */
  int32_t reserved;
} cycas_options;

/* fills defaults: the reference's Krylov methods (GMRES(30); CG for pressure; the KSP set-up of
 * DataPartition::solve*, NS/MPIStructure.cpp:234-531), Jacobi, the reference's per-call
 * tolerances (NS/navier_velocity.cpp:28, navier_pressure.cpp:28, navier_scalar.cpp:98), device 0 */
void cycas_options_default(cycas_options* o);

/* ---- device context ------------------------------------------------------------------ */
typedef struct cycas_ctx cycas_ctx;

/* Replaces the NavierStokesSolver constructor (NS/navier.cpp:749) and DataPartition's matrix and
 * vector set-up (NS/MPIStructure.cpp:9-55, 204-233): copies the mesh (and computes geometry if
 * not given) into device memory.  cycas_create_from_case does the same for a loaded case and
 * sets InitFlowField's fields (NS/navier.cpp:588-697); cycas_destroy replaces
 * ~NavierStokesSolver (NS/navier.cpp:817) and DataPartition::deinit (NS/MPIStructure.cpp:56). */
int cycas_create(const cycas_mesh_view* mesh, const cycas_params* params, const cycas_options* opt,
                 cycas_ctx** out);
/* Same from a loaded case; fields start at the case's InitFlowField state. */
int cycas_create_from_case(const cycas_case* c, const cycas_options* opt, cycas_ctx** out);
void cycas_destroy(cycas_ctx* ctx);

/* Direct access to the solver's arrays (FlowField, NS/BasicType.h:74-148; RUFace, NS/navier.h:128;
 * the Face/Cell geometry, NS/BasicType.h:151-243).
 * Named device arrays: cell fields U V W P R T TE ED deltaP VisLam VisTur Apr; face field RUFace;
 * boundary arrays BRo BU BV BW BPre BTE BED; gradients dUdX dVdX dWdX dPdX dPhidX ([3*Ncel]);
 * geometry face_x face_n face_area face_lambda face_rlencos face_xpac face_xnac cell_vol cell_x
 * bnd_distance; matrix values A_val (+ b0 b1 b2 right-hand sides) of the last assembled system.
 * Host buffers; the call synchronises the context's stream. */
int cycas_get_field(cycas_ctx* ctx, const char* name, double* dst, int64_t n);
int cycas_set_field(cycas_ctx* ctx, const char* name, const double* src, int64_t n);
int cycas_get_int(cycas_ctx* ctx, const char* name, int32_t* dst, int64_t n); /* A_rowptr, A_col */
/* Several named arrays in one call (the cycas_set_fields / cycas_get_fields of the proposed
 * replacement surface): array i is names[i], n[i] doubles at src[i] / dst[i].  All names and
 * sizes are checked first; the copies are queued on the context's stream and waited for once. */
int cycas_set_fields(cycas_ctx* ctx, int32_t count, const char* const* names, const double* const* src,
                     const int64_t* n);
int cycas_get_fields(cycas_ctx* ctx, int32_t count, const char* const* names, double* const* dst, const int64_t* n);

/* One physical time step of a transient context (NS/navier.cpp:52-111): SaveTransientOldData
 * (navier.cpp:698-740), the clock advanced by dt, then outer SIMPLE iterations (momentum,
 * pressure, k-epsilon, energy) until ResMax0 / ResMax > 100 or max_outer - 1 of them ran.
 * For outer iteration k < cap: res_hist[10k..] its residuals, resmax[k] its ResMax,
 * its[8k..] / reasons[8k..] its Krylov solves (unused slots -1).  *n_outer receives the number
 * of outer iterations, *cur_time the clock after the step.  A Krylov failure ends the step with
 * CYCAS_NOT_CONVERGED (its outer iteration recorded). */
int cycas_time_step(cycas_ctx* ctx, int32_t cap, int32_t* n_outer, double* res_hist, double* resmax, int32_t* its,
                    int32_t* reasons, double* cur_time);

typedef struct {
  int32_t its[8];      /* Krylov iterations of each solve of the iteration, in call order */
  int32_t reason[8];   /* KSP converged reason of each solve */
  double rnorm[8];     /* final preconditioned residual norm of each solve */
  int32_t nsolves;
  int32_t failed_solve;/* index of the first solve with reason < 0, or -1 */
} cycas_iter_stats;

/* One steady SIMPLE-C iteration (NS/navier.cpp:60-111): CalculateVelocity, CalculatePressure,
 * UpdateTurKEpsilon when TurModel==1.  residual[10] receives the reduced localRes, *resmax
 * vec_max(residual).  Returns CYCAS_NOT_CONVERGED if any solve reported reason < 0. */
int cycas_simple_iteration(cycas_ctx* ctx, double residual[10], double* resmax, cycas_iter_stats* stats);

/* One SIMPLE-C iteration (the loop body of NSSolve, NS/navier.cpp:60-111) with the caller's host
 * fields as its state: the nin input fields are
 * uploaded before the stage that first reads them, the nout output fields downloaded once they
 * are final, and both kinds of copies overlap the iteration where its stages allow (inputs of
 * the k-epsilon stage upload during momentum and pressure; velocity, pressure and face-flux
 * outputs download during k-epsilon).  Returns when every output is in host memory.  Results
 * are those of cycas_set_fields + cycas_simple_iteration + cycas_get_fields; pinned host
 * arrays make the copies asynchronous.  Single-case contexts only. */
int cycas_simple_iteration_io(cycas_ctx* c, int32_t nin, const char* const* in_names, const double* const* in_src,
                              const int64_t* in_n, int32_t nout, const char* const* out_names,
                              double* const* out_dst, const int64_t* out_n, double residual[10], double* resmax,
                              cycas_iter_stats* stats);
/* n passes of the loop body of NSSolve (NS/navier.cpp:60-111), as n calls of
 * cycas_simple_iteration, back to back on the device, the residual history read once at the end
 * (no host synchronisation between iterations): res_hist[10k..], resmax[k], Krylov its[8k..] and
 * reasons[8k..] of pass k */
int cycas_simple_iterations(cycas_ctx* ctx, int32_t n, double* res_hist, double* resmax, int32_t* its,
                            int32_t* reasons);

/* The steady branch of NSSolve (NS/navier.cpp:52-145, IfSteady): SIMPLE-C iterations until
 * ResMax < residual_steady (the reference's stop test, navier.cpp:141-145) or max_step of them
 * ran.  *n_iter receives the iterations run; iteration k < cap reports res_hist[10k..],
 * resmax[k], its[8k..] and reasons[8k..] as cycas_simple_iterations does (any of them may be
 * null).  The result files of NSSolve's output cadence are the caller's (cycas_dump_begin).  A
 * failed Krylov solve ends the loop with its status, as ConvergeError ends the reference's. */
int cycas_solve_steady(cycas_ctx* ctx, int32_t max_step, double residual_steady, int32_t cap, int32_t* n_iter,
                       double* res_hist, double* resmax, int32_t* its, int32_t* reasons);

/* An in-HBM restart point (no counterpart in the reference, whose restart goes through the
 * res.sav file of WriteBackupFile/ReadBackupFile, navierIO.cpp:370-404): SAVE copies every
 * field of the context (cell and boundary fields, face fluxes, gradients, systems, previous
 * time levels) and the clock into one device buffer, allocated on the first save; RESTORE puts
 * them back.  Device-to-device copies queued on the context's stream. */
#define CYCAS_RESTART_SAVE 0
#define CYCAS_RESTART_RESTORE 1
int cycas_restart_point(cycas_ctx* ctx, int32_t op);

/* The solver's members one at a time (SetBCVelocity/SetBCPressure/SetBCDeltaP,
 * NS/navier_bc.cpp:8-181; Gradient, navier_gradient.cpp:12-74; BuildVelocityMatrix,
 * navier_velocity.cpp:63-393; CalRUFace2, navier_velocity.cpp:425-477; BuildPressureMatrix,
 * navier_pressure.cpp:99-232; the corrections, navier_pressure.cpp:45-70 and 235-278;
 * UpdateTurKEpsilon, navier_scalar.cpp:11-197; SaveTransientOldData, navier.h:191).
 * Individual stages for parity tests: bc_velocity bc_pressure bc_deltap grad_uvwp grad_deltap
 * build_velocity ruface2 build_pressure correct_cells correct_ruface calculate_velocity
 * calculate_pressure keps build_te (the k rows of keps) build_ed (the epsilon rows, on the
 * current k) energy build_energy save_transient clear_residual. */
int cycas_run_stage(cycas_ctx* ctx, const char* stage);

/* DataPartition::solveVelocity_GMRES / solvePressureCorrection / solveScarlar_GMRES
 * (MPIStructure.cpp:234-531) on the system last assembled for `sys`; x is solved in place
 * (device-resident fields are used when x is NULL: U/V/W, deltaP, or the scalar being
 * transported).  tol/maxit as the reference passes them. */
typedef struct {
  int32_t its;
  int32_t reason;
  double rnorm;
} cycas_solve_stats;

/* ---- measurement hooks ------------------------------------------------------------- */
/* The CUDA stream (cudaStream_t) all work of the context is issued on (no counterpart: a
 * measurement hook). */
int cycas_get_stream(cycas_ctx* ctx, void** stream);
typedef struct {
  int64_t kernel_launches;   /* kernels this context launched since the last reset */
  int64_t krylov_launches[3];/* persistent Krylov launches per system (CYCAS_SYS_*) */
  int64_t krylov_iters[3];   /* Krylov iterations per system */
  double krylov_ms[3];       /* CUDA-event time of those launches per system (profiling on) */
  double assembly_ms;        /* CUDA-event time outside the Krylov launches (profiling on) */
} cycas_profile;
/* Graph replay: with on = 1 the next iteration is captured as one CUDA graph (every launch of
 * the iteration, cooperative Krylov launches included) and later iterations replay it with a
 * single launch; exclusive with per-solve profiling.  No counterpart in the reference. */
int cycas_set_graph(cycas_ctx* ctx, int32_t on);
/* Profiling records CUDA events around every Krylov launch on the context's stream. */
int cycas_set_profiling(cycas_ctx* ctx, int32_t on);
int cycas_get_profile(cycas_ctx* ctx, cycas_profile* out);
int cycas_reset_profile(cycas_ctx* ctx);
/* Sizes of the pressure AMG hierarchy (0 levels unless CYCAS_PC_AMG is in use): *nlev levels,
 * rows[l] and stored entries nnz[l] for the first max_levels of them, fine to coarse. */
int cycas_get_amg_levels(cycas_ctx* ctx, int32_t max_levels, int32_t* nlev, int32_t* rows, int32_t* nnz);

/* ---- result files of case k of a context (k = 0 for a single-case context; a batch's case
 * index otherwise); each call copies the case's fields off the device and writes one file.
 * Output2Tecplot (NS/navierIO.cpp:161-283): the ASCII Tecplot result (tec/res0000.dat),
 * FEBRICK zone in BLOCK packing, x y z at the vertices, p u v w ro T Ma mu [te ed] at the cells,
 * "%19.5f " numbers five to a line; c is the loaded case (vertices, connectivity). */
int cycas_write_tecplot(cycas_ctx* ctx, int32_t k, const cycas_case* c, const char* path);
/* Output2TecplotBinary (navierIO.cpp:132-159): tec/data, int32 {rank 0, nVar} then the cell
 * fields P U V W R T [TE ED] as doubles, nVar = 6 (8 with k-epsilon). */
int cycas_write_data(cycas_ctx* ctx, int32_t k, const char* path);
/* WriteBackupFile (navierIO.cpp:370-387): res.sav, one line "R U V W P T R VisLam" per cell
 * (plus "VisTur TE ED" with k-epsilon) in printf %g. */
int cycas_write_backup(cycas_ctx* ctx, int32_t k, const char* path);
/* ReadBackupFile (navierIO.cpp:389-404): sets R U V W P T VisLam [VisTur TE ED] of case k from
 * a backup file. */
int cycas_read_backup(cycas_ctx* ctx, int32_t k, const char* path);

/* Asynchronous dump of case k (no counterpart in the reference, whose writers stop the solve
 * while they gather and format): the cell fields are snapshotted on the context's stream (a
 * device-to-device copy), copied to pinned host memory on a side stream while later iterations
 * run, and formatted and written by a host thread, to the same bytes as the writers above.
 * kinds is a set of CYCAS_DUMP_* bits; c (Tecplot only) must stay loaded until the dump ends.
 * One dump is in flight per context: a second begin waits for the first; cycas_dump_wait waits
 * and returns the dump's status (a failure not yet collected is returned by the next begin). */
#define CYCAS_DUMP_TECPLOT 1
#define CYCAS_DUMP_DATA 2
#define CYCAS_DUMP_BACKUP 4
int cycas_dump_begin(cycas_ctx* ctx, int32_t k, const cycas_case* c, int32_t kinds, const char* tecplot_path,
                     const char* data_path, const char* backup_path);
int cycas_dump_wait(cycas_ctx* ctx);

/* ---- DataPartition::solve* (NS/MPIStructure.h:224-228) on the systems the context assembled
 * last (the build_velocity / build_pressure stages, or the scalar rows of the keps / build_energy
 * stages): x is the caller's host array, read as the initial guess and overwritten with the
 * solution, as the reference writes into the caller's arrays in place.  tol is the relative
 * tolerance, maxit the iteration cap; the context's preconditioner and restart apply.  A solve
 * that ends with a negative converged reason returns CYCAS_NOT_CONVERGED (the reference's
 * ConvergeError) with its report in stats.
 * solveVelocity_GMRES (MPIStructure.cpp:234-375): Au with bu, bv, bw, three right-hand sides. */
int cycas_solve_velocity(cycas_ctx* ctx, double tol, int32_t maxit, double* xu, double* xv, double* xw,
                         cycas_iter_stats* stats);
/* solvePressureCorrection (MPIStructure.cpp:449-531): Ap with bp from a zero initial guess; CG when
 * is_symmetric, GMRES otherwise (the AMG preconditioner is replaced by Jacobi for GMRES). */
int cycas_solve_pressure(cycas_ctx* ctx, double tol, int32_t maxit, double* xp, int32_t is_symmetric,
                         cycas_iter_stats* stats);
/* solveScarlar_GMRES (MPIStructure.cpp:378-446): As with bs. */
int cycas_solve_scalar(cycas_ctx* ctx, double tol, int32_t maxit, double* xs, cycas_iter_stats* stats);

/* DataPartition::solve* (NS/MPIStructure.cpp:234-531) on a caller's matrix:
 * standalone Krylov solve of A x = b for a CSR matrix in HOST memory (int32 rowptr[n+1],
 * col[nnz], double val[nnz]); b and x are host arrays, x holds the initial guess unless
 * guess_zero.  Same GMRES/PC as the SIMPLE path. */
int cycas_csr_solve(int32_t n, const int32_t* rowptr, const int32_t* col, const double* val, const double* b,
                    double* x, const cycas_ksp_options* ksp, double rtol, int32_t maxit, int32_t guess_zero,
                    cycas_solve_stats* stats);

/* ---- batches (no counterpart in the reference: it runs one case per job) -------------
 * A batch context holds several independent cases in one device mesh and advances them
 * together: every assembly kernel is one launch over all cases, and every Krylov solve is one
 * cooperative launch whose CTAs are split into teams (one team per large case, single-CTA
 * teams working through the small ones), each team synchronising only its own CTAs.  Each
 * case keeps its own pressure reference cell, outlet mass balance, residuals, AMG hierarchy
 * and Krylov state, so its iteration is the one it would have alone (up to the summation
 * order of its inner products).  The cases must share TurModel, DensityModel, URF and gravity;
 * the pressure preconditioner must be CYCAS_PC_AMG.  Fields of the batch are the cases'
 * fields concatenated (cycas_batch_offsets gives each case's cell and boundary range); the
 * other calls of a context (get/set field, profiling) work on a batch context too. */
int cycas_batch_create(const cycas_case* const* cases, int32_t ncases, const cycas_options* opt, cycas_ctx** out);
int cycas_batch_size(cycas_ctx* ctx, int32_t* ncases);
/* kind 0: off[c] = first cell of case c, off[ncases] = total cells; kind 1: boundary faces */
int cycas_batch_offsets(cycas_ctx* ctx, int32_t kind, int32_t* off);
/* One SIMPLE-C iteration of every case: resmax[c] = vec_max of case c's localRes;
 * its/reasons[c*8 + k] = Krylov report of solve k of case c (-1 / 0 when not run). */
int cycas_batch_iteration(cycas_ctx* ctx, double* resmax, int32_t* its, int32_t* reasons);
/* Picks the team schedule of the batch's Krylov launches: for every CTA count G in {all, 3/4,
 * 1/2 of the co-resident maximum} and every row-share factor f in {0.5, 1, 2} (a case gets a
 * team of its own when it holds at least f*N/G of the N rows) it times `iters` SIMPLE
 * iterations and keeps the fastest.  These are real iterations of every case (they advance
 * the solution).  Reports the choice and its time per iteration. */
int cycas_batch_autotune(cycas_ctx* ctx, int32_t iters, int32_t* best_grid, double* best_factor, double* best_ms);
/* residual[c*10 + i] = localRes[i] of case c in the last iteration */
int cycas_batch_residuals(cycas_ctx* ctx, double* residual);

/* Moves the state of case sc of batch src (fields, boundary values, face fluxes) into case dc
 * of batch dst; the two cases must be the same mesh.  Used when a batch is re-formed.  (Batches
 * have no counterpart in the reference, nor do the two calls below.) */
int cycas_batch_copy_case(cycas_ctx* dst, int32_t dc, cycas_ctx* src, int32_t sc);
/* the slice of a per-cell or per-boundary field belonging to case k of a batch */
int cycas_batch_case_field(cycas_ctx* ctx, int32_t k, const char* name, double* dst, int64_t n);

/* ---- serving (no counterpart in the reference) ------------------------------------------
 * A request loop with continuous batching: submitted cases queue in arrival order; each step
 * admits queued cases while the estimated device footprint of the active ones stays within
 * the HBM budget, re-forms the batch of every physics class (turbulence model) whose
 * membership changed (the state of continuing cases is moved on the device), advances every
 * active case by one SIMPLE-C iteration, and retires each case whose residual, the reference's
 * ResMax divided by the case's volume, is at or below the tolerance (or that reached the
 * iteration cap).  Times are seconds of a monotonic clock (cycas_server_clock). */
typedef struct cycas_server cycas_server;
enum { CYCAS_REQ_CONVERGED = 1, CYCAS_REQ_FAILED = 2, CYCAS_REQ_MAX_ITERS = 3 };
typedef struct {
  int64_t id;
  int32_t status;      /* CYCAS_REQ_* */
  int32_t iterations;  /* SIMPLE-C iterations done */
  int32_t ncel;
  int32_t pad;
  double t_arrival, t_admit, t_done;
  double resmax;       /* normalised residual at retirement */
} cycas_request_result;
/* estimated device bytes of a case in a batch (what admission counts against the budget); this and
 * the cycas_server_* calls have no counterpart in the reference */
double cycas_footprint_estimate(const cycas_case* c);
int cycas_server_create(const cycas_options* opt, double hbm_budget_bytes, double residual_tol, int32_t max_iters,
                        int32_t keep_fields, cycas_server** out);
void cycas_server_destroy(cycas_server* s);
/* Replay each batch's SIMPLE-C iterations as one CUDA graph (cycas_set_graph on every batch the
 * server builds; a batch is captured on its first iteration after a rebuild).  No counterpart in
 * the reference. */
int cycas_server_set_graph(cycas_server* s, int32_t on);
/* Admission by compute as well as by memory: requests join only while the cells of the active
 * requests stay within max_cells (0: no cap; a request larger than the cap runs alone once
 * nothing else is active).  When requests arrive faster than the GPU finishes them, the cap keeps
 * each step short and lets admitted requests finish in arrival order instead of every request
 * advancing slowly in one huge batch.  No counterpart in the reference. */
int cycas_server_set_max_cells(cycas_server* s, double max_cells);
/* Batch rebuilds on a worker thread (on = 1): while the next batch of a class is built, the
 * current one keeps iterating its members, and the server switches at the first step after the
 * build (newly admitted requests wait for it).  The build's kernels and copies then share the GPU
 * with the iterations' cooperative kernels, which occupy every SM, so a build takes several
 * times longer: worth it when requests keep arriving (the Poisson stream: 37.5 M instead of
 * 28.5 M cell-iters/s), not for a fixed set submitted at once (256 cavities: 61.8 s instead of
 * 50.6 s).  Default off.  No counterpart in the reference. */
int cycas_server_set_async_rebuild(cycas_server* s, int32_t on);
double cycas_server_clock(void);
/* queues a request; CYCAS_ERR_UNSUPPORTED for transient, energy or perfect-gas cases (batches
 * hold steady, isothermal, constant-density cases) */
int cycas_server_submit(cycas_server* s, const char* param_path, int64_t* id);
int cycas_server_step(cycas_server* s, int32_t* n_active, int32_t* n_queued);
/* results of requests finished since the last poll (at most max) */
int cycas_server_poll(cycas_server* s, cycas_request_result* out, int32_t max, int32_t* n);
/* final U V W P TE ED of a finished request (server created with keep_fields) */
int cycas_server_result_field(cycas_server* s, int64_t id, const char* name, double* dst, int64_t n);
const char* cycas_server_last_error(cycas_server* s);
/* where the loop's host time went: out[0] steps, out[1] batch rebuilds (membership changes),
 * out[2] seconds in rebuilds (union mesh, device setup, AMG hierarchies, state copies),
 * out[3] seconds in batch iterations */
int cycas_server_stats(cycas_server* s, double* out);

/* No counterpart in the reference: the GMRES solve of cycas_csr_solve for callers that cannot
 * allocate device memory (their HBM is pre-reserved by another allocator, or they must not add
 * the device-wide synchronisation of cudaMalloc/cudaFree between their kernels).  rowptr, col,
 * val, b and x are DEVICE pointers owned by the caller (a well-formed CSR: rowptr ascending
 * from 0, columns in [0, n)); x holds the initial guess unless guess_zero and receives the
 * solution.  Scratch comes from one static device array of 8,987,136 bytes per GPU: n above
 * 32768 rows or restart above 32 is rejected with CYCAS_ERR_INVALID, as are preconditioners
 * other than NONE/JACOBI and Krylov types other than DEFAULT/GMRES.  Work is issued on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) and the call returns after the
 * stream has finished it.  The first call on a device looks the array's address up with that
 * device current, and under lazy module loading (CUDA's default) that lookup is also what loads
 * the library's device code and places the static array -- the one device allocation and
 * synchronisation this entry point makes, once per device and process.  So make one warm-up call
 * per device at start-up (n = 1 will do), before any stream capture and before the phase that
 * must not allocate.  All calls on a device share the array: calls that overlap on the GPU race
 * and must be serialised by the caller. */
int cycas_csr_solve_noalloc(int32_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                            const double* b, double* x, const cycas_ksp_options* ksp, double rtol, int32_t maxit,
                            int32_t guess_zero, void* stream, cycas_solve_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* CYCASGPU_H */
