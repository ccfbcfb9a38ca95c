// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h; parity unpinned at the PETSc boundary).
// Flat C interface so tests and the benchmark's CPU arm can drive the oracle through ctypes.
#include <chrono>
#include <cstring>
#include <exception>
#include <string>

#include "oracle.h"

using namespace orc;

namespace {
thread_local std::string g_err;

struct Handle {
  Case cs;
};

template <class T>
int copy_out(const std::vector<T>& v, void* dst, long n) {
  if ((long)v.size() != n) return -2;
  std::memcpy(dst, v.data(), sizeof(T) * (size_t)n);
  return 0;
}

std::vector<double>* field(Case& cs, const std::string& nm) {
  if (nm == "U") return &cs.Un;
  if (nm == "V") return &cs.Vn;
  if (nm == "W") return &cs.Wn;
  if (nm == "P") return &cs.Pn;
  if (nm == "R") return &cs.Rn;
  if (nm == "T") return &cs.Tn;
  if (nm == "TE") return &cs.TE;
  if (nm == "ED") return &cs.ED;
  if (nm == "deltaP") return &cs.deltaP;
  if (nm == "VisLam") return &cs.VisLam;
  if (nm == "VisTur") return &cs.VisTur;
  if (nm == "Apr") return &cs.Apr;
  if (nm == "RUFace") return &cs.RUFace;
  if (nm == "dUdX") return &cs.dUdX;
  if (nm == "dVdX") return &cs.dVdX;
  if (nm == "dWdX") return &cs.dWdX;
  if (nm == "dPdX") return &cs.dPdX;
  if (nm == "dPhidX") return &cs.dPhidX;
  if (nm == "BRo") return &cs.BRo;
  if (nm == "BU") return &cs.BU;
  if (nm == "BV") return &cs.BV;
  if (nm == "BW") return &cs.BW;
  if (nm == "BPre") return &cs.BPre;
  if (nm == "BTE") return &cs.BTE;
  if (nm == "BED") return &cs.BED;
  if (nm == "bu") return &cs.bu;
  if (nm == "bv") return &cs.bv;
  if (nm == "bw") return &cs.bw;
  if (nm == "bp") return &cs.bp;
  if (nm == "bs") return &cs.bs;
  if (nm == "Au_val") return &cs.Au.val;
  if (nm == "Ap_val") return &cs.Ap.val;
  if (nm == "As_val") return &cs.As.val;
  if (nm == "Prod") return &cs.Prod;
  if (nm == "TESource") return &cs.TESource;
  if (nm == "EDSource") return &cs.EDSource;
  if (nm == "ApTE") return &cs.ApTE;
  if (nm == "ApED") return &cs.ApED;
  if (nm == "VisTE") return &cs.VisTE;
  if (nm == "VisED") return &cs.VisED;
  if (nm == "vert") return &cs.Vert;
  if (nm == "BTem") return &cs.BTem;
  if (nm == "kcond") return &cs.kcond;
  if (nm == "ESource") return &cs.ESource;
  if (nm == "ApE") return &cs.ApE;
  if (nm == "Rnp") return &cs.Rnp;
  if (nm == "Unp") return &cs.Unp;
  if (nm == "Vnp") return &cs.Vnp;
  if (nm == "Wnp") return &cs.Wnp;
  if (nm == "Tnp") return &cs.Tnp;
  if (nm == "TEp") return &cs.TEp;
  if (nm == "EDp") return &cs.EDp;
  return nullptr;
}
}  // namespace

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_load(const char* param_path) {
  try {
    Handle* h = new Handle();
    std::string p(param_path);
    read_param_file(h->cs, p);
    std::string grid = h->cs.GridFileName;
    if (!grid.empty() && grid[0] != '/') {
      size_t sl = p.find_last_of('/');
      if (sl != std::string::npos) grid = p.substr(0, sl + 1) + grid;
    }
    read_grid_and_build(h->cs, grid);
    init_flow_field(h->cs);
    return h;
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void orc_free(void* h) { delete (Handle*)h; }

// dims: Ncel, Nfac, Nbnd, Nvrt, TurModel, nnz, MaxStep, cellPressureRef
int orc_dims(void* hp, int* out) {
  Case& cs = ((Handle*)hp)->cs;
  out[0] = cs.Ncel;
  out[1] = cs.Nfac;
  out[2] = cs.Nbnd;
  out[3] = cs.Nvrt;
  out[4] = cs.TurModel;
  out[5] = (int)cs.Au.col.size();
  out[6] = cs.MaxStep;
  out[7] = cs.cellPressureRef;
  return 0;
}

int orc_get_params(void* hp, double* urf8, double* gravity3) {
  Case& cs = ((Handle*)hp)->cs;
  for (int i = 0; i < 8; i++) urf8[i] = cs.URF[i];
  for (int i = 0; i < 3; i++) gravity3[i] = cs.gravity[i];
  return 0;
}

int orc_get(void* hp, const char* name, double* dst, long n) {
  Case& cs = ((Handle*)hp)->cs;
  std::string nm(name);
  if (std::vector<double>* v = field(cs, nm)) return copy_out(*v, dst, n);
  std::vector<double> tmp;
  auto faces3 = [&](auto get) {
    tmp.resize(3 * (size_t)cs.Nfac);
    for (int i = 0; i < cs.Nfac; i++)
      for (int d = 0; d < 3; d++) tmp[3 * i + d] = get(cs.F[i])[d];
  };
  if (nm == "face_x") faces3([](const Face& f) { return f.x; });
  else if (nm == "face_n") faces3([](const Face& f) { return f.n; });
  else if (nm == "face_xpac") faces3([](const Face& f) { return f.Xpac; });
  else if (nm == "face_xnac") faces3([](const Face& f) { return f.Xnac; });
  else if (nm == "face_area" || nm == "face_lambda" || nm == "face_rlencos") {
    tmp.resize(cs.Nfac);
    for (int i = 0; i < cs.Nfac; i++)
      tmp[i] = nm == "face_area" ? cs.F[i].area : nm == "face_lambda" ? cs.F[i].lambda : cs.F[i].rlencos;
  } else if (nm == "cell_vol") {
    tmp.resize(cs.Ncel);
    for (int i = 0; i < cs.Ncel; i++) tmp[i] = cs.C[i].vol;
  } else if (nm == "cell_x") {
    tmp.resize(3 * (size_t)cs.Ncel);
    for (int i = 0; i < cs.Ncel; i++)
      for (int d = 0; d < 3; d++) tmp[3 * i + d] = cs.C[i].x[d];
  } else if (nm == "bnd_distance") {
    tmp.resize(cs.Nbnd);
    for (int i = 0; i < cs.Nbnd; i++) tmp[i] = cs.B[i].distance;
  } else if (nm == "bnd_shear") {
    tmp.resize(3 * (size_t)cs.Nbnd);
    for (int i = 0; i < cs.Nbnd; i++)
      for (int d = 0; d < 3; d++) tmp[3 * i + d] = cs.B[i].shear[d];
  } else if (nm == "residual") {
    tmp.assign(cs.Residual, cs.Residual + RESIDUAL_LEN);
  } else {
    g_err = "unknown array " + nm;
    return -1;
  }
  return copy_out(tmp, dst, n);
}

int orc_set(void* hp, const char* name, const double* src, long n) {
  Case& cs = ((Handle*)hp)->cs;
  std::vector<double>* v = field(cs, name);
  if (!v) {
    g_err = std::string("unknown or read-only array ") + name;
    return -1;
  }
  if ((long)v->size() != n) return -2;
  std::memcpy(v->data(), src, sizeof(double) * (size_t)n);
  return 0;
}

int orc_geti(void* hp, const char* name, int* dst, long n) {
  Case& cs = ((Handle*)hp)->cs;
  std::string nm(name);
  std::vector<int> tmp;
  if (nm == "face_cell1" || nm == "face_cell2" || nm == "face_bnd") {
    tmp.resize(cs.Nfac);
    for (int i = 0; i < cs.Nfac; i++)
      tmp[i] = nm == "face_cell1" ? cs.F[i].cell1 : nm == "face_cell2" ? cs.F[i].cell2 : cs.F[i].bnd;
  } else if (nm == "face_vertices") {
    tmp.resize(4 * (size_t)cs.Nfac);
    for (int i = 0; i < cs.Nfac; i++)
      for (int k = 0; k < 4; k++) tmp[4 * i + k] = cs.F[i].vertices[k];
  } else if (nm == "cell_nface" || nm == "cell_rid") {
    tmp.resize(cs.Ncel);
    for (int i = 0; i < cs.Ncel; i++) tmp[i] = nm == "cell_nface" ? cs.C[i].nface : cs.C[i].rid;
  } else if (nm == "cell_face" || nm == "cell_cell") {
    tmp.assign(6 * (size_t)cs.Ncel, -1);
    for (int i = 0; i < cs.Ncel; i++)
      for (int k = 0; k < cs.C[i].nface; k++) tmp[6 * i + k] = nm == "cell_face" ? cs.C[i].face[k] : cs.C[i].cell[k];
  } else if (nm == "cell_vertices") {
    tmp.resize(8 * (size_t)cs.Ncel);
    for (int i = 0; i < cs.Ncel; i++)
      for (int k = 0; k < 8; k++) tmp[8 * i + k] = cs.C[i].vertices[k];
  } else if (nm == "bnd_face" || nm == "bnd_rid") {
    tmp.resize(cs.Nbnd);
    for (int i = 0; i < cs.Nbnd; i++) tmp[i] = nm == "bnd_face" ? cs.B[i].face : cs.B[i].rid;
  } else if (nm == "bnd_type") {
    tmp.resize(cs.Nbnd);
    for (int i = 0; i < cs.Nbnd; i++) tmp[i] = cs.regionMap[cs.B[i].rid].type1;
  } else if (nm == "bnd_vertices") {
    tmp.resize(4 * (size_t)cs.Nbnd);
    for (int i = 0; i < cs.Nbnd; i++)
      for (int k = 0; k < 4; k++) tmp[4 * i + k] = cs.B[i].vertices[k];
  } else if (nm == "A_rowptr") {
    tmp = cs.Au.rowptr;
  } else if (nm == "A_col") {
    tmp = cs.Au.col;
  } else {
    g_err = "unknown int array " + nm;
    return -1;
  }
  return copy_out(tmp, dst, n);
}

// which: 0 velocity, 1 pressure, 2 scalar; type: 0 gmres, 1 cg; pc: 0 none, 1 jacobi, 2 ilu0
int orc_set_ksp_type(void* hp, int which, int type) {
  Case& cs = ((Handle*)hp)->cs;
  if (which < 0 || which > 2 || type < 0 || type > 1) return -1;
  cs.ksp[which].type = type;
  return 0;
}

int orc_set_ksp(void* hp, int which, int pc, int restart, double rtol_override, int maxit_override) {
  Case& cs = ((Handle*)hp)->cs;
  if (which < 0 || which > 2) return -1;
  cs.ksp[which].pc = pc;
  cs.ksp[which].restart = restart;
  cs.ksp[which].rtol_override = rtol_override;
  cs.ksp[which].maxit_override = maxit_override;
  return 0;
}

// TE^1.5 of the wall function: 0 rounded once (default, as the GPU), 1 the C library's pow (as
// the reference's own build)
int orc_set_libm_pow(void* hp, int flag) {
  ((Handle*)hp)->cs.libm_pow = flag ? 1 : 0;
  return 0;
}

int orc_set_ksp_perm(void* hp, int which, const int* perm, long n) {
  Case& cs = ((Handle*)hp)->cs;
  if (n == 0) cs.ksp[which].perm.clear();
  else cs.ksp[which].perm.assign(perm, perm + n);
  return 0;
}

int orc_stage(void* hp, const char* name) {
  Case& cs = ((Handle*)hp)->cs;
  std::string s(name);
  try {
    if (s == "bc_velocity") set_bc_velocity(cs);
    else if (s == "bc_pressure") set_bc_pressure(cs);
    else if (s == "bc_deltap") set_bc_deltap(cs);
    else if (s == "grad_uvwp") {
      gradient(cs, cs.Un.data(), cs.BU.data(), cs.dUdX.data());
      gradient(cs, cs.Vn.data(), cs.BV.data(), cs.dVdX.data());
      gradient(cs, cs.Wn.data(), cs.BW.data(), cs.dWdX.data());
      gradient(cs, cs.Pn.data(), cs.BPre.data(), cs.dPdX.data());
    } else if (s == "grad_deltap") gradient(cs, cs.deltaP.data(), cs.BPre.data(), cs.dPdX.data());
    else if (s == "build_velocity") build_velocity_matrix(cs);
    else if (s == "ruface2") cal_ruface2(cs);
    else if (s == "build_pressure") build_pressure_matrix(cs);
    else if (s == "correct_cells") correct_cells(cs);
    else if (s == "correct_ruface") correct_ruface2(cs);
    else if (s == "calculate_velocity") calculate_velocity(cs);
    else if (s == "calculate_pressure") calculate_pressure(cs);
    else if (s == "keps") update_tur_kepsilon(cs);
    else if (s == "build_te") keps_build_te(cs);
    else if (s == "build_ed") keps_build_ed(cs);
    else if (s == "build_energy") build_energy(cs);
    else if (s == "energy") update_energy(cs);
    else if (s == "save_transient") save_transient_old_data(cs);
    else if (s == "clear_residual") {
      for (int i = 0; i < RESIDUAL_LEN; i++) cs.localRes[i] = cs.Residual[i] = 0.0;
    } else {
      g_err = "unknown stage " + s;
      return -1;
    }
  } catch (std::exception& e) {
    g_err = e.what();
    return -3;
  }
  return 0;
}

// Runs nsteps steady SIMPLE iterations.  res_hist: nsteps*10, resmax: nsteps,
// ksp_its / ksp_reason: nsteps*8 (the solves of each iteration in call order,
// unused slots -1).  Returns the number of completed iterations, or <0 on error.
int orc_iterate(void* hp, int nsteps, double* res_hist, double* resmax, int* ksp_its, int* ksp_reason) {
  Case& cs = ((Handle*)hp)->cs;
  for (int s = 0; s < nsteps; s++) {
    try {
      double rm = simple_iteration(cs);
      if (resmax) resmax[s] = rm;
      if (res_hist)
        for (int i = 0; i < RESIDUAL_LEN; i++) res_hist[s * RESIDUAL_LEN + i] = cs.Residual[i];
      for (int k = 0; k < 8; k++) {
        bool have = k < (int)cs.kspLog.size();
        if (ksp_its) ksp_its[s * 8 + k] = have ? cs.kspLog[k].its : -1;
        if (ksp_reason) ksp_reason[s * 8 + k] = have ? cs.kspLog[k].reason : -1;
      }
    } catch (std::exception& e) {
      g_err = e.what();
      return -(s + 1);
    }
  }
  return nsteps;
}

// physics switches: iopt = {IfSteady, TimeScheme, MaxOuterStep, SolveEnergy, DensityModel, MaxStep},
// dopt = {dt, total_time, cur_time, PressureReference}
int orc_physics(void* hp, int* iopt, double* dopt) {
  Case& cs = ((Handle*)hp)->cs;
  int iv[6] = {cs.IfSteady, cs.TimeScheme, cs.MaxOuterStep, cs.SolveEnergy, cs.DensityModel, cs.MaxStep};
  double dv[4] = {cs.dt, cs.total_time, cs.cur_time, cs.PressureReference};
  if (iopt) std::memcpy(iopt, iv, sizeof iv);
  if (dopt) std::memcpy(dopt, dv, sizeof dv);
  return 0;
}

// One physical time step of a transient case.  Up to `cap` outer iterations are recorded:
// resmax[k], res_hist[10k..], ksp_its / ksp_reason [8k..].  Returns the number of outer
// iterations, or <0 on error.
int orc_time_step(void* hp, int cap, double* resmax, double* res_hist, int* ksp_its, int* ksp_reason) {
  Case& cs = ((Handle*)hp)->cs;
  try {
    std::vector<double> rm, rh;
    std::vector<KspResult> kl;
    int n = time_step(cs, &rm, &rh, &kl);
    for (int k = 0; k < n && k < cap; k++) {
      if (resmax) resmax[k] = rm[k];
      if (res_hist)
        for (int i = 0; i < RESIDUAL_LEN; i++) res_hist[k * RESIDUAL_LEN + i] = rh[k * RESIDUAL_LEN + i];
      for (int q = 0; q < 8; q++) {
        if (ksp_its) ksp_its[k * 8 + q] = kl[k * 8 + q].its;
        if (ksp_reason) ksp_reason[k * 8 + q] = kl[k * 8 + q].reason;
      }
    }
    return n;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// standalone Krylov solve on an arbitrary CSR system (for solver unit tests)
int orc_csr_solve(int n, const int* rowptr, const int* col, const double* val, const double* b, double* x,
                  int type, int pc, int restart, double rtol, int maxit, int guess_zero, int* its, int* reason,
                  double* rnorm) {
  try {
    Csr A;
    A.n = n;
    A.rowptr.assign(rowptr, rowptr + n + 1);
    A.col.assign(col, col + rowptr[n]);
    A.val.assign(val, val + rowptr[n]);
    A.diag.assign(n, -1);
    for (int i = 0; i < n; i++)
      for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; k++)
        if (A.col[k] == i) A.diag[i] = k;
    KspSettings s;
    s.type = type;
    s.pc = pc;
    s.restart = restart;
    KspResult r = ksp_solve(A, s, rtol, maxit, guess_zero != 0, b, x);
    *its = r.its;
    *reason = r.reason;
    *rnorm = r.rnorm;
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

}  // extern "C"
