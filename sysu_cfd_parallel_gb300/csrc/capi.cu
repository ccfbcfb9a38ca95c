// C ABI of libcycasgpu: case loading, device context, the SIMPLE iteration schedule.
//
// One context = one case resident on one GPU with one stream.  An iteration is a fixed
// sequence of kernel launches (boundary conditions, gradients, assembly, persistent GMRES
// solves, corrections) with no host synchronisation until its status block is read back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <map>
#include <string>
#include <vector>

#include "../../include/cycasgpu.h"
#include "cycas_amg.h"
#include "cycas_device.h"
#include "cycas_host.h"

struct cycas_case {
  cycas::HostCase hc;
};

namespace cycas {

thread_local std::string g_last_error;
thread_local long long g_launch_count = 0;

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct StatusError : std::runtime_error {
  int code;
  StatusError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                                          \
  do {                                                                                                 \
    cudaError_t e_ = (x);                                                                              \
    if (e_ != cudaSuccess)                                                                             \
      throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" +      \
                      std::to_string(__LINE__) + ")");                                               \
  } while (0)

template <class F>
int guard(F&& f) {
  try {
    return f();
  } catch (StatusError& e) {
    g_last_error = e.what();
    return e.code;
  } catch (CudaError& e) {
    g_last_error = e.what();
    return CYCAS_ERR_CUDA;
  } catch (IoError& e) {
    g_last_error = e.what();
    return CYCAS_ERR_IO;
  } catch (MeshError& e) {
    g_last_error = e.what();
    return CYCAS_ERR_MESH;
  } catch (ParamError& e) {
    g_last_error = e.what();
    return CYCAS_ERR_INVALID;
  } catch (std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return CYCAS_ERR_ALLOC;
  } catch (std::exception& e) {
    g_last_error = e.what();
    return CYCAS_ERR_INVALID;
  }
}

}  // namespace cycas

using namespace cycas;

struct cycas_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  DevMesh m;
  DevFields f{};
  KrylovWork kw;
  DevStatus* st = nullptr;       // device
  DevStatus* st_host = nullptr;  // pinned
  int* d_geom_err = nullptr;
  double* red = nullptr;         // residual partials
  int red_parts = 0;
  int turb = 0, density = 0, cell_pref = 0;
  double urf[8], gravity[3];
  KspConf ksp[3];
  int nsolve = 0;                // solves issued in the current iteration
  int solve_sys[8] = {0};        // system of each solve of the current iteration
  std::vector<void*> allocs;
  std::map<std::string, std::pair<double*, long>> dfields;
  std::map<std::string, std::pair<int*, long>> ifields;
  // measurement
  long long launches_base = 0;   // g_launch_count at the last profile reset
  bool profiling = false;
  cudaEvent_t ev_iter[2] = {nullptr, nullptr};
  cudaEvent_t ev_solve[8][2] = {};
  cycas_profile prof{};
  bool iter_open = false;        // begin_iteration recorded ev_iter[0]
  AmgHostView amg;               // pressure preconditioner hierarchy (PC_AMG)
  std::vector<int> amg_sizes;  // rows per AMG level (fine to coarse)
  std::vector<int> amg_nnz;    // stored entries per AMG level
  std::vector<int> case_lo, case_hi;  // row ranges of the independent cases (one for a context)

  template <class T>
  T* alloc(long n) {
    void* p = nullptr;
    size_t bytes = sizeof(T) * (size_t)(n > 0 ? n : 1);
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) throw StatusError(CYCAS_ERR_ALLOC, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    allocs.push_back(p);
    CK(cudaMemsetAsync(p, 0, bytes, stream));
    return (T*)p;
  }
  template <class T>
  T* upload(const T* h, long n) {
    T* d = alloc<T>(n);
    if (n > 0 && h) CK(cudaMemcpyAsync(d, h, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, stream));
    return d;
  }
  double* dfield(const char* name, long n) {
    double* p = alloc<double>(n);
    dfields[name] = {p, n};
    return p;
  }
  ~cycas_ctx() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto& e : ev_iter)
      if (e) cudaEventDestroy(e);
    for (auto& pr : ev_solve)
      for (auto& e : pr)
        if (e) cudaEventDestroy(e);
    for (void* p : allocs) cudaFree(p);
    if (st_host) cudaFreeHost(st_host);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

const double kRefRtol[3] = {1.e-8, 1.e-6, 1.e-8};  // navier_velocity.cpp:28, navier_pressure.cpp:28, navier_scalar.cpp:98
const int kRefMaxit[3] = {1000, 1000, 500};

void require(bool ok, const std::string& msg) {
  if (!ok) throw StatusError(CYCAS_ERR_INVALID, msg);
}

// Host-side derived structure: gradient face order, CSR pattern and slots, boundary lists.
void build_device_mesh(cycas_ctx& c, const cycas_mesh_view& v) {
  const int n = v.ncel, nf = v.nfac, nb = v.nbnd;
  require(n > 0 && nf > 0 && nb >= 0, "empty mesh");
  require(v.face_cell1 && v.face_cell2 && v.face_bnd && v.cell_nface && v.cell_face && v.cell_cell && v.bnd_face &&
              v.bnd_type,
          "mesh view is missing topology arrays");
  DevMesh& m = c.m;
  m.ncel = n;
  m.nfac = nf;
  m.nbnd = nb;
  m.nvrt = v.nvrt;
  // validate topology (bounds) before anything reaches the device
  for (int i = 0; i < nf; i++) {
    int a = v.face_cell1[i], b = v.face_cell2[i];
    require(a >= 0 && a < n, "face_cell1 out of range at face " + std::to_string(i));
    require(b < n && (b >= 0 || b == -10), "face_cell2 must be a cell or -10 at face " + std::to_string(i));
    if (b < 0) require(v.face_bnd[i] >= 0 && v.face_bnd[i] < nb, "boundary face without boundary index");
  }
  for (int i = 0; i < nb; i++) {
    require(v.bnd_face[i] == i, "boundary faces must come first in boundary order (Bnd[i].face == i)");
    require(v.face_cell2[i] < 0, "boundary face has two cells");
    int t = v.bnd_type[i];
    require(t >= 1 && t <= 4, "boundary type must be wall/inlet/outlet/symmetry");
  }
  std::vector<int> gface(6 * (size_t)n, -1), face_sm(6 * (size_t)n, -1), slot(6 * (size_t)n, -1), diag(n);
  std::vector<int> rowptr(n + 1, 0), col;
  col.reserve((size_t)n * 7);
  std::vector<int> cols;
  for (int i = 0; i < n; i++) {
    int k = v.cell_nface[i];
    require(k >= 1 && k <= 6, "cell_nface out of range");
    int tmp[6];
    cols.clear();
    cols.push_back(i);
    for (int j = 0; j < k; j++) {
      int fid = v.cell_face[6 * (size_t)i + j];
      require(fid >= 0 && fid < nf, "cell_face out of range");
      require(v.face_cell1[fid] == i || v.face_cell2[fid] == i, "cell_face does not touch its cell");
      tmp[j] = fid;
      face_sm[(size_t)j * n + i] = fid;
      int nbh = v.face_cell2[fid] < 0 ? -1 : (v.face_cell1[fid] == i ? v.face_cell2[fid] : v.face_cell1[fid]);
      if (nbh >= 0) cols.push_back(nbh);
    }
    std::sort(tmp, tmp + k);
    for (int j = 0; j < k; j++) gface[(size_t)j * n + i] = tmp[j];
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    rowptr[i + 1] = rowptr[i] + (int)cols.size();
    int base = (int)col.size();
    for (int cc : cols) col.push_back(cc);
    for (int j = 0; j < k; j++) {
      int fid = tmp[0];
      fid = v.cell_face[6 * (size_t)i + j];
      int nbh = v.face_cell2[fid] < 0 ? -1 : (v.face_cell1[fid] == i ? v.face_cell2[fid] : v.face_cell1[fid]);
      if (nbh >= 0) slot[(size_t)j * n + i] = base + (int)(std::lower_bound(cols.begin(), cols.end(), nbh) - cols.begin());
    }
    diag[i] = base + (int)(std::lower_bound(cols.begin(), cols.end(), i) - cols.begin());
  }
  m.nnz = (int)col.size();
  // boundary lists in boundary order
  std::vector<int> inl, outl, sym;
  std::vector<std::vector<int>> wall_of_cell;
  std::vector<int> wcell;
  std::map<int, int> wc_index;
  for (int i = 0; i < nb; i++) {
    int t = v.bnd_type[i];
    if (t == 2) inl.push_back(i);
    else if (t == 3) outl.push_back(i);
    else if (t == 4) sym.push_back(i);
  }
  std::vector<int> wfirst(n, -1);
  std::vector<int> wcount(n, 0);
  for (int i = 0; i < nb; i++)
    if (v.bnd_type[i] == 1) wcount[v.face_cell1[v.bnd_face[i]]]++;
  std::vector<int> wc_cell, wc_start(1, 0), wc_bnd;
  std::vector<int> wpos(n, -1);
  for (int c2 = 0; c2 < n; c2++)
    if (wcount[c2] > 0) {
      wpos[c2] = (int)wc_cell.size();
      wc_cell.push_back(c2);
      wc_start.push_back(wc_start.back() + wcount[c2]);
    }
  wc_bnd.assign(wc_start.back(), 0);
  std::vector<int> fill(wc_cell.size(), 0);
  for (int i = 0; i < nb; i++)
    if (v.bnd_type[i] == 1) {
      int cc = v.face_cell1[v.bnd_face[i]];
      int w = wpos[cc];
      wc_bnd[wc_start[w] + fill[w]++] = i;
    }

  m.f_c1 = c.upload(v.face_cell1, nf);
  m.f_c2 = c.upload(v.face_cell2, nf);
  m.f_bnd = c.upload(v.face_bnd, nf);
  m.c_nface = c.upload(v.cell_nface, n);
  m.c_face = c.upload(face_sm.data(), 6L * n);
  m.c_gface = c.upload(gface.data(), 6L * n);
  m.c_slot = c.upload(slot.data(), 6L * n);
  m.c_diag = c.upload(diag.data(), n);
  m.b_face = c.upload(v.bnd_face, nb);
  m.b_type = c.upload(v.bnd_type, nb);
  m.rowptr = c.upload(rowptr.data(), n + 1);
  m.col = c.upload(col.data(), m.nnz);
  m.n_inlet = (int)inl.size();
  m.n_outlet = (int)outl.size();
  m.n_sym = (int)sym.size();
  m.inlet_list = c.upload(inl.data(), m.n_inlet);
  m.outlet_list = c.upload(outl.data(), m.n_outlet);
  m.sym_list = c.upload(sym.data(), m.n_sym);
  m.n_wallcell = (int)wc_cell.size();
  m.wc_cell = c.upload(wc_cell.data(), m.n_wallcell);
  m.wc_start = c.upload(wc_start.data(), m.n_wallcell + 1);
  m.wc_bnd = c.upload(wc_bnd.data(), (long)wc_bnd.size());
  c.ifields["A_rowptr"] = {m.rowptr, n + 1L};
  c.ifields["A_col"] = {m.col, (long)m.nnz};

  // geometry
  m.f_x = c.dfield("face_x", 3L * nf);
  m.f_n = c.dfield("face_n", 3L * nf);
  m.f_area = c.dfield("face_area", nf);
  m.f_lambda = c.dfield("face_lambda", nf);
  m.f_rlencos = c.dfield("face_rlencos", nf);
  m.f_xpac = c.dfield("face_xpac", 3L * nf);
  m.f_xnac = c.dfield("face_xnac", 3L * nf);
  m.c_vol = c.dfield("cell_vol", n);
  m.c_x = c.dfield("cell_x", 3L * n);
  m.b_dist = c.dfield("bnd_distance", nb);
  if (v.face_x) {
    require(v.face_n && v.face_area && v.face_lambda && v.face_rlencos && v.face_xpac && v.face_xnac && v.cell_vol &&
                v.cell_x && v.bnd_distance,
            "partial geometry in mesh view");
    auto put = [&](double* d, const double* h, long cnt) {
      CK(cudaMemcpyAsync(d, h, sizeof(double) * cnt, cudaMemcpyHostToDevice, c.stream));
    };
    put(m.f_x, v.face_x, 3L * nf);
    put(m.f_n, v.face_n, 3L * nf);
    put(m.f_area, v.face_area, nf);
    put(m.f_lambda, v.face_lambda, nf);
    put(m.f_rlencos, v.face_rlencos, nf);
    put(m.f_xpac, v.face_xpac, 3L * nf);
    put(m.f_xnac, v.face_xnac, 3L * nf);
    put(m.c_vol, v.cell_vol, n);
    put(m.c_x, v.cell_x, 3L * n);
    put(m.b_dist, v.bnd_distance, nb);
  } else {
    require(v.vert && v.face_vertices && v.cell_vertices && v.nvrt > 0, "geometry or vertices required");
    for (long i = 0; i < 4L * nf; i++) require(v.face_vertices[i] >= 0 && v.face_vertices[i] < v.nvrt, "face vertex out of range");
    for (long i = 0; i < 8L * n; i++) require(v.cell_vertices[i] >= 0 && v.cell_vertices[i] < v.nvrt, "cell vertex out of range");
    m.vert = c.upload(v.vert, 3L * v.nvrt);
    m.f_vert = c.upload(v.face_vertices, 4L * nf);
    m.c_vert = c.upload(v.cell_vertices, 8L * n);
    launch_geometry(m, c.d_geom_err, c.stream);
    CK(cudaGetLastError());
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, c.d_geom_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (herr & 2) throw StatusError(CYCAS_ERR_MESH, "mesh rejected: face area check or negative wall distance");
  }
}

void alloc_fields(cycas_ctx& c) {
  const long n = c.m.ncel, nf = c.m.nfac, nb = c.m.nbnd, nnz = c.m.nnz;
  DevFields& f = c.f;
  f.U = c.dfield("U", n);
  f.V = c.dfield("V", n);
  f.W = c.dfield("W", n);
  f.P = c.dfield("P", n);
  f.R = c.dfield("R", n);
  f.T = c.dfield("T", n);
  f.TE = c.dfield("TE", n);
  f.ED = c.dfield("ED", n);
  f.dp = c.dfield("deltaP", n);
  f.VisLam = c.dfield("VisLam", n);
  f.VisTur = c.dfield("VisTur", n);
  f.Apr = c.dfield("Apr", n);
  f.RUFace = c.dfield("RUFace", nf);
  f.BRo = c.dfield("BRo", nb);
  f.BU = c.dfield("BU", nb);
  f.BV = c.dfield("BV", nb);
  f.BW = c.dfield("BW", nb);
  f.BPre = c.dfield("BPre", nb);
  f.BTE = c.dfield("BTE", nb);
  f.BED = c.dfield("BED", nb);
  f.BTem = c.dfield("BTem", nb);
  f.dUdX = c.dfield("dUdX", 3 * n);
  f.dVdX = c.dfield("dVdX", 3 * n);
  f.dWdX = c.dfield("dWdX", 3 * n);
  f.dPdX = c.dfield("dPdX", 3 * n);
  f.dPhidX = c.dfield("dPhidX", 3 * n);
  f.shear = c.dfield("bnd_shear", 3 * nb);
  f.old = c.dfield("old_uvw", 3 * n);
  f.Prod = c.dfield("Prod", n);
  f.TES = c.dfield("TESource", n);
  f.EDS = c.dfield("EDSource", n);
  f.ApTE = c.dfield("ApTE", n);
  f.ApED = c.dfield("ApED", n);
  f.VisTE = c.dfield("VisTE", n);
  f.VisED = c.dfield("VisED", n);
  f.Au = c.dfield("Au_val", nnz);
  f.Ap = c.dfield("Ap_val", nnz);
  f.As = c.dfield("As_val", nnz);
  f.bu = c.dfield("bu", n);
  f.bv = c.dfield("bv", n);
  f.bw = c.dfield("bw", n);
  f.bp = c.dfield("bp", n);
  f.bs = c.dfield("bs", n);
  f.dinv_u = c.dfield("dinv_u", n);
  f.dinv_p = c.dfield("dinv_p", n);
  f.dinv_s = c.dfield("dinv_s", n);
}

void alloc_krylov(cycas_ctx& c) {
  int maxm = 3;  // CG needs four work vectors
  for (int s = 0; s < 3; s++) maxm = std::max(maxm, c.ksp[s].restart);
  require(maxm <= kMaxRestart, "GMRES restart above " + std::to_string(kMaxRestart));
  KrylovWork& w = c.kw;
  w.m = maxm;
  w.ldv = ((long)c.m.ncel + 31) / 32 * 32;
  w.v_len = 3L * (maxm + 1) * w.ldv;  // three momentum systems in lockstep
  w.V = c.alloc<double>(w.v_len);
  w.nblocks = gmres_max_blocks(c.device);
  // per CTA and per lockstep system (up to the three momentum components)
  w.part_len = 3L * w.nblocks * kGmresPartStride;
  w.part = c.alloc<double>(w.part_len);
  w.bar = c.alloc<unsigned>(2);
  c.red_parts = std::min(residual_blocks(c.m.ncel), 1024);
  int cells_blocks = (c.m.ncel + 255) / 256;
  c.red = c.alloc<double>(3L * std::max(c.red_parts, cells_blocks));
}

// Aggregation hierarchy of the pressure system.  Strength of a connection = the face
// coefficient area/|d.n| (Face.rlencos) of the face joining the two cells.
void setup_amg(cycas_ctx& c) {
  const int n = c.m.ncel, nf = c.m.nfac, nnz = c.m.nnz;
  std::vector<double> rl(nf);
  std::vector<int> rowptr(n + 1), col(nnz), slot(6L * n), faces(6L * n), nface(n);
  CK(cudaMemcpyAsync(rl.data(), c.m.f_rlencos, sizeof(double) * nf, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(rowptr.data(), c.m.rowptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(col.data(), c.m.col, sizeof(int) * nnz, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(slot.data(), c.m.c_slot, sizeof(int) * 6L * n, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(faces.data(), c.m.c_face, sizeof(int) * 6L * n, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(nface.data(), c.m.c_nface, sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  std::vector<double> w(nnz, 0.0);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < nface[i]; j++) {
      int s = slot[(size_t)j * n + i];
      if (s >= 0) w[s] = rl[faces[(size_t)j * n + i]];
    }
  struct Up : AmgUploader {
    cycas_ctx& c;
    explicit Up(cycas_ctx& cc) : c(cc) {}
    const int* upload_int(const int* h, long n) override { return c.upload(h, n); }
    float* alloc_float(long n) override { return c.alloc<float>(n); }
    void* upload_bytes(const void* h, long bytes) override { return c.upload((const unsigned char*)h, bytes); }
  } up(c);
  amg_setup_cases(c.amg, n, rowptr.data(), col.data(), w.data(), c.m.rowptr, c.m.col, c.m.c_diag, c.f.Ap,
                  c.case_lo, c.case_hi, up);
  c.amg_sizes = c.amg.rows0;
  c.amg_nnz = c.amg.nnz0;
}

void init_ctx(cycas_ctx& c, const cycas_params* p, const cycas_options* o) {
  cycas_options def;
  cycas_options_default(&def);
  if (!o) o = &def;
  c.device = o->device;
  CK(cudaSetDevice(c.device));
  CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  require(p->density_model == 0, "only constant density (DensityModel 0) is on this path");
  require(p->turb_model == 0 || p->turb_model == 1, "TurModel must be 0 or 1");
  c.turb = p->turb_model;
  c.density = p->density_model;
  c.cell_pref = p->cell_pressure_ref;
  for (int i = 0; i < 8; i++) c.urf[i] = p->urf[i];
  for (int i = 0; i < 3; i++) c.gravity[i] = p->gravity[i];
  for (int s = 0; s < 3; s++) {
    const cycas_ksp_options& k = o->ksp[s];
    require(k.pc == CYCAS_PC_NONE || k.pc == CYCAS_PC_JACOBI || k.pc == CYCAS_PC_AMG,
            "preconditioner not available in this build");
    require(k.restart >= 1 && k.restart <= kMaxRestart, "restart out of range");
    require(k.type >= CYCAS_KSP_DEFAULT && k.type <= CYCAS_KSP_CG, "unknown Krylov type");
    c.ksp[s].type = k.type != CYCAS_KSP_DEFAULT ? k.type : (s == CYCAS_SYS_PRESSURE ? CYCAS_KSP_CG : CYCAS_KSP_GMRES);
    require(k.pc != CYCAS_PC_AMG || (s == CYCAS_SYS_PRESSURE && c.ksp[s].type == CYCAS_KSP_CG),
            "the AMG preconditioner is for the pressure system with CG");
    c.ksp[s].restart = k.restart;
    c.ksp[s].pc = k.pc;
    c.ksp[s].rtol = k.rtol > 0 ? k.rtol : kRefRtol[s];
    c.ksp[s].maxit = k.maxit > 0 ? k.maxit : kRefMaxit[s];
  }
  c.d_geom_err = c.alloc<int>(1);
  c.st = c.alloc<DevStatus>(1);
  CK(cudaMallocHost((void**)&c.st_host, sizeof(DevStatus)));
  std::memset(c.st_host, 0, sizeof(DevStatus));
}

// ---------------------------------------------------------------- iteration schedule
void solve(cycas_ctx& c, int sys, const double* val, const double* dinv, const double* b, double* x, bool guess_zero) {
  require(c.nsolve < 8, "too many solves in one iteration");
  const KspConf& k = c.ksp[sys];
  GmresCall g;
  g.n = c.m.ncel;
  g.rowptr = c.m.rowptr;
  g.col = c.m.col;
  g.val = val;
  g.dinv = k.pc == CYCAS_PC_JACOBI ? dinv : nullptr;
  g.b = b;
  g.x = x;
  g.guess_zero = guess_zero ? 1 : 0;
  g.rtol = k.rtol;
  g.maxit = k.maxit;
  g.restart = k.restart;
  int slot = c.nsolve++;
  c.solve_sys[slot] = sys;
  g.out = &c.st->ksp[slot];
  g.err = &c.st->err;
  CK(cudaMemsetAsync(c.kw.bar, 0, 2 * sizeof(unsigned), c.stream));
  if (c.profiling) CK(cudaEventRecord(c.ev_solve[slot][0], c.stream));
  if (k.pc == CYCAS_PC_AMG) {
    launch_amg_setup_values(c.amg, c.stream);
    CK(launch_cg_amg(g, c.amg, c.kw, nullptr, gmres_grid(g.n, c.kw.nblocks), g.out, c.stream));
  } else if (k.type == CYCAS_KSP_CG) {
    CK(launch_cg(g, c.kw, c.stream));
  } else {
    CK(launch_gmres(g, c.kw, c.stream));
  }
  if (c.profiling) CK(cudaEventRecord(c.ev_solve[slot][1], c.stream));
  ++g_launch_count;
  c.prof.krylov_launches[sys]++;
}

// solveVelocity_GMRES (MPIStructure.cpp:234-375): one operator, three right-hand sides, run in
// lockstep by one persistent launch (each system keeps its own GMRES state)
void solve_velocity(cycas_ctx& c) {
  require(c.nsolve + 3 <= 8, "too many solves in one iteration");
  const KspConf& k = c.ksp[CYCAS_SYS_VELOCITY];
  if (k.type == CYCAS_KSP_CG || k.pc == CYCAS_PC_AMG) {  // non-default methods: one solve at a time
    solve(c, CYCAS_SYS_VELOCITY, c.f.Au, c.f.dinv_u, c.f.bu, c.f.U, false);
    solve(c, CYCAS_SYS_VELOCITY, c.f.Au, c.f.dinv_u, c.f.bv, c.f.V, false);
    solve(c, CYCAS_SYS_VELOCITY, c.f.Au, c.f.dinv_u, c.f.bw, c.f.W, false);
    return;
  }
  GmresCall g[3];
  const double* bs[3] = {c.f.bu, c.f.bv, c.f.bw};
  double* xs[3] = {c.f.U, c.f.V, c.f.W};
  const int slot0 = c.nsolve;
  for (int q = 0; q < 3; q++) {
    g[q].n = c.m.ncel;
    g[q].rowptr = c.m.rowptr;
    g[q].col = c.m.col;
    g[q].val = c.f.Au;
    g[q].dinv = k.pc == CYCAS_PC_JACOBI ? c.f.dinv_u : nullptr;
    g[q].b = bs[q];
    g[q].x = xs[q];
    g[q].guess_zero = 0;
    g[q].rtol = k.rtol;
    g[q].maxit = k.maxit;
    g[q].restart = k.restart;
    int slot = c.nsolve++;
    c.solve_sys[slot] = CYCAS_SYS_VELOCITY;
    g[q].out = &c.st->ksp[slot];
    g[q].err = &c.st->err;
  }
  CK(cudaMemsetAsync(c.kw.bar, 0, 2 * sizeof(unsigned), c.stream));
  if (c.profiling) CK(cudaEventRecord(c.ev_solve[slot0][0], c.stream));
  CK(launch_gmres_multi(g, 3, c.kw, c.stream));
  if (c.profiling) {
    CK(cudaEventRecord(c.ev_solve[slot0][1], c.stream));
    // the two other slots share the launch: zero-length intervals
    for (int q = 1; q < 3; q++) {
      CK(cudaEventRecord(c.ev_solve[slot0 + q][0], c.stream));
      CK(cudaEventRecord(c.ev_solve[slot0 + q][1], c.stream));
    }
  }
  ++g_launch_count;
  c.prof.krylov_launches[CYCAS_SYS_VELOCITY]++;
}

void bc_velocity(cycas_ctx& c, bool with_pressure) {
  launch_bc_velocity(c.m, c.f, c.density, with_pressure, c.stream);
}

void grad_uvwp(cycas_ctx& c) {
  const double* phi[4] = {c.f.U, c.f.V, c.f.W, c.f.P};
  const double* bphi[4] = {c.f.BU, c.f.BV, c.f.BW, c.f.BPre};
  double* g[4] = {c.f.dUdX, c.f.dVdX, c.f.dWdX, c.f.dPdX};
  launch_gradient(c.m, 4, phi, bphi, g, c.stream);
}

void grad1(cycas_ctx& c, const double* phi, const double* bphi, double* g) {
  launch_gradient(c.m, 1, &phi, &bphi, &g, c.stream);
}

// BuildVelocityMatrix (navier_velocity.cpp:63-393)
void build_velocity(cycas_ctx& c) {
  bc_velocity(c, true);
  grad_uvwp(c);
  launch_momentum(c.m, c.f, c.urf, c.gravity, c.st, c.stream);
}

// CalculateVelocity (navier_velocity.cpp:10-60)
void calculate_velocity(cycas_ctx& c) {
  build_velocity(c);
  solve_velocity(c);
  launch_residual_uvw(c.m, c.f, c.red, c.st, c.stream);
}

void correct_cells(cycas_ctx& c) {
  launch_correct_cells(c.m, c.f, c.cell_pref, c.urf[3], c.red, c.stream);
  launch_finalize_residual(c.red, (c.m.ncel + 255) / 256, 3, c.st, c.stream);
}

// CalculatePressure (navier_pressure.cpp:9-97)
void calculate_pressure(cycas_ctx& c) {
  bc_velocity(c, false);
  launch_ruface2(c.m, c.f, c.stream);
  launch_pressure(c.m, c.f, c.stream);
  solve(c, CYCAS_SYS_PRESSURE, c.f.Ap, c.f.dinv_p, c.f.bp, c.f.dp, true);
  launch_bc_deltap(c.m, c.f, c.stream);
  grad1(c, c.f.dp, c.f.BPre, c.f.dPdX);
  correct_cells(c);
  bc_velocity(c, false);
  launch_correct_ruface(c.m, c.f, c.urf[3], c.stream);
}

// UpdateTurKEpsilon (navier_scalar.cpp:11-197)
void update_keps(cycas_ctx& c) {
  launch_keps_sources(c.m, c.f, c.stream);
  launch_keps_wall(c.m, c.f, c.stream);
  grad1(c, c.f.TE, c.f.BTE, c.f.dPhidX);
  launch_scalar(c.m, c.f, c.f.TE, c.f.BTE, c.f.VisTE, c.f.TES, c.f.ApTE, c.urf[5], c.st, c.stream);
  solve(c, CYCAS_SYS_SCALAR, c.f.As, c.f.dinv_s, c.f.bs, c.f.TE, false);
  launch_clip_te(c.m, c.f, c.stream);
  grad1(c, c.f.ED, c.f.BED, c.f.dPhidX);
  launch_scalar(c.m, c.f, c.f.ED, c.f.BED, c.f.VisED, c.f.EDS, c.f.ApED, c.urf[5], c.st, c.stream);
  launch_eps_wall_rows(c.m, c.f, c.stream);
  solve(c, CYCAS_SYS_SCALAR, c.f.As, c.f.dinv_s, c.f.bs, c.f.ED, false);
  launch_finish_keps(c.m, c.f, c.stream);
}

void begin_iteration(cycas_ctx& c) {
  CK(cudaMemsetAsync(c.st, 0, sizeof(DevStatus), c.stream));
  c.nsolve = 0;
  c.iter_open = true;
  if (c.profiling) CK(cudaEventRecord(c.ev_iter[0], c.stream));
}

void issue_iteration(cycas_ctx& c) {
  calculate_velocity(c);
  calculate_pressure(c);
  if (c.turb == 1) update_keps(c);
}

// reads the status block; returns the C status of the iteration
int finish_iteration(cycas_ctx& c, double* residual, double* resmax, cycas_iter_stats* stats) {
  CK(cudaGetLastError());
  const bool timed = c.profiling && c.iter_open;
  c.iter_open = false;
  if (timed) CK(cudaEventRecord(c.ev_iter[1], c.stream));
  CK(cudaMemcpyAsync(c.st_host, c.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  const DevStatus& s = *c.st_host;
  for (int k = 0; k < c.nsolve; k++) c.prof.krylov_iters[c.solve_sys[k]] += s.ksp[k].its;
  if (timed) {
    float total = 0.f, ksum = 0.f;
    CK(cudaEventElapsedTime(&total, c.ev_iter[0], c.ev_iter[1]));
    for (int k = 0; k < c.nsolve; k++) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, c.ev_solve[k][0], c.ev_solve[k][1]));
      c.prof.krylov_ms[c.solve_sys[k]] += ms;
      ksum += ms;
    }
    c.prof.assembly_ms += total - ksum;
  }
  double mx = 0.0;
  for (int i = 0; i < 10; i++) {
    if (residual) residual[i] = s.localRes[i];
    mx = mx > s.localRes[i] ? mx : s.localRes[i];  // vec_max (tools.cpp:45-51)
  }
  if (resmax) *resmax = mx;
  int failed = -1, nan = 0;
  for (int k = 0; k < c.nsolve; k++) {
    if (s.ksp[k].reason < 0 && failed < 0) failed = k;
    if (s.ksp[k].reason == CYCAS_KSP_DIVERGED_NANORINF) nan = 1;
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    for (int k = 0; k < 8; k++) {
      stats->its[k] = k < c.nsolve ? s.ksp[k].its : -1;
      stats->reason[k] = k < c.nsolve ? s.ksp[k].reason : 0;
      stats->rnorm[k] = k < c.nsolve ? s.ksp[k].rnorm : 0.0;
    }
    stats->nsolves = c.nsolve;
    stats->failed_solve = failed;
  }
  if (s.err & 1) {
    g_last_error = "a device-side grid barrier timed out; the solve was abandoned";
    return CYCAS_ERR_TIMEOUT;
  }
  if (s.err & 4) {
    g_last_error = "reverse flow get out of inlet (scalar transport); the reference stops here";
    return CYCAS_ERR_INVALID;
  }
  if (nan) {
    g_last_error = "NaN or Inf residual norm in a Krylov solve";
    return CYCAS_NAN_DETECTED;
  }
  if (failed >= 0) {
    g_last_error = "Krylov solve " + std::to_string(failed) + " did not converge (reason " +
                   std::to_string(s.ksp[failed].reason) + ", " + std::to_string(s.ksp[failed].its) + " iterations)";
    return CYCAS_NOT_CONVERGED;
  }
  return CYCAS_OK;
}

std::pair<double*, long> lookup(cycas_ctx& c, const char* name) {
  auto it = c.dfields.find(name);
  if (it == c.dfields.end()) throw StatusError(CYCAS_ERR_INVALID, std::string("unknown field ") + name);
  return it->second;
}

cycas_mesh_view view_of(const HostCase& hc) {
  cycas_mesh_view v;
  std::memset(&v, 0, sizeof v);
  v.ncel = hc.ncel;
  v.nfac = hc.nfac;
  v.nbnd = hc.nbnd;
  v.nvrt = hc.nvrt;
  v.face_cell1 = hc.face_cell1.data();
  v.face_cell2 = hc.face_cell2.data();
  v.face_bnd = hc.face_bnd.data();
  v.face_vertices = hc.face_vertices.data();
  v.cell_nface = hc.cell_nface.data();
  v.cell_face = hc.cell_face.data();
  v.cell_cell = hc.cell_cell.data();
  v.cell_vertices = hc.cell_vertices.data();
  v.bnd_face = hc.bnd_face.data();
  v.bnd_type = hc.bnd_type.data();
  v.vert = hc.vert.data();
  return v;
}

void set_field(cycas_ctx& c, const char* name, const double* src, long n) {
  auto p = lookup(c, name);
  require(p.second == n, std::string("size mismatch for ") + name);
  CK(cudaMemcpyAsync(p.first, src, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
}

}  // namespace

// ==================================================================== C ABI
extern "C" {

const char* cycas_last_error(void) { return g_last_error.c_str(); }

void cycas_options_default(cycas_options* o) {
  std::memset(o, 0, sizeof(*o));
  for (int s = 0; s < 3; s++) {
    o->ksp[s].type = CYCAS_KSP_DEFAULT;
    o->ksp[s].restart = 30;
    o->ksp[s].pc = CYCAS_PC_JACOBI;
    o->ksp[s].rtol = 0.0;
    o->ksp[s].maxit = 0;
  }
  o->device = 0;
}

int cycas_case_load(const char* param_path, cycas_case** out) {
  return guard([&]() -> int {
    require(param_path && out, "null argument");
    *out = nullptr;
    cycas_case* c = new cycas_case();
    try {
      load_case(c->hc, param_path);
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
    return CYCAS_OK;
  });
}

void cycas_case_free(cycas_case* c) { delete c; }

int cycas_case_dims(const cycas_case* c, int64_t d[8]) {
  return guard([&]() -> int {
    require(c && d, "null argument");
    const HostCase& h = c->hc;
    long nnz = h.ncel;
    for (int i = 0; i < h.ncel; i++)
      for (int j = 0; j < h.cell_nface[i]; j++)
        if (h.cell_cell[6 * (size_t)i + j] >= 0) nnz++;
    d[0] = h.ncel;
    d[1] = h.nfac;
    d[2] = h.nbnd;
    d[3] = h.nvrt;
    d[4] = h.turb_model;
    d[5] = h.max_step;
    d[6] = h.cell_pressure_ref;
    d[7] = nnz;
    return CYCAS_OK;
  });
}

int cycas_case_params(const cycas_case* c, double* residual_steady, double urf[8], double gravity[3]) {
  return guard([&]() -> int {
    require(c != nullptr, "null case");
    if (residual_steady) *residual_steady = c->hc.residual_steady;
    if (urf)
      for (int i = 0; i < 8; i++) urf[i] = c->hc.urf[i];
    if (gravity)
      for (int i = 0; i < 3; i++) gravity[i] = c->hc.gravity[i];
    return CYCAS_OK;
  });
}

int cycas_case_get_int(const cycas_case* c, const char* name, int32_t* dst, int64_t n) {
  return guard([&]() -> int {
    require(c && name && dst, "null argument");
    const HostCase& h = c->hc;
    std::string s(name);
    const std::vector<int32_t>* v = nullptr;
    if (s == "face_cell1") v = &h.face_cell1;
    else if (s == "face_cell2") v = &h.face_cell2;
    else if (s == "face_bnd") v = &h.face_bnd;
    else if (s == "face_vertices") v = &h.face_vertices;
    else if (s == "cell_nface") v = &h.cell_nface;
    else if (s == "cell_face") v = &h.cell_face;
    else if (s == "cell_cell") v = &h.cell_cell;
    else if (s == "cell_vertices") v = &h.cell_vertices;
    else if (s == "cell_rid") v = &h.cell_rid;
    else if (s == "bnd_face") v = &h.bnd_face;
    else if (s == "bnd_rid") v = &h.bnd_rid;
    else if (s == "bnd_type") v = &h.bnd_type;
    else if (s == "bnd_vertices") v = &h.bnd_vertices;
    require(v != nullptr, "unknown case array " + s);
    require((int64_t)v->size() == n, "size mismatch for " + s);
    std::memcpy(dst, v->data(), sizeof(int32_t) * (size_t)n);
    return CYCAS_OK;
  });
}

int cycas_create(const cycas_mesh_view* mesh, const cycas_params* params, const cycas_options* opt,
                 cycas_ctx** out) {
  return guard([&]() -> int {
    require(mesh && params && out, "null argument");
    *out = nullptr;
    cycas_ctx* c = new cycas_ctx();
    try {
      init_ctx(*c, params, opt);
      build_device_mesh(*c, *mesh);
      alloc_fields(*c);
      alloc_krylov(*c);
      c->case_lo = {0};
      c->case_hi = {c->m.ncel};
      if (c->ksp[CYCAS_SYS_PRESSURE].pc == CYCAS_PC_AMG) setup_amg(*c);
      CK(cudaStreamSynchronize(c->stream));
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
    return CYCAS_OK;
  });
}

int cycas_create_from_case(const cycas_case* cs, const cycas_options* opt, cycas_ctx** out) {
  return guard([&]() -> int {
    require(cs && out, "null argument");
    const HostCase& h = cs->hc;
    cycas_mesh_view v = view_of(h);
    cycas_params p;
    std::memset(&p, 0, sizeof p);
    p.turb_model = h.turb_model;
    p.density_model = h.density_model;
    p.cell_pressure_ref = h.cell_pressure_ref;
    for (int i = 0; i < 8; i++) p.urf[i] = h.urf[i];
    for (int i = 0; i < 3; i++) p.gravity[i] = h.gravity[i];
    require(h.cell_pressure_ref >= 0 && h.cell_pressure_ref < h.ncel, "PressureRef cell out of range");
    int rc = cycas_create(&v, &p, opt, out);
    if (rc != CYCAS_OK) return rc;
    cycas_ctx* c = *out;
    try {
      const long n = h.ncel, nb = h.nbnd;
      set_field(*c, "U", h.U.data(), n);
      set_field(*c, "V", h.V.data(), n);
      set_field(*c, "W", h.W.data(), n);
      set_field(*c, "P", h.P.data(), n);
      set_field(*c, "R", h.R.data(), n);
      set_field(*c, "T", h.T.data(), n);
      set_field(*c, "VisLam", h.VisLam.data(), n);
      set_field(*c, "VisTur", h.VisTur.data(), n);
      set_field(*c, "TE", h.TE.data(), n);
      set_field(*c, "ED", h.ED.data(), n);
      set_field(*c, "BU", h.BU.data(), nb);
      set_field(*c, "BV", h.BV.data(), nb);
      set_field(*c, "BW", h.BW.data(), nb);
      set_field(*c, "BRo", h.BRo.data(), nb);
      set_field(*c, "BTem", h.BTem.data(), nb);
      set_field(*c, "BTE", h.BTE.data(), nb);
      set_field(*c, "BED", h.BED.data(), nb);
      CK(cudaStreamSynchronize(c->stream));
    } catch (...) {
      cycas_destroy(c);
      *out = nullptr;
      throw;
    }
    return CYCAS_OK;
  });
}

void cycas_destroy(cycas_ctx* ctx) { delete ctx; }

int cycas_get_field(cycas_ctx* c, const char* name, double* dst, int64_t n) {
  return guard([&]() -> int {
    require(c && name && dst, "null argument");
    auto p = lookup(*c, name);
    require(p.second == n, std::string("size mismatch for ") + name);
    CK(cudaMemcpyAsync(dst, p.first, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CYCAS_OK;
  });
}

int cycas_set_field(cycas_ctx* c, const char* name, const double* src, int64_t n) {
  return guard([&]() -> int {
    require(c && name && src, "null argument");
    set_field(*c, name, src, n);
    CK(cudaStreamSynchronize(c->stream));
    return CYCAS_OK;
  });
}

int cycas_get_int(cycas_ctx* c, const char* name, int32_t* dst, int64_t n) {
  return guard([&]() -> int {
    require(c && name && dst, "null argument");
    auto it = c->ifields.find(name);
    require(it != c->ifields.end(), std::string("unknown int array ") + name);
    require(it->second.second == n, std::string("size mismatch for ") + name);
    CK(cudaMemcpyAsync(dst, it->second.first, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CYCAS_OK;
  });
}

int cycas_simple_iteration(cycas_ctx* c, double residual[10], double* resmax, cycas_iter_stats* stats) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    begin_iteration(*c);
    issue_iteration(*c);
    return finish_iteration(*c, residual, resmax, stats);
  });
}

int cycas_simple_iterations(cycas_ctx* c, int32_t n, double* res_hist, double* resmax, int32_t* its,
                            int32_t* reasons) {
  return guard([&]() -> int {
    require(c != nullptr && n >= 0, "bad argument");
    for (int s = 0; s < n; s++) {
      cycas_iter_stats st;
      double res[10], rm;
      begin_iteration(*c);
      issue_iteration(*c);
      int rc = finish_iteration(*c, res, &rm, &st);
      if (res_hist) std::memcpy(res_hist + 10L * s, res, sizeof res);
      if (resmax) resmax[s] = rm;
      for (int k = 0; k < 8; k++) {
        if (its) its[8L * s + k] = st.its[k];
        if (reasons) reasons[8L * s + k] = st.reason[k];
      }
      if (rc != CYCAS_OK) return rc;
    }
    return CYCAS_OK;
  });
}

int cycas_run_stage(cycas_ctx* c, const char* stage) {
  return guard([&]() -> int {
    require(c && stage, "null argument");
    std::string s(stage);
    cycas_ctx& x = *c;
    if (s == "clear_residual") {
      begin_iteration(x);
      CK(cudaStreamSynchronize(x.stream));
      return CYCAS_OK;
    }
    x.nsolve = 0;  // solve reports of this stage start at slot 0
    if (s == "bc_velocity") bc_velocity(x, false);
    else if (s == "bc_pressure") bc_velocity(x, true);
    else if (s == "bc_deltap") launch_bc_deltap(x.m, x.f, x.stream);
    else if (s == "grad_uvwp") grad_uvwp(x);
    else if (s == "grad_deltap") grad1(x, x.f.dp, x.f.BPre, x.f.dPdX);
    else if (s == "build_velocity") build_velocity(x);
    else if (s == "ruface2") launch_ruface2(x.m, x.f, x.stream);
    else if (s == "build_pressure") launch_pressure(x.m, x.f, x.stream);
    else if (s == "correct_cells") correct_cells(x);
    else if (s == "correct_ruface") launch_correct_ruface(x.m, x.f, x.urf[3], x.stream);
    else if (s == "calculate_velocity") calculate_velocity(x);
    else if (s == "calculate_pressure") calculate_pressure(x);
    else if (s == "keps") update_keps(x);
    else throw StatusError(CYCAS_ERR_INVALID, "unknown stage " + s);
    return finish_iteration(x, nullptr, nullptr, nullptr);
  });
}

int cycas_get_stream(cycas_ctx* c, void** stream) {
  return guard([&]() -> int {
    require(c && stream, "null argument");
    *stream = (void*)c->stream;
    return CYCAS_OK;
  });
}

int cycas_set_profiling(cycas_ctx* c, int32_t on) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    if (on && !c->ev_iter[0]) {
      for (auto& e : c->ev_iter) CK(cudaEventCreate(&e));
      for (auto& pr : c->ev_solve)
        for (auto& e : pr) CK(cudaEventCreate(&e));
    }
    c->profiling = on != 0;
    return CYCAS_OK;
  });
}

int cycas_get_amg_levels(cycas_ctx* c, int32_t max_levels, int32_t* nlev, int32_t* rows, int32_t* nnz) {
  return guard([&]() -> int {
    require(c && nlev, "null argument");
    int L = (int)c->amg_sizes.size();
    *nlev = L;
    for (int l = 0; l < L && l < max_levels; l++) {
      if (rows) rows[l] = c->amg_sizes[l];
      if (nnz) nnz[l] = c->amg_nnz[l];
    }
    return CYCAS_OK;
  });
}

int cycas_reset_profile(cycas_ctx* c) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    std::memset(&c->prof, 0, sizeof c->prof);
    c->launches_base = g_launch_count;
    return CYCAS_OK;
  });
}

int cycas_get_profile(cycas_ctx* c, cycas_profile* out) {
  return guard([&]() -> int {
    require(c && out, "null argument");
    *out = c->prof;
    out->kernel_launches = g_launch_count - c->launches_base;
    return CYCAS_OK;
  });
}

int cycas_csr_solve(int32_t n, const int32_t* rowptr, const int32_t* col, const double* val, const double* b,
                    double* x, const cycas_ksp_options* ksp, double rtol, int32_t maxit, int32_t guess_zero,
                    cycas_solve_stats* stats) {
  return guard([&]() -> int {
    require(n > 0 && rowptr && col && val && b && x && ksp, "bad argument");
    require(ksp->restart >= 1 && ksp->restart <= kMaxRestart, "restart out of range");
    require(ksp->pc == CYCAS_PC_NONE || ksp->pc == CYCAS_PC_JACOBI, "preconditioner not available in this build");
    require(ksp->type >= CYCAS_KSP_DEFAULT && ksp->type <= CYCAS_KSP_CG, "unknown Krylov type");
    int nnz = rowptr[n];
    require(rowptr[0] == 0 && nnz >= 0, "bad rowptr");
    std::vector<double> dinv(n, 0.0);
    for (int i = 0; i < n; i++) {
      require(rowptr[i + 1] >= rowptr[i], "rowptr not monotone");
      double d = 0.0;
      for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
        require(col[k] >= 0 && col[k] < n, "column out of range");
        if (col[k] == i) d = val[k];
      }
      dinv[i] = 1.0 / d;
    }
    cycas_ctx c;
    CK(cudaSetDevice(0));
    CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    int* d_rp = c.upload(rowptr, n + 1L);
    int* d_col = c.upload(col, nnz);
    double* d_val = c.upload(val, nnz);
    double* d_b = c.upload(b, n);
    double* d_x = c.upload(x, n);
    double* d_dinv = c.upload(dinv.data(), n);
    DevStatus* st = c.alloc<DevStatus>(1);
    c.kw.m = std::max(ksp->restart, 3);
    c.kw.ldv = ((long)n + 31) / 32 * 32;
    c.kw.v_len = (c.kw.m + 1) * c.kw.ldv;
    c.kw.V = c.alloc<double>(c.kw.v_len);
    c.kw.nblocks = gmres_max_blocks(0);
    c.kw.part_len = (long)c.kw.nblocks * kGmresPartStride;
    c.kw.part = c.alloc<double>(c.kw.part_len);
    c.kw.bar = c.alloc<unsigned>(2);
    GmresCall g;
    g.n = n;
    g.rowptr = d_rp;
    g.col = d_col;
    g.val = d_val;
    g.dinv = ksp->pc == CYCAS_PC_JACOBI ? d_dinv : nullptr;
    g.b = d_b;
    g.x = d_x;
    g.guess_zero = guess_zero ? 1 : 0;
    g.rtol = rtol;
    g.maxit = maxit;
    g.restart = ksp->restart;
    g.out = &st->ksp[0];
    g.err = &st->err;
    if (ksp->type == CYCAS_KSP_CG) CK(launch_cg(g, c.kw, c.stream));
    else CK(launch_gmres(g, c.kw, c.stream));
    DevStatus hs;
    CK(cudaMemcpyAsync(&hs, st, sizeof hs, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(x, d_x, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (stats) {
      stats->its = hs.ksp[0].its;
      stats->reason = hs.ksp[0].reason;
      stats->rnorm = hs.ksp[0].rnorm;
    }
    if (hs.err & 1) {
      g_last_error = "a device-side grid barrier timed out";
      return (int)CYCAS_ERR_TIMEOUT;
    }
    if (hs.ksp[0].reason == CYCAS_KSP_DIVERGED_NANORINF) return (int)CYCAS_NAN_DETECTED;
    return hs.ksp[0].reason < 0 ? (int)CYCAS_NOT_CONVERGED : (int)CYCAS_OK;
  });
}

}  // extern "C"
