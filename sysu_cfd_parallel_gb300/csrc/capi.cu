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
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cycasgpu.h"
#include "cycas_amg.h"
#include "cycas_device.h"
#include "cycas_host.h"
#include "batch_schedule.h"
#include "mesh_tables.h"

struct cycas_case {
  cycas::HostCase hc;
  // the case's pressure AMG hierarchy, built the first time a batch holds the case and reused
  // by every later batch (it depends on the case's own mesh only); serving rebuilds a batch at
  // every membership change
  mutable std::shared_ptr<const cycas::AmgHostHierarchy> amg;
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

// Asynchronous result dump of one context: the cell fields are snapshotted on the compute
// stream (device-to-device, a few microseconds), copied out on a side stream while the next
// iterations run, and formatted and written by a host thread.
struct DumpState {
  cudaStream_t side = nullptr;
  cudaEvent_t ev_snap = nullptr, ev_host = nullptr;
  double* snap = nullptr;  // device [10 * cap]
  double* host = nullptr;  // pinned [10 * cap]
  long cap = 0;
  std::thread worker;
  int rc = 0;
  std::string err;
};

// Host field transfers of cycas_simple_iteration_io that overlap the iteration: a copy
// stream and the events that order it against the compute stream.
struct IoState {
  cudaStream_t copy = nullptr;
  cudaEvent_t ev_late_in = nullptr;   // the late inputs have landed
  cudaEvent_t ev_early_out = nullptr; // the early outputs are final
};

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
  TimeConf tc;                   // transient runs: scheme 0 when steady
  int max_outer = 50;            // MaxOuterStep
  int energy = 0;                // SolveEnergy
  double pref = 1.01325e5;       // PressureReference
  double cur_time = 0.0;
  KspConf ksp[3];
  int nsolve = 0;                // solves issued in the current iteration
  int solve_sys[8] = {0};        // system of each solve of the current iteration
  std::vector<void*> allocs;
  std::map<std::string, std::pair<double*, long>> dfields;
  std::map<std::string, std::pair<int*, long>> ifields;
  double* restart_point = nullptr;   // copy of every named field (cycas_restart_point), or null
  double restart_time = 0.0;         // the clock at the restart point
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
  // CUDA graph of one iteration, captured on first use and replayed
  bool use_graph = false;
  cudaGraphExec_t gexec = nullptr;
  long long graph_launches = 0;  // kernels of one replay
  // mixed precision: FP32 Arnoldi cycles in the GMRES systems, with FP32 copies of the system
  // being solved; at level 2 also FP32 arithmetic in the gradients, the momentum rows and the
  // Rhie-Chow face flux (storage stays FP64; the pressure-correction rows and their
  // mass-imbalance sum, the corrections and the residuals stay FP64)
  bool mixed = false;
  bool fp32_assembly = false;  // mixed level 2
  double inner_rtol = 1e-4;
  float* val32 = nullptr;   // [nnz]
  float* dinv32 = nullptr;  // [ncel]
  // batch contexts: independent cases concatenated in one union mesh
  bool is_batch = false;
  int ncases = 1;
  DevBatch batch;
  std::vector<int> bnd0;              // [ncases + 1] boundary ranges of the cases
  std::vector<int> iface0;            // [ncases + 1] interior-face ranges of the cases
  BatchSchedule* d_sched = nullptr;   // teams of the Krylov launches
  int sched_grid = 0, nteams = 0;
  unsigned* team_bar = nullptr;       // [2 * nteams]
  int sched_G = 0;                    // schedule parameters in use
  double sched_factor = 1.0;
  KspOut* bksp = nullptr;             // [8][ncases] per-case Krylov reports
  std::vector<double> h_res;          // [ncases][10]
  std::vector<KspOut> h_ksp;          // [8][ncases]
  const DevBatch* bptr() const { return is_batch ? &batch : nullptr; }

  template <class T>
  T* alloc(long n, bool zero = true) {
    void* p = nullptr;
    size_t bytes = sizeof(T) * (size_t)(n > 0 ? n : 1);
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) throw StatusError(CYCAS_ERR_ALLOC, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    allocs.push_back(p);
    if (zero) CK(cudaMemsetAsync(p, 0, bytes, stream));
    return (T*)p;
  }
  template <class T>
  T* upload(const T* h, long n) {
    const bool full = n > 0 && h;  // the copy overwrites every element
    T* d = alloc<T>(n, !full);
    if (full) CK(cudaMemcpyAsync(d, h, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, stream));
    return d;
  }
  double* dfield(const char* name, long n) {
    double* p = alloc<double>(n);
    dfields[name] = {p, n};
    return p;
  }
  DumpState dump;
  IoState io;
  ~cycas_ctx() {
    if (io.copy) cudaStreamSynchronize(io.copy);
    if (io.ev_late_in) cudaEventDestroy(io.ev_late_in);
    if (io.ev_early_out) cudaEventDestroy(io.ev_early_out);
    if (io.copy) cudaStreamDestroy(io.copy);
    if (dump.worker.joinable()) dump.worker.join();
    if (dump.side) cudaStreamSynchronize(dump.side);
    if (dump.ev_snap) cudaEventDestroy(dump.ev_snap);
    if (dump.ev_host) cudaEventDestroy(dump.ev_host);
    if (dump.host) cudaFreeHost(dump.host);
    if (dump.side) cudaStreamDestroy(dump.side);
    if (stream) cudaStreamSynchronize(stream);
    if (gexec) cudaGraphExecDestroy(gexec);
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
// degree of a Jacobi-Neumann polynomial preconditioner, 0 for the others
int poly_degree(int pc) {
  switch (pc) {
    case CYCAS_PC_POLY1: return 1;
    case CYCAS_PC_POLY2: return 2;
    case CYCAS_PC_POLY3: return 3;
    case CYCAS_PC_POLY4: return 4;
    case CYCAS_PC_POLY5: return 5;
    default: return 0;
  }
}

// the same for a literal message: nothing is built unless the check fails (the mesh checks run
// per face and per vertex, where a std::string per call cost more than the checks)
void require(bool ok, const char* msg) {
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
    if (!(a >= 0 && a < n)) require(false, "face_cell1 out of range at face " + std::to_string(i));
    if (!(b < n && (b >= 0 || b == -10))) require(false, "face_cell2 must be a cell or -10 at face " + std::to_string(i));
    if (b < 0) require(v.face_bnd[i] >= 0 && v.face_bnd[i] < nb, "boundary face without boundary index");
  }
  for (int i = 0; i < nb; i++) {
    require(v.bnd_face[i] == i, "boundary faces must come first in boundary order (Bnd[i].face == i)");
    require(v.face_cell2[i] < 0, "boundary face has two cells");
    int t = v.bnd_type[i];
    require(t >= 1 && t <= 4, "boundary type must be wall/inlet/outlet/symmetry");
  }
  // CSR pattern, slots, diagonals and per-cell face orders (checks the cells' face lists)
  const MeshTables T = mesh_tables(n, nf, v.cell_nface, v.cell_face, v.face_cell1, v.face_cell2);
  m.nnz = (int)T.col.size();
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
  m.c_face = c.upload(T.face_sm.data(), 6L * n);
  m.c_gface = c.upload(T.gface.data(), 6L * n);
  m.c_slot = c.upload(T.slot.data(), 6L * n);
  m.c_diag = c.upload(T.diag.data(), n);
  m.b_face = c.upload(v.bnd_face, nb);
  m.b_type = c.upload(v.bnd_type, nb);
  m.rowptr = c.upload(T.rowptr.data(), n + 1);
  m.col = c.upload(T.col.data(), m.nnz);
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
  f.Rnp = f.Unp = f.Vnp = f.Wnp = f.Tnp = f.TEp = f.EDp = nullptr;
  if (c.tc.scheme != 0) {
    f.Rnp = c.dfield("Rnp", n);
    f.Unp = c.dfield("Unp", n);
    f.Vnp = c.dfield("Vnp", n);
    f.Wnp = c.dfield("Wnp", n);
    f.Tnp = c.dfield("Tnp", n);
    f.TEp = c.dfield("TEp", n);
    f.EDp = c.dfield("EDp", n);
  }
  f.kcond = f.ES = f.ApE = nullptr;
  if (c.energy) {
    f.kcond = c.dfield("kcond", n);
    f.ES = c.dfield("ESource", n);
    f.ApE = c.dfield("ApE", n);
  }
}

void alloc_krylov(cycas_ctx& c) {
  int maxm = 3;  // CG needs four work vectors
  for (int s = 0; s < 3; s++) maxm = std::max(maxm, c.ksp[s].restart);
  require(maxm <= kMaxRestart, "GMRES restart above " + std::to_string(kMaxRestart));
  KrylovWork& w = c.kw;
  w.m = maxm;
  w.ldv = ((long)c.m.ncel + 31) / 32 * 32;
  int poly = 0;
  for (int s = 0; s < 3; s++) poly = std::max(poly, poly_degree(c.ksp[s].pc));
  // three momentum systems in lockstep, each with two Neumann scratch vectors (three from
  // degree 3) when needed
  w.v_len = (3L * (maxm + 1) + (poly ? 3L * (poly >= 3 ? 3 : 2) : 0)) * w.ldv;
  w.V = c.alloc<double>(w.v_len);
  w.nblocks = gmres_max_blocks(c.device);
  // per CTA and per lockstep system (up to the three momentum components)
  w.part_len = 3L * w.nblocks * kGmresPartStride;
  w.part = c.alloc<double>(w.part_len);
  w.bar = c.alloc<unsigned>(2);
  if (c.mixed) {
    c.val32 = c.alloc<float>(c.m.nnz);
    c.dinv32 = c.alloc<float>(c.m.ncel);
  }
  c.red_parts = std::min(residual_blocks(c.m.ncel), 1024);
  int cells_blocks = (c.m.ncel + 255) / 256;
  c.red = c.alloc<double>(3L * std::max(c.red_parts, cells_blocks));
}

// Aggregation hierarchy of the pressure system.  Strength of a connection = the face
// coefficient area/|d.n| (Face.rlencos) of the face joining the two cells.
void setup_amg(cycas_ctx& c, std::vector<std::shared_ptr<const AmgHostHierarchy>>* cache = nullptr) {
  struct Up : AmgUploader {
    cycas_ctx& c;
    explicit Up(cycas_ctx& cc) : c(cc) {}
    const int* upload_int(const int* h, long n) override { return c.upload(h, n); }
    float* alloc_float(long n) override { return c.alloc<float>(n); }
    void* upload_bytes(const void* h, long bytes) override { return c.upload((const unsigned char*)h, bytes); }
  } up(c);
  if (cache && std::all_of(cache->begin(), cache->end(), [](const auto& h) { return h != nullptr; })) {
    // every hierarchy known: no host copy of the pattern is needed
    amg_setup_cases(c.amg, c.m.ncel, nullptr, nullptr, nullptr, c.m.rowptr, c.m.col, c.m.c_diag, c.f.Ap,
                    c.case_lo, c.case_hi, up, cache);
    c.amg_sizes = c.amg.rows0;
    c.amg_nnz = c.amg.nnz0;
    return;
  }
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
  amg_setup_cases(c.amg, n, rowptr.data(), col.data(), w.data(), c.m.rowptr, c.m.col, c.m.c_diag, c.f.Ap,
                  c.case_lo, c.case_hi, up, cache);
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
  require(p->density_model == 0 || p->density_model == 1, "DensityModel must be 0 or 1");
  require(p->turb_model == 0 || p->turb_model == 1, "TurModel must be 0 or 1");
  c.turb = p->turb_model;
  c.density = p->density_model;
  if (p->transient) {
    require(p->time_scheme == 1 || p->time_scheme == 2, "TimeScheme must be 1 (Euler) or 2 (Dual)");
    require(p->dt > 0.0, "dt must be positive");
    c.tc.scheme = p->time_scheme;
    c.tc.dt = p->dt;
    c.max_outer = p->max_outer;
  }
  c.energy = (p->solve_energy || p->density_model == 1) ? 1 : 0;  // readparamfile.cpp:337-338
  c.pref = p->pressure_reference > 0.0 ? p->pressure_reference : 1.01325e5;
  c.cell_pref = p->cell_pressure_ref;
  for (int i = 0; i < 8; i++) c.urf[i] = p->urf[i];
  for (int i = 0; i < 3; i++) c.gravity[i] = p->gravity[i];
  for (int s = 0; s < 3; s++) {
    const cycas_ksp_options& k = o->ksp[s];
    require(k.pc == CYCAS_PC_NONE || k.pc == CYCAS_PC_JACOBI || k.pc == CYCAS_PC_AMG || poly_degree(k.pc) > 0,
            "preconditioner not available in this build");
    require(poly_degree(k.pc) == 0 ||
                (s != CYCAS_SYS_PRESSURE && k.type != CYCAS_KSP_CG),
            "the polynomial preconditioner is for the GMRES systems (momentum, scalars)");
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
  require(o->mixed >= 0 && o->mixed <= 2, "mixed must be 0, 1 or 2");
  c.mixed = o->mixed != 0;
  c.fp32_assembly = o->mixed == 2;
  c.inner_rtol = o->inner_rtol > 0.0 ? o->inner_rtol : 1e-4;
  require(o->amg_omega <= 1.0f && o->amg_alpha <= 2.0f && o->amg_gamma >= 0 && o->amg_gamma <= 4,
          "AMG options out of range (omega <= 1, alpha <= 2, gamma 0..4)");
  if (o->amg_omega > 0.0f) c.amg.omega = o->amg_omega;
  if (o->amg_alpha > 0.0f) c.amg.alpha = o->amg_alpha;
  if (o->amg_gamma > 0) c.amg.gamma = o->amg_gamma;
  c.d_geom_err = c.alloc<int>(1);
  c.st = c.alloc<DevStatus>(1);
  CK(cudaMallocHost((void**)&c.st_host, sizeof(DevStatus)));
  std::memset(c.st_host, 0, sizeof(DevStatus));
}

// ---------------------------------------------------------------- iteration schedule
// mixed precision: FP32 copies of the operator and Jacobi inverse for the Arnoldi cycles
void set_mixed(cycas_ctx& c, GmresCall& g) {
  launch_to_float(g.val, c.val32, c.m.nnz, c.stream);
  if (g.dinv) launch_to_float(g.dinv, c.dinv32, c.m.ncel, c.stream);
  g.val32 = c.val32;
  g.dinv32 = g.dinv ? c.dinv32 : nullptr;
  g.inner_rtol = c.inner_rtol;
}

void solve(cycas_ctx& c, int sys, const double* val, const double* dinv, const double* b, double* x, bool guess_zero,
           const KspConf* conf = nullptr) {
  require(c.nsolve < 8, "too many solves in one iteration");
  const KspConf& k = conf ? *conf : c.ksp[sys];
  GmresCall g;
  g.n = c.m.ncel;
  g.rowptr = c.m.rowptr;
  g.col = c.m.col;
  g.val = val;
  g.dinv = (k.pc == CYCAS_PC_JACOBI || poly_degree(k.pc) > 0) ? dinv : nullptr;
  g.poly = poly_degree(k.pc);
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
  const bool gm = k.pc != CYCAS_PC_AMG && k.type != CYCAS_KSP_CG;
  if (c.mixed && gm) set_mixed(c, g);
  if (c.profiling) CK(cudaEventRecord(c.ev_solve[slot][0], c.stream));
  if (c.is_batch) {
    CK(cudaMemsetAsync(c.team_bar, 0, 2 * sizeof(unsigned) * c.nteams, c.stream));
    KrylovWork w = c.kw;
    w.bar = c.team_bar;
    KspOut* outs = c.bksp + (long)slot * c.ncases;
    if (k.pc == CYCAS_PC_AMG) {
      launch_amg_setup_values(c.amg, c.stream);
      CK(launch_cg_amg(g, c.amg, w, c.d_sched, c.sched_grid, outs, c.stream));
    } else {
      require(k.type != CYCAS_KSP_CG, "batches solve CG with the AMG preconditioner only");
      CK(launch_gmres_batch(&g, 1, w, c.d_sched, c.sched_grid, &outs, c.stream));
    }
    if (c.profiling) CK(cudaEventRecord(c.ev_solve[slot][1], c.stream));
    ++g_launch_count;
    c.prof.krylov_launches[sys]++;
    return;
  }
  CK(cudaMemsetAsync(c.kw.bar, 0, 2 * sizeof(unsigned), c.stream));
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
// xs_in: the three solution vectors (default: the context's U, V, W); conf: method override
void solve_velocity(cycas_ctx& c, double* const* xs_in = nullptr, const KspConf* conf = nullptr) {
  require(c.nsolve + 3 <= 8, "too many solves in one iteration");
  const KspConf& k = conf ? *conf : c.ksp[CYCAS_SYS_VELOCITY];
  double* xs[3] = {c.f.U, c.f.V, c.f.W};
  if (xs_in)
    for (int q = 0; q < 3; q++) xs[q] = xs_in[q];
  if (k.type == CYCAS_KSP_CG || k.pc == CYCAS_PC_AMG) {  // non-default methods: one solve at a time
    require(!c.is_batch, "batches solve the momentum equations with GMRES");
    solve(c, CYCAS_SYS_VELOCITY, c.f.Au, c.f.dinv_u, c.f.bu, xs[0], false, conf);
    solve(c, CYCAS_SYS_VELOCITY, c.f.Au, c.f.dinv_u, c.f.bv, xs[1], false, conf);
    solve(c, CYCAS_SYS_VELOCITY, c.f.Au, c.f.dinv_u, c.f.bw, xs[2], false, conf);
    return;
  }
  GmresCall g[3];
  const double* bs[3] = {c.f.bu, c.f.bv, c.f.bw};
  const int slot0 = c.nsolve;
  for (int q = 0; q < 3; q++) {
    g[q].n = c.m.ncel;
    g[q].rowptr = c.m.rowptr;
    g[q].col = c.m.col;
    g[q].val = c.f.Au;
    g[q].dinv = (k.pc == CYCAS_PC_JACOBI || poly_degree(k.pc) > 0) ? c.f.dinv_u
                                                                                                 : nullptr;
    g[q].poly = poly_degree(k.pc);
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
  if (c.mixed) {
    set_mixed(c, g[0]);
    for (int q = 1; q < 3; q++) {
      g[q].val32 = g[0].val32;
      g[q].dinv32 = g[0].dinv32;
      g[q].inner_rtol = g[0].inner_rtol;
    }
  }
  if (c.profiling) CK(cudaEventRecord(c.ev_solve[slot0][0], c.stream));
  if (c.is_batch) {
    CK(cudaMemsetAsync(c.team_bar, 0, 2 * sizeof(unsigned) * c.nteams, c.stream));
    KrylovWork w = c.kw;
    w.bar = c.team_bar;
    KspOut* outs[3];
    for (int q = 0; q < 3; q++) outs[q] = c.bksp + (long)(slot0 + q) * c.ncases;
    CK(launch_gmres_batch(g, 3, w, c.d_sched, c.sched_grid, outs, c.stream));
  } else {
    CK(cudaMemsetAsync(c.kw.bar, 0, 2 * sizeof(unsigned), c.stream));
    CK(launch_gmres_multi(g, 3, c.kw, c.stream));
  }
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
  launch_bc_velocity(c.m, c.f, c.density, with_pressure, c.stream, c.bptr());
}

void grad_uvwp(cycas_ctx& c) {
  const double* phi[4] = {c.f.U, c.f.V, c.f.W, c.f.P};
  const double* bphi[4] = {c.f.BU, c.f.BV, c.f.BW, c.f.BPre};
  double* g[4] = {c.f.dUdX, c.f.dVdX, c.f.dWdX, c.f.dPdX};
  launch_gradient(c.m, 4, phi, bphi, g, c.stream, c.fp32_assembly);
}

void grad1(cycas_ctx& c, const double* phi, const double* bphi, double* g) {
  launch_gradient(c.m, 1, &phi, &bphi, &g, c.stream, c.fp32_assembly);
}

// BuildVelocityMatrix (navier_velocity.cpp:63-393)
void build_velocity(cycas_ctx& c) {
  bc_velocity(c, true);
  grad_uvwp(c);
  launch_momentum(c.m, c.f, c.urf, c.gravity, c.st, c.stream, c.tc, c.fp32_assembly);
}

// CalculateVelocity (navier_velocity.cpp:10-60)
void calculate_velocity(cycas_ctx& c) {
  build_velocity(c);
  solve_velocity(c);
  launch_residual_uvw(c.m, c.f, c.red, c.st, c.stream, c.bptr());
}

void correct_cells(cycas_ctx& c) {
  launch_correct_cells(c.m, c.f, c.cell_pref, c.urf[3], c.red, c.stream, c.bptr(), c.density);
  launch_finalize_residual(c.red, c.is_batch ? c.batch.nblk : (c.m.ncel + 255) / 256, 3, c.st, c.stream, c.bptr());
}

// the pressure-correction rows of the context's density model
void build_pressure(cycas_ctx& c) {
  if (c.density == 1) launch_pressure_gas(c.m, c.f, c.tc, c.stream);
  else launch_pressure(c.m, c.f, c.stream);
}

// CalculatePressure (navier_pressure.cpp:9-97).  A perfect gas makes the system nonsymmetric:
// the reference then switches PETSc to GMRES (MPIStructure.cpp:462-467); here GMRES(restart)
// with the Jacobi preconditioner at the pressure system's tolerances.
void calculate_pressure(cycas_ctx& c) {
  bc_velocity(c, false);
  launch_ruface2(c.m, c.f, c.stream, c.fp32_assembly);
  build_pressure(c);
  if (c.density == 1) {
    KspConf k = c.ksp[CYCAS_SYS_PRESSURE];
    k.type = CYCAS_KSP_GMRES;
    if (k.pc == CYCAS_PC_AMG) k.pc = CYCAS_PC_JACOBI;
    solve(c, CYCAS_SYS_PRESSURE, c.f.Ap, c.f.dinv_p, c.f.bp, c.f.dp, true, &k);
  } else {
    solve(c, CYCAS_SYS_PRESSURE, c.f.Ap, c.f.dinv_p, c.f.bp, c.f.dp, true);
  }
  launch_bc_deltap(c.m, c.f, c.stream);
  grad1(c, c.f.dp, c.f.BPre, c.f.dPdX);
  correct_cells(c);
  bc_velocity(c, false);
  launch_correct_ruface(c.m, c.f, c.urf[3], c.stream, c.density);
}

// UpdateTurKEpsilon (navier_scalar.cpp:11-197), k rows: sources, wall functions and boundary
// values, unsteady terms, the assembled system in As / bs
void build_te(cycas_ctx& c) {
  launch_keps_sources(c.m, c.f, c.stream);
  launch_keps_wall(c.m, c.f, c.stream);
  if (c.tc.scheme != 0) {  // unsteady terms (navier_scalar.cpp:71-90); the epsilon source is
    // overwritten before its solve (navier_scalar.cpp:118), its diagonal share is kept
    launch_scalar_time(c.m, c.f, c.tc, c.f.TEp, c.f.ApTE, c.f.TES, c.stream);
    launch_scalar_time(c.m, c.f, c.tc, c.f.EDp, c.f.ApED, c.f.EDS, c.stream);
  }
  grad1(c, c.f.TE, c.f.BTE, c.f.dPhidX);
  launch_scalar(c.m, c.f, c.f.TE, c.f.BTE, c.f.VisTE, c.f.TES, c.f.ApTE, c.urf[5], c.st, c.stream);
}

// epsilon rows on the solved k: k clipped, epsilon sources, the wall cells' fixed rows
void build_ed(cycas_ctx& c) {
  launch_clip_te(c.m, c.f, c.stream);
  grad1(c, c.f.ED, c.f.BED, c.f.dPhidX);
  launch_scalar(c.m, c.f, c.f.ED, c.f.BED, c.f.VisED, c.f.EDS, c.f.ApED, c.urf[5], c.st, c.stream);
  launch_eps_wall_rows(c.m, c.f, c.stream);
}

void update_keps(cycas_ctx& c) {
  build_te(c);
  solve(c, CYCAS_SYS_SCALAR, c.f.As, c.f.dinv_s, c.f.bs, c.f.TE, false);
  build_ed(c);
  solve(c, CYCAS_SYS_SCALAR, c.f.As, c.f.dinv_s, c.f.bs, c.f.ED, false);
  launch_finish_keps(c.m, c.f, c.stream);
}

// UpdateEnergy (navier_scalar.cpp:204-326): temperature transport with conductivity
// cp (mu / Pr + mu_t / Pr_t) / cp, viscous heating with a perfect gas, GMRES at rtol 1e-8
void build_energy(cycas_ctx& c) {
  require(c.energy, "the energy equation is not solved in this context");
  launch_energy_sources(c.m, c.f, c.density, c.stream);
  launch_bc_temperature(c.m, c.f, c.stream);
  if (c.tc.scheme != 0) launch_scalar_time(c.m, c.f, c.tc, c.f.Tnp, c.f.ApE, c.f.ES, c.stream);
  grad1(c, c.f.T, c.f.BTem, c.f.dPhidX);
  launch_scalar(c.m, c.f, c.f.T, c.f.BTem, c.f.kcond, c.f.ES, c.f.ApE, c.urf[5], c.st, c.stream);
}

void update_energy(cycas_ctx& c) {
  build_energy(c);
  solve(c, CYCAS_SYS_SCALAR, c.f.As, c.f.dinv_s, c.f.bs, c.f.T, false);
}

// SaveTransientOldData (navier.cpp:698-740)
void save_old_level(cycas_ctx& c) {
  require(c.tc.scheme != 0, "not a transient context");
  const long n = c.m.ncel;
  const double* cur[7] = {c.f.R, c.f.U, c.f.V, c.f.W, c.f.T, c.f.TE, c.f.ED};
  double* old[7] = {c.f.Rnp, c.f.Unp, c.f.Vnp, c.f.Wnp, c.f.Tnp, c.f.TEp, c.f.EDp};
  const int nf = c.turb == 1 ? 7 : 5;
  for (int q = 0; q < nf; q++)
    CK(cudaMemcpyAsync(old[q], cur[q], sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
}

void begin_iteration(cycas_ctx& c) {
  CK(cudaMemsetAsync(c.st, 0, sizeof(DevStatus), c.stream));
  if (c.is_batch) {
    CK(cudaMemsetAsync(c.batch.res, 0, sizeof(double) * 10 * c.ncases, c.stream));
    CK(cudaMemsetAsync(c.bksp, 0, sizeof(KspOut) * 8 * c.ncases, c.stream));
  }
  c.nsolve = 0;
  c.iter_open = true;
  if (c.profiling) CK(cudaEventRecord(c.ev_iter[0], c.stream));
}

// after_pressure (optional) runs on the host once the pressure correction is queued, before
// the k-epsilon and energy stages
void issue_iteration(cycas_ctx& c, const std::function<void()>& after_pressure = nullptr) {
  calculate_velocity(c);
  calculate_pressure(c);
  if (after_pressure) after_pressure();
  if (c.turb == 1) update_keps(c);
  if (c.energy) update_energy(c);
}

// One iteration's device work.  In graph mode the first call captures begin + issue into a
// CUDA graph (the launches of an iteration do not depend on device results, so the sequence
// is the same every iteration) and every call replays it with one launch.
void run_iteration(cycas_ctx& c) {
  if (!c.use_graph) {
    begin_iteration(c);
    issue_iteration(c);
    return;
  }
  if (!c.gexec) {
    const long long l0 = g_launch_count;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed));
    cudaGraph_t g = nullptr;
    try {
      begin_iteration(c);
      issue_iteration(c);
    } catch (...) {
      cudaStreamEndCapture(c.stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    CK(cudaStreamEndCapture(c.stream, &g));
    cudaError_t e = cudaGraphInstantiate(&c.gexec, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    c.graph_launches = g_launch_count - l0;
    g_launch_count = l0;
  }
  c.iter_open = false;
  CK(cudaGraphLaunch(c.gexec, c.stream));
  g_launch_count += c.graph_launches;
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

// ---------------------------------------------------------------- batches
// (the union of a batch's cases: build_union, union_mesh.cpp)

// Teams for the batched Krylov launches (team_schedule, batch_schedule.cpp), uploaded as the
// device schedule.  G: CTAs of the Krylov launches (at most the co-resident maximum); factor
// scales the row share that earns a case its own team.
void build_schedule(cycas_ctx& c, int G, double factor) {
  const int nc = c.ncases;
  G = std::max(1, std::min(G, c.kw.nblocks));
  const TeamSchedule S = team_schedule(c.case_lo, c.case_hi, G, factor);
  c.nteams = (int)S.team_size.size();
  c.sched_grid = (int)S.cta_team.size();
  BatchSchedule hs;
  hs.cta_team = c.upload(S.cta_team.data(), (long)S.cta_team.size());
  hs.cta_rank = c.upload(S.cta_rank.data(), (long)S.cta_rank.size());
  hs.team_size = c.upload(S.team_size.data(), (long)S.team_size.size());
  hs.team_cta0 = c.upload(S.team_cta0.data(), (long)S.team_cta0.size());
  hs.team_case0 = c.upload(S.team_case0.data(), (long)S.team_case0.size());
  hs.case_list = c.upload(S.case_list.data(), (long)S.case_list.size());
  hs.case_lo = c.upload(c.case_lo.data(), nc);
  hs.case_hi = c.upload(c.case_hi.data(), nc);
  c.d_sched = c.upload(&hs, 1);
  if (!c.team_bar) c.team_bar = c.alloc<unsigned>(2L * c.kw.nblocks);
  c.sched_G = G;
  c.sched_factor = factor;
}

// per-case metadata of a batch context
void setup_batch(cycas_ctx& c, const UnionMesh& u, const std::vector<const HostCase*>& hs) {
  const int nc = (int)hs.size();
  c.is_batch = true;
  c.ncases = nc;
  c.case_lo.assign(u.cell0.begin(), u.cell0.end() - 1);
  c.case_hi.assign(u.cell0.begin() + 1, u.cell0.end());
  c.bnd0 = u.bnd0;
  c.iface0 = u.iface0;
  std::vector<int> blk_lo, blk_hi, blk_case, case_blk0, pref, in0(nc + 1, 0), out0(nc + 1, 0);
  for (int k = 0; k < nc; k++) {
    case_blk0.push_back((int)blk_lo.size());
    for (int r = c.case_lo[k]; r < c.case_hi[k]; r += 256) {
      blk_lo.push_back(r);
      blk_hi.push_back(std::min(r + 256, c.case_hi[k]));
      blk_case.push_back(k);
    }
    const int pr = hs[k]->cell_pressure_ref;
    require(pr >= 0 && pr < hs[k]->ncel, "PressureRef cell out of range");
    pref.push_back(c.case_lo[k] + pr);
    in0[k + 1] = in0[k];
    out0[k + 1] = out0[k];
    for (int b = 0; b < hs[k]->nbnd; b++) {
      if (hs[k]->bnd_type[b] == 2) in0[k + 1]++;
      if (hs[k]->bnd_type[b] == 3) out0[k + 1]++;
    }
  }
  case_blk0.push_back((int)blk_lo.size());
  DevBatch& b = c.batch;
  b.ncases = nc;
  b.nblk = (int)blk_lo.size();
  b.blk_lo = c.upload(blk_lo.data(), b.nblk);
  b.blk_hi = c.upload(blk_hi.data(), b.nblk);
  b.blk_case = c.upload(blk_case.data(), b.nblk);
  b.case_blk0 = c.upload(case_blk0.data(), nc + 1);
  b.case_pref = c.upload(pref.data(), nc);
  b.in0 = c.upload(in0.data(), nc + 1);
  b.out0 = c.upload(out0.data(), nc + 1);
  b.res = c.alloc<double>(10L * nc);
  c.red = c.alloc<double>(3L * b.nblk);
  c.bksp = c.alloc<KspOut>(8L * nc);
  c.h_res.assign(10L * nc, 0.0);
  c.h_ksp.assign(8L * nc, KspOut{});
  build_schedule(c, c.kw.nblocks, 1.0);
}

// reads the per-case residuals and Krylov reports of a batch iteration
int finish_batch(cycas_ctx& c, double* resmax, int32_t* its, int32_t* reasons) {
  CK(cudaGetLastError());
  const bool timed = c.profiling && c.iter_open;
  c.iter_open = false;
  if (timed) CK(cudaEventRecord(c.ev_iter[1], c.stream));
  CK(cudaMemcpyAsync(c.st_host, c.st, sizeof(DevStatus), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_res.data(), c.batch.res, sizeof(double) * 10 * c.ncases, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_ksp.data(), c.bksp, sizeof(KspOut) * 8 * c.ncases, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  const int nc = c.ncases;
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
  int failed = -1, nan = 0;
  for (int k = 0; k < c.nsolve; k++) {
    int mx = 0;
    for (int q = 0; q < nc; q++) {
      const KspOut& o = c.h_ksp[(long)k * nc + q];
      mx = std::max(mx, o.its);
      if (o.reason < 0 && failed < 0) failed = q;
      if (o.reason == CYCAS_KSP_DIVERGED_NANORINF) nan = 1;
    }
    c.prof.krylov_iters[c.solve_sys[k]] += mx;
  }
  for (int q = 0; q < nc; q++) {
    double mx = 0.0;
    for (int i = 0; i < 10; i++) mx = mx > c.h_res[10L * q + i] ? mx : c.h_res[10L * q + i];
    if (resmax) resmax[q] = mx;
    for (int k = 0; k < 8; k++) {
      const bool on = k < c.nsolve;
      if (its) its[8L * q + k] = on ? c.h_ksp[(long)k * nc + q].its : -1;
      if (reasons) reasons[8L * q + k] = on ? c.h_ksp[(long)k * nc + q].reason : 0;
    }
  }
  const DevStatus& s = *c.st_host;
  if (s.err & 1) {
    g_last_error = "a device-side barrier timed out; the solve was abandoned";
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
    g_last_error = "a Krylov solve of case " + std::to_string(failed) + " did not converge";
    return CYCAS_NOT_CONVERGED;
  }
  return CYCAS_OK;
}

// ---------------------------------------------------------------- result files
// The cell fields of case k (the context's only case when it is not a batch), copied to the host.
struct CaseFields {
  std::vector<double> a[10];  // P U V W R T VisLam VisTur TE ED
  CellFieldsView view;
};

void fetch_case_fields(cycas_ctx& c, int k, CaseFields& out) {
  require(k >= 0 && k < c.ncases, "case index out of range");
  static const char* names[10] = {"P", "U", "V", "W", "R", "T", "VisLam", "VisTur", "TE", "ED"};
  const long lo = c.case_lo[k], n = c.case_hi[k] - lo;
  for (int i = 0; i < 10; i++) {
    out.a[i].resize((size_t)n);
    auto p = lookup(c, names[i]);
    CK(cudaMemcpyAsync(out.a[i].data(), p.first + lo, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
  }
  CK(cudaStreamSynchronize(c.stream));
  CellFieldsView& v = out.view;
  v.ncel = n;
  v.turb = c.turb;
  v.density = c.density;
  v.pref = c.pref;
  v.P = out.a[0].data(), v.U = out.a[1].data(), v.V = out.a[2].data(), v.W = out.a[3].data();
  v.R = out.a[4].data(), v.T = out.a[5].data(), v.VisLam = out.a[6].data(), v.VisTur = out.a[7].data();
  v.TE = out.a[8].data(), v.ED = out.a[9].data();
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

int cycas_case_load(const char* param_path, cycas_case** out) { return cycas_case_load_ex(param_path, 0, out); }

int cycas_case_load_ex(const char* param_path, int32_t flags, cycas_case** out) {
  return guard([&]() -> int {
    require(param_path && out, "null argument");
    require((flags & ~CYCAS_LOAD_MSH_BINARY) == 0, "unknown load flags");
    *out = nullptr;
    cycas_case* c = new cycas_case();
    try {
      load_case(c->hc, param_path, (flags & CYCAS_LOAD_MSH_BINARY) != 0);
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

int cycas_case_physics(const cycas_case* c, int32_t iopt[6], double dopt[3]) {
  return guard([&]() -> int {
    require(c != nullptr, "null case");
    const HostCase& h = c->hc;
    if (iopt) {
      iopt[0] = h.steady;
      iopt[1] = h.time_scheme;
      iopt[2] = h.max_outer;
      iopt[3] = h.solve_energy;
      iopt[4] = h.density_model;
      iopt[5] = h.max_step;
    }
    if (dopt) {
      dopt[0] = h.dt;
      dopt[1] = h.total_time;
      dopt[2] = h.pressure_reference;
    }
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
    // the kernels read p' at this cell: checked before anything reaches the device
    require(mesh->ncel <= 0 || (params->cell_pressure_ref >= 0 && params->cell_pressure_ref < mesh->ncel),
            "PressureRef cell out of range");
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
    p.transient = h.steady ? 0 : 1;
    p.time_scheme = h.time_scheme;
    p.dt = h.dt;
    p.max_outer = h.max_outer;
    p.solve_energy = h.solve_energy;
    p.pressure_reference = h.pressure_reference;
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

int cycas_set_fields(cycas_ctx* c, int32_t count, const char* const* names, const double* const* src,
                     const int64_t* n) {
  return guard([&]() -> int {
    require(c && count >= 0 && (count == 0 || (names && src && n)), "null argument");
    for (int i = 0; i < count; i++) {  // every name and size checked before any copy is queued
      require(names[i] && src[i], "null field name or array");
      require(lookup(*c, names[i]).second == n[i], std::string("size mismatch for ") + names[i]);
    }
    for (int i = 0; i < count; i++)
      CK(cudaMemcpyAsync(lookup(*c, names[i]).first, src[i], sizeof(double) * n[i], cudaMemcpyHostToDevice,
                         c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CYCAS_OK;
  });
}

int cycas_get_fields(cycas_ctx* c, int32_t count, const char* const* names, double* const* dst, const int64_t* n) {
  return guard([&]() -> int {
    require(c && count >= 0 && (count == 0 || (names && dst && n)), "null argument");
    for (int i = 0; i < count; i++) {
      require(names[i] && dst[i], "null field name or array");
      require(lookup(*c, names[i]).second == n[i], std::string("size mismatch for ") + names[i]);
    }
    for (int i = 0; i < count; i++)
      CK(cudaMemcpyAsync(dst[i], lookup(*c, names[i]).first, sizeof(double) * n[i], cudaMemcpyDeviceToHost,
                         c->stream));
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
    run_iteration(*c);
    return finish_iteration(*c, residual, resmax, stats);
  });
}

namespace {
// Inputs first read by the k-epsilon stage, and outputs final once the pressure correction is
// done (the k-epsilon and energy stages only read them).  Checked against the kernels' argument
// lists: momentum, Rhie-Chow, pressure and corrections take no k-epsilon field, and the
// k-epsilon kernels write only TE, ED, their boundary values, sources and VisTur.
bool late_input(const cycas_ctx& c, const char* nm) {
  if (c.turb != 1) return false;
  return !std::strcmp(nm, "TE") || !std::strcmp(nm, "ED") || !std::strcmp(nm, "BTE") || !std::strcmp(nm, "BED");
}
bool early_output(const cycas_ctx& c, const char* nm) {
  if (c.turb != 1) return false;  // nothing runs after the pressure correction to overlap
  static const char* names[] = {"U", "V", "W", "P", "RUFace", "BU", "BV", "BW", "BRo", "deltaP"};
  for (const char* e : names)
    if (!std::strcmp(nm, e)) return true;
  return false;
}
}  // namespace

int cycas_simple_iteration_io(cycas_ctx* c, int32_t nin, const char* const* in_names, const double* const* in_src,
                              const int64_t* in_n, int32_t nout, const char* const* out_names,
                              double* const* out_dst, const int64_t* out_n, double residual[10], double* resmax,
                              cycas_iter_stats* stats) {
  return guard([&]() -> int {
    require(c != nullptr && nin >= 0 && nout >= 0, "bad argument");
    require(nin == 0 || (in_names && in_src && in_n), "null input arrays");
    require(nout == 0 || (out_names && out_dst && out_n), "null output arrays");
    require(!c->is_batch, "cycas_simple_iteration_io takes a single-case context");
    for (int i = 0; i < nin; i++) {
      require(in_names[i] && in_src[i], "null input field");
      require(lookup(*c, in_names[i]).second == in_n[i], std::string("size mismatch for ") + in_names[i]);
    }
    for (int i = 0; i < nout; i++) {
      require(out_names[i] && out_dst[i], "null output field");
      require(lookup(*c, out_names[i]).second == out_n[i], std::string("size mismatch for ") + out_names[i]);
    }
    cycas_ctx& x = *c;
    if (!x.io.copy) {
      CK(cudaStreamCreateWithFlags(&x.io.copy, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&x.io.ev_late_in, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&x.io.ev_early_out, cudaEventDisableTiming));
    }
    const bool overlap = !x.use_graph;  // a captured iteration has no stage boundary to hook
    auto h2d = [&](int i, cudaStream_t s) {
      CK(cudaMemcpyAsync(lookup(x, in_names[i]).first, in_src[i], sizeof(double) * in_n[i], cudaMemcpyHostToDevice, s));
    };
    auto d2h = [&](int i, cudaStream_t s) {
      CK(cudaMemcpyAsync(out_dst[i], lookup(x, out_names[i]).first, sizeof(double) * out_n[i], cudaMemcpyDeviceToHost,
                         s));
    };
    bool any_late = false, any_early = false;
    for (int i = 0; i < nin; i++) {
      const bool late = overlap && late_input(x, in_names[i]);
      any_late = any_late || late;
      h2d(i, late ? x.io.copy : x.stream);
    }
    if (any_late) CK(cudaEventRecord(x.io.ev_late_in, x.io.copy));
    if (!overlap) {
      run_iteration(x);
    } else {
      for (int i = 0; i < nout; i++) any_early = any_early || early_output(x, out_names[i]);
      begin_iteration(x);
      issue_iteration(x, [&]() {
        if (any_early) {
          CK(cudaEventRecord(x.io.ev_early_out, x.stream));
          CK(cudaStreamWaitEvent(x.io.copy, x.io.ev_early_out, 0));
          for (int i = 0; i < nout; i++)
            if (early_output(x, out_names[i])) d2h(i, x.io.copy);
        }
        if (any_late) CK(cudaStreamWaitEvent(x.stream, x.io.ev_late_in, 0));
      });
    }
    for (int i = 0; i < nout; i++)
      if (!(overlap && any_early && early_output(x, out_names[i]))) d2h(i, x.stream);
    const int rc = finish_iteration(x, residual, resmax, stats);
    CK(cudaStreamSynchronize(x.io.copy));
    return rc;
  });
}

int cycas_simple_iterations(cycas_ctx* c, int32_t n, double* res_hist, double* resmax, int32_t* its,
                            int32_t* reasons) {
  return guard([&]() -> int {
    require(c != nullptr && n >= 0, "bad argument");
    for (int s = 0; s < n; s++) {
      cycas_iter_stats st;
      double res[10], rm;
      run_iteration(*c);
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

int cycas_solve_steady(cycas_ctx* c, int32_t max_step, double residual_steady, int32_t cap, int32_t* n_iter,
                       double* res_hist, double* resmax, int32_t* its, int32_t* reasons) {
  return guard([&]() -> int {
    require(c != nullptr && max_step >= 0 && cap >= 0 && n_iter != nullptr, "bad argument");
    require(!c->is_batch && c->tc.scheme == 0, "cycas_solve_steady needs a steady single-case context");
    *n_iter = 0;
    for (int step = 1; step <= max_step; step++) {
      cycas_iter_stats st;
      double res[10], rm;
      run_iteration(*c);
      int rc = finish_iteration(*c, res, &rm, &st);
      const int k = step - 1;
      if (k < cap) {
        if (res_hist) std::memcpy(res_hist + 10L * k, res, sizeof res);
        if (resmax) resmax[k] = rm;
        for (int q = 0; q < 8; q++) {
          if (its) its[8L * k + q] = st.its[q];
          if (reasons) reasons[8L * k + q] = st.reason[q];
        }
      }
      *n_iter = step;
      if (rc != CYCAS_OK) return rc;
      if (rm < residual_steady) break;  // navier.cpp:141-145
    }
    return CYCAS_OK;
  });
}

int cycas_restart_point(cycas_ctx* c, int32_t op) {
  return guard([&]() -> int {
    require(c != nullptr && (op == CYCAS_RESTART_SAVE || op == CYCAS_RESTART_RESTORE), "bad argument");
    long total = 0;
    for (const auto& kv : c->dfields) total += kv.second.second;
    if (op == CYCAS_RESTART_SAVE && !c->restart_point) c->restart_point = c->alloc<double>(total);
    require(c->restart_point != nullptr, "no restart point saved");
    long off = 0;
    for (const auto& kv : c->dfields) {  // std::map: the same order on save and restore
      double* f = kv.second.first;
      const size_t bytes = sizeof(double) * (size_t)kv.second.second;
      double* r = c->restart_point + off;
      if (bytes)
        CK(cudaMemcpyAsync(op == CYCAS_RESTART_SAVE ? r : f, op == CYCAS_RESTART_SAVE ? f : r, bytes,
                           cudaMemcpyDeviceToDevice, c->stream));
      off += kv.second.second;
    }
    if (op == CYCAS_RESTART_RESTORE) c->cur_time = c->restart_time;
    else c->restart_time = c->cur_time;
    return CYCAS_OK;
  });
}

int cycas_time_step(cycas_ctx* c, int32_t cap, int32_t* n_outer, double* res_hist, double* resmax, int32_t* its,
                    int32_t* reasons, double* cur_time) {
  return guard([&]() -> int {
    require(c != nullptr && cap >= 0, "bad argument");
    require(!c->is_batch && c->tc.scheme != 0, "cycas_time_step needs a transient single-case context");
    save_old_level(*c);
    c->cur_time += c->tc.dt;
    double ResMax0 = 0.0;
    int rc = CYCAS_OK, done = 0;
    for (int iter = 1; iter < c->max_outer; iter++) {
      cycas_iter_stats st;
      double res[10], rm;
      run_iteration(*c);
      rc = finish_iteration(*c, res, &rm, &st);
      if (done < cap) {
        if (res_hist) std::memcpy(res_hist + 10L * done, res, sizeof res);
        if (resmax) resmax[done] = rm;
        for (int k = 0; k < 8; k++) {
          if (its) its[8L * done + k] = st.its[k];
          if (reasons) reasons[8L * done + k] = st.reason[k];
        }
      }
      done++;
      if (rc != CYCAS_OK) break;
      if (iter == 1) ResMax0 = rm;
      if (ResMax0 / (rm + 1.e-16) > 100.) break;  // two orders of residual drop (navier.cpp:104-107)
    }
    if (n_outer) *n_outer = done;
    if (cur_time) *cur_time = c->cur_time;
    return rc;
  });
}

}  // extern "C"

namespace {

// the caller's vectors in and out of a device scratch area for the DataPartition::solve* mirrors
double* solve_scratch(cycas_ctx& c) {
  auto it = c.dfields.find("x_solve");
  if (it != c.dfields.end()) return it->second.first;
  return c.dfield("x_solve", 3L * c.m.ncel);
}

KspConf solve_conf(cycas_ctx& c, int sys, double tol, int maxit) {
  require(tol > 0.0 && maxit > 0, "tol and maxIter must be positive");
  KspConf k = c.ksp[sys];
  k.rtol = tol;
  k.maxit = maxit;
  return k;
}

// runs `issue` (which queues the solves), copies the solutions back and reports like an iteration
template <class F>
int run_solves(cycas_ctx& c, double* const* hx, int nx, F issue, cycas_iter_stats* st) {
  require(!c.is_batch, "the solve entry points take a single-case context");
  const long n = c.m.ncel;
  double* d = solve_scratch(c);
  for (int q = 0; q < nx; q++) {
    require(hx[q] != nullptr, "null solution vector");
    CK(cudaMemcpyAsync(d + q * n, hx[q], sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
  }
  CK(cudaMemsetAsync(c.st, 0, sizeof(DevStatus), c.stream));
  c.nsolve = 0;
  issue(d);
  for (int q = 0; q < nx; q++)
    CK(cudaMemcpyAsync(hx[q], d + q * n, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
  return finish_iteration(c, nullptr, nullptr, st);
}

}  // namespace

extern "C" {

int cycas_solve_velocity(cycas_ctx* c, double tol, int32_t maxit, double* xu, double* xv, double* xw,
                         cycas_iter_stats* stats) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    KspConf k = solve_conf(*c, CYCAS_SYS_VELOCITY, tol, maxit);
    double* hx[3] = {xu, xv, xw};
    const long n = c->m.ncel;
    return run_solves(*c, hx, 3, [&](double* d) {
      double* xs[3] = {d, d + n, d + 2 * n};
      solve_velocity(*c, xs, &k);
    }, stats);
  });
}

int cycas_solve_pressure(cycas_ctx* c, double tol, int32_t maxit, double* xp, int32_t is_symmetric,
                         cycas_iter_stats* stats) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    KspConf k = solve_conf(*c, CYCAS_SYS_PRESSURE, tol, maxit);
    if (!is_symmetric) {
      k.type = CYCAS_KSP_GMRES;
      if (k.pc == CYCAS_PC_AMG) k.pc = CYCAS_PC_JACOBI;
    } else if (k.type != CYCAS_KSP_CG) {
      k.type = CYCAS_KSP_CG;
    }
    double* hx[1] = {xp};
    return run_solves(*c, hx, 1, [&](double* d) {
      solve(*c, CYCAS_SYS_PRESSURE, c->f.Ap, c->f.dinv_p, c->f.bp, d, true, &k);
    }, stats);
  });
}

int cycas_solve_scalar(cycas_ctx* c, double tol, int32_t maxit, double* xs, cycas_iter_stats* stats) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    KspConf k = solve_conf(*c, CYCAS_SYS_SCALAR, tol, maxit);
    double* hx[1] = {xs};
    return run_solves(*c, hx, 1, [&](double* d) {
      solve(*c, CYCAS_SYS_SCALAR, c->f.As, c->f.dinv_s, c->f.bs, d, false, &k);
    }, stats);
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
    else if (s == "build_pressure") build_pressure(x);
    else if (s == "correct_cells") correct_cells(x);
    else if (s == "correct_ruface") launch_correct_ruface(x.m, x.f, x.urf[3], x.stream, x.density);
    else if (s == "calculate_velocity") calculate_velocity(x);
    else if (s == "calculate_pressure") calculate_pressure(x);
    else if (s == "keps") update_keps(x);
    else if (s == "build_te") build_te(x);
    else if (s == "build_ed") build_ed(x);
    else if (s == "energy") update_energy(x);
    else if (s == "build_energy") build_energy(x);
    else if (s == "save_transient") save_old_level(x);
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

int cycas_set_graph(cycas_ctx* c, int32_t on) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    require(!(on && c->profiling), "per-solve profiling and graph replay are exclusive");
    if (c->gexec) {
      CK(cudaStreamSynchronize(c->stream));
      CK(cudaGraphExecDestroy(c->gexec));
      c->gexec = nullptr;
    }
    c->use_graph = on != 0;
    return CYCAS_OK;
  });
}

int cycas_set_profiling(cycas_ctx* c, int32_t on) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    require(!(on && c->use_graph), "per-solve profiling and graph replay are exclusive");
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
    const int poly = poly_degree(ksp->pc);
    require(ksp->pc == CYCAS_PC_NONE || ksp->pc == CYCAS_PC_JACOBI || poly, "preconditioner not available in this build");
    require(ksp->type >= CYCAS_KSP_DEFAULT && ksp->type <= CYCAS_KSP_CG, "unknown Krylov type");
    require(!(poly && ksp->type == CYCAS_KSP_CG), "the polynomial preconditioner is for GMRES");
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
    c.kw.v_len = (c.kw.m + 1 + (poly ? (poly >= 3 ? 3 : 2) : 0)) * c.kw.ldv;
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
    g.dinv = ksp->pc == CYCAS_PC_JACOBI || poly ? d_dinv : nullptr;
    g.poly = poly;
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

int cycas_batch_create(const cycas_case* const* cases, int32_t ncases, const cycas_options* opt, cycas_ctx** out) {
  return guard([&]() -> int {
    require(cases && out && ncases >= 1, "bad argument");
    *out = nullptr;
    std::vector<const HostCase*> hs;
    for (int k = 0; k < ncases; k++) {
      require(cases[k] != nullptr, "null case");
      hs.push_back(&cases[k]->hc);
    }
    const HostCase& h0 = *hs[0];
    for (const HostCase* h : hs) {
      bool same = h->turb_model == h0.turb_model && h->density_model == h0.density_model;
      for (int i = 0; i < 8; i++) same = same && h->urf[i] == h0.urf[i];
      for (int i = 0; i < 3; i++) same = same && h->gravity[i] == h0.gravity[i];
      require(same, "batched cases must share the turbulence model, density model, relaxation and gravity");
      require(h->steady && h->density_model == 0 && !h->solve_energy,
              "batches hold steady, isothermal, constant-density cases");
    }
    UnionMesh u = build_union(hs);
    cycas_mesh_view v = view_of(u.h);
    cycas_params p;
    std::memset(&p, 0, sizeof p);
    p.turb_model = h0.turb_model;
    p.density_model = h0.density_model;
    p.cell_pressure_ref = h0.cell_pressure_ref;
    for (int i = 0; i < 8; i++) p.urf[i] = h0.urf[i];
    for (int i = 0; i < 3; i++) p.gravity[i] = h0.gravity[i];
    cycas_ctx* c = new cycas_ctx();
    try {
      init_ctx(*c, &p, opt);
      require(c->ksp[CYCAS_SYS_PRESSURE].pc == CYCAS_PC_AMG, "batches need the AMG pressure preconditioner");
      build_device_mesh(*c, v);
      alloc_fields(*c);
      alloc_krylov(*c);
      setup_batch(*c, u, hs);
      std::vector<std::shared_ptr<const AmgHostHierarchy>> cache(ncases);
      for (int k = 0; k < ncases; k++) cache[k] = cases[k]->amg;
      setup_amg(*c, &cache);
      for (int k = 0; k < ncases; k++) cases[k]->amg = cache[k];
      const HostCase& h = u.h;
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
      delete c;
      throw;
    }
    *out = c;
    return CYCAS_OK;
  });
}

int cycas_batch_size(cycas_ctx* c, int32_t* ncases) {
  return guard([&]() -> int {
    require(c && ncases, "null argument");
    *ncases = c->is_batch ? c->ncases : 1;
    return CYCAS_OK;
  });
}

int cycas_batch_offsets(cycas_ctx* c, int32_t kind, int32_t* off) {
  return guard([&]() -> int {
    require(c && off, "null argument");
    require(kind == 0 || kind == 1, "kind must be 0 (cells) or 1 (boundary faces)");
    if (!c->is_batch) {
      off[0] = 0;
      off[1] = kind == 0 ? c->m.ncel : c->m.nbnd;
      return CYCAS_OK;
    }
    for (int k = 0; k < c->ncases; k++) off[k] = kind == 0 ? c->case_lo[k] : c->bnd0[k];
    off[c->ncases] = kind == 0 ? c->case_hi[c->ncases - 1] : c->bnd0[c->ncases];
    return CYCAS_OK;
  });
}

int cycas_batch_iteration(cycas_ctx* c, double* resmax, int32_t* its, int32_t* reasons) {
  return guard([&]() -> int {
    require(c != nullptr && c->is_batch, "not a batch context");
    run_iteration(*c);
    return finish_batch(*c, resmax, its, reasons);
  });
}

int cycas_batch_residuals(cycas_ctx* c, double* residual) {
  return guard([&]() -> int {
    require(c && residual && c->is_batch, "bad argument");
    std::memcpy(residual, c->h_res.data(), sizeof(double) * 10 * c->ncases);
    return CYCAS_OK;
  });
}

int cycas_batch_copy_case(cycas_ctx* dst, int32_t dc, cycas_ctx* src, int32_t sc) {
  return guard([&]() -> int {
    require(dst && src && dst->is_batch && src->is_batch, "not batch contexts");
    require(dc >= 0 && dc < dst->ncases && sc >= 0 && sc < src->ncases, "case index out of range");
    const long nc = src->case_hi[sc] - src->case_lo[sc], nb = src->bnd0[sc + 1] - src->bnd0[sc];
    const long ni = src->iface0[sc + 1] - src->iface0[sc];
    require(nc == dst->case_hi[dc] - dst->case_lo[dc] && nb == dst->bnd0[dc + 1] - dst->bnd0[dc] &&
                ni == dst->iface0[dc + 1] - dst->iface0[dc],
            "the two cases differ in size");
    CK(cudaStreamSynchronize(src->stream));
    static const char* cells[] = {"U", "V", "W", "P", "R", "T", "TE", "ED", "VisLam", "VisTur", "deltaP"};
    static const char* bnds[] = {"BU", "BV", "BW", "BRo", "BPre", "BTE", "BED", "BTem"};
    for (const char* nm : cells) {
      auto a = lookup(*src, nm), b = lookup(*dst, nm);
      CK(cudaMemcpyAsync(b.first + dst->case_lo[dc], a.first + src->case_lo[sc], sizeof(double) * nc,
                         cudaMemcpyDeviceToDevice, dst->stream));
    }
    for (const char* nm : bnds) {
      auto a = lookup(*src, nm), b = lookup(*dst, nm);
      CK(cudaMemcpyAsync(b.first + dst->bnd0[dc], a.first + src->bnd0[sc], sizeof(double) * nb,
                         cudaMemcpyDeviceToDevice, dst->stream));
    }
    auto a = lookup(*src, "RUFace"), b = lookup(*dst, "RUFace");
    CK(cudaMemcpyAsync(b.first + dst->bnd0[dc], a.first + src->bnd0[sc], sizeof(double) * nb,
                       cudaMemcpyDeviceToDevice, dst->stream));
    CK(cudaMemcpyAsync(b.first + dst->iface0[dc], a.first + src->iface0[sc], sizeof(double) * ni,
                       cudaMemcpyDeviceToDevice, dst->stream));
    CK(cudaStreamSynchronize(dst->stream));
    return CYCAS_OK;
  });
}

int cycas_batch_case_field(cycas_ctx* c, int32_t k, const char* name, double* dst, int64_t n) {
  return guard([&]() -> int {
    require(c && name && dst && c->is_batch && k >= 0 && k < c->ncases, "bad argument");
    auto p = lookup(*c, name);
    long lo, cnt;
    if (p.second == c->m.ncel) {
      lo = c->case_lo[k];
      cnt = c->case_hi[k] - lo;
    } else if (p.second == c->m.nbnd) {
      lo = c->bnd0[k];
      cnt = c->bnd0[k + 1] - lo;
    } else {
      throw StatusError(CYCAS_ERR_INVALID, std::string("no per-case slice of ") + name);
    }
    require(n == cnt, std::string("size mismatch for ") + name);
    CK(cudaMemcpyAsync(dst, p.first + lo, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return CYCAS_OK;
  });
}

int cycas_batch_autotune(cycas_ctx* c, int32_t iters, int32_t* best_grid, double* best_factor, double* best_ms) {
  return guard([&]() -> int {
    require(c != nullptr && c->is_batch && iters >= 1, "bad argument");
    const int G0 = c->kw.nblocks;
    const int grids[3] = {G0, std::max(1, (3 * G0) / 4), std::max(1, G0 / 2)};
    const double factors[3] = {0.5, 1.0, 2.0};
    struct Events {  // destroyed on every way out, errors included
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      ~Events() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
      }
    } ev;
    CK(cudaEventCreate(&ev.e0));
    CK(cudaEventCreate(&ev.e1));
    cudaEvent_t e0 = ev.e0, e1 = ev.e1;
    const bool graph = c->use_graph;
    int bg = G0;
    double bf = 1.0, bms = 1e300;
    int rc = CYCAS_OK;
    for (int gi = 0; gi < 3 && rc == CYCAS_OK; gi++)
      for (int fi = 0; fi < 3 && rc == CYCAS_OK; fi++) {
        build_schedule(*c, grids[gi], factors[fi]);
        if (c->gexec) {
          CK(cudaStreamSynchronize(c->stream));
          CK(cudaGraphExecDestroy(c->gexec));
          c->gexec = nullptr;
        }
        if (graph) run_iteration(*c), rc = finish_batch(*c, nullptr, nullptr, nullptr);  // capture outside the timing
        CK(cudaEventRecord(e0, c->stream));
        for (int k = 0; k < iters && (rc == CYCAS_OK || rc == CYCAS_NOT_CONVERGED); k++) {
          run_iteration(*c);
          rc = finish_batch(*c, nullptr, nullptr, nullptr);
        }
        CK(cudaEventRecord(e1, c->stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (rc == CYCAS_NOT_CONVERGED) rc = CYCAS_OK;
        if (rc == CYCAS_OK && ms < bms) {  // a schedule whose iterations failed stopped early: not a candidate
          bms = ms;
          bg = grids[gi];
          bf = factors[fi];
        }
      }
    build_schedule(*c, bg, bf);
    if (c->gexec) {
      CK(cudaStreamSynchronize(c->stream));
      CK(cudaGraphExecDestroy(c->gexec));
      c->gexec = nullptr;
    }
    if (best_grid) *best_grid = bg;
    if (best_factor) *best_factor = bf;
    if (best_ms) *best_ms = bms / iters;
    return rc;
  });
}

// ---------------------------------------------------------------- result files
int cycas_case_output(const cycas_case* c, int32_t* noutput, int32_t* restart) {
  return guard([&]() -> int {
    require(c != nullptr, "null case");
    if (noutput) *noutput = c->hc.noutput;
    if (restart) *restart = c->hc.restart;
    return CYCAS_OK;
  });
}

int cycas_case_get_field(const cycas_case* c, const char* name, double* dst, int64_t n) {
  return guard([&]() -> int {
    require(c && name && dst, "null argument");
    const HostCase& h = c->hc;
    std::string s(name);
    const std::vector<double>* v = nullptr;
    if (s == "vert") v = &h.vert;
    else if (s == "U") v = &h.U;
    else if (s == "V") v = &h.V;
    else if (s == "W") v = &h.W;
    else if (s == "P") v = &h.P;
    else if (s == "R") v = &h.R;
    else if (s == "T") v = &h.T;
    else if (s == "VisLam") v = &h.VisLam;
    else if (s == "VisTur") v = &h.VisTur;
    else if (s == "TE") v = &h.TE;
    else if (s == "ED") v = &h.ED;
    require(v != nullptr, "unknown case field " + s);
    require((int64_t)v->size() == n, "size mismatch for " + s);
    std::memcpy(dst, v->data(), sizeof(double) * (size_t)n);
    return CYCAS_OK;
  });
}

int cycas_write_grid(const cycas_case* c, const char* path, int32_t binary) {
  return guard([&]() -> int {
    require(c && path, "null argument");
    write_file(path, binary ? geo_bytes(c->hc) : grid_text(c->hc));
    return CYCAS_OK;
  });
}

int cycas_write_tecplot(cycas_ctx* c, int32_t k, const cycas_case* cs, const char* path) {
  return guard([&]() -> int {
    require(c && cs && path, "null argument");
    CaseFields f;
    fetch_case_fields(*c, k, f);
    require(cs->hc.ncel == f.view.ncel && cs->hc.turb_model == c->turb, "the case does not match the context's case");
    write_file(path, tecplot_text(cs->hc.vert.data(), cs->hc.nvrt, cs->hc.cell_vertices.data(), f.view));
    return CYCAS_OK;
  });
}

int cycas_write_data(cycas_ctx* c, int32_t k, const char* path) {
  return guard([&]() -> int {
    require(c && path, "null argument");
    CaseFields f;
    fetch_case_fields(*c, k, f);
    write_file(path, data_bytes(f.view));
    return CYCAS_OK;
  });
}

int cycas_write_backup(cycas_ctx* c, int32_t k, const char* path) {
  return guard([&]() -> int {
    require(c && path, "null argument");
    CaseFields f;
    fetch_case_fields(*c, k, f);
    write_file(path, backup_text(f.view));
    return CYCAS_OK;
  });
}

int cycas_read_backup(cycas_ctx* c, int32_t k, const char* path) {
  return guard([&]() -> int {
    require(c && path, "null argument");
    require(k >= 0 && k < c->ncases, "case index out of range");
    const long lo = c->case_lo[k], n = c->case_hi[k] - lo;
    std::vector<double> a[10];
    double* dst[10];
    for (int i = 0; i < 10; i++) a[i].assign((size_t)n, 0.0), dst[i] = a[i].data();
    read_backup(path, n, c->turb, dst);
    static const char* names[10] = {"R", "U", "V", "W", "P", "T", "VisLam", "VisTur", "TE", "ED"};
    const int nread = c->turb == 1 ? 10 : 7;
    for (int i = 0; i < nread; i++) {
      auto p = lookup(*c, names[i]);
      CK(cudaMemcpyAsync(p.first + lo, a[i].data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return CYCAS_OK;
  });
}

// ---------------------------------------------------------------- asynchronous dumps
int cycas_dump_begin(cycas_ctx* c, int32_t k, const cycas_case* cs, int32_t kinds, const char* tecplot_path,
                     const char* data_path, const char* backup_path) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    require(k >= 0 && k < c->ncases, "case index out of range");
    require(kinds != 0 && (kinds & ~(CYCAS_DUMP_TECPLOT | CYCAS_DUMP_DATA | CYCAS_DUMP_BACKUP)) == 0,
            "kinds must be a non-empty set of CYCAS_DUMP_* bits");
    require(!(kinds & CYCAS_DUMP_TECPLOT) || (cs && tecplot_path), "the Tecplot dump needs the case and a path");
    require(!(kinds & CYCAS_DUMP_DATA) || data_path, "the data dump needs a path");
    require(!(kinds & CYCAS_DUMP_BACKUP) || backup_path, "the backup dump needs a path");
    const long lo = c->case_lo[k], n = c->case_hi[k] - lo;
    if (kinds & CYCAS_DUMP_TECPLOT)
      require(cs->hc.ncel == n && cs->hc.turb_model == c->turb, "the case does not match the context's case");
    DumpState& d = c->dump;
    // one dump in flight: the previous one must have finished with the snapshot and host buffers
    if (d.worker.joinable()) d.worker.join();
    if (d.rc != CYCAS_OK) {
      int rc = d.rc;
      d.rc = CYCAS_OK;
      throw StatusError(rc, "previous dump failed: " + d.err);
    }
    if (!d.side) {
      long cap = 0;
      for (int q = 0; q < c->ncases; q++) cap = std::max(cap, (long)(c->case_hi[q] - c->case_lo[q]));
      CK(cudaStreamCreateWithFlags(&d.side, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&d.ev_snap, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&d.ev_host, cudaEventDisableTiming));
      d.snap = c->alloc<double>(10 * cap);
      void* h = nullptr;
      if (cudaMallocHost(&h, sizeof(double) * 10 * (size_t)std::max(cap, 1L)) != cudaSuccess)
        throw StatusError(CYCAS_ERR_ALLOC, "pinned host buffer of the dump");
      d.host = (double*)h;
      d.cap = cap;
    }
    static const char* names[10] = {"P", "U", "V", "W", "R", "T", "VisLam", "VisTur", "TE", "ED"};
    for (int i = 0; i < 10; i++) {
      auto p = lookup(*c, names[i]);
      CK(cudaMemcpyAsync(d.snap + i * n, p.first + lo, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    }
    CK(cudaEventRecord(d.ev_snap, c->stream));
    CK(cudaStreamWaitEvent(d.side, d.ev_snap, 0));
    CK(cudaMemcpyAsync(d.host, d.snap, sizeof(double) * 10 * n, cudaMemcpyDeviceToHost, d.side));
    CK(cudaEventRecord(d.ev_host, d.side));
    const std::string tp = tecplot_path ? tecplot_path : "", dp = data_path ? data_path : "",
                      bp = backup_path ? backup_path : "";
    const HostCase* hc = (kinds & CYCAS_DUMP_TECPLOT) ? &cs->hc : nullptr;
    const int turb = c->turb, device = c->device, density = c->density;
    const double pref = c->pref;
    d.worker = std::thread([&d, hc, kinds, tp, dp, bp, n, turb, device, density, pref]() {
      try {
        cudaSetDevice(device);
        cudaError_t e = cudaEventSynchronize(d.ev_host);
        if (e != cudaSuccess) throw CudaError(std::string("dump copy: ") + cudaGetErrorString(e));
        CellFieldsView v;
        v.ncel = n;
        v.turb = turb;
        v.density = density;
        v.pref = pref;
        const double* b = d.host;
        v.P = b, v.U = b + n, v.V = b + 2 * n, v.W = b + 3 * n, v.R = b + 4 * n, v.T = b + 5 * n;
        v.VisLam = b + 6 * n, v.VisTur = b + 7 * n, v.TE = b + 8 * n, v.ED = b + 9 * n;
        if (kinds & CYCAS_DUMP_BACKUP) write_file(bp, backup_text(v));
        if (kinds & CYCAS_DUMP_DATA) write_file(dp, data_bytes(v));
        if (kinds & CYCAS_DUMP_TECPLOT)
          write_file(tp, tecplot_text(hc->vert.data(), hc->nvrt, hc->cell_vertices.data(), v));
        d.rc = CYCAS_OK;
      } catch (CudaError& e) {
        d.rc = CYCAS_ERR_CUDA, d.err = e.what();
      } catch (IoError& e) {
        d.rc = CYCAS_ERR_IO, d.err = e.what();
      } catch (std::exception& e) {
        d.rc = CYCAS_ERR_INVALID, d.err = e.what();
      }
    });
    return CYCAS_OK;
  });
}

int cycas_dump_wait(cycas_ctx* c) {
  return guard([&]() -> int {
    require(c != nullptr, "null context");
    DumpState& d = c->dump;
    if (d.worker.joinable()) d.worker.join();
    int rc = d.rc;
    d.rc = CYCAS_OK;
    if (rc != CYCAS_OK) throw StatusError(rc, d.err);
    return CYCAS_OK;
  });
}

}  // extern "C"



