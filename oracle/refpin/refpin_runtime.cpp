// Single-rank runtime behind oracle/refpin/include/{mpi,petscsys,petscksp,metis,cgnslib}.h
// (TEST INFRASTRUCTURE ONLY).
//
// It lets the reference's own, unmodified C++ sources run as one process, so that the oracle's
// restatement can be checked against the code it restates.  Nothing here computes physics:
//   * MPI: rank 0 of a communicator of size 1.  Collectives copy; messages to oneself are queued
//     and matched by tag; every MPI_Allreduce of doubles is also appended to a log, which is how
//     refpin_main.cpp reads the residual vector NSSolve reduces each iteration (navier.cpp:94).
//   * PETSc: Vec is a double array; Mat keeps the union of every entry ever set (explicit zeros
//     included) with sorted columns; KSPSolve hands the assembled matrix to the oracle's
//     GMRES / CG (oracle/oracle_krylov.cpp) with the options PETSc would apply, and logs the
//     iteration count, reason and residual norm of every solve.
//   * METIS: one part (every element in part 0, dual graph without edges).
//   * CGNS: not available (cg_open fails).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <sys/time.h>
#include <utility>
#include <vector>

#include "cgnslib.h"
#include "metis.h"
#include "petscksp.h"
#include "../oracle.h"
#include "refpin_runtime.h"

// ------------------------------------------------------------------------------------------ MPI
namespace {

std::map<int, size_t> g_type_size = {{MPI_CHAR, 1}, {MPI_INT, 4}, {MPI_DOUBLE, 8}, {MPI_LONG, 8},
                                     {MPI_UNSIGNED_LONG, 8}};
int g_next_type = 100;

size_t type_size(MPI_Datatype t) {
  auto it = g_type_size.find(t);
  if (it == g_type_size.end()) {
    fprintf(stderr, "refpin: unknown MPI datatype %d\n", t);
    exit(3);
  }
  return it->second;
}

struct Message { int tag; std::vector<char> bytes; };
struct PendingRecv { int tag; void* buf; size_t cap; int req; };
std::deque<Message> g_messages;
std::vector<PendingRecv> g_recvs;
std::vector<char> g_req_done;

int new_request(bool done) {
  g_req_done.push_back(done ? 1 : 0);
  return (int)g_req_done.size() - 1;
}

void deliver(Message& m, void* buf, size_t cap) {
  if (m.bytes.size() > cap) {
    fprintf(stderr, "refpin: message of %zu bytes (tag %d) into a %zu-byte receive\n", m.bytes.size(), m.tag, cap);
    exit(3);
  }
  if (!m.bytes.empty()) memcpy(buf, m.bytes.data(), m.bytes.size());
}

void post_send(const void* buf, int count, MPI_Datatype type, int dest, int tag) {
  if (dest != 0) {
    fprintf(stderr, "refpin: send to rank %d in a one-rank run\n", dest);
    exit(3);
  }
  Message m;
  m.tag = tag;
  size_t n = (size_t)count * type_size(type);
  m.bytes.assign((const char*)buf, (const char*)buf + n);
  for (size_t i = 0; i < g_recvs.size(); ++i) {
    if (g_recvs[i].tag == tag) {
      deliver(m, g_recvs[i].buf, g_recvs[i].cap);
      g_req_done[g_recvs[i].req] = 1;
      g_recvs.erase(g_recvs.begin() + i);
      return;
    }
  }
  g_messages.push_back(std::move(m));
}

bool take_message(int tag, void* buf, size_t cap) {
  for (auto it = g_messages.begin(); it != g_messages.end(); ++it) {
    if (it->tag == tag) {
      deliver(*it, buf, cap);
      g_messages.erase(it);
      return true;
    }
  }
  return false;
}

std::vector<std::vector<double>> g_allreduce_log;
std::vector<refpin::KspRecord> g_ksp_log;

}  // namespace

struct refpin_file { FILE* f; };

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize() { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) {
  fflush(stdout);
  fprintf(stderr, "refpin: MPI_Abort(%d) called by the reference\n", code);
  exit(3);
}
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op, MPI_Comm) {
  if (sendbuf != MPI_IN_PLACE) memcpy(recvbuf, sendbuf, (size_t)count * type_size(type));
  if (type == MPI_DOUBLE) {
    const double* v = (const double*)recvbuf;
    g_allreduce_log.emplace_back(v, v + count);
  }
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op, int, MPI_Comm) {
  if (sendbuf != MPI_IN_PLACE) memcpy(recvbuf, sendbuf, (size_t)count * type_size(type));
  return MPI_SUCCESS;
}
int MPI_Allgather(const void* sendbuf, int scount, MPI_Datatype stype, void* recvbuf, int, MPI_Datatype, MPI_Comm) {
  memcpy(recvbuf, sendbuf, (size_t)scount * type_size(stype));
  return MPI_SUCCESS;
}
int MPI_Scatter(const void* sendbuf, int scount, MPI_Datatype stype, void* recvbuf, int, MPI_Datatype, int,
                MPI_Comm) {
  memcpy(recvbuf, sendbuf, (size_t)scount * type_size(stype));
  return MPI_SUCCESS;
}
int MPI_Scatterv(const void* sendbuf, const int* scounts, const int* displs, MPI_Datatype stype, void* recvbuf, int,
                 MPI_Datatype, int, MPI_Comm) {
  size_t s = type_size(stype);
  memcpy(recvbuf, (const char*)sendbuf + (size_t)displs[0] * s, (size_t)scounts[0] * s);
  return MPI_SUCCESS;
}
int MPI_Gatherv(const void* sendbuf, int scount, MPI_Datatype stype, void* recvbuf, const int*, const int* displs,
                MPI_Datatype rtype, int, MPI_Comm) {
  memcpy((char*)recvbuf + (size_t)displs[0] * type_size(rtype), sendbuf, (size_t)scount * type_size(stype));
  return MPI_SUCCESS;
}
int MPI_Issend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm, MPI_Request* req) {
  post_send(buf, count, type, dest, tag);
  *req = new_request(true);
  return MPI_SUCCESS;
}
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm c, MPI_Request* req) {
  return MPI_Issend(buf, count, type, dest, tag, c, req);
}
int MPI_Bsend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm) {
  post_send(buf, count, type, dest, tag);
  return MPI_SUCCESS;
}
int MPI_Send(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm c) {
  return MPI_Bsend(buf, count, type, dest, tag, c);
}
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm, MPI_Request* req) {
  size_t cap = (size_t)count * type_size(type);
  if (take_message(tag, buf, cap)) {
    *req = new_request(true);
  } else {
    *req = new_request(false);
    g_recvs.push_back({tag, buf, cap, *req});
  }
  return MPI_SUCCESS;
}
int MPI_Recv(void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm, MPI_Status* status) {
  if (!take_message(tag, buf, (size_t)count * type_size(type))) {
    fprintf(stderr, "refpin: blocking receive (tag %d) with no message queued: a one-rank deadlock\n", tag);
    exit(3);
  }
  if (status) status->MPI_TAG = tag;
  return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request* req, MPI_Status*) {
  if (!g_req_done.at(*req)) {
    fprintf(stderr, "refpin: wait on a receive nobody sends: a one-rank deadlock\n");
    exit(3);
  }
  return MPI_SUCCESS;
}
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status*) {
  for (int i = 0; i < count; ++i) MPI_Wait(reqs + i, nullptr);
  return MPI_SUCCESS;
}
int MPI_Get_address(const void* location, MPI_Aint* address) {
  *address = (MPI_Aint)location;
  return MPI_SUCCESS;
}
int MPI_Type_create_struct(int count, const int* lens, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* newtype) {
  size_t extent = 0;
  for (int i = 0; i < count; ++i) {
    size_t end = (size_t)displs[i] + (size_t)lens[i] * type_size(types[i]);
    if (end > extent) extent = end;
  }
  *newtype = g_next_type++;
  g_type_size[*newtype] = extent;
  return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
int MPI_Buffer_attach(void*, int) { return MPI_SUCCESS; }
int MPI_File_open(MPI_Comm, const char* name, int amode, MPI_Info, MPI_File* fh) {
  FILE* f = fopen(name, "r+b");
  if (!f && (amode & MPI_MODE_CREATE)) f = fopen(name, "w+b");
  if (!f) return MPI_ERR_OTHER;
  *fh = new refpin_file{f};
  return MPI_SUCCESS;
}
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype, MPI_Datatype, const char*, MPI_Info) {
  return fseeko(fh->f, (off_t)disp, SEEK_SET) == 0 ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype type, MPI_Status*) {
  size_t n = (size_t)count * type_size(type);
  return fwrite(buf, 1, n, fh->f) == n ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_File_close(MPI_File* fh) {
  fclose((*fh)->f);
  delete *fh;
  *fh = nullptr;
  return MPI_SUCCESS;
}
double MPI_Wtime() {
  timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}

// ---------------------------------------------------------------------------------------- PETSc
namespace {
std::map<std::string, std::string> g_options;   // "-name" -> value ("" for a bare flag)

bool option(const char* name, std::string* value) {
  auto it = g_options.find(name);
  if (it == g_options.end()) return false;
  if (value) *value = it->second;
  return true;
}

bool looks_like_value(const char* s) {
  if (s[0] != '-') return true;
  char* end = nullptr;
  strtod(s, &end);
  return end && *end == '\0';
}
}  // namespace

PetscErrorCode PetscInitialize(int* argc, char*** argv, const char*, const char*) {
  for (int i = 1; i < *argc; ++i) {
    const char* a = (*argv)[i];
    if (a[0] != '-' || looks_like_value(a)) continue;
    if (i + 1 < *argc && looks_like_value((*argv)[i + 1])) {
      g_options[a] = (*argv)[i + 1];
      ++i;
    } else {
      g_options[a] = "";
    }
  }
  return 0;
}
PetscErrorCode PetscFinalize() { return 0; }
PetscErrorCode PetscPrintf(MPI_Comm, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vprintf(fmt, ap);
  va_end(ap);
  return 0;
}
PetscErrorCode PetscOptionsGetString(PetscOptions, const char*, const char* name, char* value, size_t len,
                                     PetscBool* set) {
  std::string v;
  bool have = option(name, &v) && !v.empty();
  if (have) {
    strncpy(value, v.c_str(), len - 1);
    value[len - 1] = '\0';
  }
  if (set) *set = have ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetBool(PetscOptions, const char*, const char* name, PetscBool* value, PetscBool* set) {
  std::string v;
  bool have = option(name, &v);
  if (have) {
    bool f = v == "0" || v == "false" || v == "no" || v == "FALSE";
    *value = f ? PETSC_FALSE : PETSC_TRUE;
  }
  if (set) *set = have ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscLogStageRegister(const char*, PetscLogStage*) { return 0; }
PetscErrorCode PetscLogStagePush(PetscLogStage) { return 0; }
PetscErrorCode PetscLogStagePop() { return 0; }

struct refpin_vec { int n = 0; double* a = nullptr; bool own = false; };

// rows[i] holds (column, value) pairs in ascending column order
struct refpin_mat { int n = 0; std::vector<std::vector<std::pair<int, double>>> rows; bool symmetric = false; };

struct refpin_ksp {
  Mat A = nullptr;
  std::string type = KSPGMRES;
  bool nonzero_guess = false;
  double rtol = 1e-5, abstol = 1e-50, dtol = 1e4;
  int maxit = 10000, restart = 30, pc = orc::PC_ILU0;
  int its = 0, reason = 0;
  double rnorm = 0;
};

PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt n, PetscInt, Vec* v) {
  *v = new refpin_vec;
  (*v)->n = n;
  (*v)->a = new double[n > 0 ? n : 1]();
  (*v)->own = true;
  return 0;
}
PetscErrorCode VecCreateMPIWithArray(MPI_Comm, PetscInt, PetscInt n, PetscInt, const PetscScalar* array, Vec* v) {
  *v = new refpin_vec;
  (*v)->n = n;
  (*v)->a = const_cast<double*>(array);
  (*v)->own = false;
  return 0;
}
PetscErrorCode VecDuplicate(Vec v, Vec* out) { return VecCreateMPI(0, v->n, v->n, out); }
PetscErrorCode VecSet(Vec v, PetscScalar a) {
  for (int i = 0; i < v->n; ++i) v->a[i] = a;
  return 0;
}
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar a, InsertMode mode) {
  if (i < 0 || i >= v->n) {
    fprintf(stderr, "refpin: VecSetValue index %d outside [0,%d)\n", i, v->n);
    exit(3);
  }
  if (mode == ADD_VALUES) v->a[i] += a; else v->a[i] = a;
  return 0;
}
PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
PetscErrorCode VecNorm(Vec v, NormType type, PetscReal* out) {
  double s = 0;
  for (int i = 0; i < v->n; ++i) {
    double x = std::fabs(v->a[i]);
    if (type == NORM_1) s += x;
    else if (type == NORM_INFINITY) s = x > s ? x : s;
    else s += x * x;
  }
  *out = type == NORM_2 ? std::sqrt(s) : s;
  return 0;
}
PetscErrorCode VecGetArray(Vec v, PetscScalar** a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec, PetscScalar**) { return 0; }
PetscErrorCode VecView(Vec, PetscViewer) { return 0; }
PetscErrorCode VecDestroy(Vec* v) {
  if (*v) {
    if ((*v)->own) delete[] (*v)->a;
    delete *v;
    *v = nullptr;
  }
  return 0;
}

PetscErrorCode MatCreate(MPI_Comm, Mat* m) { *m = new refpin_mat; return 0; }
PetscErrorCode MatSetSizes(Mat m, PetscInt n, PetscInt, PetscInt, PetscInt) {
  m->n = n;
  m->rows.assign(n, {});
  return 0;
}
PetscErrorCode MatSetType(Mat, MatType) { return 0; }
PetscErrorCode MatMPIAIJSetPreallocation(Mat, PetscInt, const PetscInt*, PetscInt, const PetscInt*) { return 0; }
PetscErrorCode MatSetValue(Mat m, PetscInt i, PetscInt j, PetscScalar v, InsertMode mode) {
  if (i < 0 || i >= m->n || j < 0 || j >= m->n) {
    fprintf(stderr, "refpin: MatSetValue (%d,%d) outside a %d-row matrix\n", i, j, m->n);
    exit(3);
  }
  auto& row = m->rows[i];
  size_t lo = 0, hi = row.size();
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if (row[mid].first < j) lo = mid + 1; else hi = mid;
  }
  if (lo < row.size() && row[lo].first == j) {
    if (mode == ADD_VALUES) row[lo].second += v; else row[lo].second = v;
  } else {
    row.insert(row.begin() + lo, std::make_pair((int)j, (double)v));
  }
  return 0;
}
PetscErrorCode MatSetValues(Mat m, PetscInt nr, const PetscInt* rows, PetscInt nc, const PetscInt* cols,
                            const PetscScalar* v, InsertMode mode) {
  for (int r = 0; r < nr; ++r)
    for (int c = 0; c < nc; ++c) MatSetValue(m, rows[r], cols[c], v[r * nc + c], mode);
  return 0;
}
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatZeroEntries(Mat m) {
  for (auto& row : m->rows)
    for (auto& e : row) e.second = 0.0;
  return 0;
}
PetscErrorCode MatSetOption(Mat m, MatOption op, PetscBool flag) {
  if (op == MAT_SYMMETRIC) m->symmetric = flag == PETSC_TRUE;
  return 0;
}
PetscErrorCode MatGetOwnershipRange(Mat m, PetscInt* lo, PetscInt* hi) { *lo = 0; *hi = m->n; return 0; }
PetscErrorCode MatView(Mat, PetscViewer) { return 0; }
PetscErrorCode MatDestroy(Mat* m) { delete *m; *m = nullptr; return 0; }

PetscErrorCode KSPCreate(MPI_Comm, KSP* ksp) { *ksp = new refpin_ksp; return 0; }
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat) { ksp->A = A; return 0; }
PetscErrorCode KSPSetType(KSP ksp, KSPType type) { ksp->type = type; return 0; }
PetscErrorCode KSPSetInitialGuessNonzero(KSP ksp, PetscBool flag) { ksp->nonzero_guess = flag == PETSC_TRUE; return 0; }
PetscErrorCode KSPSetTolerances(KSP ksp, PetscReal rtol, PetscReal abstol, PetscReal dtol, PetscInt maxits) {
  // PETSC_DEFAULT leaves a tolerance at its current value
  if (rtol != PETSC_DEFAULT) ksp->rtol = rtol;
  if (abstol != PETSC_DEFAULT) ksp->abstol = abstol;
  if (dtol != PETSC_DEFAULT) ksp->dtol = dtol;
  if (maxits != PETSC_DEFAULT) ksp->maxit = maxits;
  return 0;
}
PetscErrorCode KSPSetFromOptions(KSP ksp) {
  std::string v;
  if (option("-ksp_type", &v)) ksp->type = v;
  if (option("-ksp_rtol", &v)) ksp->rtol = atof(v.c_str());
  if (option("-ksp_atol", &v)) ksp->abstol = atof(v.c_str());
  if (option("-ksp_divtol", &v)) ksp->dtol = atof(v.c_str());
  if (option("-ksp_max_it", &v)) ksp->maxit = atoi(v.c_str());
  if (option("-ksp_gmres_restart", &v)) ksp->restart = atoi(v.c_str());
  std::string pc = "ilu";
  if (option("-pc_type", &v)) pc = v;
  // block Jacobi on one rank is its sub-preconditioner on the whole matrix (ILU(0) by default)
  if (pc == "bjacobi") {
    pc = "ilu";
    if (option("-sub_pc_type", &v)) pc = v;
  }
  if (pc == "ilu") ksp->pc = orc::PC_ILU0;
  else if (pc == "jacobi") ksp->pc = orc::PC_JACOBI;
  else if (pc == "none") ksp->pc = orc::PC_NONE;
  else {
    fprintf(stderr, "refpin: preconditioner '%s' is not available\n", pc.c_str());
    exit(3);
  }
  return 0;
}
PetscErrorCode KSPSetUp(KSP) { return 0; }
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x) {
  const refpin_mat& M = *ksp->A;
  orc::Csr A;
  A.n = M.n;
  A.rowptr.assign(M.n + 1, 0);
  A.diag.assign(M.n, -1);
  for (int i = 0; i < M.n; ++i) A.rowptr[i + 1] = A.rowptr[i] + (int)M.rows[i].size();
  A.col.resize(A.rowptr[M.n]);
  A.val.resize(A.rowptr[M.n]);
  for (int i = 0; i < M.n; ++i) {
    int k = A.rowptr[i];
    for (const auto& e : M.rows[i]) {
      if (e.first == i) A.diag[i] = k;
      A.col[k] = e.first;
      A.val[k] = e.second;
      ++k;
    }
  }
  orc::KspSettings s;
  s.type = ksp->type == KSPCG ? orc::KSP_CG : orc::KSP_GMRES;
  s.restart = ksp->restart;
  s.pc = ksp->pc;
  s.abstol = ksp->abstol;
  s.dtol = ksp->dtol;
  orc::KspResult r = orc::ksp_solve(A, s, ksp->rtol, ksp->maxit, !ksp->nonzero_guess, b->a, x->a);
  ksp->its = r.its;
  ksp->reason = r.reason;
  ksp->rnorm = r.rnorm;
  g_ksp_log.push_back({s.type, r.its, r.reason, r.rnorm});
  return 0;
}
PetscErrorCode KSPGetConvergedReason(KSP ksp, KSPConvergedReason* reason) { *reason = ksp->reason; return 0; }
PetscErrorCode KSPGetIterationNumber(KSP ksp, PetscInt* its) { *its = ksp->its; return 0; }
PetscErrorCode KSPGetResidualNorm(KSP ksp, PetscReal* rnorm) { *rnorm = ksp->rnorm; return 0; }
PetscErrorCode KSPGetPC(KSP ksp, PC* pc) { *pc = ksp; return 0; }
PetscErrorCode KSPView(KSP, PetscViewer) { return 0; }
PetscErrorCode KSPDestroy(KSP* ksp) { delete *ksp; *ksp = nullptr; return 0; }

// ---------------------------------------------------------------------------------------- METIS
int METIS_MeshToDual(idx_t* ne, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t** xadj, idx_t** adjncy) {
  *xadj = (idx_t*)calloc((size_t)*ne + 1, sizeof(idx_t));
  *adjncy = (idx_t*)calloc(1, sizeof(idx_t));
  return METIS_OK;
}
int METIS_PartGraphKway(idx_t* nvtxs, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t* nparts, real_t*,
                        real_t*, idx_t*, idx_t* edgecut, idx_t* part) {
  if (*nparts != 1) {
    fprintf(stderr, "refpin: %d parts requested from the one-part partitioner\n", *nparts);
    exit(3);
  }
  for (idx_t i = 0; i < *nvtxs; ++i) part[i] = 0;
  *edgecut = 0;
  return METIS_OK;
}
int METIS_Free(void* ptr) { free(ptr); return METIS_OK; }

// ----------------------------------------------------------------------------------------- CGNS
const char* DataTypeName[] = {"Null", "UserDefined", "Integer", "RealSingle", "RealDouble", "Character",
                              "LongInteger"};
const char* cg_get_error() { return "CGNS input is not available in the single-rank reference build"; }
const char* cg_ZoneTypeName(ZoneType_t) { return "Null"; }
const char* cg_ElementTypeName(ElementType_t) { return "Null"; }
int cg_open(const char*, int, int*) { return CG_ERROR; }
int cg_close(int) { return CG_ERROR; }
int cg_version(int, float*) { return CG_ERROR; }
int cg_zone_read(int, int, int, char*, cgsize_t*) { return CG_ERROR; }
int cg_zone_type(int, int, int, ZoneType_t*) { return CG_ERROR; }
int cg_ncoords(int, int, int, int*) { return CG_ERROR; }
int cg_coord_info(int, int, int, int, DataType_t*, char*) { return CG_ERROR; }
int cg_coord_read(int, int, int, const char*, DataType_t, const cgsize_t*, const cgsize_t*, void*) { return CG_ERROR; }
int cg_nsections(int, int, int, int*) { return CG_ERROR; }
int cg_section_read(int, int, int, int, char*, ElementType_t*, cgsize_t*, cgsize_t*, int*, int*) { return CG_ERROR; }
int cg_ElementDataSize(int, int, int, int, cgsize_t*) { return CG_ERROR; }
int cg_elements_read(int, int, int, int, cgsize_t*, cgsize_t*) { return CG_ERROR; }
int cg_npe(ElementType_t, int*) { return CG_ERROR; }

// ---------------------------------------------------------------------------------------- logs
namespace refpin {
const std::vector<std::vector<double>>& allreduce_log() { return g_allreduce_log; }
const std::vector<KspRecord>& ksp_log() { return g_ksp_log; }
void clear_logs() {
  g_allreduce_log.clear();
  g_ksp_log.clear();
}
}  // namespace refpin
