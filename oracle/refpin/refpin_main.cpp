// Main program running the reference's own solver, compiled from its unmodified sources against the
// single-rank runtime of this folder (TEST INFRASTRUCTURE ONLY).
//
//   cycas_ref <case-dir> <out-dir> [--iters N] [--residual R] [PETSc / reference options ...]
//
// Runs, in <case-dir>, the start-up sequence of the reference's main() (NS/main.cpp:22-65:
// initSolverParam, readCommand, broadcastSolverParam, readAndPartition, broadcastPartitionInfo,
// scatterGridFile, ReadGridFile, initPetsc, CreateFaces, CellFaceInfo, CheckAndAllocate,
// InitFlowField), writes the mesh the reference built, then runs the reference's NSSolve
// (NS/navier.cpp:17-156) -- its loop, its stop test, its output cadence -- with MaxStep
// replaced by N and ResidualSteady by R when given, and writes the fields it ends with.
//
// Every array goes to <out-dir>/<name>.bin (raw, native byte order) with a line
// "<name> <f8|i4> <count>" in <out-dir>/manifest.txt.  Besides the fields:
//   residual.bin  [iterations x 10]  the vector NSSolve reduces each iteration (navier.cpp:94)
//   ksp.bin       [solves x 4]       type (0 GMRES, 1 CG), iterations, reason, residual norm
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <unistd.h>
#include <vector>

#include "navier.h"
#include "refpin_runtime.h"

ErrorHandler errorHandler;

namespace {

FILE* g_manifest = nullptr;
std::string g_out;

void dump(const char* name, const void* data, size_t count, bool is_double) {
  std::string path = g_out + "/" + name + ".bin";
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    fprintf(stderr, "cycas_ref: cannot write %s\n", path.c_str());
    exit(2);
  }
  if (count) fwrite(data, is_double ? 8 : 4, count, f);
  fclose(f);
  fprintf(g_manifest, "%s %s %zu\n", name, is_double ? "f8" : "i4", count);
}
void dumpd(const char* name, const std::vector<double>& v) { dump(name, v.data(), v.size(), true); }
void dumpi(const char* name, const std::vector<int>& v) { dump(name, v.data(), v.size(), false); }
void dumpd(const char* name, const double* p, int n) { dump(name, p, (size_t)n, true); }

std::vector<double> rows3(double** a, int n) {
  std::vector<double> v(3 * (size_t)n);
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) v[3 * i + d] = a[i][d];
  return v;
}

void dump_mesh(NavierStokesSolver& ns) {
  int nf = ns.Nfac, nc = ns.Ncel, nb = ns.Nbnd;
  std::vector<int> c1(nf), c2(nf), fb(nf), fv(4 * (size_t)nf);
  std::vector<double> fx(3 * (size_t)nf), fn(3 * (size_t)nf), fpac(3 * (size_t)nf), fnac(3 * (size_t)nf);
  std::vector<double> area(nf), lam(nf), rlc(nf);
  for (int i = 0; i < nf; ++i) {
    const FaceData& F = ns.Face[i];
    c1[i] = F.cell1; c2[i] = F.cell2; fb[i] = F.bnd;
    for (int k = 0; k < 4; ++k) fv[4 * i + k] = F.vertices[k];
    for (int d = 0; d < 3; ++d) {
      fx[3 * i + d] = F.x[d]; fn[3 * i + d] = F.n[d]; fpac[3 * i + d] = F.Xpac[d]; fnac[3 * i + d] = F.Xnac[d];
    }
    area[i] = F.area; lam[i] = F.lambda; rlc[i] = F.rlencos;
  }
  dumpi("face_cell1", c1); dumpi("face_cell2", c2); dumpi("face_bnd", fb); dumpi("face_vertices", fv);
  dumpd("face_x", fx); dumpd("face_n", fn); dumpd("face_xpac", fpac); dumpd("face_xnac", fnac);
  dumpd("face_area", area); dumpd("face_lambda", lam); dumpd("face_rlencos", rlc);

  std::vector<int> nface(nc), rid(nc), cf(6 * (size_t)nc), cc(6 * (size_t)nc), cv(8 * (size_t)nc), gi(nc);
  std::vector<double> vol(nc), cx(3 * (size_t)nc);
  for (int i = 0; i < nc; ++i) {
    const CellData& C = ns.Cell[i];
    nface[i] = C.nface; rid[i] = C.rid; gi[i] = C.globalIdx; vol[i] = C.vol;
    for (int k = 0; k < 6; ++k) { cf[6 * i + k] = C.face[k]; cc[6 * i + k] = C.cell[k]; }
    for (int k = 0; k < 8; ++k) cv[8 * i + k] = C.vertices[k];
    for (int d = 0; d < 3; ++d) cx[3 * i + d] = C.x[d];
  }
  dumpi("cell_nface", nface); dumpi("cell_rid", rid); dumpi("cell_face", cf); dumpi("cell_cell", cc);
  dumpi("cell_vertices", cv); dumpi("cell_globalidx", gi); dumpd("cell_vol", vol); dumpd("cell_x", cx);

  std::vector<int> bf(nb), brid(nb), bv(4 * (size_t)nb);
  std::vector<double> dist(nb);
  for (int i = 0; i < nb; ++i) {
    const BoundaryData& B = ns.Bnd[i];
    bf[i] = B.face; brid[i] = B.rid; dist[i] = B.distance;
    for (int k = 0; k < 4; ++k) bv[4 * i + k] = B.vertices[k];
  }
  dumpi("bnd_face", bf); dumpi("bnd_rid", brid); dumpi("bnd_vertices", bv); dumpd("bnd_distance", dist);
  std::vector<double> vert(3 * (size_t)ns.Nvrt);
  for (int i = 0; i < ns.Nvrt; ++i)
    for (int d = 0; d < 3; ++d) vert[3 * i + d] = ns.Vert[i][d];
  dumpd("vert", vert);
}

void dump_fields(NavierStokesSolver& ns) {
  int nc = ns.Ncel, nb = ns.Nbnd;
  dumpd("U", ns.Un, nc); dumpd("V", ns.Vn, nc); dumpd("W", ns.Wn, nc); dumpd("P", ns.Pn, nc);
  dumpd("R", ns.Rn, nc); dumpd("T", ns.Tn, nc); dumpd("VisLam", ns.VisLam, nc); dumpd("VisTur", ns.VisTur, nc);
  dumpd("deltaP", ns.deltaP, nc); dumpd("Apr", ns.Apr, nc); dumpd("RUFace", ns.RUFace, ns.Nfac);
  if (ns.TurModel == 1) { dumpd("TE", ns.TE, nc); dumpd("ED", ns.ED, nc); dumpd("BTE", ns.BTE, nb); dumpd("BED", ns.BED, nb); }
  dumpd("BU", ns.BU, nb); dumpd("BV", ns.BV, nb); dumpd("BW", ns.BW, nb); dumpd("BRo", ns.BRo, nb);
  dumpd("BPre", ns.BPre, nb);
  dumpd("dPdX", rows3(ns.dPdX, nc)); dumpd("dUdX", rows3(ns.dUdX, nc));
  dumpd("dVdX", rows3(ns.dVdX, nc)); dumpd("dWdX", rows3(ns.dWdX, nc));
  std::vector<double> res;
  for (const auto& v : refpin::allreduce_log())
    if (v.size() == RESIDUAL_LEN) res.insert(res.end(), v.begin(), v.end());
  dumpd("residual", res);
  std::vector<double> ksp;
  for (const auto& k : refpin::ksp_log()) {
    ksp.push_back(k.type); ksp.push_back(k.its); ksp.push_back(k.reason); ksp.push_back(k.rnorm);
  }
  dumpd("ksp", ksp);
  std::vector<int> info = {ns.Ncel, ns.Nfac, ns.Nbnd, ns.Nvrt, ns.step, ns.TurModel};
  dumpi("info", info);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: cycas_ref <case-dir> <out-dir> [--iters N] [--residual R] [options]\n");
    return 2;
  }
  std::string case_dir = argv[1];
  g_out = argv[2];
  int iters = -1;
  double residual = -1.0;
  std::vector<char*> args = {argv[0]};
  for (int i = 3; i < argc; ++i) {
    if (!strcmp(argv[i], "--iters") && i + 1 < argc) iters = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--residual") && i + 1 < argc) residual = atof(argv[++i]);
    else args.push_back(argv[i]);
  }
  if (g_out[0] != '/') {
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return 2;
    g_out = std::string(cwd) + "/" + g_out;
  }
  if (chdir(case_dir.c_str()) != 0) {
    fprintf(stderr, "cycas_ref: no case directory %s\n", case_dir.c_str());
    return 2;
  }
  // the reference writes its log, result and geometry files below the working directory
  for (const char* d : {"log", "tec", "geo", "res"}) {
    std::string cmd = std::string("mkdir -p ") + d;
    if (system(cmd.c_str()) != 0) return 2;
  }
  std::string mf = g_out + "/manifest.txt";
  g_manifest = fopen(mf.c_str(), "w");
  if (!g_manifest) {
    fprintf(stderr, "cycas_ref: cannot write %s\n", mf.c_str());
    return 2;
  }
  int pargc = (int)args.size();
  char** pargv = args.data();
  PetscInitialize(&pargc, &pargv, NULL, NULL);

  std::map<std::string, bool> commandline;
  observeCommand(commandline, "-readLocally");
  observeCommand(commandline, "-mshBinary");
  observeCommand(commandline, "-outBinary");
  observeCommand(commandline, "-cgns");
  parseCommand(commandline);

  NavierStokesSolver* ns = new NavierStokesSolver;
  ns->initSolverParam();
  ns->readCommand(commandline);
  ns->broadcastSolverParam();
  int* elementBuffer = NULL;
  double* vertexBuffer = NULL;
  int* interfaceBuffer = NULL;
  ns->readAndPartition(getCommand(commandline, "-mshBinary"), getCommand(commandline, "-cgns"));
  ns->broadcastPartitionInfo();
  ns->scatterGridFile(&elementBuffer, &vertexBuffer, &interfaceBuffer);
  ns->ReadGridFile(elementBuffer, vertexBuffer, interfaceBuffer);
  ns->dataPartition->initPetsc();
  ns->CreateFaces();
  ns->CellFaceInfo();
  ns->CheckAndAllocate();
  ns->InitFlowField();
  dump_mesh(*ns);

  if (iters >= 0) ns->MaxStep = iters;
  if (residual >= 0) ns->ResidualSteady = residual;
  refpin::clear_logs();
  ns->NSSolve();
  dump_fields(*ns);
  fclose(g_manifest);
  fflush(stdout);
  // the reference's destructors and PETSc teardown are not needed for the comparison
  _exit(0);
}
