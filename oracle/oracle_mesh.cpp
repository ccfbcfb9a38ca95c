// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h; parity unpinned at the PETSc boundary).
// Setup path of the reference at one MPI rank: param.in, gmsh read, the N=1
// element reorder, face construction, geometry, initial fields.
#include "oracle.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <set>
#include <stdexcept>

namespace orc {

// ---- small vector helpers with the reference's summation order (tools.cpp:16-51) ----
static inline void vminus(double* a, const double* b, const double* c) {
  for (int i = 0; i < 3; i++) a[i] = b[i] - c[i];
}
static inline double vdot(const double* a, const double* b) {
  double s = 0.;
  for (int i = 0; i < 3; i++) s += a[i] * b[i];
  return s;
}
static inline double vlen(const double* a) {
  double s = 0.;
  for (int i = 0; i < 3; i++) s += a[i] * a[i];
  return std::sqrt(s);
}
static inline void vcross(double* a, const double* b, const double* c) {
  a[0] = b[1] * c[2] - b[2] * c[1];
  a[1] = -b[0] * c[2] + b[2] * c[0];
  a[2] = b[0] * c[1] - b[1] * c[0];
}

// ---- param.in (readparamfile.cpp:10-344) ----
static char* trim(char* str) {  // tools.cpp trimwhitespace
  while (std::isspace((unsigned char)*str)) str++;
  if (*str == 0) return str;
  char* end = str + std::strlen(str) - 1;
  while (end > str && std::isspace((unsigned char)*end)) end--;
  *(end + 1) = 0;
  return str;
}

void read_param_file(Case& cs, const std::string& path) {
  std::ifstream fin(path.c_str());
  if (!fin.is_open()) throw std::runtime_error("param file not found: " + path);
  std::string str;
  int line = 0;
  char buf[20][64];
  while (std::getline(fin, str)) {
    line++;
    if (str.size() >= 2 && str[0] == '/' && str[1] == '/') continue;
    if (str.size() == 1 || str.size() == 0) continue;
    int ikey = 0, j = 0;
    for (int i = 0; i < 20; i++) buf[i][0] = 0;
    for (size_t i = 0; i < str.size() && str[i] != '\0'; i++) {
      if (str[i] != ',') {
        if (j < 63) buf[ikey][j++] = str[i];
      } else {
        buf[ikey][j] = 0;
        if (ikey < 19) ikey++;
        j = 0;
      }
    }
    buf[ikey][j] = 0;
    char* k[20];
    for (int i = 0; i < 20; i++) k[i] = trim(buf[i]);
    auto fail = [&](const std::string& m) {
      throw std::runtime_error("Error in reading param.in line " + std::to_string(line) + ": " + m);
    };
    if (!std::strcmp(k[0], "gridfile")) {
      cs.GridFileName = k[1];
    } else if (!std::strcmp(k[0], "steady")) {
      cs.IfSteady = 1;
      cs.MaxStep = std::atoi(k[1]);
      cs.ResidualSteady = std::atof(k[2]);
    } else if (!std::strcmp(k[0], "transient")) {  // readparamfile.cpp:84-101
      if (ikey != 4) fail("transient requies 3 parameters");
      cs.IfSteady = 0;
      cs.dt = std::atof(k[1]);
      cs.total_time = std::atof(k[2]);
      cs.MaxStep = (int)(cs.total_time / cs.dt);
      cs.MaxOuterStep = (int)std::atof(k[3]);
      if (!std::strcmp(k[4], "Euler")) cs.TimeScheme = 1;
      else if (!std::strcmp(k[4], "Dual")) cs.TimeScheme = 2;
      else fail(std::string("unknown time scheme: ") + k[4]);
    } else if (!std::strcmp(k[0], "energy")) {
      if (!std::strcmp(k[1], "on")) cs.SolveEnergy = 1;
      else if (!std::strcmp(k[1], "off")) cs.SolveEnergy = 0;
      else fail("unknown energy model");
    } else if (!std::strcmp(k[0], "density")) {
      cs.DensityModel = std::atoi(k[1]);
    } else if (!std::strcmp(k[0], "turbulence")) {
      if (!std::strcmp(k[1], "no")) cs.TurModel = 0;
      else if (!std::strcmp(k[1], "ke")) cs.TurModel = 1;
      else fail("unknown turbulence model");
    } else if (!std::strcmp(k[0], "gravity")) {
      for (int i = 0; i < 3; i++) cs.gravity[i] = std::atof(k[1 + i]);
    } else if (!std::strcmp(k[0], "PressureRef")) {
      cs.PressureReference = std::atof(k[1]);
      if (std::strlen(k[2]) > 0) cs.cellPressureRef = std::atoi(k[2]) - 1;
    } else if (!std::strcmp(k[0], "relaxation")) {
      cs.URF[0] = cs.URF[1] = cs.URF[2] = std::atof(k[1]);
      cs.URF[3] = std::atof(k[2]);
      cs.URF[4] = std::atof(k[3]);
    } else if (!std::strcmp(k[0], "limiter")) {
      if (!std::strcmp(k[1], "no")) cs.limiter = 0;
      else if (!std::strcmp(k[1], "Barth")) cs.limiter = 1;
      else if (!std::strcmp(k[1], "MLP")) cs.limiter = 2;
      else if (!std::strcmp(k[1], "WENO")) cs.limiter = 3;
      else fail("unknown limiter definition");
    } else if (!std::strcmp(k[0], "restart")) {
      if (!std::strcmp(k[1], "yes")) cs.IfReadBackup = 1;
      else if (!std::strcmp(k[1], "no")) cs.IfReadBackup = 0;
      else fail("unknown restart command");
    } else if (!std::strcmp(k[0], "initflow")) {
      Region& r = cs.regionMap[0];
      r.name = "default fluid";
      r.type1 = 5;
      r.type2 = 0;
      for (int i = 1; i <= ikey && i <= 10; i++) r.initvalues[i - 1] = std::atof(k[i]);
    } else if (!std::strcmp(k[0], "bound")) {
      int bid = std::atoi(k[1]);
      if (bid == 0) fail("default rid 0 is occupied");
      if (cs.regionMap.count(bid)) fail("repeating rid definition");
      Region& r = cs.regionMap[bid];
      r.name = k[3];
      if (!std::strcmp(k[2], "Twall")) {
        if (ikey != 4) fail("temperature wall field requied 1 parameters");
        r.type1 = 1; r.type2 = 0; r.fixedValue = std::atof(k[4]);
      } else if (!std::strcmp(k[2], "Hwall")) {
        if (ikey != 4) fail("heat flux wall field requied 1 parameters");
        r.type1 = 1; r.type2 = 1; r.fixedValue = std::atof(k[4]);
      } else if (!std::strcmp(k[2], "sym")) {
        if (ikey != 3) fail("symmetric field requied no parameters");
        r.type1 = 4; r.type2 = 0; r.fixedValue = 0.0;
      } else if (!std::strcmp(k[2], "inlet")) {
        if (ikey != 11) fail("inlet field requied 8 parameters");
        r.type1 = 2; r.type2 = 0;
        for (int i = 0; i < 6; i++) r.initvalues[i] = std::atof(k[4 + i]);
        if (cs.TurModel == 1) {
          r.initvalues[6] = std::atof(k[10]);
          r.initvalues[7] = std::atof(k[11]);
        }
      } else if (!std::strcmp(k[2], "outlet")) {
        if (ikey != 4) fail("outlet field requied 1 parameter");
        r.type1 = 3; r.type2 = 0; r.fixedValue = std::atof(k[4]);
      } else if (!std::strcmp(k[2], "period")) {
        fail("periodic boundaries are not on the single-partition path");
      } else {
        fail(std::string("unknown boundry type in bound ") + k[2]);
      }
    } else if (!std::strcmp(k[0], "volumn")) {
      int bid = std::atoi(k[1]);
      if (bid == 0) fail("default rid 0 is occupied");
      if (cs.regionMap.count(bid)) fail("repeating rid definition");
      Region& r = cs.regionMap[bid];
      r.name = k[3];
      if (!std::strcmp(k[2], "fluid")) {
        r.type1 = 5; r.type2 = 0;
        if (ikey != 11) fail("fluid field required 8 parameters");
        for (int i = 4; i <= ikey; i++) r.initvalues[i - 4] = std::atof(k[i]);
      } else if (!std::strcmp(k[2], "solid")) {
        r.type1 = 5; r.type2 = 1;
        if (ikey != 5) fail("solid field required 3 parameters");
        for (int i = 4; i <= ikey; i++) r.initvalues[i - 4] = std::atof(k[i]);
      } else {
        fail(std::string("unknown boundry type in bound ") + k[2]);
      }
    } else if (!std::strcmp(k[0], "output")) {
      cs.noutput = std::atoi(k[1]);
      cs.outputFormat = !std::strcmp(k[2], "vtk") ? 1 : 0;
    } else {
      fail(std::string("no such command: ") + k[0]);
    }
  }
  if (cs.DensityModel == 1) cs.SolveEnergy = 1;
}

// ---- mesh read + N=1 partition + local buffers -----------------------------
namespace {
const int kNodesOf[8] = {0, 2, 3, 4, 4, 8, 6, 5};  // RootStructure.cpp:18-20
struct InputElement {
  int type, ntag, tag[10], vertex[8], pid, idx;
};
struct ByPart {  // _SortAccordingToPart, RootStructure.cpp:664-668
  bool operator()(InputElement* l, InputElement* r) const { return l->pid < r->pid ? true : false; }
};
}  // namespace

void read_grid_and_build(Case& cs, const std::string& meshPath) {
  // RootProcess::read (RootStructure.cpp:428-487)
  std::ifstream in(meshPath.c_str());
  if (!in) throw std::runtime_error("cant find grid file " + meshPath);
  std::string tok;
  do {
    if (!(in >> tok)) throw std::runtime_error("no $Nodes section");
  } while (tok != "$Nodes");
  size_t nvert = 0;
  in >> nvert;
  if (nvert == 0) throw std::runtime_error("vertex less than 0");
  std::vector<double> rootVerts(3 * nvert);
  for (size_t i = 0; i < nvert; i++) {
    int id;
    in >> id >> rootVerts[3 * i] >> rootVerts[3 * i + 1] >> rootVerts[3 * i + 2];
  }
  in >> tok >> tok;
  size_t nelem = 0;
  in >> nelem;
  if (nelem == 0) throw std::runtime_error("elements of the mesh file less than 0");
  std::vector<InputElement> store(nelem);
  std::vector<InputElement*> elems(nelem);
  int nGlobal = 0;
  for (size_t i = 0; i < nelem; i++) {
    InputElement& e = store[i];
    int id;
    in >> id >> e.type >> e.ntag;
    if (e.type < 0 || e.type > 7 || e.ntag < 0 || e.ntag > 10) throw std::runtime_error("bad element record");
    for (int j = 0; j < e.ntag; j++) in >> e.tag[j];
    for (int j = 0; j < kNodesOf[e.type]; j++) {
      int v;
      in >> v;
      e.vertex[j] = v - 1;
    }
    if (!in) throw std::runtime_error("truncated element list");
    if (e.type > 3) nGlobal++;
    e.pid = 0;  // METIS_PartGraphKway into one part assigns part 0 to every element
    elems[i] = &e;
  }
  // RootProcess::partition, N=1 (RootStructure.cpp:797-816): the same std::sort call
  // with the same comparator on the element pointer array.  All keys are equal, so the
  // result is libstdc++'s introsort permutation of equal elements.
  std::sort(elems.begin(), elems.end(), ByPart());
  int counter = 0;
  for (size_t i = 0; i < nelem; i++) elems[i]->idx = elems[i]->type > 3 ? counter++ : -1;

  // getVertexSendBuffer (RootStructure.cpp:930-968): std::map over referenced vertices
  std::map<int, int> nodesPool;
  for (size_t i = 0; i < nelem; i++)
    for (int k = 0; k < kNodesOf[elems[i]->type]; k++) nodesPool.insert(std::make_pair(elems[i]->vertex[k], 0));
  cs.Nvrt = (int)nodesPool.size();
  cs.Vert.assign(3 * cs.Nvrt, 0.0);
  {
    int lid = 0;
    for (auto& kv : nodesPool) {
      kv.second = lid;
      for (int d = 0; d < 3; d++) cs.Vert[3 * lid + d] = rootVerts[3 * kv.first + d];
      lid++;
    }
  }
  cs.Ncel = nGlobal;
  cs.Nbnd = (int)nelem - nGlobal;  // navier.cpp:302

  // ReadGridFile (geometry.cpp:47-218)
  cs.B.assign(cs.Nbnd, Bnd());
  cs.C.assign(cs.Ncel, Cell());
  int icel = 0, ibnd = 0;
  for (size_t i = 0; i < nelem; i++) {
    const InputElement& e = *elems[i];
    int v[8];
    for (int k = 0; k < kNodesOf[e.type]; k++) v[k] = nodesPool[e.vertex[k]];
    if (e.ntag != 2 && e.ntag != 3) throw std::runtime_error("element with neither 2 nor 3 tags");
    if (e.type == 2 || e.type == 3) {
      Bnd& b = cs.B[ibnd];
      b.rid = e.tag[0];
      b.vertices[0] = v[0];
      b.vertices[1] = v[1];
      b.vertices[2] = v[2];
      b.vertices[3] = e.type == 2 ? v[2] : v[3];
      ibnd++;
    } else if (e.type >= 4 && e.type <= 7) {
      Cell& c = cs.C[icel];
      c.rid = e.tag[0];
      if (e.type == 4) {
        for (int p = 0; p < 3; p++) c.vertices[p] = v[p];
        c.vertices[3] = v[2];
        for (int p = 4; p < 8; p++) c.vertices[p] = v[3];
      } else if (e.type == 5) {
        for (int p = 0; p < 8; p++) c.vertices[p] = v[p];
      } else if (e.type == 6) {
        for (int p = 0; p < 3; p++) c.vertices[p] = v[p];
        c.vertices[3] = v[2];
        for (int p = 4; p < 7; p++) c.vertices[p] = v[p - 1];
        c.vertices[7] = v[5];
      } else {
        for (int p = 0; p < 4; p++) c.vertices[p] = v[p];
        for (int p = 4; p < 8; p++) c.vertices[p] = v[4];
      }
      icel++;
    } else {
      throw std::runtime_error("unknown element type in local grid file");
    }
  }
  if (icel != cs.Ncel || ibnd != cs.Nbnd) throw std::runtime_error("element count mismatch");

  // CreateFaces + FindFace (geometry.cpp:222-358)
  std::vector<std::set<int>> NodeFace(cs.Nvrt);
  for (int i = 0; i < cs.Ncel; i++) cs.C[i].nface = 0;
  cs.F.clear();
  cs.F.reserve((size_t)cs.Nbnd + 4 * (size_t)cs.Ncel);
  for (int i = 0; i < cs.Nbnd; i++) {
    Face f;
    cs.B[i].face = (int)cs.F.size();
    for (int j = 0; j < 4; j++) f.vertices[j] = cs.B[i].vertices[j];
    f.bnd = i;
    f.cell2 = VOID_CELL_ON_BOUNDARY;
    f.cell1 = -9999999;
    for (int j = 0; j < 4; j++) NodeFace[f.vertices[j]].insert((int)cs.F.size());
    cs.F.push_back(f);
  }
  auto findFace = [&](int ic, int n1, int n2, int n3, int n4) {
    int irepeat = 0;
    if (n1 == n2 || n1 == n3 || n1 == n4) irepeat++;
    if (n2 == n3 || n2 == n4) irepeat++;
    if (n3 == n4) irepeat++;
    if (irepeat > 1) return;
    int fid = -100;
    for (int iface : NodeFace[n1]) {
      const int* fv = cs.F[iface].vertices;
      auto in4 = [&](int q) { return q == n1 || q == n2 || q == n3 || q == n4; };
      if (in4(fv[0]) && in4(fv[1]) && in4(fv[2]) && in4(fv[3])) {
        fid = iface;
        break;
      }
    }
    Cell& c = cs.C[ic];
    if (fid < 0) {
      Face f;
      f.vertices[0] = n1; f.vertices[1] = n2; f.vertices[2] = n3; f.vertices[3] = n4;
      f.cell1 = ic;
      f.cell2 = VOID_CELL_ON_INTERFACE;
      f.bnd = INNER_FACE_BOUNDARY;
      int nf = (int)cs.F.size();
      c.face[c.nface++] = nf;
      for (int k = 0; k < 4; k++) NodeFace[f.vertices[k]].insert(nf);
      cs.F.push_back(f);
    } else {
      if (cs.F[fid].bnd >= 0) cs.F[fid].cell1 = ic;
      else cs.F[fid].cell2 = ic;
      c.face[c.nface++] = fid;
    }
  };
  for (int i = 0; i < cs.Ncel; i++) {
    const int* v = cs.C[i].vertices;
    findFace(i, v[0], v[1], v[2], v[3]);
    findFace(i, v[4], v[5], v[6], v[7]);
    findFace(i, v[0], v[1], v[5], v[4]);
    findFace(i, v[1], v[2], v[6], v[5]);
    findFace(i, v[3], v[2], v[6], v[7]);
    findFace(i, v[0], v[3], v[7], v[4]);
  }
  cs.Nfac = (int)cs.F.size();

  // CellFaceInfo (geometry.cpp:391-752)
  const double* X = cs.Vert.data();
  auto vert = [&](int id) { return X + 3 * id; };
  auto tri3DArea = [&](const double* x1, const double* x2, const double* x3) {
    double v1[3], v2[3];
    vminus(v1, x2, x1);
    vminus(v2, x3, x1);
    double a1 = v1[1] * v2[2] - v1[2] * v2[1];
    double a2 = -v1[0] * v2[2] + v1[2] * v2[0];
    double a3 = v1[0] * v2[1] - v1[1] * v2[0];
    return 0.5 * std::sqrt(a1 * a1 + a2 * a2 + a3 * a3);
  };
  auto tetVolum = [&](const double* x1, const double* x2, const double* x3, const double* x4) {
    double v1[3], d1[3], d2[3], d3[3];
    vminus(d1, x2, x1);
    vminus(d2, x3, x1);
    vminus(d3, x4, x1);
    vcross(v1, d1, d2);
    return 1. / 6. * std::fabs(vdot(v1, d3));
  };
  for (int i = 0; i < cs.Ncel; i++) {
    Cell& c = cs.C[i];
    const double *x1 = vert(c.vertices[0]), *x2 = vert(c.vertices[1]), *x3 = vert(c.vertices[2]),
                 *x4 = vert(c.vertices[3]), *x5 = vert(c.vertices[4]), *x6 = vert(c.vertices[5]),
                 *x7 = vert(c.vertices[6]), *x8 = vert(c.vertices[7]);
    double V1 = tetVolum(x1, x2, x4, x6), V2 = tetVolum(x1, x5, x4, x6), V3 = tetVolum(x4, x5, x8, x6);
    double V4 = tetVolum(x2, x3, x4, x7), V5 = tetVolum(x2, x6, x4, x7), V6 = tetVolum(x8, x4, x6, x7);
    c.vol = V1 + V2 + V3 + V4 + V5 + V6;
    double xc[6][3];
    for (int j = 0; j < 3; j++) {
      xc[0][j] = 0.25 * (x1[j] + x2[j] + x4[j] + x6[j]);
      xc[1][j] = 0.25 * (x1[j] + x5[j] + x4[j] + x6[j]);
      xc[2][j] = 0.25 * (x4[j] + x5[j] + x8[j] + x6[j]);
      xc[3][j] = 0.25 * (x2[j] + x3[j] + x4[j] + x7[j]);
      xc[4][j] = 0.25 * (x2[j] + x6[j] + x4[j] + x7[j]);
      xc[5][j] = 0.25 * (x8[j] + x4[j] + x6[j] + x7[j]);
    }
    double Vsum = V1 + V2 + V3 + V4 + V5 + V6;
    for (int j = 0; j < 3; j++)
      c.x[j] = 1. / Vsum * (V1 * xc[0][j] + V2 * xc[1][j] + V3 * xc[2][j] + V4 * xc[3][j] + V5 * xc[4][j] + V6 * xc[5][j]);
  }
  for (int i = 0; i < cs.Ncel; i++) {
    Cell& c = cs.C[i];
    for (int j = 0; j < c.nface; j++) {
      int iface = c.face[j];
      int nc = cs.F[iface].cell1;
      if (nc == i) nc = cs.F[iface].cell2;
      c.cell[j] = nc;
    }
    c.globalIdx = i;  // iStart + i with iStart = 0 (geometry.cpp:537-543)
  }
  for (int i = 0; i < cs.Nfac; i++) {
    Face& f = cs.F[i];
    const double *v1 = vert(f.vertices[0]), *v2 = vert(f.vertices[1]), *v3 = vert(f.vertices[2]),
                 *v4 = vert(f.vertices[3]);
    double area1 = tri3DArea(v1, v2, v4);
    double area2 = tri3DArea(v2, v3, v4);
    double xc1[3], xc2[3];
    for (int j = 0; j < 3; j++) {
      xc1[j] = 1. / 3 * (v1[j] + v2[j] + v4[j]);
      xc2[j] = 1. / 3 * (v2[j] + v3[j] + v4[j]);
    }
    for (int j = 0; j < 3; j++) f.x[j] = (area1 * xc1[j] + area2 * xc2[j]) / (area1 + area2);
    double dx1[3], dx2[3], dx[3];
    vminus(dx1, v1, v3);
    vminus(dx2, v2, v4);
    vcross(f.n, dx1, dx2);
    for (int j = 0; j < 3; j++) f.n[j] = 0.5 * f.n[j];
    if (f.cell1 < 0 || f.cell1 >= cs.Ncel) throw std::runtime_error("boundary face not attached to any cell");
    vminus(dx, f.x, cs.C[f.cell1].x);
    if (vdot(f.n, dx) < 0.)
      for (int j = 0; j < 3; j++) f.n[j] = -f.n[j];
    f.area = vlen(f.n);
    if (std::fabs((area1 + area2 - f.area) / f.area) > 1.e-4)
      throw std::runtime_error("area is not correct at face " + std::to_string(i));
    if (f.cell2 >= 0) {
      vminus(dx1, f.x, cs.C[f.cell1].x);
      vminus(dx2, f.x, cs.C[f.cell2].x);
      double r1 = vlen(dx1), r2 = vlen(dx2);
      f.lambda = r2 / (r1 + r2);
    } else {
      f.lambda = 1.;
    }
  }
  for (int i = 0; i < cs.Nbnd; i++) {
    int jf = cs.B[i].face;
    int jc = cs.F[jf].cell1;
    double dx[3];
    vminus(dx, cs.F[jf].x, cs.C[jc].x);
    cs.B[i].distance = vdot(dx, cs.F[jf].n) / cs.F[jf].area;
    if (cs.B[i].distance < 0.) throw std::runtime_error("wall distance is negative");
  }
  for (int i = 0; i < cs.Nfac; i++) {
    Face& f = cs.F[i];
    int ic1 = f.cell1, ic2 = f.cell2;
    double dx[3];
    if (ic2 == VOID_CELL_ON_BOUNDARY) {
      vminus(dx, f.x, cs.C[ic1].x);
      f.rlencos = f.area / (vdot(dx, f.n) / f.area);
    } else {
      vminus(dx, cs.C[ic2].x, cs.C[ic1].x);
      f.rlencos = f.area / std::fabs(vdot(dx, f.n) / f.area);
    }
    if (ic2 >= 0) {
      double d[3], ss;
      vminus(d, f.x, cs.C[ic1].x);
      ss = vdot(d, f.n) / f.area;
      for (int j = 0; j < 3; j++) d[j] = ss * f.n[j] / f.area;
      vminus(f.Xpac, f.x, d);
      vminus(d, f.x, cs.C[ic2].x);
      ss = vdot(d, f.n) / f.area;
      for (int j = 0; j < 3; j++) d[j] = ss * f.n[j] / f.area;
      vminus(f.Xnac, f.x, d);
    } else {
      for (int j = 0; j < 3; j++) f.Xpac[j] = f.Xnac[j] = 0.0;
    }
  }
  // CheckAndAllocate (geometry.cpp:754-768)
  for (int i = 0; i < cs.Nfac; i++) {
    int c2 = cs.F[i].cell2;
    if (!(c2 == VOID_CELL_ON_BOUNDARY || c2 >= 0))
      throw std::runtime_error("error in face right hand side, face " + std::to_string(i));
  }
  size_t n = cs.Ncel;
  for (auto* v : {&cs.Rn, &cs.Un, &cs.Vn, &cs.Wn, &cs.Pn, &cs.Tn, &cs.deltaP, &cs.VisLam, &cs.VisTur, &cs.Apr})
    v->assign(n, 0.0);
  if (cs.TurModel == 1) {
    cs.TE.assign(n, 0.0);
    cs.ED.assign(n, 0.0);
  }
  if (!cs.IfSteady)
    for (auto* v : {&cs.Rnp, &cs.Unp, &cs.Vnp, &cs.Wnp, &cs.Tnp, &cs.TEp, &cs.EDp, &cs.Rnp2, &cs.Unp2, &cs.Vnp2,
                    &cs.Wnp2, &cs.Tnp2, &cs.TEp2, &cs.EDp2})
      v->assign(n, 0.0);
  for (auto* v : {&cs.dPdX, &cs.dUdX, &cs.dVdX, &cs.dWdX, &cs.dPhidX}) v->assign(3 * n, 0.0);
  for (auto* v : {&cs.BRo, &cs.BU, &cs.BV, &cs.BW, &cs.BPre, &cs.BTem, &cs.BTE, &cs.BED}) v->assign(cs.Nbnd, 0.0);
  cs.RUFace.assign(cs.Nfac, 0.0);
  build_pattern(cs);
}

// AIJ pattern: diagonal plus one entry per interior-face neighbour, sorted.
void build_pattern(Case& cs) {
  Csr A;
  A.n = cs.Ncel;
  A.rowptr.assign(cs.Ncel + 1, 0);
  std::vector<int> cols;
  for (int i = 0; i < cs.Ncel; i++) {
    cols.clear();
    cols.push_back(i);
    for (int j = 0; j < cs.C[i].nface; j++) {
      int nb = cs.C[i].cell[j];
      if (nb >= 0) cols.push_back(nb);
    }
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    A.rowptr[i + 1] = A.rowptr[i] + (int)cols.size();
    for (int c : cols) A.col.push_back(c);
  }
  A.diag.assign(cs.Ncel, -1);
  for (int i = 0; i < cs.Ncel; i++)
    for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; k++)
      if (A.col[k] == i) A.diag[i] = k;
  A.val.assign(A.col.size(), 0.0);
  cs.Au = A;
  cs.Ap = A;
  cs.As = A;
  cs.bu.assign(cs.Ncel, 0.0);
  cs.bv.assign(cs.Ncel, 0.0);
  cs.bw.assign(cs.Ncel, 0.0);
  cs.bp.assign(cs.Ncel, 0.0);
  cs.bs.assign(cs.Ncel, 0.0);
}

void Csr::insert(int row, int c, double v) {
  int lo = rowptr[row], hi = rowptr[row + 1];
  int k = (int)(std::lower_bound(col.begin() + lo, col.begin() + hi, c) - col.begin());
  if (k >= hi || col[k] != c) throw std::runtime_error("insert outside the preallocated pattern");
  val[k] = v;
}

// InitFlowField (navier.cpp:588-697), steady, no restart
void init_flow_field(Case& cs) {
  using std::vector;
  const double Cmu = 0.09;
  auto initCell = [&](int i, const double* iv) {
    cs.Un[i] = iv[0];
    cs.Vn[i] = iv[1];
    cs.Wn[i] = iv[2];
    cs.Rn[i] = iv[3];
    cs.Tn[i] = iv[4];
    cs.Pn[i] = 0.;
    if (cs.DensityModel == 1) cs.Rn[i] = (cs.Pn[i] + cs.PressureReference) / (cs.Rcpcv * cs.Tn[i]);
    cs.VisLam[i] = iv[5];
    cs.VisTur[i] = 0.;
    if (cs.TurModel == 1) {
      cs.TE[i] = iv[6];
      cs.ED[i] = iv[7];
      cs.VisTur[i] = cs.Rn[i] * Cmu * cs.TE[i] * cs.TE[i] / (cs.ED[i] + SMALL);
    }
  };
  if (cs.IfReadBackup) throw std::runtime_error("restart from res.sav is not on the measured path");
  if (cs.regionMap.count(0))
    for (int i = 0; i < cs.Ncel; i++) initCell(i, cs.regionMap[0].initvalues);
  for (int i = 0; i < cs.Ncel; i++) {
    auto it = cs.regionMap.find(cs.C[i].rid);
    if (it == cs.regionMap.end()) throw std::runtime_error("cell region not defined in param file");
    initCell(i, it->second.initvalues);
  }
  std::fill(cs.deltaP.begin(), cs.deltaP.end(), 0.0);
  for (int i = 0; i < cs.Nbnd; i++) {
    auto it = cs.regionMap.find(cs.B[i].rid);
    if (it == cs.regionMap.end()) throw std::runtime_error("boundary region not defined in param file");
    const Region& reg = it->second;
    if (reg.type1 == 1) {
      if (reg.type2 == 0) cs.BTem[i] = reg.fixedValue;
      else if (reg.type2 == 1) cs.B[i].q = reg.fixedValue;
      else if (reg.type2 == 2) cs.B[i].q = 0.0;
    } else if (reg.type1 == 2) {
      cs.BU[i] = reg.initvalues[0];
      cs.BV[i] = reg.initvalues[1];
      cs.BW[i] = reg.initvalues[2];
      cs.BRo[i] = reg.initvalues[4];
      cs.BTem[i] = reg.initvalues[5];
      cs.BTE[i] = reg.initvalues[6];
      cs.BED[i] = reg.initvalues[7];
    } else if (reg.type1 == 3) {
    } else if (reg.type1 == 4) {
      cs.B[i].q = 0.0;
    } else {
      throw std::runtime_error("bounday didnt match, bid " + std::to_string(cs.B[i].rid));
    }
  }
  std::fill(cs.RUFace.begin(), cs.RUFace.end(), 0.0);
}

}  // namespace orc
