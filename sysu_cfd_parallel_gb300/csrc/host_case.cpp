// Host side of the drop-in: param.in, gmsh v2 ASCII mesh, one-rank element numbering,
// face list and initial fields.  Produces the topology that libcycasgpu uploads; the
// geometry itself is computed on the device (geometry.cu).
//
// Reference behaviour mirrored here:
//   param.in keys            NS/readparamfile.cpp:10-344
//   gmsh reader              NS/RootStructure.cpp:428-487 (ASCII), 61-116 (compressed binary,
//                            the -mshBinary switch of main.cpp:27,48)
//   one-rank numbering       NS/RootStructure.cpp:797-816 (std::sort by part id) and the
//                            vertex pool of getVertexSendBuffer, RootStructure.cpp:930-968
//   element -> Cell/Bnd      NS/geometry.cpp:47-218 (hex-form vertex lists)
//   face discovery order     NS/geometry.cpp:222-358 (CreateFaces / FindFace)
//   neighbours               NS/geometry.cpp:461-473
//   initial fields           NS/navier.cpp:588-697 (InitFlowField, steady; restart yes reads
//                            res.sav beside param.in, ReadBackupFile navierIO.cpp:389-404)
//
// The face list is built by sorting (vertex-set key, discovery rank) records instead of the
// reference's per-vertex std::set search and per-face realloc; it reproduces the same face
// indices, owner/neighbour and per-cell face slots for conforming meshes.
#include <algorithm>
#include <sys/stat.h>
#include <mutex>
#include <memory>
#include <cctype>
#include <cerrno>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "cycas_host.h"

namespace cycas {

// ------------------------------------------------------------------ param.in
static std::string trim_ws(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

void load_params(HostCase& hc, const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw IoError("param file not found: " + path);
  std::string text;
  char buf[65536];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  std::fclose(f);
  size_t pos = 0;
  int lineNo = 0;
  while (pos <= text.size()) {
    size_t nl = text.find('\n', pos);
    std::string line = text.substr(pos, nl == std::string::npos ? std::string::npos : nl - pos);
    pos = nl == std::string::npos ? text.size() + 1 : nl + 1;
    lineNo++;
    if (line.size() >= 2 && line[0] == '/' && line[1] == '/') continue;
    if (line.size() <= 1) continue;
    std::vector<std::string> kw;
    size_t s = 0;
    for (;;) {
      size_t c = line.find(',', s);
      kw.push_back(trim_ws(line.substr(s, c == std::string::npos ? std::string::npos : c - s)));
      if (c == std::string::npos) break;
      s = c + 1;
    }
    int nk = (int)kw.size() - 1;  // the reference's ikey: number of commas
    while (kw.size() < 20) kw.push_back("");
    auto bad = [&](const std::string& m) {
      throw ParamError("param.in line " + std::to_string(lineNo) + ": " + m);
    };
    auto num = [&](int i) { return std::atof(kw[i].c_str()); };
    const std::string& key = kw[0];
    if (key == "gridfile") {
      hc.gridfile = kw[1];
    } else if (key == "steady") {
      hc.steady = 1;
      hc.max_step = std::atoi(kw[1].c_str());
      hc.residual_steady = num(2);
    } else if (key == "transient") {  // readparamfile.cpp:84-101
      if (nk != 4) bad("transient requies 3 parameters");
      hc.steady = 0;
      hc.dt = num(1);
      hc.total_time = num(2);
      hc.max_step = (int)(hc.total_time / hc.dt);
      hc.max_outer = (int)num(3);
      if (kw[4] == "Euler") hc.time_scheme = 1;
      else if (kw[4] == "Dual") hc.time_scheme = 2;
      else bad("unknown time scheme: " + kw[4]);
    } else if (key == "energy") {
      if (kw[1] == "on") hc.solve_energy = 1;
      else if (kw[1] == "off") hc.solve_energy = 0;
      else bad("unknown energy model");
    } else if (key == "density") {
      hc.density_model = std::atoi(kw[1].c_str());
    } else if (key == "turbulence") {
      if (kw[1] == "no") hc.turb_model = 0;
      else if (kw[1] == "ke") hc.turb_model = 1;
      else bad("unknown turbulence model");
    } else if (key == "gravity") {
      for (int d = 0; d < 3; d++) hc.gravity[d] = num(1 + d);
    } else if (key == "PressureRef") {
      hc.pressure_reference = num(1);
      if (!kw[2].empty()) hc.cell_pressure_ref = std::atoi(kw[2].c_str()) - 1;
    } else if (key == "relaxation") {
      hc.urf[0] = hc.urf[1] = hc.urf[2] = num(1);
      hc.urf[3] = num(2);
      hc.urf[4] = num(3);
    } else if (key == "limiter") {
      if (kw[1] == "no") hc.limiter = 0;
      else if (kw[1] == "Barth") hc.limiter = 1;
      else if (kw[1] == "MLP") hc.limiter = 2;
      else if (kw[1] == "WENO") hc.limiter = 3;
      else bad("unknown limiter definition");
    } else if (key == "restart") {
      if (kw[1] == "yes") hc.restart = 1;
      else if (kw[1] == "no") hc.restart = 0;
      else bad("unknown restart command");
    } else if (key == "initflow") {
      Region& r = hc.regions[0];
      r.type1 = 5;
      r.type2 = 0;
      for (int i = 1; i <= nk && i <= 10; i++) r.init[i - 1] = num(i);
    } else if (key == "bound") {
      int bid = std::atoi(kw[1].c_str());
      if (bid == 0) bad("default rid 0 is occupied");
      if (hc.regions.count(bid)) bad("repeating rid definition");
      Region& r = hc.regions[bid];
      const std::string& kind = kw[2];
      if (kind == "Twall" || kind == "Hwall") {
        if (nk != 4) bad("wall requires 1 parameter");
        r.type1 = 1;
        r.type2 = kind == "Twall" ? 0 : 1;
        r.fixed = num(4);
      } else if (kind == "sym") {
        if (nk != 3) bad("symmetric requires no parameters");
        r.type1 = 4;
        r.type2 = 0;
      } else if (kind == "inlet") {
        if (nk != 11) bad("inlet requires 8 parameters");
        r.type1 = 2;
        r.type2 = 0;
        for (int i = 0; i < 6; i++) r.init[i] = num(4 + i);
        if (hc.turb_model == 1) {  // k and epsilon are stored only if turbulence was set earlier
          r.init[6] = num(10);
          r.init[7] = num(11);
        }
      } else if (kind == "outlet") {
        if (nk != 4) bad("outlet requires 1 parameter");
        r.type1 = 3;
        r.type2 = 0;
        r.fixed = num(4);
      } else if (kind == "period") {
        bad("periodic boundaries are outside the single-partition path");
      } else {
        bad("unknown boundary type " + kind);
      }
    } else if (key == "volumn") {
      int bid = std::atoi(kw[1].c_str());
      if (bid == 0) bad("default rid 0 is occupied");
      if (hc.regions.count(bid)) bad("repeating rid definition");
      Region& r = hc.regions[bid];
      if (kw[2] == "fluid") {
        if (nk != 11) bad("fluid requires 8 parameters");
        r.type1 = 5;
        r.type2 = 0;
      } else if (kw[2] == "solid") {
        if (nk != 5) bad("solid requires 3 parameters");
        r.type1 = 5;
        r.type2 = 1;
      } else {
        bad("unknown volume type " + kw[2]);
      }
      for (int i = 4; i <= nk; i++) r.init[i - 4] = num(i);
    } else if (key == "output") {
      hc.noutput = std::atoi(kw[1].c_str());
    } else {
      bad("no such command: " + key);
    }
  }
  if (hc.density_model == 1) hc.solve_energy = 1;
}

// ------------------------------------------------------------------ gmsh v2 ASCII
namespace {
const int kNodes[8] = {0, 2, 3, 4, 4, 8, 6, 5};

struct Tokenizer {
  const char* p;
  const char* end;
  bool word(std::string& out) {
    while (p < end && std::isspace((unsigned char)*p)) p++;
    if (p >= end) return false;
    const char* s = p;
    while (p < end && !std::isspace((unsigned char)*p)) p++;
    out.assign(s, p);
    return true;
  }
  long integer() {
    while (p < end && std::isspace((unsigned char)*p)) p++;
    char* e;
    long v = std::strtol(p, &e, 10);
    if (e == p) throw MeshError("malformed integer in mesh file");
    p = e;
    return v;
  }
  double real() {
    while (p < end && std::isspace((unsigned char)*p)) p++;
    char* e;
    double v = std::strtod(p, &e);
    if (e == p) throw MeshError("malformed number in mesh file");
    p = e;
    return v;
  }
};

// little-endian fixed-size records of the compressed mesh, bounds-checked
struct ByteReader {
  const char* p;
  const char* end;
  template <class T>
  T take() {
    if (end - p < (long)sizeof(T)) throw MeshError("truncated binary mesh file");
    T v;
    std::memcpy(&v, p, sizeof(T));
    p += sizeof(T);
    return v;
  }
};

struct RawElem {
  int type, tag0;
  int v[8];
};
}  // namespace

void load_gmsh(HostCase& hc, const std::string& path, bool binary) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw IoError("cant find grid file " + path);
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> data((size_t)sz + 1, 0);
  if (sz > 0 && std::fread(data.data(), 1, (size_t)sz, f) != (size_t)sz) {
    std::fclose(f);
    throw IoError("short read on " + path);
  }
  std::fclose(f);
  long nv = 0, ne = 0;
  std::vector<double> raw;
  std::vector<RawElem> el;
  auto check_elem = [&](RawElem& e, int ntag) {
    if (e.type < 0 || e.type > 7 || ntag < 0 || ntag > 10) throw MeshError("bad element record");
    if (ntag != 2 && ntag != 3) throw MeshError("element with neither 2 nor 3 tags");
  };
  if (binary) {
    // compressed gmsh (RootProcess::readBin, RootStructure.cpp:61-116): size_t vertex count,
    // per vertex {int32 id, 3 doubles}; size_t element count, per element {int32 id, int32
    // type, int32 ntag, ntag int32 tags, the type's int32 one-based vertex ids}
    ByteReader br{data.data(), data.data() + sz};
    nv = (long)br.take<uint64_t>();
    if (nv <= 0 || nv > (sz / 28)) throw MeshError("vertex less than 0");
    raw.resize(3 * (size_t)nv);
    for (long i = 0; i < nv; i++) {
      br.take<int32_t>();
      for (int d = 0; d < 3; d++) raw[3 * i + d] = br.take<double>();
    }
    ne = (long)br.take<uint64_t>();
    if (ne <= 0 || ne > (sz / 12)) throw MeshError("elements of the mesh file less than 0");
    el.resize((size_t)ne);
    for (long i = 0; i < ne; i++) {
      br.take<int32_t>();
      RawElem& e = el[i];
      e.type = br.take<int32_t>();
      int ntag = br.take<int32_t>();
      check_elem(e, ntag);
      for (int t = 0; t < ntag; t++) {
        int32_t tg = br.take<int32_t>();
        if (t == 0) e.tag0 = tg;
      }
      for (int k = 0; k < kNodes[e.type]; k++) {
        long v = (long)br.take<int32_t>() - 1;
        if (v < 0 || v >= nv) throw MeshError("vertex id out of range");
        e.v[k] = (int)v;
      }
    }
  } else {
    Tokenizer tk{data.data(), data.data() + sz};
    std::string w;
    do {
      if (!tk.word(w)) throw MeshError("no $Nodes section");
    } while (w != "$Nodes");
    nv = tk.integer();
    if (nv <= 0) throw MeshError("vertex less than 0");
    raw.resize(3 * (size_t)nv);
    for (long i = 0; i < nv; i++) {
      tk.integer();
      raw[3 * i] = tk.real();
      raw[3 * i + 1] = tk.real();
      raw[3 * i + 2] = tk.real();
    }
    tk.word(w);
    tk.word(w);
    ne = tk.integer();
    if (ne <= 0) throw MeshError("elements of the mesh file less than 0");
    el.resize((size_t)ne);
    for (long i = 0; i < ne; i++) {
      tk.integer();
      RawElem& e = el[i];
      e.type = (int)tk.integer();
      int ntag = (int)tk.integer();
      check_elem(e, ntag);
      for (int t = 0; t < ntag; t++) {
        long tg = tk.integer();
        if (t == 0) e.tag0 = (int)tg;
      }
      for (int k = 0; k < kNodes[e.type]; k++) {
        long v = tk.integer() - 1;
        if (v < 0 || v >= nv) throw MeshError("vertex id out of range");
        e.v[k] = (int)v;
      }
    }
  }

  // One-rank element numbering: the reference sorts the element pointer array by partition
  // id with std::sort; with a single part every key compares equal and the result is the
  // fixed permutation libstdc++'s introsort produces for n equal keys.  The same call with
  // the same comparison outcomes on an index array yields that permutation.
  std::vector<int> order((size_t)ne);
  std::iota(order.begin(), order.end(), 0);
  std::vector<int> part((size_t)ne, 0);
  std::sort(order.begin(), order.end(), [&](int a, int b) { return part[a] < part[b]; });

  // vertex pool: referenced vertices, renumbered by increasing file id
  std::vector<int> local((size_t)nv, -1);
  for (const RawElem& e : el)
    for (int k = 0; k < kNodes[e.type]; k++) local[e.v[k]] = 0;
  int nloc = 0;
  for (long i = 0; i < nv; i++)
    if (local[i] == 0) local[i] = nloc++;
  hc.nvrt = nloc;
  hc.vert.resize(3 * (size_t)nloc);
  for (long i = 0; i < nv; i++)
    if (local[i] >= 0)
      for (int d = 0; d < 3; d++) hc.vert[3 * (size_t)local[i] + d] = raw[3 * i + d];

  int ncel = 0, nbnd = 0;
  for (const RawElem& e : el) {
    if (e.type >= 4 && e.type <= 7) ncel++;
    else if (e.type == 2 || e.type == 3) nbnd++;
    else throw MeshError("unknown element type in local grid file");
  }
  hc.ncel = ncel;
  hc.nbnd = nbnd;
  hc.cell_vertices.assign(8 * (size_t)ncel, 0);
  hc.cell_rid.assign(ncel, 0);
  hc.bnd_vertices.assign(4 * (size_t)nbnd, 0);
  hc.bnd_rid.assign(nbnd, 0);
  int ic = 0, ib = 0;
  for (int oi : order) {
    const RawElem& e = el[oi];
    int v[8];
    for (int k = 0; k < kNodes[e.type]; k++) v[k] = local[e.v[k]];
    if (e.type == 2 || e.type == 3) {
      int32_t* b = &hc.bnd_vertices[4 * (size_t)ib];
      b[0] = v[0];
      b[1] = v[1];
      b[2] = v[2];
      b[3] = e.type == 2 ? v[2] : v[3];
      hc.bnd_rid[ib++] = e.tag0;
    } else {
      int32_t* c = &hc.cell_vertices[8 * (size_t)ic];
      switch (e.type) {
        case 4:  // tetra: v0 v1 v2 v2 v3 v3 v3 v3
          c[0] = v[0]; c[1] = v[1]; c[2] = v[2]; c[3] = v[2];
          c[4] = c[5] = c[6] = c[7] = v[3];
          break;
        case 5:
          for (int k = 0; k < 8; k++) c[k] = v[k];
          break;
        case 6:  // prism: v0 v1 v2 v2 v3 v4 v5 v5
          c[0] = v[0]; c[1] = v[1]; c[2] = v[2]; c[3] = v[2];
          c[4] = v[3]; c[5] = v[4]; c[6] = v[5]; c[7] = v[5];
          break;
        default:  // pyramid: v0 v1 v2 v3 v4 v4 v4 v4
          for (int k = 0; k < 4; k++) c[k] = v[k];
          c[4] = c[5] = c[6] = c[7] = v[4];
      }
      hc.cell_rid[ic++] = e.tag0;
    }
  }
}

// ------------------------------------------------------------------ faces
namespace {
// local faces of the hex-form cell, in the order the reference probes them
const int kLocalFace[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};

struct Key {
  int32_t v[4];  // distinct vertex ids ascending, padded with INT32_MAX
  bool operator<(const Key& o) const {
    for (int i = 0; i < 4; i++)
      if (v[i] != o.v[i]) return v[i] < o.v[i];
    return false;
  }
  bool operator==(const Key& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2] && v[3] == o.v[3]; }
};

Key make_key(int a, int b, int c, int d) {
  Key k{{a, b, c, d}};
  std::sort(k.v, k.v + 4);
  int m = 1;
  for (int i = 1; i < 4; i++)
    if (k.v[i] != k.v[m - 1]) k.v[m++] = k.v[i];
  for (int i = m; i < 4; i++) k.v[i] = INT32_MAX;
  return k;
}

// FindFace's degeneracy rule (geometry.cpp:302-306)
bool degenerate(int n1, int n2, int n3, int n4) {
  int r = 0;
  if (n1 == n2 || n1 == n3 || n1 == n4) r++;
  if (n2 == n3 || n2 == n4) r++;
  if (n3 == n4) r++;
  return r > 1;
}

struct Probe {
  Key key;
  int64_t rank;  // 6*cell + local face: the order the reference visits them
};
}  // namespace

void build_faces(HostCase& hc) {
  const int ncel = hc.ncel, nbnd = hc.nbnd;
  std::vector<Probe> probes;
  probes.reserve(6 * (size_t)ncel);
  for (int i = 0; i < ncel; i++) {
    const int32_t* cv = &hc.cell_vertices[8 * (size_t)i];
    for (int k = 0; k < 6; k++) {
      int n1 = cv[kLocalFace[k][0]], n2 = cv[kLocalFace[k][1]], n3 = cv[kLocalFace[k][2]], n4 = cv[kLocalFace[k][3]];
      if (degenerate(n1, n2, n3, n4)) continue;
      probes.push_back({make_key(n1, n2, n3, n4), 6 * (int64_t)i + k});
    }
  }
  std::sort(probes.begin(), probes.end(), [](const Probe& a, const Probe& b) {
    if (a.key == b.key) return a.rank < b.rank;
    return a.key < b.key;
  });
  // boundary faces: key -> lowest boundary index with that key
  std::vector<std::pair<Key, int>> bkeys((size_t)nbnd);
  for (int j = 0; j < nbnd; j++) {
    const int32_t* bv = &hc.bnd_vertices[4 * (size_t)j];
    bkeys[j] = {make_key(bv[0], bv[1], bv[2], bv[3]), j};
  }
  std::sort(bkeys.begin(), bkeys.end(), [](const std::pair<Key, int>& a, const std::pair<Key, int>& b) {
    if (a.first == b.first) return a.second < b.second;
    return a.first < b.first;
  });

  // walk the groups of equal keys
  struct Group {
    size_t begin, end;
    int bnd;  // matching boundary face or -1
  };
  std::vector<Group> groups;
  {
    size_t bi = 0;
    for (size_t s = 0; s < probes.size();) {
      size_t e = s + 1;
      while (e < probes.size() && probes[e].key == probes[s].key) e++;
      while (bi < bkeys.size() && bkeys[bi].first < probes[s].key) bi++;
      int bnd = (bi < bkeys.size() && bkeys[bi].first == probes[s].key) ? bkeys[bi].second : -1;
      groups.push_back({s, e, bnd});
      s = e;
    }
  }
  // interior faces are numbered after the boundary faces in order of first discovery
  std::vector<size_t> created;
  for (size_t g = 0; g < groups.size(); g++)
    if (groups[g].bnd < 0) created.push_back(g);
  std::sort(created.begin(), created.end(),
            [&](size_t a, size_t b) { return probes[groups[a].begin].rank < probes[groups[b].begin].rank; });
  const int nfac = nbnd + (int)created.size();
  hc.nfac = nfac;
  hc.face_cell1.assign(nfac, -9999999);
  hc.face_cell2.assign(nfac, VOID_CELL_ON_INTERFACE);
  hc.face_bnd.assign(nfac, INNER_FACE_BOUNDARY);
  hc.face_vertices.assign(4 * (size_t)nfac, 0);
  hc.bnd_face.assign(nbnd, 0);
  for (int j = 0; j < nbnd; j++) {
    hc.bnd_face[j] = j;
    hc.face_bnd[j] = j;
    hc.face_cell2[j] = VOID_CELL_ON_BOUNDARY;
    for (int q = 0; q < 4; q++) hc.face_vertices[4 * (size_t)j + q] = hc.bnd_vertices[4 * (size_t)j + q];
  }
  std::vector<int> faceOfGroup(groups.size(), -1);
  for (size_t r = 0; r < created.size(); r++) faceOfGroup[created[r]] = nbnd + (int)r;
  for (size_t g = 0; g < groups.size(); g++)
    if (groups[g].bnd >= 0) faceOfGroup[g] = groups[g].bnd;

  // per-cell face slots in probe order
  std::vector<int32_t> slotFace(6 * (size_t)ncel, -1);
  for (size_t g = 0; g < groups.size(); g++) {
    int fid = faceOfGroup[g];
    for (size_t q = groups[g].begin; q < groups[g].end; q++) {
      int64_t rank = probes[q].rank;
      int cell = (int)(rank / 6), k = (int)(rank % 6);
      slotFace[6 * (size_t)cell + k] = fid;
      if (groups[g].bnd >= 0) {
        hc.face_cell1[fid] = cell;  // FindFace on a boundary face sets cell1
      } else if (q == groups[g].begin) {
        hc.face_cell1[fid] = cell;
        const int32_t* cv = &hc.cell_vertices[8 * (size_t)cell];
        for (int m = 0; m < 4; m++) hc.face_vertices[4 * (size_t)fid + m] = cv[kLocalFace[k][m]];
      } else {
        hc.face_cell2[fid] = cell;
      }
    }
  }
  hc.cell_nface.assign(ncel, 0);
  hc.cell_face.assign(6 * (size_t)ncel, -1);
  hc.cell_cell.assign(6 * (size_t)ncel, -1);
  for (int i = 0; i < ncel; i++) {
    int nf = 0;
    for (int k = 0; k < 6; k++) {
      int fid = slotFace[6 * (size_t)i + k];
      if (fid >= 0) hc.cell_face[6 * (size_t)i + nf++] = fid;
    }
    hc.cell_nface[i] = nf;
  }
  // CheckAndAllocate (geometry.cpp:760-768): every face has a neighbour or is a boundary
  for (int f = 0; f < nfac; f++) {
    if (hc.face_cell1[f] < 0) throw MeshError("boundary face " + std::to_string(f) + " touches no cell");
    int c2 = hc.face_cell2[f];
    if (!(c2 == VOID_CELL_ON_BOUNDARY || c2 >= 0))
      throw MeshError("face " + std::to_string(f) + " has one cell and is not a boundary face");
  }
  for (int i = 0; i < ncel; i++)
    for (int j = 0; j < hc.cell_nface[i]; j++) {
      int fid = hc.cell_face[6 * (size_t)i + j];
      int nc = hc.face_cell1[fid];
      if (nc == i) nc = hc.face_cell2[fid];
      hc.cell_cell[6 * (size_t)i + j] = nc;
    }
}

// ------------------------------------------------------------------ InitFlowField
void init_fields(HostCase& hc) {
  const double Cmu = 0.09;
  const int n = hc.ncel, nb = hc.nbnd;
  for (auto* v : {&hc.U, &hc.V, &hc.W, &hc.R, &hc.T, &hc.P, &hc.VisLam, &hc.VisTur, &hc.TE, &hc.ED})
    v->assign(n, 0.0);
  for (auto* v : {&hc.BU, &hc.BV, &hc.BW, &hc.BRo, &hc.BTem, &hc.BTE, &hc.BED}) v->assign(nb, 0.0);
  auto apply = [&](int i, const double* iv) {
    hc.U[i] = iv[0];
    hc.V[i] = iv[1];
    hc.W[i] = iv[2];
    hc.R[i] = iv[3];
    hc.T[i] = iv[4];
    hc.P[i] = 0.;
    if (hc.density_model == 1) {  // perfect gas with the reference's constants (navier.cpp:486-493)
      const double cp = 1006., cv = cp / 1.4;
      hc.R[i] = (hc.P[i] + hc.pressure_reference) / ((cp - cv) * hc.T[i]);
    }
    hc.VisLam[i] = iv[5];
    hc.VisTur[i] = 0.;
    if (hc.turb_model == 1) {
      hc.TE[i] = iv[6];
      hc.ED[i] = iv[7];
      hc.VisTur[i] = hc.R[i] * Cmu * hc.TE[i] * hc.TE[i] / (hc.ED[i] + 1.e-16);
    }
  };
  if (hc.restart) {
    // restart yes: the cell fields come from the backup file alone (navier.cpp:590-591)
    double* const dst[10] = {hc.R.data(), hc.U.data(), hc.V.data(), hc.W.data(), hc.P.data(),
                             hc.T.data(), hc.VisLam.data(), hc.VisTur.data(), hc.TE.data(), hc.ED.data()};
    read_backup(hc.backup_path, n, hc.turb_model, dst);
  } else {
    auto r0 = hc.regions.find(0);
    if (r0 != hc.regions.end())
      for (int i = 0; i < n; i++) apply(i, r0->second.init);
    for (int i = 0; i < n; i++) {
      auto it = hc.regions.find(hc.cell_rid[i]);
      if (it == hc.regions.end()) throw ParamError("cell region " + std::to_string(hc.cell_rid[i]) + " not defined");
      apply(i, it->second.init);
    }
  }
  hc.bnd_type.assign(nb, 0);
  for (int i = 0; i < nb; i++) {
    auto it = hc.regions.find(hc.bnd_rid[i]);
    if (it == hc.regions.end()) throw ParamError("boundary region " + std::to_string(hc.bnd_rid[i]) + " not defined");
    const Region& r = it->second;
    hc.bnd_type[i] = r.type1;
    if (r.type1 == 1) {
      if (r.type2 == 0) hc.BTem[i] = r.fixed;
    } else if (r.type1 == 2) {
      hc.BU[i] = r.init[0];
      hc.BV[i] = r.init[1];
      hc.BW[i] = r.init[2];
      hc.BRo[i] = r.init[4];
      hc.BTem[i] = r.init[5];
      hc.BTE[i] = r.init[6];
      hc.BED[i] = r.init[7];
    } else if (r.type1 == 3 || r.type1 == 4) {
    } else {
      throw ParamError("boundary region " + std::to_string(hc.bnd_rid[i]) + " is not a boundary type");
    }
  }
}

namespace {

// Parsed meshes (gmsh ingest + face discovery), shared by every case that loads the same file:
// a request server loads many cases that differ only in their param.in (Reynolds number, inlet
// velocity) over a few dozen meshes.  Keyed by the file's path, size, inode and modification
// time, so a rewritten file is parsed again; bounded in bytes, least recently used first out.
struct MeshEntry {
  std::shared_ptr<const HostCase> mesh;  // only the mesh arrays are filled
  size_t bytes = 0;
  uint64_t used = 0;
};
std::mutex g_mesh_mu;
std::map<std::string, MeshEntry> g_meshes;
uint64_t g_mesh_clock = 0;
size_t g_mesh_bytes = 0;
constexpr size_t kMeshCacheBytes = size_t(4) << 30;

template <class T>
size_t vbytes(const std::vector<T>& v) { return v.size() * sizeof(T); }

size_t mesh_bytes(const HostCase& h) {
  return vbytes(h.vert) + vbytes(h.cell_vertices) + vbytes(h.cell_rid) + vbytes(h.cell_nface) +
         vbytes(h.cell_face) + vbytes(h.cell_cell) + vbytes(h.bnd_vertices) + vbytes(h.bnd_rid) +
         vbytes(h.bnd_face) + vbytes(h.face_cell1) + vbytes(h.face_cell2) + vbytes(h.face_bnd) +
         vbytes(h.face_vertices);
}

void copy_mesh(HostCase& dst, const HostCase& src) {
  dst.ncel = src.ncel;
  dst.nfac = src.nfac;
  dst.nbnd = src.nbnd;
  dst.nvrt = src.nvrt;
  dst.vert = src.vert;
  dst.cell_vertices = src.cell_vertices;
  dst.cell_rid = src.cell_rid;
  dst.cell_nface = src.cell_nface;
  dst.cell_face = src.cell_face;
  dst.cell_cell = src.cell_cell;
  dst.bnd_vertices = src.bnd_vertices;
  dst.bnd_rid = src.bnd_rid;
  dst.bnd_face = src.bnd_face;
  dst.face_cell1 = src.face_cell1;
  dst.face_cell2 = src.face_cell2;
  dst.face_bnd = src.face_bnd;
  dst.face_vertices = src.face_vertices;
}

// the mesh arrays of `grid` into hc, parsed once per file version
void load_mesh_cached(HostCase& hc, const std::string& grid, bool binary) {
  struct stat st;
  if (stat(grid.c_str(), &st) != 0) throw IoError("cant find grid file " + grid);
  const std::string key = grid + "|" + std::to_string((long long)st.st_size) + "|" +
                          std::to_string((unsigned long long)st.st_ino) + "|" +
                          std::to_string((long long)st.st_mtim.tv_sec) + "." +
                          std::to_string((long long)st.st_mtim.tv_nsec) + (binary ? "|b" : "|a");
  {
    std::lock_guard<std::mutex> lk(g_mesh_mu);
    auto it = g_meshes.find(key);
    if (it != g_meshes.end()) {
      it->second.used = ++g_mesh_clock;
      copy_mesh(hc, *it->second.mesh);
      return;
    }
  }
  auto m = std::make_shared<HostCase>();
  load_gmsh(*m, grid, binary);
  build_faces(*m);
  copy_mesh(hc, *m);
  const size_t b = mesh_bytes(*m);
  std::lock_guard<std::mutex> lk(g_mesh_mu);
  if (b > kMeshCacheBytes || g_meshes.count(key)) return;
  while (g_mesh_bytes + b > kMeshCacheBytes && !g_meshes.empty()) {
    auto lru = g_meshes.begin();
    for (auto it = g_meshes.begin(); it != g_meshes.end(); ++it)
      if (it->second.used < lru->second.used) lru = it;
    g_mesh_bytes -= lru->second.bytes;
    g_meshes.erase(lru);
  }
  g_meshes[key] = MeshEntry{m, b, ++g_mesh_clock};
  g_mesh_bytes += b;
}

}  // namespace

void load_case(HostCase& hc, const std::string& paramPath, bool msh_binary) {
  load_params(hc, paramPath);
  std::string grid = hc.gridfile;
  if (grid.empty()) throw ParamError("no gridfile line in " + paramPath);
  if (grid[0] != '/') {
    size_t sl = paramPath.find_last_of('/');
    if (sl != std::string::npos) grid = paramPath.substr(0, sl + 1) + grid;
  }
  load_mesh_cached(hc, grid, msh_binary);
  size_t sl = paramPath.find_last_of('/');
  hc.backup_path = (sl == std::string::npos ? std::string() : paramPath.substr(0, sl + 1)) + "res.sav";
  init_fields(hc);
}

}  // namespace cycas
