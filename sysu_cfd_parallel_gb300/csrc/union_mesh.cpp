// Batches: independent cases concatenated into one mesh (UnionMesh, cycas_host.h).  The sizes of
// every case's slices are known from the cases, so the union's arrays are sized once and every
// case writes its own slices on the host's threads.
#include <algorithm>
#include <vector>

#include "cycas_host.h"
#include "host_threads.h"

namespace cycas {

namespace {

// the InitFlowField arrays of a case: per cell, then per boundary face
std::vector<double> HostCase::* const kCellFields[] = {&HostCase::U, &HostCase::V, &HostCase::W, &HostCase::P,
                                                       &HostCase::R, &HostCase::T, &HostCase::VisLam,
                                                       &HostCase::VisTur, &HostCase::TE, &HostCase::ED};
std::vector<double> HostCase::* const kBndFields[] = {&HostCase::BU, &HostCase::BV, &HostCase::BW, &HostCase::BRo,
                                                      &HostCase::BTem, &HostCase::BTE, &HostCase::BED};

}  // namespace

UnionMesh build_union(const std::vector<const HostCase*>& hs) {
  UnionMesh u;
  HostCase& U = u.h;
  const int nc = (int)hs.size();
  // first cell, boundary face, interior face (counted from the first interior face) and vertex
  // of every case, and the first element of every concatenated array
  std::vector<long> c0(nc + 1, 0), b0(nc + 1, 0), i0(nc + 1, 0), v0(nc + 1, 0), x0(nc + 1, 0);
  constexpr int kNF = sizeof(kCellFields) / sizeof(kCellFields[0]) + sizeof(kBndFields) / sizeof(kBndFields[0]);
  std::vector<std::vector<long>> f0(kNF, std::vector<long>(nc + 1, 0));
  for (int k = 0; k < nc; k++) {
    const HostCase& h = *hs[k];
    c0[k + 1] = c0[k] + h.ncel;
    b0[k + 1] = b0[k] + h.nbnd;
    i0[k + 1] = i0[k] + (h.nfac - h.nbnd);
    v0[k + 1] = v0[k] + h.nvrt;
    x0[k + 1] = x0[k] + (long)h.vert.size();
    int q = 0;
    for (auto m : kCellFields) f0[q][k + 1] = f0[q][k] + (long)(h.*m).size(), q++;
    for (auto m : kBndFields) f0[q][k + 1] = f0[q][k] + (long)(h.*m).size(), q++;
  }
  const long NC = c0[nc], NB = b0[nc], NF = NB + i0[nc];
  U.ncel = (int)NC;
  U.nbnd = (int)NB;
  U.nfac = (int)NF;
  U.nvrt = (int)v0[nc];
  U.face_cell1.resize(NF);
  U.face_cell2.resize(NF);
  U.face_bnd.resize(NF);
  U.face_vertices.resize(4 * NF);
  U.cell_nface.resize(NC);
  U.cell_rid.resize(NC);
  U.cell_face.resize(6 * NC);
  U.cell_cell.resize(6 * NC);
  U.cell_vertices.resize(8 * NC);
  U.bnd_face.resize(NB);
  U.bnd_type.resize(NB);
  U.bnd_rid.resize(NB);
  U.vert.resize(x0[nc]);
  {
    int q = 0;
    for (auto m : kCellFields) (U.*m).resize(f0[q++][nc]);
    for (auto m : kBndFields) (U.*m).resize(f0[q++][nc]);
  }
  u.cell0.assign(nc + 1, 0);
  u.bnd0.assign(nc + 1, 0);
  u.iface0.assign(nc + 1, 0);
  for (int k = 0; k <= nc; k++) {
    u.cell0[k] = (int)c0[k];
    u.bnd0[k] = (int)b0[k];
    u.iface0[k] = (int)(NB + i0[k]);
  }

  std::vector<long> work(nc);
  for (int k = 0; k < nc; k++) work[k] = hs[k]->nfac + 8L * hs[k]->ncel;
  rethrow_first(for_each_case(work, [&](int k) {
    const HostCase& h = *hs[k];
    for (int f = 0; f < h.nfac; f++)
      if ((h.face_bnd[f] >= 0) != (f < h.nbnd) || (f < h.nbnd && h.face_bnd[f] != f))
        throw MeshError("a batched case does not number its boundary faces first");
    const int cb = (int)c0[k], bb = (int)b0[k], ib = (int)(NB + i0[k]), vb = (int)v0[k];
    auto fmap = [&](int f) { return f < h.nbnd ? bb + f : ib + (f - h.nbnd); };
    for (int f = 0; f < h.nfac; f++) {
      const long g = fmap(f);
      U.face_cell1[g] = h.face_cell1[f] + cb;
      U.face_cell2[g] = h.face_cell2[f] >= 0 ? h.face_cell2[f] + cb : h.face_cell2[f];
      U.face_bnd[g] = h.face_bnd[f] >= 0 ? h.face_bnd[f] + bb : h.face_bnd[f];
      for (int q = 0; q < 4; q++) U.face_vertices[4 * g + q] = h.face_vertices[4L * f + q] + vb;
    }
    for (int i = 0; i < h.ncel; i++) {
      const long c = cb + i;
      U.cell_nface[c] = h.cell_nface[i];
      U.cell_rid[c] = h.cell_rid[i];
      for (int j = 0; j < 6; j++) {
        const int f = h.cell_face[6L * i + j], cc = h.cell_cell[6L * i + j];
        U.cell_face[6 * c + j] = f >= 0 ? fmap(f) : f;
        U.cell_cell[6 * c + j] = cc >= 0 ? cc + cb : cc;
      }
      for (int q = 0; q < 8; q++) U.cell_vertices[8 * c + q] = h.cell_vertices[8L * i + q] + vb;
    }
    for (int b = 0; b < h.nbnd; b++) {
      U.bnd_face[bb + b] = fmap(h.bnd_face[b]);
      U.bnd_type[bb + b] = h.bnd_type[b];
      U.bnd_rid[bb + b] = h.bnd_rid[b];
    }
    std::copy(h.vert.begin(), h.vert.end(), U.vert.begin() + x0[k]);
    int q = 0;
    for (auto m : kCellFields) std::copy((h.*m).begin(), (h.*m).end(), (U.*m).begin() + f0[q++][k]);
    for (auto m : kBndFields) std::copy((h.*m).begin(), (h.*m).end(), (U.*m).begin() + f0[q++][k]);
  }));
  return u;
}

}  // namespace cycas
