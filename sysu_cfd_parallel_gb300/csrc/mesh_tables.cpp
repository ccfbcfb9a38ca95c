// Host tables derived from a mesh's topology: CSR pattern, slots, diagonal positions and the
// per-cell face orders (see mesh_tables.h).  Two passes over the cells, each split into
// contiguous chunks on the host's threads: the row lengths (with the topology checks), then, after
// a prefix sum gives the row starts, every row's columns and the cell's tables.
#include "mesh_tables.h"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>

namespace cycas {

namespace {

// Runs body(chunk, lo, hi) over `chunks` contiguous ranges of [0, n) on as many threads.
template <class Body>
void run_chunks(int n, int chunks, const Body& body) {
  std::vector<std::thread> pool;
  int started = 1;
  for (int t = 1; t < chunks; t++) {
    try {
      pool.emplace_back([&, t]() { body(t, (int)((long)n * t / chunks), (int)((long)n * (t + 1) / chunks)); });
      started++;
    } catch (const std::system_error&) {  // no more threads: the calling thread takes the rest
      break;
    }
  }
  body(0, 0, (int)((long)n / chunks));
  for (int t = started; t < chunks; t++) body(t, (int)((long)n * t / chunks), (int)((long)n * (t + 1) / chunks));
  for (auto& th : pool) th.join();
}

int neighbour(int fid, int i, const int* face_cell1, const int* face_cell2) {
  return face_cell2[fid] < 0 ? -1 : (face_cell1[fid] == i ? face_cell2[fid] : face_cell1[fid]);
}

// the cell's own index and its face neighbours, sorted and unique; returns how many
int row_columns(int i, int k, const int* faces, const int* face_cell1, const int* face_cell2, int* cols) {
  int m = 0;
  cols[m++] = i;
  for (int j = 0; j < k; j++) {
    const int nbh = neighbour(faces[j], i, face_cell1, face_cell2);
    if (nbh >= 0) cols[m++] = nbh;
  }
  std::sort(cols, cols + m);
  return (int)(std::unique(cols, cols + m) - cols);
}

}  // namespace

MeshTables mesh_tables(int n, int nf, const int* cell_nface, const int* cell_face, const int* face_cell1,
                       const int* face_cell2) {
  MeshTables T;
  const size_t sn = (size_t)n;
  // every entry is written once below, by the thread that owns its cell
  T.rowptr.resize(sn + 1);
  T.rowptr[0] = 0;
  T.diag.resize(sn);
  T.face_sm.resize(6 * sn);
  T.gface.resize(6 * sn);
  T.slot.resize(6 * sn);
  const int hw = (int)std::thread::hardware_concurrency();
  const int chunks = n < (1 << 16) ? 1 : std::max(1, std::min(hw, 16));

  // pass 1: checks and row lengths (rowptr[i + 1] = length of row i); each chunk keeps its first
  // failing cell, and the lowest one over all chunks is reported, as a serial pass would
  std::vector<int> bad_cell(chunks, -1);
  std::vector<std::string> bad_msg(chunks);
  run_chunks(n, chunks, [&](int ch, int lo, int hi) {
    int cols[7];
    for (int i = lo; i < hi; i++) {
      const int k = cell_nface[i];
      const char* err = nullptr;
      if (k < 1 || k > 6) err = "cell_nface out of range";
      for (int j = 0; j < k && !err; j++) {
        const int fid = cell_face[6 * (size_t)i + j];
        if (fid < 0 || fid >= nf) err = "cell_face out of range";
        else if (face_cell1[fid] != i && face_cell2[fid] != i) err = "cell_face does not touch its cell";
      }
      if (err) {
        bad_cell[ch] = i;
        bad_msg[ch] = err;
        return;
      }
      T.rowptr[i + 1] = row_columns(i, k, cell_face + 6 * (size_t)i, face_cell1, face_cell2, cols);
    }
  });
  for (int ch = 0; ch < chunks; ch++)
    if (bad_cell[ch] >= 0) throw std::runtime_error(bad_msg[ch]);
  for (size_t i = 0; i < sn; i++) T.rowptr[i + 1] += T.rowptr[i];
  T.col.resize((size_t)T.rowptr[sn]);

  // pass 2: every row's columns and the cell's tables
  run_chunks(n, chunks, [&](int, int lo, int hi) {
    int cols[7], sorted[6];
    for (int i = lo; i < hi; i++) {
      const int k = cell_nface[i];
      const int* faces = cell_face + 6 * (size_t)i;
      const int m = row_columns(i, k, faces, face_cell1, face_cell2, cols);
      const int base = T.rowptr[i];
      std::copy(cols, cols + m, T.col.begin() + base);
      for (int j = 0; j < k; j++) {
        T.face_sm[(size_t)j * sn + i] = faces[j];
        sorted[j] = faces[j];
        const int nbh = neighbour(faces[j], i, face_cell1, face_cell2);
        T.slot[(size_t)j * sn + i] = nbh >= 0 ? base + (int)(std::lower_bound(cols, cols + m, nbh) - cols) : -1;
      }
      std::sort(sorted, sorted + k);
      for (int j = 0; j < k; j++) T.gface[(size_t)j * sn + i] = sorted[j];
      for (int j = k; j < 6; j++) T.face_sm[(size_t)j * sn + i] = T.gface[(size_t)j * sn + i] = T.slot[(size_t)j * sn + i] = -1;
      T.diag[i] = base + (int)(std::lower_bound(cols, cols + m, i) - cols);
    }
  });
  return T;
}

}  // namespace cycas
