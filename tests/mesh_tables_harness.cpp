// Test infrastructure: exposes the host mesh tables (sysu_cfd_parallel_gb300/csrc/mesh_tables.cpp,
// unmodified) through a C ABI for tests/test_cpu_mesh_tables.py.
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "../sysu_cfd_parallel_gb300/csrc/mesh_tables.h"

namespace {
std::unique_ptr<cycas::MeshTables> g;
std::string g_err;
}  // namespace

extern "C" {

// 0 and the number of CSR entries in *nnz, or 1 with the error text in mt_error()
int mt_build(int n, int nf, const int* cell_nface, const int* cell_face, const int* face_cell1, const int* face_cell2,
             long* nnz) {
  try {
    g.reset(new cycas::MeshTables(cycas::mesh_tables(n, nf, cell_nface, cell_face, face_cell1, face_cell2)));
  } catch (const std::exception& e) {
    g_err = e.what();
    g.reset();
    return 1;
  }
  *nnz = (long)g->col.size();
  return 0;
}

const char* mt_error(void) { return g_err.c_str(); }

// "rowptr" [n + 1], "col" [nnz], "diag" [n], "face_sm" / "gface" / "slot" [6 n]
int mt_get(const char* name, int* dst, long n) {
  if (!g) return 1;
  const cycas::IntTable* v = !std::strcmp(name, "rowptr")    ? &g->rowptr
                              : !std::strcmp(name, "col")     ? &g->col
                              : !std::strcmp(name, "diag")    ? &g->diag
                              : !std::strcmp(name, "face_sm") ? &g->face_sm
                              : !std::strcmp(name, "gface")   ? &g->gface
                              : !std::strcmp(name, "slot")    ? &g->slot
                                                              : nullptr;
  if (!v || (long)v->size() != n) return 1;
  std::memcpy(dst, v->data(), sizeof(int) * n);
  return 0;
}

}  // extern "C"
