// Test infrastructure: loads cases with the library's host loader and concatenates them with the
// batch union (sysu_cfd_parallel_gb300/csrc/{host_case,union_mesh}.cpp, unmodified), exposing the
// arrays through a C ABI for tests/test_cpu_union_mesh.py.
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../sysu_cfd_parallel_gb300/csrc/cycas_host.h"

namespace {
std::vector<std::unique_ptr<cycas::HostCase>> g_cases;
std::unique_ptr<cycas::UnionMesh> g_union;
std::string g_err;

const cycas::HostCase* pick(int k) {
  if (k < 0) return g_union ? &g_union->h : nullptr;
  return k < (int)g_cases.size() ? g_cases[k].get() : nullptr;
}

const std::vector<int32_t>* int_array(const cycas::HostCase& h, const char* nm) {
  if (!std::strcmp(nm, "face_cell1")) return &h.face_cell1;
  if (!std::strcmp(nm, "face_cell2")) return &h.face_cell2;
  if (!std::strcmp(nm, "face_bnd")) return &h.face_bnd;
  if (!std::strcmp(nm, "face_vertices")) return &h.face_vertices;
  if (!std::strcmp(nm, "cell_nface")) return &h.cell_nface;
  if (!std::strcmp(nm, "cell_rid")) return &h.cell_rid;
  if (!std::strcmp(nm, "cell_face")) return &h.cell_face;
  if (!std::strcmp(nm, "cell_cell")) return &h.cell_cell;
  if (!std::strcmp(nm, "cell_vertices")) return &h.cell_vertices;
  if (!std::strcmp(nm, "bnd_face")) return &h.bnd_face;
  if (!std::strcmp(nm, "bnd_type")) return &h.bnd_type;
  if (!std::strcmp(nm, "bnd_rid")) return &h.bnd_rid;
  return nullptr;
}

const std::vector<double>* dbl_array(const cycas::HostCase& h, const char* nm) {
  static const char* names[] = {"vert", "U", "V", "W", "P", "R", "T", "VisLam", "VisTur", "TE", "ED",
                                "BU", "BV", "BW", "BRo", "BTem", "BTE", "BED"};
  const std::vector<double>* arrays[] = {&h.vert, &h.U, &h.V, &h.W, &h.P, &h.R, &h.T, &h.VisLam, &h.VisTur,
                                         &h.TE, &h.ED, &h.BU, &h.BV, &h.BW, &h.BRo, &h.BTem, &h.BTE, &h.BED};
  for (size_t q = 0; q < sizeof(names) / sizeof(names[0]); q++)
    if (!std::strcmp(nm, names[q])) return arrays[q];
  return nullptr;
}
}  // namespace

extern "C" {

const char* un_error(void) { return g_err.c_str(); }

// loads the cases (param.in paths); 0, or 1 with the loader's error
int un_load(const char* const* params, int n) {
  g_cases.clear();
  g_union.reset();
  try {
    for (int k = 0; k < n; k++) {
      g_cases.emplace_back(new cycas::HostCase());
      cycas::load_case(*g_cases.back(), params[k]);
    }
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// the union of the loaded cases; broken >= 0 first marks boundary face 0 of that case interior
// (a case that does not number its boundary faces first).  0, or 1 with the error text
int un_build(int broken) {
  try {
    std::vector<cycas::HostCase> copy;
    std::vector<const cycas::HostCase*> hs;
    if (broken >= 0) {
      for (auto& c : g_cases) copy.push_back(*c);
      copy[broken].face_bnd[0] = -1;
      for (auto& c : copy) hs.push_back(&c);
    } else {
      for (auto& c : g_cases) hs.push_back(c.get());
    }
    g_union.reset(new cycas::UnionMesh(cycas::build_union(hs)));
  } catch (const std::exception& e) {
    g_err = e.what();
    g_union.reset();
    return 1;
  }
  return 0;
}

// {ncel, nfac, nbnd, nvrt} of case k (k < 0: the union)
int un_dims(int k, long* out) {
  const cycas::HostCase* h = pick(k);
  if (!h) return 1;
  out[0] = h->ncel;
  out[1] = h->nfac;
  out[2] = h->nbnd;
  out[3] = h->nvrt;
  return 0;
}

// the union's per-case offsets: kind 0 cell0, 1 bnd0, 2 iface0 ([ncases + 1])
int un_offsets(int kind, int* dst) {
  if (!g_union) return 1;
  const std::vector<int>& v = kind == 0 ? g_union->cell0 : kind == 1 ? g_union->bnd0 : g_union->iface0;
  std::memcpy(dst, v.data(), sizeof(int) * v.size());
  return 0;
}

// array length of case k (k < 0: the union), -1 for an unknown name
long un_len(int k, const char* nm) {
  const cycas::HostCase* h = pick(k);
  if (!h) return -1;
  if (auto a = int_array(*h, nm)) return (long)a->size();
  if (auto a = dbl_array(*h, nm)) return (long)a->size();
  return -1;
}

int un_geti(int k, const char* nm, int32_t* dst, long n) {
  const cycas::HostCase* h = pick(k);
  const std::vector<int32_t>* a = h ? int_array(*h, nm) : nullptr;
  if (!a || (long)a->size() != n) return 1;
  std::memcpy(dst, a->data(), sizeof(int32_t) * n);
  return 0;
}

int un_getd(int k, const char* nm, double* dst, long n) {
  const cycas::HostCase* h = pick(k);
  const std::vector<double>* a = h ? dbl_array(*h, nm) : nullptr;
  if (!a || (long)a->size() != n) return 1;
  std::memcpy(dst, a->data(), sizeof(double) * n);
  return 0;
}

}  // extern "C"
