// Test infrastructure: runs the AMG setup of the pressure preconditioner
// (sysu_cfd_parallel_gb300/csrc/amg_setup.cpp, unmodified) on the host, with an uploader that keeps
// every "device" array in host memory, and exposes the resulting hierarchy through a C ABI so that
// tests/test_cpu_amg_setup.py can check it independently (numpy / scipy) without a GPU.
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../sysu_cfd_parallel_gb300/csrc/cycas_amg.h"

namespace {

struct HostUploader : cycas::AmgUploader {
  std::vector<std::unique_ptr<char[]>> blocks;
  void* take(long bytes) {
    blocks.emplace_back(new char[bytes > 0 ? bytes : 1]());
    return blocks.back().get();
  }
  const int* upload_int(const int* h, long n) override {
    void* p = take(4 * n);
    std::memcpy(p, h, 4 * n);
    return (const int*)p;
  }
  float* alloc_float(long n) override { return (float*)take(4 * n); }
  void* upload_bytes(const void* h, long bytes) override {
    void* p = take(bytes);
    std::memcpy(p, h, bytes);
    return p;
  }
};

struct State {
  HostUploader up;
  cycas::AmgHostView v;
  std::vector<std::shared_ptr<const cycas::AmgHostHierarchy>> cache;
};
std::unique_ptr<State> g;
std::string g_err;

const cycas::AmgDevLevel* level(int c, int l) {
  if (!g || c < 0 || c >= g->v.ncases || l < 0 || l >= g->v.cases[c].nlev) return nullptr;
  return &g->v.levels[c][l];
}

int copy_int(const int* src, long n, int* dst) {
  if (!src) return 1;
  std::memcpy(dst, src, 4 * n);
  return 0;
}

}  // namespace

extern "C" {

const char* amgt_error(void) { return g_err.c_str(); }

// Builds the hierarchies of the cases [lo[c], hi[c]) of the pattern (rowptr/col, strength weight
// per entry).  reuse = 1 keeps the hierarchies of the previous call's cases as the cache (a case
// whose entry is kept is taken as it is).  Returns 0, or 1 with the setup's error text.
int amgt_build(int n, const int* rowptr, const int* col, const double* weight, int ncases, const int* lo,
               const int* hi, int reuse, int gamma) {
  std::vector<std::shared_ptr<const cycas::AmgHostHierarchy>> cache(ncases);
  if (reuse && g && (int)g->cache.size() == ncases) cache = g->cache;
  g.reset(new State());
  g->v.gamma = gamma;
  try {
    cycas::amg_setup_cases(g->v, n, rowptr, col, weight, rowptr, col, nullptr, nullptr,
                           std::vector<int>(lo, lo + ncases), std::vector<int>(hi, hi + ncases), g->up, &cache);
  } catch (const std::exception& e) {
    g_err = e.what();
    g.reset();
    return 1;
  }
  g->cache = cache;
  return 0;
}

// {ncases, depths, smem_bytes}
void amgt_view(int* out) {
  out[0] = g ? g->v.ncases : 0;
  out[1] = g ? (int)g->v.dep.size() : 0;
  out[2] = g ? g->v.smem_bytes : 0;
}

// {nrows, nnz, nnz_next}
int amgt_depth(int l, int* out) {
  if (!g || l < 0 || l >= (int)g->v.dep.size()) return 1;
  const auto& d = g->v.dep[l];
  out[0] = d.nrows;
  out[1] = d.nnz;
  out[2] = d.nnz_next;
  return 0;
}

// depth arrays: "diag" (level > 0) [nrows], "diag_row" [nnz], "cptr" [nnz_next + 1], "csrc"
int amgt_depth_int(int l, const char* name, int* dst, long n) {
  if (!g || l < 0 || l >= (int)g->v.dep.size()) return 1;
  const auto& d = g->v.dep[l];
  if (!std::strcmp(name, "diag")) return copy_int(d.diag, n, dst);
  if (!std::strcmp(name, "diag_row")) return copy_int(d.diag_row, n, dst);
  if (!std::strcmp(name, "cptr")) return copy_int(d.cptr, n, dst);
  if (!std::strcmp(name, "csrc")) return copy_int(d.csrc, n, dst);
  return 1;
}

// {lo, hi, nlev, gamma, tail, tail bytes, offset of the dense inverse}
int amgt_case(int c, int* out) {
  if (!g || c < 0 || c >= g->v.ncases) return 1;
  const auto& cd = g->v.cases[c];
  out[0] = cd.lo;
  out[1] = cd.hi;
  out[2] = cd.nlev;
  out[3] = cd.gamma;
  out[4] = cd.tl.tail;
  out[5] = cd.tl.bytes;
  out[6] = cd.tl.inv;
  return 0;
}

// offsets of tail level l in shared memory, in TailLevelOff order:
// {rowptr, col, val, wdinv, agg, ptptr, ptrow, R, X, T, perm}
int amgt_tail_off(int c, int l, int* out) {
  if (!g || c < 0 || c >= g->v.ncases || l < 0 || l >= cycas::kAmgMaxLevels) return 1;
  std::memcpy(out, &g->v.cases[c].tl.lv[l], sizeof(cycas::TailLevelOff));
  return 0;
}

// {n, nnz, maxagg, nnz_off, sell_len, first row in the depth's rows (level 0: the system's)}
int amgt_level(int c, int l, int* out) {
  const cycas::AmgDevLevel* e = level(c, l);
  if (!e) return 1;
  out[0] = e->n;
  out[1] = e->nnz;
  out[2] = e->maxagg;
  out[3] = e->nnz_off;
  out[4] = e->sell_len;
  out[5] = l == 0 ? g->v.cases[c].lo : (int)(e->wdinv - g->v.dep[l].wdinv);
  return 0;
}

// level arrays (levels >= 1 in the case's local numbering; level 0 arrays are the system's):
// "rowptr" [n + 1], "col" [nnz], "diag" [n], "agg" [n], "ptptr" [n_next + 1], "ptrow" [n],
// "aggcol" [nnz], "sell_ptr" [ceil(n/32) + 1], "sell_src" [sell_len]
int amgt_level_int(int c, int l, const char* name, int* dst, long n) {
  const cycas::AmgDevLevel* e = level(c, l);
  if (!e) return 1;
  if (!std::strcmp(name, "rowptr")) return copy_int(e->rowptr, n, dst);
  if (!std::strcmp(name, "col")) return copy_int(e->col, n, dst);
  if (!std::strcmp(name, "diag")) return copy_int(e->diag, n, dst);
  if (!std::strcmp(name, "agg")) return copy_int(e->agg, n, dst);
  if (!std::strcmp(name, "ptptr")) return copy_int(e->ptptr, n, dst);
  if (!std::strcmp(name, "ptrow")) return copy_int(e->ptrow, n, dst);
  if (!std::strcmp(name, "aggcol")) return copy_int(e->aggcol, n, dst);
  if (!std::strcmp(name, "sell_ptr")) return copy_int(e->sell_ptr, n, dst);
  if (!std::strcmp(name, "sell_src")) return copy_int(e->sell_src, n, dst);
  return 1;
}

// 16-bit level arrays: "sell_col" [sell_len], "sell_row" [32 ceil(n/32)]
int amgt_level_u16(int c, int l, const char* name, unsigned short* dst, long n) {
  const cycas::AmgDevLevel* e = level(c, l);
  if (!e) return 1;
  const unsigned short* src = !std::strcmp(name, "sell_col") ? e->sell_col : !std::strcmp(name, "sell_row") ? e->sell_row : nullptr;
  if (!src) return 1;
  std::memcpy(dst, src, 2 * n);
  return 0;
}

// the library's constants the layout follows: {kAmgMaxLevels, kAmgCoarseMax, kAmgDownBuf,
// kAmgTailBudget, kAmgWRows}
void amgt_constants(int* out) {
  out[0] = cycas::kAmgMaxLevels;
  out[1] = cycas::kAmgCoarseMax;
  out[2] = cycas::kAmgDownBuf;
  out[3] = cycas::kAmgTailBudget;
  out[4] = cycas::kAmgWRows;
}

}  // extern "C"
