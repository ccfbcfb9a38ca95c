// Test infrastructure: a deterministic stand-in for the calls of include/cycasgpu.h that the
// request server (sysu_cfd_parallel_gb300/csrc/server.cpp) makes -- case loading, batch
// contexts, one batch iteration, state moves between batches -- so that the server's host logic
// (admission under the HBM budget and the cell cap, batch re-forming, retirement, budget release,
// the worker-thread rebuild) runs and is checked without a GPU.  tests/test_cpu_server_host.py
// links it with the unmodified server.cpp.
//
// A case is named by its "param path": comma-separated key=value pairs
//   cells=N    cells of the mesh (default 100)
//   turb=T     turbulence model (default 0)
//   conv=K     the iteration whose normalised residual first falls to 0.9e-6 (default 10)
//   nan=K      the residual is NaN from iteration K on (default never)
//   steady=0   a transient case (the server must refuse it)
// A case's state in a batch is its iteration count `it`; after iteration `it` its normalised
// residual (localRes max over the case's volume) is 0.9e-6 * 2^(conv - it).  A request's outcome
// thus depends on that count alone, and state lost or mixed up when a batch is re-formed shows in
// the iterations the request reports and in its kept field U (= it at retirement).
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "../include/cycasgpu.h"

struct cycas_case {
  int64_t cells = 100;
  int turb = 0, conv = 10, nan_at = 0, steady = 1;
  bool freed = false;
};

struct Spec {
  int64_t cells;
  int turb, conv, nan_at;
};

struct cycas_ctx {
  std::vector<Spec> cases;
  std::vector<int> it;
  std::vector<int32_t> off;
};

namespace {

thread_local std::string g_err;
std::mutex g_mu;
std::set<const cycas_ctx*> g_live_ctx;
std::vector<cycas_case*> g_graveyard;  // freed cases, kept so that a late read is detected
std::atomic<long> g_live_cases{0}, g_creates{0}, g_worker_creates{0}, g_overlapped{0}, g_copies{0},
    g_use_after_free{0}, g_building{0}, g_largest{0}, g_max_cells{0};
std::thread::id g_main;
int g_build_ms = 0, g_iter_us = 0, g_fail_create_at = 0, g_fail_copy_at = 0;

int err(int rc, const char* msg) {
  g_err = msg;
  return rc;
}

void bump_max(std::atomic<long>& a, long v) {
  long cur = a.load();
  while (v > cur && !a.compare_exchange_weak(cur, v)) {
  }
}

double rho(const Spec& s, int it) {
  if (s.nan_at > 0 && it >= s.nan_at) return std::nan("");
  return 0.9e-6 * std::ldexp(1.0, s.conv - it);
}

}  // namespace

extern "C" {

// build_ms: host time of one batch create; iter_us: of one batch iteration; fail_create_at /
// fail_copy_at: the n-th create / state copy fails (1-based, 0: never).  Also resets the counters
// and takes the calling thread as the server's own.
void fake_configure(int build_ms, int iter_us, int fail_create_at, int fail_copy_at) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_build_ms = build_ms;
  g_iter_us = iter_us;
  g_fail_create_at = fail_create_at;
  g_fail_copy_at = fail_copy_at;
  for (cycas_case* c : g_graveyard) delete c;
  g_graveyard.clear();
  g_creates = g_worker_creates = g_overlapped = g_copies = g_use_after_free = g_largest = g_max_cells = 0;
  g_main = std::this_thread::get_id();
}

// [0] live cases [1] live batch contexts [2] creates [3] creates on a thread other than the
// server's [4] batch iterations run while a create was in progress [5] most cases in one batch
// [6] state copies [7] reads of a freed case by a create [8] most cells in one batch
void fake_counters(int64_t* out) {
  std::lock_guard<std::mutex> lk(g_mu);
  out[0] = g_live_cases;
  out[1] = (int64_t)g_live_ctx.size();
  out[2] = g_creates;
  out[3] = g_worker_creates;
  out[4] = g_overlapped;
  out[5] = g_largest;
  out[6] = g_copies;
  out[7] = g_use_after_free;
  out[8] = g_max_cells;
}

const char* cycas_last_error(void) { return g_err.c_str(); }

void cycas_options_default(cycas_options* o) { std::memset(o, 0, sizeof(*o)); }

int cycas_case_load(const char* param_path, cycas_case** out) {
  if (!param_path || !out) return err(CYCAS_ERR_INVALID, "null argument");
  auto* c = new cycas_case();
  std::string s(param_path);
  size_t p = 0;
  while (p < s.size()) {
    size_t q = s.find(',', p);
    if (q == std::string::npos) q = s.size();
    const std::string kv = s.substr(p, q - p);
    const size_t e = kv.find('=');
    if (e == std::string::npos) {
      delete c;
      return err(CYCAS_ERR_IO, "fake case: expected key=value");
    }
    const std::string k = kv.substr(0, e);
    const long v = std::atol(kv.c_str() + e + 1);
    if (k == "cells") c->cells = v;
    else if (k == "turb") c->turb = (int)v;
    else if (k == "conv") c->conv = (int)v;
    else if (k == "nan") c->nan_at = (int)v;
    else if (k == "steady") c->steady = (int)v;
    else {
      delete c;
      return err(CYCAS_ERR_IO, "fake case: unknown key");
    }
    p = q + 1;
  }
  g_live_cases++;
  *out = c;
  return CYCAS_OK;
}

void cycas_case_free(cycas_case* c) {
  if (!c) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (c->freed) {
    g_use_after_free++;  // a second free
    return;
  }
  c->freed = true;
  g_live_cases--;
  g_graveyard.push_back(c);
}

int cycas_case_dims(const cycas_case* c, int64_t d[8]) {
  if (!c) return CYCAS_ERR_INVALID;
  std::memset(d, 0, 8 * sizeof(int64_t));
  d[0] = c->cells;
  d[1] = 3 * c->cells;
  d[4] = c->turb;
  d[7] = 7 * c->cells;
  return CYCAS_OK;
}

int cycas_case_physics(const cycas_case* c, int32_t iopt[6], double dopt[3]) {
  if (!c) return CYCAS_ERR_INVALID;
  std::memset(iopt, 0, 6 * sizeof(int32_t));
  std::memset(dopt, 0, 3 * sizeof(double));
  iopt[0] = c->steady;
  return CYCAS_OK;
}

int cycas_batch_create(const cycas_case* const* cases, int32_t ncases, const cycas_options* opt, cycas_ctx** out) {
  if (!cases || ncases < 1 || !opt || !out) return err(CYCAS_ERR_INVALID, "fake create: bad arguments");
  g_building++;
  if (g_build_ms > 0) std::this_thread::sleep_for(std::chrono::milliseconds(g_build_ms));
  const long n = ++g_creates;
  if (std::this_thread::get_id() != g_main) g_worker_creates++;
  auto* x = new cycas_ctx();
  x->off.push_back(0);
  bool bad = false;
  for (int k = 0; k < ncases; k++) {  // read after the delay: a case freed meanwhile is caught
    const cycas_case* c = cases[k];
    if (c->freed) g_use_after_free++;
    if (c->turb != cases[0]->turb) bad = true;
    x->cases.push_back({c->cells, c->turb, c->conv, c->nan_at});
    x->it.push_back(0);
    x->off.push_back(x->off.back() + (int32_t)c->cells);
  }
  g_building--;
  if (bad || opt->ksp[CYCAS_SYS_PRESSURE].pc != CYCAS_PC_AMG) {
    delete x;
    return err(CYCAS_ERR_INVALID, "fake create: cases of one batch must share the physics class, AMG pressure");
  }
  if (n == g_fail_create_at) {
    delete x;
    return err(CYCAS_ERR_ALLOC, "fake create: injected allocation failure");
  }
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_live_ctx.insert(x);
  }
  bump_max(g_largest, ncases);
  bump_max(g_max_cells, x->off.back());
  *out = x;
  return CYCAS_OK;
}

static bool live(const cycas_ctx* x) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_live_ctx.count(x) > 0;
}

void cycas_destroy(cycas_ctx* x) {
  if (!x) return;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_live_ctx.erase(x)) {
      g_use_after_free++;  // destroyed twice
      return;
    }
  }
  delete x;
}

int cycas_set_graph(cycas_ctx* x, int32_t) { return live(x) ? CYCAS_OK : err(CYCAS_ERR_INVALID, "dead context"); }

int cycas_batch_offsets(cycas_ctx* x, int32_t kind, int32_t* off) {
  if (!live(x) || !off) return err(CYCAS_ERR_INVALID, "dead context");
  for (size_t k = 0; k < x->off.size(); k++) off[k] = kind == 0 ? x->off[k] : 0;
  return CYCAS_OK;
}

int cycas_batch_iteration(cycas_ctx* x, double* resmax, int32_t* its, int32_t* reasons) {
  if (!live(x)) return err(CYCAS_ERR_INVALID, "iteration of a dead context");
  if (g_building > 0) g_overlapped++;
  if (g_iter_us > 0) std::this_thread::sleep_for(std::chrono::microseconds(g_iter_us));
  int rc = CYCAS_OK;
  for (size_t k = 0; k < x->cases.size(); k++) {
    const Spec& s = x->cases[k];
    const int it = ++x->it[k];
    const double r = rho(s, it);
    resmax[k] = r * (0.5 * (double)s.cells);  // every cell has volume 0.5
    for (int q = 0; q < 8; q++) {
      its[8 * k + q] = q < 4 ? 1 : -1;
      reasons[8 * k + q] = 0;
    }
    if (std::isnan(r)) {
      reasons[8 * k] = CYCAS_KSP_DIVERGED_NANORINF;
      rc = CYCAS_NAN_DETECTED;
    }
  }
  return rc;
}

int cycas_batch_copy_case(cycas_ctx* dst, int32_t dc, cycas_ctx* src, int32_t sc) {
  if (!live(dst) || !live(src)) return err(CYCAS_ERR_INVALID, "copy between dead contexts");
  if (dc < 0 || sc < 0 || dc >= (int)dst->cases.size() || sc >= (int)src->cases.size())
    return err(CYCAS_ERR_INVALID, "copy: case index out of range");
  const Spec &a = dst->cases[dc], &b = src->cases[sc];
  if (a.cells != b.cells || a.conv != b.conv || a.turb != b.turb || a.nan_at != b.nan_at)
    return err(CYCAS_ERR_INVALID, "copy: the two cases are not the same mesh");
  if (++g_copies == g_fail_copy_at) return err(CYCAS_ERR_CUDA, "fake copy: injected copy failure");
  dst->it[dc] = src->it[sc];
  return CYCAS_OK;
}

int cycas_batch_case_field(cycas_ctx* x, int32_t k, const char* name, double* dst, int64_t n) {
  if (!live(x) || !name || !dst || k < 0 || k >= (int)x->cases.size()) return err(CYCAS_ERR_INVALID, "field: bad arguments");
  if (n != x->cases[k].cells) return err(CYCAS_ERR_INVALID, "field: size mismatch");
  double v;
  if (!std::strcmp(name, "cell_vol")) v = 0.5;
  else if (!std::strcmp(name, "U")) v = x->it[k];
  else if (!std::strcmp(name, "P")) v = x->cases[k].conv;
  else if (!std::strcmp(name, "V") || !std::strcmp(name, "W") || !std::strcmp(name, "TE") || !std::strcmp(name, "ED")) v = 0.0;
  else return err(CYCAS_ERR_INVALID, "field: unknown name");
  for (int64_t i = 0; i < n; i++) dst[i] = v;
  return CYCAS_OK;
}

}  // extern "C"
