// Request server: continuous batching of steady SIMPLE-C solves on one GPU.
//
// Requests (a param.in each) queue in arrival order.  Every step the server
//   1. admits queued requests while the estimated device footprint of the active cases stays
//      within the HBM budget (first come, first served: a request that does not fit blocks the
//      ones behind it, so large cases are not starved; one larger than the whole budget runs
//      alone; with cycas_server_set_max_cells also while the active requests' cells stay within
//      a cap, which bounds the time of one step when more work arrives than the GPU does) -- at
//      once when the server is idle, otherwise once the iterations since the last
//      admission have taken as long as the batch rebuild that admission cost (a rebuild of a
//      batch of millions of cells costs about a second of host time; admitting at every step
//      of a busy server would spend most of its time rebuilding);
//   2. rebuilds the batch of every physics class whose membership changed (cases of one batch
//      share the turbulence model and relaxation factors), moving the state of the cases that
//      stay from the old batch to the new one on the device;
//   3. advances every active case by one SIMPLE-C iteration (one batch iteration per class);
//   4. retires every case whose residual, max_i localRes[i] divided by the case's volume, is
//      at or below the tolerance, that reached the iteration cap, or whose fields stopped being
//      finite, recording its times (and fields).  A retired case leaves its batch at the next
//      rebuild, which comes when new requests join the class or when retired cases hold a
//      quarter of the batch's cells: rebuilding a batch of millions of cells costs about a
//      second of host time, so rebuilding at every retirement would cost more than iterating
//      the retired cases along (their results are taken at retirement and no longer change).
// A case's iterations are exactly those it would do alone; only the Krylov inner products
// sum in another order (see the batch contexts).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/cycasgpu.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t id = 0;
  std::string param;
  cycas_case* cs = nullptr;
  int64_t dims[8] = {0};
  double volume = 0.0;
  double footprint = 0.0;
  int turb = 0;
  double t_arrival = 0.0, t_admit = 0.0, t_done = 0.0;
  int iterations = 0;
  double resmax = 0.0;
  int status = 0;  // CYCAS_REQ_*
  std::map<std::string, std::vector<double>> fields;
};

}  // namespace

// device bytes of one case: fields and geometry per cell and face, the CSR systems, the
// Krylov basis (3 systems x (m+1) vectors), and the AMG levels
extern "C" double cycas_footprint_estimate(const cycas_case* cs) {
  int64_t d[8];
  if (!cs || cycas_case_dims(cs, d) != CYCAS_OK) return 0.0;
  const double nc = (double)d[0], nf = (double)d[1], nnz = (double)d[7];
  return nc * (60 * 8.0) + nf * (24 * 8.0) + nnz * (4.0 + 3 * 8.0 + 2 * 4.0) + nc * 3 * 31 * 8.0 + nnz * 10.0;
}

struct cycas_server {
  cycas_options opt;
  double budget = 0.0, tol = 1e-6;
  int max_iters = 10000;
  int keep_fields = 0;
  int graph = 0;  // replay every batch's iterations as one CUDA graph (cycas_server_set_graph)
  double max_cells = 0.0;  // cap on the cells of the active requests (0: none), cycas_server_set_max_cells
  double active_cells = 0.0;
  int64_t next_id = 1;
  std::deque<std::unique_ptr<Request>> queue;
  struct Class {
    std::vector<std::unique_ptr<Request>> active;
    cycas_ctx* ctx = nullptr;
    std::vector<Request*> members;  // case order of ctx (retired members stay until the next rebuild)
    bool dirty = false;
    double cells = 0.0, retired_cells = 0.0;  // of the batch, and of its retired members
    double retired_footprint = 0.0;           // released from the budget at the next rebuild
  };
  std::map<int, Class> classes;  // by turbulence model
  std::vector<std::unique_ptr<Request>> finished;
  double in_use = 0.0;
  std::string err;
  // host wall time of the loop's parts (cycas_server_stats)
  double t_rebuild = 0.0, t_iterate = 0.0, t_admin = 0.0;
  // admission is held back while the iterations since the last admission rebuild have taken
  // less time than that rebuild, so rebuild time stays at most about half of the loop
  double last_admit_rebuild_s = 0.0, iterate_since_admit_s = 0.0;
  int64_t n_rebuild = 0, n_steps = 0;
};

namespace {

int fail(cycas_server* s, int rc) {
  s->err = cycas_last_error();
  return rc;
}

// new batch of class K from its active cases; the state of cases already in the old batch is
// copied over on the device, and newly admitted cases get their volume (the residual of a case
// is normalised by it)
int rebuild(cycas_server* s, cycas_server::Class& K) {
  cycas_ctx* old = K.ctx;
  std::vector<Request*> old_members = K.members;
  K.ctx = nullptr;
  K.members.clear();
  if (!K.active.empty()) {
    std::vector<const cycas_case*> cases;
    for (auto& r : K.active) {
      cases.push_back(r->cs);
      K.members.push_back(r.get());
    }
    int rc = cycas_batch_create(cases.data(), (int32_t)cases.size(), &s->opt, &K.ctx);
    if (rc != CYCAS_OK) return fail(s, rc);
    if (s->graph) {
      rc = cycas_set_graph(K.ctx, 1);  // captured on the batch's first iteration
      if (rc != CYCAS_OK) return fail(s, rc);
    }
    // continuing cases keep their state
    for (size_t k = 0; k < K.members.size(); k++) {
      auto it = std::find(old_members.begin(), old_members.end(), K.members[k]);
      if (it != old_members.end()) {
        rc = cycas_batch_copy_case(K.ctx, (int32_t)k, old, (int32_t)(it - old_members.begin()));
        if (rc != CYCAS_OK) return fail(s, rc);
      }
    }
    // volumes of newly admitted cases
    std::vector<int32_t> off(K.members.size() + 1);
    cycas_batch_offsets(K.ctx, 0, off.data());
    for (size_t k = 0; k < K.members.size(); k++) {
      Request* r = K.members[k];
      if (r->volume > 0.0) continue;
      std::vector<double> vol(off[k + 1] - off[k]);
      rc = cycas_batch_case_field(K.ctx, (int32_t)k, "cell_vol", vol.data(), (int64_t)vol.size());
      if (rc != CYCAS_OK) return fail(s, rc);
      r->volume = std::accumulate(vol.begin(), vol.end(), 0.0);
    }
  }
  if (old) cycas_destroy(old);
  K.dirty = false;
  K.cells = 0.0;
  for (Request* r : K.members) K.cells += (double)r->dims[0];
  K.retired_cells = 0.0;
  s->in_use -= K.retired_footprint;
  K.retired_footprint = 0.0;
  return CYCAS_OK;
}

}  // namespace

extern "C" {

int cycas_server_create(const cycas_options* opt, double hbm_budget_bytes, double residual_tol, int32_t max_iters,
                        int32_t keep_fields, cycas_server** out) {
  if (!out || hbm_budget_bytes <= 0.0 || residual_tol <= 0.0 || max_iters < 1) return CYCAS_ERR_INVALID;
  cycas_server* s = new cycas_server();
  if (opt) s->opt = *opt;
  else cycas_options_default(&s->opt);
  s->opt.ksp[CYCAS_SYS_PRESSURE].pc = CYCAS_PC_AMG;
  s->budget = hbm_budget_bytes;
  s->tol = residual_tol;
  s->max_iters = max_iters;
  s->keep_fields = keep_fields;
  *out = s;
  return CYCAS_OK;
}

int cycas_server_set_max_cells(cycas_server* s, double max_cells) {
  if (!s || max_cells < 0.0) return CYCAS_ERR_INVALID;
  s->max_cells = max_cells;
  return CYCAS_OK;
}

int cycas_server_set_graph(cycas_server* s, int32_t on) {
  if (!s) return CYCAS_ERR_INVALID;
  s->graph = on ? 1 : 0;
  for (auto& kv : s->classes)
    if (kv.second.ctx) {
      int rc = cycas_set_graph(kv.second.ctx, s->graph);
      if (rc != CYCAS_OK) return fail(s, rc);
    }
  return CYCAS_OK;
}

void cycas_server_destroy(cycas_server* s) {
  if (!s) return;
  for (auto& kv : s->classes)
    if (kv.second.ctx) cycas_destroy(kv.second.ctx);
  auto free_req = [](Request* r) {
    if (r->cs) cycas_case_free(r->cs);
  };
  for (auto& r : s->queue) free_req(r.get());
  for (auto& kv : s->classes)
    for (auto& r : kv.second.active) free_req(r.get());
  for (auto& r : s->finished) free_req(r.get());
  delete s;
}

double cycas_server_clock(void) { return now_s(); }

int cycas_server_submit(cycas_server* s, const char* param_path, int64_t* id) {
  if (!s || !param_path) return CYCAS_ERR_INVALID;
  auto r = std::make_unique<Request>();
  r->t_arrival = now_s();
  r->param = param_path;
  int rc = cycas_case_load(param_path, &r->cs);
  if (rc != CYCAS_OK) return fail(s, rc);
  int32_t iopt[6];
  double dopt[3];
  cycas_case_physics(r->cs, iopt, dopt);
  if (!iopt[0] || iopt[3] || iopt[4]) {  // batches hold steady, isothermal, constant-density cases
    cycas_case_free(r->cs);
    s->err = std::string("the server runs steady, isothermal, constant-density requests: ") + param_path;
    return CYCAS_ERR_UNSUPPORTED;
  }
  cycas_case_dims(r->cs, r->dims);
  r->turb = (int)r->dims[4];
  r->footprint = cycas_footprint_estimate(r->cs);
  r->id = s->next_id++;
  if (id) *id = r->id;
  s->queue.push_back(std::move(r));
  return CYCAS_OK;
}

int cycas_server_step(cycas_server* s, int32_t* n_active, int32_t* n_queued) {
  if (!s) return CYCAS_ERR_INVALID;
  s->n_steps++;
  // 1. admission, first come first served within the budget (a request larger than the whole
  // budget runs alone once nothing else is active)
  auto idle = [&]() {
    for (auto& kv : s->classes)
      if (!kv.second.active.empty()) return false;
    return true;
  };
  // the budget still counts retired cases until their batch is rebuilt: when the first queued
  // request does not fit, rebuild the batches that hold retired cases to release them
  if (!s->queue.empty() && s->in_use + s->queue.front()->footprint > s->budget) {
    for (auto& kv : s->classes) {
      auto& K = kv.second;
      if (K.retired_footprint <= 0.0) continue;
      const double t0 = now_s();
      int rc = rebuild(s, K);
      s->t_rebuild += now_s() - t0;
      s->n_rebuild++;
      if (rc != CYCAS_OK) return rc;
    }
  }
  const bool was_idle = idle();
  const bool admit = was_idle || s->iterate_since_admit_s >= s->last_admit_rebuild_s;
  std::map<int, bool> admitted;  // classes that took new requests this step
  auto fits = [&](const Request& r) {
    return s->in_use + r.footprint <= s->budget &&
           (s->max_cells <= 0.0 || s->active_cells + (double)r.dims[0] <= s->max_cells);
  };
  while (admit && !s->queue.empty() && (fits(*s->queue.front()) || idle())) {
    std::unique_ptr<Request> r = std::move(s->queue.front());
    s->queue.pop_front();
    r->t_admit = now_s();
    s->in_use += r->footprint;
    s->active_cells += (double)r->dims[0];
    auto& K = s->classes[r->turb];
    admitted[r->turb] = true;
    K.active.push_back(std::move(r));
    K.dirty = true;
  }
  if (!admitted.empty()) {
    s->last_admit_rebuild_s = 0.0;
    s->iterate_since_admit_s = 0.0;
  }
  // 2-4. per class: rebuild if needed, one iteration, retire
  for (auto& kv : s->classes) {
    auto& K = kv.second;
    if (K.dirty) {
      const double t0 = now_s();
      int rc = rebuild(s, K);
      const double dt = now_s() - t0;
      s->t_rebuild += dt;
      s->n_rebuild++;
      if (admitted.count(kv.first)) s->last_admit_rebuild_s += dt;
      if (rc != CYCAS_OK) return rc;
    }
    if (K.members.empty()) continue;
    const int nc = (int)K.members.size();
    std::vector<double> resmax(nc);
    std::vector<int32_t> its(8L * nc), reasons(8L * nc);
    const double t0 = now_s();
    int rc = cycas_batch_iteration(K.ctx, resmax.data(), its.data(), reasons.data());
    s->t_iterate += now_s() - t0;
    s->iterate_since_admit_s += now_s() - t0;
    // per-case outcomes are judged below; only errors of the batch itself stop the server
    if (rc != CYCAS_OK && rc != CYCAS_NOT_CONVERGED && rc != CYCAS_NAN_DETECTED) return fail(s, rc);
    std::vector<int> retire;
    for (int k = 0; k < nc; k++) {
      Request* r = K.members[k];
      if (r->status != 0) continue;  // retired earlier, iterated along until the next rebuild
      r->iterations++;
      r->resmax = resmax[k] / (r->volume > 0.0 ? r->volume : 1.0);
      // a Krylov solve that stops short (iteration cap, breakdown near a converged field) does
      // not end the request: the outer iteration goes on with its iterate, as long as the
      // fields stay finite
      bool failed = !std::isfinite(r->resmax);
      for (int q = 0; q < 8; q++) failed = failed || reasons[8L * k + q] == CYCAS_KSP_DIVERGED_NANORINF;
      if (failed) r->status = CYCAS_REQ_FAILED;
      else if (r->resmax <= s->tol) r->status = CYCAS_REQ_CONVERGED;
      else if (r->iterations >= s->max_iters) r->status = CYCAS_REQ_MAX_ITERS;
      if (r->status != 0) retire.push_back(k);
    }
    if (!retire.empty()) {
      const double t = now_s();
      for (int k : retire) {
        Request* r = K.members[k];
        r->t_done = t;
        if (s->keep_fields) {
          static const char* names[] = {"U", "V", "W", "P", "TE", "ED"};
          std::vector<int32_t> off(nc + 1);
          cycas_batch_offsets(K.ctx, 0, off.data());
          for (const char* nm : names) {
            std::vector<double> v(off[k + 1] - off[k]);
            if (cycas_batch_case_field(K.ctx, k, nm, v.data(), (int64_t)v.size()) == CYCAS_OK) r->fields[nm] = v;
          }
        }
      }
      std::vector<std::unique_ptr<Request>> keep;
      for (auto& r : K.active) {
        if (r->status != 0) {
          K.retired_footprint += r->footprint;
          K.retired_cells += (double)r->dims[0];
          s->active_cells -= (double)r->dims[0];
          cycas_case_free(r->cs);
          r->cs = nullptr;
          s->finished.push_back(std::move(r));
        } else {
          keep.push_back(std::move(r));
        }
      }
      K.active.swap(keep);
      if (K.active.empty() || K.retired_cells >= 0.25 * K.cells) K.dirty = true;
    }
  }
  int act = 0;
  for (auto& kv : s->classes) act += (int)kv.second.active.size();
  if (n_active) *n_active = act;
  if (n_queued) *n_queued = (int32_t)s->queue.size();
  return CYCAS_OK;
}

int cycas_server_poll(cycas_server* s, cycas_request_result* out, int32_t max, int32_t* n) {
  if (!s || !n) return CYCAS_ERR_INVALID;
  int k = 0;
  for (auto& r : s->finished) {
    if (r->status < 0) continue;  // already reported
    if (k >= max) break;
    cycas_request_result& o = out[k++];
    o.id = r->id;
    o.status = r->status;
    o.iterations = r->iterations;
    o.ncel = (int32_t)r->dims[0];
    o.t_arrival = r->t_arrival;
    o.t_admit = r->t_admit;
    o.t_done = r->t_done;
    o.resmax = r->resmax;
    r->status = -r->status;  // mark reported
  }
  *n = k;
  return CYCAS_OK;
}

int cycas_server_result_field(cycas_server* s, int64_t id, const char* name, double* dst, int64_t n) {
  if (!s || !name || !dst) return CYCAS_ERR_INVALID;
  for (auto& r : s->finished)
    if (r->id == id) {
      auto it = r->fields.find(name);
      if (it == r->fields.end() || (int64_t)it->second.size() != n) return CYCAS_ERR_INVALID;
      std::memcpy(dst, it->second.data(), sizeof(double) * n);
      return CYCAS_OK;
    }
  return CYCAS_ERR_INVALID;
}

const char* cycas_server_last_error(cycas_server* s) { return s ? s->err.c_str() : ""; }

int cycas_server_stats(cycas_server* s, double* out) {
  if (!s || !out) return CYCAS_ERR_INVALID;
  out[0] = (double)s->n_steps;
  out[1] = (double)s->n_rebuild;
  out[2] = s->t_rebuild;
  out[3] = s->t_iterate;
  return CYCAS_OK;
}

}  // extern "C"
