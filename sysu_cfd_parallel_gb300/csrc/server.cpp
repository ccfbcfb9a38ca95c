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
//      stay from the old batch to the new one on the device.  With cycas_server_set_async_rebuild
//      the new batch is built on a worker thread while the old one keeps iterating its members,
//      and the server switches to it at the first step after it is ready (newly admitted cases
//      start iterating then);
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
#include <future>
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
  int in_build = 0;         // batches being built from this request's case
  bool free_case = false;   // free cs once no build reads it
};

void release_case(Request* r) {
  if (r->cs && r->in_build == 0) {
    cycas_case_free(r->cs);
    r->cs = nullptr;
    r->free_case = false;
  } else if (r->cs) {
    r->free_case = true;
  }
}

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
  int async = 0;  // build new batches on a worker thread (cycas_server_set_async_rebuild)
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
    // the next batch, built on a worker thread from a snapshot of the active cases
    struct Build {
      std::future<int> done;
      cycas_ctx* ctx = nullptr;
      std::vector<Request*> members;
      double seconds = 0.0;  // host time of the build
      std::string error;
      bool admitted = false;  // started for newly admitted requests (admission pacing)
    };
    std::unique_ptr<Build> build;
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

// starts building the next batch of class K from its active cases on a worker thread (each
// batch context has its own stream; the library's error text and launch count are per thread)
void start_build(cycas_server* s, cycas_server::Class& K) {
  auto B = std::make_unique<cycas_server::Class::Build>();
  std::vector<const cycas_case*> cases;
  for (auto& r : K.active) {
    cases.push_back(r->cs);
    B->members.push_back(r.get());
    r->in_build++;
  }
  cycas_server::Class::Build* Bp = B.get();
  const cycas_options opt = s->opt;
  const int graph = s->graph;
  auto job = [Bp, cases, opt, graph]() -> int {
    const double t0 = now_s();
    int rc = cycas_batch_create(cases.data(), (int32_t)cases.size(), &opt, &Bp->ctx);
    if (rc == CYCAS_OK && graph) rc = cycas_set_graph(Bp->ctx, 1);  // captured on its first iteration
    if (rc != CYCAS_OK) Bp->error = cycas_last_error();
    Bp->seconds = now_s() - t0;
    return rc;
  };
  try {
    B->done = std::async(s->async ? std::launch::async : std::launch::deferred, job);
  } catch (const std::exception&) {  // no worker thread: build when the result is asked for
    B->done = std::async(std::launch::deferred, job);
  }
  K.build = std::move(B);
  K.dirty = false;
}

bool build_ready(const cycas_server::Class& K) {
  if (!K.build) return false;
  const std::future_status st = K.build->done.wait_for(std::chrono::seconds(0));
  return st == std::future_status::ready || st == std::future_status::deferred;  // deferred: built on get()
}

// the built batch becomes K's batch (waiting for the worker if needed): the state of cases
// already in the old batch is copied over on the device (it has advanced while the new batch was
// built), newly admitted cases get their volume (the residual of a case is normalised by it), the
// old batch is destroyed and the budget of the cases that left with it is released
int finish_build(cycas_server* s, cycas_server::Class& K) {
  std::unique_ptr<cycas_server::Class::Build> B = std::move(K.build);
  const int brc = B->done.get();
  for (Request* r : B->members) {
    r->in_build--;
    if (r->free_case) release_case(r);
  }
  s->t_rebuild += B->seconds;
  s->n_rebuild++;
  if (B->admitted) s->last_admit_rebuild_s += B->seconds;
  if (brc != CYCAS_OK) {
    if (B->ctx) cycas_destroy(B->ctx);
    s->err = B->error;
    return brc;
  }
  cycas_ctx* old = K.ctx;
  const std::vector<Request*> old_members = K.members;
  K.ctx = B->ctx;
  K.members = B->members;
  // an error leaves the server unusable; the old batch goes all the same
  auto give_up = [&](int rc) {
    const int out = fail(s, rc);
    if (old) cycas_destroy(old);
    return out;
  };
  for (size_t k = 0; k < K.members.size(); k++) {
    auto it = std::find(old_members.begin(), old_members.end(), K.members[k]);
    if (it != old_members.end()) {
      int rc = cycas_batch_copy_case(K.ctx, (int32_t)k, old, (int32_t)(it - old_members.begin()));
      if (rc != CYCAS_OK) return give_up(rc);
    }
  }
  std::vector<int32_t> off(K.members.size() + 1);
  cycas_batch_offsets(K.ctx, 0, off.data());
  for (size_t k = 0; k < K.members.size(); k++) {
    Request* r = K.members[k];
    if (r->volume > 0.0) continue;
    std::vector<double> vol(off[k + 1] - off[k]);
    int rc = cycas_batch_case_field(K.ctx, (int32_t)k, "cell_vol", vol.data(), (int64_t)vol.size());
    if (rc != CYCAS_OK) return give_up(rc);
    r->volume = std::accumulate(vol.begin(), vol.end(), 0.0);
  }
  if (old) cycas_destroy(old);
  // members that retired while the batch was built stay in it until the next rebuild
  double cells = 0.0, rcells = 0.0, rfoot = 0.0;
  for (Request* r : K.members) {
    cells += (double)r->dims[0];
    if (r->status != 0) {
      rcells += (double)r->dims[0];
      rfoot += r->footprint;
    }
  }
  s->in_use -= K.retired_footprint - rfoot;
  K.retired_footprint = rfoot;
  K.cells = cells;
  K.retired_cells = rcells;
  if (rcells > 0.0 && rcells >= 0.25 * cells) K.dirty = true;
  return CYCAS_OK;
}

// a class without active cases: its batch goes, with the budget of its (retired) members
void drop_batch(cycas_server* s, cycas_server::Class& K) {
  if (K.ctx) cycas_destroy(K.ctx);
  K.ctx = nullptr;
  K.members.clear();
  s->in_use -= K.retired_footprint;
  K.retired_footprint = 0.0;
  K.cells = K.retired_cells = 0.0;
  K.dirty = false;
}

// synchronous rebuild (a class with no batch to iterate meanwhile, or budget to release now)
int rebuild_now(cycas_server* s, cycas_server::Class& K) {
  if (K.build) {
    int rc = finish_build(s, K);
    if (rc != CYCAS_OK) return rc;
  }
  if (K.active.empty()) {
    drop_batch(s, K);
    return CYCAS_OK;
  }
  start_build(s, K);
  return finish_build(s, K);
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

int cycas_server_set_async_rebuild(cycas_server* s, int32_t on) {
  if (!s) return CYCAS_ERR_INVALID;
  s->async = on ? 1 : 0;
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
  for (auto& kv : s->classes) {
    auto& K = kv.second;
    if (K.build) {
      K.build->done.wait();
      if (K.build->ctx) cycas_destroy(K.build->ctx);
      for (Request* r : K.build->members) r->in_build--;
      K.build.reset();
    }
    if (K.ctx) cycas_destroy(K.ctx);
  }
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
      int rc = rebuild_now(s, K);
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
  // 2-4. per class: switch to a built batch, start a rebuild if needed, one iteration, retire
  for (auto& kv : s->classes) {
    auto& K = kv.second;
    if (build_ready(K)) {
      int rc = finish_build(s, K);
      if (rc != CYCAS_OK) return rc;
    }
    if (K.dirty && !K.build) {
      if (K.active.empty()) {
        drop_batch(s, K);
      } else {
        start_build(s, K);
        K.build->admitted = admitted.count(kv.first) > 0;
        if (!K.ctx || !s->async) {  // nothing to iterate meanwhile, or built in line
          int rc = finish_build(s, K);
          if (rc != CYCAS_OK) return rc;
        }
      }
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
          release_case(r.get());  // at once, or when no batch build reads it any more
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
