// Test infrastructure: exposes the team schedule of batched Krylov launches
// (sysu_cfd_parallel_gb300/csrc/batch_schedule.cpp, unmodified) through a C ABI for
// tests/test_cpu_batch_schedule.py.
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../sysu_cfd_parallel_gb300/csrc/batch_schedule.h"

namespace {
std::unique_ptr<cycas::TeamSchedule> g;
std::string g_err;

const std::vector<int>* array(const char* nm) {
  if (!g) return nullptr;
  if (!std::strcmp(nm, "cta_team")) return &g->cta_team;
  if (!std::strcmp(nm, "cta_rank")) return &g->cta_rank;
  if (!std::strcmp(nm, "team_size")) return &g->team_size;
  if (!std::strcmp(nm, "team_cta0")) return &g->team_cta0;
  if (!std::strcmp(nm, "team_case0")) return &g->team_case0;
  if (!std::strcmp(nm, "case_list")) return &g->case_list;
  return nullptr;
}
}  // namespace

extern "C" {

const char* bs_error(void) { return g_err.c_str(); }

// 0, or 1 with the error text
int bs_build(const int* lo, const int* hi, int nc, int G, double factor) {
  try {
    g.reset(new cycas::TeamSchedule(
        cycas::team_schedule(std::vector<int>(lo, lo + nc), std::vector<int>(hi, hi + nc), G, factor)));
  } catch (const std::exception& e) {
    g_err = e.what();
    g.reset();
    return 1;
  }
  return 0;
}

long bs_len(const char* nm) {
  const std::vector<int>* a = array(nm);
  return a ? (long)a->size() : -1;
}

int bs_get(const char* nm, int* dst, long n) {
  const std::vector<int>* a = array(nm);
  if (!a || (long)a->size() != n) return 1;
  std::memcpy(dst, a->data(), sizeof(int) * n);
  return 0;
}

}  // extern "C"
