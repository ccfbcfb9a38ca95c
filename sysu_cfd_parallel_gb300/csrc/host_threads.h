// Case-parallel host work: independent jobs (one per case of a batch) on the host's threads.
#pragma once
#include <algorithm>
#include <atomic>
#include <exception>
#include <numeric>
#include <system_error>
#include <thread>
#include <vector>

namespace cycas {

// Runs job(k) for every k in [0, work.size()), the largest work[k] first, on up to 16 of the
// host's hardware threads (on the calling thread alone when the work sums to less than 65536).
// Every job must write only its own k's outputs, so the results do not depend on the thread
// count.  Returns the exception each job raised (null where none), so that the caller can report
// them in index order.
template <class Job>
std::vector<std::exception_ptr> for_each_case(const std::vector<long>& work, const Job& job) {
  const int n = (int)work.size();
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
  const long total = std::accumulate(work.begin(), work.end(), 0L);
  const int hw = (int)std::thread::hardware_concurrency();
  const int nt = total < (1L << 16) ? 1 : std::max(1, std::min(std::min(n, hw), 16));
  std::vector<std::exception_ptr> err(n);
  std::atomic<int> next{0};
  auto run = [&]() {
    for (int q = next++; q < n; q = next++) {
      try {
        job(order[q]);
      } catch (...) {
        err[order[q]] = std::current_exception();
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) {
    try {
      pool.emplace_back(run);
    } catch (const std::system_error&) {  // no more threads: the ones running share the jobs
      break;
    }
  }
  run();
  for (auto& th : pool) th.join();
  return err;
}

inline void rethrow_first(const std::vector<std::exception_ptr>& err) {
  for (const auto& e : err)
    if (e) std::rethrow_exception(e);
}

}  // namespace cycas
