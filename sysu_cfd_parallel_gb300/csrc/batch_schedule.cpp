// Teams of the batched Krylov launches (see batch_schedule.h).
#include "batch_schedule.h"

#include <algorithm>
#include <stdexcept>

namespace cycas {

TeamSchedule team_schedule(const std::vector<int>& case_lo, const std::vector<int>& case_hi, int G, double factor) {
  const int nc = (int)case_lo.size();
  if (G < 1 || (int)case_hi.size() != nc) throw std::runtime_error("batch schedule: bad arguments");
  auto rows = [&](int k) { return case_hi[k] - case_lo[k]; };
  long N = 0;
  for (int k = 0; k < nc; k++) N += rows(k);
  const double target = factor * (double)N / G;
  std::vector<int> k_of(nc, 0);  // CTAs of the case's own team, 0 for the smaller cases
  int used = 0;
  bool small = false;
  for (int k = 0; k < nc; k++) {
    if (rows(k) >= target) {
      k_of[k] = std::max(1, (int)(rows(k) / target));
      used += k_of[k];
    } else {
      small = true;
    }
  }
  // the own teams may take every CTA but the one the smaller cases need (if there are any)
  while (used > G - (small ? 1 : 0)) {
    int big = -1;
    for (int k = 0; k < nc; k++)
      if (k_of[k] > 1 && (big < 0 || k_of[k] > k_of[big])) big = k;
    if (big < 0) {  // every own team has one CTA: the smallest case joins the smaller cases
      int sm = -1;
      for (int k = 0; k < nc; k++)
        if (k_of[k] == 1 && (sm < 0 || rows(k) < rows(sm))) sm = k;
      k_of[sm] = 0;
      small = true;
    } else {
      k_of[big]--;
    }
    used--;
  }
  TeamSchedule S;
  auto add_team = [&](int size, const std::vector<int>& cases) {
    const int t = (int)S.team_size.size();
    S.team_cta0.push_back((int)S.cta_team.size());
    S.team_size.push_back(size);
    S.team_case0.push_back((int)S.case_list.size());
    S.case_list.insert(S.case_list.end(), cases.begin(), cases.end());
    for (int r = 0; r < size; r++) {
      S.cta_team.push_back(t);
      S.cta_rank.push_back(r);
    }
  };
  for (int k = 0; k < nc; k++)
    if (k_of[k] > 0) add_team(k_of[k], {k});
  const int rest = G - (int)S.cta_team.size();
  if (small) {
    if (rest < 1) throw std::runtime_error("batch schedule left no CTA for the small cases");
    std::vector<int> order;
    for (int k = 0; k < nc; k++)
      if (k_of[k] == 0) order.push_back(k);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rows(a) > rows(b); });
    const int nteam = std::min(rest, (int)order.size());
    std::vector<long> load(nteam, 0);
    std::vector<std::vector<int>> lists(nteam);
    for (int k : order) {
      const int t = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      lists[t].push_back(k);
      load[t] += rows(k);
    }
    for (int t = 0; t < nteam; t++) {
      std::sort(lists[t].begin(), lists[t].end());
      add_team(1, lists[t]);
    }
  }
  S.team_case0.push_back((int)S.case_list.size());
  return S;
}

}  // namespace cycas
