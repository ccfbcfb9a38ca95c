// Teams of the batched Krylov launches: how the CTAs of one cooperative launch are split among
// the cases of a batch (host side; the device copy is BatchSchedule, cycas_device.h).
#pragma once
#include <vector>

namespace cycas {

struct TeamSchedule {
  std::vector<int> cta_team;    // [grid] team of each CTA
  std::vector<int> cta_rank;    // [grid] rank of each CTA in its team
  std::vector<int> team_size;   // [nteams] CTAs per team
  std::vector<int> team_cta0;   // [nteams] first CTA of the team
  std::vector<int> team_case0;  // [nteams + 1] the team's cases are case_list[team_case0[t] .. team_case0[t+1])
  std::vector<int> case_list;   // case indices in team order
};

// Teams for G CTAs (G >= 1) over the cases [case_lo[k], case_hi[k]) of N rows in all: a case with
// at least factor * N / G rows gets a team of about rows * G / (factor * N) CTAs of its own (fewer,
// largest teams first, when they would not leave a CTA for the smaller cases; if every such case is
// down to one CTA, the smallest of them joins the smaller cases); the smaller cases are spread over
// single-CTA teams, largest first onto the least loaded team, each team's cases in ascending order.
// Every case is in exactly one team, and the teams hold at most G CTAs.
TeamSchedule team_schedule(const std::vector<int>& case_lo, const std::vector<int>& case_hi, int G, double factor);

}  // namespace cycas
