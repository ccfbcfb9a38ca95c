// Logs the single-rank runtime keeps for the main program (refpin_main.cpp) (TEST INFRASTRUCTURE ONLY).
#pragma once
#include <vector>

namespace refpin {
struct KspRecord { int type; int its; int reason; double rnorm; };   // type: 0 GMRES, 1 CG
// every MPI_Allreduce of doubles, in call order (the residual vector of each SIMPLE iteration is
// the one of length 10, navier.cpp:94)
const std::vector<std::vector<double>>& allreduce_log();
// every KSPSolve, in call order
const std::vector<KspRecord>& ksp_log();
void clear_logs();
}  // namespace refpin
