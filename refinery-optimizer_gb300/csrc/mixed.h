// Mixed-precision restarted adaptive PDHG (scaled, FP32 SpMV, FP64 reductions).
#pragma once

#include "common.cuh"
#include "host.h"

namespace sihg {

int solve_mixed(const HostProblem& hp, const sih_pdhg_config& cfg, const sih_pdhg_options& opts,
                sih_pdhg_result* r);

void pack_solution(const sih_pdhg_problem* p, const sih_pdhg_options& opts, const std::vector<double>& x,
                   const std::vector<double>& y, sih_pdhg_result* r);

}  // namespace sihg
