#include "mixed.h"

namespace sihg {
int solve_mixed(const HostProblem&, const sih_pdhg_config&, const sih_pdhg_options&, sih_pdhg_result*) {
    return fail(SIH_PDHG_ERR_UNSUPPORTED, "mixed algorithm not built yet");
}
}  // namespace sihg
