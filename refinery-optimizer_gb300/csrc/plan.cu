// Launch plans of the SpMV core (see spmv.cuh).
#include <algorithm>

#include "spmv.cuh"

namespace sihg {

// About kBatch entries per lane for a mean-length segment: one batch of
// loads covers it.  Power of two in [1, 32].
int default_lanes(double mean_len) {
    int L = 1;
    while (L < 32 && (double)(2 * L * kBatch) <= mean_len * 2.0) L *= 2;
    return L;
}

SpmvPlan make_plan(const std::vector<int>& ptr, int lanes, int heavy_factor, bool exact, int sm_count,
                   std::vector<int>& heavy) {
    SpmvPlan P{};
    const int nseg = (int)ptr.size() - 1;
    const long long nnz = nseg > 0 ? ptr[nseg] : 0;
    P.threads = 256;
    const int wpb = P.threads / 32;
    heavy.clear();
    if (exact) {
        P.lanes = 1;
        P.heavy_threshold = 0x7fffffff;
        P.heavy_count = 0;
        P.heavy_blocks = 0;
        P.light_blocks = std::max(1, std::min((nseg + P.threads - 1) / P.threads, sm_count * 8));
        return P;
    }
    if (lanes <= 0) lanes = default_lanes(nseg > 0 ? (double)nnz / nseg : 1.0);
    lanes = std::max(1, std::min(32, lanes));
    while (lanes & (lanes - 1)) lanes &= lanes - 1;  // round down to a power of two
    if (heavy_factor <= 0) heavy_factor = 16;
    P.lanes = lanes;
    P.heavy_threshold = std::max(lanes * heavy_factor, 32);
    long long heavy_nnz = 0;
    for (int s = 0; s < nseg; ++s) {
        const int len = ptr[s + 1] - ptr[s];
        if (len > P.heavy_threshold) {
            heavy.push_back(s);
            heavy_nnz += len;
        }
    }
    P.heavy_count = (int)heavy.size();
    const int cap = sm_count * 8;  // 8 resident 256-thread blocks per SM
    const int groups_per_block = wpb * (32 / lanes);
    const int light_needed = std::max(1, (nseg + groups_per_block - 1) / groups_per_block);
    if (P.heavy_count == 0) {
        P.heavy_blocks = 0;
        P.light_blocks = std::min(light_needed, cap);
    } else {
        // split the resident blocks in proportion to the nonzeros each class holds
        const double share = nnz > 0 ? (double)heavy_nnz / (double)nnz : 0.0;
        int hb = std::max(1, (int)(cap * share + 0.5));
        hb = std::min(hb, (P.heavy_count + wpb - 1) / wpb);
        P.heavy_blocks = hb;
        P.light_blocks = std::max(1, std::min(light_needed, cap - hb));
    }
    return P;
}

}  // namespace sihg
