// TaskLayout: schedules of both sides and element chunks on the device.
#include <algorithm>
#include <cstring>

#include "mixed.h"

namespace sihg {

namespace {

int upload(DevMem& d, const void* h, size_t bytes, cudaStream_t s) {
    SIHG_TRY(d.alloc(bytes));
    if (bytes) SIHG_CUDA(cudaMemcpyAsync(d.as<void>(), h, bytes, cudaMemcpyHostToDevice, s));
    return SIH_PDHG_OK;
}

// One side's schedule in one device buffer (16-byte aligned sections) plus
// its partial slots; tick = this side's [B tickets | 2 counters | group tickets].
int upload_side(const SideSchedule& sc, int B, const SegMatrix& A, unsigned* tick, DevMem& mem, DevMem& part,
                cudaStream_t s, Side& side) {
    const size_t nt = sc.tasks.size(), ng = sc.group_begin.size() - 1;
    const size_t bytes = sizeof(Task) * nt +
                         sizeof(int) * (sc.list_idx.size() + sc.light_max.size() + sc.task_group.size() +
                                        sc.group_begin.size() + sc.inst_group_begin.size() +
                                        sc.inst_task_begin.size()) +
                         7 * 16;
    std::vector<char> buf(bytes, 0);
    size_t off = 0;
    auto put = [&](const void* src, size_t n) {
        const size_t at = off;
        if (n) std::memcpy(buf.data() + at, src, n);
        off += (n + 15) & ~(size_t)15;
        return at;
    };
    const size_t o_t = put(sc.tasks.data(), sizeof(Task) * nt);
    const size_t o_h = put(sc.list_idx.data(), sizeof(int) * sc.list_idx.size());
    const size_t o_x = put(sc.light_max.data(), sizeof(int) * sc.light_max.size());
    const size_t o_g = put(sc.task_group.data(), sizeof(int) * sc.task_group.size());
    const size_t o_b = put(sc.group_begin.data(), sizeof(int) * sc.group_begin.size());
    const size_t o_i = put(sc.inst_group_begin.data(), sizeof(int) * sc.inst_group_begin.size());
    const size_t o_s = put(sc.inst_task_begin.data(), sizeof(int) * sc.inst_task_begin.size());
    buf.resize(std::max<size_t>(off, 16));
    SIHG_TRY(upload(mem, buf.data(), buf.size(), s));
    SIHG_TRY(part.alloc(sizeof(float2) * kQ * (std::max<size_t>(1, nt) + std::max<size_t>(1, ng))));
    char* d = mem.as<char>();
    float2* tp = part.as<float2>();
    side = Side{A,
                (const Task*)(d + o_t),
                (int)nt,
                (const int*)(d + o_h),
                (const int*)(d + o_x),
                (const int*)(d + o_g),
                (const int*)(d + o_b),
                (const int*)(d + o_i),
                tp,
                tp + (size_t)kQ * std::max<size_t>(1, nt),
                tick + B + 2,  // group tickets
                tick,          // instance tickets
                tick + B,      // counters
                (const int*)(d + o_s),
                nullptr,
                nullptr};
    return SIH_PDHG_OK;
}

}  // namespace

int TaskLayout::build(const std::vector<int>& csr_ptr, const std::vector<int>& csc_ptr, const std::vector<int>& roff,
                      const std::vector<int>& coff, const SegMatrix& rows_A, const SegMatrix& cols_A, int task_nnz,
                      bool all_active, cudaStream_t s, int row_lanes, int col_lanes, int max_segs) {
    const int B = (int)roff.size() - 1;
    SideSchedule rs, cs;
    make_schedule(csr_ptr, roff, task_nnz, rs, row_lanes, max_segs);
    make_schedule(csc_ptr, coff, task_nnz, cs, col_lanes, max_segs);
    // per side: tickets [B] + counters [2] + group tickets [ngroups], zeroed once;
    // the kernels leave the tickets zero
    const size_t ng_r = rs.group_begin.size() - 1, ng_c = cs.group_begin.size() - 1;
    const size_t nticket = 2 * ((size_t)B + 2) + ng_r + ng_c;
    SIHG_TRY(tickets_.alloc(sizeof(unsigned) * nticket));
    SIHG_CUDA(cudaMemsetAsync(tickets_.as<void>(), 0, sizeof(unsigned) * nticket, s));
    unsigned* tk = tickets_.as<unsigned>();
    SIHG_TRY(upload_side(rs, B, rows_A, tk, row_sched_, row_part_, s, rows));
    SIHG_TRY(upload_side(cs, B, cols_A, tk + B + 2 + ng_r, col_sched_, col_part_, s, cols));
    // element chunks, grouped by instance: columns then rows of each
    std::vector<int4> ch;
    std::vector<int> ch_begin(B + 1, 0);
    for (int b = 0; b < B; ++b) {
        ch_begin[b] = (int)ch.size();
        for (int side = 0; side < 2; ++side) {
            const std::vector<int>& off = side == 0 ? coff : roff;
            for (int e0 = off[b]; e0 < off[b + 1]; e0 += kChunk)
                ch.push_back(make_int4(e0, std::min(off[b + 1], e0 + kChunk), b, side == 0 ? 1 : 0));
        }
    }
    ch_begin[B] = (int)ch.size();
    const size_t nch = ch.size();
    std::vector<char> buf(sizeof(int4) * std::max<size_t>(1, nch) + sizeof(int) * (B + 1), 0);
    std::memcpy(buf.data(), ch.data(), sizeof(int4) * nch);
    std::memcpy(buf.data() + sizeof(int4) * std::max<size_t>(1, nch), ch_begin.data(), sizeof(int) * (B + 1));
    SIHG_TRY(upload(chunks_, buf.data(), buf.size(), s));
    // active lists: row tasks, column tasks, chunks; 3 counts; 3 x B offsets
    const size_t nr = rows.ntasks, nc = cols.ntasks;
    const size_t nact = nr + nc + nch + 3 + 3 * (size_t)B + 8;
    if (all_active) {
        std::vector<int> a(nact, 0);
        for (size_t k = 0; k < nr; ++k) a[k] = (int)k;
        for (size_t k = 0; k < nc; ++k) a[nr + k] = (int)k;
        for (size_t k = 0; k < nch; ++k) a[nr + nc + k] = (int)k;
        a[nr + nc + nch] = (int)nr;
        a[nr + nc + nch + 1] = (int)nc;
        a[nr + nc + nch + 2] = (int)nch;
        SIHG_TRY(upload(active_, a.data(), sizeof(int) * nact, s));
    } else {
        SIHG_TRY(active_.alloc(sizeof(int) * nact));
    }
    int* a = active_.as<int>();
    rows.active = a;
    cols.active = a + nr;
    int* cnt = a + nr + nc + nch;
    rows.nactive = cnt;
    cols.nactive = cnt + 1;
    chunks = Chunks{chunks_.as<int4>(), (int)nch,
                    (const int*)(chunks_.as<char>() + sizeof(int4) * std::max<size_t>(1, nch)), a + nr + nc, cnt + 2};
    return SIH_PDHG_OK;
}

}  // namespace sihg
