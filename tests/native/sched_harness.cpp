// Test harness: the blocked layout's gather schedule (gather_schedule.hpp)
// through a C entry point, compiled by tests/test_cpu_gather_schedule.py.
#include <vector>

#include "gather_schedule.hpp"

extern "C" {

// n_of[32]: entries per lane; addr: their staging addresses, lane after lane.
// W steps, zero run [zero, zero + zrun). q_out[W*32]: staging index read at
// (step, lane); e_out[W*32]: the entry (index into addr) or -1 for padding.
// Returns 1 when every entry was placed.
int sched_warp(const int *n_of, const int *addr, int W, int zero, int zrun, int *q_out, int *e_out) {
    static thread_local axgb::WarpSchedule S;
    int base = 0;
    for (int lane = 0; lane < 32; ++lane) {
        S.cand[lane].clear();
        for (int j = 0; j < n_of[lane]; ++j) S.cand[lane].push_back({base + j, addr[base + j]});
        base += n_of[lane];
    }
    S.left.assign(zero + zrun, 0);
    std::vector<int> q, e;
    const bool ok = S.run(W, zero, zrun, q, e);
    for (size_t i = 0; i < q.size() && i < static_cast<size_t>(W) * 32; ++i) {
        q_out[i] = q[i];
        e_out[i] = e[i];
    }
    return ok ? 1 : 0;
}

}
