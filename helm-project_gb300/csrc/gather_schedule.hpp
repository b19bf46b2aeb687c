// Gather schedule of a warp for the blocked split-FP32 layout (host code,
// no CUDA: staged.cu builds the layout with it, and a CPU test compiles it
// alone).
//
// At step k of a warp each of its 32 lanes reads one staged float (entry k
// of its row in the schedule, or a padding read) in one shared-memory load;
// lanes reading different addresses of one bank serialise, so a step costs
// as many wavefronts as the most distinct addresses a bank holds. The
// schedule is built step by step as a bipartite matching of lanes to banks:
// lanes with no slack (as many entries left as steps) first, then by
// increasing slack; each lane is placed on an address already chosen this
// step, else on the free bank with the most unplaced addresses (the hardest
// to spread over the remaining steps), else by moving the single lane of a
// bank to another of its entries (augmenting path). A lane with slack that
// cannot be placed without a conflict reads padding this step, as do lanes
// whose rows are done; padding reads the zero run [zero, zero + zrun) at its
// least used bank. A lane with no slack left takes the entry that costs the
// fewest extra wavefronts.
#pragma once

#include <algorithm>
#include <vector>

namespace axgb {

struct WarpSchedule {
    struct Cand {
        int e;     // caller's entry index (a CSR index)
        int addr;  // staging index
    };
    std::vector<Cand> cand[32];  // per lane: the entries not yet placed (the caller fills these)
    std::vector<int> placed[32];  // per lane: entries in the order scheduled (output)
    int choice[32];              // index into cand for this step, -1: none
    int bank_addr[32], bank_users[32], bank_lane[32];
    int press[32];               // distinct unplaced addresses per bank
    std::vector<int> extra[32];  // further addresses of a bank this step (conflicts)
    std::vector<int> left;       // unplaced entries per staging address

    void commit(int l, int ci) {
        const int a = cand[l][ci].addr, b = a & 31;
        if (bank_addr[b] == a) {
            ++bank_users[b];
        } else {
            bank_addr[b] = a;
            bank_users[b] = 1;
            bank_lane[b] = l;
        }
        choice[l] = ci;
    }
    void uncommit(int l) {
        const int b = cand[l][choice[l]].addr & 31;
        if (--bank_users[b] == 0) bank_addr[b] = -1;
        choice[l] = -1;
    }
    // Places lane l on one of its entries without a second address in any
    // bank (seen: banks already on the augmenting path); false if it cannot.
    bool place(int l, unsigned &seen) {
        const auto &c = cand[l];
        const int n = static_cast<int>(c.size());
        for (int i = 0; i < n; ++i)
            if (bank_addr[c[i].addr & 31] == c[i].addr) {
                commit(l, i);
                return true;
            }
        int best = -1, bp = -1;
        for (int i = 0; i < n; ++i) {
            const int b = c[i].addr & 31;
            if (bank_addr[b] < 0 && press[b] > bp) {
                bp = press[b];
                best = i;
            }
        }
        if (best >= 0) {
            commit(l, best);
            return true;
        }
        for (int i = 0; i < n; ++i) {
            const int b = c[i].addr & 31;
            if (seen & (1u << b)) continue;
            seen |= 1u << b;
            if (bank_users[b] != 1) continue;
            const int l2 = bank_lane[b], c2 = choice[l2];
            uncommit(l2);
            commit(l, i);
            if (place(l2, seen)) return true;
            uncommit(l);
            commit(l2, c2);
        }
        return false;
    }

    // Schedules the entries in cand[] over W steps (W at least the longest
    // lane's count). Appends, step-major, each lane's staging index to q_out
    // and its entry (or -1 for padding) to e_out; fills placed[]. Addresses
    // must be below zero + zrun. Returns false if an entry was left unplaced.
    bool run(int W, int zero, int zrun, std::vector<int> &q_out, std::vector<int> &e_out) {
        if (static_cast<int>(left.size()) < zero + zrun) left.assign(zero + zrun, 0);
        for (int lane = 0; lane < 32; ++lane) placed[lane].clear();
        for (int b = 0; b < 32; ++b) press[b] = 0;
        for (int lane = 0; lane < 32; ++lane)
            for (auto &c : cand[lane])
                if (left[c.addr]++ == 0) ++press[c.addr & 31];
        for (int k = 0; k < W; ++k) {
            const int rounds = W - k;
            for (int b = 0; b < 32; ++b) {
                bank_addr[b] = -1;
                bank_users[b] = 0;
                extra[b].clear();
            }
            for (int lane = 0; lane < 32; ++lane) choice[lane] = -1;
            int order[32], no = 0;
            for (int lane = 0; lane < 32; ++lane)
                if (!cand[lane].empty()) order[no++] = lane;
            std::stable_sort(order, order + no, [&](int a, int b) {
                const int sa = rounds - static_cast<int>(cand[a].size());
                const int sb = rounds - static_cast<int>(cand[b].size());
                if (sa != sb) return sa < sb;
                return cand[a].size() > cand[b].size();
            });
            for (int i = 0; i < no; ++i) {
                unsigned seen = 0;
                place(order[i], seen);
            }
            // lanes left without a conflict-free entry: those with no slack
            // take the entry costing the fewest extra wavefronts
            for (int i = 0; i < no; ++i) {
                const int l = order[i];
                if (choice[l] >= 0 || static_cast<int>(cand[l].size()) < rounds) continue;
                int best = 0, bc = 1 << 30;
                for (int j = 0; j < static_cast<int>(cand[l].size()); ++j) {
                    const int a = cand[l][j].addr, b = a & 31;
                    int cost;
                    if (bank_addr[b] == a || std::find(extra[b].begin(), extra[b].end(), a) != extra[b].end())
                        cost = 0;
                    else
                        cost = (bank_addr[b] >= 0 ? 1 : 0) + static_cast<int>(extra[b].size());
                    if (cost < bc) {
                        bc = cost;
                        best = j;
                    }
                }
                const int a = cand[l][best].addr, b = a & 31;
                if (bank_addr[b] < 0) {
                    commit(l, best);
                } else {
                    if (bank_addr[b] != a && std::find(extra[b].begin(), extra[b].end(), a) == extra[b].end())
                        extra[b].push_back(a);
                    choice[l] = best;
                }
            }
            // padding: one address for all padding lanes, in the least used
            // bank the zero run covers
            int pad = zero, pc = 1 << 30;
            for (int i = 0; i < zrun; ++i) {
                const int b = (zero + i) & 31;
                const int c = (bank_addr[b] >= 0 ? 1 : 0) + static_cast<int>(extra[b].size());
                if (c < pc) {
                    pc = c;
                    pad = zero + i;
                }
            }
            for (int lane = 0; lane < 32; ++lane) {
                const int ci = choice[lane];
                if (ci < 0) {
                    q_out.push_back(pad);
                    e_out.push_back(-1);
                    continue;
                }
                auto &c = cand[lane];
                q_out.push_back(c[ci].addr);
                e_out.push_back(c[ci].e);
                placed[lane].push_back(c[ci].e);
                if (--left[c[ci].addr] == 0) --press[c[ci].addr & 31];
                c.erase(c.begin() + ci);
            }
        }
        bool ok = true;
        for (int lane = 0; lane < 32; ++lane) ok = ok && cand[lane].empty();
        return ok;
    }
};

}  // namespace axgb
