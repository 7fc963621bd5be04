// RPA schedule builder (see rpa_schedule.hpp).
#include "rpa_schedule.hpp"
#include "error.hpp"
#include <algorithm>
#include <cstring>
#include <numeric>

namespace spn {

namespace {

struct Pair {
    int rid, a, b, m;
};

// IEEE binary16 bits of an integer 1 <= m <= 255 (exact).
int half_bits(int m) {
    int e = 0;
    while ((m >> (e + 1)) != 0) ++e;
    const int mant = ((m << 10) >> e) & 0x3ff;
    return ((e + 15) << 10) | mant;
}

}  // namespace

RpaHostSchedule build_rpa_schedule(int nl, const int *ptr, const int *r1, const int *r2, int lanes, bool products) {
    if (products && nl > 32) throw Error(ErrorType::Internal, "product-encoded RPA schedule needs Nl <= 32");
    // distinct (rid, rid1, rid2) with multiplicity, in rid order
    std::vector<Pair> pairs;
    std::vector<int> mult(size_t(nl) * nl);
    for (int r = 0; r < nl; ++r) {
        std::fill(mult.begin(), mult.end(), 0);
        for (int i = ptr[r]; i < ptr[r + 1]; ++i) ++mult[size_t(r1[i]) * nl + r2[i]];
        for (int a = 0; a < nl; ++a)
            for (int b = 0; b < nl; ++b) {
                const int m = mult[size_t(a) * nl + b];
                if (!m) continue;
                if (m > 255) throw Error(ErrorType::Unsupported, "RPA pair multiplicity above 255");
                pairs.push_back({r, a, b, m});
            }
    }
    RpaHostSchedule s;
    s.lanes = lanes;
    const int P = int(pairs.size());
    const int L = std::max(1, (P + lanes - 1) / lanes);
    s.len = L;
    s.sched.assign(size_t(L) * lanes, 0);
    s.count.assign(lanes, 0);
    s.slot_base.assign(lanes, 0);
    s.seg_ptr.assign(nl + 1, -1);

    // chunks, segments and the order of the pairs inside each lane
    std::vector<std::vector<Pair>> order(lanes);
    std::vector<std::vector<int>> seg_end(lanes);  // end position (exclusive) of each segment of a lane
    int seg = -1;
    for (int l = 0; l < lanes; ++l) {
        const int b0 = l * L, b1 = std::min(P, (l + 1) * L);
        s.count[l] = std::max(0, b1 - b0);
        s.slot_base[l] = seg + 1;
        for (int i = b0; i < b1; ++i) {
            const Pair &p = pairs[i];
            if (i == b0 || pairs[i - 1].rid != p.rid) {
                ++seg;
                if (s.seg_ptr[p.rid] < 0) s.seg_ptr[p.rid] = seg;
            }
            if (i + 1 == b1 || pairs[i + 1].rid != p.rid) seg_end[l].push_back(i + 1 - b0);
            order[l].push_back(p);
        }
    }
    s.n_seg = seg + 1;
    s.seg_ptr[nl] = s.n_seg;
    for (int r = nl - 1; r >= 0; --r)
        if (s.seg_ptr[r] < 0) s.seg_ptr[r] = s.seg_ptr[r + 1];

    if (nl <= 32) {
        // Reorder inside segments: at step i the lanes that share a half-warp should read
        // P[ab] at distinct banks.  A lane group of `lanes` lanes fills min(lanes, 16) lanes of
        // a half-warp; its reads are conflict-free when the ab of those lanes differ modulo
        // that width (the kernel spaces the groups of a half-warp accordingly).
        const int hw = std::min(lanes, 16);
        std::vector<std::vector<Pair>> placed(lanes);
        std::vector<size_t> seg_idx(lanes, 0);
        std::vector<std::vector<Pair>> pool(lanes);
        std::vector<int> seg_start(lanes, 0);
        auto refill = [&](int l) {
            const int e = seg_end[l][seg_idx[l]];
            pool[l].assign(order[l].begin() + seg_start[l], order[l].begin() + e);
        };
        for (int l = 0; l < lanes; ++l)
            if (s.count[l] > 0) refill(l);
        std::vector<int> used(hw);
        std::vector<int> lane_order(hw);
        for (int i = 0; i < L; ++i) {
            for (int h0 = 0; h0 < lanes; h0 += hw) {
                std::fill(used.begin(), used.end(), 0);
                std::iota(lane_order.begin(), lane_order.end(), h0);
                // lanes with the fewest choices pick first
                std::stable_sort(lane_order.begin(), lane_order.end(),
                                 [&](int x, int y) { return pool[x].size() < pool[y].size(); });
                for (int l : lane_order) {
                    if (i >= s.count[l]) continue;
                    size_t best = 0;
                    int best_use = 1 << 30;
                    for (size_t k = 0; k < pool[l].size(); ++k) {
                        const int key = (pool[l][k].a * nl + pool[l][k].b) % hw;
                        if (used[key] < best_use) {
                            best_use = used[key];
                            best = k;
                            if (best_use == 0) break;
                        }
                    }
                    const Pair p = pool[l][best];
                    pool[l].erase(pool[l].begin() + best);
                    ++used[(p.a * nl + p.b) % hw];
                    placed[l].push_back(p);
                    if (pool[l].empty() && i + 1 < s.count[l]) {
                        seg_start[l] = seg_end[l][seg_idx[l]];
                        ++seg_idx[l];
                        refill(l);
                    }
                }
            }
        }
        order.swap(placed);
    }

    for (int l = 0; l < lanes; ++l) {
        size_t si = 0;
        for (int i = 0; i < s.count[l]; ++i) {
            const Pair &p = order[l][i];
            const bool last = (i + 1 == seg_end[l][si]);
            if (last) ++si;
            const size_t at = size_t(i) * lanes + l;
            if (products) {
                s.sched[at] = (p.a * nl + p.b) | (last ? (1 << 15) : 0) | int(unsigned(half_bits(p.m)) << 16);
            } else {
                s.sched[at] = p.a | (p.b << 7) | (p.m << 14) | (last ? (1 << 22) : 0);
            }
        }
    }
    return s;
}

}  // namespace spn
