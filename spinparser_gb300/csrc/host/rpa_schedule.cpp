// RPA schedule builder (see rpa_schedule.hpp).
#include "rpa_schedule.hpp"
#include "error.hpp"
#include <algorithm>

namespace spn {

namespace {

struct Pair {
    int rid, a, b, m;
};

}  // namespace

RpaHostSchedule build_rpa_schedule(int nl, const int *ptr, const int *r1, const int *r2, int lanes) {
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

    s.packed = nl <= 32;
    s.width = s.packed ? rpa_outer_width(nl) : 0;

    // Order the entries inside each segment against shared-memory bank collisions: the walk
    // reads the float2 element M[rid1][rid2], and a 64-bit read is served per half warp, 16
    // lanes in one wavefront when they hit 16 distinct bank pairs.  Step by step, each lane of a
    // half warp takes from the rest of its current segment the first entry whose bank pair
    // ((rid1 * row + rid2) mod 16; the row width is a multiple of 16 above 32 sites) no lower
    // lane of the half warp took at that step (else one whose bank pair the fewest took).  A
    // segment's sum is the same set of terms in another order.
    auto bank = [&](const Pair &p) { return int(unsigned(s.packed ? p.a * s.width + p.b : p.b) & 15u); };
    for (int h0 = 0; h0 < lanes; h0 += 16) {
        const int h1 = std::min(lanes, h0 + 16);
        std::vector<size_t> si(size_t(h1 - h0), 0);
        for (int i = 0; i < L; ++i) {
            int taken[16] = {0};
            for (int l = h0; l < h1; ++l) {
                if (i >= s.count[l]) continue;
                size_t &k = si[size_t(l - h0)];
                if (i == seg_end[l][k]) ++k;  // position i opens the lane's next segment
                const int end = seg_end[l][k];
                auto &o = order[l];
                int pick = i;
                for (int j = i; j < end && taken[bank(o[size_t(pick)])] > 0; ++j)
                    if (taken[bank(o[size_t(j)])] < taken[bank(o[size_t(pick)])]) pick = j;
                std::swap(o[size_t(i)], o[size_t(pick)]);
                ++taken[bank(o[size_t(i)])];
            }
        }
    }

    for (int l = 0; l < lanes; ++l) {
        size_t si = 0;
        for (int i = 0; i < s.count[l]; ++i) {
            const Pair &p = order[l][i];
            const bool last = (i + 1 == seg_end[l][si]);
            if (last) ++si;
            s.sched[size_t(i) * lanes + l] =
                s.packed ? int(unsigned(p.a * s.width + p.b) * 8u | unsigned(p.m) << 16 | (last ? 0x80000000u : 0u))
                         : p.a | (p.b << 7) | (p.m << 14) | (last ? (1 << 22) : 0);
        }
    }
    return s;
}

int xyz_walk_addr(int e, int k, int nl) {
    return k == 0 ? ((e >> 14) & 7) * nl + (e & 127) : ((e >> 17) & 7) * nl + ((e >> 7) & 127);
}

int tri_walk_addr(int e, int k, int nl) {
    const int f = k >> 4, a = (k >> 2) & 3, b = k & 3;
    const int rid = f ? (e >> 7) & 127 : e & 127, sh = f ? 20 : 14;
    const int pa = a == 3 ? 3 : (e >> (sh + 2 * a)) & 3, pb = b == 3 ? 3 : (e >> (sh + 2 * b)) & 3;
    return (4 * pa + pb) * nl + rid;
}

LaneSchedule xyz_lane_schedule(int nl, const int *ptr, const std::vector<int> &packed) {
    return lane_schedule(nl, ptr, packed, 32, 20, 2, 8, 8, xyz_walk_addr);
}

LaneSchedule tri_lane_schedule(int nl, const int *ptr, const std::vector<int> &packed) {
    return lane_schedule(nl, ptr, packed, 32, 26, 32, 32, 32, tri_walk_addr);
}

LaneSchedule lane_schedule(int nl, const int *ptr, const std::vector<int> &packed, int lanes, int last_bit, int reads,
                           int banks, int group, int (*addr)(int word, int k, int nl)) {
    const int P = int(packed.size());
    const int L = std::max(1, (P + lanes - 1) / lanes);
    LaneSchedule r;
    r.len = L;
    r.sched.assign(size_t(L) * lanes, 0);
    r.count.assign(size_t(lanes), 0);
    r.slot_base.assign(size_t(lanes), 0);
    r.seg_ptr.assign(size_t(nl) + 1, -1);
    std::vector<int> owner(static_cast<size_t>(P));  // the site of each pair
    for (int j = 0; j < nl; ++j)
        for (int i = ptr[j]; i < ptr[j + 1]; ++i) owner[size_t(i)] = j;
    std::vector<std::vector<int>> words(static_cast<size_t>(lanes)), ends(static_cast<size_t>(lanes));
    int seg = -1;
    for (int l = 0; l < lanes; ++l) {
        const int b0 = l * L, b1 = std::min(P, (l + 1) * L);
        r.count[size_t(l)] = std::max(0, b1 - b0);
        r.slot_base[size_t(l)] = seg + 1;
        for (int i = b0; i < b1; ++i) {
            if (i == b0 || owner[size_t(i - 1)] != owner[size_t(i)]) {
                ++seg;
                if (r.seg_ptr[size_t(owner[size_t(i)])] < 0) r.seg_ptr[size_t(owner[size_t(i)])] = seg;
            }
            words[size_t(l)].push_back(packed[size_t(i)]);
            if (i + 1 == b1 || owner[size_t(i + 1)] != owner[size_t(i)]) ends[size_t(l)].push_back(i + 1 - b0);
        }
    }
    r.n_seg = seg + 1;
    r.seg_ptr[size_t(nl)] = r.n_seg;
    for (int j = nl - 1; j >= 0; --j)
        if (r.seg_ptr[size_t(j)] < 0) r.seg_ptr[size_t(j)] = r.seg_ptr[size_t(j + 1)];
    if (reads > 0 && addr && group > 0 && banks > 0) {
        // per (read, bank): the distinct addresses lower lanes of the group read at this step (a
        // repeated address is a broadcast, a new one in an occupied bank one more wavefront)
        std::vector<std::vector<int>> taken(size_t(reads) * banks);
        auto cost_of = [&](int word) {
            int c = 0;
            for (int x = 0; x < reads; ++x) {
                const int a = addr(word, x, nl);
                const auto &t = taken[size_t(x) * banks + size_t(a & (banks - 1))];
                if (std::find(t.begin(), t.end(), a) == t.end()) c += int(t.size());
            }
            return c;
        };
        for (int g0 = 0; g0 < lanes; g0 += group) {
            const int g1 = std::min(lanes, g0 + group);
            std::vector<size_t> si(size_t(g1 - g0), 0);
            for (int i = 0; i < L; ++i) {
                for (auto &t : taken) t.clear();
                for (int l = g0; l < g1; ++l) {
                    if (i >= r.count[size_t(l)]) continue;
                    size_t &k = si[size_t(l - g0)];
                    if (i == ends[size_t(l)][k]) ++k;  // position i opens the lane's next segment
                    auto &w = words[size_t(l)];
                    int pick = i, best = 1 << 30;
                    for (int q = i; q < ends[size_t(l)][k] && best > 0; ++q) {
                        const int cost = cost_of(w[size_t(q)]);
                        if (cost < best) {
                            best = cost;
                            pick = q;
                        }
                    }
                    std::swap(w[size_t(i)], w[size_t(pick)]);
                    for (int x = 0; x < reads; ++x) {
                        const int a = addr(w[size_t(i)], x, nl);
                        auto &t = taken[size_t(x) * banks + size_t(a & (banks - 1))];
                        if (std::find(t.begin(), t.end(), a) == t.end()) t.push_back(a);
                    }
                }
            }
        }
    }
    for (int l = 0; l < lanes; ++l) {
        size_t k = 0;
        for (int i = 0; i < r.count[size_t(l)]; ++i) {
            const bool last = i + 1 == ends[size_t(l)][k];
            if (last) ++k;
            r.sched[size_t(i) * lanes + l] = words[size_t(l)][size_t(i)] | (last ? 1 << last_bit : 0);
        }
    }
    return r;
}

}  // namespace spn
