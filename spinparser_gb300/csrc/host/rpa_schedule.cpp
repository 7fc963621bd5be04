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

}  // namespace spn
