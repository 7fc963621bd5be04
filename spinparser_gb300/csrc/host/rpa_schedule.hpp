// Lane-balanced schedule of the RPA lattice sum (SU2FrgCore.cpp:249-266):
//   out[rid] = sum over the pairs i of getOverlap(rid) of A[rid1_i] * B[rid2_i]
// for all rids at once, evaluated by `lanes` lanes of a warp.  The pair lists of all rids are
// merged into distinct (rid, rid1, rid2) triples with a multiplicity, sorted by rid, and cut
// into `lanes` contiguous chunks of equal length; a run of one rid inside a chunk is a
// segment, whose partial sum goes to the lane's next slot (slot_base[l], +1, ...); rid r sums
// the slots seg_ptr[r] .. seg_ptr[r+1]-1 in order.  Entry i of lane l is sched[i * lanes + l].
// Either way the kernel accumulates acc += m * (A[rid1] * B[rid2]) in the same order, so the
// two encodings give the same bits.
//
// Two encodings:
//   factors:  rid1 | rid2 << 7 | m << 14 | last << 22 -- the kernel reads A[rid1] and B[rid2]
//             (any Nl <= 128);
//   products: rid1 * Nl + rid2 | last << 15 | fp16(m) << 16 -- the kernel first forms the
//             products P[rid1 * Nl + rid2] = A[rid1] * B[rid2] of both channels as float2 and
//             then reads P[ab] (Nl <= 32).
// For Nl <= 32 the pairs of each segment are ordered so that at every step the lanes of a
// half-warp read P at different banks where possible (the same order serves both encodings).
#pragma once
#include <vector>

namespace spn {

struct RpaHostSchedule {
    std::vector<int> sched, count, slot_base, seg_ptr;
    int lanes = 0, n_seg = 0, len = 0;
};

RpaHostSchedule build_rpa_schedule(int nl, const int *ptr, const int *r1, const int *r2, int lanes, bool products);

}  // namespace spn
