// Lane-balanced schedule of the RPA lattice sum (SU2FrgCore.cpp:249-266):
//   out[rid] = sum over the pairs i of getOverlap(rid) of A[rid1_i] * B[rid2_i]
// for all rids at once, evaluated by `lanes` lanes of a warp.  The pair lists of all rids are
// merged into distinct (rid, rid1, rid2) triples with a multiplicity, sorted by rid, and cut
// into `lanes` contiguous chunks of equal length; a run of one rid inside a chunk is a
// segment, whose partial sum goes to the lane's next slot (slot_base[l], +1, ...); rid r sums
// the slots seg_ptr[r] .. seg_ptr[r+1]-1 in order.  Entry i of lane l is sched[i * lanes + l].
// The kernel accumulates acc += (A[rid1] * m) * B[rid2] for spin and density.  Entries:
//   Nl <= 32 ("packed"): off1 | off2 << 8 | m << 16 | last << 31 with byte offsets of the
//            exchanged values -- 8 rid (interleaved (spin, density) float2 arrays) for Nl <= 16,
//            where every element has its own 8-byte bank pair, and 4 rid (separate 32-bit
//            arrays, conflict-free) for 16 < Nl <= 32;
//   Nl > 32: rid1 | rid2 << 7 | m << 14 | last << 22.
#pragma once
#include <vector>

namespace spn {

struct RpaHostSchedule {
    std::vector<int> sched, count, slot_base, seg_ptr;
    int lanes = 0, n_seg = 0, len = 0;
    bool packed = false;
};

RpaHostSchedule build_rpa_schedule(int nl, const int *ptr, const int *r1, const int *r2, int lanes);

}  // namespace spn
