// Lane-balanced schedule of the RPA lattice sum (SU2FrgCore.cpp:249-266):
//   out[rid] = sum over the pairs i of getOverlap(rid) of A[rid1_i] * B[rid2_i]
// for all rids at once, evaluated by `lanes` lanes of a warp.  The pair lists of all rids are
// merged into distinct (rid, rid1, rid2) triples with a multiplicity, sorted by rid, and cut
// into `lanes` contiguous chunks of equal length; a run of one rid inside a chunk is a
// segment, whose partial sum goes to the lane's next slot (slot_base[l], +1, ...); rid r sums
// the slots seg_ptr[r] .. seg_ptr[r+1]-1 in order.  Entry i of lane l is sched[i * lanes + l].
// Entries:
//   Nl <= 32 ("packed", outer-product form): off | m << 16 | last << 31, off = the byte offset
//            (rid1 * W + rid2) * 8 of the (spin, density) float2 element M[rid1][rid2] of a
//            row-major W x W matrix, W = rpa_outer_width(Nl).  The kernel accumulates
//            M = sum over nodes of (c A) x B first and walks the schedule once per triple:
//            acc += m * M[rid1][rid2];
//   Nl > 32: rid1 | rid2 << 7 | m << 14 | last << 22; the kernel accumulates
//            acc += (A[rid1] * m) * B[rid2] per node.
#pragma once
#include <vector>

#ifdef __CUDACC__
#define SPN_HD __host__ __device__
#else
#define SPN_HD
#endif

namespace spn {

// Row width of the outer-product RPA matrix of a lattice with nl <= 32 sites: 8 x the rows of
// M one lane accumulates (the warp's 32 lanes form an 8 x 4 grid of blocks of w/8 x w/4).
SPN_HD inline int rpa_outer_width(int nl) { return nl <= 8 ? 8 : (nl <= 16 ? 16 : (nl <= 24 ? 24 : 32)); }

struct RpaHostSchedule {
    std::vector<int> sched, count, slot_base, seg_ptr;
    int lanes = 0, n_seg = 0, len = 0;
    int width = 0;  // outer-product matrix row width (packed form)
    bool packed = false;
};

RpaHostSchedule build_rpa_schedule(int nl, const int *ptr, const int *r1, const int *r2, int lanes);

// Lane-balanced walk over per-site RPA pair lists (the XYZ and TRI t channels, where a pair
// carries spin permutations and pairs are not merged): the packed pair words in site order
// (site j's at ptr[j] .. ptr[j+1]) cut into `lanes` chunks of equal length; a run of one site in
// a chunk is a segment.  Entry i of lane l is sched[i * lanes + l], the word with bit `last_bit`
// set on a segment's last entry; a segment's partial goes to slot slot_base[l], +1, ...; site j
// sums slots seg_ptr[j] .. seg_ptr[j+1] - 1 in order.  With `reads` > 0 the entries inside each
// segment are ordered against shared-memory bank collisions: addr(word, k) is the word address
// (in bank-width units) of the pair's k-th read, its bank addr mod `banks` (a power of two),
// `group` lanes are served together, and step by step each lane takes the entry of its segment
// whose reads add the fewest new addresses to banks that lower lanes of its group already read.
struct LaneSchedule {
    std::vector<int> sched, count, slot_base, seg_ptr;
    int n_seg = 0, len = 0;
};
LaneSchedule lane_schedule(int nl, const int *ptr, const std::vector<int> &packed, int lanes, int last_bit,
                           int reads = 0, int banks = 0, int group = 0, int (*addr)(int word, int k, int nl) = nullptr);

// The shared-memory reads of the two walks.  XYZ (word rid1 | rid2 << 7 | perm1 << 14 | perm2 << 17,
// last-entry bit 20): the two 16-byte reads A6[perm1 nl + rid1] and B6[perm2 nl + rid2], eight
// bank positions, eight lanes per phase.  TRI (word rid1 | rid2 << 7 | the images of X, Y, Z under
// perm1, 2 bits each, << 14 | the same for perm2 << 20, last-entry bit 26): reads 0..15 take
// component (P1(a), P1(b)) of the first factor at (4 P1(a) + P1(b)) nl + rid1, reads 16..31 the
// same for the second factor; 4-byte words, 32 banks, one 32-lane phase.
int xyz_walk_addr(int word, int k, int nl);
int tri_walk_addr(int word, int k, int nl);
LaneSchedule xyz_lane_schedule(int nl, const int *ptr, const std::vector<int> &packed);
LaneSchedule tri_lane_schedule(int nl, const int *ptr, const std::vector<int> &packed);

}  // namespace spn
