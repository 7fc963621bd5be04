// Order of the RPA overlap pairs of each site, chosen against shared-memory bank collisions.
//
// A walk of the RPA pairs of site j in lane j of a warp (32 sites per warp step): at step k every
// lane reads, for each of `slots` load instructions, one word of its k-th pair; lanes of one
// phase (all 32 for 4-byte reads, 8 for 16-byte reads) whose different words fall into the same
// bank serialise.  Any order of a site's pairs gives the same RPA sum up to rounding, so the
// pairs are chosen greedily, step by step and site by site, with the fewest new collisions.  The
// XYZ and TRI vertex kernels walk the site-ordered lists in lane-balanced chunks instead
// (lane_schedule, rpa_schedule.hpp), which orders the entries of each run again for that walk.
#pragma once

#include <functional>
#include <vector>

namespace spn {

struct PairBankModel {
    int slots;        // load instructions per pair
    int phase_lanes;  // lanes served together: 32 (4-byte words) or 8 (16-byte words)
    int banks;        // distinct bank positions of a word: 32 / (word bytes / 4)
};

// words(i, w) writes the `slots` word addresses (in word units) pair i reads.  Returns the
// pair indices in the new order: out[ptr[j] .. ptr[j+1]) is a permutation of site j's pairs.
std::vector<int> order_pairs_by_banks(int n_sites, const int *ptr, const PairBankModel &m,
                                      const std::function<void(int, int *)> &words);

// The RPA reads of the XYZ kernel: A6[perm1 nl + rid1] and B6[6 nl + perm2 nl + rid2], one
// float4 each (two slots, eight-lane phases, eight bank positions).
PairBankModel xyz_rpa_model();
std::function<void(int, int *)> xyz_rpa_words(int nl, const int *rid1, const int *rid2, const int *perm1,
                                              const int *perm2);
// The RPA reads of the TRI kernel: the 16 permuted components (4 P(a) + P(b)) nl + rid of both
// factors, 4-byte words (32 slots, one 32-lane phase, 32 banks).  P is the spin permutation of
// spn_lattice_get_spin_tables; the density index stays.
PairBankModel tri_rpa_model();
std::function<void(int, int *)> tri_rpa_words(int nl, const int *rid1, const int *rid2, const int *perm1,
                                              const int *perm2);

// Collisions of an order under the same model (sum over steps, slots and phases of the extra
// distinct words per bank): the figure the greedy choice lowers.
long long pair_bank_collisions(int n_sites, const int *ptr, const int *order, const PairBankModel &m,
                               const std::function<void(int, int *)> &words);

}  // namespace spn
