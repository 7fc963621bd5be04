// Types shared by the SU(2) flow translation units: the per-flow kernel argument block and
// the launch interface of the vertex-flow kernel.
#pragma once
#include <cuda_runtime.h>

namespace spn {

constexpr unsigned kStatusNaN = 1u;           // a NaN was written into the flow
constexpr unsigned kStatusNodeOverflow = 2u;  // a loop-frequency node table overflowed

// Lane-balanced RPA schedule: the RPA pair lists of all rids, merged into distinct
// (rid1, rid2) pairs with their multiplicity, sorted by output rid, and cut into `lanes`
// contiguous chunks.  Entry i of lane l is sched[i * lanes + l]:
//   bits 0-6 rid1, bits 7-13 rid2, bits 14-21 multiplicity, bit 22 "last pair of a segment".
// A segment is a run of pairs of one output rid inside one chunk; its partial sum goes to the
// next slot of the lane (slot_base[l], slot_base[l]+1, ...), and rid r sums the slots
// seg_ptr[r] .. seg_ptr[r+1]-1 in order.
struct RpaSchedule {
    const int *sched;
    const int *count;      // [lanes] entries of each lane
    const int *slot_base;  // [lanes]
    const int *seg_ptr;    // [Nl + 1]
    int lanes, n_seg;
    int len;       // entries per lane (sched holds len * lanes ints)
    int in_smem;   // the kernel stages the schedule in shared memory
};

// Shared-memory words of a staged schedule (sched, count, slot_base, seg_ptr).
__host__ __device__ inline int rpa_smem_ints(const RpaSchedule &r, int nl) {
    return r.len * r.lanes + 2 * r.lanes + nl + 1;
}

struct FlowArgs {
    int n, nl, fn, wsite, max_nodes, n_range;
    float cutoff, spin;
    const float *freq;
    const float *ss, *dd;  // state
    float *dss, *ddd;      // flow
    const float *v2;       // self-energy state
    float *dv2;            // self-energy flow
    const double *v2d;     // FP64 self-energy state (used when fp64_sigma)
    double *dv2d;          // FP64 self-energy flow
    int fp64_sigma;
    const int *sites, *inv_sites, *ov_ptr, *ov_r1, *ov_r2, *range_rid, *range_inv;
    float *node_wp, *node_c;
    int *node_cnt;
    int *work_counter;
    unsigned *status;
    RpaSchedule rpa;
};

// Vertex-flow kernel (su2_vertex.cu): dynamic shared memory per block, the number of blocks
// per SM it achieves, and the launch.
// `npi`: loop-frequency nodes a site group evaluates per iteration (1 or 2); whether the RPA
// schedule is staged in shared memory is a.rpa.in_smem.  Both are chosen per flow by timing.
size_t vertex_flow_smem_bytes(int nl, const RpaSchedule &rpa, int npi);
int vertex_flow_blocks_per_sm(int nl, const RpaSchedule &rpa, int npi);
void launch_vertex_flow(const FlowArgs &a, int npi, int grid, cudaStream_t stream);

// Largest schedule staged in shared memory; larger ones are read from global memory.
constexpr int kRpaSmemMaxInts = 8192;

}  // namespace spn
