// Types shared by the SU(2) flow translation units: the per-flow kernel argument block and
// the launch interface of the vertex-flow kernel.
#pragma once
#include <cuda_runtime.h>
#include "host/rpa_schedule.hpp"
#include "su2_device.cuh"

namespace spn {

constexpr unsigned kStatusNaN = 1u;           // a NaN was written into the flow
constexpr unsigned kStatusNodeOverflow = 2u;  // a loop-frequency node table overflowed
constexpr unsigned kStatusStageTimeout = 4u;  // a bulk copy to shared memory did not complete in
                                              // time; the kernel read global memory instead

// Lane-balanced RPA schedule (built by host/rpa_schedule.cpp): the RPA pair lists of all
// rids merged into distinct (rid, rid1, rid2) with their multiplicity, sorted by rid and cut
// into `lanes` (32) contiguous chunks.  Entry i of lane l is sched[i * lanes + l]; the entry
// encodings are described in host/rpa_schedule.hpp.  A segment is a run of pairs of one output
// rid inside one chunk; its partial sum goes to the next slot of the lane (slot_base[l],
// slot_base[l]+1, ...), and rid r sums the slots seg_ptr[r] .. seg_ptr[r+1]-1 in order.
struct RpaSchedule {
    const int *sched;
    const int *count;      // [lanes] entries of each lane
    const int *slot_base;  // [lanes]
    const int *seg_ptr;    // [Nl + 1]
    int lanes, n_seg;
    int len;       // entries per lane
    int in_smem;   // the kernel stages the schedule in shared memory
    const int *image;  // sched | count | slot_base | seg_ptr contiguous, as staged (16-byte aligned)
    int image_bytes;   // multiple of 16
};

// Shared-memory words of a staged schedule (sched, count, slot_base, seg_ptr).
__host__ __device__ inline int rpa_smem_ints(const RpaSchedule &r, int nl) {
    return r.len * r.lanes + 2 * r.lanes + nl + 1;
}

// Argument block of one flow in working precision T (float: the reference's types; double:
// the FP64 flow, SPN_SU2_FP64).  The cutoff list is float in both (the task file's values).
// Vertex arrays hold (spin, density) pairs per element, index ((s(s+1)/2+u)*N + t)*Nl + rid.
template <class T>
struct FlowArgsT {
    int n, nl, fn, wsite, max_nodes, n_range;
    float cutoff, spin;
    const T *freq;
    const unsigned short *mesh_lo;  // bucket index of the mesh (dev::MeshIndex; FP32 flows)
    unsigned mesh_base;
    int mesh_shift;
    const dev::pair_t<T> *sd;  // state
    dev::pair_t<T> *dsd;       // flow
    const T *v2;           // self-energy state
    T *dv2;                // self-energy flow
    const double *v2d;     // FP64 self-energy state (used when fp64_sigma)
    double *dv2d;          // FP64 self-energy flow
    int fp64_sigma;
    const int *sites, *inv_sites, *ov_ptr, *ov_r1, *ov_r2, *range_rid, *range_inv;
    T *node_wp, *node_c;
    int *node_cnt;
    int *work_counter;
    unsigned *status;
    RpaSchedule rpa;
};
using FlowArgs = FlowArgsT<float>;

// Correlation measurement (nu = 0) of one flow: the state it reads (sd, or the separate
// arrays ss/dd of a caller of the allocation-free measurement), the per-node partial sums and
// the output zz[n_corr], dd[n_corr], chi_s[nl], chi_d[nl].
template <class T>
struct CorrArgsT {
    int n, nl, n_corr;
    float cutoff, spin;
    const T *freq, *v2;
    const dev::pair_t<T> *sd;
    const T *ss, *dd;
    const double *v2d;  // FP64 self-energy, read instead of v2 when not NULL
    const int *sites, *inv_sites, *corr_rid;
    double *partial;  // [max_nodes][2][nl]
    T *out;
    int wsite;
};
using CorrArgs = CorrArgsT<float>;

// ------------------------------------------------------------------------------------
// Batches: many flows advanced together (include/spn_su2.h, spn_batch_*).  Each flow has a
// device-resident record; the batched kernels take the record array and a list of the flows
// they work on, and read every per-step quantity (cutoff, step index, phase) from the record,
// so a captured step can be replayed without the host.
// ------------------------------------------------------------------------------------
constexpr int kPhaseFlowing = 0;  // computes the flow, measures, steps to the next cutoff
constexpr int kPhaseFinal = 1;    // at the last cutoff: only the final measurement is left
constexpr int kPhaseDone = 2;     // finished (or diverged)

constexpr unsigned kFlagDiverged = 1u;
constexpr unsigned kFlagNodeOverflow = 2u;

struct BatchFlow {
    FlowArgs a;            // a.cutoff is the current cutoff, a.status the per-step status word
    CorrArgs c;            // c.cutoff / c.out are derived per step from the fields below
    const float *cutoffs;  // [n_cutoffs] descending
    float *hist;           // [n_cutoffs][2 * n_corr + 2 * nl] measurement at every cutoff
    int n_cutoffs;
    int step;              // index of the current cutoff
    int phase;
    unsigned flags;
};

// Vertex-flow kernel (su2_vertex.cu): dynamic shared memory per block, the number of blocks
// per SM it achieves, and the launch.
// `npi`: loop-frequency nodes a site group evaluates per iteration (1 or 2); whether the RPA
// schedule is staged in shared memory is a.rpa.in_smem.  Both are chosen per flow by timing.
size_t vertex_flow_smem_bytes(int nl, const RpaSchedule &rpa, int npi);
int vertex_flow_blocks_per_sm(int nl, const RpaSchedule &rpa, int npi);
void launch_vertex_flow(const FlowArgs &a, int npi, int grid, cudaStream_t stream);
// FP64 flow (su2_vertex64.cu): one warp per triple over a persistent grid.
void launch_vertex_flow_f64(const FlowArgsT<double> &a, int grid, cudaStream_t stream);
int vertex_flow_f64_blocks_per_sm(int nl);

// Largest schedule staged in shared memory; larger ones are read from global memory.
constexpr int kRpaSmemMaxInts = 8192;

// Batched vertex flow: one persistent launch over the ragged work list of all flows of one
// vertex class (vertex_class below).  Work item w belongs to flow list[f] with
// prefix[f] <= w < prefix[f+1] (prefix[f+1] - prefix[f] = that flow's triple count).
// `warp_area` is the per-warp shared-memory bytes the largest flow of the list needs.
// `sched_ints` > 0: each warp stages the RPA schedule of its current flow in shared memory
// (room for that many ints; every flow of the list must fit), else it reads global memory.
struct BatchVertexArgs {
    BatchFlow *flows;
    const int *list, *prefix;
    int n_list, total, n_max;
    int *counter;
    int warp_area;
    int sched_ints;
    int n_seg_max;  // classes 6-8 (CTA per triple): the largest RPA segment count of the list
};
// Grouped batches (flows sharing mesh, lattice tables and cutoff; see su2_vertex.cu): one
// persistent launch per vertex class 0..3 over (subgroup, triple) items.  A subgroup holds up
// to group_vertex_gmax(cls) flows: members[sg * gmax + q] is the record index of member q, -1
// after the last; its items are prefix[sg] .. prefix[sg + 1] - 1 (its flows' F_N triples).
// n_seg_max: the largest RPA segment count of the flows in the launch.
struct GroupVertexArgs {
    BatchFlow *flows;
    const int *members, *prefix;
    int n_sg, total, gmax;
    int *counter;
    int n_seg_max;
};
bool group_vertex_eligible(int nl);  // 5 <= nl <= 32
int group_vertex_gmax(int cls);
size_t group_vertex_smem_bytes(int cls, int n_seg_max);
int group_vertex_blocks_per_sm(int cls, int n_seg_max);
void launch_group_vertex(const GroupVertexArgs &g, int cls, int grid, cudaStream_t stream);
size_t batch_vertex_warp_area(int nl, int n_seg, int npi);
size_t batch_vertex_smem_bytes(int n_max, size_t warp_area, int sched_ints);
int batch_vertex_blocks_per_sm(int cls, int npi, size_t smem);
void launch_batch_vertex(const BatchVertexArgs &b, int cls, int npi, int grid, cudaStream_t stream);
int vertex_spt(int nl);  // sites per lane of a flow with nl sites
// Vertex-kernel class of a flow (one kernel instance per class): 0-3 for nl <= 32 (outer-product
// RPA with w = 8, 16, 24, 32, a warp per triple), 6-10 for 33 <= nl <= 128 (outer-product RPA
// with w = 48, 64, 80, 96, 128, a CTA per triple); 4 and 5 are unused.
constexpr int kVertexClasses = 11;
int vertex_class(int nl);
// Lanes of the RPA schedule the vertex kernel of an nl-site flow walks: 32 (a warp per triple)
// or the CTA's threads (33 to 128 sites).
int vertex_rpa_lanes(int nl);
size_t batch_big_smem_bytes(int cls, int n_seg_max);

}  // namespace spn
