// The flow handle of the C ABI (struct spn_su2) and the host helpers shared by the single-flow
// entry points (su2_flow.cu) and the batch engine (su2_batch.cu).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <utility>
#include <vector>
#include "su2_common.cuh"
#include "host/capi_common.hpp"
#include "../../include/spn_su2.h"

namespace spn {

void cuda_check(cudaError_t e, const char *what);
int wsite_for(int nl);  // lanes of a site group: next power of two >= nl (32 above 32 sites)
int spt_for(int nl);    // sites per lane: 1, 2 or 4
constexpr int kMaxSites = 128;

}  // namespace spn

struct spn_su2 {
    int device = 0;
    int n = 0, nl = 0, n_range = 0, n_corr = 0, max_nodes = 0, flags = 0, n_overlap = 0;
    long long fn = 0;
    float spin = 0.5f, cutoff = 0.0f;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int vertex_grid = 0;
    float *freq = nullptr, *v2 = nullptr, *dv2 = nullptr;
    float2 *sd = nullptr, *dsd = nullptr;  // vertex state and flow, (spin, density) per element
    float *stage = nullptr;  // 2 F_N Nl floats for state copies in the reference layout (on first use)
    unsigned short *mesh_lo = nullptr;  // bucket index of the frequency mesh
    unsigned mesh_base = 0;
    int mesh_shift = 0;
    float *node_wp = nullptr, *node_c = nullptr, *corr_out = nullptr;
    int *node_cnt = nullptr, *work_counter = nullptr;
    unsigned *status = nullptr;
    int *sites = nullptr, *inv_sites = nullptr, *ov_ptr = nullptr, *ov_r1 = nullptr, *ov_r2 = nullptr;
    int *range_rid = nullptr, *range_inv = nullptr, *corr_rid = nullptr;
    double *corr_partial = nullptr;
    double *v2d = nullptr, *dv2d = nullptr;  // FP64 self-energy (SPN_SU2_FP64_SELF_ENERGY)
    // FP64 flow (SPN_SU2_FP64): state, flow, node tables and measurement output in double;
    // the float arrays above other than v2/dv2 stay unallocated.
    double *freq64 = nullptr;
    double2 *sd64 = nullptr, *dsd64 = nullptr;
    double *node_wp64 = nullptr, *node_c64 = nullptr, *corr_out64 = nullptr;
    int *rpa_image = nullptr;  // sched | count | slot_base | seg_ptr in one allocation (the staged layout)
    int *rpa_sched = nullptr, *rpa_count = nullptr, *rpa_slot_base = nullptr, *rpa_seg_ptr = nullptr;  // into rpa_image
    int rpa_image_bytes = 0;
    int rpa_lanes = 0, rpa_n_seg = 0, rpa_len = 0, rpa_in_smem = 0;
    int vertex_npi = 1;       // loop-frequency nodes per site-group iteration
    int sms = 0;
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, int>> ev_vertex, ev_step;  // indices into ev_pool

    spn::FlowArgs args() const {
        spn::FlowArgs a;
        a.n = n;
        a.nl = nl;
        a.fn = int(fn);
        a.wsite = spn::wsite_for(nl);
        a.max_nodes = max_nodes;
        a.n_range = n_range;
        a.cutoff = cutoff;
        a.spin = spin;
        a.freq = freq;
        a.mesh_lo = mesh_lo;
        a.mesh_base = mesh_base;
        a.mesh_shift = mesh_shift;
        a.sd = sd;
        a.dsd = dsd;
        a.v2 = v2;
        a.dv2 = dv2;
        a.v2d = v2d;
        a.dv2d = dv2d;
        a.fp64_sigma = (flags & SPN_SU2_FP64_SELF_ENERGY) ? 1 : 0;
        a.sites = sites;
        a.inv_sites = inv_sites;
        a.ov_ptr = ov_ptr;
        a.ov_r1 = ov_r1;
        a.ov_r2 = ov_r2;
        a.range_rid = range_rid;
        a.range_inv = range_inv;
        a.node_wp = node_wp;
        a.node_c = node_c;
        a.node_cnt = node_cnt;
        a.work_counter = work_counter;
        a.status = status;
        a.rpa.sched = rpa_sched;
        a.rpa.count = rpa_count;
        a.rpa.slot_base = rpa_slot_base;
        a.rpa.seg_ptr = rpa_seg_ptr;
        a.rpa.image = rpa_image;
        a.rpa.image_bytes = rpa_image_bytes;
        a.rpa.lanes = rpa_lanes;
        a.rpa.n_seg = rpa_n_seg;
        a.rpa.len = rpa_len;
        a.rpa.in_smem = rpa_in_smem;
        return a;
    }

    bool fp64() const { return (flags & SPN_SU2_FP64) != 0; }

    // Argument block of an FP64 flow: every array in double, the self-energy in v2d/dv2d.
    spn::FlowArgsT<double> args64() const {
        const spn::FlowArgs f = args();
        spn::FlowArgsT<double> a;
        a.n = f.n;
        a.nl = f.nl;
        a.fn = f.fn;
        a.wsite = f.wsite;
        a.max_nodes = f.max_nodes;
        a.n_range = f.n_range;
        a.cutoff = f.cutoff;
        a.spin = f.spin;
        a.freq = freq64;
        a.mesh_lo = mesh_lo;
        a.mesh_base = mesh_base;
        a.mesh_shift = mesh_shift;
        a.sd = sd64;
        a.dsd = dsd64;
        a.v2 = v2d;
        a.dv2 = dv2d;
        a.v2d = v2d;
        a.dv2d = dv2d;
        a.fp64_sigma = 0;
        a.sites = f.sites;
        a.inv_sites = f.inv_sites;
        a.ov_ptr = f.ov_ptr;
        a.ov_r1 = f.ov_r1;
        a.ov_r2 = f.ov_r2;
        a.range_rid = f.range_rid;
        a.range_inv = f.range_inv;
        a.node_wp = node_wp64;
        a.node_c = node_c64;
        a.node_cnt = f.node_cnt;
        a.work_counter = f.work_counter;
        a.status = f.status;
        a.rpa = f.rpa;
        return a;
    }

    int event() {
        cudaEvent_t e;
        spn::cuda_check(cudaEventCreate(&e), "cudaEventCreate");
        ev_pool.push_back(e);
        return int(ev_pool.size()) - 1;
    }

    void release() {
        cudaSetDevice(device);
        for (auto e : ev_pool) cudaEventDestroy(e);
        ev_pool.clear();
        void *ptrs[] = {freq,      sd,     dsd,       stage,     v2,           dv2,       node_wp,  node_c,
                        corr_out,  node_cnt, work_counter, status, sites,     inv_sites,    ov_ptr,    ov_r1,
                        ov_r2,     range_rid, range_inv, corr_rid, corr_partial, rpa_image, v2d,      dv2d,
                        freq64,    sd64,   dsd64,     node_wp64, node_c64,  corr_out64, mesh_lo};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};


namespace spn {

// Allocates and initialises one flow (spn_su2_create); work is queued on `stream`, or on a
// stream of its own when `stream` is NULL.
spn_su2 *create_flow(const spn_su2_desc *d, cudaStream_t stream);
// Argument block of the correlation measurement of a flow at its current cutoff.
CorrArgs corr_args(const spn_su2 *h);
// State movement in the reference layout (separate spin and density arrays of F_N*Nl floats)
// for an FP32 flow, through `stage` (2 F_N Nl device floats): the two halves are copied and
// interleaved into the flow's state, or the state is split into them and copied out.  Queued
// on `stream`; the host arrays must stay valid until it is synchronised.
void upload_state(spn_su2 *h, const float *v4ss, const float *v4dd, float *stage, cudaStream_t stream);
void download_state(const spn_su2 *h, const float2 *src, float *v4ss, float *v4dd, float *stage, cudaStream_t stream);
// Builds the node tables and evaluates the vertex flow etc. of one flow: see su2_flow.cu.

}  // namespace spn
