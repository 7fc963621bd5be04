// Batched SU(2) flows on one GPU: many flows (different lattices, ranges, frequency counts,
// cutoff lists) advanced together, each step one launch per kernel for all of them.
//
// Per step, for the flows still flowing:
//   prepare      status words and work counters cleared
//   self-energy  grid (frequency, flow)                    body: self_energy_body
//   node tables  grid (frequency block, flow)              body: node_table_body
//   vertex flow  one persistent launch per site class over the ragged (flow, triple) list
//   correlation  grid (outer node, flow) + grid (flow)     bodies: corr_inner_body / corr_final_body
//                (also for flows at their last cutoff, whose final measurement is due)
//   Euler        grid (block, flow), skipped for a flow whose step produced a NaN
//   advance      per flow: next cutoff, or final / done / diverged
// Every per-step quantity (cutoff, step index, phase) lives in the flow's device record, so the
// captured step (a CUDA graph) is replayed unchanged while the set of flows and their phases
// stay the same; the host rebuilds the plan only when a flow joins, finishes or diverges.
// The kernels evaluate each flow with the same device functions as the single-flow path, so
// a flow's results do not depend on the other flows of the batch.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <utility>
#include <vector>
#include "su2_common.cuh"
#include "su2_device.cuh"
#include "su2_kernels.cuh"
#include "su2_handle.cuh"

using namespace spn;
using namespace spn::dev;

namespace {

constexpr int kClasses = 3;  // measurement classes: sites per lane 1, 2, 4
constexpr int kBatchSchedMaxInts = 3072;  // per-warp staged RPA schedule (12 KB) at most
constexpr int kGroupClasses = 4;  // grouped vertex classes: vertex classes 0..3
constexpr int kCounters = kVertexClasses + kGroupClasses;

__global__ void batch_prepare_kernel(BatchFlow *flows, const int *list, int n, int *counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kCounters && blockIdx.x == 0) counters[i] = 0;
    if (i >= n) return;
    BatchFlow &f = flows[list[i]];
    if (f.phase != kPhaseDone) *f.a.status = 0u;
}

__global__ void __launch_bounds__(128) batch_self_energy_kernel(const BatchFlow *flows, const int *list) {
    const BatchFlow &f = flows[list[blockIdx.y]];
    if (f.phase != kPhaseFlowing) return;
    const FlowArgs a = f.a;
    if (int(blockIdx.x) >= a.n) return;
    self_energy_body(a, blockIdx.x);
}

__global__ void batch_node_table_kernel(const BatchFlow *flows, const int *list) {
    const BatchFlow &f = flows[list[blockIdx.y]];
    if (f.phase != kPhaseFlowing) return;
    const FlowArgs a = f.a;
    if (int(blockIdx.x * blockDim.x) >= a.n) return;
    node_table_body(a, blockIdx.x);
}

__device__ __forceinline__ CorrArgs batch_corr_args(const BatchFlow &f) {
    CorrArgs c = f.c;
    c.cutoff = f.a.cutoff;
    c.out = f.hist + size_t(f.step) * (2 * size_t(c.n_corr) + 2 * c.nl);
    return c;
}

template <int SPT>
__global__ void __launch_bounds__(128) batch_corr_inner_kernel(const BatchFlow *flows, const int *list) {
    const BatchFlow &f = flows[list[blockIdx.y]];
    if (f.phase == kPhaseDone) return;
    const CorrArgs c = batch_corr_args(f);
    if (int(blockIdx.x) >= 2 * c.n + 4) return;
    corr_inner_body<SPT>(c, PairedState<float>{c.sd}, blockIdx.x);
}

__global__ void batch_corr_final_kernel(const BatchFlow *flows, const int *list) {
    const BatchFlow &f = flows[list[blockIdx.x]];
    if (f.phase == kPhaseDone) return;
    corr_final_body(batch_corr_args(f));
}

// Euler step of every flowing flow without a NaN in this step's flow (a flow whose step
// produced a NaN stops before the update, as SpinParser::runCore does).
__global__ void batch_euler_kernel(const BatchFlow *flows, const int *list) {
    const BatchFlow &f = flows[list[blockIdx.y]];
    if (f.phase != kPhaseFlowing || (*f.a.status & (kStatusNaN | kStatusNodeOverflow))) return;
    const FlowArgs &a = f.a;
    const float step = __fsub_rn(f.cutoffs[f.step + 1], f.cutoffs[f.step]);
    // the (spin, density) state is one array of 2 F_N Nl floats (F_N Nl float2, 8-byte aligned)
    const long long n2 = (long long)a.fn * a.nl;
    const long long stride = (long long)gridDim.x * blockDim.x;
    float2 *x = const_cast<float2 *>(a.sd);
    const float2 *dx = a.dsd;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += stride) {
        float2 v = x[i];
        const float2 d = dx[i];
        v.x = euler_update(v.x, d.x, step);
        v.y = euler_update(v.y, d.y, step);
        x[i] = v;
    }
    if (blockIdx.x == 0) {
        float *v2 = const_cast<float *>(a.v2);
        for (int i = threadIdx.x; i < a.n; i += blockDim.x) {
            if (a.fp64_sigma) {
                double *v2d = const_cast<double *>(a.v2d);
                const double v = euler_update_f64(v2d[i], a.dv2d[i], step);
                v2d[i] = v;
                v2[i] = float(v);
            } else {
                v2[i] = euler_update(v2[i], a.dv2[i], step);
            }
        }
    }
}

__global__ void batch_advance_kernel(BatchFlow *flows, const int *list, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BatchFlow &f = flows[list[i]];
    if (f.phase == kPhaseFinal) {
        f.phase = kPhaseDone;
    } else if (f.phase == kPhaseFlowing) {
        const unsigned st = *f.a.status;
        if (st & kStatusNodeOverflow) {
            f.flags |= kFlagNodeOverflow;
            f.phase = kPhaseDone;
        } else if (st & kStatusNaN) {
            f.flags |= kFlagDiverged;
            f.phase = kPhaseDone;
        } else {
            f.step += 1;
            f.a.cutoff = f.cutoffs[f.step];
            if (f.step == f.n_cutoffs - 1) f.phase = kPhaseFinal;
        }
    }
}

template <class T>
T *dalloc(size_t count, const char *what) {
    void *p = nullptr;
    cuda_check(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), what);
    return static_cast<T *>(p);
}

int class_of(int nl) {
    const int spt = spt_for(nl);
    return spt == 1 ? 0 : (spt == 2 ? 1 : 2);
}

}  // namespace

struct spn_batch {
    struct Flow {
        spn_su2 *h = nullptr;
        float *cutoffs = nullptr, *hist = nullptr;
        std::vector<float> host_cutoffs;
        // what the vertex flow of flows in one group must share: mesh, lattice tables, spin
        // length and cutoff list (the bytes of each, in a fixed order)
        std::vector<unsigned char> share_key;
        int share_id = -1;
        int n_cutoffs = 0, step = 0, phase = kPhaseDone;
        unsigned flags = 0;
        bool used = false;
        bool paused = false;  // held out of the steps (keeps its state and phase)
        size_t hist_row = 0;
    };
    int device = 0, sms = 0, npi = 1;
    bool use_graph = true;
    // grouped vertex flow: groups of at least min_group flows (0 = off) share node supports,
    // in subgroups of at most gmax / group_cap_div flows per CTA
    int min_group = 0, group_cap_div = 1;
    bool stage_sched = false;  // per-flow kernel: each warp stages its flow's RPA schedule in shared memory
    int next_share_id = 0;
    cudaStream_t stream = nullptr;
    std::vector<Flow> flows;
    BatchFlow *d_flows = nullptr;
    int capacity = 0;
    int *d_lists = nullptr, *d_counters = nullptr;
    size_t lists_cap = 0;
    BatchFlow *h_status = nullptr;  // pinned: device records copied back after each step
    cudaEvent_t status_ev = nullptr;
    bool status_pending = false;
    // plan
    bool plan_valid = false;
    std::vector<int> lists;  // flowing | measure | per-class measure | per-class vertex list | per-class prefix
    int n_flowing = 0, n_measure = 0, n_max = 2;
    int off_flowing = 0, off_measure = 0;
    int off_cm[kClasses] = {}, n_cm[kClasses] = {};  // per measurement class
    // per vertex class (vertex_class): work lists, prefixes, shared memory, grid
    int off_cv[kVertexClasses] = {}, n_cv[kVertexClasses] = {}, off_cp[kVertexClasses] = {}, total_cv[kVertexClasses] = {};
    int warp_area[kVertexClasses] = {}, nl_max = 1, vgrid[kVertexClasses] = {}, sched_ints[kVertexClasses] = {};
    int nseg_v[kVertexClasses] = {};  // classes 6-8: the largest RPA segment count of the list
    // per grouped class: subgroup member table, item prefix, grid
    int off_gm[kGroupClasses] = {}, off_gp[kGroupClasses] = {}, n_sg[kGroupClasses] = {}, total_g[kGroupClasses] = {};
    int nseg_g[kGroupClasses] = {}, ggrid[kGroupClasses] = {};
    int n_grouped = 0;  // flows evaluated by the grouped kernel in the current plan
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long steps_run = 0, graph_builds = 0;

    ~spn_batch() {
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        for (auto &f : flows) release(f);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (d_flows) cudaFree(d_flows);
        if (d_lists) cudaFree(d_lists);
        if (d_counters) cudaFree(d_counters);
        if (h_status) cudaFreeHost(h_status);
        if (status_ev) cudaEventDestroy(status_ev);
        if (stream) cudaStreamDestroy(stream);
    }

    static void release(Flow &f) {
        if (f.h) {
            f.h->release();
            delete f.h;
            f.h = nullptr;
        }
        if (f.cutoffs) cudaFree(f.cutoffs);
        if (f.hist) cudaFree(f.hist);
        f.cutoffs = f.hist = nullptr;
        f.used = false;
        f.phase = kPhaseDone;
    }

    void ensure_capacity(int n) {
        if (n <= capacity) return;
        int cap = std::max(16, capacity * 2);
        while (cap < n) cap *= 2;
        cuda_check(cudaStreamSynchronize(stream), "batch sync");
        BatchFlow *nf = dalloc<BatchFlow>(cap, "alloc batch records");
        BatchFlow *nh = nullptr;
        cuda_check(cudaMallocHost(&nh, sizeof(BatchFlow) * cap), "alloc pinned batch records");
        if (d_flows) {
            cuda_check(cudaMemcpyAsync(nf, d_flows, sizeof(BatchFlow) * capacity, cudaMemcpyDeviceToDevice, stream), "copy records");
            cuda_check(cudaStreamSynchronize(stream), "batch sync");
            cudaFree(d_flows);
        }
        if (h_status) {
            std::memcpy(nh, h_status, sizeof(BatchFlow) * capacity);
            cudaFreeHost(h_status);
        }
        d_flows = nf;
        h_status = nh;
        capacity = cap;
        plan_valid = false;
    }

    void ensure_lists(size_t n) {
        if (n <= lists_cap) return;
        if (d_lists) {
            cuda_check(cudaStreamSynchronize(stream), "batch sync");
            cudaFree(d_lists);
        }
        lists_cap = std::max<size_t>(n, 2 * lists_cap);
        d_lists = dalloc<int>(lists_cap, "alloc batch lists");
    }

    // Reads the device records of the previous step (lagging one step behind the host) and
    // takes over divergence and overflow, which only the device knows.
    void absorb_status(bool wait) {
        if (!status_pending) return;
        if (!wait && cudaEventQuery(status_ev) == cudaErrorNotReady) return;
        cuda_check(cudaEventSynchronize(status_ev), "batch status sync");
        status_pending = false;
        for (size_t i = 0; i < flows.size(); ++i) {
            Flow &f = flows[i];
            if (!f.used) continue;
            const BatchFlow &r = h_status[i];
            if (r.flags & ~f.flags) {
                f.flags |= r.flags;
                f.phase = kPhaseDone;
                f.step = r.step;
                plan_valid = false;
            }
        }
    }

    void build_plan() {
        lists.clear();
        n_max = 2;
        nl_max = 1;
        std::vector<int> flowing, measure, cm[kClasses], cv[kVertexClasses];
        std::map<std::pair<int, int>, std::vector<int>> buckets;  // (share id, step) -> flows
        for (size_t i = 0; i < flows.size(); ++i) {
            const Flow &f = flows[i];
            if (!f.used || f.phase == kPhaseDone || f.paused) continue;
            const int c = class_of(f.h->nl);
            measure.push_back(int(i));
            cm[c].push_back(int(i));
            const int vc = vertex_class(f.h->nl);
            n_max = std::max(n_max, f.h->n);
            nl_max = std::max(nl_max, f.h->nl);
            if (f.phase == kPhaseFlowing) {
                flowing.push_back(int(i));
                if (min_group > 0 && vc < kGroupClasses && group_vertex_eligible(f.h->nl))
                    buckets[{f.share_id, f.step}].push_back(int(i));
                else
                    cv[vc].push_back(int(i));
            }
        }
        // groups large enough go to the grouped kernel in balanced subgroups of at most
        // gmax / group_cap_div flows; the rest to the per-flow kernel
        std::vector<int> gm[kGroupClasses], gp[kGroupClasses];
        n_grouped = 0;
        for (int c = 0; c < kGroupClasses; ++c) {
            gp[c].assign(1, 0);
            nseg_g[c] = 0;
        }
        for (auto &kv : buckets) {
            const std::vector<int> &v = kv.second;
            const int vc = vertex_class(flows[v[0]].h->nl);
            if (int(v.size()) < min_group) {
                cv[vc].insert(cv[vc].end(), v.begin(), v.end());
                continue;
            }
            const int gmax = group_vertex_gmax(vc);
            const int cap = std::max(1, gmax / group_cap_div);
            const int parts = (int(v.size()) + cap - 1) / cap;
            size_t at = 0;
            for (int q = 0; q < parts; ++q) {
                const size_t take = (v.size() - at) / size_t(parts - q);  // balanced sizes
                for (int m = 0; m < gmax; ++m) gm[vc].push_back(m < int(take) ? v[at + m] : -1);
                const long long next = gp[vc].back() + flows[v[at]].h->fn;
                if (next >= (1ll << 31)) throw Error(ErrorType::Unsupported, "batch work list beyond 2^31 items");
                gp[vc].push_back(int(next));
                for (size_t m = 0; m < take; ++m) nseg_g[vc] = std::max(nseg_g[vc], flows[v[at + m]].h->rpa_n_seg);
                at += take;
                n_grouped += int(take);
            }
        }
        auto put = [&](const std::vector<int> &v) {
            const int off = int(lists.size());
            lists.insert(lists.end(), v.begin(), v.end());
            return off;
        };
        off_flowing = put(flowing);
        n_flowing = int(flowing.size());
        off_measure = put(measure);
        n_measure = int(measure.size());
        for (int c = 0; c < kClasses; ++c) {
            off_cm[c] = put(cm[c]);
            n_cm[c] = int(cm[c].size());
        }
        for (int c = 0; c < kVertexClasses; ++c) {
            off_cv[c] = put(cv[c]);
            n_cv[c] = int(cv[c].size());
            std::vector<int> prefix(1, 0);
            size_t area = 0;
            int sched = 0, nseg = 0;
            for (int i : cv[c]) {
                const spn_su2 *h = flows[i].h;
                const long long next = prefix.back() + h->fn;
                if (next >= (1ll << 31)) throw Error(ErrorType::Unsupported, "batch work list beyond 2^31 items");
                prefix.push_back(int(next));
                if (c < 6) area = std::max(area, batch_vertex_warp_area(h->nl, h->rpa_n_seg, npi));
                sched = std::max(sched, rpa_smem_ints(h->args().rpa, h->nl));
                nseg = std::max(nseg, h->rpa_n_seg);
            }
            nseg_v[c] = nseg;
            off_cp[c] = put(prefix);
            total_cv[c] = prefix.back();
            warp_area[c] = int((area + 15) / 16 * 16);
            // each warp stages its flow's RPA schedule when the largest one is small (warp-per-
            // triple classes; the CTA-per-triple classes 6-8 read it from global memory)
            sched_ints[c] = (c < 6 && stage_sched && sched <= kBatchSchedMaxInts) ? sched : 0;
            vgrid[c] = 0;
            if (n_cv[c] > 0) {
                const size_t smem = c >= 6 ? batch_big_smem_bytes(c, nseg_v[c])
                                           : batch_vertex_smem_bytes(n_max, warp_area[c], sched_ints[c]);
                const int per_sm = batch_vertex_blocks_per_sm(c, npi, smem);
                cudaGetLastError();
                if (per_sm < 1) throw Error(ErrorType::Unsupported, "batched vertex-flow kernel does not fit for this batch");
                vgrid[c] = sms * per_sm;
            }
        }
        for (int c = 0; c < kGroupClasses; ++c) {
            off_gm[c] = put(gm[c]);
            off_gp[c] = put(gp[c]);
            n_sg[c] = int(gp[c].size()) - 1;
            total_g[c] = gp[c].back();
            ggrid[c] = 0;
            if (n_sg[c] > 0) {
                const int per_sm = group_vertex_blocks_per_sm(c, nseg_g[c]);
                cudaGetLastError();
                if (per_sm < 1) throw Error(ErrorType::Unsupported, "grouped vertex-flow kernel does not fit for this batch");
                ggrid[c] = sms * per_sm;
            }
        }
        ensure_lists(lists.size());
        cuda_check(cudaStreamSynchronize(stream), "batch sync");
        if (!lists.empty())
            cuda_check(cudaMemcpyAsync(d_lists, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice, stream),
                       "upload batch lists");
        cuda_check(cudaStreamSynchronize(stream), "batch sync");
        if (exec) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        if (graph) {
            cudaGraphDestroy(graph);
            graph = nullptr;
        }
        plan_valid = true;
    }

    // A step: enqueue_front (status and counters cleared, self-energy flow, node tables),
    // enqueue_vertex (the vertex flow), enqueue_back (measurement, Euler, advance).
    void enqueue_step() {
        enqueue_front();
        enqueue_vertex();
        enqueue_back();
    }

    void enqueue_front() {
        const int *L = d_lists;
        batch_prepare_kernel<<<(std::max(n_measure, kCounters) + 127) / 128, 128, 0, stream>>>(d_flows, L + off_measure,
                                                                                               n_measure, d_counters);
        if (n_flowing > 0) {
            batch_self_energy_kernel<<<dim3(n_max, n_flowing), 128, 0, stream>>>(d_flows, L + off_flowing);
            batch_node_table_kernel<<<dim3((n_max + 63) / 64, n_flowing), 64, 0, stream>>>(d_flows, L + off_flowing);
        }
    }

    void enqueue_vertex() {
        const int *L = d_lists;
        if (n_flowing > 0) {
            for (int c = 0; c < kVertexClasses; ++c) {
                if (n_cv[c] == 0) continue;
                BatchVertexArgs b;
                b.flows = d_flows;
                b.list = L + off_cv[c];
                b.prefix = L + off_cp[c];
                b.n_list = n_cv[c];
                b.total = total_cv[c];
                b.n_max = n_max;
                b.counter = d_counters + c;
                b.warp_area = warp_area[c];
                b.sched_ints = sched_ints[c];
                b.n_seg_max = nseg_v[c];
                launch_batch_vertex(b, c, npi, vgrid[c], stream);
            }
            for (int c = 0; c < kGroupClasses; ++c) {
                if (n_sg[c] == 0) continue;
                GroupVertexArgs g;
                g.flows = d_flows;
                g.members = L + off_gm[c];
                g.prefix = L + off_gp[c];
                g.n_sg = n_sg[c];
                g.total = total_g[c];
                g.gmax = group_vertex_gmax(c);
                g.counter = d_counters + kVertexClasses + c;
                g.n_seg_max = nseg_g[c];
                launch_group_vertex(g, c, ggrid[c], stream);
            }
        }
    }

    void enqueue_back() {
        const int *L = d_lists;
        for (int c = 0; c < kClasses; ++c) {
            if (n_cm[c] == 0) continue;
            const dim3 g(2 * n_max + 4, n_cm[c]);
            if (c == 0) batch_corr_inner_kernel<1><<<g, 128, 0, stream>>>(d_flows, L + off_cm[c]);
            else if (c == 1) batch_corr_inner_kernel<2><<<g, 128, 0, stream>>>(d_flows, L + off_cm[c]);
            else batch_corr_inner_kernel<4><<<g, 128, 0, stream>>>(d_flows, L + off_cm[c]);
        }
        if (n_measure > 0)
            batch_corr_final_kernel<<<n_measure, 128, 2 * nl_max * sizeof(double), stream>>>(d_flows, L + off_measure);
        if (n_flowing > 0) batch_euler_kernel<<<dim3(48, n_flowing), 256, 0, stream>>>(d_flows, L + off_flowing);
        batch_advance_kernel<<<(std::max(n_measure, 1) + 127) / 128, 128, 0, stream>>>(d_flows, L + off_measure, n_measure);
        cuda_check(cudaGetLastError(), "batch step launch");
    }
};

namespace {

// The bytes that decide whether two flows' vertex flows can share node supports: frequency
// mesh, lattice tables, spin length and cutoff list (equal keys = equal inputs of every
// support and of the RPA schedule).
std::vector<unsigned char> share_key_of(const spn_su2_desc *d, int n_cutoffs, const float *cutoffs) {
    std::vector<unsigned char> k;
    auto put = [&](const void *p, size_t bytes) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        k.insert(k.end(), c, c + bytes);
    };
    const int nov = d->overlap_ptr ? d->overlap_ptr[d->n_sites] : 0;
    put(&d->n_freq, sizeof(int));
    put(&d->n_sites, sizeof(int));
    put(&nov, sizeof(int));
    put(&n_cutoffs, sizeof(int));
    put(&d->spin_length, sizeof(float));
    put(d->freq, sizeof(float) * d->n_freq);
    put(d->sites_rid, sizeof(int) * d->n_sites);
    put(d->inv_sites_rid, sizeof(int) * d->n_sites);
    if (d->overlap_ptr) {
        put(d->overlap_ptr, sizeof(int) * (d->n_sites + 1));
        put(d->overlap_rid1, sizeof(int) * nov);
        put(d->overlap_rid2, sizeof(int) * nov);
    }
    put(cutoffs, sizeof(float) * n_cutoffs);
    return k;
}

size_t footprint_bytes(const spn_su2_desc *d, int n_cutoffs) {
    const size_t n = size_t(d->n_freq), nl = size_t(d->n_sites);
    const size_t fn = n * n * (n + 1) / 2;
    const size_t nov = size_t(d->overlap_ptr ? d->overlap_ptr[d->n_sites] : 0);
    size_t b = 4 * fn * nl * sizeof(float);                       // state and flow
    b += n * (4 * sizeof(float) + 2 * sizeof(double));             // mesh, self-energy
    b += n * (2 * n + 8) * 2 * sizeof(float) + n * sizeof(int);    // node tables
    b += size_t(2 * n + 8) * 2 * nl * sizeof(double);              // correlation scratch
    b += size_t(n_cutoffs) * (2 * size_t(d->n_corr) + 2 * nl) * sizeof(float);  // measurement history
    b += (4 * nl + 3 * nov + 2 * size_t(d->n_range) + size_t(d->n_corr)) * sizeof(int);
    return b;
}

}  // namespace

extern "C" int spn_batch_create(int device, spn_batch **out) {
    return guarded([&] {
        if (!out) throw Error(ErrorType::Argument, "null output handle");
        std::unique_ptr<spn_batch> b(new spn_batch);
        b->device = device;
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        cuda_check(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device), "device attribute");
        cuda_check(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        cuda_check(cudaEventCreateWithFlags(&b->status_ev, cudaEventDisableTiming), "cudaEventCreate");
        b->d_counters = dalloc<int>(kCounters, "alloc batch counters");
        b->ensure_capacity(16);
        *out = b.release();
    });
}

extern "C" int spn_batch_destroy(spn_batch *b) {
    delete b;
    return SPN_OK;
}

extern "C" int spn_batch_set_variant(spn_batch *b, int npi, int use_graph) {
    return guarded([&] {
        if (!b) throw Error(ErrorType::Argument, "null handle");
        if (npi != 1 && npi != 2) throw Error(ErrorType::Argument, "nodes per iteration must be 1 or 2");
        b->npi = npi;
        b->use_graph = use_graph != 0;
        b->plan_valid = false;
    });
}

extern "C" int spn_batch_set_grouping(spn_batch *b, int min_group, int cap_divisor) {
    return guarded([&] {
        if (!b) throw Error(ErrorType::Argument, "null handle");
        if (min_group < 0 || min_group == 1) throw Error(ErrorType::Argument, "min_group must be 0 (off) or >= 2");
        if (cap_divisor != 1 && cap_divisor != 2 && cap_divisor != 4)
            throw Error(ErrorType::Argument, "cap_divisor must be 1, 2 or 4");
        b->min_group = min_group;
        b->group_cap_div = cap_divisor;
        b->plan_valid = false;
    });
}

extern "C" int spn_batch_footprint(const spn_su2_desc *desc, int n_cutoffs, long long *bytes) {
    return guarded([&] {
        if (!desc || !bytes || n_cutoffs < 1) throw Error(ErrorType::Argument, "spn_batch_footprint: bad argument");
        *bytes = (long long)footprint_bytes(desc, n_cutoffs);
    });
}

extern "C" int spn_batch_add(spn_batch *b, const spn_su2_desc *desc, int n_cutoffs, const float *cutoffs, const float *v2,
                             const float *v4ss, const float *v4dd, int *flow_id) {
    return guarded([&] {
        if (!b || !desc || !cutoffs || n_cutoffs < 1 || !v2 || !v4ss || !v4dd || !flow_id)
            throw Error(ErrorType::Argument, "spn_batch_add: bad argument");
        if (desc->device != b->device) throw Error(ErrorType::Argument, "spn_batch_add: flow device differs from the batch's");
        if (desc->flags & SPN_SU2_FP64) throw Error(ErrorType::Unsupported, "spn_batch_add: FP64 flows run alone (spn_su2_create)");
        for (int k = 1; k < n_cutoffs; ++k)
            if (!(cutoffs[k] < cutoffs[k - 1])) throw Error(ErrorType::Argument, "spn_batch_add: cutoffs must descend");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        b->absorb_status(true);
        int slot = -1;
        for (size_t i = 0; i < b->flows.size(); ++i)
            if (!b->flows[i].used) {
                slot = int(i);
                break;
            }
        if (slot < 0) {
            slot = int(b->flows.size());
            b->flows.emplace_back();
        }
        b->ensure_capacity(slot + 1);
        spn_batch::Flow &f = b->flows[slot];
        try {
            f.share_key = share_key_of(desc, n_cutoffs, cutoffs);
            f.share_id = -1;
            for (const auto &o : b->flows)
                if (&o != &f && o.used && o.share_key == f.share_key) {
                    f.share_id = o.share_id;
                    break;
                }
            if (f.share_id < 0) f.share_id = b->next_share_id++;
            f.h = create_flow(desc, b->stream);
            f.n_cutoffs = n_cutoffs;
            f.host_cutoffs.assign(cutoffs, cutoffs + n_cutoffs);
            f.cutoffs = dalloc<float>(n_cutoffs, "alloc batch cutoffs");
            f.hist_row = 2 * size_t(f.h->n_corr) + 2 * f.h->nl;
            f.hist = dalloc<float>(size_t(n_cutoffs) * f.hist_row, "alloc measurement history");
            cuda_check(cudaMemcpyAsync(f.cutoffs, cutoffs, n_cutoffs * sizeof(float), cudaMemcpyHostToDevice, b->stream), "H2D");
            cuda_check(cudaMemcpyAsync(f.h->v2, v2, f.h->n * sizeof(float), cudaMemcpyHostToDevice, b->stream), "H2D");
            // staged through the new flow's (still unused) flow buffer
            upload_state(f.h, v4ss, v4dd, reinterpret_cast<float *>(f.h->dsd), b->stream);
            std::vector<double> v2d(v2, v2 + f.h->n);
            cuda_check(cudaMemcpyAsync(f.h->v2d, v2d.data(), f.h->n * sizeof(double), cudaMemcpyHostToDevice, b->stream), "H2D");
            f.h->cutoff = cutoffs[0];
            BatchFlow r;
            std::memset(&r, 0, sizeof(r));
            r.a = f.h->args();
            r.c = corr_args(f.h);
            r.cutoffs = f.cutoffs;
            r.hist = f.hist;
            r.n_cutoffs = n_cutoffs;
            r.step = 0;
            r.phase = n_cutoffs > 1 ? kPhaseFlowing : kPhaseFinal;
            r.flags = 0;
            cuda_check(cudaMemcpyAsync(b->d_flows + slot, &r, sizeof(r), cudaMemcpyHostToDevice, b->stream), "H2D record");
            cuda_check(cudaStreamSynchronize(b->stream), "batch add sync");
            f.step = 0;
            f.phase = r.phase;
            f.flags = 0;
            f.used = true;
            b->h_status[slot] = r;
        } catch (...) {
            spn_batch::release(f);
            throw;
        }
        b->plan_valid = false;
        *flow_id = slot;
    });
}

extern "C" int spn_batch_step(spn_batch *b, int *n_active) {
    return guarded([&] {
        if (!b) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        b->absorb_status(false);
        if (!b->plan_valid) b->build_plan();
        if (b->n_measure > 0) {
            if (b->use_graph) {
                if (!b->exec) {
                    cuda_check(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
                    b->enqueue_step();
                    cuda_check(cudaStreamEndCapture(b->stream, &b->graph), "end capture");
                    cuda_check(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
                    ++b->graph_builds;
                }
                cuda_check(cudaGraphLaunch(b->exec, b->stream), "graph launch");
            } else {
                b->enqueue_step();
            }
            ++b->steps_run;
            // the host's view of every flow advances the same way the advance kernel does
            for (auto &f : b->flows) {
                if (!f.used || f.paused) continue;
                if (f.phase == kPhaseFinal) {
                    f.phase = kPhaseDone;
                    b->plan_valid = false;
                } else if (f.phase == kPhaseFlowing) {
                    ++f.step;
                    if (f.step == f.n_cutoffs - 1) {
                        f.phase = kPhaseFinal;
                        b->plan_valid = false;
                    }
                }
            }
            if (!b->status_pending) {
                cuda_check(cudaMemcpyAsync(b->h_status, b->d_flows, sizeof(BatchFlow) * b->flows.size(), cudaMemcpyDeviceToHost,
                                           b->stream),
                           "D2H records");
                cuda_check(cudaEventRecord(b->status_ev, b->stream), "record");
                b->status_pending = true;
            }
        }
        if (n_active) {
            int n = 0;
            for (auto &f : b->flows) n += (f.used && f.phase != kPhaseDone);
            *n_active = n;
        }
    });
}

extern "C" int spn_batch_synchronize(spn_batch *b) {
    return guarded([&] {
        if (!b) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(b->stream), "batch sync");
        b->absorb_status(true);
        // a fresh copy of the records: the pending one may predate the last steps
        cuda_check(cudaMemcpyAsync(b->h_status, b->d_flows, sizeof(BatchFlow) * b->flows.size(), cudaMemcpyDeviceToHost, b->stream),
                   "D2H records");
        cuda_check(cudaEventRecord(b->status_ev, b->stream), "record");
        b->status_pending = true;
        b->absorb_status(true);
    });
}

extern "C" int spn_batch_poll(spn_batch *b, int flow_id, int *phase, int *step, int *flags) {
    return guarded([&] {
        if (!b || flow_id < 0 || flow_id >= int(b->flows.size()) || !b->flows[flow_id].used)
            throw Error(ErrorType::Argument, "spn_batch_poll: unknown flow");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        b->absorb_status(false);
        const spn_batch::Flow &f = b->flows[flow_id];
        if (phase) *phase = f.phase;
        if (step) *step = f.step;
        if (flags) *flags = int(f.flags);
    });
}

extern "C" int spn_batch_get_result(spn_batch *b, int flow_id, int *n_measured, float *cutoffs, float *zz, float *dd,
                                    float *chi_zz, float *chi_dd) {
    return guarded([&] {
        if (!b || flow_id < 0 || flow_id >= int(b->flows.size()) || !b->flows[flow_id].used)
            throw Error(ErrorType::Argument, "spn_batch_get_result: unknown flow");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(b->stream), "batch sync");
        const spn_batch::Flow &f = b->flows[flow_id];
        BatchFlow r;
        cuda_check(cudaMemcpy(&r, b->d_flows + flow_id, sizeof(r), cudaMemcpyDeviceToHost), "D2H record");
        // rows 0..step hold measurements; the row of the current step exists once measured
        const int rows = (r.phase == kPhaseDone) ? r.step + 1 : r.step;
        const int nc = f.h->n_corr, nl = f.h->nl;
        std::vector<float> hist(size_t(std::max(rows, 0)) * f.hist_row);
        if (rows > 0)
            cuda_check(cudaMemcpy(hist.data(), f.hist, hist.size() * sizeof(float), cudaMemcpyDeviceToHost), "D2H history");
        for (int k = 0; k < rows; ++k) {
            const float *row = hist.data() + size_t(k) * f.hist_row;
            if (cutoffs) cutoffs[k] = f.host_cutoffs[k];
            if (zz) std::memcpy(zz + size_t(k) * nc, row, nc * sizeof(float));
            if (dd) std::memcpy(dd + size_t(k) * nc, row + nc, nc * sizeof(float));
            if (chi_zz) std::memcpy(chi_zz + size_t(k) * nl, row + 2 * nc, nl * sizeof(float));
            if (chi_dd) std::memcpy(chi_dd + size_t(k) * nl, row + 2 * nc + nl, nl * sizeof(float));
        }
        if (n_measured) *n_measured = rows;
    });
}

extern "C" int spn_batch_get_state(spn_batch *b, int flow_id, float *cutoff, float *v2, float *v4ss, float *v4dd) {
    return guarded([&] {
        if (!b || flow_id < 0 || flow_id >= int(b->flows.size()) || !b->flows[flow_id].used)
            throw Error(ErrorType::Argument, "spn_batch_get_state: unknown flow");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(b->stream), "batch sync");
        const spn_batch::Flow &f = b->flows[flow_id];
        BatchFlow r;
        cuda_check(cudaMemcpy(&r, b->d_flows + flow_id, sizeof(r), cudaMemcpyDeviceToHost), "D2H record");
        if (cutoff) *cutoff = r.a.cutoff;
        if (v2) cuda_check(cudaMemcpy(v2, f.h->v2, f.h->n * sizeof(float), cudaMemcpyDeviceToHost), "D2H");
        // staged through the flow buffer: between batch steps it holds nothing that is used again
        download_state(f.h, f.h->sd, v4ss, v4dd, reinterpret_cast<float *>(f.h->dsd), b->stream);
        cuda_check(cudaStreamSynchronize(b->stream), "batch get_state sync");
    });
}

extern "C" int spn_batch_remove(spn_batch *b, int flow_id) {
    return guarded([&] {
        if (!b || flow_id < 0 || flow_id >= int(b->flows.size()) || !b->flows[flow_id].used)
            throw Error(ErrorType::Argument, "spn_batch_remove: unknown flow");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(b->stream), "batch sync");
        b->absorb_status(true);
        spn_batch::release(b->flows[flow_id]);
        BatchFlow r;
        std::memset(&r, 0, sizeof(r));
        r.phase = kPhaseDone;
        cuda_check(cudaMemcpy(b->d_flows + flow_id, &r, sizeof(r), cudaMemcpyHostToDevice), "H2D record");
        b->plan_valid = false;
    });
}

// Times the vertex flow of the batch's current flows under each candidate configuration and
// keeps the fastest: nodes per group iteration of the per-flow kernel (1, 2) x its RPA schedule
// (read from global memory, staged per warp in shared memory: more shared memory, fewer
// resident blocks) without sharing, and, when the caller enabled sharing, (1, 2) x cross-flow
// sharing in subgroups of the grouped kernel's full block or of half of it.  The front of a
// step runs once first (self-energy flow and node tables of the current states); the timed
// launches write only the flows' vertex-flow buffers, which hold nothing between steps, so
// no flow's state or results change.  It replaces the reference LoadManager's choice of chunk
// sizes (src/lib/LoadManager.hpp:796-852) for the batch.
extern "C" int spn_batch_autotune(spn_batch *b, int reps, int *npi, int *min_group, int *cap_divisor, float *best_ms) {
    return guarded([&] {
        if (!b || reps < 1) throw Error(ErrorType::Argument, "spn_batch_autotune: bad argument");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(b->stream), "batch sync");
        b->absorb_status(true);
        struct Cand {
            int npi, min_group, cap;
            bool stage;
        };
        const Cand cands[] = {{1, 0, 1, false}, {2, 0, 1, false}, {1, 0, 1, true}, {2, 0, 1, true},
                              {1, 2, 1, false}, {2, 2, 1, false}, {1, 2, 2, false}, {2, 2, 2, false}};
        const Cand keep{b->npi, b->min_group, b->group_cap_div, b->stage_sched};
        // sharing is a candidate only when the caller enabled it (spn_batch_set_grouping): on
        // a scan it wins in the first steps and loses in the later ones, which dominate
        const bool sharing = b->min_group > 0;
        Cand best = keep;
        float best_t = -1.0f;
        struct Events {  // released on every path out
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            ~Events() {
                if (e0) cudaEventDestroy(e0);
                if (e1) cudaEventDestroy(e1);
            }
        } ev;
        cuda_check(cudaEventCreate(&ev.e0), "cudaEventCreate");
        cuda_check(cudaEventCreate(&ev.e1), "cudaEventCreate");
        cudaEvent_t e0 = ev.e0, e1 = ev.e1;
        auto restore = [&](const Cand &c) {
            b->npi = c.npi;
            b->min_group = c.min_group;
            b->group_cap_div = c.cap;
            b->stage_sched = c.stage;
            b->plan_valid = false;
        };
        bool front_done = false;
        try {
            for (const Cand &c : cands) {
                b->npi = c.npi;
                b->min_group = c.min_group;
                b->group_cap_div = c.cap;
                b->stage_sched = c.stage;
                if (c.min_group > 0 && !sharing) continue;
                b->build_plan();
                if (b->n_flowing == 0) break;
                if (c.min_group > 0 && (!sharing || b->n_grouped == 0)) continue;  // not enabled / nothing to share
                if (!front_done) {
                    b->enqueue_front();
                    front_done = true;
                }
                cuda_check(cudaMemsetAsync(b->d_counters, 0, kCounters * sizeof(int), b->stream), "memset");
                b->enqueue_vertex();  // warm-up
                cuda_check(cudaEventRecord(e0, b->stream), "record");
                for (int r = 0; r < reps; ++r) {
                    cuda_check(cudaMemsetAsync(b->d_counters, 0, kCounters * sizeof(int), b->stream), "memset");
                    b->enqueue_vertex();
                }
                cuda_check(cudaEventRecord(e1, b->stream), "record");
                cuda_check(cudaEventSynchronize(e1), "sync");
                cuda_check(cudaGetLastError(), "autotune launch");
                float ms = 0.0f;
                cuda_check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
                ms /= float(reps);
                if (best_t < 0.0f || ms < best_t) {
                    best_t = ms;
                    best = c;
                }
            }
        } catch (...) {
            restore(keep);  // a failed candidate leaves the batch as it was
            throw;
        }
        restore(best);
        if (npi) *npi = best.npi;
        if (min_group) *min_group = best.min_group;
        if (cap_divisor) *cap_divisor = best.cap;
        if (best_ms) *best_ms = best_t;
    });
}

extern "C" int spn_batch_set_paused(spn_batch *b, int flow_id, int paused) {
    return guarded([&] {
        if (!b || flow_id < 0 || flow_id >= int(b->flows.size()) || !b->flows[flow_id].used)
            throw Error(ErrorType::Argument, "spn_batch_set_paused: unknown flow");
        spn_batch::Flow &f = b->flows[flow_id];
        if (f.paused != (paused != 0)) {
            f.paused = paused != 0;
            b->plan_valid = false;
        }
    });
}

extern "C" int spn_batch_grouped_flows(spn_batch *b, int *n_grouped) {
    return guarded([&] {
        if (!b || !n_grouped) throw Error(ErrorType::Argument, "null argument");
        cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
        if (!b->plan_valid) b->build_plan();
        *n_grouped = b->n_grouped;
    });
}

extern "C" int spn_batch_stats(spn_batch *b, long long *steps, long long *graph_builds, int *n_flows) {
    return guarded([&] {
        if (!b) throw Error(ErrorType::Argument, "null handle");
        if (steps) *steps = b->steps_run;
        if (graph_builds) *graph_builds = b->graph_builds;
        if (n_flows) {
            int n = 0;
            for (auto &f : b->flows) n += f.used;
            *n_flows = n;
        }
    });
}
