// GB300 (sm_103a) kernels of the SU(2) pf-FRG flow right-hand side and the device half of
// the C ABI in include/spn_su2.h.
//
// One flow's state lives in HBM in the reference layout (vertex index
// ((s(s+1)/2+u)*N + t)*Nl + rid, src/SU2/SU2VertexTwoParticle.hpp:603).  A compute step is
//   1. su2_self_energy_kernel   Sigma-dot(w_i), one CTA per frequency   (SU2FrgCore.cpp:139-169)
//   2. su2_node_table_kernel    per transfer frequency x: the loop-frequency nodes wp of the
//                               conventional (wp = +-Lambda) and Katanin (trapezoid) terms with
//                               their propagator x quadrature coefficients, in FP64
//                               (SU2FrgCore.cpp:336-424, Integrator.hpp:137-287)
//   3. su2_vertex_flow_kernel   Gamma-dot for every (s,t,u) triple (SU2FrgCore.cpp:171-431)
// and finalize_step is su2_euler_kernel (SU2FrgCore.cpp:111-137).
//
// Vertex-flow work distribution: a persistent grid whose warps pull triples from a device
// atomic counter (this replaces the reference's MPI/OpenMP LoadManager).  Inside a warp the
// lanes are split into G groups of W lanes: lane = (loop-frequency node group, lattice site),
// so each group evaluates one loop-frequency node for all Nl sites at once, the slab reads of
// a support are one coalesced segment, and the group results are combined with warp shuffles.
// The T-channel RPA lattice sum exchanges the per-site bubble values through shared memory.
// Accumulation over loop frequencies is Kahan-compensated FP32.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "su2_common.cuh"
#include "su2_device.cuh"
#include "su2_kernels.cuh"
#include "su2_handle.cuh"
#include "cuda_host.cuh"
#include "host/rpa_schedule.hpp"
#include "host/capi_common.hpp"
#include "../../include/spn_su2.h"

using namespace spn;
using namespace spn::dev;

namespace {

// ------------------------------------------------------------------------------------
// single-flow kernels (bodies in su2_kernels.cuh)
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) su2_self_energy_kernel(FlowArgs a) { self_energy_body(a, blockIdx.x); }

__global__ void su2_node_table_kernel(FlowArgs a) { node_table_body(a, blockIdx.x); }

template <int SPT>
__global__ void __launch_bounds__(128) su2_corr_inner_kernel(CorrArgs a) {
    corr_inner_body<SPT>(a, PairedState<float>{a.sd}, blockIdx.x);
}

// the allocation-free measurement: the caller's separate spin and density arrays
template <int SPT>
__global__ void __launch_bounds__(128) su2_corr_inner_split_kernel(CorrArgs a) {
    corr_inner_body<SPT>(a, SplitState<float>{a.ss, a.dd}, blockIdx.x);
}

__global__ void su2_corr_final_kernel(CorrArgs a) { corr_final_body(a); }

// FP64 flow (SPN_SU2_FP64): the same bodies in double
__global__ void __launch_bounds__(128) su2_self_energy_f64_kernel(FlowArgsT<double> a) { self_energy_body(a, blockIdx.x); }

__global__ void su2_node_table_f64_kernel(FlowArgsT<double> a) { node_table_body(a, blockIdx.x); }

template <int SPT>
__global__ void __launch_bounds__(128) su2_corr_inner_f64_kernel(CorrArgsT<double> a) {
    corr_inner_body<SPT>(a, PairedState<double>{a.sd}, blockIdx.x);
}

__global__ void su2_corr_final_f64_kernel(CorrArgsT<double> a) { corr_final_body(a); }

// ------------------------------------------------------------------------------------
// Euler step  x += step * dx  (rounded like the reference: product, then sum)
// ------------------------------------------------------------------------------------
__global__ void su2_euler_kernel(float *__restrict__ x, const float *__restrict__ dx, long long n, float step) {
    const long long n4 = n / 4;
    float4 *x4 = reinterpret_cast<float4 *>(x);
    const float4 *d4 = reinterpret_cast<const float4 *>(dx);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        float4 v = x4[i], d = __ldg(d4 + i);
        v.x = euler_update(v.x, d.x, step);
        v.y = euler_update(v.y, d.y, step);
        v.z = euler_update(v.z, d.z, step);
        v.w = euler_update(v.w, d.w, step);
        x4[i] = v;
    }
    for (long long i = 4 * n4 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = euler_update(x[i], dx[i], step);
}

// FP64 self-energy Euler step; keeps the FP32 mirror (what get_state returns) in sync.
__global__ void su2_euler_f64_kernel(double *__restrict__ x, const double *__restrict__ dx, float *__restrict__ xf, int n,
                                     float step) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = euler_update_f64(x[i], dx[i], step);
        x[i] = v;
        xf[i] = float(v);
    }
}

// State copies between the reference layout (two arrays: stage[0, n) spin, stage[n, 2n)
// density) and the device layout ((spin, density) per element).
__global__ void su2_pair_kernel(const float *__restrict__ stage, float2 *__restrict__ sd, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        sd[i] = make_float2(stage[i], stage[n + i]);
}
__global__ void su2_split_kernel(const float2 *__restrict__ sd, float *__restrict__ stage, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = sd[i];
        stage[i] = v.x;
        stage[n + i] = v.y;
    }
}

// Euler step of an FP64 flow: x += step * dx in double, step = new - old cutoff in double
// (the float cutoffs widened first).
__global__ void su2_euler_flow_f64_kernel(double *__restrict__ x, const double *__restrict__ dx, long long n, double step) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = euler_update_f64(x[i], dx[i], step);
}

// ------------------------------------------------------------------------------------
// FP32 FMA throughput probe: independent FMA chains, no memory traffic (the roofline
// denominator for the vertex-flow kernel, which runs on the FP32 CUDA cores).
// ------------------------------------------------------------------------------------
constexpr int kPeakChains = 8;
constexpr int kPeakIters = 4096;

__global__ void __launch_bounds__(256) fp32_peak_kernel(float *out, float seed) {
    float a[kPeakChains];
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) a[k] = seed + float(threadIdx.x + k);
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < kPeakIters; ++i) {
#pragma unroll
        for (int k = 0; k < kPeakChains; ++k) a[k] = fmaf(a[k], m, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) s += a[k];
    if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

// Gather probe: each warp sums, for kGatherK slabs read from a table, the segment of n_sites
// float2 pairs starting at slab * n_sites -- the slab gather of the vertex flow without its
// arithmetic.  Slab indices are < n_slabs and lane < n_sites, so every load is in bounds.
constexpr int kGatherK = 256;

__global__ void __launch_bounds__(128) gather_peak_kernel(const float2 *__restrict__ st, const int *__restrict__ slabs,
                                                          int n_sites, float *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int *sl = slabs + warp * kGatherK;
    float ax = 0.0f, ay = 0.0f;
    for (int k = 0; k < kGatherK; ++k) {
        const int s = __ldg(sl + k);
        if (lane < n_sites) {
            const float2 v = __ldg(st + (long long)s * n_sites + lane);
            ax += v.x;
            ay += v.y;
        }
    }
    if (ax + ay == 12345.678f) out[0] = ax;  // keeps the loads live
}

}  // namespace

// ------------------------------------------------------------------------------------
// host helpers (declared in su2_handle.cuh)
// ------------------------------------------------------------------------------------
namespace spn {

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(ErrorType::Cuda, std::string(what) + ": " + cudaGetErrorString(e));
}

int wsite_for(int nl) {
    if (nl > 32) return 32;
    int w = 1;
    while (w < nl) w <<= 1;
    return w;
}

int spt_for(int nl) { return nl <= 32 ? 1 : (nl <= 64 ? 2 : 4); }

}  // namespace spn

namespace {

template <class T>
T *dev_alloc(size_t count, const char *what) {
    void *p = nullptr;
    cuda_check(cudaMalloc(&p, count * sizeof(T) + 16), what);
    return static_cast<T *>(p);
}

template <class T>
void upload(T *dst, const T *src, size_t count, cudaStream_t s) {
    if (count) cuda_check(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync H2D");
}

float *stage_of(spn_su2 *h) {
    if (!h->stage) h->stage = dev_alloc<float>(2 * size_t(h->fn) * h->nl, "alloc state stage");
    return h->stage;
}

int copy_grid(long long n) { return int(std::min<long long>((n + 255) / 256, 4096)); }

void launch_vertex(spn_su2 *h) {
    if (h->fp64()) launch_vertex_flow_f64(h->args64(), h->vertex_grid, h->stream);
    else launch_vertex_flow(h->args(), h->vertex_npi, h->vertex_grid, h->stream);
    cuda_check(cudaGetLastError(), "vertex flow launch");
}

template <class T>
std::vector<T> download(const T *src, size_t count, cudaStream_t s) {
    std::vector<T> v(count);
    if (count) cuda_check(cudaMemcpyAsync(v.data(), src, count * sizeof(T), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(s), "D2H sync");
    return v;
}

// Copies n doubles from the device into float `out` (the float entry points of an FP64 flow).
void download_as_float(float *out, const double *src, size_t count, cudaStream_t s) {
    if (!out) return;
    std::vector<double> v = download(src, count, s);
    for (size_t i = 0; i < count; ++i) out[i] = float(v[i]);
}

// FP64 flows: (spin, density) pairs from / into separate host arrays (converted on the host).
template <class S>
void upload_pairs64(double2 *dst, const S *ss, const S *dd, size_t count, cudaStream_t s) {
    std::vector<double2> v(count);
    for (size_t i = 0; i < count; ++i) v[i] = make_double2(double(ss[i]), double(dd[i]));
    upload(dst, v.data(), count, s);
    cuda_check(cudaStreamSynchronize(s), "H2D sync");
}
template <class S>
void download_pairs64(S *ss, S *dd, const double2 *src, size_t count, cudaStream_t s) {
    if (!ss && !dd) return;
    const std::vector<double2> v = download(src, count, s);
    for (size_t i = 0; i < count; ++i) {
        if (ss) ss[i] = S(v[i].x);
        if (dd) dd[i] = S(v[i].y);
    }
}

// Selects a vertex-flow variant: nodes per iteration and where the RPA schedule lives (all
// variants give the same bits); the persistent grid fills every SM to the variant's
// occupancy.  Returns false if it cannot run.
bool select_variant(spn_su2 *h, int npi, int in_smem) {
    if (h->fp64()) {  // one FP64 kernel
        const int per_sm = vertex_flow_f64_blocks_per_sm(h->nl);
        cudaGetLastError();
        if (per_sm < 1 || npi != 1 || in_smem) return false;
        h->vertex_npi = 1;
        h->rpa_in_smem = 0;
        h->vertex_grid = h->sms * per_sm;
        return true;
    }
    if (in_smem) {
        RpaSchedule r = h->args().rpa;
        if (rpa_smem_ints(r, h->nl) > kRpaSmemMaxInts) return false;
    }
    const int old_smem = h->rpa_in_smem;
    h->rpa_in_smem = in_smem;
    const int per_sm = vertex_flow_blocks_per_sm(h->nl, h->args().rpa, npi);
    cudaGetLastError();
    if (per_sm < 1) {
        h->rpa_in_smem = old_smem;
        return false;
    }
    h->vertex_npi = npi;
    h->vertex_grid = h->sms * per_sm;
    return true;
}

void validate_desc(const spn_su2_desc *d) {
    if (!d) throw Error(ErrorType::Argument, "null descriptor");
    if (d->n_freq < 2 || d->n_freq > kMaxFreq)
        throw Error(ErrorType::Unsupported, "n_freq must be in [2, " + std::to_string(kMaxFreq) + "]");
    if (d->n_sites < 1 || d->n_sites > kMaxSites)
        throw Error(ErrorType::Unsupported, "n_sites must be in [1, " + std::to_string(kMaxSites) + "]");
    if (!d->freq || !d->sites_rid || !d->inv_sites_rid || !d->overlap_ptr || (d->n_range > 0 && (!d->range_rid || !d->range_inv_rid)) ||
        (d->n_corr > 0 && !d->corr_rid))
        throw Error(ErrorType::Argument, "descriptor table pointer is NULL");
    for (int i = 0; i < d->n_freq; ++i) {
        if (!(d->freq[i] > 0.0f)) throw Error(ErrorType::Argument, "frequencies must be positive");
        if (i > 0 && !(d->freq[i] > d->freq[i - 1])) throw Error(ErrorType::Argument, "frequencies must be strictly ascending");
    }
    const long long fn = (long long)d->n_freq * d->n_freq * (d->n_freq + 1) / 2;
    if (fn * d->n_sites >= (1ll << 31)) throw Error(ErrorType::Unsupported, "vertex larger than 2^31 elements");
    auto in_range = [&](const int *v, int cnt, int hi, const char *what) {
        for (int i = 0; i < cnt; ++i)
            if (v[i] < 0 || v[i] >= hi) throw Error(ErrorType::Argument, std::string(what) + " entry out of range");
    };
    in_range(d->sites_rid, d->n_sites, d->n_sites, "sites_rid");
    in_range(d->inv_sites_rid, d->n_sites, d->n_sites, "inv_sites_rid");
    if (d->overlap_ptr[0] != 0) throw Error(ErrorType::Argument, "overlap_ptr[0] must be 0");
    for (int r = 0; r < d->n_sites; ++r)
        if (d->overlap_ptr[r + 1] < d->overlap_ptr[r]) throw Error(ErrorType::Argument, "overlap_ptr must be non-decreasing");
    const int nov = d->overlap_ptr[d->n_sites];
    if (nov > 0 && (!d->overlap_rid1 || !d->overlap_rid2)) throw Error(ErrorType::Argument, "overlap pair table is NULL");
    in_range(d->overlap_rid1, nov, d->n_sites, "overlap_rid1");
    in_range(d->overlap_rid2, nov, d->n_sites, "overlap_rid2");
    in_range(d->range_rid, d->n_range, d->n_sites, "range_rid");
    in_range(d->range_inv_rid, d->n_range, d->n_sites, "range_inv_rid");
    in_range(d->corr_rid, d->n_corr, d->n_sites, "corr_rid");
}

}  // namespace

extern "C" int spn_device_count(int *count) {
    return guarded([&] {
        if (!count) throw Error(ErrorType::Argument, "null count");
        int c = 0;
        if (cudaGetDeviceCount(&c) != cudaSuccess) c = 0;
        cudaGetLastError();
        *count = c;
    });
}

extern "C" int spn_device_memory(int device, long long *free_bytes, long long *total_bytes) {
    return guarded([&] {
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        size_t f = 0, t = 0;
        cuda_check(cudaMemGetInfo(&f, &t), "cudaMemGetInfo");
        if (free_bytes) *free_bytes = (long long)f;
        if (total_bytes) *total_bytes = (long long)t;
    });
}

extern "C" int spn_measure_fp32_peak(int device, double *tflops, double *sm_clock_ghz_est) {
    return guarded([&] {
        if (!tflops) throw Error(ErrorType::Argument, "null output");
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        int sms = 0;
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device attribute");
        float *out = nullptr;
        cuda_check(cudaMalloc(&out, sizeof(float)), "alloc");
        cudaEvent_t e0, e1;
        cuda_check(cudaEventCreate(&e0), "event");
        cuda_check(cudaEventCreate(&e1), "event");
        const int blocks = sms * 8, threads = 256;
        double best = 0.0;
        for (int rep = 0; rep < 6; ++rep) {
            cuda_check(cudaEventRecord(e0), "record");
            fp32_peak_kernel<<<blocks, threads>>>(out, 1.0f + rep);
            cuda_check(cudaEventRecord(e1), "record");
            cuda_check(cudaEventSynchronize(e1), "sync");
            float ms = 0.0f;
            cuda_check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            const double flops = 2.0 * double(blocks) * threads * kPeakChains * kPeakIters;
            if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(out);
        *tflops = best;
        // 128 FP32 lanes x 2 flops per SM per clock
        if (sm_clock_ghz_est) *sm_clock_ghz_est = best * 1e12 / (double(sms) * 256.0) / 1e9;
    });
}

namespace {
// Bucket index of an ascending positive mesh (dev::MeshIndex): the smallest shift that puts the
// bit patterns of pos[0] .. pos[n-1] into kMeshBuckets buckets, and per bucket the first index
// >= 1 whose mesh value lies at or above the bucket's start.
struct MeshBuckets {
    std::vector<unsigned short> lo;
    unsigned base = 0;
    int shift = 0;
};
MeshBuckets mesh_buckets(const float *pos, int n) {
    auto bits = [](float x) { unsigned u; std::memcpy(&u, &x, sizeof u); return u; };
    MeshBuckets m;
    m.base = bits(pos[0]);
    const unsigned span = bits(pos[n - 1]) - m.base;
    while ((span >> m.shift) >= unsigned(kMeshBuckets)) ++m.shift;
    m.lo.assign(kMeshBuckets, 0);
    int i = 0;
    for (int b = 0; b < kMeshBuckets; ++b) {
        const unsigned long long start = (unsigned long long)m.base + ((unsigned long long)b << m.shift);
        while (i < n && (unsigned long long)bits(pos[i]) < start) ++i;
        m.lo[size_t(b)] = (unsigned short)std::max(1, i);
    }
    return m;
}

// The state of a diagnostic read: the two arrays of the reference's layout on the host.
struct HostState {
    const float *ss, *dd;
    __host__ __device__ float spin(int i) const { return ss[i]; }
    __host__ __device__ float density(int i) const { return dd[i]; }
};

void check_mesh(const float *pos, int n) { cuh::check_mesh(pos, n, kMaxFreq); }

// The emitter of spn_quadrature_nodes: the first cap nodes into (wp, weight), k counts all.
struct NodeList {
    float *wp;
    double *weight;
    int cap, k;
    __host__ __device__ void operator()(float x, double c) {
        if (k < cap) {
            wp[k] = x;
            weight[k] = c;
        }
        ++k;
    }
};
}  // namespace

extern "C" int spn_mesh_probe(const float *pos, int n, float w, float *lesser, float *greater, int *offset, int *lo,
                              int *hi, float *bias) {
    return guarded([&] {
        check_mesh(pos, n);
        if (lesser) *lesser = dev::full_value(pos, n, dev::full_lesser(pos, n, w));
        if (greater) *greater = dev::full_value(pos, n, dev::full_greater(pos, n, w));
        const float a = w < 0.0f ? -w : w;
        if (offset) *offset = dev::mesh_offset(pos, n, a);
        int l = 0, h = 0;
        float b = 0.0f;
        dev::mesh_interp(pos, n, a, l, h, b);
        if (lo) *lo = l;
        if (hi) *hi = h;
        if (bias) *bias = b;
    });
}

extern "C" int spn_mesh_index_check(const float *pos, int n, const float *w, int count, int *mismatches) {
    return guarded([&] {
        check_mesh(pos, n);
        if (count < 0 || (count > 0 && !w) || !mismatches) throw Error(ErrorType::Argument, "spn_mesh_index_check: bad argument");
        const MeshBuckets mb = mesh_buckets(pos, n);
        const dev::MeshIndex mi{pos, n, mb.lo.data(), mb.base, mb.shift};
        const dev::MeshSearch<float> ms{pos, n};
        int bad = 0;
        for (int k = 0; k < count; ++k)
            if (mi.first_greater(w[k]) != ms.first_greater(w[k]) || mi.first_geq(w[k]) != ms.first_geq(w[k])) ++bad;
        *mismatches = bad;
    });
}

extern "C" int spn_vertex_probe(const float *pos, int n, int n_sites, const float *ss, const float *dd, int rid12,
                                int rid21, float s, float t, float u, int channel, int density, float *value) {
    return guarded([&] {
        check_mesh(pos, n);
        if (n_sites < 1 || n_sites > kMaxSites || !ss || !dd || !value || rid12 < 0 || rid12 >= n_sites || rid21 < 0 ||
            rid21 >= n_sites || channel < -1 || channel > 3)
            throw Error(ErrorType::Argument, "spn_vertex_probe: bad argument");
        const HostState v{ss, dd};
        if (channel < 0) {
            *value = dev::value_none(pos, n, n_sites, v, density != 0, rid12, rid21, s, t, u);
            return;
        }
        auto read = [&](const int *off, const float *w, const float *sw, bool exch, int q) {
            const int site = exch ? rid21 : rid12;
            float g = 0.0f;
            for (int k = 0; k < q; ++k) g += (density ? sw[k] : w[k]) * (density ? v.density(off[k] + site) : v.spin(off[k] + site));
            return g;
        };
        const dev::MeshSearch<float> m{pos, n};
        if (channel == 3) {
            dev::AB8 ab;
            dev::access8(pos, n, n_sites, s, t, u, ab);
            *value = read(ab.off, ab.w, ab.sw, ab.exch, 8);
            return;
        }
        dev::AB4 ab;
        if (channel == 0) dev::access4m<dev::kS>(m, n_sites, s, t, u, ab);
        else if (channel == 1) dev::access4m<dev::kT>(m, n_sites, s, t, u, ab);
        else dev::access4m<dev::kU>(m, n_sites, s, t, u, ab);
        *value = read(ab.off, ab.w, ab.sw, ab.exch, 4);
    });
}

extern "C" int spn_self_energy_probe(const float *pos, int n, const float *data, float w, double *value) {
    return guarded([&] {
        check_mesh(pos, n);
        if (!data || !value) throw Error(ErrorType::Argument, "spn_self_energy_probe: bad argument");
        *value = dev::odd_interp(pos, n, data, w);
    });
}

extern "C" int spn_quadrature_nodes(const float *pos, int n, int rule, float min, float max, float *wp, double *weight,
                                    int cap, int *count) {
    return guarded([&] {
        check_mesh(pos, n);
        if (rule < 0 || rule > 2 || !count || cap < 0 || (cap > 0 && (!wp || !weight)))
            throw Error(ErrorType::Argument, "spn_quadrature_nodes: bad argument");
        NodeList emit{wp, weight, cap, 0};
        if (rule == 0) dev::nodes_left(pos, n, min, emit);
        else if (rule == 1) dev::nodes_right(pos, n, max, emit);
        else dev::nodes_both(pos, n, min, max, emit);
        *count = emit.k;
    });
}

extern "C" int spn_measure_gather_peak(int device, int n_sites, int n_slabs, double *segments_per_s) {
    return guarded([&] {
        if (!segments_per_s || n_sites < 1 || n_sites > 32 || n_slabs < 1)
            throw Error(ErrorType::Argument, "spn_measure_gather_peak: need 1 <= n_sites <= 32 and n_slabs >= 1");
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        int sms = 0;
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device attribute");
        const int threads = 128, blocks = sms * 16;
        const long long warps = (long long)blocks * threads / 32;
        std::vector<int> table(size_t(warps) * kGatherK);
        unsigned x = 12345u;
        for (auto &t : table) {
            x = x * 1664525u + 1013904223u;
            t = int((x >> 8) % unsigned(n_slabs));
        }
        float2 *st = nullptr;
        int *sl = nullptr;
        float *out = nullptr;
        cuda_check(cudaMalloc(&st, size_t(n_slabs) * n_sites * sizeof(float2)), "alloc");
        cuda_check(cudaMalloc(&sl, table.size() * sizeof(int)), "alloc");
        cuda_check(cudaMalloc(&out, sizeof(float)), "alloc");
        cuda_check(cudaMemset(st, 0, size_t(n_slabs) * n_sites * sizeof(float2)), "memset");
        cuda_check(cudaMemcpy(sl, table.data(), table.size() * sizeof(int), cudaMemcpyHostToDevice), "H2D");
        cudaEvent_t e0, e1;
        cuda_check(cudaEventCreate(&e0), "event");
        cuda_check(cudaEventCreate(&e1), "event");
        double best = 0.0;
        for (int rep = 0; rep < 6; ++rep) {
            cuda_check(cudaEventRecord(e0), "record");
            gather_peak_kernel<<<blocks, threads>>>(st, sl, n_sites, out);
            cuda_check(cudaEventRecord(e1), "record");
            cuda_check(cudaEventSynchronize(e1), "sync");
            float ms = 0.0f;
            cuda_check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            if (rep > 0) best = std::max(best, double(warps) * kGatherK / (ms * 1e-3));
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(st);
        cudaFree(sl);
        cudaFree(out);
        *segments_per_s = best;
    });
}

spn_su2 *spn::create_flow(const spn_su2_desc *d, cudaStream_t stream) {
        validate_desc(d);
        auto *h = new spn_su2;
        try {
            h->device = d->device;
            cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
            h->n = d->n_freq;
            h->nl = d->n_sites;
            h->fn = (long long)h->n * h->n * (h->n + 1) / 2;
            h->n_range = d->n_range;
            h->n_corr = d->n_corr;
            h->n_overlap = d->overlap_ptr[d->n_sites];
            h->flags = d->flags;
            h->spin = d->spin_length;
            h->max_nodes = 2 * h->n + 8;
            if (stream) {
                h->stream = stream;
                h->own_stream = false;
            } else {
                cuda_check(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate");
                h->own_stream = true;
            }
            const size_t vsz = size_t(h->fn) * h->nl;
            const bool f64 = h->fp64();
            h->freq = dev_alloc<float>(h->n, "alloc freq");
            h->v2 = dev_alloc<float>(h->n, "alloc v2");
            h->dv2 = dev_alloc<float>(h->n, "alloc dv2");
            h->v2d = dev_alloc<double>(h->n, "alloc v2 (fp64)");
            h->dv2d = dev_alloc<double>(h->n, "alloc dv2 (fp64)");
            if (f64) {
                h->freq64 = dev_alloc<double>(h->n, "alloc freq (fp64)");
                h->sd64 = dev_alloc<double2>(vsz, "alloc vertex state (fp64)");
                h->dsd64 = dev_alloc<double2>(vsz, "alloc vertex flow (fp64)");
                h->node_wp64 = dev_alloc<double>(size_t(h->n) * h->max_nodes, "alloc node table (fp64)");
                h->node_c64 = dev_alloc<double>(size_t(h->n) * h->max_nodes, "alloc node table (fp64)");
                h->corr_out64 = dev_alloc<double>(2 * size_t(h->n_corr) + 2 * h->nl, "alloc corr out (fp64)");
                std::vector<double> f(d->freq, d->freq + h->n);
                upload(h->freq64, f.data(), h->n, h->stream);
                cuda_check(cudaMemsetAsync(h->sd64, 0, vsz * sizeof(double2), h->stream), "memset");
                cuda_check(cudaMemsetAsync(h->dsd64, 0, vsz * sizeof(double2), h->stream), "memset");
                cuda_check(cudaStreamSynchronize(h->stream), "create sync");  // f leaves scope
            } else {
                h->sd = dev_alloc<float2>(vsz, "alloc vertex state");
                h->dsd = dev_alloc<float2>(vsz, "alloc vertex flow");
                h->node_wp = dev_alloc<float>(size_t(h->n) * h->max_nodes, "alloc node table");
                h->node_c = dev_alloc<float>(size_t(h->n) * h->max_nodes, "alloc node table");
                cuda_check(cudaMemsetAsync(h->sd, 0, vsz * sizeof(float2), h->stream), "memset");
                cuda_check(cudaMemsetAsync(h->dsd, 0, vsz * sizeof(float2), h->stream), "memset");
            }
            h->node_cnt = dev_alloc<int>(h->n, "alloc node counts");
            h->work_counter = dev_alloc<int>(1, "alloc work counter");
            h->status = dev_alloc<unsigned>(1, "alloc status");
            h->sites = dev_alloc<int>(h->nl, "alloc sites");
            h->inv_sites = dev_alloc<int>(h->nl, "alloc inv sites");
            h->ov_ptr = dev_alloc<int>(h->nl + 1, "alloc overlap ptr");
            h->ov_r1 = dev_alloc<int>(h->n_overlap + 1, "alloc overlap");
            h->ov_r2 = dev_alloc<int>(h->n_overlap + 1, "alloc overlap");
            h->range_rid = dev_alloc<int>(h->n_range + 1, "alloc range");
            h->range_inv = dev_alloc<int>(h->n_range + 1, "alloc range");
            h->corr_rid = dev_alloc<int>(h->n_corr + 1, "alloc corr map");
            h->corr_partial = dev_alloc<double>(size_t(kMaxCorrNodes) * 2 * h->nl, "alloc corr scratch");
            if (!f64) h->corr_out = dev_alloc<float>(2 * size_t(h->n_corr) + 2 * h->nl, "alloc corr out");
            upload(h->freq, d->freq, h->n, h->stream);
            {
                const MeshBuckets mb = mesh_buckets(d->freq, h->n);
                h->mesh_lo = dev_alloc<unsigned short>(kMeshBuckets, "alloc mesh index");
                upload(h->mesh_lo, mb.lo.data(), kMeshBuckets, h->stream);
                h->mesh_base = mb.base;
                h->mesh_shift = mb.shift;
                cuda_check(cudaStreamSynchronize(h->stream), "mesh index sync");  // mb leaves scope
            }
            upload(h->sites, d->sites_rid, h->nl, h->stream);
            upload(h->inv_sites, d->inv_sites_rid, h->nl, h->stream);
            upload(h->ov_ptr, d->overlap_ptr, h->nl + 1, h->stream);
            upload(h->ov_r1, d->overlap_rid1, h->n_overlap, h->stream);
            upload(h->ov_r2, d->overlap_rid2, h->n_overlap, h->stream);
            upload(h->range_rid, d->range_rid, h->n_range, h->stream);
            upload(h->range_inv, d->range_inv_rid, h->n_range, h->stream);
            upload(h->corr_rid, d->corr_rid, h->n_corr, h->stream);
            cuda_check(cudaMemsetAsync(h->v2, 0, h->n * sizeof(float), h->stream), "memset");
            cuda_check(cudaMemsetAsync(h->dv2, 0, h->n * sizeof(float), h->stream), "memset");
            cuda_check(cudaMemsetAsync(h->v2d, 0, h->n * sizeof(double), h->stream), "memset");
            cuda_check(cudaMemsetAsync(h->dv2d, 0, h->n * sizeof(double), h->stream), "memset");
            cuda_check(cudaMemsetAsync(h->status, 0, sizeof(unsigned), h->stream), "memset");
            // RPA schedule balanced over the lanes that walk it (a warp's 32, or the 128 or 256
            // threads of the CTA-per-triple kernel above 32 sites)
            RpaHostSchedule rpa = build_rpa_schedule(h->nl, d->overlap_ptr, d->overlap_rid1, d->overlap_rid2,
                                                     vertex_rpa_lanes(h->nl));
            h->rpa_lanes = rpa.lanes;
            h->rpa_n_seg = rpa.n_seg;
            h->rpa_len = rpa.len;
            // one image in the staged layout (what the kernel copies to shared memory in one bulk
            // transfer), padded to 16 bytes
            std::vector<int> image(rpa.sched);
            image.insert(image.end(), rpa.count.begin(), rpa.count.end());
            image.insert(image.end(), rpa.slot_base.begin(), rpa.slot_base.end());
            image.insert(image.end(), rpa.seg_ptr.begin(), rpa.seg_ptr.end());
            image.resize((image.size() + 3) / 4 * 4, 0);
            h->rpa_image = dev_alloc<int>(image.size(), "alloc rpa schedule");
            upload(h->rpa_image, image.data(), image.size(), h->stream);
            h->rpa_image_bytes = int(image.size() * sizeof(int));
            h->rpa_sched = h->rpa_image;
            h->rpa_count = h->rpa_sched + rpa.sched.size();
            h->rpa_slot_base = h->rpa_count + rpa.count.size();
            h->rpa_seg_ptr = h->rpa_slot_base + rpa.slot_base.size();
            // persistent vertex grid: every SM filled to its occupancy limit
            int sms = 0;
            cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device), "device attribute");
            h->sms = sms;
            // default variant (schedule staged in shared memory where it fits); spn_su2_autotune
            // can pick a faster one for this flow
            if (!select_variant(h, 1, f64 ? 0 : 1) && !select_variant(h, 1, 0))
                throw Error(ErrorType::Unsupported, "vertex-flow kernel does not fit on this device");
            cuda_check(cudaStreamSynchronize(h->stream), "create sync");
        } catch (...) {
            h->release();
            delete h;
            throw;
        }
        return h;
}

extern "C" int spn_su2_create(const spn_su2_desc *d, spn_su2 **out) {
    return guarded([&] {
        if (!out) throw Error(ErrorType::Argument, "null output handle");
        *out = create_flow(d, nullptr);
    });
}

extern "C" int spn_su2_destroy(spn_su2 *h) {
    if (!h) return SPN_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->release();
    delete h;
    return SPN_OK;
}

extern "C" int spn_su2_set_stream(spn_su2 *h, void *stream) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(h->stream), "stream sync");
        if (stream) {
            if (h->own_stream) cudaStreamDestroy(h->stream);
            h->stream = static_cast<cudaStream_t>(stream);
            h->own_stream = false;
        } else if (!h->own_stream) {
            cuda_check(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate");
            h->own_stream = true;
        }
    });
}

extern "C" int spn_su2_get_sizes(const spn_su2 *h, int *n_freq, int *n_sites, long long *n_triples) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        if (n_freq) *n_freq = h->n;
        if (n_sites) *n_sites = h->nl;
        if (n_triples) *n_triples = h->fn;
    });
}

extern "C" int spn_su2_set_state(spn_su2 *h, float cutoff, const float *v2, const float *v4ss, const float *v4dd) {
    return guarded([&] {
        if (!h || !v2 || !v4ss || !v4dd) throw Error(ErrorType::Argument, "null argument");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        const size_t vsz = size_t(h->fn) * h->nl;
        upload(h->v2, v2, h->n, h->stream);
        if (h->fp64()) upload_pairs64(h->sd64, v4ss, v4dd, vsz, h->stream);
        else upload_state(h, v4ss, v4dd, stage_of(h), h->stream);
        std::vector<double> v2d(v2, v2 + h->n);  // the FP64 self-energy starts from the given values
        upload(h->v2d, v2d.data(), h->n, h->stream);
        h->cutoff = cutoff;
        cuda_check(cudaStreamSynchronize(h->stream), "set_state sync");
    });
}

extern "C" int spn_su2_get_state(spn_su2 *h, float *cutoff, float *v2, float *v4ss, float *v4dd) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        const size_t vsz = size_t(h->fn) * h->nl;
        if (cutoff) *cutoff = h->cutoff;
        if (h->fp64()) {
            download_as_float(v2, h->v2d, h->n, h->stream);
            download_pairs64(v4ss, v4dd, h->sd64, vsz, h->stream);
            return;
        }
        if (v2) cuda_check(cudaMemcpyAsync(v2, h->v2, h->n * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        download_state(h, h->sd, v4ss, v4dd, stage_of(h), h->stream);
        cuda_check(cudaStreamSynchronize(h->stream), "get_state sync");
    });
}

extern "C" int spn_su2_set_cutoff(spn_su2 *h, float cutoff) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        h->cutoff = cutoff;
    });
}

extern "C" int spn_su2_get_node_counts(spn_su2 *h, int *counts) {
    return guarded([&] {
        if (!h || !counts) throw Error(ErrorType::Argument, "null argument");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        cuda_check(cudaMemcpyAsync(counts, h->node_cnt, h->n * sizeof(int), cudaMemcpyDeviceToHost, h->stream), "D2H");
        cuda_check(cudaStreamSynchronize(h->stream), "node count sync");
    });
}

extern "C" int spn_su2_compute_step(spn_su2 *h) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        int e0 = -1, e1 = -1, e2 = -1;
        if (h->profiling) {
            e0 = h->event();
            cuda_check(cudaEventRecord(h->ev_pool[e0], h->stream), "event record");
        }
        cuda_check(cudaMemsetAsync(h->status, 0, sizeof(unsigned), h->stream), "memset status");
        cuda_check(cudaMemsetAsync(h->work_counter, 0, sizeof(int), h->stream), "memset counter");
        if (h->fp64()) {
            const FlowArgsT<double> a = h->args64();
            su2_self_energy_f64_kernel<<<h->n, 128, 0, h->stream>>>(a);
            cuda_check(cudaGetLastError(), "self-energy launch");
            su2_node_table_f64_kernel<<<(h->n + 63) / 64, 64, 0, h->stream>>>(a);
            cuda_check(cudaGetLastError(), "node table launch");
        } else {
            const FlowArgs a = h->args();
            su2_self_energy_kernel<<<h->n, 128, 0, h->stream>>>(a);
            cuda_check(cudaGetLastError(), "self-energy launch");
            su2_node_table_kernel<<<(h->n + 63) / 64, 64, 0, h->stream>>>(a);
            cuda_check(cudaGetLastError(), "node table launch");
        }
        if (h->profiling) {
            e1 = h->event();
            cuda_check(cudaEventRecord(h->ev_pool[e1], h->stream), "event record");
        }
        launch_vertex(h);
        if (h->profiling) {
            e2 = h->event();
            cuda_check(cudaEventRecord(h->ev_pool[e2], h->stream), "event record");
            h->ev_vertex.emplace_back(e1, e2);
            h->ev_step.emplace_back(e0, e2);
        }
    });
}

extern "C" int spn_su2_set_variant(spn_su2 *h, int npi, int sched_in_smem) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        if (npi != 1 && npi != 2) throw Error(ErrorType::Argument, "nodes per iteration must be 1 or 2");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        if (h->fp64() && (npi != 1 || sched_in_smem))
            throw Error(ErrorType::Unsupported, "an FP64 flow has one vertex-flow kernel (npi 1, schedule in global memory)");
        if (!select_variant(h, npi, sched_in_smem ? 1 : 0))
            throw Error(ErrorType::Unsupported, "vertex-flow variant does not fit on this device for this lattice");
    });
}

extern "C" int spn_su2_autotune(spn_su2 *h, int reps, int *npi, int *sched_in_smem, int *grid) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        reps = std::max(1, std::min(reps, 16));
        if (h->fp64()) {  // nothing to choose
            if (npi) *npi = h->vertex_npi;
            if (sched_in_smem) *sched_in_smem = h->rpa_in_smem;
            if (grid) *grid = h->vertex_grid;
            return;
        }
        cudaEvent_t e0, e1;
        cuda_check(cudaEventCreate(&e0), "event");
        cuda_check(cudaEventCreate(&e1), "event");
        const bool prof = h->profiling;
        h->profiling = false;
        float best = 0.0f;
        int best_npi = h->vertex_npi, best_smem = h->rpa_in_smem;
        try {
            // the node tables of the current cutoff (compute_step leaves the state untouched)
            cuda_check(spn_su2_compute_step(h) == 0 ? cudaSuccess : cudaErrorUnknown, "autotune step");
            for (int npi = 1; npi <= 2; ++npi)
                for (int sm = 0; sm <= 1; ++sm) {
                    if (!select_variant(h, npi, sm)) continue;
                    std::vector<float> ms;
                    for (int r = 0; r <= reps; ++r) {
                        cuda_check(cudaMemsetAsync(h->work_counter, 0, sizeof(int), h->stream), "memset counter");
                        cuda_check(cudaEventRecord(e0, h->stream), "record");
                        launch_vertex(h);
                        cuda_check(cudaEventRecord(e1, h->stream), "record");
                        cuda_check(cudaEventSynchronize(e1), "sync");
                        float t = 0.0f;
                        cuda_check(cudaEventElapsedTime(&t, e0, e1), "elapsed");
                        if (r > 0) ms.push_back(t);  // first launch warms caches
                    }
                    std::sort(ms.begin(), ms.end());
                    const float med = ms[ms.size() / 2];
                    if (best == 0.0f || med < best) {
                        best = med;
                        best_npi = npi;
                        best_smem = sm;
                    }
                }
        } catch (...) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            h->profiling = prof;
            throw;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        h->profiling = prof;
        if (!select_variant(h, best_npi, best_smem)) throw Error(ErrorType::Internal, "autotune: chosen variant unavailable");
        if (npi) *npi = h->vertex_npi;
        if (sched_in_smem) *sched_in_smem = h->rpa_in_smem;
        if (grid) *grid = h->vertex_grid;
    });
}

extern "C" int spn_su2_get_flow(spn_su2 *h, float *dv2, float *dv4ss, float *dv4dd) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        const size_t vsz = size_t(h->fn) * h->nl;
        if (h->fp64()) {
            download_as_float(dv2, h->dv2d, h->n, h->stream);
            download_pairs64(dv4ss, dv4dd, h->dsd64, vsz, h->stream);
            return;
        }
        if (dv2) cuda_check(cudaMemcpyAsync(dv2, h->dv2, h->n * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        download_state(h, h->dsd, dv4ss, dv4dd, stage_of(h), h->stream);
        cuda_check(cudaStreamSynchronize(h->stream), "get_flow sync");
    });
}

extern "C" int spn_su2_finalize_step(spn_su2 *h, float new_cutoff) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        const float step = new_cutoff - h->cutoff;
        const long long vsz = h->fn * h->nl;
        if (h->fp64()) {
            const double step64 = double(new_cutoff) - double(h->cutoff);
            su2_euler_flow_f64_kernel<<<1, 64, 0, h->stream>>>(h->v2d, h->dv2d, h->n, step64);
            su2_euler_flow_f64_kernel<<<copy_grid(2 * vsz), 256, 0, h->stream>>>(
                reinterpret_cast<double *>(h->sd64), reinterpret_cast<const double *>(h->dsd64), 2 * vsz, step64);
            cuda_check(cudaGetLastError(), "euler launch");
            h->cutoff = new_cutoff;
            return;
        }
        if (h->flags & SPN_SU2_FP64_SELF_ENERGY)
            su2_euler_f64_kernel<<<1, 64, 0, h->stream>>>(h->v2d, h->dv2d, h->v2, h->n, step);
        else
            su2_euler_kernel<<<1, 64, 0, h->stream>>>(h->v2, h->dv2, h->n, step);
        // the (spin, density) arrays are updated as one array of 2 F_N Nl floats
        const int grid = int(std::min<long long>((2 * vsz / 4 + 255) / 256 + 1, 4096));
        su2_euler_kernel<<<grid, 256, 0, h->stream>>>(reinterpret_cast<float *>(h->sd), reinterpret_cast<const float *>(h->dsd),
                                                      2 * vsz, step);
        cuda_check(cudaGetLastError(), "euler launch");
        h->cutoff = new_cutoff;
    });
}

namespace {

}  // namespace

void spn::upload_state(spn_su2 *h, const float *v4ss, const float *v4dd, float *stage, cudaStream_t stream) {
    const size_t vsz = size_t(h->fn) * h->nl;
    upload(stage, v4ss, vsz, stream);
    upload(stage + vsz, v4dd, vsz, stream);
    su2_pair_kernel<<<copy_grid((long long)vsz), 256, 0, stream>>>(stage, h->sd, (long long)vsz);
    cuda_check(cudaGetLastError(), "state pair launch");
}

void spn::download_state(const spn_su2 *h, const float2 *src, float *v4ss, float *v4dd, float *stage, cudaStream_t stream) {
    if (!v4ss && !v4dd) return;
    const size_t vsz = size_t(h->fn) * h->nl;
    su2_split_kernel<<<copy_grid((long long)vsz), 256, 0, stream>>>(src, stage, (long long)vsz);
    cuda_check(cudaGetLastError(), "state split launch");
    if (v4ss) cuda_check(cudaMemcpyAsync(v4ss, stage, vsz * sizeof(float), cudaMemcpyDeviceToHost, stream), "D2H");
    if (v4dd) cuda_check(cudaMemcpyAsync(v4dd, stage + vsz, vsz * sizeof(float), cudaMemcpyDeviceToHost, stream), "D2H");
}

CorrArgs spn::corr_args(const spn_su2 *h) {
        CorrArgs a;
        a.n = h->n;
        a.nl = h->nl;
        a.n_corr = h->n_corr;
        a.cutoff = h->cutoff;
        a.spin = h->spin;
        a.freq = h->freq;
        a.sd = h->sd;
        a.ss = nullptr;
        a.dd = nullptr;
        a.v2 = h->v2;
        a.v2d = (h->flags & SPN_SU2_FP64_SELF_ENERGY) ? h->v2d : nullptr;
        a.sites = h->sites;
        a.inv_sites = h->inv_sites;
        a.corr_rid = h->corr_rid;
        a.partial = h->corr_partial;
        a.out = h->corr_out;
        a.wsite = wsite_for(h->nl);
        return a;
}

namespace {

CorrArgsT<double> corr_args64(const spn_su2 *h) {
        const CorrArgs f = corr_args(h);
        CorrArgsT<double> a;
        a.n = f.n;
        a.nl = f.nl;
        a.n_corr = f.n_corr;
        a.cutoff = f.cutoff;
        a.spin = f.spin;
        a.freq = h->freq64;
        a.sd = h->sd64;
        a.ss = nullptr;
        a.dd = nullptr;
        a.v2 = h->v2d;
        a.v2d = nullptr;
        a.sites = f.sites;
        a.inv_sites = f.inv_sites;
        a.corr_rid = f.corr_rid;
        a.partial = f.partial;
        a.out = h->corr_out64;
        a.wsite = f.wsite;
        return a;
}

void launch_correlation(spn_su2 *h) {
        if (h->fp64()) {
            const CorrArgsT<double> a = corr_args64(h);
            const int spt = spt_for(h->nl);
            const int blocks = 2 * h->n + 4;
            if (spt == 1) su2_corr_inner_f64_kernel<1><<<blocks, 128, 0, h->stream>>>(a);
            else if (spt == 2) su2_corr_inner_f64_kernel<2><<<blocks, 128, 0, h->stream>>>(a);
            else su2_corr_inner_f64_kernel<4><<<blocks, 128, 0, h->stream>>>(a);
            cuda_check(cudaGetLastError(), "correlation launch");
            su2_corr_final_f64_kernel<<<1, 128, 2 * h->nl * sizeof(double), h->stream>>>(a);
            cuda_check(cudaGetLastError(), "correlation final launch");
            return;
        }
        const CorrArgs a = corr_args(h);
        const int spt = spt_for(h->nl);
        const int blocks = 2 * h->n + 4;
        if (spt == 1) su2_corr_inner_kernel<1><<<blocks, 128, 0, h->stream>>>(a);
        else if (spt == 2) su2_corr_inner_kernel<2><<<blocks, 128, 0, h->stream>>>(a);
        else su2_corr_inner_kernel<4><<<blocks, 128, 0, h->stream>>>(a);
        cuda_check(cudaGetLastError(), "correlation launch");
        su2_corr_final_kernel<<<1, 128, 2 * h->nl * sizeof(double), h->stream>>>(a);
        cuda_check(cudaGetLastError(), "correlation final launch");
}

void copy_correlation(spn_su2 *h, float *zz, float *dd, float *chi_zz, float *chi_dd) {
        if (h->fp64()) {
            const std::vector<double> v = download(h->corr_out64, 2 * size_t(h->n_corr) + 2 * h->nl, h->stream);
            auto put = [&](float *out, size_t off, int cnt) {
                if (out)
                    for (int i = 0; i < cnt; ++i) out[i] = float(v[off + i]);
            };
            put(zz, 0, h->n_corr);
            put(dd, h->n_corr, h->n_corr);
            put(chi_zz, 2 * size_t(h->n_corr), h->nl);
            put(chi_dd, 2 * size_t(h->n_corr) + h->nl, h->nl);
            return;
        }
        if (zz) cuda_check(cudaMemcpyAsync(zz, h->corr_out, h->n_corr * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        if (dd)
            cuda_check(cudaMemcpyAsync(dd, h->corr_out + h->n_corr, h->n_corr * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        if (chi_zz)
            cuda_check(cudaMemcpyAsync(chi_zz, h->corr_out + 2 * h->n_corr, h->nl * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        if (chi_dd)
            cuda_check(cudaMemcpyAsync(chi_dd, h->corr_out + 2 * h->n_corr + h->nl, h->nl * sizeof(float), cudaMemcpyDeviceToHost, h->stream),
                       "D2H");
        cuda_check(cudaStreamSynchronize(h->stream), "correlation sync");
}

}  // namespace

extern "C" int spn_su2_measure_correlation(spn_su2 *h, float *zz, float *dd, float *chi_zz, float *chi_dd) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        launch_correlation(h);
        copy_correlation(h, zz, dd, chi_zz, chi_dd);
    });
}

// ---- double-precision data movement of an FP64 flow ----
namespace {
void require_fp64(const spn_su2 *h) {
    if (!h) throw Error(ErrorType::Argument, "null handle");
    if (!h->fp64()) throw Error(ErrorType::Unsupported, "the flow was not created with SPN_SU2_FP64");
}
}  // namespace

extern "C" int spn_su2_set_state_f64(spn_su2 *h, float cutoff, const double *v2, const double *v4ss, const double *v4dd) {
    return guarded([&] {
        require_fp64(h);
        if (!v2 || !v4ss || !v4dd) throw Error(ErrorType::Argument, "null argument");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        const size_t vsz = size_t(h->fn) * h->nl;
        upload(h->v2d, v2, h->n, h->stream);
        upload_pairs64(h->sd64, v4ss, v4dd, vsz, h->stream);
        h->cutoff = cutoff;
        cuda_check(cudaStreamSynchronize(h->stream), "set_state sync");
    });
}

extern "C" int spn_su2_get_state_f64(spn_su2 *h, float *cutoff, double *v2, double *v4ss, double *v4dd) {
    return guarded([&] {
        require_fp64(h);
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        const size_t vsz = size_t(h->fn) * h->nl;
        if (cutoff) *cutoff = h->cutoff;
        if (v2) cuda_check(cudaMemcpyAsync(v2, h->v2d, h->n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H");
        download_pairs64(v4ss, v4dd, h->sd64, vsz, h->stream);
        cuda_check(cudaStreamSynchronize(h->stream), "get_state sync");
    });
}

extern "C" int spn_su2_get_flow_f64(spn_su2 *h, double *dv2, double *dv4ss, double *dv4dd) {
    return guarded([&] {
        require_fp64(h);
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        const size_t vsz = size_t(h->fn) * h->nl;
        if (dv2) cuda_check(cudaMemcpyAsync(dv2, h->dv2d, h->n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H");
        download_pairs64(dv4ss, dv4dd, h->dsd64, vsz, h->stream);
        cuda_check(cudaStreamSynchronize(h->stream), "get_flow sync");
    });
}

extern "C" int spn_su2_measure_correlation_f64(spn_su2 *h, double *zz, double *dd, double *chi_zz, double *chi_dd) {
    return guarded([&] {
        require_fp64(h);
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        launch_correlation(h);
        const std::vector<double> v = download(h->corr_out64, 2 * size_t(h->n_corr) + 2 * h->nl, h->stream);
        auto put = [&](double *out, size_t off, int cnt) {
            if (out) std::copy(v.begin() + off, v.begin() + off + cnt, out);
        };
        put(zz, 0, h->n_corr);
        put(dd, h->n_corr, h->n_corr);
        put(chi_zz, 2 * size_t(h->n_corr), h->nl);
        put(chi_dd, 2 * size_t(h->n_corr) + h->nl, h->nl);
    });
}

extern "C" int spn_su2_launch_correlation(spn_su2 *h) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        launch_correlation(h);
    });
}

extern "C" int spn_su2_get_correlation(spn_su2 *h, float *zz, float *dd, float *chi_zz, float *chi_dd) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        copy_correlation(h, zz, dd, chi_zz, chi_dd);
    });
}

extern "C" int spn_su2_is_diverged(spn_su2 *h, int *diverged) {
    return guarded([&] {
        if (!h || !diverged) throw Error(ErrorType::Argument, "null argument");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        unsigned st = 0;
        cuda_check(cudaMemcpyAsync(&st, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream), "D2H");
        cuda_check(cudaStreamSynchronize(h->stream), "status sync");
        if (st & kStatusNodeOverflow) throw Error(ErrorType::Device, "loop-frequency node table overflow");
        *diverged = (st & kStatusNaN) ? 1 : 0;
    });
}

extern "C" int spn_su2_synchronize(spn_su2 *h) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
    });
}

extern "C" int spn_su2_set_profiling(spn_su2 *h, int enable) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(h->stream), "stream sync");
        for (auto e : h->ev_pool) cudaEventDestroy(e);
        h->ev_pool.clear();
        h->ev_vertex.clear();
        h->ev_step.clear();
        h->profiling = enable != 0;
    });
}

extern "C" int spn_su2_get_profile(spn_su2 *h, double *vertex_ms, int *vertex_launches, double *step_ms, int *steps) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        cuda_check(cudaSetDevice(h->device), "cudaSetDevice");
        cuda_check(cudaStreamSynchronize(h->stream), "stream sync");
        double vm = 0.0, sm = 0.0;
        for (auto &p : h->ev_vertex) {
            float ms = 0.0f;
            cuda_check(cudaEventElapsedTime(&ms, h->ev_pool[p.first], h->ev_pool[p.second]), "elapsed");
            vm += ms;
        }
        for (auto &p : h->ev_step) {
            float ms = 0.0f;
            cuda_check(cudaEventElapsedTime(&ms, h->ev_pool[p.first], h->ev_pool[p.second]), "elapsed");
            sm += ms;
        }
        if (vertex_ms) *vertex_ms = vm;
        if (vertex_launches) *vertex_launches = int(h->ev_vertex.size());
        if (step_ms) *step_ms = sm;
        if (steps) *steps = int(h->ev_step.size());
    });
}

// ------------------------------------------------------------------------------------
// Allocation-free correlation measurement
//
// Some callers cannot allocate device memory when they want a measurement: a host framework
// that reserves the GPU's memory up front in its own pool (a cudaMalloc from this library
// would fail or bypass the pool's accounting), or a time-critical loop that must not enter the
// CUDA allocator (cudaMalloc/cudaFree can synchronise the device and take driver locks).  For
// them spn_su2_correlation_noalloc runs the same two measurement kernels as
// spn_su2_measure_correlation, with the per-node partial sums in the fixed array below instead
// of memory owned by a flow handle.  The caller passes every input and the output in device
// memory it already owns; this entry point allocates nothing.
//
// The array holds (2 * kMaxFreq + 8) x 2 x kMaxSites doubles (1 064 960 bytes) and is
// resident on every GPU that loads the library until the process exits.  It is shared by all
// calls on a device and keeps the contents of the last call; no entry needs clearing, because
// the first kernel writes every partial sum the second kernel reads.  Two calls whose work
// overlaps on the GPU (different streams, no ordering between them) race on it.
// ------------------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) double g_corr_scratch[size_t(kMaxCorrNodes) * 2 * kMaxSites];

// Device address of g_corr_scratch per device.  In host code the array's name is only a
// host-side stand-in, so the address is looked up once per device with that device current.
// The cache is never invalidated: after a cudaDeviceReset() the address belongs to a context
// that no longer exists (the header tells callers not to use this entry point after a reset).
double *g_corr_scratch_addr[kNoAllocMaxDevices] = {};

double *corr_scratch_for_current_device() {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kNoAllocMaxDevices) throw Error(ErrorType::Unsupported, "device ordinal beyond 63");
    double *p = __atomic_load_n(&g_corr_scratch_addr[dev], __ATOMIC_ACQUIRE);
    if (!p) {
        void *addr = nullptr;
        cuda_check(cudaGetSymbolAddress(&addr, g_corr_scratch), "cudaGetSymbolAddress(g_corr_scratch)");
        p = static_cast<double *>(addr);
        __atomic_store_n(&g_corr_scratch_addr[dev], p, __ATOMIC_RELEASE);
    }
    return p;
}

}  // namespace

extern "C" int spn_su2_correlation_noalloc(int n_freq, const float *freq, int n_sites, const int *sites_rid,
                                           const int *inv_sites_rid, int n_corr, const int *corr_rid, float spin_length,
                                           float cutoff, const float *v2, const float *v4ss, const float *v4dd, float *out,
                                           void *stream) {
    return guarded([&] {
        if (n_freq < 2 || n_freq > kMaxFreq)
            throw Error(ErrorType::Unsupported, "spn_su2_correlation_noalloc: n_freq must be in [2, " +
                                                    std::to_string(kMaxFreq) + "] (fixed scratch size)");
        if (n_sites < 1 || n_sites > kMaxSites)
            throw Error(ErrorType::Unsupported, "spn_su2_correlation_noalloc: n_sites must be in [1, " +
                                                    std::to_string(kMaxSites) + "] (fixed scratch size)");
        if (n_corr < 0) throw Error(ErrorType::Argument, "spn_su2_correlation_noalloc: n_corr must be >= 0");
        if (!freq || !sites_rid || !inv_sites_rid || (n_corr > 0 && !corr_rid) || !v2 || !v4ss || !v4dd || !out)
            throw Error(ErrorType::Argument, "spn_su2_correlation_noalloc: null device pointer");
        CorrArgs a;
        a.n = n_freq;
        a.nl = n_sites;
        a.n_corr = n_corr;
        a.cutoff = cutoff;
        a.spin = spin_length;
        a.freq = freq;
        a.sd = nullptr;
        a.ss = v4ss;
        a.dd = v4dd;
        a.v2 = v2;
        a.v2d = nullptr;
        a.sites = sites_rid;
        a.inv_sites = inv_sites_rid;
        a.corr_rid = corr_rid;
        a.partial = corr_scratch_for_current_device();
        a.out = out;
        a.wsite = wsite_for(n_sites);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const int spt = spt_for(n_sites);
        const int blocks = 2 * n_freq + 4;
        if (spt == 1) su2_corr_inner_split_kernel<1><<<blocks, 128, 0, s>>>(a);
        else if (spt == 2) su2_corr_inner_split_kernel<2><<<blocks, 128, 0, s>>>(a);
        else su2_corr_inner_split_kernel<4><<<blocks, 128, 0, s>>>(a);
        cuda_check(cudaGetLastError(), "correlation launch");
        su2_corr_final_kernel<<<1, 128, 2 * n_sites * sizeof(double), s>>>(a);
        cuda_check(cudaGetLastError(), "correlation final launch");
    });
}
