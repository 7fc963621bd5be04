// GB300 kernels of the XYZ pf-FRG flow right-hand side (models with diagonal, possibly
// anisotropic couplings: Heisenberg-Kitaev, XXZ, ...) and the device half of the spn_xyz_* C
// ABI in include/spn_su2.h.  Restates XYZFrgCore (src/XYZ/XYZFrgCore.cpp:161-570), the XYZ
// vertex access (src/XYZ/XYZVertexTwoParticle.hpp:185-612) and XYZMeasurementCorrelation
// (src/XYZ/XYZMeasurementCorrelation.cpp:98-184).
//
// The vertex has four components per element, X, Y, Z and density D, stored as one float4
// per element ((s(s+1)/2+u)*N + t)*Nl + rid, so an interpolation support is one 16-byte load.
// A lattice symmetry map may permute X, Y, Z: site j of the superbundle reads component
// perm[p_j][c] of its representative, and each RPA pair carries the permutations of its two
// factors (spn_lattice_get_spin_tables).
//
// A step: the self-energy flow (one CTA per frequency), the loop-frequency node tables (the
// SU(2) core's, shared), the vertex flow and the Euler update.  The vertex-flow kernel runs a
// persistent grid whose warps take one (s,t,u) triple at a time from a device counter.  Per
// channel, nodes go in batches of 16: first a lane builds one node's access buffers (and
// the t channel's site-local values) into a shared-memory descriptor, then the lanes hold
// the sites (up to four each) and walk the batch's nodes in order.  The t channel's RPA sum
// exchanges the first two slabs of a node through shared memory in all six spin
// permutations, so a pair (rid1, rid2, perm1, perm2) is two 16-byte loads and four FMAs.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include "su2_common.cuh"
#include "su2_device.cuh"
#include "su2_kernels.cuh"
#include "cuda_host.cuh"
#include "host/capi_common.hpp"
#include "host/pair_order.hpp"
#include "../../include/spn_su2.h"

using namespace spn;
using namespace spn::dev;

namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kSpt = 4;  // sites per lane at most (Nl <= 128); the vertex kernel takes 1, 2 or 4
constexpr int X = 0, Y = 1, Z = 2, D = 3;

// The six spin permutations (X,Y,Z) (X,Z,Y) (Y,X,Z) (Y,Z,X) (Z,X,Y) (Z,Y,X): 2 bits per image
// component, 6 bits per permutation.
constexpr unsigned long long kPermBits =
    36ull | (24ull << 6) | (33ull << 12) | (9ull << 18) | (18ull << 24) | (6ull << 30);
__host__ __device__ __forceinline__ int perm_c(int p, int c) { return int((kPermBits >> (6 * p + 2 * c)) & 3ull); }

SPN_HDI float comp_of(const float4 &v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w)); }

struct XyzArgs {
    int n, nl, fn, max_nodes, n_range, n_corr;
    float cutoff;
    const float *freq;
    const float4 *sd;  // state
    float4 *dsd;       // flow
    const float *v2;
    float *dv2;
    const int *sites, *sites_perm, *inv_sites, *inv_sites_perm;
    // the t channel's RPA pairs of all sites in one lane-balanced walk (lane_schedule): entry i
    // of lane l is sched[32 i + l], the pair's word rid1 | rid2 << 7 | perm1 << 14 | perm2 << 17
    // (order_rpa_pairs) with bit 20 set on the last entry of a site's run in the lane; count[l]
    // entries; the runs' partial sums go to slots slot_base[l], ... and site j sums slots
    // seg_ptr[j] .. seg_ptr[j + 1] - 1
    const int *rpa_sched, *rpa_count, *rpa_slot_base, *rpa_seg_ptr;
    int rpa_n_seg;
    const int *range_rid, *range_inv;
    const float *node_wp, *node_c;
    const int *node_cnt;
    int *work_counter;
    unsigned *status;
    const int *corr_rid, *corr_perm;
    double *partial;  // [kMaxCorrNodes][4][nl]
    float *out;       // [4][n_corr] correlations, then chi [4][nl]
};

// One component of the state for value_none (su2_device.cuh): c < 3 reads X, Y or Z (its
// "spin" accessor), c == 3 the density (with the density's sign on an s <-> u swap).
struct QuadComp {
    const float4 *v;
    int c;
    SPN_HDI float spin(int i) const { return comp_of(ro_load(v + i), c); }
    SPN_HDI float density(int i) const { return ro_load(v + i).w; }
};

SPN_HDI float value4(const float *pos, const XyzArgs &a, int c, int rid12, int rid21, float s, float t, float u) {
    return value_none(pos, a.n, a.nl, QuadComp{a.sd, c}, c == D, rid12, rid21, s, t, u);
}

// ------------------------------------------------------------------------------------
// self-energy flow, one CTA per frequency (XYZFrgCore.cpp:161-194)
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) xyz_self_energy_kernel(XyzArgs a) {
    __shared__ float pos[kMaxFreq];
    __shared__ double red[4];
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    const int i = blockIdx.x;
    const float w = pos[i], L = a.cutoff;
    const float wpl = w + L, wml = w - L;
    double part = 0.0;
    for (int j = threadIdx.x; j < a.n_range; j += blockDim.x) {
        const int r12 = a.range_rid[j], r21 = a.range_inv[j];
        part += double(value4(pos, a, D, r12, r21, wpl, 0.0f, wml)) - double(value4(pos, a, D, r12, r21, wml, 0.0f, wpl));
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int k = 0; k < int(blockDim.x >> 5); ++k) sum += red[k];
        double val = -2.0 * sum;
        for (int c = 0; c < 4; ++c)
            val += double(value4(pos, a, c, 0, 0, wpl, wml, 0.0f)) - double(value4(pos, a, c, 0, 0, wml, wpl, 0.0f));
        val /= (2.0 * kPiD * (double(L) + odd_interp(pos, a.n, a.v2, L)));
        const float outv = float(val);
        a.dv2[i] = outv;
        if (isnan(outv)) atomicOr(a.status, kStatusNaN);
    }
}

// Loop-frequency node tables: the SU(2) core's body on an argument block of this flow.
__global__ void xyz_node_table_kernel(FlowArgs f) { node_table_body(f, blockIdx.x); }

// ------------------------------------------------------------------------------------
// vertex flow
// ------------------------------------------------------------------------------------
template <int SPT>
struct LaneT {
    int j[SPT], rid[SPT], prm[SPT], irid[SPT], iprm[SPT];
    bool valid[SPT];
};
using Lane4 = LaneT<kSpt>;

// Interpolated slab of one access buffer for the lane's sites (getValueSuperbundle): X, Y, Z
// of site j read the permuted components of its representative, D the signed density.  The
// four supports are summed per stored component (one fused multiply-add each) and the sums
// permuted once, instead of selecting a permuted component of every support.
template <int SPT>
SPN_HDI void gather4(const XyzArgs &a, const AB4 &ab, const LaneT<SPT> &ln, float4 *out) {
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (ln.valid[k]) {
            const int r = ab.exch ? ln.irid[k] : ln.rid[k];
            const int p = ab.exch ? ln.iprm[k] : ln.prm[k];
            float4 h = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 v = ro_load(a.sd + ab.off[q] + r);
                h.x += ab.w[q] * v.x;
                h.y += ab.w[q] * v.y;
                h.z += ab.w[q] * v.z;
                h.w += ab.sw[q] * v.w;
            }
            g = make_float4(comp_of(h, perm_c(p, 0)), comp_of(h, perm_c(p, 1)), comp_of(h, perm_c(p, 2)), h.w);
        }
        out[k] = g;
    }
}

// getValueLocal of the four components at rid 0 (identity permutation).
SPN_HDI float4 local4(const XyzArgs &a, const AB4 &ab) {
    float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float4 v = ro_load(a.sd + ab.off[q]);
        g.x += ab.w[q] * v.x;
        g.y += ab.w[q] * v.y;
        g.z += ab.w[q] * v.z;
        g.w += ab.sw[q] * v.w;
    }
    return g;
}

// The products of a pair of slabs (a, b) in the s integrand: per component (D,c) and (c,D)
// added, the two others crossed and subtracted (XYZFrgCore.cpp:230-261).
__device__ __forceinline__ float4 s_terms(const float4 &a, const float4 &b) {
    float4 r;
    r.x = a.w * b.x + a.x * b.w - a.z * b.y - a.y * b.z;
    r.y = a.w * b.y + a.y * b.w - a.z * b.x - a.x * b.z;
    r.z = a.w * b.z + a.z * b.w - a.x * b.y - a.y * b.x;
    r.w = a.w * b.w + a.x * b.x + a.y * b.y + a.z * b.z;
    return r;
}

// The u integrand subtracts all four products of every component (XYZFrgCore.cpp:436-469):
// the cross terms keep the sign of the others, unlike the s integrand.
__device__ __forceinline__ float4 u_terms(const float4 &a, const float4 &b) {
    float4 r;
    r.x = -(a.w * b.x + a.x * b.w + a.z * b.y + a.y * b.z);
    r.y = -(a.w * b.y + a.y * b.w + a.z * b.x + a.x * b.z);
    r.z = -(a.w * b.z + a.z * b.w + a.x * b.y + a.y * b.x);
    r.w = -(a.w * b.w + a.x * b.x + a.y * b.y + a.z * b.z);
    return r;
}

// v with X, Y, Z replaced by components perm[p][0..2] of v (density unchanged).
template <int P>
__device__ __forceinline__ float4 permuted(const float4 &v) {
    constexpr int c0 = int((kPermBits >> (6 * P)) & 3ull), c1 = int((kPermBits >> (6 * P + 2)) & 3ull),
                  c2 = int((kPermBits >> (6 * P + 4)) & 3ull);
    return make_float4(comp_of(v, c0), comp_of(v, c1), comp_of(v, c2), v.w);
}

// Node descriptor (lane = node in phase A): the four access buffers of the node and, for the
// t channel, the four site-local values (getValueLocal of ab4..ab7, four components each).
struct __align__(16) XDesc {
    int4 off[4];
    float4 w[4], sw[4];
    float4 lv[4];
    int exch;  // bit i: buffer i reads the site-exchanged pairs
    float c;   // node coefficient
    int pad[2];
};

__device__ __forceinline__ void put_desc(XDesc &d, int i, const AB4 &ab) {
    d.off[i] = make_int4(ab.off[0], ab.off[1], ab.off[2], ab.off[3]);
    d.w[i] = make_float4(ab.w[0], ab.w[1], ab.w[2], ab.w[3]);
    d.sw[i] = make_float4(ab.sw[0], ab.sw[1], ab.sw[2], ab.sw[3]);
}

// Phase A: the descriptor of one node of channel ch (0 = s, 1 = t, 2 = u).  The channel's own
// coordinate is a mesh value, so its offset is the triple's index e.
__device__ __forceinline__ void make_xdesc(const XyzArgs &a, const float *pos, int ch, int e, float s, float t, float u,
                                           float w1p, float w1, float w2p, float w2, float wp, float c, XDesc &d) {
    const MeshSearch<float> m{pos, a.n};
    const int nl = a.nl, n = a.n;
    AB4 ab;
    int ex = 0;
    // each pair of buffers interpolates two of the node's four distinct magnitudes (a
    // coordinate and its negation fold alike; -a - b is bitwise -(a + b))
    if (ch == 0) {  // integralKernelS, XYZFrgCore.cpp:218-224
        {
            const Interp<float> iA = interp_abs(m, w1 + wp), iB = interp_abs(m, w2 + wp);
            access4i<kS>(n, nl, s, -w1 - wp, -w2 - wp, iA, iB, e, ab); put_desc(d, 0, ab); ex |= ab.exch << 0;
            access4i<kS>(n, nl, s, w2 + wp, w1 + wp, iB, iA, e, ab); put_desc(d, 2, ab); ex |= ab.exch << 2;
        }
        {
            const Interp<float> iP = interp_abs(m, w1p + wp), iQ = interp_abs(m, w2p + wp);
            access4i<kS>(n, nl, s, w1p + wp, -w2p - wp, iP, iQ, e, ab); put_desc(d, 1, ab); ex |= ab.exch << 1;
            access4i<kS>(n, nl, s, -w2p - wp, w1p + wp, iQ, iP, e, ab); put_desc(d, 3, ab); ex |= ab.exch << 3;
        }
    } else if (ch == 1) {  // integralKernelT, XYZFrgCore.cpp:268-276, 323-345
        {
            const Interp<float> iC = interp_abs(m, w1 - wp), iP = interp_abs(m, w1p + wp);
            access4i<kT>(n, nl, w1 - wp, t, w1p + wp, iC, iP, e, ab); put_desc(d, 0, ab); ex |= ab.exch << 0;
            access4i<kT>(n, nl, w1p + wp, t, w1 - wp, iP, iC, e, ab); put_desc(d, 2, ab); ex |= ab.exch << 2;
            access4i<kU>(n, nl, w1 - wp, -w1p - wp, -t, iC, iP, e, ab); d.lv[1] = local4(a, ab);
            access4i<kU>(n, nl, w1p + wp, wp - w1, -t, iP, iC, e, ab); d.lv[3] = local4(a, ab);
        }
        {
            const Interp<float> iD = interp_abs(m, w2p - wp), iB = interp_abs(m, w2 + wp);
            access4i<kT>(n, nl, w2p - wp, t, -w2 - wp, iD, iB, e, ab); put_desc(d, 1, ab); ex |= ab.exch << 1;
            access4i<kT>(n, nl, w2 + wp, t, wp - w2p, iB, iD, e, ab); put_desc(d, 3, ab); ex |= ab.exch << 3;
            access4i<kU>(n, nl, w2p - wp, -w2 - wp, t, iD, iB, e, ab); d.lv[0] = local4(a, ab);
            access4i<kU>(n, nl, w2 + wp, wp - w2p, t, iB, iD, e, ab); d.lv[2] = local4(a, ab);
        }
    } else {  // integralKernelU, XYZFrgCore.cpp:424-430
        {
            const Interp<float> iA = interp_abs(m, w1 + wp), iD = interp_abs(m, w2p - wp);
            access4i<kU>(n, nl, w1 + wp, wp - w2p, u, iA, iD, e, ab); put_desc(d, 0, ab); ex |= ab.exch << 0;
            access4i<kU>(n, nl, w2p - wp, -w1 - wp, u, iD, iA, e, ab); put_desc(d, 2, ab); ex |= ab.exch << 2;
        }
        {
            const Interp<float> iP = interp_abs(m, w1p + wp), iE = interp_abs(m, w2 - wp);
            access4i<kU>(n, nl, w1p + wp, w2 - wp, u, iP, iE, e, ab); put_desc(d, 1, ab); ex |= ab.exch << 1;
            access4i<kU>(n, nl, w2 - wp, w1p + wp, u, iE, iP, e, ab); put_desc(d, 3, ab); ex |= ab.exch << 3;
        }
    }
    d.exch = ex;
    d.c = c;
}

// Phase B gather of buffer i of a descriptor (see gather4).
template <int SPT>
__device__ __forceinline__ void gather_desc(const XyzArgs &a, const XDesc &d, int i, const LaneT<SPT> &ln, float4 *out) {
    AB4 ab;
    const int4 o = d.off[i];
    const float4 w = d.w[i], sw = d.sw[i];
    ab.off[0] = o.x; ab.off[1] = o.y; ab.off[2] = o.z; ab.off[3] = o.w;
    ab.w[0] = w.x; ab.w[1] = w.y; ab.w[2] = w.z; ab.w[3] = w.w;
    ab.sw[0] = sw.x; ab.sw[1] = sw.y; ab.sw[2] = sw.z; ab.sw[3] = sw.w;
    ab.exch = (d.exch >> i) & 1;
    gather4(a, ab, ln, out);
}

constexpr int kXBatch = 4;  // nodes whose descriptors a warp builds at once

template <int SPT>
__global__ void __launch_bounds__(kThreads) xyz_vertex_kernel(XyzArgs a) {
    __shared__ float pos[kMaxFreq];
    // per warp: kXBatch node descriptors, then the first two t slabs of every site in all six
    // spin permutations, A6[p][nl] and B6[p][nl], then the RPA walk's run partials
    extern __shared__ float4 xs[];
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = a.n, nl = a.nl;
    const int warp_f4 = kXBatch * int(sizeof(XDesc) / sizeof(float4)) + 12 * nl + a.rpa_n_seg;
    XDesc *desc = reinterpret_cast<XDesc *>(xs + size_t(warp) * warp_f4);
    float4 *A6 = xs + size_t(warp) * warp_f4 + kXBatch * (sizeof(XDesc) / sizeof(float4)), *B6 = A6 + 6 * nl;
    float4 *slots = B6 + 6 * nl;
    const int rpa_cnt = a.rpa_count[lane], rpa_base = a.rpa_slot_base[lane];
    LaneT<SPT> ln;
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        const int j = lane + 32 * k;
        ln.j[k] = j;
        ln.valid[k] = j < nl;
        ln.rid[k] = ln.valid[k] ? a.sites[j] : 0;
        ln.prm[k] = ln.valid[k] ? a.sites_perm[j] : 0;
        ln.irid[k] = ln.valid[k] ? a.inv_sites[j] : 0;
        ln.iprm[k] = ln.valid[k] ? a.inv_sites_perm[j] : 0;
    }
    const float two_pi = 2.0f * float(kPiD);

    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.work_counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= a.fn) break;
        const int su = it / n, ti = it - su * n;
        int si = int((sqrtf(8.0f * float(su) + 1.0f) - 1.0f) * 0.5f);
        while (si * (si + 1) / 2 > su) --si;
        while ((si + 1) * (si + 2) / 2 <= su) ++si;
        const int ui = su - si * (si + 1) / 2;
        const float s = pos[si], t = pos[ti], u = pos[ui];
        const float w1p = 0.5f * (s + t + u), w1 = 0.5f * (s - t + u), w2p = 0.5f * (s - t - u), w2 = 0.5f * (s + t - u);

        float4 acc[SPT];
#pragma unroll
        for (int k = 0; k < SPT; ++k) acc[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int ch = 0; ch < 3; ++ch) {
            const int xi = ch == 0 ? si : (ch == 1 ? ti : ui);
            const int cnt = a.node_cnt[xi];
            const float *nwp = a.node_wp + size_t(xi) * a.max_nodes;
            const float *nc = a.node_c + size_t(xi) * a.max_nodes;
            for (int b0 = 0; b0 < cnt; b0 += kXBatch) {
                const int nb = min(kXBatch, cnt - b0);
                if (lane < nb)  // phase A: lane = node
                    make_xdesc(a, pos, ch, xi, s, t, u, w1p, w1, w2p, w2, nwp[b0 + lane], nc[b0 + lane], desc[lane]);
                __syncwarp();
                for (int b = 0; b < nb; ++b) {  // phase B: lane = site
                    const XDesc &d = desc[b];
                    float4 S0[SPT], S1[SPT], S2[SPT], S3[SPT], r[SPT];
                    gather_desc(a, d, 0, ln, S0);
                    gather_desc(a, d, 1, ln, S1);
                    gather_desc(a, d, 2, ln, S2);
                    gather_desc(a, d, 3, ln, S3);
                    if (ch == 0) {  // XYZFrgCore.cpp:229-261
#pragma unroll
                        for (int k = 0; k < SPT; ++k) {
                            const float4 p = s_terms(S0[k], S1[k]), q = s_terms(S2[k], S3[k]);
                            r[k] = make_float4(p.x + q.x, p.y + q.y, p.z + q.z, p.w + q.w);
                        }
                    } else if (ch == 2) {  // XYZFrgCore.cpp:436-469
#pragma unroll
                        for (int k = 0; k < SPT; ++k) {
                            const float4 p = u_terms(S0[k], S1[k]), q = u_terms(S2[k], S3[k]);
                            r[k] = make_float4(p.x + q.x, p.y + q.y, p.z + q.z, p.w + q.w);
                        }
                    } else {  // t channel: RPA over the first two slabs of all sites, then local terms
#pragma unroll
                        for (int k = 0; k < SPT; ++k)
                            if (ln.valid[k]) {
                                const int j = ln.j[k];
                                A6[0 * nl + j] = permuted<0>(S0[k]);
                                A6[1 * nl + j] = permuted<1>(S0[k]);
                                A6[2 * nl + j] = permuted<2>(S0[k]);
                                A6[3 * nl + j] = permuted<3>(S0[k]);
                                A6[4 * nl + j] = permuted<4>(S0[k]);
                                A6[5 * nl + j] = permuted<5>(S0[k]);
                                B6[0 * nl + j] = permuted<0>(S1[k]);
                                B6[1 * nl + j] = permuted<1>(S1[k]);
                                B6[2 * nl + j] = permuted<2>(S1[k]);
                                B6[3 * nl + j] = permuted<3>(S1[k]);
                                B6[4 * nl + j] = permuted<4>(S1[k]);
                                B6[5 * nl + j] = permuted<5>(S1[k]);
                            }
                        __syncwarp();
                        const float4 cb = d.lv[0], ica = d.lv[1], cb2 = d.lv[2], ica2 = d.lv[3];
                        const float cbv[4] = {cb.x, cb.y, cb.z, cb.w}, icav[4] = {ica.x, ica.y, ica.z, ica.w};
                        const float cb2v[4] = {cb2.x, cb2.y, cb2.z, cb2.w}, ica2v[4] = {ica2.x, ica2.y, ica2.z, ica2.w};
                        {  // RPA (XYZFrgCore.cpp:282-305): every site's pairs in one lane-balanced walk
                            float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                            int slot = rpa_base;
                            for (int i = 0; i < rpa_cnt; ++i) {
                                const int e = __ldg(a.rpa_sched + 32 * i + lane);
                                const float4 x1 = A6[((e >> 14) & 7) * nl + (e & 127)];
                                const float4 x2 = B6[((e >> 17) & 7) * nl + ((e >> 7) & 127)];
                                p.x += x1.x * x2.x;
                                p.y += x1.y * x2.y;
                                p.z += x1.z * x2.z;
                                p.w += x1.w * x2.w;
                                if (e & (1 << 20)) {
                                    slots[slot++] = p;
                                    p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                                }
                            }
                        }
                        __syncwarp();
#pragma unroll
                        for (int k = 0; k < SPT; ++k) {
                            float rp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                            if (ln.valid[k]) {  // the site's run partials, in order
                                for (int q = a.rpa_seg_ptr[ln.j[k]]; q < a.rpa_seg_ptr[ln.j[k] + 1]; ++q) {
                                    const float4 v = slots[q];
                                    rp[0] += v.x;
                                    rp[1] += v.y;
                                    rp[2] += v.z;
                                    rp[3] += v.w;
                                }
                            }
                            const float a0[4] = {S0[k].x, S0[k].y, S0[k].z, S0[k].w};
                            const float a1[4] = {S1[k].x, S1[k].y, S1[k].z, S1[k].w};
                            const float a2[4] = {S2[k].x, S2[k].y, S2[k].z, S2[k].w};
                            const float a3[4] = {S3[k].x, S3[k].y, S3[k].z, S3[k].w};
                            float rv[4];
#pragma unroll
                            for (int cc = 0; cc < 3; ++cc) {  // XYZFrgCore.cpp:347-401
                                const int pA = cc == X ? Y : X, pB = cc == Z ? Y : Z;
                                const int qA = cc == Z ? X : Z, qB = cc == X ? Y : (cc == Y ? X : Y);
                                float v = 4.0f * rp[cc];
                                v -= a0[cc] * cbv[D];
                                v += a0[cc] * cbv[pA];
                                v += a0[cc] * cbv[pB];
                                v -= a0[cc] * cbv[cc];
                                v -= icav[D] * a1[cc];
                                v += icav[qA] * a1[cc];
                                v += icav[qB] * a1[cc];
                                v -= icav[cc] * a1[cc];
                                v -= a2[cc] * cb2v[D];
                                v += a2[cc] * cb2v[pA];
                                v += a2[cc] * cb2v[pB];
                                v -= a2[cc] * cb2v[cc];
                                v -= ica2v[D] * a3[cc];
                                v += ica2v[qA] * a3[cc];
                                v += ica2v[qB] * a3[cc];
                                v -= ica2v[cc] * a3[cc];
                                rv[cc] = v;
                            }
                            {  // XYZFrgCore.cpp:402-417
                                float v = 4.0f * rp[D];
                                v -= a0[D] * cbv[D];
                                v -= a0[D] * cbv[X];
                                v -= a0[D] * cbv[Y];
                                v -= a0[D] * cbv[Z];
                                v -= icav[D] * a1[D];
                                v -= icav[X] * a1[D];
                                v -= icav[Y] * a1[D];
                                v -= icav[Z] * a1[D];
                                v -= a2[D] * cb2v[D];
                                v -= a2[D] * cb2v[X];
                                v -= a2[D] * cb2v[Y];
                                v -= a2[D] * cb2v[Z];
                                v -= ica2v[D] * a3[D];
                                v -= ica2v[X] * a3[D];
                                v -= ica2v[Y] * a3[D];
                                v -= ica2v[Z] * a3[D];
                                rv[D] = v;
                            }
                            r[k] = make_float4(rv[0], rv[1], rv[2], rv[3]);
                        }
                        __syncwarp();
                    }
                    const float c = d.c;
#pragma unroll
                    for (int k = 0; k < SPT; ++k) {
                        acc[k].x += c * r[k].x;
                        acc[k].y += c * r[k].y;
                        acc[k].z += c * r[k].z;
                        acc[k].w += c * r[k].w;
                    }
                }
                __syncwarp();
            }
        }
#pragma unroll
        for (int k = 0; k < SPT; ++k)
            if (ln.valid[k]) {
                const float4 o = make_float4(acc[k].x / two_pi, acc[k].y / two_pi, acc[k].z / two_pi, acc[k].w / two_pi);
                a.dsd[size_t(it) * nl + ln.j[k]] = o;
                if (isnan(o.x) || isnan(o.y) || isnan(o.z) || isnan(o.w)) atomicOr(a.status, kStatusNaN);
            }
    }
}

// ------------------------------------------------------------------------------------
// correlation measurement at nu = 0 (XYZMeasurementCorrelation.cpp:98-184): one CTA per
// outer node accumulates the inner integral per site in FP64, a final CTA adds the outer
// weights and the on-site term and scatters to (basis, site in range) entries.
// ------------------------------------------------------------------------------------
// getValueSuperbundle through a trilinear buffer for one site: X, Y, Z the components of the
// representative r under permutation p, D the signed density.
SPN_HDI void bundle8(const XyzArgs &a, const AB8 &ab, int r, int p, float g[4]) {
    g[0] = g[1] = g[2] = g[3] = 0.0f;
    for (int q = 0; q < 8; ++q) {
        const float4 v = ro_load(a.sd + ab.off[q] + r);
        for (int c = 0; c < 3; ++c) g[c] += ab.w[q] * comp_of(v, perm_c(p, c));
        g[3] += ab.sw[q] * v.w;
    }
}

__global__ void __launch_bounds__(128) xyz_corr_inner_kernel(XyzArgs a) {
    __shared__ float pos[kMaxFreq];
    __shared__ float nwp[kMaxCorrNodes];
    __shared__ double nw[kMaxCorrNodes];
    __shared__ int ncnt;
    __shared__ double red[kWarps][4][32 * kSpt];
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    if (threadIdx.x == 0) ncnt = corr_nodes(pos, a.n, a.cutoff, nwp, nw);
    __syncthreads();
    const int ia = blockIdx.x;
    if (ia >= ncnt) return;
    const float w = nwp[ia];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nl = a.nl;
    Lane4 ln;
#pragma unroll
    for (int k = 0; k < kSpt; ++k) {
        const int j = lane + 32 * k;
        ln.j[k] = j;
        ln.valid[k] = j < nl;
        ln.rid[k] = ln.valid[k] ? a.sites[j] : 0;
        ln.prm[k] = ln.valid[k] ? a.sites_perm[j] : 0;
        ln.irid[k] = ln.valid[k] ? a.inv_sites[j] : 0;
        ln.iprm[k] = ln.valid[k] ? a.inv_sites_perm[j] : 0;
    }
    const double dw = double(w) + odd_interp(pos, a.n, a.v2, w);
    double acc[kSpt][4];
#pragma unroll
    for (int k = 0; k < kSpt; ++k)
        for (int c = 0; c < 4; ++c) acc[k][c] = 0.0;
    for (int b = warp; b < ncnt; b += kWarps) {
        const float wp = nwp[b];
        AB8 ab;
        access8(pos, a.n, nl, w + wp + 0.0f, 0.0f, w - wp, ab);
        float vv[4];
        for (int c = 0; c < 4; ++c) vv[c] = value4(pos, a, c, 0, 0, w + wp + 0.0f, w - wp, 0.0f);
        const double dwp = double(wp) + odd_interp(pos, a.n, a.v2, wp);
        const double cw = nw[b] / (dw * dw * dwp * dwp * (4.0 * kPiD * kPiD));
#pragma unroll
        for (int k = 0; k < kSpt; ++k) {
            if (!ln.valid[k]) continue;
            float g[4];
            bundle8(a, ab, ab.exch ? ln.irid[k] : ln.rid[k], ab.exch ? ln.iprm[k] : ln.prm[k], g);
            double rr[4] = {-double(g[0]), -double(g[1]), -double(g[2]), -4.0 * double(g[3])};  // dumbbell
            if (ln.j[k] == 0) {  // egg diagram
                rr[0] += 0.5 * (double(vv[0]) - vv[1] - vv[2] + vv[3]);
                rr[1] += 0.5 * (-double(vv[0]) + vv[1] - vv[2] + vv[3]);
                rr[2] += 0.5 * (-double(vv[0]) - vv[1] + vv[2] + vv[3]);
                rr[3] += 2.0 * (double(vv[0]) + vv[1] + vv[2] + vv[3]);
            }
            for (int c = 0; c < 4; ++c) acc[k][c] += cw * rr[c];
        }
    }
#pragma unroll
    for (int k = 0; k < kSpt; ++k)
        for (int c = 0; c < 4; ++c) red[warp][c][lane + 32 * k] = acc[k][c];
    __syncthreads();
    for (int e = threadIdx.x; e < 4 * nl; e += blockDim.x) {
        const int c = e / nl, j = e - c * nl;
        double sum = 0.0;
        for (int q = 0; q < kWarps; ++q) sum += red[q][c][j];
        a.partial[(size_t(ia) * 4 + c) * nl + j] = sum;
    }
}

__global__ void xyz_corr_final_kernel(XyzArgs a) {
    __shared__ float pos[kMaxFreq];
    __shared__ float nwp[kMaxCorrNodes];
    __shared__ double nw[kMaxCorrNodes];
    __shared__ int ncnt;
    extern __shared__ double chi[];  // [4][nl]
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    if (threadIdx.x == 0) ncnt = corr_nodes(pos, a.n, a.cutoff, nwp, nw);
    __syncthreads();
    const int nl = a.nl;
    for (int e = threadIdx.x; e < 4 * nl; e += blockDim.x) {
        const int c = e / nl, j = e - c * nl;
        double sum = 0.0;
        for (int ia = 0; ia < ncnt; ++ia) {
            double v = a.partial[(size_t(ia) * 4 + c) * nl + j];
            if (j == 0) {  // on-site term
                const float w = nwp[ia];
                const double dw = double(w) + odd_interp(pos, a.n, a.v2, w);
                const double t1 = 1.0 / (dw * dw);
                v += c == D ? t1 / kPiD : t1 / (4.0 * kPiD);
            }
            sum += nw[ia] * v;
        }
        chi[e] = sum;
        a.out[4 * size_t(a.n_corr) + e] = float(sum);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < a.n_corr; q += blockDim.x) {
        const int r = a.corr_rid[q], p = a.corr_perm[q];
        for (int c = 0; c < 3; ++c) a.out[size_t(c) * a.n_corr + q] = float(chi[perm_c(p, c) * nl + r]);
        a.out[3 * size_t(a.n_corr) + q] = float(chi[3 * nl + r]);
    }
}

// ------------------------------------------------------------------------------------
// Euler step, state layout changes
// ------------------------------------------------------------------------------------
__global__ void xyz_euler_kernel(float *__restrict__ x, const float *__restrict__ dx, long long n, float step) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = __fadd_rn(x[i], __fmul_rn(step, dx[i]));
}

// stage[c * n + i] (four arrays in the reference layout) <-> v[i] (one float4 per element)
__global__ void xyz_pack_kernel(const float *__restrict__ stage, float4 *__restrict__ v, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = make_float4(stage[i], stage[n + i], stage[2 * n + i], stage[3 * n + i]);
}
__global__ void xyz_unpack_kernel(const float4 *__restrict__ v, float *__restrict__ stage, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 e = v[i];
        stage[i] = e.x;
        stage[n + i] = e.y;
        stage[2 * n + i] = e.z;
        stage[3 * n + i] = e.w;
    }
}

using cuh::check_cuda;
using cuh::copy_grid;
using cuh::dalloc;
using cuh::h2d;

}  // namespace

struct spn_xyz {
    int device = 0, n = 0, nl = 0, n_range = 0, n_corr = 0, n_overlap = 0, max_nodes = 0, sms = 0, grid = 0;
    int spt = 4;  // sites per lane of the vertex kernel
    long long fn = 0;
    float cutoff = 0.0f;
    cudaStream_t stream = nullptr;
    float *freq = nullptr, *v2 = nullptr, *dv2 = nullptr, *stage = nullptr, *node_wp = nullptr, *node_c = nullptr,
          *corr_out = nullptr;
    float4 *sd = nullptr, *dsd = nullptr;
    int *ints = nullptr;  // all integer tables in one allocation
    int *sites, *sites_perm, *inv_sites, *inv_sites_perm, *range_rid, *range_inv, *corr_rid, *corr_perm, *node_cnt,
        *work_counter, *rpa_sched, *rpa_count, *rpa_slot_base, *rpa_seg_ptr;
    int rpa_n_seg = 0;
    unsigned *status = nullptr;
    double *partial = nullptr;

    XyzArgs args() const {
        XyzArgs a;
        a.n = n;
        a.nl = nl;
        a.fn = int(fn);
        a.max_nodes = max_nodes;
        a.n_range = n_range;
        a.n_corr = n_corr;
        a.cutoff = cutoff;
        a.freq = freq;
        a.sd = sd;
        a.dsd = dsd;
        a.v2 = v2;
        a.dv2 = dv2;
        a.sites = sites;
        a.sites_perm = sites_perm;
        a.inv_sites = inv_sites;
        a.inv_sites_perm = inv_sites_perm;
        a.rpa_sched = rpa_sched;
        a.rpa_count = rpa_count;
        a.rpa_slot_base = rpa_slot_base;
        a.rpa_seg_ptr = rpa_seg_ptr;
        a.rpa_n_seg = rpa_n_seg;
        a.range_rid = range_rid;
        a.range_inv = range_inv;
        a.node_wp = node_wp;
        a.node_c = node_c;
        a.node_cnt = node_cnt;
        a.work_counter = work_counter;
        a.status = status;
        a.corr_rid = corr_rid;
        a.corr_perm = corr_perm;
        a.partial = partial;
        a.out = corr_out;
        return a;
    }

    // argument block of the SU(2) node-table body (self-energy, mesh, node tables only)
    FlowArgs node_args() const {
        FlowArgs f;
        std::memset(&f, 0, sizeof(f));
        f.n = n;
        f.nl = nl;
        f.max_nodes = max_nodes;
        f.cutoff = cutoff;
        f.freq = freq;
        f.v2 = v2;
        f.dv2 = dv2;
        f.fp64_sigma = 0;
        f.node_wp = node_wp;
        f.node_c = node_c;
        f.node_cnt = node_cnt;
        f.status = status;
        return f;
    }

    void release() {
        cudaSetDevice(device);
        void *ptrs[] = {freq, v2, dv2, stage, node_wp, node_c, corr_out, sd, dsd, ints, status, partial};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

void validate(const spn_xyz_desc *d) {
    if (!d) throw Error(ErrorType::Argument, "null descriptor");
    if (d->n_freq < 2 || d->n_freq > kMaxFreq)
        throw Error(ErrorType::Unsupported, "n_freq must be in [2, " + std::to_string(kMaxFreq) + "]");
    if (d->n_sites < 1 || d->n_sites > 32 * kSpt)
        throw Error(ErrorType::Unsupported, "n_sites must be in [1, " + std::to_string(32 * kSpt) + "]");
    if (!d->freq || !d->sites_rid || !d->sites_perm || !d->inv_sites_rid || !d->inv_sites_perm || !d->overlap_ptr ||
        (d->n_range > 0 && (!d->range_rid || !d->range_inv_rid)) || (d->n_corr > 0 && (!d->corr_rid || !d->corr_perm)))
        throw Error(ErrorType::Argument, "descriptor table pointer is NULL");
    for (int i = 0; i < d->n_freq; ++i) {
        if (!(d->freq[i] > 0.0f)) throw Error(ErrorType::Argument, "frequencies must be positive");
        if (i > 0 && !(d->freq[i] > d->freq[i - 1])) throw Error(ErrorType::Argument, "frequencies must be strictly ascending");
    }
    const long long fn = (long long)d->n_freq * d->n_freq * (d->n_freq + 1) / 2;
    if (fn * d->n_sites >= (1ll << 31)) throw Error(ErrorType::Unsupported, "vertex larger than 2^31 elements");
    const int nl = d->n_sites;
    auto in_range = [&](const int *v, int cnt, int hi, const char *what) {
        for (int i = 0; i < cnt; ++i)
            if (v[i] < 0 || v[i] >= hi) throw Error(ErrorType::Argument, std::string(what) + " entry out of range");
    };
    in_range(d->sites_rid, nl, nl, "sites_rid");
    in_range(d->inv_sites_rid, nl, nl, "inv_sites_rid");
    in_range(d->sites_perm, nl, 6, "sites_perm");
    in_range(d->inv_sites_perm, nl, 6, "inv_sites_perm");
    if (d->overlap_ptr[0] != 0) throw Error(ErrorType::Argument, "overlap_ptr[0] must be 0");
    for (int r = 0; r < nl; ++r)
        if (d->overlap_ptr[r + 1] < d->overlap_ptr[r]) throw Error(ErrorType::Argument, "overlap_ptr must be non-decreasing");
    const int nov = d->overlap_ptr[nl];
    if (nov > 0 && (!d->overlap_rid1 || !d->overlap_rid2 || !d->overlap_perm1 || !d->overlap_perm2))
        throw Error(ErrorType::Argument, "overlap pair table is NULL");
    in_range(d->overlap_rid1, nov, nl, "overlap_rid1");
    in_range(d->overlap_rid2, nov, nl, "overlap_rid2");
    in_range(d->overlap_perm1, nov, 6, "overlap_perm1");
    in_range(d->overlap_perm2, nov, 6, "overlap_perm2");
    in_range(d->range_rid, d->n_range, nl, "range_rid");
    in_range(d->range_inv_rid, d->n_range, nl, "range_inv_rid");
    in_range(d->corr_rid, d->n_corr, nl, "corr_rid");
    in_range(d->corr_perm, d->n_corr, 6, "corr_perm");
}

// the vertex kernel for SPT sites per lane (1 for Nl <= 32, 2 for Nl <= 64, else 4)
const void *vertex_kernel(int spt) {
    if (spt == 1) return reinterpret_cast<const void *>(&xyz_vertex_kernel<1>);
    if (spt == 2) return reinterpret_cast<const void *>(&xyz_vertex_kernel<2>);
    return reinterpret_cast<const void *>(&xyz_vertex_kernel<4>);
}

// The RPA pairs of each site in the order of host/pair_order (against bank collisions of the
// kernel's 16-byte reads of A6 and B6), packed rid1 | rid2 << 7 | perm1 << 14 | perm2 << 17.
std::vector<int> order_rpa_pairs(const spn_xyz_desc *d) {
    const int nl = d->n_sites;
    const std::vector<int> order =
        order_pairs_by_banks(nl, d->overlap_ptr, xyz_rpa_model(),
                             xyz_rpa_words(nl, d->overlap_rid1, d->overlap_rid2, d->overlap_perm1, d->overlap_perm2));
    std::vector<int> out(order.size());
    for (size_t k = 0; k < order.size(); ++k) {
        const int i = order[k];
        out[k] = d->overlap_rid1[i] | d->overlap_rid2[i] << 7 | d->overlap_perm1[i] << 14 | d->overlap_perm2[i] << 17;
    }
    return out;
}

size_t vertex_smem(int nl, int n_seg) {
    return size_t(kWarps) * (kXBatch * sizeof(XDesc) + (12 * size_t(nl) + size_t(n_seg)) * sizeof(float4));
}

void launch_correlation(spn_xyz *h) {
    const XyzArgs a = h->args();
    xyz_corr_inner_kernel<<<2 * h->n + 4, 128, 0, h->stream>>>(a);
    check_cuda(cudaGetLastError(), "correlation launch");
    xyz_corr_final_kernel<<<1, 128, 4 * h->nl * sizeof(double), h->stream>>>(a);
    check_cuda(cudaGetLastError(), "correlation final launch");
}

}  // namespace

extern "C" int spn_xyz_create(const spn_xyz_desc *d, spn_xyz **out) {
    return guarded([&] {
        if (!out) throw Error(ErrorType::Argument, "null output handle");
        validate(d);
        auto *h = new spn_xyz;
        try {
            h->device = d->device;
            check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
            h->n = d->n_freq;
            h->nl = d->n_sites;
            h->fn = (long long)h->n * h->n * (h->n + 1) / 2;
            h->n_range = d->n_range;
            h->n_corr = d->n_corr;
            h->n_overlap = d->overlap_ptr[d->n_sites];
            h->max_nodes = 2 * h->n + 8;
            check_cuda(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate");
            const size_t vsz = size_t(h->fn) * h->nl;
            h->freq = dalloc<float>(h->n, "alloc freq");
            h->v2 = dalloc<float>(h->n, "alloc v2");
            h->dv2 = dalloc<float>(h->n, "alloc dv2");
            h->sd = dalloc<float4>(vsz, "alloc vertex state");
            h->dsd = dalloc<float4>(vsz, "alloc vertex flow");
            h->node_wp = dalloc<float>(size_t(h->n) * h->max_nodes, "alloc node table");
            h->node_c = dalloc<float>(size_t(h->n) * h->max_nodes, "alloc node table");
            h->corr_out = dalloc<float>(4 * size_t(h->n_corr) + 4 * h->nl, "alloc correlation output");
            h->partial = dalloc<double>(size_t(kMaxCorrNodes) * 4 * h->nl, "alloc correlation scratch");
            h->status = dalloc<unsigned>(1, "alloc status");
            // integer tables, one allocation
            const int nl = h->nl, nr = h->n_range, nc = h->n_corr;
            std::vector<int> img;
            std::vector<size_t> at;
            auto put = [&](const int *src, int cnt) {
                at.push_back(img.size());
                if (src) img.insert(img.end(), src, src + cnt);
                else img.insert(img.end(), size_t(cnt), 0);
            };
            put(d->sites_rid, nl);
            put(d->sites_perm, nl);
            put(d->inv_sites_rid, nl);
            put(d->inv_sites_perm, nl);
            const std::vector<int> packed = order_rpa_pairs(d);
            const LaneSchedule rpa = xyz_lane_schedule(nl, d->overlap_ptr, packed);
            h->rpa_n_seg = rpa.n_seg;
            put(d->range_rid, nr);
            put(d->range_inv_rid, nr);
            put(d->corr_rid, nc);
            put(d->corr_perm, nc);
            put(nullptr, h->n);  // node counts
            put(nullptr, 1);     // work counter
            put(rpa.sched.data(), int(rpa.sched.size()));
            put(rpa.count.data(), 32);
            put(rpa.slot_base.data(), 32);
            put(rpa.seg_ptr.data(), nl + 1);
            h->ints = dalloc<int>(img.size(), "alloc lattice tables");
            h2d(h->ints, img.data(), img.size(), h->stream);
            int **fields[] = {&h->sites, &h->sites_perm, &h->inv_sites, &h->inv_sites_perm, &h->range_rid, &h->range_inv,
                              &h->corr_rid, &h->corr_perm, &h->node_cnt, &h->work_counter, &h->rpa_sched,
                              &h->rpa_count, &h->rpa_slot_base, &h->rpa_seg_ptr};
            for (size_t k = 0; k < at.size(); ++k) *fields[k] = h->ints + at[k];
            h2d(h->freq, d->freq, h->n, h->stream);
            check_cuda(cudaMemsetAsync(h->sd, 0, vsz * sizeof(float4), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->dsd, 0, vsz * sizeof(float4), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->v2, 0, h->n * sizeof(float), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->dv2, 0, h->n * sizeof(float), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->status, 0, sizeof(unsigned), h->stream), "memset");
            check_cuda(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device), "device attribute");
            int per_sm = 0;
            h->spt = h->nl <= 32 ? 1 : (h->nl <= 64 ? 2 : 4);
            const void *fn = vertex_kernel(h->spt);
            check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(vertex_smem(h->nl, h->rpa_n_seg))),
                       "shared memory limit");
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, vertex_smem(h->nl, h->rpa_n_seg)), "occupancy");
            if (per_sm < 1) throw Error(ErrorType::Unsupported, "XYZ vertex-flow kernel does not fit on this device");
            h->grid = h->sms * per_sm;
            check_cuda(cudaStreamSynchronize(h->stream), "create sync");
        } catch (...) {
            h->release();
            delete h;
            throw;
        }
        *out = h;
    });
}

extern "C" int spn_xyz_destroy(spn_xyz *h) {
    if (!h) return SPN_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->release();
    delete h;
    return SPN_OK;
}

namespace {
float *stage_of(spn_xyz *h) {
    if (!h->stage) h->stage = dalloc<float>(4 * size_t(h->fn) * h->nl, "alloc state stage");
    return h->stage;
}
}  // namespace

extern "C" int spn_xyz_set_state(spn_xyz *h, float cutoff, const float *v2, const float *xx, const float *yy, const float *zz,
                                 const float *dd) {
    return guarded([&] {
        if (!h || !v2 || !xx || !yy || !zz || !dd) throw Error(ErrorType::Argument, "null argument");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        const size_t vsz = size_t(h->fn) * h->nl;
        float *st = stage_of(h);
        const float *src[4] = {xx, yy, zz, dd};
        for (int c = 0; c < 4; ++c) h2d(st + c * vsz, src[c], vsz, h->stream);
        xyz_pack_kernel<<<copy_grid((long long)vsz), 256, 0, h->stream>>>(st, h->sd, (long long)vsz);
        check_cuda(cudaGetLastError(), "pack launch");
        h2d(h->v2, v2, h->n, h->stream);
        h->cutoff = cutoff;
        check_cuda(cudaStreamSynchronize(h->stream), "set_state sync");
    });
}

namespace {
void copy_out(spn_xyz *h, const float4 *src, float *const dst[4]) {
    const size_t vsz = size_t(h->fn) * h->nl;
    float *st = stage_of(h);
    xyz_unpack_kernel<<<copy_grid((long long)vsz), 256, 0, h->stream>>>(src, st, (long long)vsz);
    check_cuda(cudaGetLastError(), "unpack launch");
    for (int c = 0; c < 4; ++c)
        if (dst[c])
            check_cuda(cudaMemcpyAsync(dst[c], st + c * vsz, vsz * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
}
}  // namespace

extern "C" int spn_xyz_get_state(spn_xyz *h, float *cutoff, float *v2, float *xx, float *yy, float *zz, float *dd) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        if (cutoff) *cutoff = h->cutoff;
        if (v2) check_cuda(cudaMemcpyAsync(v2, h->v2, h->n * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        float *const dst[4] = {xx, yy, zz, dd};
        copy_out(h, h->sd, dst);
        check_cuda(cudaStreamSynchronize(h->stream), "get_state sync");
    });
}

extern "C" int spn_xyz_get_flow(spn_xyz *h, float *dv2, float *xx, float *yy, float *zz, float *dd) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        if (dv2) check_cuda(cudaMemcpyAsync(dv2, h->dv2, h->n * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        float *const dst[4] = {xx, yy, zz, dd};
        copy_out(h, h->dsd, dst);
        check_cuda(cudaStreamSynchronize(h->stream), "get_flow sync");
    });
}

extern "C" int spn_xyz_compute_step(spn_xyz *h) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        check_cuda(cudaMemsetAsync(h->status, 0, sizeof(unsigned), h->stream), "memset status");
        check_cuda(cudaMemsetAsync(h->work_counter, 0, sizeof(int), h->stream), "memset counter");
        const XyzArgs a = h->args();
        xyz_self_energy_kernel<<<h->n, 128, 0, h->stream>>>(a);
        check_cuda(cudaGetLastError(), "self-energy launch");
        xyz_node_table_kernel<<<(h->n + 63) / 64, 64, 0, h->stream>>>(h->node_args());
        check_cuda(cudaGetLastError(), "node table launch");
        check_cuda(cudaFuncSetAttribute(vertex_kernel(h->spt), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(vertex_smem(h->nl, h->rpa_n_seg))),
                   "shared memory limit");
        if (h->spt == 1) xyz_vertex_kernel<1><<<h->grid, kThreads, vertex_smem(h->nl, h->rpa_n_seg), h->stream>>>(a);
        else if (h->spt == 2) xyz_vertex_kernel<2><<<h->grid, kThreads, vertex_smem(h->nl, h->rpa_n_seg), h->stream>>>(a);
        else xyz_vertex_kernel<4><<<h->grid, kThreads, vertex_smem(h->nl, h->rpa_n_seg), h->stream>>>(a);
        check_cuda(cudaGetLastError(), "vertex flow launch");
    });
}

extern "C" int spn_xyz_finalize_step(spn_xyz *h, float new_cutoff) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        const float step = new_cutoff - h->cutoff;
        const long long n4 = 4 * h->fn * h->nl;
        xyz_euler_kernel<<<1, 64, 0, h->stream>>>(h->v2, h->dv2, h->n, step);
        xyz_euler_kernel<<<copy_grid(n4), 256, 0, h->stream>>>(reinterpret_cast<float *>(h->sd),
                                                              reinterpret_cast<const float *>(h->dsd), n4, step);
        check_cuda(cudaGetLastError(), "euler launch");
        h->cutoff = new_cutoff;
    });
}

extern "C" int spn_xyz_measure_correlation(spn_xyz *h, float *xx, float *yy, float *zz, float *dd, float *chi) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        launch_correlation(h);
        float *const dst[4] = {xx, yy, zz, dd};
        for (int c = 0; c < 4; ++c)
            if (dst[c])
                check_cuda(cudaMemcpyAsync(dst[c], h->corr_out + size_t(c) * h->n_corr, h->n_corr * sizeof(float),
                                           cudaMemcpyDeviceToHost, h->stream),
                           "D2H");
        if (chi)
            check_cuda(cudaMemcpyAsync(chi, h->corr_out + 4 * size_t(h->n_corr), 4 * h->nl * sizeof(float),
                                       cudaMemcpyDeviceToHost, h->stream),
                       "D2H");
        check_cuda(cudaStreamSynchronize(h->stream), "correlation sync");
    });
}

extern "C" int spn_xyz_is_diverged(spn_xyz *h, int *diverged) {
    return guarded([&] {
        if (!h || !diverged) throw Error(ErrorType::Argument, "null argument");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        unsigned st = 0;
        check_cuda(cudaMemcpyAsync(&st, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream), "D2H");
        check_cuda(cudaStreamSynchronize(h->stream), "status sync");
        if (st & kStatusNodeOverflow) throw Error(ErrorType::Device, "loop-frequency node table overflow");
        *diverged = (st & kStatusNaN) ? 1 : 0;
    });
}

extern "C" int spn_xyz_vertex_probe(const float *pos, int n, int n_sites, const float *xx, const float *yy,
                                    const float *zz, const float *dd, int rid12, int rid21, int perm12, int perm21,
                                    float s, float t, float u, int channel, int local, float *value) {
    return guarded([&] {
        cuh::check_mesh(pos, n, kMaxFreq);
        if (n_sites < 1 || n_sites > 32 * kSpt || !xx || !yy || !zz || !dd || !value || rid12 < 0 ||
            rid12 >= n_sites || rid21 < 0 || rid21 >= n_sites || perm12 < 0 || perm12 > 5 || perm21 < 0 ||
            perm21 > 5 || channel < -1 || channel > 3 || (channel < 0 && (local || perm12 || perm21)))
            throw Error(ErrorType::Argument, "spn_xyz_vertex_probe: bad argument");
        // the device layout: one float4 (X, Y, Z, D) per element
        const size_t vsz = size_t(n) * n * (n + 1) / 2 * n_sites;
        std::vector<float4> sd(vsz);
        for (size_t i = 0; i < vsz; ++i) sd[i] = make_float4(xx[i], yy[i], zz[i], dd[i]);
        XyzArgs a{};
        a.n = n;
        a.nl = n_sites;
        a.sd = sd.data();
        float g[4];
        if (channel < 0) {
            for (int c = 0; c < 4; ++c) g[c] = value4(pos, a, c, rid12, rid21, s, t, u);
        } else if (channel == 3) {
            AB8 ab;
            access8(pos, n, n_sites, s, t, u, ab);
            if (local) bundle8(a, ab, 0, 0, g);
            else bundle8(a, ab, ab.exch ? rid21 : rid12, ab.exch ? perm21 : perm12, g);
        } else {
            // the channel's own frequency is a mesh value; the two others are interpolated in
            // the order access4i takes them (t, u for S; s, u for T; s, t for U)
            const MeshSearch<float> m{pos, n};
            const float own[3] = {s, t, u};
            const int e = cuh::mesh_index_of(pos, n, own[channel]);
            const Interp<float> ia = interp_abs(m, channel == 0 ? t : s), ib = interp_abs(m, channel == 2 ? t : u);
            AB4 ab;
            if (channel == 0) access4i<kS>(n, n_sites, s, t, u, ia, ib, e, ab);
            else if (channel == 1) access4i<kT>(n, n_sites, s, t, u, ia, ib, e, ab);
            else access4i<kU>(n, n_sites, s, t, u, ia, ib, e, ab);
            float4 v;
            if (local) {
                v = local4(a, ab);
            } else {
                LaneT<1> ln;
                ln.j[0] = 0;
                ln.valid[0] = true;
                ln.rid[0] = rid12;
                ln.prm[0] = perm12;
                ln.irid[0] = rid21;
                ln.iprm[0] = perm21;
                gather4(a, ab, ln, &v);
            }
            g[0] = v.x;
            g[1] = v.y;
            g[2] = v.z;
            g[3] = v.w;
        }
        for (int c = 0; c < 4; ++c) value[c] = g[c];
    });
}
