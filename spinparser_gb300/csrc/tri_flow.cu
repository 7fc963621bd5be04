// GB300 kernels of the TRI pf-FRG flow right-hand side (time-reversal-invariant spin models
// with general, also off-diagonal, couplings: Heisenberg-Kitaev-Gamma, ...) and the device
// half of the spn_tri_* C ABI in include/spn_su2.h.  Restates TRIFrgCore
// (src/TRI/TRIFrgCore.cpp:122-3001), the TRI vertex access (src/TRI/TRIVertexTwoParticle.hpp:
// 190-677) and TRIMeasurementCorrelation (src/TRI/TRIMeasurementCorrelation.cpp:147-285).
//
// The vertex keeps the reference's layout: 16 components (a, b) per element, a, b in X, Y, Z,
// density, as [(s(s+1)/2+u)*N + t][4a+b][site].  An access buffer carries, besides offsets and
// weights, the sign rules of TRIVertexTwoParticleAccessBuffer: a zeta(a) zeta(b) factor when
// exactly one of t, u was negated, and -zeta of the stored second component for a support
// whose s and u were exchanged.  A lattice symmetry map permutes X, Y, Z of both indices.
// The flow equations' coefficients come from tri_algebra.hpp (Pauli products) and fold to
// constants in the unrolled loops.
//
// A step: the self-energy flow (one CTA per frequency), the loop-frequency node tables (the
// SU(2) core's, shared), the vertex flow and the Euler update.  The vertex-flow kernel runs a
// persistent grid whose warps take one (s,t,u) triple at a time from a device counter.  Per
// channel, nodes go in batches of 16: a lane first builds one node's access buffers into a
// shared-memory descriptor; then, node by node, the warp gathers the four 16-component slabs
// of all sites into shared memory (t: and the 64 site-local values of the chalice diagrams),
// and each lane evaluates the products for its sites from registers.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>
#include "su2_common.cuh"
#include "su2_device.cuh"
#include "su2_kernels.cuh"
#include "tri_algebra.hpp"
#include "cuda_host.cuh"
#include "host/capi_common.hpp"
#include "host/pair_order.hpp"
#include "../../include/spn_su2.h"

using namespace spn;
using namespace spn::dev;

namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSites = 128;
constexpr int kTBatch = 4;  // nodes whose descriptors a warp builds at once (a quad of lanes each)
constexpr int kCorrOut = 10;  // XX XY XZ YX YY YZ ZX ZY ZZ DD

// The six spin permutations (X,Y,Z) (X,Z,Y) (Y,X,Z) (Y,Z,X) (Z,X,Y) (Z,Y,X): 2 bits per image
// component, 6 bits per permutation; the density maps to itself.
constexpr unsigned long long kPermBits =
    36ull | (24ull << 6) | (33ull << 12) | (9ull << 18) | (18ull << 24) | (6ull << 30);
__host__ __device__ __forceinline__ int permc(int p, int c) {
    return c == 3 ? 3 : int((kPermBits >> (6 * p + 2 * c)) & 3ull);
}
SPN_HDI float zeta(int c) { return c <= 2 ? -1.0f : 1.0f; }

struct TriArgs {
    int n, nl, fn, max_nodes, n_range, n_corr;
    float cutoff;
    const float *freq;
    const float *v4;  // state [F_N][16][nl]
    float *dv4;       // flow
    const float *v2;
    float *dv2;
    const int *sites, *sites_perm, *inv_sites, *inv_sites_perm;
    // the t channel's RPA pairs of all sites in one lane-balanced walk (lane_schedule): entry i of
    // lane l is sched[32 i + l], the pair's word rid1 | rid2 << 7 | the images of X, Y, Z under
    // perm1 (2 bits each) << 14 | the same for perm2 << 20 (order_rpa_pairs), bit 26 set on the
    // last entry of a site's run in the lane; the runs' partial sums (16 components) go to slots
    // slot_base[l], ... and site j sums slots seg_ptr[j] .. seg_ptr[j + 1] - 1
    const int *rpa_sched, *rpa_count, *rpa_slot_base, *rpa_seg_ptr;
    int rpa_n_seg;
    const int *range_rid, *range_inv;
    const float *node_wp, *node_c;
    const int *node_cnt;
    int *work_counter;
    unsigned *status;
    const int *corr_rid, *corr_perm;
    double *partial;  // [kMaxCorrNodes][16][nl]
    float *out;       // [10][n_corr] correlations, then chi [16][nl]
};

// ---- access buffers (TRIVertexTwoParticleAccessBuffer) ----
constexpr int kFlExch = 1 << 8;  // read the site-exchanged pair
constexpr int kFlTu = 1 << 9;    // zeta(a) zeta(b): exactly one of t, u negated
// bits 0..7: support i's s and u offsets were exchanged

template <int K>
struct TABT {
    int off[K];
    float w[K];
    int fl;
};
using TAB4 = TABT<4>;
using TAB8 = TABT<8>;

// sign[i][a][b] of the access buffer (TRIVertexTwoParticle.hpp:401-448, 643-671)
SPN_HDI float tab_sign(int fl, int i, int a, int b) {
    float s = 1.0f;
    if (fl & kFlTu) s *= zeta(a) * zeta(b);
    if ((fl >> i) & 1) s *= -((fl & kFlExch) ? zeta(a) : zeta(b));
    return s;
}

SPN_HDI int tri_fold(float &s, float &t, float &u) {
    int fl = 0;
    if (s < 0) {
        s = -s;
        fl ^= kFlExch;
    }
    if (t < 0) {
        t = -t;
        fl ^= kFlTu;
    }
    if (u < 0) {
        u = -u;
        fl ^= kFlExch | kFlTu;
    }
    return fl;
}

SPN_HDI void tri_slab(int si, int ti, int ui, int step_su, int step_t, int i, int &off, int &fl) {
    if (si < ui) {
        off = (ui * (ui + 1) / 2 + si) * step_su + ti * step_t;
        fl |= 1 << i;
    } else {
        off = (si * (si + 1) / 2 + ui) * step_su + ti * step_t;
    }
}

// generateAccessBuffer(s, t, u, channel) (TRIVertexTwoParticle.hpp:401-505) with e the exact mesh
// index of the channel's own coordinate, which every caller knows, and the two interpolations
// given (interp_abs of the interpolated coordinates, as for access4i): a node's buffers
// interpolate four distinct magnitudes, each looked up once.
template <int CH>
SPN_HDI void tri_access4i(int n, int nl, float s, float t, float u, int e, const Interp<float> &ia,
                          const Interp<float> &ib, TAB4 &ab) {
    int fl = tri_fold(s, t, u);
    const int step_t = 16 * nl, step_su = n * step_t;
    const int la = ia.lo, ua = ia.hi, lb = ib.lo, ub = ib.hi;
    const float ba = ia.b, bb = ib.b;
    const float na = rn_sub(1.0f, ba), nb = rn_sub(1.0f, bb);
    ab.w[0] = rn_mul(nb, na);
    ab.w[1] = rn_mul(nb, ba);
    ab.w[2] = rn_mul(bb, na);
    ab.w[3] = rn_mul(bb, ba);
    if (CH == kS) {
        tri_slab(e, la, lb, step_su, step_t, 0, ab.off[0], fl);
        tri_slab(e, ua, lb, step_su, step_t, 1, ab.off[1], fl);
        tri_slab(e, la, ub, step_su, step_t, 2, ab.off[2], fl);
        tri_slab(e, ua, ub, step_su, step_t, 3, ab.off[3], fl);
    } else if (CH == kT) {
        tri_slab(la, e, lb, step_su, step_t, 0, ab.off[0], fl);
        tri_slab(ua, e, lb, step_su, step_t, 1, ab.off[1], fl);
        tri_slab(la, e, ub, step_su, step_t, 2, ab.off[2], fl);
        tri_slab(ua, e, ub, step_su, step_t, 3, ab.off[3], fl);
    } else {
        tri_slab(la, lb, e, step_su, step_t, 0, ab.off[0], fl);
        tri_slab(ua, lb, e, step_su, step_t, 1, ab.off[1], fl);
        tri_slab(la, ub, e, step_su, step_t, 2, ab.off[2], fl);
        tri_slab(ua, ub, e, step_su, step_t, 3, ab.off[3], fl);
    }
    ab.fl = fl;
}

// generateAccessBuffer(s, t, u): trilinear (TRIVertexTwoParticle.hpp:514-584)
SPN_HDI void tri_access8(const float *pos, int n, int nl, float s, float t, float u, TAB8 &ab) {
    int fl = tri_fold(s, t, u);
    const int step_t = 16 * nl, step_su = n * step_t;
    int ls, us, lt, ut, lu, uu;
    float bs, bt, bu;
    mesh_interp(pos, n, s, ls, us, bs);
    mesh_interp(pos, n, t, lt, ut, bt);
    mesh_interp(pos, n, u, lu, uu, bu);
    const float ns = rn_sub(1.0f, bs), nt = rn_sub(1.0f, bt), nu = rn_sub(1.0f, bu);
    ab.w[0] = rn_mul(rn_mul(nt, ns), nu);
    ab.w[1] = rn_mul(rn_mul(nt, bs), nu);
    ab.w[2] = rn_mul(rn_mul(bt, ns), nu);
    ab.w[3] = rn_mul(rn_mul(bt, bs), nu);
    ab.w[4] = rn_mul(rn_mul(nt, ns), bu);
    ab.w[5] = rn_mul(rn_mul(nt, bs), bu);
    ab.w[6] = rn_mul(rn_mul(bt, ns), bu);
    ab.w[7] = rn_mul(rn_mul(bt, bs), bu);
    tri_slab(ls, lt, lu, step_su, step_t, 0, ab.off[0], fl);
    tri_slab(us, lt, lu, step_su, step_t, 1, ab.off[1], fl);
    tri_slab(ls, ut, lu, step_su, step_t, 2, ab.off[2], fl);
    tri_slab(us, ut, lu, step_su, step_t, 3, ab.off[3], fl);
    tri_slab(ls, lt, uu, step_su, step_t, 4, ab.off[4], fl);
    tri_slab(us, lt, uu, step_su, step_t, 5, ab.off[5], fl);
    tri_slab(ls, ut, uu, step_su, step_t, 6, ab.off[6], fl);
    tri_slab(us, ut, uu, step_su, step_t, 7, ab.off[7], fl);
    ab.fl = fl;
}

// getValueLocal(a, b, ab) (TRIVertexTwoParticle.hpp:347-356): the components are exchanged
// first and index the sign table in that order.  getValue and getValueSuperbundle (tri_bundle)
// index it with the original order, so for a site-exchanging buffer the two differ in the sign
// of the mixed spin/density components on supports whose stored sector swaps s and u; this is
// the reference's convention, kept.
template <int K>
SPN_HDI float tri_local(const float *v4, int nl, const TABT<K> &ab, int ca, int cb) {
    if (ab.fl & kFlExch) {
        const int x = ca;
        ca = cb;
        cb = x;
    }
    const int o = (4 * ca + cb) * nl;
    float v = 0.0f;
#pragma unroll
    for (int i = 0; i < K; ++i) v += tab_sign(ab.fl, i, ca, cb) * ab.w[i] * ro_load(v4 + ab.off[i] + o);
    return v;
}

// getValueSuperbundle component c of site j (TRIVertexTwoParticle.hpp:364-391): the
// (exchanged, then permuted) component of the site's representative.
template <int K>
SPN_HDI float tri_bundle(const float *v4, int nl, const TABT<K> &ab, int c, int r, int p) {
    const int ca = c >> 2, cb = c & 3;
    const bool ex = ab.fl & kFlExch;
    const int o = (4 * permc(p, ex ? cb : ca) + permc(p, ex ? ca : cb)) * nl + r;
    float v = 0.0f;
#pragma unroll
    for (int i = 0; i < K; ++i) v += tab_sign(ab.fl, i, ca, cb) * ab.w[i] * ro_load(v4 + ab.off[i] + o);
    return v;
}

// getValue(i1, i2, s, t, u, a, b, FrequencyChannel::None) (TRIVertexTwoParticle.hpp:190-312)
// for the pairs the self-energy reads: through rid12 / rid21 with identity spin maps, on the
// state v4 of n frequencies and nl sites.
__host__ __device__ float tri_value_none(const float *pos, int n, int nl, const float *v4, int ca, int cb, int rid12,
                                         int rid21, float s, float t, float u) {
    float sign = 1.0f;
    bool sw = false;
    if (s < 0) {
        s = -s;
        const int x = ca; ca = cb; cb = x;
        sw = !sw;
    }
    if (t < 0) {
        t = -t;
        sign *= zeta(ca) * zeta(cb);
    }
    if (u < 0) {
        u = -u;
        const int x = ca; ca = cb; cb = x;
        sw = !sw;
        sign *= zeta(ca) * zeta(cb);
    }
    const int site = sw ? rid21 : rid12;
    const int step_t = 16 * nl, step_su = n * step_t, co = (4 * ca + cb) * nl + site;
    const float zb = -zeta(cb);
    int ls, us, lt, ut, lu, uu;
    float bs, bt, bu;
    mesh_interp(pos, n, s, ls, us, bs);
    mesh_interp(pos, n, t, lt, ut, bt);
    mesh_interp(pos, n, u, lu, uu, bu);
    auto Dv = [&](int x, int y, int z) {
        if (x >= z) return ro_load(v4 + (x * (x + 1) / 2 + z) * step_su + y * step_t + co);
        return zb * ro_load(v4 + (z * (z + 1) / 2 + x) * step_su + y * step_t + co);
    };
    return sign * ((1 - bu) * ((1 - bt) * ((1 - bs) * Dv(ls, lt, lu) + bs * Dv(us, lt, lu)) +
                               bt * ((1 - bs) * Dv(ls, ut, lu) + bs * Dv(us, ut, lu))) +
                   bu * ((1 - bt) * ((1 - bs) * Dv(ls, lt, uu) + bs * Dv(us, lt, uu)) +
                         bt * ((1 - bs) * Dv(ls, ut, uu) + bs * Dv(us, ut, uu))));
}

// ------------------------------------------------------------------------------------
// self-energy flow, one CTA per frequency (TRIFrgCore.cpp:122-151)
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) tri_self_energy_kernel(TriArgs a) {
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
        part += double(tri_value_none(pos, a.n, a.nl, a.v4, 3, 3, r12, r21, wpl, 0.0f, wml)) -
                double(tri_value_none(pos, a.n, a.nl, a.v4, 3, 3, r12, r21, wml, 0.0f, wpl));
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int k = 0; k < int(blockDim.x >> 5); ++k) sum += red[k];
        double val = -2.0 * sum;
        for (int c = 0; c < 4; ++c)
            val += double(tri_value_none(pos, a.n, a.nl, a.v4, c, c, 0, 0, wpl, wml, 0.0f)) -
                   double(tri_value_none(pos, a.n, a.nl, a.v4, c, c, 0, 0, wml, wpl, 0.0f));
        val /= (2.0 * kPiD * (double(L) + odd_interp(pos, a.n, a.v2, L)));
        const float outv = float(val);
        a.dv2[i] = outv;
        if (isnan(outv)) atomicOr(a.status, kStatusNaN);
    }
}

// Loop-frequency node tables: the SU(2) core's body on an argument block of this flow.
__global__ void tri_node_table_kernel(FlowArgs f) { node_table_body(f, blockIdx.x); }

// ------------------------------------------------------------------------------------
// vertex flow
// ------------------------------------------------------------------------------------
// Node descriptor (built by a quad of lanes, make_tpart): the four access buffers of the channel's
// integrand and, for the t channel, the four of the chalice diagrams' site-local values.
struct __align__(16) TDesc {
    TAB4 ab[8];
    float c;  // node coefficient
    int pad[3];
};

// Phase A: the descriptor of one node of channel ch (0 = s, 1 = t, 2 = u), built by the four
// lanes of a quad (q = 0..3): integralKernelS (TRIFrgCore.cpp:184-188), integralKernelT
// (TRIFrgCore.cpp:718-724, 1257-1259, 1814-1816) and integralKernelU (TRIFrgCore.cpp:2375-2379)
// read four access buffers each (the t channel four more for its chalice diagrams' site-local
// values), and every buffer interpolates two of the node's four distinct magnitudes A = |w1 + wp|,
// B = |w2 + wp|, C = |w1 - wp|, D = |w2p - wp|, E = |w2 - wp|, P = |w1p + wp|, Q = |w2p + wp|
// (a coordinate and its negation fold alike; -a - b is bitwise -(a + b), -a + b is b - a).  Lane
// q builds the buffers of one pair of magnitudes, with the coordinates from selects, so the quad
// runs one instruction stream: slot q ^ 2 (s channel), slot q (u channel), slots (q & 1) << 1 |
// q >> 1 and 4 + (q ^ 2) (t channel).
__device__ __forceinline__ void make_tpart(const TriArgs &a, const float *pos, int ch, int e, float s, float t, float u,
                                           float w1p, float w1, float w2p, float w2, float wp, int q, TDesc &d) {
    const MeshSearch<float> m{pos, a.n};
    const int nl = a.nl, n = a.n;
    const bool lo2 = q < 2, odd = q & 1;
    if (ch == 0) {
        // slots (t, u): 2 (-A, -B), 3 (P, -Q), 0 (B, A), 1 (-Q, P); (y1, y2) = (A, B) or (P, Q)
        const float y1 = odd ? w1p + wp : w1 + wp, y2 = odd ? w2p + wp : w2 + wp;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        tri_access4i<kS>(n, nl, s, lo2 ? (odd ? y1 : -y1) : (odd ? -y2 : y2), lo2 ? -y2 : y1, e, lo2 ? i1 : i2,
                         lo2 ? i2 : i1, d.ab[q ^ 2]);
    } else if (ch == 2) {
        // slots (s, t): 0 (A, -D), 1 (P, E), 2 (D, -A), 3 (E, P); (y1, y2) = (A, D) or (P, E)
        const float y1 = odd ? w1p + wp : w1 + wp, y2 = odd ? w2 - wp : w2p - wp;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        tri_access4i<kU>(n, nl, lo2 ? y1 : y2, lo2 ? (odd ? y2 : -y2) : (odd ? y1 : -y1), u, e, lo2 ? i1 : i2,
                         lo2 ? i2 : i1, d.ab[q]);
    } else {
        // main slots (s, u): 0 (C, P), 2 (P, C), 1 (D, -B), 3 (B, -D); chalice slots (s, t, u):
        // 6 (C, -P, -t), 7 (P, -C, -t), 4 (D, -B, t), 5 (B, -D, t); (y1, y2) = (C, P), (P, C),
        // (D, B), (B, D) for q = 0..3
        const float x1 = lo2 ? w1 - wp : w2p - wp, x2 = lo2 ? w1p + wp : w2 + wp;
        const float y1 = odd ? x2 : x1, y2 = odd ? x1 : x2;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        tri_access4i<kT>(n, nl, y1, t, lo2 ? y2 : -y2, e, i1, i2, d.ab[(int(odd) << 1) | (q >> 1)]);
        tri_access4i<kU>(n, nl, y1, -y2, lo2 ? -t : t, e, i1, i2, d.ab[4 + (q ^ 2)]);
    }
}

// Entry goff[e][c][j] of gather_slab's offsets: component c = 4a + b of the site whose
// representative is r under spin permutation p; e = 1 for the site-exchanged pair (components
// swapped, then permuted).
SPN_HDI int gather_offset(int e, int c, int nl, int r, int p) {
    const int ca = c >> 2, cb = c & 3;
    return (4 * permc(p, e ? cb : ca) + permc(p, e ? ca : cb)) * nl + r;
}

// One slab of a node for all sites (getValueSuperbundle): goff[e][c][j] is the offset of
// component c of site j (gather_offset of the site's representative and permutation).  The sign of support i depends on the component only through
// zeta(a) and zeta(b), so the four signed weights of each zeta class are formed once.
SPN_HDI void gather_slab(const float *__restrict__ v4, const TAB4 &ab, const int *goff, int nl, int lane, float *S) {
    const int fl = ab.fl;
    const bool ex = fl & kFlExch, tu = fl & kFlTu;
    float sw[4][4];  // [class: bit 0 a is a spin component, bit 1 b is][support]
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float za = (k & 1) ? -1.0f : 1.0f, zb = (k & 2) ? -1.0f : 1.0f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float sg = tu ? za * zb : 1.0f;
            if ((fl >> i) & 1) sg *= -(ex ? za : zb);
            sw[k][i] = sg * ab.w[i];
        }
    }
    const int *g = goff + (ex ? 16 * nl : 0);
    for (int j = lane; j < nl; j += 32) {
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            const int k = ((c >> 2) < 3 ? 1 : 0) | ((c & 3) < 3 ? 2 : 0);
            const int o = g[c * nl + j];
            float v = 0.0f;
#pragma unroll
            for (int i = 0; i < 4; ++i) v += sw[k][i] * ro_load(v4 + ab.off[i] + o);
            S[c * nl + j] = v;
        }
    }
}

// The two ladders for one site: per output c, a = 15..0 with the slab pairs (0,1) and (2,3)
// (TRIFrgCore.cpp:198-711 particle-particle, 2389-2902 particle-hole).
template <bool PH>
__device__ __forceinline__ void ladder(const float *S, int nl, int j, float *r) {
    float A0[16], A1[16], A2[16], A3[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        A0[c] = S[c * nl + j];
        A1[c] = S[(16 + c) * nl + j];
        A2[c] = S[(32 + c) * nl + j];
        A3[c] = S[(48 + c) * nl + j];
    }
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        float v = 0.0f;
#pragma unroll
        for (int n = 0; n < 16; ++n) {
            const int x = 15 - n, y = x ^ c ^ 15;
            if ((PH ? tri::ph_sign(c, x) : tri::pp_sign(c, x)) > 0) {
                v += A0[x] * A1[y];
                v += A2[x] * A3[y];
            } else {
                v -= A0[x] * A1[y];
                v -= A2[x] * A3[y];
            }
        }
        r[c] = v;
    }
}

// One overlap pair (packed word e) of the t integrand's RPA lattice sum (TRIFrgCore.cpp:733-2368)
// added to v[16]: 4x4 products over the inner spin index, the factors' components permuted by the
// pair's maps.  The RPA reads component (P a, P b) of a factor at (4 P(a) + P(b)) nl + rid: a row
// base per a plus a column offset per b, from the permutation images packed into the pair word.
// The products are summed without the factor 2 of the reference's terms; t_terms doubles the sum
// (scaling by 2 commutes with every rounding).
__device__ __forceinline__ void rpa_pair(const float *S, int nl, int e, float *v) {
    const float *S0 = S, *S1 = S + 16 * nl, *S2 = S + 32 * nl, *S3 = S + 48 * nl;
    {
        const int r1 = e & 127, r2 = (e >> 7) & 127;
        int col1[4], col2[4];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            col1[q] = ((e >> (14 + 2 * q)) & 3) * nl;
            col2[q] = ((e >> (20 + 2 * q)) & 3) * nl;
        }
        col1[3] = col2[3] = 3 * nl;
        float x0[16], x2[16], y1[16], y3[16];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int ra = 4 * col1[q] + r1, rb = 4 * col2[q] + r2;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                x0[4 * q + u] = S0[ra + col1[u]];
                x2[4 * q + u] = S2[ra + col1[u]];
                y1[4 * q + u] = S1[rb + col2[u]];
                y3[4 * q + u] = S3[rb + col2[u]];
            }
        }
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            const int mu = c >> 2, nu = c & 3;
#pragma unroll
            for (int n = 0; n < 4; ++n) {
                const int k = tri::inner(n);
                if (tri::rpa_sign(c, k) > 0) {
                    v[c] += x0[4 * mu + k] * y1[4 * k + nu];
                    v[c] += x2[4 * mu + k] * y3[4 * k + nu];
                } else {
                    v[c] -= x0[4 * mu + k] * y1[4 * k + nu];
                    v[c] -= x2[4 * mu + k] * y3[4 * k + nu];
                }
            }
        }
    }
}

// The lane-balanced walk of the RPA pairs of all sites (TriArgs::rpa_*) for the t-channel node
// whose slabs are in S: each lane sums its chunk's runs into slots (16 floats per run).
__device__ __forceinline__ void rpa_walk(const TriArgs &a, const float *S, int nl, int lane, int cnt, int base,
                                         float *slots) {
    float p[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) p[c] = 0.0f;
    int slot = base;
    for (int i = 0; i < cnt; ++i) {
        const int e = __ldg(a.rpa_sched + 32 * i + lane);
        rpa_pair(S, nl, e, p);
        if (e & (1 << 26)) {
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                slots[16 * slot + c] = p[c];
                p[c] = 0.0f;
            }
            ++slot;
        }
    }
}

// The t integrand for one site j (TRIFrgCore.cpp:733-2368): the RPA lattice sum (the site's run
// partials of rpa_walk, in order, doubled), then the chalice diagrams with the site-local values L.
__device__ __forceinline__ void t_terms(const TriArgs &a, const float *S, const float *L, const float *slots, int nl,
                                        int j, float *r) {
    const float *S0 = S, *S1 = S + 16 * nl, *S2 = S + 32 * nl, *S3 = S + 48 * nl;
    float v[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) v[c] = 0.0f;
    for (int q = a.rpa_seg_ptr[j]; q < a.rpa_seg_ptr[j + 1]; ++q)  // the site's run partials, in order
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] += slots[16 * q + c];
#pragma unroll
    for (int c = 0; c < 16; ++c) v[c] *= 2.0f;
    {  // chalice: slabs 0 and 2 with the local values of ab4, ab5.  For an inner pair (kappa,
       // lambda) the outputs (c1, c2) read the row L(lambda, .) at rho = c2 ^ kappa ^ lambda, so
       // the row is loaded once; every output still adds its terms in (kappa, lambda) order.
        float X0[16], X2[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            X0[c] = S0[c * nl + j];
            X2[c] = S2[c * nl + j];
        }
        const float4 *L4 = reinterpret_cast<const float4 *>(L), *L5 = reinterpret_cast<const float4 *>(L + 16);
#pragma unroll
        for (int n = 0; n < 16; ++n) {
            const int kap = tri::inner(n >> 2), lam = tri::inner(n & 3);
            const float4 q4 = L4[lam], q5 = L5[lam];
            const float r4[4] = {q4.x, q4.y, q4.z, q4.w}, r5[4] = {q5.x, q5.y, q5.z, q5.w};
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                const int ai = 4 * (c >> 2) + kap, rho = (c & 3) ^ kap ^ lam;
                if (tri::chal_sign(c, kap, lam) > 0) {
                    v[c] += X0[ai] * r4[rho];
                    v[c] += X2[ai] * r5[rho];
                } else {
                    v[c] -= X0[ai] * r4[rho];
                    v[c] -= X2[ai] * r5[rho];
                }
            }
        }
    }
    {  // inverse chalice: the local values of ab6, ab7 with slabs 1 and 3, each value loaded
       // once; every output adds its terms in the order l = 15 .. 0
        float X1[16], X3[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            X1[c] = S1[c * nl + j];
            X3[c] = S3[c * nl + j];
        }
#pragma unroll
        for (int n = 0; n < 16; ++n) {
            const int l = 15 - n;
            const float l6 = L[32 + l], l7 = L[48 + l];
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                const int bi = 4 * ((c >> 2) ^ (l >> 2) ^ (l & 3)) + (c & 3);
                if (tri::ichal_sign(c, l) > 0) {
                    v[c] += l6 * X1[bi];
                    v[c] += l7 * X3[bi];
                } else {
                    v[c] -= l6 * X1[bi];
                    v[c] -= l7 * X3[bi];
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 16; ++c) r[c] = v[c];
}

__host__ __device__ constexpr size_t tri_warp_floats(int nl, int n_seg) {
    return 80 * size_t(nl) + 64 + kTBatch * (sizeof(TDesc) / sizeof(float)) + 16 * size_t(n_seg);
}
// per CTA: the gather offsets goff[2][16][nl] (ints), then the warps' areas
__host__ __device__ constexpr size_t tri_cta_head_floats(int nl) { return (32 * size_t(nl) + 3) / 4 * 4; }

__global__ void __launch_bounds__(kThreads) tri_vertex_kernel(TriArgs a) {
    __shared__ float pos[kMaxFreq];
    // per CTA: gather offsets goff[2][16][nl]; per warp: slabs S[4][16][nl], accumulator
    // acc[16][nl], local values L[64], node descriptors
    extern __shared__ __align__(16) float tsm[];
    const int n = a.n, nl = a.nl;
    int *goff = reinterpret_cast<int *>(tsm);
    for (int i = threadIdx.x; i < n; i += blockDim.x) pos[i] = a.freq[i];
    for (int i = threadIdx.x; i < 32 * nl; i += blockDim.x) {
        const int e = i / (16 * nl), c = (i / nl) & 15, j = i % nl;
        const int r = e ? a.inv_sites[j] : a.sites[j], p = e ? a.inv_sites_perm[j] : a.sites_perm[j];
        goff[i] = gather_offset(e, c, nl, r, p);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *S = tsm + tri_cta_head_floats(nl) + size_t(warp) * tri_warp_floats(nl, a.rpa_n_seg);
    float *acc = S + 64 * nl;
    float *L = acc + 16 * nl;
    TDesc *desc = reinterpret_cast<TDesc *>(L + 64);
    float *slots = reinterpret_cast<float *>(desc + kTBatch);
    const int rpa_cnt = a.rpa_count[lane], rpa_base = a.rpa_slot_base[lane];
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
        for (int q = lane; q < 16 * nl; q += 32) acc[q] = 0.0f;
        __syncwarp();
        for (int ch = 0; ch < 3; ++ch) {
            const int xi = ch == 0 ? si : (ch == 1 ? ti : ui);
            const int cnt = a.node_cnt[xi];
            const float *nwp = a.node_wp + size_t(xi) * a.max_nodes;
            const float *nc = a.node_c + size_t(xi) * a.max_nodes;
            for (int b0 = 0; b0 < cnt; b0 += kTBatch) {
                const int nb = min(kTBatch, cnt - b0);
                if ((lane >> 2) < nb) {  // phase A: a quad of lanes per node
                    const int k = lane >> 2;
                    make_tpart(a, pos, ch, xi, s, t, u, w1p, w1, w2p, w2, nwp[b0 + k], lane & 3, desc[k]);
                    if ((lane & 3) == 0) desc[k].c = nc[b0 + k];
                }
                __syncwarp();
                for (int b = 0; b < nb; ++b) {
                    const TDesc &d = desc[b];
                    // gather the four slabs of all sites
#pragma unroll 1
                    for (int q = 0; q < 4; ++q) gather_slab(a.v4, d.ab[q], goff, nl, lane, S + q * 16 * nl);
                    if (ch == 1)
                        for (int q = lane; q < 64; q += 32) L[q] = tri_local(a.v4, nl, d.ab[4 + (q >> 4)], (q & 15) >> 2, q & 3);
                    __syncwarp();
                    if (ch == 1) {
                        rpa_walk(a, S, nl, lane, rpa_cnt, rpa_base, slots);
                        __syncwarp();
                    }
                    const float cw = d.c;
                    for (int j = lane; j < nl; j += 32) {
                        float r[16];
                        if (ch == 0) ladder<false>(S, nl, j, r);
                        else if (ch == 2) ladder<true>(S, nl, j, r);
                        else t_terms(a, S, L, slots, nl, j, r);
#pragma unroll
                        for (int c = 0; c < 16; ++c) acc[c * nl + j] += cw * r[c];
                    }
                    __syncwarp();
                }
            }
        }
        float *dst = a.dv4 + size_t(it) * 16 * nl;
        bool bad = false;
        for (int q = lane; q < 16 * nl; q += 32) {
            const float o = acc[q] / two_pi;
            dst[q] = o;
            bad |= isnan(o);
        }
        if (bad) atomicOr(a.status, kStatusNaN);
        __syncwarp();
    }
}

// ------------------------------------------------------------------------------------
// correlation measurement at nu = 0 (TRIMeasurementCorrelation.cpp:147-285): one CTA per
// outer node accumulates the inner integral per site and component in FP64, a final CTA adds
// the outer weights and the on-site term and scatters to (basis, site in range) entries.
// ------------------------------------------------------------------------------------
__constant__ int kOutComp[kCorrOut] = {0, 1, 2, 4, 5, 6, 8, 9, 10, 15};

__global__ void __launch_bounds__(128) tri_corr_inner_kernel(TriArgs a) {
    __shared__ float pos[kMaxFreq];
    __shared__ float nwp[kMaxCorrNodes];
    __shared__ double nw[kMaxCorrNodes];
    __shared__ int ncnt;
    extern __shared__ double red[];  // [kWarps][kCorrOut][nl]
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    if (threadIdx.x == 0) ncnt = corr_nodes(pos, a.n, a.cutoff, nwp, nw);
    __syncthreads();
    const int ia = blockIdx.x;
    if (ia >= ncnt) return;
    const float w = nwp[ia];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nl = a.nl;
    const double dw = double(w) + odd_interp(pos, a.n, a.v2, w);
    for (int j0 = 0; j0 < nl; j0 += 32) {
        const int j = j0 + lane;
        const bool valid = j < nl;
        const int r0 = valid ? a.sites[j] : 0, p0 = valid ? a.sites_perm[j] : 0;
        const int r1 = valid ? a.inv_sites[j] : 0, p1 = valid ? a.inv_sites_perm[j] : 0;
        double acc[kCorrOut];
#pragma unroll
        for (int q = 0; q < kCorrOut; ++q) acc[q] = 0.0;
        for (int b = warp; b < ncnt; b += kWarps) {
            const float wp = nwp[b];
            TAB8 ab, ab1;
            tri_access8(pos, a.n, nl, w + wp + 0.0f, 0.0f, w - wp, ab);
            const double dwp = double(wp) + odd_interp(pos, a.n, a.v2, wp);
            const double cw = nw[b] / (dw * dw * dwp * dwp * (4.0 * kPiD * kPiD));
            if (!valid) continue;
            const bool ex = ab.fl & kFlExch;
            double rr[kCorrOut];
#pragma unroll
            for (int q = 0; q < kCorrOut; ++q) {
                const int c = kOutComp[q];
                const float g = tri_bundle(a.v4, nl, ab, c, ex ? r1 : r0, ex ? p1 : p0);
                rr[q] = c == 15 ? -4.0 * double(g) : -double(g);  // dumbbell
            }
            if (j == 0) {  // egg diagram, TRIMeasurementCorrelation.cpp:211-251
                tri_access8(pos, a.n, nl, w + wp + 0.0f, w - wp, 0.0f, ab1);
#pragma unroll
                for (int q = 0; q < kCorrOut; ++q) {
                    const int c = kOutComp[q];
                    const double f = c == 15 ? 2.0 : 0.5;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int lam = tri::inner(k), rho = (c >> 2) ^ (c & 3) ^ lam;
                        const int sg = tri::egg_sign(c, lam);
                        if (sg != 0) rr[q] += f * sg * double(tri_local(a.v4, nl, ab1, lam, rho));
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kCorrOut; ++q) acc[q] += cw * rr[q];
        }
        if (valid)
            for (int q = 0; q < kCorrOut; ++q) red[(size_t(warp) * kCorrOut + q) * nl + j] = acc[q];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kCorrOut * nl; e += blockDim.x) {
        double sum = 0.0;
        for (int q = 0; q < kWarps; ++q) sum += red[size_t(q) * kCorrOut * nl + e];
        a.partial[size_t(ia) * kCorrOut * nl + e] = sum;
    }
}

__global__ void tri_corr_final_kernel(TriArgs a) {
    __shared__ float pos[kMaxFreq];
    __shared__ float nwp[kMaxCorrNodes];
    __shared__ double nw[kMaxCorrNodes];
    __shared__ int ncnt;
    extern __shared__ double chi[];  // [16][nl]
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    if (threadIdx.x == 0) ncnt = corr_nodes(pos, a.n, a.cutoff, nwp, nw);
    __syncthreads();
    const int nl = a.nl;
    for (int e = threadIdx.x; e < 16 * nl; e += blockDim.x) chi[e] = 0.0;
    __syncthreads();
    for (int e = threadIdx.x; e < kCorrOut * nl; e += blockDim.x) {
        const int q = e / nl, j = e - q * nl, c = kOutComp[q];
        double sum = 0.0;
        for (int ia = 0; ia < ncnt; ++ia) {
            double v = a.partial[size_t(ia) * kCorrOut * nl + e];
            if (j == 0 && (c == 0 || c == 5 || c == 10 || c == 15)) {  // on-site term
                const float w = nwp[ia];
                const double dw = double(w) + odd_interp(pos, a.n, a.v2, w);
                const double t1 = 1.0 / (dw * dw);
                v += c == 15 ? t1 / kPiD : t1 / (4.0 * kPiD);
            }
            sum += nw[ia] * v;
        }
        chi[c * nl + j] = sum;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 16 * nl; e += blockDim.x) a.out[size_t(kCorrOut) * a.n_corr + e] = float(chi[e]);
    for (int q = threadIdx.x; q < a.n_corr; q += blockDim.x) {
        const int r = a.corr_rid[q], p = a.corr_perm[q];
        int k = 0;
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y, ++k)
                a.out[size_t(k) * a.n_corr + q] = float(chi[(4 * permc(p, x) + permc(p, y)) * nl + r]);
        a.out[size_t(9) * a.n_corr + q] = float(chi[15 * nl + r]);
    }
}

__global__ void tri_euler_kernel(float *__restrict__ x, const float *__restrict__ dx, long long n, float step) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = __fadd_rn(x[i], __fmul_rn(step, dx[i]));
}

using cuh::check_cuda;
using cuh::copy_grid;
using cuh::dalloc;
using cuh::h2d;

size_t vertex_smem(int nl, int n_seg) {
    return (tri_cta_head_floats(nl) + size_t(kWarps) * tri_warp_floats(nl, n_seg)) * sizeof(float);
}

}  // namespace

struct spn_tri {
    int device = 0, n = 0, nl = 0, n_range = 0, n_corr = 0, n_overlap = 0, max_nodes = 0, sms = 0, grid = 0;
    long long fn = 0;
    float cutoff = 0.0f;
    cudaStream_t stream = nullptr;
    float *freq = nullptr, *v2 = nullptr, *dv2 = nullptr, *v4 = nullptr, *dv4 = nullptr, *node_wp = nullptr,
          *node_c = nullptr, *corr_out = nullptr;
    int *ints = nullptr;  // all integer tables in one allocation
    int *sites, *sites_perm, *inv_sites, *inv_sites_perm, *range_rid, *range_inv, *corr_rid,
        *corr_perm, *node_cnt, *work_counter, *rpa_sched, *rpa_count, *rpa_slot_base, *rpa_seg_ptr;
    int rpa_n_seg = 0;
    unsigned *status = nullptr;
    double *partial = nullptr;

    long long vsize() const { return 16 * fn * nl; }

    TriArgs args() const {
        TriArgs a;
        a.n = n;
        a.nl = nl;
        a.fn = int(fn);
        a.max_nodes = max_nodes;
        a.n_range = n_range;
        a.n_corr = n_corr;
        a.cutoff = cutoff;
        a.freq = freq;
        a.v4 = v4;
        a.dv4 = dv4;
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
        void *ptrs[] = {freq, v2, dv2, v4, dv4, node_wp, node_c, corr_out, ints, status, partial};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

void validate(const spn_tri_desc *d) {
    if (!d) throw Error(ErrorType::Argument, "null descriptor");
    if (d->n_freq < 2 || d->n_freq > kMaxFreq)
        throw Error(ErrorType::Unsupported, "n_freq must be in [2, " + std::to_string(kMaxFreq) + "]");
    if (d->n_sites < 1 || d->n_sites > kMaxSites)
        throw Error(ErrorType::Unsupported, "n_sites must be in [1, " + std::to_string(kMaxSites) + "]");
    if (!d->freq || !d->sites_rid || !d->sites_perm || !d->inv_sites_rid || !d->inv_sites_perm || !d->overlap_ptr ||
        (d->n_range > 0 && (!d->range_rid || !d->range_inv_rid)) || (d->n_corr > 0 && (!d->corr_rid || !d->corr_perm)))
        throw Error(ErrorType::Argument, "descriptor table pointer is NULL");
    for (int i = 0; i < d->n_freq; ++i) {
        if (!(d->freq[i] > 0.0f)) throw Error(ErrorType::Argument, "frequencies must be positive");
        if (i > 0 && !(d->freq[i] > d->freq[i - 1])) throw Error(ErrorType::Argument, "frequencies must be strictly ascending");
    }
    const long long fn = (long long)d->n_freq * d->n_freq * (d->n_freq + 1) / 2;
    if (16 * fn * d->n_sites >= (1ll << 31)) throw Error(ErrorType::Unsupported, "vertex larger than 2^31 elements");
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

// The RPA pairs of each site in the order of host/pair_order (against bank collisions of the
// kernel's shared-memory reads), packed as the words of TriArgs::rpa_sched.
std::vector<int> order_rpa_pairs(const spn_tri_desc *d) {
    const int nl = d->n_sites;
    const std::vector<int> order =
        order_pairs_by_banks(nl, d->overlap_ptr, tri_rpa_model(),
                             tri_rpa_words(nl, d->overlap_rid1, d->overlap_rid2, d->overlap_perm1, d->overlap_perm2));
    std::vector<int> out(order.size());
    for (size_t k = 0; k < order.size(); ++k) {
        const int i = order[k];
        int word = d->overlap_rid1[i] | d->overlap_rid2[i] << 7;
        for (int q = 0; q < 3; ++q)
            word |= permc(d->overlap_perm1[i], q) << (14 + 2 * q) | permc(d->overlap_perm2[i], q) << (20 + 2 * q);
        out[k] = word;
    }
    return out;
}

void launch_correlation(spn_tri *h) {
    const TriArgs a = h->args();
    tri_corr_inner_kernel<<<2 * h->n + 4, 128, size_t(kWarps) * kCorrOut * h->nl * sizeof(double), h->stream>>>(a);
    check_cuda(cudaGetLastError(), "correlation launch");
    tri_corr_final_kernel<<<1, 128, 16 * h->nl * sizeof(double), h->stream>>>(a);
    check_cuda(cudaGetLastError(), "correlation final launch");
}

}  // namespace

extern "C" int spn_tri_create(const spn_tri_desc *d, spn_tri **out) {
    return guarded([&] {
        if (!out) throw Error(ErrorType::Argument, "null output handle");
        validate(d);
        auto *h = new spn_tri;
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
            const size_t vsz = size_t(h->vsize());
            h->freq = dalloc<float>(h->n, "alloc freq");
            h->v2 = dalloc<float>(h->n, "alloc v2");
            h->dv2 = dalloc<float>(h->n, "alloc dv2");
            h->v4 = dalloc<float>(vsz, "alloc vertex state");
            h->dv4 = dalloc<float>(vsz, "alloc vertex flow");
            h->node_wp = dalloc<float>(size_t(h->n) * h->max_nodes, "alloc node table");
            h->node_c = dalloc<float>(size_t(h->n) * h->max_nodes, "alloc node table");
            h->corr_out = dalloc<float>(size_t(kCorrOut) * h->n_corr + 16 * h->nl, "alloc correlation output");
            h->partial = dalloc<double>(size_t(kMaxCorrNodes) * kCorrOut * h->nl, "alloc correlation scratch");
            h->status = dalloc<unsigned>(1, "alloc status");
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
            const LaneSchedule rpa = tri_lane_schedule(nl, d->overlap_ptr, packed);
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
            int **fields[] = {&h->sites, &h->sites_perm, &h->inv_sites, &h->inv_sites_perm,
                              &h->range_rid, &h->range_inv, &h->corr_rid, &h->corr_perm, &h->node_cnt, &h->work_counter,
                              &h->rpa_sched, &h->rpa_count, &h->rpa_slot_base, &h->rpa_seg_ptr};
            for (size_t k = 0; k < at.size(); ++k) *fields[k] = h->ints + at[k];
            h2d(h->freq, d->freq, h->n, h->stream);
            check_cuda(cudaMemsetAsync(h->v4, 0, vsz * sizeof(float), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->dv4, 0, vsz * sizeof(float), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->v2, 0, h->n * sizeof(float), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->dv2, 0, h->n * sizeof(float), h->stream), "memset");
            check_cuda(cudaMemsetAsync(h->status, 0, sizeof(unsigned), h->stream), "memset");
            check_cuda(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device), "device attribute");
            int per_sm = 0;
            check_cuda(cudaFuncSetAttribute(tri_vertex_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            int(vertex_smem(h->nl, h->rpa_n_seg))),
                       "shared memory limit");
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tri_vertex_kernel, kThreads, vertex_smem(h->nl, h->rpa_n_seg)),
                       "occupancy");
            if (per_sm < 1) throw Error(ErrorType::Unsupported, "TRI vertex-flow kernel does not fit on this device");
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

extern "C" int spn_tri_destroy(spn_tri *h) {
    if (!h) return SPN_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->release();
    delete h;
    return SPN_OK;
}

extern "C" int spn_tri_set_state(spn_tri *h, float cutoff, const float *v2, const float *v4) {
    return guarded([&] {
        if (!h || !v2 || !v4) throw Error(ErrorType::Argument, "null argument");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        h2d(h->v4, v4, size_t(h->vsize()), h->stream);
        h2d(h->v2, v2, h->n, h->stream);
        h->cutoff = cutoff;
        check_cuda(cudaStreamSynchronize(h->stream), "set_state sync");
    });
}

extern "C" int spn_tri_get_state(spn_tri *h, float *cutoff, float *v2, float *v4) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        if (cutoff) *cutoff = h->cutoff;
        if (v2) check_cuda(cudaMemcpyAsync(v2, h->v2, h->n * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        if (v4)
            check_cuda(cudaMemcpyAsync(v4, h->v4, size_t(h->vsize()) * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        check_cuda(cudaStreamSynchronize(h->stream), "get_state sync");
    });
}

extern "C" int spn_tri_get_flow(spn_tri *h, float *dv2, float *dv4) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        if (dv2) check_cuda(cudaMemcpyAsync(dv2, h->dv2, h->n * sizeof(float), cudaMemcpyDeviceToHost, h->stream), "D2H");
        if (dv4)
            check_cuda(cudaMemcpyAsync(dv4, h->dv4, size_t(h->vsize()) * sizeof(float), cudaMemcpyDeviceToHost, h->stream),
                       "D2H");
        check_cuda(cudaStreamSynchronize(h->stream), "get_flow sync");
    });
}

extern "C" int spn_tri_compute_step(spn_tri *h) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        check_cuda(cudaMemsetAsync(h->status, 0, sizeof(unsigned), h->stream), "memset status");
        check_cuda(cudaMemsetAsync(h->work_counter, 0, sizeof(int), h->stream), "memset counter");
        const TriArgs a = h->args();
        tri_self_energy_kernel<<<h->n, 128, 0, h->stream>>>(a);
        check_cuda(cudaGetLastError(), "self-energy launch");
        tri_node_table_kernel<<<(h->n + 63) / 64, 64, 0, h->stream>>>(h->node_args());
        check_cuda(cudaGetLastError(), "node table launch");
        check_cuda(cudaFuncSetAttribute(tri_vertex_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(vertex_smem(h->nl, h->rpa_n_seg))),
                   "shared memory limit");
        tri_vertex_kernel<<<h->grid, kThreads, vertex_smem(h->nl, h->rpa_n_seg), h->stream>>>(a);
        check_cuda(cudaGetLastError(), "vertex flow launch");
    });
}

extern "C" int spn_tri_finalize_step(spn_tri *h, float new_cutoff) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        const float step = new_cutoff - h->cutoff;
        tri_euler_kernel<<<1, 64, 0, h->stream>>>(h->v2, h->dv2, h->n, step);
        tri_euler_kernel<<<copy_grid(h->vsize()), 256, 0, h->stream>>>(h->v4, h->dv4, h->vsize(), step);
        check_cuda(cudaGetLastError(), "euler launch");
        h->cutoff = new_cutoff;
    });
}

extern "C" int spn_tri_measure_correlation(spn_tri *h, float *corr, float *chi) {
    return guarded([&] {
        if (!h) throw Error(ErrorType::Argument, "null handle");
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        launch_correlation(h);
        if (corr)
            check_cuda(cudaMemcpyAsync(corr, h->corr_out, size_t(kCorrOut) * h->n_corr * sizeof(float), cudaMemcpyDeviceToHost,
                                       h->stream),
                       "D2H");
        if (chi)
            check_cuda(cudaMemcpyAsync(chi, h->corr_out + size_t(kCorrOut) * h->n_corr, 16 * h->nl * sizeof(float),
                                       cudaMemcpyDeviceToHost, h->stream),
                       "D2H");
        check_cuda(cudaStreamSynchronize(h->stream), "correlation sync");
    });
}

extern "C" int spn_tri_is_diverged(spn_tri *h, int *diverged) {
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

extern "C" int spn_tri_vertex_probe(const float *pos, int n, int n_sites, const float *v4, int rid12, int rid21,
                                    int perm12, int perm21, float s, float t, float u, int channel, int local,
                                    float *value) {
    return guarded([&] {
        cuh::check_mesh(pos, n, kMaxFreq);
        if (n_sites < 1 || n_sites > kMaxSites || !v4 || !value || rid12 < 0 || rid12 >= n_sites || rid21 < 0 ||
            rid21 >= n_sites || perm12 < 0 || perm12 > 5 || perm21 < 0 || perm21 > 5 || channel < -1 || channel > 3 ||
            (channel < 0 && (local || perm12 || perm21)))
            throw Error(ErrorType::Argument, "spn_tri_vertex_probe: bad argument");
        const int nl = n_sites;
        if (channel < 0) {
            for (int c = 0; c < 16; ++c) value[c] = tri_value_none(pos, n, nl, v4, c >> 2, c & 3, rid12, rid21, s, t, u);
            return;
        }
        if (channel == 3) {
            TAB8 ab;
            tri_access8(pos, n, nl, s, t, u, ab);
            const bool ex = ab.fl & kFlExch;
            for (int c = 0; c < 16; ++c)
                value[c] = local ? tri_local(v4, nl, ab, c >> 2, c & 3)
                                 : tri_bundle(v4, nl, ab, c, ex ? rid21 : rid12, ex ? perm21 : perm12);
            return;
        }
        // the channel's own frequency is a mesh value; the two others are interpolated in the
        // order tri_access4i takes them (t, u for S; s, u for T; s, t for U)
        const MeshSearch<float> m{pos, n};
        const float own[3] = {s, t, u};
        const int e = cuh::mesh_index_of(pos, n, own[channel]);
        const Interp<float> ia = interp_abs(m, channel == 0 ? t : s), ib = interp_abs(m, channel == 2 ? t : u);
        TAB4 ab;
        if (channel == 0) tri_access4i<kS>(n, nl, s, t, u, e, ia, ib, ab);
        else if (channel == 1) tri_access4i<kT>(n, nl, s, t, u, e, ia, ib, ab);
        else tri_access4i<kU>(n, nl, s, t, u, e, ia, ib, ab);
        if (local) {
            for (int c = 0; c < 16; ++c) value[c] = tri_local(v4, nl, ab, c >> 2, c & 3);
            return;
        }
        // the vertex kernel's slab gather, every site of the table standing for the probed pair
        std::vector<int> goff(32 * size_t(nl));
        for (int i = 0; i < 32 * nl; ++i) {
            const int ex = i / (16 * nl), c = (i / nl) & 15;
            goff[i] = gather_offset(ex, c, nl, ex ? rid21 : rid12, ex ? perm21 : perm12);
        }
        std::vector<float> S(16 * size_t(nl));
        gather_slab(v4, ab, goff.data(), nl, 0, S.data());
        for (int c = 0; c < 16; ++c) value[c] = S[size_t(c) * nl];
    });
}
