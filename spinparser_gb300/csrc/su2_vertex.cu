// Two-particle vertex flow of the SU(2) pf-FRG right-hand side on sm_103a
// (SU2FrgCore::_calculateVertexTwoParticle, src/SU2/SU2FrgCore.cpp:171-431).
//
// For one frequency triple (s,t,u) the flow is
//   sum over channels X in {s,t,u} of sum over loop-frequency nodes (wp, c) of c * K_X(wp)
// where the node lists (conventional terms at wp = +-Lambda and the trapezoid nodes of the
// Katanin integrals, with propagators folded into c) depend only on the channel's transfer
// frequency and are built per step by su2_node_table_kernel.
//
// Work distribution: a persistent grid; each warp pulls triples from a device atomic
// counter.  For a triple and channel, nodes are handled in batches of 32:
//   phase A, lane = node: the node's interpolation supports (access buffers: folding, mesh
//            searches, weights) are computed once and written to shared memory as a
//            NodeDesc; for the t channel the four site-local vertex values are gathered too;
//   phase B, lane = (node group, site): each group of W lanes (W = next power of two >= Nl)
//            takes one node at a time, reads its descriptor (broadcast), gathers the four
//            interpolated vertex slabs for its sites (coalesced: a slab is Nl contiguous
//            floats) and forms K_X.
// The t channel's RPA lattice sum sum_i A[rid1_i] B[rid2_i] (A, B: the third and fourth slab
// of the node) is linear in the node, so for Nl <= 32 the warp first accumulates the matrix
//   M = sum over the channel's nodes of (c A) x B        (Nl x Nl, spin and density)
// in registers -- the 32 lanes own an 8 x 4 grid of blocks, updated with packed f32x2 FMAs
// from a per-node shared-memory panel -- and then walks the merged pair list once per triple,
// sum m M[rid1][rid2] per rid (every (rid1, rid2) occurs: the pair matrix is dense).  For
// Nl > 32 each node walks the merged pair list itself.  Both walks follow a lane-balanced
// schedule with deterministic segment partials (no divergent per-rid loops).
// Accumulation over nodes is Kahan-compensated FP32 for the local terms (the RPA matrix sums
// are plain FP32); group partials are combined by shuffles.
#include <type_traits>
#include "su2_common.cuh"
#include "su2_device.cuh"

namespace spn {
namespace {

using namespace spn::dev;

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kBatch = 32;  // nodes whose descriptors a warp builds at once (phase A)
constexpr double kPi = 3.14159265358979323846;

struct __align__(16) NodeDesc {
    int4 off[4];
    float4 w[4];  // per buffer: the four interpolation weights
    int exch;  // bit i: buffer i reads the site-exchanged pairs (inverted sites); bit 4 + 4i + q:
               // support q of buffer i is a swapped (s < u) slab, whose density weight is -w
    float c;   // node coefficient, channel sign included
    float lv[8];  // t channel: site-local values cbs, cbd, icas, icad, cbs2, cbd2, icas2, icad2
    int pad[2];
};
static_assert(sizeof(NodeDesc) % 16 == 0, "NodeDesc must stay 16-byte aligned");

template <int SPT>
struct Lane {
    int site[SPT], isite[SPT], j[SPT];
    bool valid[SPT];
};

struct Transfer {
    float s, t, u, w1p, w1, w2p, w2;
    int si, ti, ui;  // mesh indices of s, t, u: the channel coordinate's offset in every buffer
};

// Packed single-precision pairs (fma.rn.f32x2): per element the same IEEE round-to-nearest
// result as fmaf.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 x, y, z, w;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\tmov.b64 z, {%6, %7};\n\t"
        "fma.rn.f32x2 w, x, y, z;\n\tmov.b64 {%0, %1}, w;\n}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

// Stores buffer i of a node; returns its sign bits (bit 4 + 4i + q set when sw[q] = -w[q], the
// density weight of a swapped slab; sw is exactly +-w, so the pair is rebuilt without loss).
__device__ __forceinline__ int put_ab(NodeDesc &d, int i, const AB4 &ab) {
    d.off[i] = make_int4(ab.off[0], ab.off[1], ab.off[2], ab.off[3]);
    d.w[i] = make_float4(ab.w[0], ab.w[1], ab.w[2], ab.w[3]);
    int bits = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) bits |= int(__float_as_int(ab.sw[q]) != __float_as_int(ab.w[q])) << q;
    return bits << (4 + 4 * i);
}

// (w, sign * w) of support q from the weight and the descriptor's sign bit.
__device__ __forceinline__ float2 wpair(float w, int exch, int bit) {
    return make_float2(w, __int_as_float(__float_as_int(w) ^ (((exch >> bit) & 1) << 31)));
}

// Site-local (rid 0) (spin, density) value of an access buffer: spin sum w * ss, density sum
// (sign * w) * dd, one packed FMA per support.
__device__ __forceinline__ void local_pair(const FlowArgs &a, const AB4 &ab, float &vs, float &vd) {
    float2 g = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int q = 0; q < 4; ++q) g = fma2(make_float2(ab.w[q], ab.sw[q]), __ldg(a.sd + ab.off[q]), g);
    vs = g.x;
    vd = g.y;
}

// Phase A: descriptor of one node (lane = node).  The node's access buffers interpolate four
// distinct magnitudes (interp_abs), each looked up once; folding, weights and offsets are
// access4m's, so the descriptor is the one eight (s, u) or sixteen (t) separate lookups give.
template <int CH>
__device__ __forceinline__ void make_desc(const FlowArgs &a, const float *pos, const Transfer &f, float wp, float c,
                                          NodeDesc &d) {
    AB4 ab;
    int exch = 0;
    const int nl = a.nl, n = a.n;
    const MeshIndex m{pos, a.n, a.mesh_lo, a.mesh_base, a.mesh_shift};
    if (CH == kS) {  // integralKernelS, SU2FrgCore.cpp:202-206
        {  // buffers 0 and 2 interpolate |w1 + wp| and |w2 + wp|
            const Interp<float> iA = interp_abs(m, f.w1 + wp), iB = interp_abs(m, f.w2 + wp);
            access4i<kS>(n, nl, f.s, -f.w1 - wp, -f.w2 - wp, iA, iB, f.si, ab); exch |= put_ab(d, 0, ab) | (int(ab.exch) << 0);
            access4i<kS>(n, nl, f.s, f.w2 + wp, f.w1 + wp, iB, iA, f.si, ab); exch |= put_ab(d, 2, ab) | (int(ab.exch) << 2);
        }
        {  // buffers 1 and 3: |w1p + wp| and |w2p + wp|
            const Interp<float> iP = interp_abs(m, f.w1p + wp), iQ = interp_abs(m, f.w2p + wp);
            access4i<kS>(n, nl, f.s, f.w1p + wp, -f.w2p - wp, iP, iQ, f.si, ab); exch |= put_ab(d, 1, ab) | (int(ab.exch) << 1);
            access4i<kS>(n, nl, f.s, -f.w2p - wp, f.w1p + wp, iQ, iP, f.si, ab); exch |= put_ab(d, 3, ab) | (int(ab.exch) << 3);
        }
    } else if (CH == kT) {  // integralKernelT, SU2FrgCore.cpp:233-239, 269-284
        float v0, v1;
        {  // buffers 0, 2 and local buffers 1, 3: |w1 - wp| and |w1p + wp|
            const Interp<float> iC = interp_abs(m, f.w1 - wp), iP = interp_abs(m, f.w1p + wp);
            access4i<kT>(n, nl, f.w1 - wp, f.t, f.w1p + wp, iC, iP, f.ti, ab); exch |= put_ab(d, 0, ab) | (int(ab.exch) << 0);
            access4i<kT>(n, nl, f.w1p + wp, f.t, f.w1 - wp, iP, iC, f.ti, ab); exch |= put_ab(d, 2, ab) | (int(ab.exch) << 2);
            access4i<kU>(n, nl, f.w1 - wp, -f.w1p - wp, -f.t, iC, iP, f.ti, ab); local_pair(a, ab, v0, v1); d.lv[2] = v0; d.lv[3] = v1;
            access4i<kU>(n, nl, f.w1p + wp, wp - f.w1, -f.t, iP, iC, f.ti, ab); local_pair(a, ab, v0, v1); d.lv[6] = v0; d.lv[7] = v1;
        }
        {  // buffers 1, 3 and local buffers 0, 2: |w2p - wp| and |w2 + wp|
            const Interp<float> iD = interp_abs(m, f.w2p - wp), iB = interp_abs(m, f.w2 + wp);
            access4i<kT>(n, nl, f.w2p - wp, f.t, -f.w2 - wp, iD, iB, f.ti, ab); exch |= put_ab(d, 1, ab) | (int(ab.exch) << 1);
            access4i<kT>(n, nl, f.w2 + wp, f.t, wp - f.w2p, iB, iD, f.ti, ab); exch |= put_ab(d, 3, ab) | (int(ab.exch) << 3);
            access4i<kU>(n, nl, f.w2p - wp, -f.w2 - wp, f.t, iD, iB, f.ti, ab); local_pair(a, ab, v0, v1); d.lv[0] = v0; d.lv[1] = v1;
            access4i<kU>(n, nl, f.w2 + wp, wp - f.w2p, f.t, iB, iD, f.ti, ab); local_pair(a, ab, v0, v1); d.lv[4] = v0; d.lv[5] = v1;
        }
    } else {  // integralKernelU, SU2FrgCore.cpp:309-313
        {  // buffers 0 and 2: |w1 + wp| and |w2p - wp|
            const Interp<float> iA = interp_abs(m, f.w1 + wp), iD = interp_abs(m, f.w2p - wp);
            access4i<kU>(n, nl, f.w1 + wp, wp - f.w2p, f.u, iA, iD, f.ui, ab); exch |= put_ab(d, 0, ab) | (int(ab.exch) << 0);
            access4i<kU>(n, nl, f.w2p - wp, -f.w1 - wp, f.u, iD, iA, f.ui, ab); exch |= put_ab(d, 2, ab) | (int(ab.exch) << 2);
        }
        {  // buffers 1 and 3: |w1p + wp| and |w2 - wp|
            const Interp<float> iP = interp_abs(m, f.w1p + wp), iE = interp_abs(m, f.w2 - wp);
            access4i<kU>(n, nl, f.w1p + wp, f.w2 - wp, f.u, iP, iE, f.ui, ab); exch |= put_ab(d, 1, ab) | (int(ab.exch) << 1);
            access4i<kU>(n, nl, f.w2 - wp, f.w1p + wp, f.u, iE, iP, f.ui, ab); exch |= put_ab(d, 3, ab) | (int(ab.exch) << 3);
        }
    }
    d.exch = exch;
    d.c = c;
}

// Supports of the four site-local access buffers of a t-channel node (the values cbs ... icad2
// of make_desc are local_pair of these with a flow's state).
struct LocDesc {
    int4 off[4];
    float4 w[4];
    float4 sw[4];
};

// Phase A for flows that share the mesh, the lattice tables and the cutoff (a grouped batch):
// the node's supports only, as make_desc builds them (same access buffers, same arguments);
// the coefficient and the t channel's site-local values are per flow (group_local_values).
template <int CH>
__device__ __forceinline__ void make_supports(const FlowArgs &a, const float *pos, const Transfer &f, float wp, NodeDesc &d,
                                              LocDesc &loc) {
    AB4 ab;
    int exch = 0;
    const int nl = a.nl, n = a.n;
    const MeshIndex m{pos, a.n, a.mesh_lo, a.mesh_base, a.mesh_shift};
    if (CH == kS) {
        {  // buffers 0 and 2 interpolate |w1 + wp| and |w2 + wp|
            const Interp<float> iA = interp_abs(m, f.w1 + wp), iB = interp_abs(m, f.w2 + wp);
            access4i<kS>(n, nl, f.s, -f.w1 - wp, -f.w2 - wp, iA, iB, f.si, ab); exch |= put_ab(d, 0, ab) | (int(ab.exch) << 0);
            access4i<kS>(n, nl, f.s, f.w2 + wp, f.w1 + wp, iB, iA, f.si, ab); exch |= put_ab(d, 2, ab) | (int(ab.exch) << 2);
        }
        {  // buffers 1 and 3: |w1p + wp| and |w2p + wp|
            const Interp<float> iP = interp_abs(m, f.w1p + wp), iQ = interp_abs(m, f.w2p + wp);
            access4i<kS>(n, nl, f.s, f.w1p + wp, -f.w2p - wp, iP, iQ, f.si, ab); exch |= put_ab(d, 1, ab) | (int(ab.exch) << 1);
            access4i<kS>(n, nl, f.s, -f.w2p - wp, f.w1p + wp, iQ, iP, f.si, ab); exch |= put_ab(d, 3, ab) | (int(ab.exch) << 3);
        }
    } else if (CH == kT) {
        auto put_loc = [&](int i) {
            loc.off[i] = make_int4(ab.off[0], ab.off[1], ab.off[2], ab.off[3]);
            loc.w[i] = make_float4(ab.w[0], ab.w[1], ab.w[2], ab.w[3]);
            loc.sw[i] = make_float4(ab.sw[0], ab.sw[1], ab.sw[2], ab.sw[3]);
        };
        {
            const Interp<float> iC = interp_abs(m, f.w1 - wp), iP = interp_abs(m, f.w1p + wp);
            access4i<kT>(n, nl, f.w1 - wp, f.t, f.w1p + wp, iC, iP, f.ti, ab); exch |= put_ab(d, 0, ab) | (int(ab.exch) << 0);
            access4i<kT>(n, nl, f.w1p + wp, f.t, f.w1 - wp, iP, iC, f.ti, ab); exch |= put_ab(d, 2, ab) | (int(ab.exch) << 2);
            access4i<kU>(n, nl, f.w1 - wp, -f.w1p - wp, -f.t, iC, iP, f.ti, ab); put_loc(1);
            access4i<kU>(n, nl, f.w1p + wp, wp - f.w1, -f.t, iP, iC, f.ti, ab); put_loc(3);
        }
        {
            const Interp<float> iD = interp_abs(m, f.w2p - wp), iB = interp_abs(m, f.w2 + wp);
            access4i<kT>(n, nl, f.w2p - wp, f.t, -f.w2 - wp, iD, iB, f.ti, ab); exch |= put_ab(d, 1, ab) | (int(ab.exch) << 1);
            access4i<kT>(n, nl, f.w2 + wp, f.t, wp - f.w2p, iB, iD, f.ti, ab); exch |= put_ab(d, 3, ab) | (int(ab.exch) << 3);
            access4i<kU>(n, nl, f.w2p - wp, -f.w2 - wp, f.t, iD, iB, f.ti, ab); put_loc(0);
            access4i<kU>(n, nl, f.w2 + wp, wp - f.w2p, f.t, iB, iD, f.ti, ab); put_loc(2);
        }
    } else {
        {  // buffers 0 and 2: |w1 + wp| and |w2p - wp|
            const Interp<float> iA = interp_abs(m, f.w1 + wp), iD = interp_abs(m, f.w2p - wp);
            access4i<kU>(n, nl, f.w1 + wp, wp - f.w2p, f.u, iA, iD, f.ui, ab); exch |= put_ab(d, 0, ab) | (int(ab.exch) << 0);
            access4i<kU>(n, nl, f.w2p - wp, -f.w1 - wp, f.u, iD, iA, f.ui, ab); exch |= put_ab(d, 2, ab) | (int(ab.exch) << 2);
        }
        {  // buffers 1 and 3: |w1p + wp| and |w2 - wp|
            const Interp<float> iP = interp_abs(m, f.w1p + wp), iE = interp_abs(m, f.w2 - wp);
            access4i<kU>(n, nl, f.w1p + wp, f.w2 - wp, f.u, iP, iE, f.ui, ab); exch |= put_ab(d, 1, ab) | (int(ab.exch) << 1);
            access4i<kU>(n, nl, f.w2 - wp, f.w1p + wp, f.u, iE, iP, f.ui, ab); exch |= put_ab(d, 3, ab) | (int(ab.exch) << 3);
        }
    }
    d.exch = exch;
    d.c = 0.0f;
}

// make_supports split over the four threads of a quad (q = 0..3), for a CTA that builds 32
// nodes with 128 threads.  Thread q builds main buffer b(q) and, in the t channel, local buffer
// l(q), from the two magnitudes (y1, y2) that those buffers interpolate; the coordinates come
// from selects, so the quad runs one instruction stream.  Every coordinate is the value
// make_supports passes (negations are exact), so the supports are the same bits.  Returns the
// exchange and sign bits of the thread's buffer; the quad ORs them into d.exch.
template <int CH>
__device__ __forceinline__ int make_part(const FlowArgs &a, const float *pos, const Transfer &f, float wp, int q,
                                         NodeDesc &d, LocDesc &loc) {
    AB4 ab;
    const int nl = a.nl, n = a.n;
    const MeshIndex m{pos, a.n, a.mesh_lo, a.mesh_base, a.mesh_shift};
    const bool lo2 = q < 2, odd = q & 1;
    if (CH == kS) {
        // buffers (t, u): 0 (-A, -B), 1 (P, -Q), 2 (B, A), 3 (-Q, P); (y1, y2) = (A, B) or (P, Q)
        const float y1 = odd ? f.w1p + wp : f.w1 + wp, y2 = odd ? f.w2p + wp : f.w2 + wp;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        const float t = lo2 ? (odd ? y1 : -y1) : (odd ? -y2 : y2);
        const float u = lo2 ? -y2 : y1;
        access4i<kS>(n, nl, f.s, t, u, lo2 ? i1 : i2, lo2 ? i2 : i1, f.si, ab);
        return put_ab(d, q, ab) | (int(ab.exch) << q);
    } else if (CH == kU) {
        // buffers (s, t): 0 (A, -D), 1 (P, E), 2 (D, -A), 3 (E, P); (y1, y2) = (A, D) or (P, E)
        const float y1 = odd ? f.w1p + wp : f.w1 + wp, y2 = odd ? f.w2 - wp : f.w2p - wp;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        const float sv = lo2 ? y1 : y2;
        const float t = lo2 ? (odd ? y2 : -y2) : (odd ? y1 : -y1);
        access4i<kU>(n, nl, sv, t, f.u, lo2 ? i1 : i2, lo2 ? i2 : i1, f.ui, ab);
        return put_ab(d, q, ab) | (int(ab.exch) << q);
    } else {
        // main buffers (s, u): 0 (C, P), 2 (P, C), 1 (D, -B), 3 (B, -D); local buffers (s, t, u):
        // 1 (C, -P, -t), 3 (P, -C, -t), 0 (D, -B, t), 2 (B, -D, t); (y1, y2) = (C, P), (P, C),
        // (D, B), (B, D) for q = 0..3
        const float C = f.w1 - wp, P = f.w1p + wp, D = f.w2p - wp, B = f.w2 + wp;
        const float x1 = lo2 ? C : D, x2 = lo2 ? P : B;
        const float y1 = odd ? x2 : x1, y2 = odd ? x1 : x2;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        const int bi = (int(odd) << 1) | (q >> 1), li = (int(odd) << 1) | (1 - (q >> 1));
        access4i<kT>(n, nl, y1, f.t, lo2 ? y2 : -y2, i1, i2, f.ti, ab);
        const int bits = put_ab(d, bi, ab) | (int(ab.exch) << bi);
        access4i<kU>(n, nl, y1, -y2, lo2 ? -f.t : f.t, i1, i2, f.ti, ab);
        loc.off[li] = make_int4(ab.off[0], ab.off[1], ab.off[2], ab.off[3]);
        loc.w[li] = make_float4(ab.w[0], ab.w[1], ab.w[2], ab.w[3]);
        loc.sw[li] = make_float4(ab.sw[0], ab.sw[1], ab.sw[2], ab.sw[3]);
        return bits;
    }
}

// make_desc split over the two threads of a lane pair (h = 0, 1), for a CTA that builds 128
// nodes with 256 threads.  Thread h builds the two main buffers that share its pair of
// interpolated magnitudes, buffers h and h + 2 (and in the t channel the two local buffers of
// the same magnitudes, whose values go to lv); the coordinates come from selects, so the pair
// runs one instruction stream.  Every coordinate is the value make_desc passes (negations are
// exact), so the descriptor is the same bits.  Returns the exchange and sign bits of the
// thread's buffers; the pair ORs them into d.exch.
template <int CH>
__device__ __forceinline__ int make_pair(const FlowArgs &a, const float *pos, const Transfer &f, float wp, int h,
                                         NodeDesc &d) {
    AB4 ab;
    const int nl = a.nl, n = a.n;
    const MeshIndex m{pos, a.n, a.mesh_lo, a.mesh_base, a.mesh_shift};
    const bool odd = h & 1;
    int bits = 0;
    if (CH == kS) {
        // buffers (t, u): 0 (-A, -B), 2 (B, A) from (A, B); 1 (P, -Q), 3 (-Q, P) from (P, Q)
        const float y1 = odd ? f.w1p + wp : f.w1 + wp, y2 = odd ? f.w2p + wp : f.w2 + wp;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        access4i<kS>(n, nl, f.s, odd ? y1 : -y1, -y2, i1, i2, f.si, ab);
        bits |= put_ab(d, h, ab) | (int(ab.exch) << h);
        access4i<kS>(n, nl, f.s, odd ? -y2 : y2, y1, i2, i1, f.si, ab);
        bits |= put_ab(d, h + 2, ab) | (int(ab.exch) << (h + 2));
    } else if (CH == kU) {
        // buffers (s, t): 0 (A, -D), 2 (D, -A) from (A, D); 1 (P, E), 3 (E, P) from (P, E)
        const float y1 = odd ? f.w1p + wp : f.w1 + wp, y2 = odd ? f.w2 - wp : f.w2p - wp;
        const Interp<float> i1 = interp_abs(m, y1), i2 = interp_abs(m, y2);
        access4i<kU>(n, nl, y1, odd ? y2 : -y2, f.u, i1, i2, f.ui, ab);
        bits |= put_ab(d, h, ab) | (int(ab.exch) << h);
        access4i<kU>(n, nl, y2, odd ? y1 : -y1, f.u, i2, i1, f.ui, ab);
        bits |= put_ab(d, h + 2, ab) | (int(ab.exch) << (h + 2));
    } else {
        // main buffers (s, u): 0 (C, P), 2 (P, C) from (C, P); 1 (D, -B), 3 (B, -D) from (D, B);
        // local buffers (s, t, u) to lv: 1 (C, -P, -t), 3 (P, -C, -t); 0 (D, -B, t), 2 (B, -D, t)
        const float x1 = odd ? f.w2p - wp : f.w1 - wp, x2 = odd ? f.w2 + wp : f.w1p + wp;
        const Interp<float> i1 = interp_abs(m, x1), i2 = interp_abs(m, x2);
        access4i<kT>(n, nl, x1, f.t, odd ? -x2 : x2, i1, i2, f.ti, ab);
        bits |= put_ab(d, h, ab) | (int(ab.exch) << h);
        access4i<kT>(n, nl, x2, f.t, odd ? -x1 : x1, i2, i1, f.ti, ab);
        bits |= put_ab(d, h + 2, ab) | (int(ab.exch) << (h + 2));
        const float tl = odd ? f.t : -f.t;
        float v0, v1;
        access4i<kU>(n, nl, x1, -x2, tl, i1, i2, f.ti, ab);
        local_pair(a, ab, v0, v1);
        d.lv[odd ? 0 : 2] = v0;
        d.lv[odd ? 1 : 3] = v1;
        access4i<kU>(n, nl, x2, -x1, tl, i2, i1, f.ti, ab);
        local_pair(a, ab, v0, v1);
        d.lv[odd ? 4 : 6] = v0;
        d.lv[odd ? 5 : 7] = v1;
    }
    return bits;
}

// The t channel's eight site-local values of one node for one flow's state (make_desc's
// local_pair of each local buffer, in the same order).
__device__ __forceinline__ void group_local_values(const float2 *sd, const LocDesc &loc, float *lv) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int4 o = loc.off[i];
        const float4 w = loc.w[i], sw = loc.sw[i];
        float2 g = make_float2(0.0f, 0.0f);
        g = fma2(make_float2(w.x, sw.x), __ldg(sd + o.x), g);
        g = fma2(make_float2(w.y, sw.y), __ldg(sd + o.y), g);
        g = fma2(make_float2(w.z, sw.z), __ldg(sd + o.z), g);
        g = fma2(make_float2(w.w, sw.w), __ldg(sd + o.w), g);
        lv[2 * i] = g.x;
        lv[2 * i + 1] = g.y;
    }
}

// Phase B: interpolated slab of buffer i for this lane's sites (getValueSuperbundle): per
// support one 64-bit load of the (spin, density) element and one packed FMA.
template <int SPT, class A>
__device__ __forceinline__ void gather(const A &a, const NodeDesc &d, int i, const Lane<SPT> &ln, float *vs,
                                       float *vd) {
    const int4 o = d.off[i];
    const float4 w = d.w[i];
    const int ex = d.exch;
    const float2 p0 = wpair(w.x, ex, 4 + 4 * i), p1 = wpair(w.y, ex, 5 + 4 * i);
    const float2 p2 = wpair(w.z, ex, 6 + 4 * i), p3 = wpair(w.w, ex, 7 + 4 * i);
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        const float2 *v = a.sd + (((ex >> i) & 1) ? ln.isite[k] : ln.site[k]);
        float2 g = make_float2(0.0f, 0.0f);
        g = fma2(p0, __ldg(v + o.x), g);
        g = fma2(p1, __ldg(v + o.y), g);
        g = fma2(p2, __ldg(v + o.z), g);
        g = fma2(p3, __ldg(v + o.w), g);
        vs[k] = g.x;
        vd[k] = g.y;
    }
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float v) {
    const float y = v - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// Shared-memory exchange area of a node's t channel: its panel, A2[w] = c * (spin, density) of
// the third slab and B2[w] = (spin, density) of the fourth slab per site (w >= Nl); the owner
// adds the panels' outer products to its M accumulators and walks the RPA schedule once per
// triple.
struct TExchange {
    float2 *A2, *B2;
    const int *sched, *count, *slot_base, *seg_ptr;  // RPA schedule (shared or global memory)
};

// Outer-product RPA accumulators of one lane (Nl <= 32): an MB x 2MB block of the
// (8 MB) x (8 MB) matrix M, (spin, density) per element.  Lane l owns rows (l >> 2) * MB ...
// and columns (l & 3) * 2MB ...
template <int MB>
struct OuterAcc {
    float2 m[MB > 0 ? MB : 1][MB > 0 ? 2 * MB : 1];
};

// A node as one lane group sees it: the supports (descriptor) and the flow's own coefficient
// and t-channel site-local values.  In a single flow both come from the descriptor; flows that
// share a descriptor (grouped batches) each bring their own.
struct NodeView {
    const NodeDesc *d;
    float c;
    const float *lv;
};

// K_X at NPI nodes for this lane's sites (one group evaluates NPI nodes per iteration so that
// the t channel decodes each RPA schedule entry once for all of them).  `a` provides the
// state (a.sd), the spin length and, for SPT > 1, the RPA schedule.
// The t channel writes the node's panel (c * third slab, fourth slab) for every site of the
// lane; the caller adds its outer product to M and walks the RPA pair list once per triple.
template <int CH, int SPT, int NPI, class A>
__device__ __forceinline__ void node_term(const A &a, const NodeView *v, const Lane<SPT> &ln, int jl,
                                          const TExchange *tx, float (*rs)[SPT], float (*rd)[SPT]) {
    float S0[NPI][SPT], S1[NPI][SPT], S2[NPI][SPT], S3[NPI][SPT], D0[NPI][SPT], D1[NPI][SPT], D2[NPI][SPT],
        D3[NPI][SPT];
#pragma unroll
    for (int n = 0; n < NPI; ++n) {
        gather<SPT>(a, *v[n].d, 0, ln, S0[n], D0[n]);
        gather<SPT>(a, *v[n].d, 1, ln, S1[n], D1[n]);
        gather<SPT>(a, *v[n].d, 2, ln, S2[n], D2[n]);
        gather<SPT>(a, *v[n].d, 3, ln, S3[n], D3[n]);
    }
    if (CH == kS || CH == kU) {
#pragma unroll
        for (int n = 0; n < NPI; ++n)
#pragma unroll
            for (int k = 0; k < SPT; ++k) {
                float x = 0.0f, y = 0.0f;
                if (CH == kS) {  // SU2FrgCore.cpp:216-226
                    x -= 0.5f * S0[n][k] * S1[n][k];
                    x -= 0.5f * S2[n][k] * S3[n][k];
                    x += D0[n][k] * S1[n][k];
                    x += D2[n][k] * S3[n][k];
                    x += S0[n][k] * D1[n][k];
                    x += S2[n][k] * D3[n][k];
                } else {  // SU2FrgCore.cpp:323-328
                    x += 0.5f * S0[n][k] * S1[n][k];
                    x += 0.5f * S2[n][k] * S3[n][k];
                    x += S0[n][k] * D1[n][k];
                    x += S2[n][k] * D3[n][k];
                    x += D0[n][k] * S1[n][k];
                    x += D2[n][k] * S3[n][k];
                }
                y += (3.0f / 16.0f) * S0[n][k] * S1[n][k];
                y += (3.0f / 16.0f) * S2[n][k] * S3[n][k];
                y += D0[n][k] * D1[n][k];
                y += D2[n][k] * D3[n][k];
                rs[n][k] = x;
                rd[n][k] = y;
            }
        return;
    }
    // t channel: RPA lattice sum (SU2FrgCore.cpp:249-266)
    {
        // outer-product form: the node's panel (c * third slab, fourth slab); the caller adds
        // the panels' outer products to its M accumulators
#pragma unroll
        for (int k = 0; k < SPT; ++k)
            if (ln.valid[k]) {
                const int j = ln.j[k];
#pragma unroll
                for (int n = 0; n < NPI; ++n) {
                    const float c = v[n].c;
                    tx[n].A2[j] = make_float2(c * S2[n][k], c * D2[n][k]);
                    tx[n].B2[j] = make_float2(S3[n][k], D3[n][k]);
                }
            }
    }
    const float s2 = 2.0f * a.spin, s8 = 8.0f * a.spin;
#pragma unroll
    for (int n = 0; n < NPI; ++n) {
        const float cbs = v[n].lv[0], cbd = v[n].lv[1], icas = v[n].lv[2], icad = v[n].lv[3];
        const float cbs2 = v[n].lv[4], cbd2 = v[n].lv[5], icas2 = v[n].lv[6], icad2 = v[n].lv[7];
#pragma unroll
        for (int k = 0; k < SPT; ++k) {
            const float rpa_s = 0.0f, rpa_d = 0.0f;  // the RPA term enters once per triple
            float x = 0.0f + s2 * rpa_s;  // SU2FrgCore.cpp:265, 286-293
            x -= cbd * S0[n][k];
            x += (0.25f * cbs) * S0[n][k];
            x -= icad * S1[n][k];
            x += (0.25f * icas) * S1[n][k];
            x -= cbd2 * S2[n][k];
            x += (0.25f * cbs2) * S2[n][k];
            x -= icad2 * S3[n][k];
            x += (0.25f * icas2) * S3[n][k];
            float y = 0.0f + s8 * rpa_d;  // SU2FrgCore.cpp:266, 295-302
            y -= cbd * D0[n][k];
            y -= (0.75f * cbs) * D0[n][k];
            y -= icad * D1[n][k];
            y -= (0.75f * icas) * D1[n][k];
            y -= cbd2 * D2[n][k];
            y -= (0.75f * cbs2) * D2[n][k];
            y -= icad2 * D3[n][k];
            y -= (0.75f * icas2) * D3[n][k];
            rs[n][k] = x;
            rd[n][k] = y;
        }
    }
}

// Adds the outer products of the panels of nodes k = (r*NPI+n)*G+gg < nb (ascending k) to the
// lane's block of M.  `pan`: the warp's first panel; panel (gg, n) starts pstride float2 later
// per step of gg * NPI + n.
template <int NPI, int MB>
__device__ __forceinline__ void outer_update(const float2 *pan, int pstride, int lane, int r, int G, int nb,
                                             OuterAcc<MB> &M) {
    constexpr int W = 8 * MB;
    const int rb = lane >> 2, cb = lane & 3;
#pragma unroll
    for (int n = 0; n < NPI; ++n)
        for (int gg = 0; gg < G; ++gg) {
            const int k = (r * NPI + n) * G + gg;
            if (k >= nb) break;
            const float2 *A = pan + (gg * NPI + n) * pstride + rb * MB;
            const float2 *B = pan + (gg * NPI + n) * pstride + W + cb * 2 * MB;
            float2 av[MB], bv[2 * MB];
#pragma unroll
            for (int i = 0; i < MB; ++i) av[i] = A[i];
#pragma unroll
            for (int j = 0; j < 2 * MB; ++j) bv[j] = B[j];
#pragma unroll
            for (int i = 0; i < MB; ++i)
#pragma unroll
                for (int j = 0; j < 2 * MB; ++j) M.m[i][j] = fma2(av[i], bv[j], M.m[i][j]);
        }
}

template <int CH, int SPT, int NPI, int MB>
__device__ __forceinline__ void channel_sum(const FlowArgs &a, const float *pos, const Transfer &f, int xi, int lane, int g,
                                            int G, int jl, const Lane<SPT> &ln, NodeDesc *desc, const TExchange *tx,
                                            const float2 *pan, int pstride, OuterAcc<MB> &M,
                                            float *acc_s, float *cmp_s, float *acc_d, float *cmp_d) {
    const int cnt = __ldg(a.node_cnt + xi);
    const float *nwp = a.node_wp + size_t(xi) * a.max_nodes;
    const float *nc = a.node_c + size_t(xi) * a.max_nodes;
    for (int b0 = 0; b0 < cnt; b0 += kBatch) {
        const int nb = min(kBatch, cnt - b0);
        if (lane < nb) {
            const float wp = __ldg(nwp + b0 + lane);
            float c = __ldg(nc + b0 + lane);
            if (CH == kU) c = -c;
            make_desc<CH>(a, pos, f, wp, c, desc[lane]);
        }
        __syncwarp();
        const int trips = (nb + G * NPI - 1) / (G * NPI);
        for (int r = 0; r < trips; ++r) {
            const NodeDesc *d[NPI];
            bool active[NPI];
#pragma unroll
            for (int n = 0; n < NPI; ++n) {
                const int k = (r * NPI + n) * G + g;  // group g: nodes g, g+G, g+2G, ... for every NPI
                active[n] = k < nb;
                d[n] = &desc[active[n] ? k : 0];
            }
            NodeView v[NPI];
#pragma unroll
            for (int n = 0; n < NPI; ++n) v[n] = NodeView{d[n], d[n]->c, d[n]->lv};
            float rs[NPI][SPT], rd[NPI][SPT];
            node_term<CH, SPT, NPI>(a, v, ln, jl, tx, rs, rd);
#pragma unroll
            for (int n = 0; n < NPI; ++n)
                if (active[n]) {
                    const float c = v[n].c;
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        kahan_add(acc_s[q], cmp_s[q], c * rs[n][q]);
                        kahan_add(acc_d[q], cmp_d[q], c * rd[n][q]);
                    }
                }
            if constexpr (CH == kT && SPT == 1) {
                __syncwarp();  // panels written
                outer_update<NPI, MB>(pan, pstride, lane, r, G, nb, M);
                __syncwarp();  // panels read
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------------------
// Bulk copies global -> shared through the copy engine (cp.async.bulk) completing on an
// mbarrier.  Addresses and sizes are multiples of 16 bytes.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) { return unsigned(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Waits for phase `parity` of the barrier to complete, at most kStageSpin polls; false on timeout.
constexpr int kStageSpin = 1 << 20;
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
    for (int i = 0; i < kStageSpin; ++i) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.b32 %0, 1, 0, p;\n}"
                     : "=r"(done)
                     : "r"(smem_u32(bar)), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

// Shared memory of the single-flow kernel: frequency mesh; the RPA schedule when it is staged;
// then per warp: 32 node descriptors and, per node group, NPI t-channel exchange areas (Nl <=
// 32: a panel of 2 w float2; otherwise four arrays of W*SPT sites and n_seg slots).  For Nl <=
// 32 the same warp area holds, between the t and the u channel, the matrix M (w x w float2)
// and the n_seg segment partials of the pair walk.
__host__ __device__ inline size_t node_area_bytes(int wsite, int spt, int n_seg, int w) {
    if (spt == 1) return sizeof(float2) * 2 * size_t(w);  // w is a multiple of 8: 16-byte aligned
    return (sizeof(float) * 4 * size_t(wsite) * spt + sizeof(float2) * n_seg + 15) / 16 * 16;
}
__host__ __device__ inline size_t group_area_bytes(int wsite, int spt, int npi, int n_seg, int w) {
    return (32 / wsite) * npi * node_area_bytes(wsite, spt, n_seg, w);
}
__host__ __device__ inline size_t outer_stage_bytes(int w, int n_seg) {
    return (sizeof(float2) * (size_t(w) * w + n_seg) + 15) / 16 * 16;
}
__host__ __device__ inline size_t warp_bytes(int wsite, int spt, int npi, int n_seg, int w) {
    const size_t main = kBatch * sizeof(NodeDesc) + group_area_bytes(wsite, spt, npi, n_seg, w);
    if (spt != 1) return main;
    const size_t st = outer_stage_bytes(w, n_seg);
    return main > st ? main : st;
}
__host__ __device__ inline size_t sched_bytes(const RpaSchedule &r, int nl) {
    return r.in_smem ? (sizeof(int) * size_t(rpa_smem_ints(r, nl)) + 15) / 16 * 16 : 0;
}
__host__ __device__ inline size_t align16(size_t x) { return (x + 15) / 16 * 16; }

// What one warp needs to evaluate triples of one flow: lane roles, site indices and the
// shared-memory areas.
template <int SPT, int NPI>
struct WarpCtx {
    NodeDesc *desc;
    TExchange tx[NPI];
    Lane<SPT> ln;
    int W, G, g, jl;
    float2 *panel;  // Nl <= 32: first t-channel panel of the warp
    int pstride;    // float2 from one panel to the next
};

// `groups`: the warp's node-group areas; sched..seg_ptr: the RPA schedule (shared or global).
template <int SPT, int NPI, int MB>
__device__ __forceinline__ void setup_ctx(const FlowArgs &a, int lane, NodeDesc *desc, unsigned char *groups,
                                          const int *sched, const int *count, const int *slot_base, const int *seg_ptr,
                                          WarpCtx<SPT, NPI> &c) {
    c.desc = desc;
    c.W = (SPT == 1) ? a.wsite : 32;
    c.G = 32 / c.W;
    c.g = lane / c.W;
    c.jl = lane - c.g * c.W;
    const size_t nab = node_area_bytes(c.W, SPT, a.rpa.n_seg, 8 * MB);
    c.panel = reinterpret_cast<float2 *>(groups);
    c.pstride = int(nab / sizeof(float2));
    if (SPT == 1) {  // panel entries of sites >= Nl stay zero
        float4 *z = reinterpret_cast<float4 *>(groups);
        const int n16 = int(c.G * NPI * nab / 16);
        for (int i = lane; i < n16; i += 32) z[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        __syncwarp();
    }
    unsigned char *gbase = groups + size_t(c.g) * NPI * nab;
#pragma unroll
    for (int n = 0; n < NPI; ++n) {
        float *gx = reinterpret_cast<float *>(gbase + n * nab);
        c.tx[n].A2 = reinterpret_cast<float2 *>(gx);
        c.tx[n].B2 = reinterpret_cast<float2 *>(gx) + 8 * MB;
        c.tx[n].sched = sched;
        c.tx[n].count = count;
        c.tx[n].slot_base = slot_base;
        c.tx[n].seg_ptr = seg_ptr;
    }
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        const int j = c.jl + k * c.W;
        c.ln.j[k] = j;
        c.ln.valid[k] = j < a.nl;
        c.ln.site[k] = c.ln.valid[k] ? a.sites[j] : 0;
        c.ln.isite[k] = c.ln.valid[k] ? a.inv_sites[j] : 0;
    }
}

// The flow of triple `it` of flow `a` (all lanes of the warp take part).  The single-flow and
// the batched kernel both evaluate triples with this function, so a flow's result does not
// depend on the kernel, the launch or the other flows of a batch.
// Nl <= 32, after the t channel: the lane's block of M goes to the warp area, the warp walks
// the merged pair list once (segment partials after M), and group 0 adds its rid's sum
// s2 * sum m M[rid1][rid2] (spin) and s8 * ... (density) to its accumulators.
template <int SPT, int NPI, int MB>
__device__ __forceinline__ void outer_gather(const FlowArgs &a, const WarpCtx<SPT, NPI> &c, int lane,
                                             const OuterAcc<MB> &M, float *acc_s, float *cmp_s, float *acc_d,
                                             float *cmp_d) {
    constexpr int W = 8 * MB;
    float2 *Ms = reinterpret_cast<float2 *>(c.desc);  // descriptors and panels are free here
    float2 *slots = Ms + W * W;
    const int rb = lane >> 2, cb = lane & 3;
#pragma unroll
    for (int i = 0; i < MB; ++i)
#pragma unroll
        for (int j = 0; j < 2 * MB; ++j) Ms[(rb * MB + i) * W + cb * 2 * MB + j] = M.m[i][j];
    __syncwarp();
    const int lanes = a.rpa.lanes;
    const int cnt = c.tx[0].count[lane];
    int slot = c.tx[0].slot_base[lane];
    const int *sched = c.tx[0].sched + lane;
    const char *mb = reinterpret_cast<const char *>(Ms);
    float2 acc = make_float2(0.0f, 0.0f);
    auto step = [&](int e, float2 v) {
        const float m = float((e >> 16) & 0xff);
        acc = fma2(make_float2(m, m), v, acc);
        if (e < 0) {  // last pair of a segment
            slots[slot++] = acc;
            acc = make_float2(0.0f, 0.0f);
        }
    };
    constexpr int kU = 4;
    int i = 0;
    for (; i + kU <= cnt; i += kU) {
        int e[kU];
        float2 v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) e[u] = sched[(i + u) * lanes];
#pragma unroll
        for (int u = 0; u < kU; ++u) v[u] = *reinterpret_cast<const float2 *>(mb + (e[u] & 0xffff));
#pragma unroll
        for (int u = 0; u < kU; ++u) step(e[u], v[u]);
    }
    for (; i < cnt; ++i) {
        const int e = sched[i * lanes];
        step(e, *reinterpret_cast<const float2 *>(mb + (e & 0xffff)));
    }
    __syncwarp();
    if (c.g == 0 && c.ln.valid[0]) {
        const int r = c.ln.j[0];
        float os = 0.0f, od = 0.0f;
        for (int q = c.tx[0].seg_ptr[r]; q < c.tx[0].seg_ptr[r + 1]; ++q) {
            const float2 p = slots[q];
            os += p.x;
            od += p.y;
        }
        kahan_add(acc_s[0], cmp_s[0], (2.0f * a.spin) * os);  // SU2FrgCore.cpp:265-266
        kahan_add(acc_d[0], cmp_d[0], (8.0f * a.spin) * od);
    }
    __syncwarp();
}

template <int SPT, int NPI, int MB>
__device__ __forceinline__ void vertex_triple(const FlowArgs &a, const float *pos, int it, const WarpCtx<SPT, NPI> &c,
                                              int lane) {
    const float two_pi = 2.0f * float(kPi);
    const int su = it / a.n, ti = it - su * a.n;
    int si = int((sqrtf(8.0f * float(su) + 1.0f) - 1.0f) * 0.5f);
    while (si * (si + 1) / 2 > su) --si;
    while ((si + 1) * (si + 2) / 2 <= su) ++si;
    const int ui = su - si * (si + 1) / 2;

    Transfer f;
    f.s = pos[si];
    f.t = pos[ti];
    f.u = pos[ui];
    f.w1p = 0.5f * (f.s + f.t + f.u);
    f.w1 = 0.5f * (f.s - f.t + f.u);
    f.w2p = 0.5f * (f.s - f.t - f.u);
    f.w2 = 0.5f * (f.s + f.t - f.u);
    f.si = si;
    f.ti = ti;
    f.ui = ui;

    float acc_s[SPT], cmp_s[SPT], acc_d[SPT], cmp_d[SPT];
#pragma unroll
    for (int k = 0; k < SPT; ++k) acc_s[k] = cmp_s[k] = acc_d[k] = cmp_d[k] = 0.0f;
    OuterAcc<MB> M;
#pragma unroll
    for (int i = 0; i < (MB > 0 ? MB : 1); ++i)
#pragma unroll
        for (int j = 0; j < (MB > 0 ? 2 * MB : 1); ++j) M.m[i][j] = make_float2(0.0f, 0.0f);
    channel_sum<kS, SPT, NPI, MB>(a, pos, f, si, lane, c.g, c.G, c.jl, c.ln, c.desc, c.tx, c.panel, c.pstride, M, acc_s,
                                  cmp_s, acc_d, cmp_d);
    channel_sum<kT, SPT, NPI, MB>(a, pos, f, ti, lane, c.g, c.G, c.jl, c.ln, c.desc, c.tx, c.panel, c.pstride, M, acc_s,
                                  cmp_s, acc_d, cmp_d);
    if constexpr (SPT == 1) outer_gather<SPT, NPI, MB>(a, c, lane, M, acc_s, cmp_s, acc_d, cmp_d);
    channel_sum<kU, SPT, NPI, MB>(a, pos, f, ui, lane, c.g, c.G, c.jl, c.ln, c.desc, c.tx, c.panel, c.pstride, M, acc_s,
                                  cmp_s, acc_d, cmp_d);

#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        float vs = acc_s[k] - cmp_s[k], vd = acc_d[k] - cmp_d[k];
        for (int o = c.W; o < 32; o <<= 1) {
            vs += __shfl_xor_sync(0xffffffffu, vs, o);
            vd += __shfl_xor_sync(0xffffffffu, vd, o);
        }
        if (c.g == 0 && c.ln.valid[k]) {
            const float os = vs / two_pi, od = vd / two_pi;
            a.dsd[size_t(it) * a.nl + c.ln.j[k]] = make_float2(os, od);
            if (isnan(os) || isnan(od)) atomicOr(a.status, kStatusNaN);
        }
    }
}

template <int SPT, int NPI, int MB>
__global__ void __launch_bounds__(kThreads) su2_vertex_flow_kernel(FlowArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long stage_bar;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = (SPT == 1) ? a.wsite : 32;
    const int n_seg = a.rpa.n_seg;
    unsigned char *sbase = smem_raw + kMaxFreq * sizeof(float);

    // Stage the frequency mesh and (if selected) the RPA schedule image in shared memory with
    // the bulk-copy engine: one thread arms an mbarrier with the byte count and issues the
    // copies; every thread waits on the barrier (bounded; on timeout the kernel records
    // kStatusStageTimeout and reads the global copies instead).
    const unsigned pos_bytes = (unsigned(a.n) * sizeof(float) + 15u) & ~15u;
    const unsigned img_bytes = a.rpa.in_smem ? unsigned(a.rpa.image_bytes) : 0u;
    if (threadIdx.x == 0) {
        mbar_init(&stage_bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&stage_bar, pos_bytes + img_bytes);
        bulk_copy_g2s(smem_raw, a.freq, pos_bytes, &stage_bar);
        if (img_bytes) bulk_copy_g2s(sbase, a.rpa.image, img_bytes, &stage_bar);
    }
    const bool staged = mbar_wait(&stage_bar, 0);
    if (!staged) atomicOr(a.status, kStatusStageTimeout);

    const float *pos = staged ? reinterpret_cast<const float *>(smem_raw) : a.freq;
    const int *sched, *count, *slot_base, *seg_ptr;
    if (a.rpa.in_smem && staged) {
        const int *s = reinterpret_cast<const int *>(sbase);
        const int ns = a.rpa.len * a.rpa.lanes, nc = a.rpa.lanes;
        sched = s;
        count = s + ns;
        slot_base = s + ns + nc;
        seg_ptr = s + ns + 2 * nc;
    } else {
        sched = a.rpa.sched;
        count = a.rpa.count;
        slot_base = a.rpa.slot_base;
        seg_ptr = a.rpa.seg_ptr;
    }
    unsigned char *wbase = sbase + sched_bytes(a.rpa, a.nl) + warp * warp_bytes(W, SPT, NPI, n_seg, 8 * MB);
    WarpCtx<SPT, NPI> c;
    setup_ctx<SPT, NPI, MB>(a, lane, reinterpret_cast<NodeDesc *>(wbase), wbase + kBatch * sizeof(NodeDesc), sched, count,
                            slot_base, seg_ptr, c);
    __syncthreads();

    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.work_counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= a.fn) break;
        vertex_triple<SPT, NPI, MB>(a, pos, it, c, lane);
    }
    // a copy that timed out must still land before the block's shared memory is released
    if (!staged && threadIdx.x == 0) mbar_wait(&stage_bar, 0);
}

// Batched vertex flow: a persistent grid over the ragged list of (flow, triple) items of all
// flows of one site class.  A warp keeps the flow it works on (argument block, frequency
// mesh, lane roles) in its own shared-memory area and reloads it only when an item of another
// flow comes up; items are numbered flow by flow, so that happens rarely.  The RPA schedule
// is read from global memory (it differs between flows).
template <int SPT, int NPI, int MB>
__global__ void __launch_bounds__(kThreads) su2_vertex_batch_kernel(BatchVertexArgs b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t fa_bytes = align16(sizeof(FlowArgs)), pos_bytes = align16(sizeof(float) * b.n_max);
    const size_t sch_bytes = align16(sizeof(int) * size_t(b.sched_ints));
    unsigned char *wbase =
        smem_raw + size_t(warp) * (fa_bytes + pos_bytes + sch_bytes + kBatch * sizeof(NodeDesc) + b.warp_area);
    FlowArgs *fa = reinterpret_cast<FlowArgs *>(wbase);
    float *pos = reinterpret_cast<float *>(wbase + fa_bytes);
    int *sch = reinterpret_cast<int *>(wbase + fa_bytes + pos_bytes);
    NodeDesc *desc = reinterpret_cast<NodeDesc *>(wbase + fa_bytes + pos_bytes + sch_bytes);
    unsigned char *groups = wbase + fa_bytes + pos_bytes + sch_bytes + kBatch * sizeof(NodeDesc);

    WarpCtx<SPT, NPI> c;
    int cur = -1, base = 0;
    bool skip = false;
    for (;;) {
        int w = 0;
        if (lane == 0) w = atomicAdd(b.counter, 1);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= b.total) break;
        int lo = 0, hi = b.n_list - 1;  // last f with prefix[f] <= w
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(b.prefix + mid) <= w) lo = mid;
            else hi = mid - 1;
        }
        if (lo != cur) {
            cur = lo;
            base = __ldg(b.prefix + lo);
            const BatchFlow *bf = b.flows + __ldg(b.list + lo);
            __syncwarp();
            const int *src = reinterpret_cast<const int *>(&bf->a);
            int *dst = reinterpret_cast<int *>(fa);
            for (int i = lane; i < int(sizeof(FlowArgs) / sizeof(int)); i += 32) dst[i] = src[i];
            skip = bf->phase != kPhaseFlowing;
            __syncwarp();
            for (int i = lane; i < fa->n; i += 32) pos[i] = fa->freq[i];
            if (b.sched_ints > 0) {  // the host checked that every flow's schedule fits
                const RpaSchedule &r = fa->rpa;
                const int ns = r.len * r.lanes, nc = r.lanes;
                for (int i = lane; i < ns; i += 32) sch[i] = __ldg(r.sched + i);
                for (int i = lane; i < nc; i += 32) {
                    sch[ns + i] = __ldg(r.count + i);
                    sch[ns + nc + i] = __ldg(r.slot_base + i);
                }
                for (int i = lane; i <= fa->nl; i += 32) sch[ns + 2 * nc + i] = __ldg(r.seg_ptr + i);
                setup_ctx<SPT, NPI, MB>(*fa, lane, desc, groups, sch, sch + ns, sch + ns + nc, sch + ns + 2 * nc, c);
            } else {
                setup_ctx<SPT, NPI, MB>(*fa, lane, desc, groups, fa->rpa.sched, fa->rpa.count, fa->rpa.slot_base,
                                        fa->rpa.seg_ptr, c);
            }
            __syncwarp();
        }
        if (skip) continue;
        vertex_triple<SPT, NPI, MB>(*fa, pos, w - base, c, lane);
    }
}

// ------------------------------------------------------------------------------------
// Grouped batches: flows that share the frequency mesh, the lattice tables and the current
// cutoff (a parameter scan's members of one lattice, range and frequency count, started
// together) have the same loop-frequency node positions and the same interpolation supports
// for every (triple, node); only the state, the node coefficients (through the self-energy)
// and the t channel's site-local values differ.  A CTA takes one triple for a subgroup of up to
// kGroupWarps * 32 / W flows: its threads build each node's supports once, in chunks of 32
// nodes, and every warp evaluates them for 32 / W flows at once, lane = (flow, site).
//
// The result of every flow is the single-flow kernel's, bit for bit: a flow's W lanes keep the
// single-flow kernel's G = 32 / W Kahan accumulator pairs (node k of a channel adds into pair
// k mod G, the RPA term into pair 0 after the t channel) and combine them in its order, and
// the outer-product matrix M adds the nodes' panels in ascending order.  The pair walk follows
// the same 32-chunk schedule, each of the flow's W lanes walking chunks l, l + W, ...
// ------------------------------------------------------------------------------------
constexpr int kGroupWarps = 4;
constexpr int kGroupChunk = 32;  // nodes whose supports the CTA builds at once (four threads per node)
static_assert(kGroupWarps * 32 == 4 * kGroupChunk, "the grouped kernel builds a chunk with four threads per node");

// What a lane of a grouped warp needs of its flow (node_term reads a.sd and a.spin).
struct GroupLaneArgs {
    const float2 *sd;
    float spin;
};

__host__ __device__ constexpr int group_cb(int W) { return W == 8 ? 2 : 4; }

// Adds the outer product of the flow's panel (A2 = c * third slab, B2 = fourth slab; w entries
// each) to the lane's R x C block of M; the flow's W lanes form a (W / Cb) x Cb grid.
template <int W, int MB>
__device__ __forceinline__ void group_outer_update(const float2 *pan, int jl, float2 (*m)[8 * MB / group_cb(W)]) {
    constexpr int w = 8 * MB, Cb = group_cb(W), Rb = W / Cb, R = w / Rb, C = w / Cb;
    const int rb = jl / Cb, cb = jl % Cb;
    float2 av[R], bv[C];
#pragma unroll
    for (int i = 0; i < R; ++i) av[i] = pan[rb * R + i];
#pragma unroll
    for (int j = 0; j < C; ++j) bv[j] = pan[w + cb * C + j];
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < C; ++j) m[i][j] = fma2(av[i], bv[j], m[i][j]);
}

template <int W, int MB>
struct GroupShape {
    static constexpr int F = 32 / W;                 // flows per warp
    static constexpr int GMAX = kGroupWarps * F;     // flows per CTA
    static constexpr int G = 32 / W;                 // single-flow node groups (accumulator pairs)
    static constexpr int w = 8 * MB;                 // outer-product width
    static constexpr int Cb = group_cb(W), R = w / (W / Cb), C = w / Cb;
};

// Shared-memory layout of the grouped kernel (bytes from the dynamic base, all 16-aligned).
struct GroupSmem {
    size_t fa, ptrs, pos, build_desc, build_loc, build_c, build_lv, stage, panels, total;
};
__host__ __device__ inline GroupSmem group_smem_layout(int W, int MB, int n_seg_max) {
    const int F = 32 / W, GMAX = kGroupWarps * F, w = 8 * MB;
    GroupSmem L;
    size_t o = 0;
    L.fa = o; o += align16(sizeof(FlowArgs));
    L.ptrs = o; o += align16(size_t(GMAX) * (2 * sizeof(void *) + sizeof(void *) + sizeof(void *) + sizeof(int)));
    L.pos = o; o += align16(sizeof(float) * kMaxFreq);
    // union: the chunk build area, or (after the t channel) each flow's staged M and slots
    const size_t u0 = o;
    L.build_desc = o; o += kGroupChunk * sizeof(NodeDesc);
    L.build_loc = o; o += kGroupChunk * sizeof(LocDesc);
    L.build_c = o; o += align16(sizeof(float) * kGroupChunk * GMAX);
    L.build_lv = o; o += align16(sizeof(float) * 8 * kGroupChunk * GMAX);
    const size_t build_end = o;
    L.stage = u0;
    const size_t stage_end = u0 + align16(sizeof(float2) * size_t(GMAX) * (size_t(w) * w + n_seg_max));
    o = build_end > stage_end ? build_end : stage_end;
    L.panels = o; o += align16(sizeof(float2) * size_t(GMAX) * 2 * w);
    L.total = o;
    return L;
}

template <int W, int MB>
__global__ void __launch_bounds__(kGroupWarps * 32) su2_vertex_group_kernel(GroupVertexArgs g) {
    using S = GroupShape<W, MB>;
    constexpr int F = S::F, GMAX = S::GMAX, G = S::G, w = S::w, R = S::R, C = S::C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    const GroupSmem L = group_smem_layout(W, MB, g.n_seg_max);
    FlowArgs *fa = reinterpret_cast<FlowArgs *>(smem_raw + L.fa);
    unsigned char *pb = smem_raw + L.ptrs;
    const float2 **m_sd = reinterpret_cast<const float2 **>(pb);
    float2 **m_dsd = reinterpret_cast<float2 **>(pb + GMAX * sizeof(void *));
    const float **m_nc = reinterpret_cast<const float **>(pb + 2 * GMAX * sizeof(void *));
    unsigned **m_status = reinterpret_cast<unsigned **>(pb + 3 * GMAX * sizeof(void *));
    int *m_on = reinterpret_cast<int *>(pb + 4 * GMAX * sizeof(void *));  // member flowing this step
    float *pos = reinterpret_cast<float *>(smem_raw + L.pos);
    NodeDesc *desc = reinterpret_cast<NodeDesc *>(smem_raw + L.build_desc);
    LocDesc *loc = reinterpret_cast<LocDesc *>(smem_raw + L.build_loc);
    float *ctab = reinterpret_cast<float *>(smem_raw + L.build_c);   // [node][member]
    float *lvtab = reinterpret_cast<float *>(smem_raw + L.build_lv);  // [node][member][8]
    float2 *stage = reinterpret_cast<float2 *>(smem_raw + L.stage);
    float2 *panels = reinterpret_cast<float2 *>(smem_raw + L.panels);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gg = lane / W, jl = lane - gg * W;  // flow slot in the warp, site
    const int fs = warp * F + gg;                 // member index in the subgroup
    float2 *pan = panels + size_t(fs) * 2 * w;
    // panel entries of sites >= Nl are never written and stay zero
    for (int i = tid; i < GMAX * 2 * w; i += blockDim.x) panels[i] = make_float2(0.0f, 0.0f);

    int cur = -1, base = 0, nf = 0;
    bool live = false;
    for (;;) {
        __syncthreads();  // the previous item is finished with the shared areas
        if (tid == 0) s_item = atomicAdd(g.counter, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= g.total) break;
        int lo = 0, hi = g.n_sg - 1;  // last subgroup with prefix <= item
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(g.prefix + mid) <= item) lo = mid;
            else hi = mid - 1;
        }
        if (lo != cur) {
            cur = lo;
            base = __ldg(g.prefix + lo);
            // leader: the first member that is flowing this step (its node tables are current)
            int lead = -1, cnt = 0;
            for (int q = 0; q < GMAX; ++q) {
                const int fi = __ldg(g.members + size_t(lo) * GMAX + q);
                if (fi < 0) break;
                ++cnt;
                if (lead < 0 && g.flows[fi].phase == kPhaseFlowing) lead = fi;
            }
            nf = cnt;
            live = lead >= 0;
            if (live) {
                const BatchFlow *lf = g.flows + lead;
                const int *src = reinterpret_cast<const int *>(&lf->a);
                int *dst = reinterpret_cast<int *>(fa);
                for (int i = tid; i < int(sizeof(FlowArgs) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
                if (tid < GMAX) {
                    const int fi = tid < cnt ? __ldg(g.members + size_t(lo) * GMAX + tid) : -1;
                    const bool on = fi >= 0 && g.flows[fi].phase == kPhaseFlowing;
                    const BatchFlow *bf = g.flows + (on ? fi : lead);  // idle slots read the leader's data
                    m_sd[tid] = bf->a.sd;
                    m_dsd[tid] = bf->a.dsd;
                    m_nc[tid] = bf->a.node_c;
                    m_status[tid] = bf->a.status;
                    m_on[tid] = on ? 1 : 0;
                }
            }
            __syncthreads();
            if (live)
                for (int i = tid; i < fa->n; i += blockDim.x) pos[i] = fa->freq[i];
            __syncthreads();
        }
        if (!live) continue;
        const int it = item - base;
        const FlowArgs &a = *fa;

        // the triple (as vertex_triple decodes it)
        const int su = it / a.n, ti = it - su * a.n;
        int si = int((sqrtf(8.0f * float(su) + 1.0f) - 1.0f) * 0.5f);
        while (si * (si + 1) / 2 > su) --si;
        while ((si + 1) * (si + 2) / 2 <= su) ++si;
        const int ui = su - si * (si + 1) / 2;
        Transfer f;
        f.s = pos[si];
        f.t = pos[ti];
        f.u = pos[ui];
        f.w1p = 0.5f * (f.s + f.t + f.u);
        f.w1 = 0.5f * (f.s - f.t + f.u);
        f.w2p = 0.5f * (f.s - f.t - f.u);
        f.w2 = 0.5f * (f.s + f.t - f.u);
        f.si = si;
        f.ti = ti;
        f.ui = ui;

        const bool mine = fs < nf && m_on[fs];
        const GroupLaneArgs la{m_sd[fs < nf ? fs : 0], a.spin};
        Lane<1> ln;
        ln.j[0] = jl;
        ln.valid[0] = jl < a.nl;
        ln.site[0] = ln.valid[0] ? a.sites[jl] : 0;
        ln.isite[0] = ln.valid[0] ? a.inv_sites[jl] : 0;
        TExchange tx;
        tx.A2 = pan;
        tx.B2 = pan + w;

        float acc_s[G], cmp_s[G], acc_d[G], cmp_d[G];
#pragma unroll
        for (int q = 0; q < G; ++q) acc_s[q] = cmp_s[q] = acc_d[q] = cmp_d[q] = 0.0f;
        float2 M[R][C];
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < C; ++j) M[i][j] = make_float2(0.0f, 0.0f);

        // node k of a channel adds into pair k mod G: the pairs rotate after every node, and
        // pair 0 is realigned at the end of each channel
        auto rotate = [&]() {
#pragma unroll
            for (int q = 0; q + 1 < G; ++q) {
                float t;
                t = acc_s[q]; acc_s[q] = acc_s[q + 1]; acc_s[q + 1] = t;
                t = cmp_s[q]; cmp_s[q] = cmp_s[q + 1]; cmp_s[q + 1] = t;
                t = acc_d[q]; acc_d[q] = acc_d[q + 1]; acc_d[q + 1] = t;
                t = cmp_d[q]; cmp_d[q] = cmp_d[q + 1]; cmp_d[q + 1] = t;
            }
        };

        auto channel = [&](auto chc, int xi) {
            constexpr int CH = decltype(chc)::value;
            const int cnt = __ldg(a.node_cnt + xi);
            const float *nwp = a.node_wp + size_t(xi) * a.max_nodes;
            for (int b0 = 0; b0 < cnt; b0 += kGroupChunk) {
                const int nb = min(kGroupChunk, cnt - b0);
                __syncthreads();  // the previous chunk is consumed
                {  // four threads per node build its supports (the CTA's 128 threads: 32 nodes)
                    const int k = tid >> 2, q = tid & 3;
                    int bits = 0;
                    if (k < nb) bits = make_part<CH>(a, pos, f, __ldg(nwp + b0 + k), q, desc[k], loc[k]);
                    bits |= __shfl_xor_sync(0xffffffffu, bits, 1);
                    bits |= __shfl_xor_sync(0xffffffffu, bits, 2);
                    if (k < nb && q == 0) {
                        desc[k].exch = bits;
                        desc[k].c = 0.0f;
                    }
                    for (int p = tid; p < nb * GMAX; p += blockDim.x) {
                        const int kk = p / GMAX, qq = p - kk * GMAX;
                        float c = __ldg(m_nc[qq] + size_t(xi) * a.max_nodes + b0 + kk);
                        if (CH == kU) c = -c;
                        ctab[p] = c;
                    }
                }
                __syncthreads();
                if constexpr (CH == kT) {
                    for (int p = tid; p < nb * GMAX; p += blockDim.x) {
                        const int k = p / GMAX, q = p - k * GMAX;
                        group_local_values(m_sd[q], loc[k], lvtab + size_t(p) * 8);
                    }
                    __syncthreads();
                }
                for (int k = 0; k < nb; ++k) {
                    const int p = k * GMAX + fs;
                    NodeView v{&desc[k], ctab[p], lvtab + size_t(p) * 8};
                    float rs[1][1], rd[1][1];
                    node_term<CH, 1, 1>(la, &v, ln, jl, &tx, rs, rd);
                    kahan_add(acc_s[0], cmp_s[0], v.c * rs[0][0]);
                    kahan_add(acc_d[0], cmp_d[0], v.c * rd[0][0]);
                    rotate();
                    if constexpr (CH == kT) {
                        __syncwarp();  // panel written
                        group_outer_update<W, MB>(pan, jl, M);
                        __syncwarp();  // panel read
                    }
                }
            }
            // realign: pair 0 holds residue 0 again
            const int extra = (G - cnt % G) % G;
            for (int r = 0; r < extra; ++r) rotate();
        };

        channel(std::integral_constant<int, kS>{}, si);
        channel(std::integral_constant<int, kT>{}, ti);

        // RPA term: stage each flow's M, walk the 32-chunk schedule (chunks jl, jl + W, ...)
        __syncthreads();  // the build area is free
        {
            float2 *Ms = stage + size_t(fs) * (size_t(w) * w + g.n_seg_max);
            float2 *slots = Ms + w * w;
            const int rb = jl / S::Cb, cb = jl % S::Cb;
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int j = 0; j < C; ++j) Ms[(rb * R + i) * w + cb * C + j] = M[i][j];
            __syncwarp();
            const int lanes = a.rpa.lanes;
            const char *mb = reinterpret_cast<const char *>(Ms);
            for (int ch = jl; ch < lanes; ch += W) {
                const int cntq = __ldg(a.rpa.count + ch);
                int slot = __ldg(a.rpa.slot_base + ch);
                const int *sched = a.rpa.sched + ch;
                float2 acc = make_float2(0.0f, 0.0f);
                for (int i = 0; i < cntq; ++i) {
                    const int e = __ldg(sched + size_t(i) * lanes);
                    const float2 v = *reinterpret_cast<const float2 *>(mb + (e & 0xffff));
                    const float m = float((e >> 16) & 0xff);
                    acc = fma2(make_float2(m, m), v, acc);
                    if (e < 0) {
                        slots[slot++] = acc;
                        acc = make_float2(0.0f, 0.0f);
                    }
                }
            }
            __syncwarp();
            if (ln.valid[0]) {
                float os = 0.0f, od = 0.0f;
                for (int q = __ldg(a.rpa.seg_ptr + jl); q < __ldg(a.rpa.seg_ptr + jl + 1); ++q) {
                    const float2 p = slots[q];
                    os += p.x;
                    od += p.y;
                }
                kahan_add(acc_s[0], cmp_s[0], (2.0f * a.spin) * os);  // SU2FrgCore.cpp:265-266
                kahan_add(acc_d[0], cmp_d[0], (8.0f * a.spin) * od);
            }
        }
        channel(std::integral_constant<int, kU>{}, ui);

        // the single-flow kernel's combination of its groups: xor-shuffle order
        float vs[G], vd[G];
#pragma unroll
        for (int q = 0; q < G; ++q) {
            vs[q] = acc_s[q] - cmp_s[q];
            vd[q] = acc_d[q] - cmp_d[q];
        }
        float ts = vs[0], td = vd[0];
        if constexpr (G == 2) {
            ts = vs[0] + vs[1];
            td = vd[0] + vd[1];
        } else if constexpr (G == 4) {
            ts = (vs[0] + vs[1]) + (vs[2] + vs[3]);
            td = (vd[0] + vd[1]) + (vd[2] + vd[3]);
        }
        if (mine && ln.valid[0]) {
            const float two_pi = 2.0f * float(kPi);
            const float os = ts / two_pi, od = td / two_pi;
            m_dsd[fs][size_t(it) * a.nl + jl] = make_float2(os, od);
            if (isnan(os) || isnan(od)) atomicOr(m_status[fs], kStatusNaN);
        }
    }
}

// ------------------------------------------------------------------------------------
// Lattices of 33 to 128 sites: one CTA per triple (su2_vertex_big_kernel<R, NT>).
//
// Above 32 sites the t channel's outer-product matrix M = sum over nodes of (c A) x B (w x w,
// w = 16 R >= Nl) no longer fits one warp's registers, and a warp that owns a triple would walk
// the whole merged RPA pair list for every t-channel node (585 entries per lane and node for the
// 70-site pyrochlore range 7).  Here the CTA's NT threads (128 or 256) share a triple: they
// build up to 128 node descriptors at once (one per thread at 128 threads, one per lane pair
// at 256, make_pair), the NT / 32 warps evaluate the
// nodes round-robin (lane = site, ceil(w / 32) sites per lane), and in the t channel each warp
// writes its node's panel to shared memory (double-buffered: one block barrier per round of
// NT / 32 nodes), after which every thread adds the round's panels to its block of M (the
// threads form a 16 x NT/16 grid; a block is R x 2R for 128 threads, R x R for 256).  After
// the t channel M is staged in shared memory and the merged pair list is walked once per triple.
// Each warp keeps Kahan sums over its nodes per site; the warps' sums and the RPA term are
// combined in a fixed order, so results do not depend on the launch.
// ------------------------------------------------------------------------------------
constexpr int kBigBatch = 128;  // node descriptors built at once

__host__ __device__ constexpr int big_spt(int R) { return (16 * R + 31) / 32; }
// CTAs per SM the register budget is sized for (128 registers a thread up to w = 96; M of
// w = 128 takes a whole SM's shared memory anyway)
__host__ __device__ constexpr int big_min_blocks(int R, int NT) { return R > 6 ? 1 : 65536 / (128 * NT); }

struct BigSmem {
    size_t pos, u, panels, parts, rpa, total;
};
__host__ __device__ inline BigSmem big_smem_layout(int R, int NT, int n_seg) {
    const int w = 16 * R, NW = NT / 32;
    BigSmem L;
    size_t o = 0;
    L.pos = o; o += align16(sizeof(float) * kMaxFreq);
    // union: the descriptors of a node batch, or (after the t channel) M and the pair walk's
    // segment partials
    L.u = o;
    const size_t d = kBigBatch * sizeof(NodeDesc), m = sizeof(float2) * (size_t(w) * w + n_seg);
    o += align16(d > m ? d : m);
    L.panels = o; o += align16(sizeof(float2) * 2 * NW * 2 * size_t(w));  // 2 buffers x warps x (A, B)
    L.parts = o; o += align16(sizeof(float2) * NW * size_t(w));           // per warp and site
    L.rpa = o; o += align16(sizeof(float2) * size_t(w));
    L.total = o;
    return L;
}

// Adds a panel (A = c * third slab, B = fourth slab, w entries each) to the thread's block of M.
template <int R, int NT>
__device__ __forceinline__ void big_outer_update(const float2 *pan, int tid, float2 (*M)[16 * R / (NT / 16)]) {
    constexpr int w = 16 * R, TC = NT / 16, C = w / TC;
    const int tr = tid / TC, tc = tid % TC;
    float2 av[R], bv[C];
#pragma unroll
    for (int i = 0; i < R; ++i) av[i] = pan[tr * R + i];
#pragma unroll
    for (int j = 0; j < C; ++j) bv[j] = pan[w + tc * C + j];
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < C; ++j) M[i][j] = fma2(av[i], bv[j], M[i][j]);
}

// The flow of triple `it` of flow `a` by the whole CTA; `pos` the mesh in shared memory.
template <int R, int NT>
__device__ __forceinline__ void big_triple(const FlowArgs &a, const float *pos, int it, unsigned char *smem,
                                           const BigSmem &L) {
    constexpr int SPT = big_spt(R), w = 16 * R, NW = NT / 32, TC = NT / 16, C = w / TC;
    static_assert(NW == 4 || NW == 8, "the warps' sums combine as a tree of 4 or 8");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    NodeDesc *desc = reinterpret_cast<NodeDesc *>(smem + L.u);
    float2 *Ms = reinterpret_cast<float2 *>(smem + L.u);
    float2 *slots = Ms + w * w;
    float2 *panels = reinterpret_cast<float2 *>(smem + L.panels);
    float2 *parts = reinterpret_cast<float2 *>(smem + L.parts);
    float2 *rpa = reinterpret_cast<float2 *>(smem + L.rpa);

    const int su = it / a.n, ti = it - su * a.n;
    int si = int((sqrtf(8.0f * float(su) + 1.0f) - 1.0f) * 0.5f);
    while (si * (si + 1) / 2 > su) --si;
    while ((si + 1) * (si + 2) / 2 <= su) ++si;
    const int ui = su - si * (si + 1) / 2;
    Transfer f;
    f.s = pos[si];
    f.t = pos[ti];
    f.u = pos[ui];
    f.w1p = 0.5f * (f.s + f.t + f.u);
    f.w1 = 0.5f * (f.s - f.t + f.u);
    f.w2p = 0.5f * (f.s - f.t - f.u);
    f.w2 = 0.5f * (f.s + f.t - f.u);
    f.si = si;
    f.ti = ti;
    f.ui = ui;

    Lane<SPT> ln;
#pragma unroll
    for (int k = 0; k < SPT; ++k) {
        const int j = lane + 32 * k;
        ln.j[k] = j;
        ln.valid[k] = j < a.nl;
        // a lane past the last site reads the last site's element (never used), which lies
        // among the elements its slot's valid lanes read, not the slab's first line
        const int jc = ln.valid[k] ? j : a.nl - 1;
        ln.site[k] = a.sites[jc];
        ln.isite[k] = a.inv_sites[jc];
    }
    float acc_s[SPT], cmp_s[SPT], acc_d[SPT], cmp_d[SPT];
#pragma unroll
    for (int k = 0; k < SPT; ++k) acc_s[k] = cmp_s[k] = acc_d[k] = cmp_d[k] = 0.0f;
    float2 M[R][C];
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < C; ++j) M[i][j] = make_float2(0.0f, 0.0f);
    int round = 0;

    auto channel = [&](auto chc, int xi) {
        constexpr int CH = decltype(chc)::value;
        const int cnt = __ldg(a.node_cnt + xi);
        const float *nwp = a.node_wp + size_t(xi) * a.max_nodes;
        const float *nc = a.node_c + size_t(xi) * a.max_nodes;
        for (int b0 = 0; b0 < cnt; b0 += kBigBatch) {
            const int nb = min(kBigBatch, cnt - b0);
            __syncthreads();  // the previous batch's descriptors (or M) are no longer read
            if constexpr (NT >= 2 * kBigBatch) {  // a lane pair per node, half its buffers each
                const int k = tid >> 1;
                float c = 0.0f;
                int bits = 0;
                if (k < nb) {
                    c = __ldg(nc + b0 + k);
                    if (CH == kU) c = -c;
                    bits = make_pair<CH>(a, pos, f, __ldg(nwp + b0 + k), tid & 1, desc[k]);
                }
                bits |= __shfl_xor_sync(0xffffffffu, bits, 1);
                if (k < nb && !(tid & 1)) {
                    desc[k].exch = bits;
                    desc[k].c = c;
                }
            } else if (tid < nb) {
                float c = __ldg(nc + b0 + tid);
                if (CH == kU) c = -c;
                make_desc<CH>(a, pos, f, __ldg(nwp + b0 + tid), c, desc[tid]);
            }
            __syncthreads();
            if constexpr (CH != kT) {
                for (int k = warp; k < nb; k += NW) {
                    const NodeView v{&desc[k], desc[k].c, desc[k].lv};
                    float rs[1][SPT], rd[1][SPT];
                    node_term<CH, SPT, 1>(a, &v, ln, lane, nullptr, rs, rd);
#pragma unroll
                    for (int q = 0; q < SPT; ++q) {
                        kahan_add(acc_s[q], cmp_s[q], v.c * rs[0][q]);
                        kahan_add(acc_d[q], cmp_d[q], v.c * rd[0][q]);
                    }
                }
            } else {
                for (int r0 = 0; r0 < nb; r0 += NW, ++round) {
                    const int k = r0 + warp;
                    float2 *buf = panels + size_t(round & 1) * NW * 2 * w;
                    if (k < nb) {
                        const NodeView v{&desc[k], desc[k].c, desc[k].lv};
                        TExchange tx;
                        tx.A2 = buf + warp * 2 * w;
                        tx.B2 = tx.A2 + w;
                        float rs[1][SPT], rd[1][SPT];
                        node_term<kT, SPT, 1>(a, &v, ln, lane, &tx, rs, rd);
#pragma unroll
                        for (int q = 0; q < SPT; ++q) {
                            kahan_add(acc_s[q], cmp_s[q], v.c * rs[0][q]);
                            kahan_add(acc_d[q], cmp_d[q], v.c * rd[0][q]);
                        }
                    }
                    __syncthreads();  // the round's panels are written
                    const int np = min(NW, nb - r0);
                    for (int p = 0; p < np; ++p) big_outer_update<R, NT>(buf + p * 2 * w, tid, M);
                }
            }
        }
    };

    channel(std::integral_constant<int, kS>{}, si);
    channel(std::integral_constant<int, kT>{}, ti);
    // RPA term: M staged, the merged pair list walked once (one chunk per thread), per-site sums
    __syncthreads();  // every panel update and every descriptor read is done
    {
        const int tr = tid / TC, tc = tid % TC;
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < C; ++j) Ms[(tr * R + i) * w + tc * C + j] = M[i][j];
    }
    __syncthreads();
    if (tid < a.rpa.lanes) {  // the schedule of these lattices has one chunk per thread
        const int lanes = a.rpa.lanes;
        const int cntq = __ldg(a.rpa.count + tid);
        int slot = __ldg(a.rpa.slot_base + tid);
        const int *sched = a.rpa.sched + tid;
        float2 acc = make_float2(0.0f, 0.0f);
        for (int i = 0; i < cntq; ++i) {
            const int e = __ldg(sched + size_t(i) * lanes);
            const float m = float((e >> 14) & 0xff);
            const int ra = e & 0x7f, rb = (e >> 7) & 0x7f;
            acc = fma2(make_float2(m, m), Ms[ra * w + rb], acc);
            if (e & (1 << 22)) {
                slots[slot++] = acc;
                acc = make_float2(0.0f, 0.0f);
            }
        }
    }
    __syncthreads();
    if (tid < a.nl) {
        float2 sum = make_float2(0.0f, 0.0f);
        for (int q = __ldg(a.rpa.seg_ptr + tid); q < __ldg(a.rpa.seg_ptr + tid + 1); ++q) {
            const float2 p = slots[q];
            sum.x += p.x;
            sum.y += p.y;
        }
        rpa[tid] = sum;
    }
    channel(std::integral_constant<int, kU>{}, ui);  // its first barrier publishes rpa[]

    // the warps' sums per site (a pairwise tree), then the RPA term (SU2FrgCore.cpp:265-266)
#pragma unroll
    for (int k = 0; k < SPT; ++k)
        if (ln.valid[k]) parts[warp * w + ln.j[k]] = make_float2(acc_s[k] - cmp_s[k], acc_d[k] - cmp_d[k]);
    __syncthreads();
    if (tid < a.nl) {
        float2 p[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) p[q] = parts[q * w + tid];
        float vs = (p[0].x + p[1].x) + (p[2].x + p[3].x), vd = (p[0].y + p[1].y) + (p[2].y + p[3].y);
        if constexpr (NW == 8) {
            vs = vs + ((p[4].x + p[5].x) + (p[6].x + p[7].x));
            vd = vd + ((p[4].y + p[5].y) + (p[6].y + p[7].y));
        }
        const float2 r = rpa[tid];
        vs = vs + (2.0f * a.spin) * r.x;
        vd = vd + (8.0f * a.spin) * r.y;
        const float two_pi = 2.0f * float(kPi);
        const float os = vs / two_pi, od = vd / two_pi;
        a.dsd[size_t(it) * a.nl + tid] = make_float2(os, od);
        if (isnan(os) || isnan(od)) atomicOr(a.status, kStatusNaN);
    }
}

template <int R, int NT>
__global__ void __launch_bounds__(NT, big_min_blocks(R, NT)) su2_vertex_big_kernel(FlowArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    const BigSmem L = big_smem_layout(R, NT, a.rpa.n_seg);
    float *pos = reinterpret_cast<float *>(smem_raw + L.pos);
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    for (;;) {
        __syncthreads();  // the previous triple is finished with shared memory
        if (threadIdx.x == 0) s_item = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.fn) break;
        big_triple<R, NT>(a, pos, it, smem_raw, L);
    }
}

// Batched form: a persistent grid over the ragged (flow, triple) list of the batch's flows of
// one big class; the CTA reloads the flow's argument block and mesh when the flow changes
// (items are numbered flow by flow).
template <int R, int NT>
__global__ void __launch_bounds__(NT, big_min_blocks(R, NT)) su2_vertex_big_batch_kernel(BatchVertexArgs b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    __shared__ __align__(16) FlowArgs fa;
    const BigSmem L = big_smem_layout(R, NT, b.n_seg_max);
    float *pos = reinterpret_cast<float *>(smem_raw + L.pos);
    int cur = -1, base = 0;
    bool skip = false;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(b.counter, 1);
        __syncthreads();
        const int w = s_item;
        if (w >= b.total) break;
        int lo = 0, hi = b.n_list - 1;  // last f with prefix[f] <= w
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(b.prefix + mid) <= w) lo = mid;
            else hi = mid - 1;
        }
        if (lo != cur) {
            cur = lo;
            base = __ldg(b.prefix + lo);
            const BatchFlow *bf = b.flows + __ldg(b.list + lo);
            const int *src = reinterpret_cast<const int *>(&bf->a);
            int *dst = reinterpret_cast<int *>(&fa);
            for (int i = threadIdx.x; i < int(sizeof(FlowArgs) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
            skip = bf->phase != kPhaseFlowing;
            __syncthreads();
            for (int i = threadIdx.x; i < fa.n; i += blockDim.x) pos[i] = fa.freq[i];
            __syncthreads();
        }
        if (skip) continue;
        big_triple<R, NT>(fa, pos, w - base, smem_raw, L);
    }
}

int spt_of(int nl) { return nl <= 32 ? 1 : (nl <= 64 ? 2 : 4); }

int wsite_of(int nl) {
    if (nl > 32) return 32;
    int w = 1;
    while (w < nl) w <<= 1;
    return w;
}

int outer_w_of(int nl) { return nl <= 32 ? rpa_outer_width(nl) : 0; }

}  // namespace

// Lattices of 33 to 128 sites use the CTA-per-triple kernel: w = 16 R >= Nl, R = 3 with 128
// threads, R = 4, 5, 6, 8 with 256 (classes 6..10).
int big_r_of(int nl) {
    return nl <= 32 ? 0 : (nl <= 48 ? 3 : (nl <= 64 ? 4 : (nl <= 80 ? 5 : (nl <= 96 ? 6 : 8))));
}
int big_class_r(int cls) { return cls == 6 ? 3 : (cls == 7 ? 4 : (cls == 8 ? 5 : (cls == 9 ? 6 : 8))); }
int big_threads(int r) { return r <= 3 ? 128 : 256; }

int vertex_rpa_lanes(int nl) { return big_r_of(nl) ? big_threads(big_r_of(nl)) : 32; }

int vertex_class(int nl) {
    switch (big_r_of(nl)) {
        case 0: return rpa_outer_width(nl) / 8 - 1;  // 0..3: a warp per triple, blocks of 1..4 rows
        case 3: return 6;
        case 4: return 7;
        case 5: return 8;
        case 6: return 9;
        default: return 10;
    }
}

size_t vertex_flow_smem_bytes(int nl, const RpaSchedule &rpa, int npi) {
    if (const int r = big_r_of(nl)) return big_smem_layout(r, big_threads(r), rpa.n_seg).total;
    const int spt = spt_of(nl);
    return kMaxFreq * sizeof(float) + sched_bytes(rpa, nl) +
           kWarps * warp_bytes(spt == 1 ? wsite_of(nl) : 32, spt, npi, rpa.n_seg, outer_w_of(nl));
}

namespace {
using VertexKernel = void (*)(FlowArgs);
template <int SPT, int MB>
VertexKernel vertex_kernel_npi(int npi) {
    return npi == 1 ? su2_vertex_flow_kernel<SPT, 1, MB> : su2_vertex_flow_kernel<SPT, 2, MB>;
}
VertexKernel vertex_kernel(int cls, int npi) {
    switch (cls) {
        case 0: return vertex_kernel_npi<1, 1>(npi);
        case 1: return vertex_kernel_npi<1, 2>(npi);
        case 2: return vertex_kernel_npi<1, 3>(npi);
        case 3: return vertex_kernel_npi<1, 4>(npi);
        case 6: return su2_vertex_big_kernel<3, 128>;
        case 7: return su2_vertex_big_kernel<4, 256>;
        case 8: return su2_vertex_big_kernel<5, 256>;
        case 9: return su2_vertex_big_kernel<6, 256>;
        default: return su2_vertex_big_kernel<8, 256>;
    }
}
int threads_of(int cls) { return cls >= 6 ? big_threads(big_class_r(cls)) : kThreads; }
}  // namespace

// The CTA-per-triple kernel (33..128 sites) has no variants: nodes per iteration and the
// schedule's place do not apply, and every setting launches the same kernel.
int vertex_flow_blocks_per_sm(int nl, const RpaSchedule &rpa, int npi) {
    const size_t smem = vertex_flow_smem_bytes(nl, rpa, npi);
    const int cls = vertex_class(nl);
    VertexKernel k = vertex_kernel(cls, npi);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads_of(cls), smem) != cudaSuccess) return -1;
    return per_sm;
}

void launch_vertex_flow(const FlowArgs &a, int npi, int grid, cudaStream_t stream) {
    const size_t smem = vertex_flow_smem_bytes(a.nl, a.rpa, npi);
    const int cls = vertex_class(a.nl);
    VertexKernel k = vertex_kernel(cls, npi);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    k<<<grid, threads_of(cls), smem, stream>>>(a);
}

int vertex_spt(int nl) { return spt_of(nl); }

size_t batch_vertex_warp_area(int nl, int n_seg, int npi) {
    const int spt = spt_of(nl);
    // everything after the descriptors: the group areas, or the outer-product stage
    return warp_bytes(spt == 1 ? wsite_of(nl) : 32, spt, npi, n_seg, outer_w_of(nl)) - kBatch * sizeof(NodeDesc);
}

size_t batch_vertex_smem_bytes(int n_max, size_t warp_area, int sched_ints) {
    return kWarps * (align16(sizeof(FlowArgs)) + align16(sizeof(float) * n_max) + align16(sizeof(int) * size_t(sched_ints)) +
                     kBatch * sizeof(NodeDesc) + warp_area);
}

namespace {
using BatchKernel = void (*)(BatchVertexArgs);
template <int SPT, int MB>
BatchKernel batch_kernel_npi(int npi) {
    return npi == 1 ? su2_vertex_batch_kernel<SPT, 1, MB> : su2_vertex_batch_kernel<SPT, 2, MB>;
}
BatchKernel batch_kernel(int cls, int npi) {
    switch (cls) {
        case 0: return batch_kernel_npi<1, 1>(npi);
        case 1: return batch_kernel_npi<1, 2>(npi);
        case 2: return batch_kernel_npi<1, 3>(npi);
        case 3: return batch_kernel_npi<1, 4>(npi);
        case 6: return su2_vertex_big_batch_kernel<3, 128>;
        case 7: return su2_vertex_big_batch_kernel<4, 256>;
        case 8: return su2_vertex_big_batch_kernel<5, 256>;
        case 9: return su2_vertex_big_batch_kernel<6, 256>;
        default: return su2_vertex_big_batch_kernel<8, 256>;
    }
}
}  // namespace

size_t batch_big_smem_bytes(int cls, int n_seg_max) {
    const int r = big_class_r(cls);
    return big_smem_layout(r, big_threads(r), n_seg_max).total;
}

int batch_vertex_blocks_per_sm(int cls, int npi, size_t smem) {
    BatchKernel k = batch_kernel(cls, npi);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads_of(cls), smem) != cudaSuccess) return -1;
    return per_sm;
}

// The kernel's shared-memory limit is raised by batch_vertex_blocks_per_sm when the plan is
// built, so this launch can be captured into a graph.
void launch_batch_vertex(const BatchVertexArgs &b, int cls, int npi, int grid, cudaStream_t stream) {
    const size_t smem = cls >= 6 ? batch_big_smem_bytes(cls, b.n_seg_max)
                                 : batch_vertex_smem_bytes(b.n_max, size_t(b.warp_area), b.sched_ints);
    batch_kernel(cls, npi)<<<grid, threads_of(cls), smem, stream>>>(b);
}

namespace {
using GroupKernel = void (*)(GroupVertexArgs);
GroupKernel group_kernel(int cls) {
    switch (cls) {
        case 0: return su2_vertex_group_kernel<8, 1>;
        case 1: return su2_vertex_group_kernel<16, 2>;
        case 2: return su2_vertex_group_kernel<32, 3>;
        default: return su2_vertex_group_kernel<32, 4>;
    }
}
int group_w(int cls) { return cls == 0 ? 8 : (cls == 1 ? 16 : 32); }
}  // namespace

bool group_vertex_eligible(int nl) { return nl >= 5 && nl <= 32; }

int group_vertex_gmax(int cls) { return kGroupWarps * (32 / group_w(cls)); }

size_t group_vertex_smem_bytes(int cls, int n_seg_max) {
    return group_smem_layout(group_w(cls), cls + 1, n_seg_max).total;
}

int group_vertex_blocks_per_sm(int cls, int n_seg_max) {
    GroupKernel k = group_kernel(cls);
    const size_t smem = group_vertex_smem_bytes(cls, n_seg_max);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kGroupWarps * 32, smem) != cudaSuccess) return -1;
    return per_sm;
}

// The shared-memory limit is raised by group_vertex_blocks_per_sm when the plan is built, so
// this launch can be captured into a graph.
void launch_group_vertex(const GroupVertexArgs &g, int cls, int grid, cudaStream_t stream) {
    group_kernel(cls)<<<grid, kGroupWarps * 32, group_vertex_smem_bytes(cls, g.n_seg_max), stream>>>(g);
}

}  // namespace spn
