// Device-side building blocks of the SU(2) flow: Matsubara-mesh searches, vertex access
// buffers (frequency folding + interpolation supports) and the trapezoid quadrature nodes.
//
// Every float operation that decides an index, a branch or a site exchange is written so
// that it rounds exactly like the reference's scalar C++ (no fused multiply-add can form in
// these expressions: they are single adds/subtracts, products of differences, or IEEE
// divisions).  The searches are binary searches over the ascending positive mesh with the
// tie rules of the reference's linear scans (src/FrequencyDiscretization.hpp:253-356).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>

namespace spn {
namespace dev {

constexpr int kMaxFreq = 256;  // largest supported N (positive frequencies)

// (spin, density) pair of the working precision: the element type of a device vertex array.
template <class T>
struct pair_of;
template <>
struct pair_of<float> {
    using type = float2;
};
template <>
struct pair_of<double> {
    using type = double2;
};
template <class T>
using pair_t = typename pair_of<T>::type;

// Read access to a vertex state by element index ((s(s+1)/2+u)*N + t)*Nl + rid.
// PairedState: the device layout, (spin, density) interleaved per element;
// SplitState: two separate arrays (the reference's layout, as callers of the allocation-free
// measurement hold it).
template <class T>
struct PairedState {
    const pair_t<T> *v;
    __device__ __forceinline__ T spin(int i) const { return __ldg(reinterpret_cast<const T *>(v) + 2 * i); }
    __device__ __forceinline__ T density(int i) const { return __ldg(reinterpret_cast<const T *>(v) + 2 * i + 1); }
    __device__ __forceinline__ pair_t<T> both(int i) const { return __ldg(v + i); }
};
template <class T>
struct SplitState {
    const T *ss, *dd;
    __device__ __forceinline__ T spin(int i) const { return __ldg(ss + i); }
    __device__ __forceinline__ T density(int i) const { return __ldg(dd + i); }
    __device__ __forceinline__ pair_t<T> both(int i) const {
        pair_t<T> p;
        p.x = __ldg(ss + i);
        p.y = __ldg(dd + i);
        return p;
    }
};

// The mesh searches, interpolations and quadrature rules below also compile for the host, where
// the library's diagnostics (spn_mesh_probe, spn_quadrature_nodes) run the same code.
#define SPN_HDI __host__ __device__ __forceinline__

// Single IEEE operations rounded to nearest in the working precision T (float: the
// reference's types; double: the FP64 flow).  On the host: plain operators, compiled without
// floating-point contraction.
#ifdef __CUDA_ARCH__
SPN_HDI float rn_add(float a, float b) { return __fadd_rn(a, b); }
SPN_HDI double rn_add(double a, double b) { return __dadd_rn(a, b); }
SPN_HDI float rn_sub(float a, float b) { return __fsub_rn(a, b); }
SPN_HDI double rn_sub(double a, double b) { return __dsub_rn(a, b); }
SPN_HDI float rn_mul(float a, float b) { return __fmul_rn(a, b); }
SPN_HDI double rn_mul(double a, double b) { return __dmul_rn(a, b); }
SPN_HDI float rn_div(float a, float b) { return __fdiv_rn(a, b); }
SPN_HDI double rn_div(double a, double b) { return __ddiv_rn(a, b); }
#else
SPN_HDI float rn_add(float a, float b) { return a + b; }
SPN_HDI double rn_add(double a, double b) { return a + b; }
SPN_HDI float rn_sub(float a, float b) { return a - b; }
SPN_HDI double rn_sub(double a, double b) { return a - b; }
SPN_HDI float rn_mul(float a, float b) { return a * b; }
SPN_HDI double rn_mul(double a, double b) { return a * b; }
SPN_HDI float rn_div(float a, float b) { return a / b; }
SPN_HDI double rn_div(double a, double b) { return a / b; }
#endif

// A read of the flow's read-only state: through the non-coherent cache on the device, a plain
// read on the host.
template <class T>
SPN_HDI T ro_load(const T *p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

// First index i in [1, n) with pos[i] > w; n if none (also for NaN w).
template <class T>
SPN_HDI int first_greater(const T *pos, int n, T w) {
    int lo = 1, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (pos[mid] > w) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// First index i in [1, n) with pos[i] >= w; n if none.
template <class T>
SPN_HDI int first_geq(const T *pos, int n, T w) {
    int lo = 1, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (pos[mid] >= w) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// FrequencyDiscretization::offset (w >= 0): index of the mesh point equal to w.
template <class T>
SPN_HDI int mesh_offset(const T *pos, int n, T w) {
    if (w <= pos[0]) return 0;
    int i = first_geq(pos, n, w);
    return i < n ? i : n - 1;
}

// FrequencyDiscretization::interpolateOffset (w >= 0).
template <class T>
SPN_HDI void mesh_interp(const T *pos, int n, T w, int &lo, int &hi, T &bias) {
    if (w <= pos[0]) {
        lo = hi = 0;
        bias = T(0);
        return;
    }
    int i = first_greater(pos, n, w);
    if (i < n) {
        hi = i;
        lo = i - 1;
        bias = rn_div(rn_sub(w, pos[lo]), rn_sub(pos[hi], pos[lo]));
    } else {
        lo = hi = n - 1;
        bias = T(0);
    }
}

// Bucket index over the float bit patterns of the positive mesh (FP32 flows; built on the
// host by build_mesh_index): bucket b covers the patterns [base + (b << shift), base +
// (b+1 << shift)), and lo[b] is the first i >= 1 with pos[i] at or above the bucket's start.
// Every i below lo[bucket(w)] has pos[i] < w, so the searches start there and finish with the
// same comparisons as the binary searches above (identical results, NaN included); for a
// mesh whose buckets hold at most a point or two that is one table read and a step or two.
constexpr int kMeshBuckets = 512;

struct MeshIndex {
    const float *pos;
    int n;
    const unsigned short *lo;  // [kMeshBuckets]
    unsigned base;
    int shift;
    SPN_HDI int start(float w) const {
#ifdef __CUDA_ARCH__
        const unsigned key = __float_as_uint(w);
#else
        unsigned key;
        std::memcpy(&key, &w, sizeof key);
#endif
        unsigned b = key >= base ? (key - base) >> shift : 0u;
        if (b >= unsigned(kMeshBuckets)) b = kMeshBuckets - 1;
#ifdef __CUDA_ARCH__
        return __ldg(lo + b);
#else
        return lo[b];
#endif
    }
    SPN_HDI int first_greater(float w) const {  // as first_greater(pos, n, w)
        int i = start(w);
        while (i < n && !(pos[i] > w)) ++i;
        return i;
    }
    SPN_HDI int first_geq(float w) const {  // as first_geq(pos, n, w)
        int i = start(w);
        while (i < n && !(pos[i] >= w)) ++i;
        return i;
    }
};

// The two mesh lookups an access buffer needs, by binary search (MeshSearch) or through a
// bucket index (MeshIndex); w >= 0.
template <class T>
struct MeshSearch {
    const T *pos;
    int n;
    SPN_HDI int first_greater(T w) const { return dev::first_greater(pos, n, w); }
    SPN_HDI int first_geq(T w) const { return dev::first_geq(pos, n, w); }
};

template <class T, class M>
SPN_HDI int mesh_offset_m(const M &m, T w) {
    if (w <= m.pos[0]) return 0;
    int i = m.first_geq(w);
    return i < m.n ? i : m.n - 1;
}

template <class T, class M>
SPN_HDI void mesh_interp_m(const M &m, T w, int &lo, int &hi, T &bias) {
    if (w <= m.pos[0]) {
        lo = hi = 0;
        bias = T(0);
        return;
    }
    int i = m.first_greater(w);
    if (i < m.n) {
        hi = i;
        lo = i - 1;
        bias = rn_div(rn_sub(w, m.pos[lo]), rn_sub(m.pos[hi], m.pos[lo]));
    } else {
        lo = hi = m.n - 1;
        bias = T(0);
    }
}

// Index into the symmetric mesh -w[n-1] .. -w[0], w[0] .. w[n-1] (0 .. 2n-1).
template <class T>
SPN_HDI T full_value(const T *pos, int n, int k) { return k < n ? -pos[n - 1 - k] : pos[k - n]; }

template <class T>
SPN_HDI int pos_lesser(const T *pos, int n, T w) {  // w >= 0, returns positive index
    if (w <= pos[0]) return 0;
    int i = first_greater(pos, n, w);
    return i < n ? i - 1 : n - 1;
}
template <class T>
SPN_HDI int pos_greater(const T *pos, int n, T w) {  // w >= 0
    if (w <= pos[0]) return 0;
    int i = first_greater(pos, n, w);
    return i < n ? i : n - 1;
}
// FrequencyDiscretization::lesser / greater on the full mesh (full index).
template <class T>
SPN_HDI int full_lesser(const T *pos, int n, T w) {
    if (w < 0) return n - 1 - pos_greater(pos, n, -w);
    return n + pos_lesser(pos, n, w);
}
template <class T>
SPN_HDI int full_greater(const T *pos, int n, T w) {
    if (w < 0) return n - 1 - pos_lesser(pos, n, -w);
    return n + pos_greater(pos, n, w);
}

// Linear interpolation of a function stored on the positive mesh and odd in w
// (SU2VertexSingleParticle::getValue, src/SU2/SU2VertexSingleParticle.hpp:73-87).
template <class P, class T>
SPN_HDI double odd_interp(const P *pos, int n, const T *data, P w) {
    double sign = 1.0;
    if (w < 0) {
        w = -w;
        sign = -1.0;
    }
    int lo, hi;
    P b;
    mesh_interp(pos, n, w, lo, hi, b);
    return sign * ((1.0 - double(b)) * double(data[lo]) + double(b) * double(data[hi]));
}

// Access buffer with four interpolation supports (SU2VertexTwoParticleAccessBuffer<4>).
template <class T>
struct AB4T {
    int off[4];    // element offset of the (s,t,u) slab start; add the site index
    T w[4];        // interpolation weight
    T sw[4];       // sign * weight (density channel)
    bool exch;     // read the site-exchanged pair
};

template <class T>
struct AB8T {
    int off[8];
    T w[8];
    T sw[8];
    bool exch;
};
using AB4 = AB4T<float>;
using AB8 = AB8T<float>;

// _generateAccessBufferOffset: storage keeps s >= u; a swapped pair flips the density sign.
template <class T>
SPN_HDI void slab(int si, int ti, int ui, int stepT, int nl, int &off, T w, T &wout, T &swout) {
    if (si < ui) {
        off = (ui * (ui + 1) / 2 + si) * stepT + ti * nl;
        wout = w;
        swout = -w;
    } else {
        off = (si * (si + 1) / 2 + ui) * stepT + ti * nl;
        wout = w;
        swout = w;
    }
}

// Frequency folding into the stored sector (SU2VertexTwoParticle.hpp:405-427).
template <class T>
SPN_HDI bool fold(T &s, T &t, T &u) {
    bool exch = false;
    if (s < 0 && u < 0) {
        s = -s;
        u = -u;
    } else {
        if (s < 0) {
            s = -s;
            exch = true;
        } else if (u < 0) {
            u = -u;
            exch = true;
        }
    }
    if (t < 0) t = -t;
    return exch;
}

enum Channel { kS = 0, kT = 1, kU = 2 };

// generateAccessBuffer(s, t, u, channel) for channel in {S, T, U}
// (src/SU2/SU2VertexTwoParticle.hpp:399-490); `m` looks up the positive mesh.  `e_known` >= 0:
// the exact mesh index of the channel's own coordinate, which the caller knows when that
// coordinate is (up to sign) a mesh value (offset(w_i) = i on a strictly ascending mesh).
template <int CH, class T, class M>
SPN_HDI void access4m(const M &m, int nl, T s, T t, T u, AB4T<T> &ab, int e_known = -1) {
    ab.exch = fold(s, t, u);
    const int stepT = m.n * nl;
    int e, la, ua, lb, ub;
    T ba, bb;
    if (CH == kS) {
        e = e_known >= 0 ? e_known : mesh_offset_m(m, s);
        mesh_interp_m(m, t, la, ua, ba);
        mesh_interp_m(m, u, lb, ub, bb);
    } else if (CH == kT) {
        e = e_known >= 0 ? e_known : mesh_offset_m(m, t);
        mesh_interp_m(m, s, la, ua, ba);
        mesh_interp_m(m, u, lb, ub, bb);
    } else {
        e = e_known >= 0 ? e_known : mesh_offset_m(m, u);
        mesh_interp_m(m, s, la, ua, ba);
        mesh_interp_m(m, t, lb, ub, bb);
    }
    const T na = rn_sub(T(1), ba), nb = rn_sub(T(1), bb);
    const T w0 = rn_mul(nb, na), w1 = rn_mul(nb, ba), w2 = rn_mul(bb, na), w3 = rn_mul(bb, ba);
    if (CH == kS) {
        slab(e, la, lb, stepT, nl, ab.off[0], w0, ab.w[0], ab.sw[0]);
        slab(e, ua, lb, stepT, nl, ab.off[1], w1, ab.w[1], ab.sw[1]);
        slab(e, la, ub, stepT, nl, ab.off[2], w2, ab.w[2], ab.sw[2]);
        slab(e, ua, ub, stepT, nl, ab.off[3], w3, ab.w[3], ab.sw[3]);
    } else if (CH == kT) {
        slab(la, e, lb, stepT, nl, ab.off[0], w0, ab.w[0], ab.sw[0]);
        slab(ua, e, lb, stepT, nl, ab.off[1], w1, ab.w[1], ab.sw[1]);
        slab(la, e, ub, stepT, nl, ab.off[2], w2, ab.w[2], ab.sw[2]);
        slab(ua, e, ub, stepT, nl, ab.off[3], w3, ab.w[3], ab.sw[3]);
    } else {
        slab(la, lb, e, stepT, nl, ab.off[0], w0, ab.w[0], ab.sw[0]);
        slab(ua, lb, e, stepT, nl, ab.off[1], w1, ab.w[1], ab.sw[1]);
        slab(la, ub, e, stepT, nl, ab.off[2], w2, ab.w[2], ab.sw[2]);
        slab(ua, ub, e, stepT, nl, ab.off[3], w3, ab.w[3], ab.sw[3]);
    }
}

// One mesh interpolation (lo, hi, bias) of |w|.  The access buffers of a node interpolate at
// most four distinct magnitudes: a coordinate and its negation (-a - b is bitwise -(a + b)
// under round-to-nearest) fold to the same value, so make_desc looks each up once.
template <class T>
struct Interp {
    int lo, hi;
    T b;
};
template <class T, class M>
SPN_HDI Interp<T> interp_abs(const M &m, T w) {
    Interp<T> r;
    mesh_interp_m(m, w < T(0) ? -w : w, r.lo, r.hi, r.b);
    return r;
}

// access4m with the two interpolations given: ia for the first interpolated coordinate after
// folding (t for S, s for T and U), ib for the second (u for S and T, t for U).  The caller
// passes interp_abs of the matching coordinates; folding, weights and offsets are access4m's.
template <int CH, class T>
SPN_HDI void access4i(int n, int nl, T s, T t, T u, const Interp<T> &ia, const Interp<T> &ib,
                                         int e, AB4T<T> &ab) {
    ab.exch = fold(s, t, u);
    const int stepT = n * nl;
    const int la = ia.lo, ua = ia.hi, lb = ib.lo, ub = ib.hi;
    const T ba = ia.b, bb = ib.b;
    const T na = rn_sub(T(1), ba), nb = rn_sub(T(1), bb);
    const T w0 = rn_mul(nb, na), w1 = rn_mul(nb, ba), w2 = rn_mul(bb, na), w3 = rn_mul(bb, ba);
    if (CH == kS) {
        slab(e, la, lb, stepT, nl, ab.off[0], w0, ab.w[0], ab.sw[0]);
        slab(e, ua, lb, stepT, nl, ab.off[1], w1, ab.w[1], ab.sw[1]);
        slab(e, la, ub, stepT, nl, ab.off[2], w2, ab.w[2], ab.sw[2]);
        slab(e, ua, ub, stepT, nl, ab.off[3], w3, ab.w[3], ab.sw[3]);
    } else if (CH == kT) {
        slab(la, e, lb, stepT, nl, ab.off[0], w0, ab.w[0], ab.sw[0]);
        slab(ua, e, lb, stepT, nl, ab.off[1], w1, ab.w[1], ab.sw[1]);
        slab(la, e, ub, stepT, nl, ab.off[2], w2, ab.w[2], ab.sw[2]);
        slab(ua, e, ub, stepT, nl, ab.off[3], w3, ab.w[3], ab.sw[3]);
    } else {
        slab(la, lb, e, stepT, nl, ab.off[0], w0, ab.w[0], ab.sw[0]);
        slab(ua, lb, e, stepT, nl, ab.off[1], w1, ab.w[1], ab.sw[1]);
        slab(la, ub, e, stepT, nl, ab.off[2], w2, ab.w[2], ab.sw[2]);
        slab(ua, ub, e, stepT, nl, ab.off[3], w3, ab.w[3], ab.sw[3]);
    }
}

template <int CH, class T>
SPN_HDI void access4(const T *pos, int n, int nl, T s, T t, T u, AB4T<T> &ab) {
    access4m<CH>(MeshSearch<T>{pos, n}, nl, s, t, u, ab);
}

// generateAccessBuffer(s, t, u): trilinear, eight supports (SU2VertexTwoParticle.hpp:500-557).
template <class T>
SPN_HDI void access8(const T *pos, int n, int nl, T s, T t, T u, AB8T<T> &ab) {
    ab.exch = fold(s, t, u);
    const int stepT = n * nl;
    int ls, us, lt, ut, lu, uu;
    T bs, bt, bu;
    mesh_interp(pos, n, s, ls, us, bs);
    mesh_interp(pos, n, t, lt, ut, bt);
    mesh_interp(pos, n, u, lu, uu, bu);
    const T ns = rn_sub(T(1), bs), nt = rn_sub(T(1), bt), nu = rn_sub(T(1), bu);
    slab(ls, lt, lu, stepT, nl, ab.off[0], rn_mul(rn_mul(nt, ns), nu), ab.w[0], ab.sw[0]);
    slab(us, lt, lu, stepT, nl, ab.off[1], rn_mul(rn_mul(nt, bs), nu), ab.w[1], ab.sw[1]);
    slab(ls, ut, lu, stepT, nl, ab.off[2], rn_mul(rn_mul(bt, ns), nu), ab.w[2], ab.sw[2]);
    slab(us, ut, lu, stepT, nl, ab.off[3], rn_mul(rn_mul(bt, bs), nu), ab.w[3], ab.sw[3]);
    slab(ls, lt, uu, stepT, nl, ab.off[4], rn_mul(rn_mul(nt, ns), bu), ab.w[4], ab.sw[4]);
    slab(us, lt, uu, stepT, nl, ab.off[5], rn_mul(rn_mul(nt, bs), bu), ab.w[5], ab.sw[5]);
    slab(ls, ut, uu, stepT, nl, ab.off[6], rn_mul(rn_mul(bt, ns), bu), ab.w[6], ab.sw[6]);
    slab(us, ut, uu, stepT, nl, ab.off[7], rn_mul(rn_mul(bt, bs), bu), ab.w[7], ab.sw[7]);
}

// SU2VertexTwoParticle::_directAccessMapFrequencyExchange for one site (density: the density
// channel, whose sign flips when the stored sector swaps s and u; else the spin channel).
template <class T, class S>
SPN_HDI T direct(const S &v, int si, int ti, int ui, int site, int stepT, int nl, bool density) {
    if (si >= ui) {
        const int i = (si * (si + 1) / 2 + ui) * stepT + ti * nl + site;
        return density ? v.density(i) : v.spin(i);
    }
    const int i = (ui * (ui + 1) / 2 + si) * stepT + ti * nl + site;
    return density ? -v.density(i) : v.spin(i);
}

// getValue(i1, i2, s, t, u, symmetry, FrequencyChannel::None) where the site pair enters
// through its rid (rid12) and the rid of the exchanged pair (rid21).
template <class T, class S>
SPN_HDI T value_none(const T *pos, int n, int nl, const S &v, bool density, int rid12, int rid21,
                                        T s, T t, T u) {
    bool exch = fold(s, t, u);
    const int site = exch ? rid21 : rid12;
    const int stepT = n * nl;
    int ls, us, lt, ut, lu, uu;
    T bs, bt, bu;
    mesh_interp(pos, n, s, ls, us, bs);
    mesh_interp(pos, n, t, lt, ut, bt);
    mesh_interp(pos, n, u, lu, uu, bu);
    auto D = [&](int a, int b, int c) { return direct<T>(v, a, b, c, site, stepT, nl, density); };
    return (1 - bu) * ((1 - bt) * ((1 - bs) * D(ls, lt, lu) + bs * D(us, lt, lu)) + bt * ((1 - bs) * D(ls, ut, lu) + bs * D(us, ut, lu))) +
           bu * ((1 - bt) * ((1 - bs) * D(ls, lt, uu) + bs * D(us, lt, uu)) + bt * ((1 - bs) * D(ls, ut, uu) + bs * D(us, ut, uu)));
}

// ---- trapezoid quadrature nodes (ImplicitIntegrator, src/lib/Integrator.hpp:137-287) ----
// Each rule calls emit(wp, weight) once per integrand evaluation of the reference, in the
// same order, with weight = 0.5 * (the float node spacing the reference multiplies by).

// integrateWithObscureLeftBoundary(min, last)
template <class T, class Emit>
__host__ __device__ void nodes_left(const T *pos, int n, T min, Emit &&emit) {
    const int maxi = 2 * n - 1;
    int um = full_greater(pos, n, min);
    if (um != maxi) {
        emit(min, 0.5 * double(rn_sub(full_value(pos, n, um), min)));
        emit(full_value(pos, n, um), 0.5 * double(rn_sub(full_value(pos, n, um + 1), min)));
        while (++um != maxi)
            emit(full_value(pos, n, um), 0.5 * double(rn_sub(full_value(pos, n, um + 1), full_value(pos, n, um - 1))));
        emit(full_value(pos, n, um), 0.5 * double(rn_sub(full_value(pos, n, um), full_value(pos, n, um - 1))));
    } else {
        const double w = double(rn_mul(T(0.5), rn_sub(full_value(pos, n, um), min)));
        emit(min, w);
        emit(full_value(pos, n, um), w);
    }
}

// integrateWithObscureRightBoundary(beginNegative, max)
template <class T, class Emit>
__host__ __device__ void nodes_right(const T *pos, int n, T max, Emit &&emit) {
    int um = 0;
    const int ux = full_lesser(pos, n, max);
    if (um != ux) {
        emit(full_value(pos, n, um), 0.5 * double(rn_sub(full_value(pos, n, um + 1), full_value(pos, n, um))));
        while (++um != ux)
            emit(full_value(pos, n, um), 0.5 * double(rn_sub(full_value(pos, n, um + 1), full_value(pos, n, um - 1))));
        emit(full_value(pos, n, um), 0.5 * double(rn_sub(max, full_value(pos, n, um - 1))));
        emit(max, 0.5 * double(rn_sub(max, full_value(pos, n, um))));
    } else {
        const double w = double(rn_mul(T(0.5), rn_sub(max, full_value(pos, n, um))));
        emit(max, w);
        emit(full_value(pos, n, um), w);
    }
}

// integrateWithObscureBoundaries(min, max)
template <class T, class Emit>
__host__ __device__ void nodes_both(const T *pos, int n, T min, T max, Emit &&emit) {
    int um = full_greater(pos, n, min);
    const int ux = full_lesser(pos, n, max);
    if (ux >= um) {
        emit(min, 0.5 * double(rn_sub(full_value(pos, n, um), min)));
        if (ux != um) {
            emit(full_value(pos, n, um), 0.5 * double(rn_sub(full_value(pos, n, um + 1), min)));
            while (++um != ux)
                emit(full_value(pos, n, um), 0.5 * double(rn_sub(full_value(pos, n, um + 1), full_value(pos, n, um - 1))));
            emit(full_value(pos, n, um), 0.5 * double(rn_sub(max, full_value(pos, n, um - 1))));
        } else {
            emit(full_value(pos, n, um), 0.5 * double(rn_sub(max, min)));
        }
        emit(max, 0.5 * double(rn_sub(max, full_value(pos, n, um))));
    } else {
        const double w = double(rn_mul(T(0.5), rn_sub(max, min)));
        emit(max, w);
        emit(min, w);
    }
}

}  // namespace dev
}  // namespace spn
