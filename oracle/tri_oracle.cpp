// ORACLE — test infrastructure only.  This file is the CPU checker for the GB300 TRI pf-FRG
// flow right-hand side (time-reversal-invariant models with general, also off-diagonal,
// couplings: Heisenberg-Kitaev-Gamma, ...); nothing in the product links or calls it.  Only
// the tests load it.
//
// It restates, in plain C++ and in the reference's operation order, SpinParser's TRI core:
//   TRIVertexSingleParticle::getValue                 src/TRI/TRIVertexSingleParticle.hpp:73-87
//   TRIVertexTwoParticle::getValue (channel None)     src/TRI/TRIVertexTwoParticle.hpp:190-312
//   getValueLocal / getValueSuperbundle               src/TRI/TRIVertexTwoParticle.hpp:347-391
//   generateAccessBuffer<4>, <8>                      src/TRI/TRIVertexTwoParticle.hpp:401-584
//   _directAccessMapFrequencyExchange, _generateAccessBufferOffsetMapFrequencyExchange, _zeta
//                                                     src/TRI/TRIVertexTwoParticle.hpp:598-677
//   TRIFrgCore::_calculateVertexSingleParticle        src/TRI/TRIFrgCore.cpp:122-151
//   TRIFrgCore::_calculateVertexTwoParticle           src/TRI/TRIFrgCore.cpp:153-3001
//   TRIFrgCore::finalizeStep (Euler)                  src/TRI/TRIFrgCore.cpp:98-120
//   TRIMeasurementCorrelation::_calculateCorrelation  src/TRI/TRIMeasurementCorrelation.cpp:147-285
// and shares the frequency mesh searches and trapezoid rules with the SU(2) and XYZ oracles
// (src/FrequencyDiscretization.hpp:253-356, src/lib/Integrator.hpp:137-287).
//
// The vertex has 16 components (a, b) per site, a and b in {0 = X, 1 = Y, 2 = Z, 3 = density},
// stored as [s,u][t][a][b][site] (component index 4a + b).  The reference spells out the
// products of the flow equations term by term (about 2300 generated lines).  Every one of
// those coefficients is a Pauli-matrix product: with sigma_a sigma_b = i^k sigma_(a.b) and
// mixed spin/density components carrying a factor -i, the particle-particle ladder is
//   d(c) += [sigma_a1 sigma_b1]_(c1) [sigma_a2 sigma_b2]_(c2) -i(a) -i(b) / -i(c)  A(a) B(b),
// the particle-hole ladder the same with the second product reversed and an overall minus,
// the RPA a trace over the inner index, the chalice diagrams a triple product.  This file
// builds those tables from the algebra (tri_tables) and walks them in the reference's order,
// so that every sum rounds as the reference's does.  Built with -ffp-contract=off.
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
// Same member layout as the XYZ oracle's descriptor.
typedef struct {
    int n_freq;                // N positive frequencies
    const float *freq;         // [N] ascending, > 0
    int n_sites;               // Nl representatives
    const int *sites_rid;      // [Nl] getSites()[j].rid
    const int *sites_perm;     // [Nl] getSites()[j].spinPermutation (index)
    const int *inv_sites_rid;  // [Nl] getInvertedSites()[j].rid
    const int *inv_sites_perm; // [Nl]
    const int *overlap_ptr;    // [Nl+1]
    const int *overlap_rid1;   // [sum]
    const int *overlap_rid2;   // [sum]
    const int *overlap_perm1;  // [sum] permutation of the pair (0, j)
    const int *overlap_perm2;  // [sum] permutation of the pair (j, rid)
    int n_range;               // sites in range of the origin
    const int *range_rid;      // [n_range] symmetryTransform(origin, j)
    const int *range_inv_rid;  // [n_range] symmetryTransform(j, origin)
} TriOracleDesc;
}

namespace {

constexpr int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
constexpr int D = 3;
constexpr int kSpinOrder[4] = {3, 2, 1, 0};  // density, Z, Y, X: the reference's order of inner indices

const float kTwoPiProd = 2.0f * float(M_PI);          // 2.0f * (float)M_PI
const float kTwoPiCast = float(2.0f * M_PI);          // float(2.0f * M_PI)
const float kFourPi2Cast = float(4.0f * M_PI * M_PI);  // float(4.0f * M_PI * M_PI)

inline float zeta(int c) { return c <= 2 ? -1.0f : 1.0f; }
inline int permc(int p, int c) { return c == D ? D : kPerm[p][c]; }

// ---- Pauli algebra of the coefficient tables ----
// sigma_a sigma_b = i^k sigma_c, components 0..2 = x, y, z, 3 = identity.
void pauli(int a, int b, int &c, int &k) {
    if (a == D) { c = b; k = 0; return; }
    if (b == D) { c = a; k = 0; return; }
    if (a == b) { c = D; k = 0; return; }
    c = 3 - a - b;
    k = ((b - a + 3) % 3 == 1) ? 1 : 3;  // +i for cyclic (x,y), (y,z), (z,x)
}
// -i (power 3) for a mixed spin/density component
inline int eta(int a, int b) { return ((a == D) != (b == D)) ? 3 : 0; }
// i^k as a real sign; -2 marks an imaginary (never used) coefficient
inline int real_sign(int k) {
    k &= 3;
    return k == 0 ? 1 : (k == 2 ? -1 : -2);
}

struct Pair { signed char a, b, sg; };  // one product A(a) * B(b) with sign sg
struct Tables {
    Pair pp[16][16];      // s channel: per output, a = 15..0
    Pair ph[16][16];      // u channel
    Pair rpa[16][4];      // t channel RPA: inner index in density, Z, Y, X order; a = (mu, k), b = (k, nu) unpermuted
    Pair chal[16][16];    // chalice: a = (mu, kappa), b = local (lambda, rho)
    Pair ichal[16][16];   // inverse chalice: a = local (lambda, rho), b = (kappa, nu)
    Pair egg[16][4];      // measurement egg: a = local component, sg * factor below
    int bad = 0;
};

Tables build_tables() {
    Tables T;
    for (int c = 0; c < 16; ++c) {
        const int c1 = c >> 2, c2 = c & 3;
        for (int n = 0; n < 16; ++n) {
            const int a = 15 - n, b = a ^ c ^ 15;
            const int a1 = a >> 2, a2 = a & 3, b1 = b >> 2, b2 = b & 3;
            int r1, r2, k1, k2;
            pauli(a1, b1, r1, k1);
            pauli(a2, b2, r2, k2);
            if (r1 != c1 || r2 != c2) ++T.bad;
            int s = real_sign(k1 + k2 + eta(a1, a2) + eta(b1, b2) - eta(c1, c2));
            T.pp[c][n] = {(signed char)a, (signed char)b, (signed char)s};
            pauli(b2, a2, r2, k2);
            s = real_sign(2 + k1 + k2 + eta(a1, a2) + eta(b1, b2) - eta(c1, c2));
            T.ph[c][n] = {(signed char)a, (signed char)b, (signed char)s};
        }
        for (int n = 0; n < 4; ++n) {
            const int k = kSpinOrder[n];
            const int s = real_sign(eta(c1, k) + eta(k, c2) - eta(c1, c2));
            T.rpa[c][n] = {(signed char)(4 * c1 + k), (signed char)(4 * k + c2), (signed char)s};
        }
        for (int n = 0; n < 16; ++n) {
            // chalice: kappa outer, lambda inner, both in density, Z, Y, X order
            const int kap = kSpinOrder[n >> 2], lam = kSpinOrder[n & 3];
            const int rho = c2 ^ kap ^ lam;
            int r, k, r3, k3;
            pauli(lam, kap, r, k);
            pauli(r, rho, r3, k3);
            if (r3 != c2) ++T.bad;
            int s = real_sign(2 + k + k3 + eta(c1, kap) + eta(lam, rho) - eta(c1, c2));
            T.chal[c][n] = {(signed char)(4 * c1 + kap), (signed char)(4 * lam + rho), (signed char)s};
            // inverse chalice: local component l = 15..0, kappa from the product
            const int l = 15 - n, lam2 = l >> 2, rho2 = l & 3;
            const int kap2 = c1 ^ lam2 ^ rho2;
            pauli(lam2, kap2, r, k);
            pauli(r, rho2, r3, k3);
            if (r3 != c1) ++T.bad;
            s = real_sign(2 + k + k3 + eta(kap2, c2) + eta(lam2, rho2) - eta(c1, c2));
            T.ichal[c][n] = {(signed char)l, (signed char)(4 * kap2 + c2), (signed char)s};
        }
        for (int n = 0; n < 4; ++n) {
            // egg: tr(sigma_c1 sigma_lam sigma_c2 sigma_rho) / 2 with the -i of a mixed local component
            const int lam = kSpinOrder[n], rho = c1 ^ c2 ^ lam;
            int r, k, r2, k2, r3, k3;
            pauli(c1, lam, r, k);
            pauli(r, c2, r2, k2);
            pauli(r2, rho, r3, k3);
            // imaginary (odd power) only for the mixed outputs, which the measurement skips
            const int s = r3 == D && real_sign(k + k2 + k3 + eta(lam, rho)) != -2 ? real_sign(k + k2 + k3 + eta(lam, rho)) : 0;
            T.egg[c][n] = {(signed char)(4 * lam + rho), 0, (signed char)s};
        }
    }
    for (int c = 0; c < 16; ++c)
        for (int n = 0; n < 16; ++n)
            if (T.pp[c][n].sg == -2 || T.ph[c][n].sg == -2 || T.chal[c][n].sg == -2 || T.ichal[c][n].sg == -2) ++T.bad;
    return T;
}

const Tables &tables() {
    static const Tables T = build_tables();
    return T;
}

struct Mesh {
    int n;
    std::vector<float> full;  // 2N values: -w[N-1] .. -w[0], w[0] .. w[N-1]
    const float *pos;
    explicit Mesh(const TriOracleDesc &d) : n(d.n_freq), full(2 * d.n_freq) {
        for (int i = 0; i < n; ++i) {
            full[n + i] = d.freq[i];
            full[n - 1 - i] = -d.freq[i];
        }
        pos = full.data() + n;
    }
    int lesser(float w) const {
        if (w < 0) return n - (greater(-w) - n + 1);
        if (w <= pos[0]) return n;
        for (int i = 1; i < n; ++i)
            if (pos[i] > w) return n + i - 1;
        return n + n - 1;
    }
    int greater(float w) const {
        if (w < 0) return n - (lesser(-w) - n + 1);
        if (w <= pos[0]) return n;
        for (int i = 1; i < n; ++i)
            if (pos[i] > w) return n + i;
        return n + n - 1;
    }
    int offset(float w) const {
        if (w <= pos[0]) return 0;
        for (int i = 1; i < n; ++i)
            if (pos[i] >= w) return i;
        return n - 1;
    }
    void interpolate(float w, int &lo, int &hi, float &bias) const {
        if (w <= pos[0]) {
            lo = hi = 0;
            bias = 0.0f;
            return;
        }
        for (int i = 1; i < n; ++i)
            if (pos[i] > w) {
                hi = i;
                lo = i - 1;
                bias = (w - pos[lo]) / (pos[hi] - pos[lo]);
                return;
            }
        lo = hi = n - 1;
        bias = 0.0f;
    }
};

// TRIVertexTwoParticleAccessBuffer<K>: the sign table sign[i][a][b] is the product of
// zeta(a) zeta(b) when exactly one of t, u was negated, and, for a support whose s and u
// offsets were exchanged, -zeta(a) (pair exchange) or -zeta(b).
template <int K>
struct AccessBuffer {
    int off[K];
    float wgt[K];
    bool fx[K];
    bool exch = false;
    bool tu = false;
    float sign(int i, int a, int b) const {
        float s = 1.0f;
        if (tu) s *= zeta(a) * zeta(b);
        if (fx[i]) s *= -(exch ? zeta(a) : zeta(b));
        return s;
    }
};

// ValueSuperbundle<float, 16>
struct Bundle16 {
    std::vector<float> c[16];
    explicit Bundle16(int nl = 0) {
        for (auto &v : c) v.assign(nl, 0.0f);
    }
    void reset() {
        for (auto &v : c) std::fill(v.begin(), v.end(), 0.0f);
    }
};

void axpy(Bundle16 &y, float a, const Bundle16 &x) {
    for (int k = 0; k < 16; ++k)
        for (size_t i = 0; i < y.c[k].size(); ++i) y.c[k][i] += a * x.c[k][i];
}
void add(Bundle16 &y, const Bundle16 &x) {
    for (int k = 0; k < 16; ++k)
        for (size_t i = 0; i < y.c[k].size(); ++i) y.c[k][i] += x.c[k][i];
}
void scale(Bundle16 &y, float a) {
    for (auto &v : y.c)
        for (auto &e : v) e *= a;
}

struct Tri {
    const TriOracleDesc &dsc;
    Mesh mesh;
    int N, Nl;
    long long stepT, stepSU;  // 16 Nl per t, N 16 Nl per (s,u)
    const float *v2, *dv2;
    const float *v4;          // [F_N][16][Nl]

    Tri(const TriOracleDesc &d, const float *v2_, const float *dv2_, const float *v4_)
        : dsc(d), mesh(d), N(d.n_freq), Nl(d.n_sites), stepT(16LL * d.n_sites), stepSU(16LL * d.n_sites * d.n_freq),
          v2(v2_), dv2(dv2_), v4(v4_) {}

    float sigma(const float *data, float w) const {
        float sign = 1.0f;
        if (w < 0) {
            w = -w;
            sign = -1.0f;
        }
        int lo, hi;
        float b;
        mesh.interpolate(w, lo, hi, b);
        return sign * ((1 - b) * data[lo] + b * data[hi]);
    }

    template <int K>
    void gen_offset(int s, int t, int u, int i, AccessBuffer<K> &ab) const {
        if (s < u) {
            ab.fx[i] = true;
            ab.off[i] = int(stepSU * (u * (u + 1) / 2 + s) + t * stepT);
        } else {
            ab.fx[i] = false;
            ab.off[i] = int(stepSU * (s * (s + 1) / 2 + u) + t * stepT);
        }
    }

    template <int K>
    static void fold(float &s, float &t, float &u, AccessBuffer<K> &ab) {
        if (s < 0) {
            s = -s;
            ab.exch = !ab.exch;
        }
        if (t < 0) {
            t = -t;
            ab.tu = !ab.tu;
        }
        if (u < 0) {
            u = -u;
            ab.exch = !ab.exch;
            ab.tu = !ab.tu;
        }
    }

    AccessBuffer<4> access4(float s, float t, float u, int channel) const {
        AccessBuffer<4> ab;
        fold(s, t, u, ab);
        int e, la, ua, lb, ub;
        float ba, bb;
        if (channel == 0) {
            e = mesh.offset(s);
            mesh.interpolate(t, la, ua, ba);
            mesh.interpolate(u, lb, ub, bb);
            ab.wgt[0] = (1 - bb) * (1 - ba); gen_offset(e, la, lb, 0, ab);
            ab.wgt[1] = (1 - bb) * ba;       gen_offset(e, ua, lb, 1, ab);
            ab.wgt[2] = bb * (1 - ba);       gen_offset(e, la, ub, 2, ab);
            ab.wgt[3] = bb * ba;             gen_offset(e, ua, ub, 3, ab);
        } else if (channel == 1) {
            e = mesh.offset(t);
            mesh.interpolate(s, la, ua, ba);
            mesh.interpolate(u, lb, ub, bb);
            ab.wgt[0] = (1 - bb) * (1 - ba); gen_offset(la, e, lb, 0, ab);
            ab.wgt[1] = (1 - bb) * ba;       gen_offset(ua, e, lb, 1, ab);
            ab.wgt[2] = bb * (1 - ba);       gen_offset(la, e, ub, 2, ab);
            ab.wgt[3] = bb * ba;             gen_offset(ua, e, ub, 3, ab);
        } else {
            e = mesh.offset(u);
            mesh.interpolate(s, la, ua, ba);
            mesh.interpolate(t, lb, ub, bb);
            ab.wgt[0] = (1 - bb) * (1 - ba); gen_offset(la, lb, e, 0, ab);
            ab.wgt[1] = (1 - bb) * ba;       gen_offset(ua, lb, e, 1, ab);
            ab.wgt[2] = bb * (1 - ba);       gen_offset(la, ub, e, 2, ab);
            ab.wgt[3] = bb * ba;             gen_offset(ua, ub, e, 3, ab);
        }
        return ab;
    }

    AccessBuffer<8> access8(float s, float t, float u) const {
        AccessBuffer<8> ab;
        fold(s, t, u, ab);
        int ls, us, lt, ut, lu, uu;
        float bs, bt, bu;
        mesh.interpolate(s, ls, us, bs);
        mesh.interpolate(t, lt, ut, bt);
        mesh.interpolate(u, lu, uu, bu);
        ab.wgt[0] = (1 - bt) * (1 - bs) * (1 - bu); gen_offset(ls, lt, lu, 0, ab);
        ab.wgt[1] = (1 - bt) * bs * (1 - bu);       gen_offset(us, lt, lu, 1, ab);
        ab.wgt[2] = bt * (1 - bs) * (1 - bu);       gen_offset(ls, ut, lu, 2, ab);
        ab.wgt[3] = bt * bs * (1 - bu);             gen_offset(us, ut, lu, 3, ab);
        ab.wgt[4] = (1 - bt) * (1 - bs) * bu;       gen_offset(ls, lt, uu, 4, ab);
        ab.wgt[5] = (1 - bt) * bs * bu;             gen_offset(us, lt, uu, 5, ab);
        ab.wgt[6] = bt * (1 - bs) * bu;             gen_offset(ls, ut, uu, 6, ab);
        ab.wgt[7] = bt * bs * bu;                   gen_offset(us, ut, uu, 7, ab);
        return ab;
    }

    // getValueSuperbundle: component (a, b) of site j reads the representative's component
    // (a', b') = the (exchanged, then permuted) pair; the sign is indexed by (a, b).
    template <int K>
    void superbundle(const AccessBuffer<K> &ab, Bundle16 &out) const {
        out.reset();
        const int *rid = ab.exch ? dsc.inv_sites_rid : dsc.sites_rid;
        const int *prm = ab.exch ? dsc.inv_sites_perm : dsc.sites_perm;
        for (int i = 0; i < K; ++i)
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) {
                    const float sw = ab.sign(i, a, b) * ab.wgt[i];
                    for (int j = 0; j < Nl; ++j) {
                        const int a1 = permc(prm[j], ab.exch ? b : a);
                        const int b1 = permc(prm[j], ab.exch ? a : b);
                        out.c[4 * a + b][j] += sw * v4[ab.off[i] + (4 * a1 + b1) * Nl + rid[j]];
                    }
                }
    }

    // getValueLocal: the components are exchanged first and the sign is indexed by the
    // exchanged pair.
    template <int K>
    float local(int a, int b, const AccessBuffer<K> &ab) const {
        if (ab.exch) std::swap(a, b);
        float v = 0.0f;
        for (int i = 0; i < K; ++i) v += ab.sign(i, a, b) * ab.wgt[i] * v4[ab.off[i] + (4 * a + b) * Nl];
        return v;
    }

    float direct(int site, int so, int to, int uo, int a, int b) const {
        if (so >= uo) return v4[stepSU * (so * (so + 1) / 2 + uo) + stepT * to + (4 * a + b) * Nl + site];
        return -zeta(b) * v4[stepSU * (uo * (uo + 1) / 2 + so) + stepT * to + (4 * a + b) * Nl + site];
    }

    // getValue(i1, i2, s, t, u, a, b, FrequencyChannel::None) for the pairs the self-energy
    // reads: (origin, j) through rid12 / rid21 with identity spin maps, a == b.
    float value_none(int rid12, int rid21, float s, float t, float u, int a, int b) const {
        float sign = 1.0f;
        bool swapped = false;
        if (s < 0) {
            s = -s;
            std::swap(a, b);
            swapped = !swapped;
        }
        if (t < 0) {
            t = -t;
            sign *= zeta(a) * zeta(b);
        }
        if (u < 0) {
            u = -u;
            std::swap(a, b);
            swapped = !swapped;
            sign *= zeta(a) * zeta(b);
        }
        const int site = swapped ? rid21 : rid12;
        int ls, us, lt, ut, lu, uu;
        float bs, bt, bu;
        mesh.interpolate(s, ls, us, bs);
        mesh.interpolate(t, lt, ut, bt);
        mesh.interpolate(u, lu, uu, bu);
        auto Dv = [&](int x, int y, int z) { return direct(site, x, y, z, a, b); };
        return sign * ((1 - bu) * ((1 - bt) * ((1 - bs) * Dv(ls, lt, lu) + bs * Dv(us, lt, lu)) +
                                   bt * ((1 - bs) * Dv(ls, ut, lu) + bs * Dv(us, ut, lu))) +
                       bu * ((1 - bt) * ((1 - bs) * Dv(ls, lt, uu) + bs * Dv(us, lt, uu)) +
                             bt * ((1 - bs) * Dv(ls, ut, uu) + bs * Dv(us, ut, uu))));
    }

    // ---- trapezoid rules with off-mesh boundaries (Integrator.hpp:137-287) ----
    template <class F>
    void int_left(float min, F &&f, Bundle16 &ib, Bundle16 &res) const {
        res.reset();
        const int maxi = 2 * N - 1;
        int um = mesh.greater(min);
        const float *fl = mesh.full.data();
        if (um != maxi) {
            f(min, ib); axpy(res, fl[um] - min, ib);
            f(fl[um], ib); axpy(res, fl[um + 1] - min, ib);
            while (++um != maxi) {
                f(fl[um], ib);
                axpy(res, fl[um + 1] - fl[um - 1], ib);
            }
            f(fl[um], ib); axpy(res, fl[um] - fl[um - 1], ib);
            scale(res, 0.5f);
        } else {
            f(min, ib); add(res, ib);
            f(fl[um], ib); add(res, ib);
            scale(res, 0.5f * (fl[um] - min));
        }
    }
    template <class F>
    void int_right(float max, F &&f, Bundle16 &ib, Bundle16 &res) const {
        res.reset();
        const float *fl = mesh.full.data();
        int um = 0;
        int ux = mesh.lesser(max);
        if (um != ux) {
            f(fl[um], ib); axpy(res, fl[um + 1] - fl[um], ib);
            while (++um != ux) {
                f(fl[um], ib);
                axpy(res, fl[um + 1] - fl[um - 1], ib);
            }
            f(fl[um], ib); axpy(res, max - fl[um - 1], ib);
            f(max, ib); axpy(res, max - fl[um], ib);
            scale(res, 0.5f);
        } else {
            f(max, ib); add(res, ib);
            f(fl[um], ib); add(res, ib);
            scale(res, 0.5f * (max - fl[um]));
        }
    }
    template <class F>
    void int_both(float min, float max, F &&f, Bundle16 &ib, Bundle16 &res) const {
        res.reset();
        const float *fl = mesh.full.data();
        int um = mesh.greater(min);
        int ux = mesh.lesser(max);
        if (ux >= um) {
            f(min, ib); axpy(res, fl[um] - min, ib);
            if (ux != um) {
                f(fl[um], ib); axpy(res, fl[um + 1] - min, ib);
                while (++um != ux) {
                    f(fl[um], ib);
                    axpy(res, fl[um + 1] - fl[um - 1], ib);
                }
                f(fl[um], ib); axpy(res, max - fl[um - 1], ib);
            } else {
                f(fl[um], ib); axpy(res, max - min, ib);
            }
            f(max, ib); axpy(res, max - fl[um], ib);
            scale(res, 0.5f);
        } else {
            f(max, ib); add(res, ib);
            f(min, ib); add(res, ib);
            scale(res, 0.5f * (max - min));
        }
    }

    // ---- self-energy flow, one frequency (TRIFrgCore.cpp:122-151) ----
    float self_energy_flow(int i, float cutoff) const {
        const float w = mesh.pos[i];
        float val = 0.0f;
        float sum = 0.0f;
        for (int j = 0; j < dsc.n_range; ++j) {
            sum += value_none(dsc.range_rid[j], dsc.range_inv_rid[j], w + cutoff, 0.0f, w - cutoff, D, D);
            sum -= value_none(dsc.range_rid[j], dsc.range_inv_rid[j], w - cutoff, 0.0f, w + cutoff, D, D);
        }
        val -= 2.0f * sum;
        for (int c : {0, 1, 2, D})
            val += value_none(0, 0, w + cutoff, w - cutoff, 0.0f, c, c) - value_none(0, 0, w - cutoff, w + cutoff, 0.0f, c, c);
        val /= (kTwoPiProd * (cutoff + sigma(v2, cutoff)));
        return val;
    }

    // ---- two-particle vertex flow, one frequency triple (TRIFrgCore.cpp:153-3001) ----
    struct Scratch {
        Bundle16 b1, b2, rpa, acc, st[4];
        explicit Scratch(int nl) : b1(nl), b2(nl), rpa(nl), acc(nl), st{Bundle16(nl), Bundle16(nl), Bundle16(nl), Bundle16(nl)} {}
    };

    // the two ladders: per output, a = 15..0 with the pairs (0,1) then (2,3) (TRIFrgCore.cpp:198-711, 2389-2902)
    void ladder(const Pair (&tab)[16][16], const Bundle16 *sb, Bundle16 &r) const {
        r.reset();
        for (int c = 0; c < 16; ++c)
            for (int n = 0; n < 16; ++n) {
                const Pair &q = tab[c][n];
                for (int p = 0; p < 4; p += 2)
                    for (int j = 0; j < Nl; ++j) {
                        if (q.sg > 0) r.c[c][j] += sb[p].c[q.a][j] * sb[p + 1].c[q.b][j];
                        else r.c[c][j] -= sb[p].c[q.a][j] * sb[p + 1].c[q.b][j];
                    }
            }
    }

    void vertex_flow(int it, float cutoff, Scratch &sc, float *out) const {
        const Tables &T = tables();
        const int su = it / N;
        const float t = mesh.pos[it % N];
        float s = 0.0f, u = 0.0f;
        for (int so = 0; so <= su; ++so)
            for (int uo = 0; uo <= so; ++uo)
                if (su == so * (so + 1) / 2 + uo) {
                    s = mesh.pos[so];
                    u = mesh.pos[uo];
                }
        const float w1p = 0.5f * (s + t + u);
        const float w1 = 0.5f * (s - t + u);
        const float w2p = 0.5f * (s - t - u);
        const float w2 = 0.5f * (s + t - u);
        Bundle16 *sb = sc.st;

        auto kernelS = [&](float wp, Bundle16 &r) {  // TRIFrgCore.cpp:181-712
            superbundle(access4(s, w2 + wp, w1 + wp, 0), sb[0]);
            superbundle(access4(s, -w2p - wp, w1p + wp, 0), sb[1]);
            superbundle(access4(s, -w1 - wp, -w2 - wp, 0), sb[2]);
            superbundle(access4(s, w1p + wp, -w2p - wp, 0), sb[3]);
            ladder(T.pp, sb, r);
        };

        auto kernelT = [&](float wp, Bundle16 &r) {  // TRIFrgCore.cpp:714-2369
            superbundle(access4(w1 - wp, t, w1p + wp, 1), sb[0]);
            superbundle(access4(w2p - wp, t, -w2 - wp, 1), sb[1]);
            superbundle(access4(w1p + wp, t, w1 - wp, 1), sb[2]);
            superbundle(access4(w2 + wp, t, -w2p + wp, 1), sb[3]);
            r.reset();
            sc.rpa.reset();
            for (int rid = 0; rid < Nl; ++rid) {
                const int i0 = dsc.overlap_ptr[rid], i1 = dsc.overlap_ptr[rid + 1];
                for (int c = 0; c < 16; ++c) {
                    const int mu = c >> 2, nu = c & 3;
                    for (int n = 0; n < 4; ++n) {
                        const int k = kSpinOrder[n];
                        const int sg = T.rpa[c][n].sg;
                        for (int p = 0; p < 4; p += 2)
                            for (int i = i0; i < i1; ++i) {
                                const int P1 = dsc.overlap_perm1[i], P2 = dsc.overlap_perm2[i];
                                const float x = sb[p].c[4 * permc(P1, mu) + permc(P1, k)][dsc.overlap_rid1[i]];
                                const float y = sb[p + 1].c[4 * permc(P2, k) + permc(P2, nu)][dsc.overlap_rid2[i]];
                                if (sg > 0) sc.rpa.c[c][rid] += 2 * x * y;
                                else sc.rpa.c[c][rid] -= 2 * x * y;
                            }
                    }
                }
            }
            add(r, sc.rpa);
            const AccessBuffer<4> a4 = access4(w2p - wp, -w2 - wp, t, 2);
            const AccessBuffer<4> a5 = access4(w2 + wp, -w2p + wp, t, 2);
            float L4[16], L5[16];
            for (int l = 0; l < 16; ++l) {
                L4[l] = local(l >> 2, l & 3, a4);
                L5[l] = local(l >> 2, l & 3, a5);
            }
            for (int c = 0; c < 16; ++c)
                for (int n = 0; n < 16; ++n) {
                    const Pair &q = T.chal[c][n];
                    for (int j = 0; j < Nl; ++j) {
                        if (q.sg > 0) {
                            r.c[c][j] += sb[0].c[q.a][j] * L4[q.b];
                            r.c[c][j] += sb[2].c[q.a][j] * L5[q.b];
                        } else {
                            r.c[c][j] -= sb[0].c[q.a][j] * L4[q.b];
                            r.c[c][j] -= sb[2].c[q.a][j] * L5[q.b];
                        }
                    }
                }
            const AccessBuffer<4> a6 = access4(w1 - wp, -w1p - wp, -t, 2);
            const AccessBuffer<4> a7 = access4(w1p + wp, -w1 + wp, -t, 2);
            float L6[16], L7[16];
            for (int l = 0; l < 16; ++l) {
                L6[l] = local(l >> 2, l & 3, a6);
                L7[l] = local(l >> 2, l & 3, a7);
            }
            for (int c = 0; c < 16; ++c)
                for (int n = 0; n < 16; ++n) {
                    const Pair &q = T.ichal[c][n];
                    for (int j = 0; j < Nl; ++j) {
                        if (q.sg > 0) {
                            r.c[c][j] += L6[q.a] * sb[1].c[q.b][j];
                            r.c[c][j] += L7[q.a] * sb[3].c[q.b][j];
                        } else {
                            r.c[c][j] -= L6[q.a] * sb[1].c[q.b][j];
                            r.c[c][j] -= L7[q.a] * sb[3].c[q.b][j];
                        }
                    }
                }
        };

        auto kernelU = [&](float wp, Bundle16 &r) {  // TRIFrgCore.cpp:2371-2903
            superbundle(access4(w1 + wp, -w2p + wp, u, 2), sb[0]);
            superbundle(access4(w1p + wp, w2 - wp, u, 2), sb[1]);
            superbundle(access4(w2p - wp, -w1 - wp, u, 2), sb[2]);
            superbundle(access4(w2 - wp, w1p + wp, u, 2), sb[3]);
            ladder(T.ph, sb, r);
        };

        auto p = [&](float a, float b) { return 1.0f / ((a + sigma(v2, a)) * (b + sigma(v2, b))); };
        auto pK = [&](float a, float b) {
            const float den = a + sigma(v2, a);
            return sigma(dv2, a) / (den * den * (b + sigma(v2, b)));
        };

        Bundle16 &acc = sc.acc;
        acc.reset();
        kernelS(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + s), sc.b1);
        if (s > 2.0f * cutoff) { kernelS(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - s), sc.b1); }
        kernelT(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + t), sc.b1);
        if (t > 2.0f * cutoff) { kernelT(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - t), sc.b1); }
        kernelU(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + u), sc.b1);
        if (u > 2.0f * cutoff) { kernelU(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - u), sc.b1); }

        auto kS = [&](float wp, Bundle16 &r) { kernelS(wp, r); scale(r, pK(wp, s + wp)); };
        auto kT = [&](float wp, Bundle16 &r) { kernelT(wp, r); scale(r, pK(wp, t + wp)); };
        auto kU = [&](float wp, Bundle16 &r) { kernelU(wp, r); scale(r, pK(wp, u + wp)); };
        const float wmax = mesh.pos[N - 1];
        const float wneg = mesh.full[0];
        auto katanin = [&](float x, auto &kern) {
            if (-(x + cutoff) > wneg) { int_right(-(x + cutoff), kern, sc.b1, sc.b2); add(acc, sc.b2); }
            if (x - cutoff > cutoff) { int_both(cutoff - x, -cutoff, kern, sc.b1, sc.b2); add(acc, sc.b2); }
            if (cutoff < wmax) { int_left(cutoff, kern, sc.b1, sc.b2); add(acc, sc.b2); }
        };
        katanin(s, kS);
        katanin(t, kT);
        katanin(u, kU);

        for (int c = 0; c < 16; ++c)
            for (int j = 0; j < Nl; ++j) out[c * Nl + j] = acc.c[c][j] / kTwoPiProd;
    }

    // ---- static susceptibility at nu = 0 (TRIMeasurementCorrelation.cpp:147-285) ----
    void correlation(float cut, float *chi) const {
        const Tables &T = tables();
        const float nu = 0.0f;
        Bundle16 sus(Nl), stk(Nl), b1(Nl), b2(Nl), b3(Nl), b4(Nl);
        const float wmax = mesh.pos[N - 1];
        const float wneg = mesh.full[0];
        static const int kOut[10] = {15, 0, 1, 2, 4, 5, 6, 8, 9, 10};
        auto outer = [&](float w, Bundle16 &ret) {
            ret.reset();
            const float term1 = 1.0f / ((w + sigma(v2, w)) * (w + nu + sigma(v2, w + nu)));
            ret.c[15][0] += 2.0f * term1 / kTwoPiCast;
            ret.c[0][0] += 0.5f * term1 / kTwoPiCast;
            ret.c[5][0] += 0.5f * term1 / kTwoPiCast;
            ret.c[10][0] += 0.5f * term1 / kTwoPiCast;
            auto inner = [&](float wp, Bundle16 &r) {
                r.reset();
                superbundle(access8(w + wp + nu, nu, w - wp), stk);
                const AccessBuffer<8> ab1 = access8(w + wp + nu, w - wp, nu);
                float L[16];
                for (int l = 0; l < 16; ++l) L[l] = local(l >> 2, l & 3, ab1);
                // dumbbell
                for (int j = 0; j < Nl; ++j) r.c[15][j] -= 4.0f * stk.c[15][j];
                for (int q = 1; q < 10; ++q)
                    for (int j = 0; j < Nl; ++j) r.c[kOut[q]][j] -= 1.0f * stk.c[kOut[q]][j];
                // egg
                for (int q = 0; q < 10; ++q) {
                    const int c = kOut[q];
                    const float f = c == 15 ? 2.0f : 0.5f;
                    for (int n = 0; n < 4; ++n) {
                        const Pair &e = T.egg[c][n];
                        if (e.sg > 0) r.c[c][0] += f * L[e.a];
                        else if (e.sg < 0) r.c[c][0] -= f * L[e.a];
                    }
                }
                const float norm = 1.0f / ((w + sigma(v2, w)) * (w + nu + sigma(v2, w + nu)) * (wp + sigma(v2, wp)) *
                                           (wp + nu + sigma(v2, wp + nu)) * kFourPi2Cast);
                scale(r, norm);
            };
            if (-(nu + cut) > wneg) { int_right(-cut - nu, inner, b3, b4); add(ret, b4); }
            if (nu - cut > cut) { int_both(-nu + cut, -cut, inner, b3, b4); add(ret, b4); }
            if (cut < wmax) { int_left(cut, inner, b3, b4); add(ret, b4); }
        };
        if (-(nu + cut) > wneg) { int_right(-cut - nu, outer, b1, b2); add(sus, b2); }
        if (nu - cut > cut) { int_both(-nu + cut, -cut, outer, b1, b2); add(sus, b2); }
        if (cut < wmax) { int_left(cut, outer, b1, b2); add(sus, b2); }
        for (int c = 0; c < 16; ++c)
            for (int j = 0; j < Nl; ++j) chi[c * Nl + j] = sus.c[c][j];
    }
};

}  // namespace

extern "C" {

// The coefficient tables as (table, output, n, a, b, sign) rows, for inspection by the tests.
// Tables: 0 = s ladder, 1 = u ladder, 2 = RPA, 3 = chalice, 4 = inverse chalice, 5 = egg.
// Returns the number of rows (1152), or -1 if the algebra gave an imaginary
// coefficient or an inconsistent product.
int oracle_tri_tables(int *rows) {
    const Tables &T = tables();
    if (T.bad) return -1;
    int n = 0;
    auto put = [&](int tab, int c, int k, const Pair &p) {
        int *r = rows + 6 * n++;
        r[0] = tab; r[1] = c; r[2] = k; r[3] = p.a; r[4] = p.b; r[5] = p.sg;
    };
    for (int c = 0; c < 16; ++c) {
        for (int k = 0; k < 16; ++k) put(0, c, k, T.pp[c][k]);
        for (int k = 0; k < 16; ++k) put(1, c, k, T.ph[c][k]);
        for (int k = 0; k < 4; ++k) put(2, c, k, T.rpa[c][k]);
        for (int k = 0; k < 16; ++k) put(3, c, k, T.chal[c][k]);
        for (int k = 0; k < 16; ++k) put(4, c, k, T.ichal[c][k]);
        for (int k = 0; k < 4; ++k) put(5, c, k, T.egg[c][k]);
    }
    return n;
}

// One flow right-hand side: self-energy flow dv2[N], then the vertex flow dv4[F_N*16*Nl].
int oracle_tri_rhs_f32(const TriOracleDesc *d, float cutoff, const float *v2, const float *v4, float *dv2, float *dv4,
                       int nthreads) {
    if (!d || d->n_freq < 2 || d->n_sites < 1) return -2;
    if (tables().bad) return -3;
    const int N = d->n_freq, Nl = d->n_sites;
    const int FN = N * N * (N + 1) / 2;
    {
        Tri core(*d, v2, nullptr, v4);
        for (int i = 0; i < N; ++i) dv2[i] = core.self_energy_flow(i, cutoff);
    }
    Tri core(*d, v2, dv2, v4);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        Tri::Scratch sc(Nl);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 8)
#endif
        for (int it = 0; it < FN; ++it) core.vertex_flow(it, cutoff, sc, dv4 + (long long)it * 16 * Nl);
    }
    return 0;
}

// Static susceptibility chi[16][Nl] at the given cutoff (the mixed components stay zero).
int oracle_tri_correlation_f32(const TriOracleDesc *d, float cutoff, const float *v2, const float *v4, float *chi) {
    if (!d) return -2;
    if (tables().bad) return -3;
    Tri core(*d, v2, nullptr, v4);
    core.correlation(cutoff, chi);
    return 0;
}

// Complete flow over a cutoff list: measurement at every cutoff before the Euler step, stop
// at a NaN.  chi receives n_cutoffs * 16 * Nl values; returns the number of measurements.
int oracle_tri_flow_f32(const TriOracleDesc *d, const float *cutoffs, int n_cutoffs, float *v2, float *v4, float *chi,
                        int nthreads) {
    if (!d || n_cutoffs < 2) return -2;
    if (tables().bad) return -3;
    const int N = d->n_freq, Nl = d->n_sites;
    const long long size = (long long)N * N * (N + 1) / 2 * 16 * Nl;
    std::vector<float> dv2(N), dv4(size);
    int k = 0;
    float cutoff = cutoffs[0];
    for (; k < n_cutoffs - 1; ++k) {
        oracle_tri_rhs_f32(d, cutoff, v2, v4, dv2.data(), dv4.data(), nthreads);
        oracle_tri_correlation_f32(d, cutoff, v2, v4, chi + (long long)k * 16 * Nl);
        bool nan = false;
        for (int i = 0; i < N && !nan; ++i) nan = std::isnan(dv2[i]);
        for (long long i = 0; i < size && !nan; ++i) nan = std::isnan(dv4[i]);
        if (nan) break;
        const float next = cutoffs[k + 1];
        const float step = next - cutoff;  // TRIFrgCore.cpp:98-120
        for (int i = 0; i < N; ++i) v2[i] += step * dv2[i];
        for (long long i = 0; i < size; ++i) v4[i] += step * dv4[i];
        cutoff = next;
    }
    oracle_tri_correlation_f32(d, cutoff, v2, v4, chi + (long long)k * 16 * Nl);
    return k + 1;
}

}  // extern "C"
