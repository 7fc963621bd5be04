// ORACLE — test infrastructure only.  This file is the CPU checker for the GB300 XYZ pf-FRG
// flow right-hand side (models with diagonal, possibly anisotropic couplings: Kitaev,
// XXZ, ...); nothing in the product links or calls it.  Only the tests load it.
//
// It restates, in plain C++ and in the reference's operation order, SpinParser's XYZ core:
//   XYZVertexSingleParticle::getValue            src/XYZ/XYZVertexSingleParticle.hpp:73-87
//   XYZVertexTwoParticle::getValue (None)        src/XYZ/XYZVertexTwoParticle.hpp:185-305
//   getValueLocal / getValueSuperbundle          src/XYZ/XYZVertexTwoParticle.hpp:355-410
//   generateAccessBuffer<4>, <8>                 src/XYZ/XYZVertexTwoParticle.hpp:419-580
//   _directAccessMapFrequencyExchange            src/XYZ/XYZVertexTwoParticle.hpp:589-612
//   XYZFrgCore::_calculateVertexSingleParticle   src/XYZ/XYZFrgCore.cpp:161-194
//   XYZFrgCore::_calculateVertexTwoParticle      src/XYZ/XYZFrgCore.cpp:196-570
//   XYZFrgCore::finalizeStep (Euler)             src/XYZ/XYZFrgCore.cpp:128-159
//   XYZMeasurementCorrelation::_calculateCorrelation  src/XYZ/XYZMeasurementCorrelation.cpp:98-184
//   XYZEffectiveAction initial condition         src/XYZ/XYZEffectiveAction.hpp:38-60
// and shares the frequency mesh searches and trapezoid rules with the SU(2) oracle
// (src/FrequencyDiscretization.hpp:253-356, src/lib/Integrator.hpp:137-287).
//
// Spin components are indexed 0 = X, 1 = Y, 2 = Z, 3 = density ("None").  A lattice
// symmetry map may permute X, Y, Z: permutation p sends component c of a site pair to
// component kPerm[p][c] of its representative (LatticeSiteDescriptor::spinPermutation).
// Built with -ffp-contract=off so that no fused multiply-add changes a rounding.
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
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
} XyzOracleDesc;
}

namespace {

constexpr int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
constexpr int X = 0, Y = 1, Z = 2, D = 3;

const float kPiF = float(M_PI);
const float kTwoPiProd = 2.0f * float(M_PI);          // 2.0f * (float)M_PI
const float kFourPiCast = float(4.0f * M_PI);         // float(4.0f * M_PI)
const float kFourPi2Cast = float(4.0f * M_PI * M_PI);  // float(4.0f * M_PI * M_PI)

struct Mesh {
    int n;
    std::vector<float> full;  // 2N values: -w[N-1] .. -w[0], w[0] .. w[N-1]
    const float *pos;
    explicit Mesh(const XyzOracleDesc &d) : n(d.n_freq), full(2 * d.n_freq) {
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

template <int K>
struct AccessBuffer {
    int off[K];
    float wgt[K];
    int sgn[K];
    bool exch = false;
};

// ValueSuperbundle<float, 4>: four length-Nl bundles X, Y, Z, D.
struct Bundle4 {
    std::vector<float> c[4];
    explicit Bundle4(int nl = 0) {
        for (auto &v : c) v.assign(nl, 0.0f);
    }
    void reset() {
        for (auto &v : c) std::fill(v.begin(), v.end(), 0.0f);
    }
};

void axpy(Bundle4 &y, float a, const Bundle4 &x) {
    for (int k = 0; k < 4; ++k)
        for (size_t i = 0; i < y.c[k].size(); ++i) y.c[k][i] += a * x.c[k][i];
}
void add(Bundle4 &y, const Bundle4 &x) {
    for (int k = 0; k < 4; ++k)
        for (size_t i = 0; i < y.c[k].size(); ++i) y.c[k][i] += x.c[k][i];
}
void scale(Bundle4 &y, float a) {
    for (auto &v : y.c)
        for (auto &e : v) e *= a;
}

struct Xyz {
    const XyzOracleDesc &dsc;
    Mesh mesh;
    int N, Nl;
    long long stepLat, stepLatT;
    const float *v2, *dv2;
    const float *base[4];  // xx, yy, zz, dd [F_N * Nl]

    Xyz(const XyzOracleDesc &d, const float *v2_, const float *dv2_, const float *xx, const float *yy, const float *zz,
        const float *dd)
        : dsc(d), mesh(d), N(d.n_freq), Nl(d.n_sites), stepLat(d.n_sites), stepLatT((long long)d.n_sites * d.n_freq),
          v2(v2_), dv2(dv2_) {
        base[X] = xx;
        base[Y] = yy;
        base[Z] = zz;
        base[D] = dd;
    }

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

    int gen_offset(int s, int t, int u, int &sign) const {
        if (s < u) {
            sign = -1;
            return int(stepLatT * (u * (u + 1) / 2 + s) + t * stepLat);
        }
        sign = 1;
        return int(stepLatT * (s * (s + 1) / 2 + u) + t * stepLat);
    }

    static void fold(float &s, float &t, float &u, bool &exch) {
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
    }

    AccessBuffer<4> access4(float s, float t, float u, int channel) const {
        AccessBuffer<4> ab;
        fold(s, t, u, ab.exch);
        int e, la, ua, lb, ub;
        float ba, bb;
        if (channel == 0) {
            e = mesh.offset(s);
            mesh.interpolate(t, la, ua, ba);
            mesh.interpolate(u, lb, ub, bb);
            ab.wgt[0] = (1 - bb) * (1 - ba); ab.off[0] = gen_offset(e, la, lb, ab.sgn[0]);
            ab.wgt[1] = (1 - bb) * ba;       ab.off[1] = gen_offset(e, ua, lb, ab.sgn[1]);
            ab.wgt[2] = bb * (1 - ba);       ab.off[2] = gen_offset(e, la, ub, ab.sgn[2]);
            ab.wgt[3] = bb * ba;             ab.off[3] = gen_offset(e, ua, ub, ab.sgn[3]);
        } else if (channel == 1) {
            e = mesh.offset(t);
            mesh.interpolate(s, la, ua, ba);
            mesh.interpolate(u, lb, ub, bb);
            ab.wgt[0] = (1 - bb) * (1 - ba); ab.off[0] = gen_offset(la, e, lb, ab.sgn[0]);
            ab.wgt[1] = (1 - bb) * ba;       ab.off[1] = gen_offset(ua, e, lb, ab.sgn[1]);
            ab.wgt[2] = bb * (1 - ba);       ab.off[2] = gen_offset(la, e, ub, ab.sgn[2]);
            ab.wgt[3] = bb * ba;             ab.off[3] = gen_offset(ua, e, ub, ab.sgn[3]);
        } else {
            e = mesh.offset(u);
            mesh.interpolate(s, la, ua, ba);
            mesh.interpolate(t, lb, ub, bb);
            ab.wgt[0] = (1 - bb) * (1 - ba); ab.off[0] = gen_offset(la, lb, e, ab.sgn[0]);
            ab.wgt[1] = (1 - bb) * ba;       ab.off[1] = gen_offset(ua, lb, e, ab.sgn[1]);
            ab.wgt[2] = bb * (1 - ba);       ab.off[2] = gen_offset(la, ub, e, ab.sgn[2]);
            ab.wgt[3] = bb * ba;             ab.off[3] = gen_offset(ua, ub, e, ab.sgn[3]);
        }
        return ab;
    }

    AccessBuffer<8> access8(float s, float t, float u) const {
        AccessBuffer<8> ab;
        fold(s, t, u, ab.exch);
        int ls, us, lt, ut, lu, uu;
        float bs, bt, bu;
        mesh.interpolate(s, ls, us, bs);
        mesh.interpolate(t, lt, ut, bt);
        mesh.interpolate(u, lu, uu, bu);
        ab.wgt[0] = (1 - bt) * (1 - bs) * (1 - bu); ab.off[0] = gen_offset(ls, lt, lu, ab.sgn[0]);
        ab.wgt[1] = (1 - bt) * bs * (1 - bu);       ab.off[1] = gen_offset(us, lt, lu, ab.sgn[1]);
        ab.wgt[2] = bt * (1 - bs) * (1 - bu);       ab.off[2] = gen_offset(ls, ut, lu, ab.sgn[2]);
        ab.wgt[3] = bt * bs * (1 - bu);             ab.off[3] = gen_offset(us, ut, lu, ab.sgn[3]);
        ab.wgt[4] = (1 - bt) * (1 - bs) * bu;       ab.off[4] = gen_offset(ls, lt, uu, ab.sgn[4]);
        ab.wgt[5] = (1 - bt) * bs * bu;             ab.off[5] = gen_offset(us, lt, uu, ab.sgn[5]);
        ab.wgt[6] = bt * (1 - bs) * bu;             ab.off[6] = gen_offset(ls, ut, uu, ab.sgn[6]);
        ab.wgt[7] = bt * bs * bu;                   ab.off[7] = gen_offset(us, ut, uu, ab.sgn[7]);
        return ab;
    }

    // getValueSuperbundle: X, Y, Z of site j read the representative's permuted components.
    template <int K>
    void superbundle(const AccessBuffer<K> &ab, Bundle4 &out) const {
        out.reset();
        const int *rid = ab.exch ? dsc.inv_sites_rid : dsc.sites_rid;
        const int *prm = ab.exch ? dsc.inv_sites_perm : dsc.sites_perm;
        for (int i = 0; i < K; ++i) {
            const float w = ab.wgt[i];
            const float sw = float(ab.sgn[i]) * ab.wgt[i];
            const int o = ab.off[i];
            for (int j = 0; j < Nl; ++j) {
                const int *P = kPerm[prm[j]];
                out.c[X][j] += w * base[P[0]][o + rid[j]];
                out.c[Y][j] += w * base[P[1]][o + rid[j]];
                out.c[Z][j] += w * base[P[2]][o + rid[j]];
                out.c[D][j] += sw * base[D][o + rid[j]];
            }
        }
    }

    template <int K>
    float local(int comp, const AccessBuffer<K> &ab) const {
        float v = 0.0f;
        if (comp != D)
            for (int i = 0; i < K; ++i) v += ab.wgt[i] * base[comp][ab.off[i]];
        else
            for (int i = 0; i < K; ++i) v += float(ab.sgn[i]) * ab.wgt[i] * base[D][ab.off[i]];
        return v;
    }

    float direct(int site, int so, int to, int uo, int comp) const {
        if (so >= uo) return base[comp][stepLatT * (so * (so + 1) / 2 + uo) + stepLat * to + site];
        const float x = base[comp][stepLatT * (uo * (uo + 1) / 2 + so) + stepLat * to + site];
        return comp != D ? x : -x;
    }

    // getValue(i1, i2, s, t, u, comp, FrequencyChannel::None): the pair enters through its rid
    // and spin permutation (rid12/perm12 for (i1,i2), rid21/perm21 for the swapped pair).
    float value_none(int rid12, int perm12, int rid21, int perm21, float s, float t, float u, int comp) const {
        bool swapped = false;
        fold(s, t, u, swapped);
        const int site = swapped ? rid21 : rid12;
        if (comp != D) comp = kPerm[swapped ? perm21 : perm12][comp];
        int ls, us, lt, ut, lu, uu;
        float bs, bt, bu;
        mesh.interpolate(s, ls, us, bs);
        mesh.interpolate(t, lt, ut, bt);
        mesh.interpolate(u, lu, uu, bu);
        auto Dv = [&](int a, int b, int c) { return direct(site, a, b, c, comp); };
        return (1 - bu) * ((1 - bt) * ((1 - bs) * Dv(ls, lt, lu) + bs * Dv(us, lt, lu)) +
                           bt * ((1 - bs) * Dv(ls, ut, lu) + bs * Dv(us, ut, lu))) +
               bu * ((1 - bt) * ((1 - bs) * Dv(ls, lt, uu) + bs * Dv(us, lt, uu)) +
                     bt * ((1 - bs) * Dv(ls, ut, uu) + bs * Dv(us, ut, uu)));
    }

    // ---- trapezoid rules with off-mesh boundaries (Integrator.hpp:137-287) ----
    template <class F>
    void int_left(float min, F &&f, Bundle4 &ib, Bundle4 &res) const {
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
    void int_right(float max, F &&f, Bundle4 &ib, Bundle4 &res) const {
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
    void int_both(float min, float max, F &&f, Bundle4 &ib, Bundle4 &res) const {
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

    // ---- self-energy flow, one frequency (XYZFrgCore.cpp:161-194) ----
    float self_energy_flow(int i, float cutoff) const {
        const float w = mesh.pos[i];
        float val = 0.0f;
        float sum = 0.0f;
        for (int j = 0; j < dsc.n_range; ++j) {
            sum += value_none(dsc.range_rid[j], 0, dsc.range_inv_rid[j], 0, w + cutoff, 0.0f, w - cutoff, D);
            sum -= value_none(dsc.range_rid[j], 0, dsc.range_inv_rid[j], 0, w - cutoff, 0.0f, w + cutoff, D);
        }
        val -= 2.0f * sum;
        for (int c : {X, Y, Z, D})
            val += value_none(0, 0, 0, 0, w + cutoff, w - cutoff, 0.0f, c) - value_none(0, 0, 0, 0, w - cutoff, w + cutoff, 0.0f, c);
        val /= (kTwoPiProd * (cutoff + sigma(v2, cutoff)));
        return val;
    }

    // ---- two-particle vertex flow, one frequency triple (XYZFrgCore.cpp:196-570) ----
    struct Scratch {
        Bundle4 b1, b2, rpa, acc, st[4];
        explicit Scratch(int nl) : b1(nl), b2(nl), rpa(nl), acc(nl), st{Bundle4(nl), Bundle4(nl), Bundle4(nl), Bundle4(nl)} {}
    };

    void vertex_flow(int it, float cutoff, Scratch &sc, float *const out[4]) const {
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
        Bundle4 *sb = sc.st;
        auto el = [&](int b, int c, int j) { return sb[b].c[c][j]; };

        auto kernelS = [&](float wp, Bundle4 &r) {  // XYZFrgCore.cpp:215-262
            superbundle(access4(s, -w1 - wp, -w2 - wp, 0), sb[0]);
            superbundle(access4(s, w1p + wp, -w2p - wp, 0), sb[1]);
            superbundle(access4(s, w2 + wp, w1 + wp, 0), sb[2]);
            superbundle(access4(s, -w2p - wp, w1p + wp, 0), sb[3]);
            r.reset();
            for (int p = 0; p < 4; p += 2)  // the pairs (0,1) then (2,3)
                for (int j = 0; j < Nl; ++j) {
                    float &x = r.c[X][j];
                    x += el(p, D, j) * el(p + 1, X, j);
                    x += el(p, X, j) * el(p + 1, D, j);
                    x -= el(p, Z, j) * el(p + 1, Y, j);
                    x -= el(p, Y, j) * el(p + 1, Z, j);
                }
            for (int p = 0; p < 4; p += 2)
                for (int j = 0; j < Nl; ++j) {
                    float &y = r.c[Y][j];
                    y += el(p, D, j) * el(p + 1, Y, j);
                    y += el(p, Y, j) * el(p + 1, D, j);
                    y -= el(p, Z, j) * el(p + 1, X, j);
                    y -= el(p, X, j) * el(p + 1, Z, j);
                }
            for (int p = 0; p < 4; p += 2)
                for (int j = 0; j < Nl; ++j) {
                    float &z = r.c[Z][j];
                    z += el(p, D, j) * el(p + 1, Z, j);
                    z += el(p, Z, j) * el(p + 1, D, j);
                    z -= el(p, X, j) * el(p + 1, Y, j);
                    z -= el(p, Y, j) * el(p + 1, X, j);
                }
            for (int p = 0; p < 4; p += 2)
                for (int j = 0; j < Nl; ++j) {
                    float &d = r.c[D][j];
                    d += el(p, D, j) * el(p + 1, D, j);
                    d += el(p, X, j) * el(p + 1, X, j);
                    d += el(p, Y, j) * el(p + 1, Y, j);
                    d += el(p, Z, j) * el(p + 1, Z, j);
                }
        };

        auto kernelT = [&](float wp, Bundle4 &r) {  // XYZFrgCore.cpp:264-418
            superbundle(access4(w1 - wp, t, w1p + wp, 1), sb[0]);
            superbundle(access4(w2p - wp, t, -w2 - wp, 1), sb[1]);
            superbundle(access4(w1p + wp, t, w1 - wp, 1), sb[2]);
            superbundle(access4(w2 + wp, t, wp - w2p, 1), sb[3]);
            r.reset();
            sc.rpa.reset();
            for (int rid = 0; rid < Nl; ++rid) {
                const int i0 = dsc.overlap_ptr[rid], i1 = dsc.overlap_ptr[rid + 1];
                for (int c = 0; c < 3; ++c)
                    for (int i = i0; i < i1; ++i)
                        sc.rpa.c[c][rid] += sb[0].c[kPerm[dsc.overlap_perm1[i]][c]][dsc.overlap_rid1[i]] *
                                            sb[1].c[kPerm[dsc.overlap_perm2[i]][c]][dsc.overlap_rid2[i]];
                for (int i = i0; i < i1; ++i)
                    sc.rpa.c[D][rid] += sb[0].c[D][dsc.overlap_rid1[i]] * sb[1].c[D][dsc.overlap_rid2[i]];
            }
            axpy(r, 4.0f, sc.rpa);
            const AccessBuffer<4> a4 = access4(w2p - wp, -w2 - wp, t, 2);
            const AccessBuffer<4> a5 = access4(w1 - wp, -w1p - wp, -t, 2);
            const AccessBuffer<4> a6 = access4(w2 + wp, wp - w2p, t, 2);
            const AccessBuffer<4> a7 = access4(w1p + wp, wp - w1, -t, 2);
            float cb[4], ica[4], cb2[4], ica2[4];
            for (int c = 0; c < 4; ++c) {
                cb[c] = local(c, a4);
                ica[c] = local(c, a5);
                cb2[c] = local(c, a6);
                ica2[c] = local(c, a7);
            }
            // per component c the local values: minus the same component and the density,
            // plus the other two (density: minus all four), for each of the four slabs
            for (int c = 0; c < 3; ++c) {
                // the two other components, in the reference's order of the "plus" terms:
                // with the chalice values (slabs 0, 2) and with the inverse ones (slabs 1, 3)
                const int pA = c == X ? Y : X, pB = c == Z ? Y : Z;
                const int qA = c == Z ? X : Z, qB = c == X ? Y : (c == Y ? X : Y);
                for (int j = 0; j < Nl; ++j) {
                    float &v = r.c[c][j];
                    const float a0 = el(0, c, j), a1 = el(1, c, j), a2 = el(2, c, j), a3 = el(3, c, j);
                    v -= a0 * cb[D];
                    v += a0 * cb[pA];
                    v += a0 * cb[pB];
                    v -= a0 * cb[c];
                    v -= ica[D] * a1;
                    v += ica[qA] * a1;
                    v += ica[qB] * a1;
                    v -= ica[c] * a1;
                    v -= a2 * cb2[D];
                    v += a2 * cb2[pA];
                    v += a2 * cb2[pB];
                    v -= a2 * cb2[c];
                    v -= ica2[D] * a3;
                    v += ica2[qA] * a3;
                    v += ica2[qB] * a3;
                    v -= ica2[c] * a3;
                }
            }
            for (int j = 0; j < Nl; ++j) {
                float &v = r.c[D][j];
                const float a0 = el(0, D, j), a1 = el(1, D, j), a2 = el(2, D, j), a3 = el(3, D, j);
                v -= a0 * cb[D];
                v -= a0 * cb[X];
                v -= a0 * cb[Y];
                v -= a0 * cb[Z];
                v -= ica[D] * a1;
                v -= ica[X] * a1;
                v -= ica[Y] * a1;
                v -= ica[Z] * a1;
                v -= a2 * cb2[D];
                v -= a2 * cb2[X];
                v -= a2 * cb2[Y];
                v -= a2 * cb2[Z];
                v -= ica2[D] * a3;
                v -= ica2[X] * a3;
                v -= ica2[Y] * a3;
                v -= ica2[Z] * a3;
            }
        };

        auto kernelU = [&](float wp, Bundle4 &r) {  // XYZFrgCore.cpp:420-470
            superbundle(access4(w1 + wp, wp - w2p, u, 2), sb[0]);
            superbundle(access4(w1p + wp, w2 - wp, u, 2), sb[1]);
            superbundle(access4(w2p - wp, -w1 - wp, u, 2), sb[2]);
            superbundle(access4(w2 - wp, w1p + wp, u, 2), sb[3]);
            r.reset();
            const int A[4][4][2] = {
                {{D, X}, {X, D}, {Z, Y}, {Y, Z}},  // X
                {{D, Y}, {Y, D}, {Z, X}, {X, Z}},  // Y
                {{D, Z}, {Z, D}, {X, Y}, {Y, X}},  // Z
                {{D, D}, {X, X}, {Y, Y}, {Z, Z}},  // D
            };
            for (int c = 0; c < 4; ++c)
                for (int p = 0; p < 4; p += 2)
                    for (int j = 0; j < Nl; ++j)
                        for (int q = 0; q < 4; ++q) r.c[c][j] -= el(p, A[c][q][0], j) * el(p + 1, A[c][q][1], j);
        };

        auto p = [&](float a, float b) { return 1.0f / ((a + sigma(v2, a)) * (b + sigma(v2, b))); };
        auto pK = [&](float a, float b) {
            const float den = a + sigma(v2, a);
            return sigma(dv2, a) / (den * den * (b + sigma(v2, b)));
        };

        Bundle4 &acc = sc.acc;
        acc.reset();
        kernelS(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + s), sc.b1);
        if (s > 2.0f * cutoff) { kernelS(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - s), sc.b1); }
        kernelT(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + t), sc.b1);
        if (t > 2.0f * cutoff) { kernelT(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - t), sc.b1); }
        kernelU(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + u), sc.b1);
        if (u > 2.0f * cutoff) { kernelU(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - u), sc.b1); }

        auto kS = [&](float wp, Bundle4 &r) { kernelS(wp, r); scale(r, pK(wp, s + wp)); };
        auto kT = [&](float wp, Bundle4 &r) { kernelT(wp, r); scale(r, pK(wp, t + wp)); };
        auto kU = [&](float wp, Bundle4 &r) { kernelU(wp, r); scale(r, pK(wp, u + wp)); };
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

        for (int c = 0; c < 4; ++c)
            for (int j = 0; j < Nl; ++j) out[c][j] = acc.c[c][j] / kTwoPiProd;
    }

    // ---- static susceptibility at nu = 0 (XYZMeasurementCorrelation.cpp:98-163) ----
    void correlation(float cut, float *const chi[4]) const {
        const float nu = 0.0f;
        Bundle4 sus(Nl), stk(Nl), b1(Nl), b2(Nl), b3(Nl), b4(Nl);
        const float wmax = mesh.pos[N - 1];
        const float wneg = mesh.full[0];
        auto outer = [&](float w, Bundle4 &ret) {
            ret.reset();
            const float term1 = 1.0f / ((w + sigma(v2, w)) * (w + nu + sigma(v2, w + nu)));
            ret.c[X][0] += term1 / kFourPiCast;
            ret.c[Y][0] += term1 / kFourPiCast;
            ret.c[Z][0] += term1 / kFourPiCast;
            ret.c[D][0] += term1 / kPiF;
            auto inner = [&](float wp, Bundle4 &r) {
                r.reset();
                superbundle(access8(w + wp + nu, nu, w - wp), stk);
                const float vx = value_none(0, 0, 0, 0, w + wp + nu, w - wp, nu, X);
                const float vy = value_none(0, 0, 0, 0, w + wp + nu, w - wp, nu, Y);
                const float vz = value_none(0, 0, 0, 0, w + wp + nu, w - wp, nu, Z);
                const float vd = value_none(0, 0, 0, 0, w + wp + nu, w - wp, nu, D);
                for (int c = 0; c < 3; ++c)
                    for (int j = 0; j < Nl; ++j) r.c[c][j] -= 1.0f * stk.c[c][j];
                for (int j = 0; j < Nl; ++j) r.c[D][j] -= 4.0f * stk.c[D][j];
                r.c[X][0] += 0.5f * (vx - vy - vz + vd);
                r.c[Y][0] += 0.5f * (-vx + vy - vz + vd);
                r.c[Z][0] += 0.5f * (-vx - vy + vz + vd);
                r.c[D][0] += 2.0f * (vx + vy + vz + vd);
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
        for (int c = 0; c < 4; ++c)
            for (int j = 0; j < Nl; ++j) chi[c][j] = sus.c[c][j];
    }
};

}  // namespace

extern "C" {

// One flow right-hand side: self-energy flow dv2[N], then the vertex flow of the four
// components dv4[c][F_N*Nl] (c = X, Y, Z, density).
int oracle_xyz_rhs_f32(const XyzOracleDesc *d, float cutoff, const float *v2, const float *const *v4, float *dv2,
                       float *const *dv4, int nthreads) {
    if (!d || d->n_freq < 2 || d->n_sites < 1) return -2;
    const int N = d->n_freq, Nl = d->n_sites;
    const int FN = N * N * (N + 1) / 2;
    {
        Xyz core(*d, v2, nullptr, v4[0], v4[1], v4[2], v4[3]);
        for (int i = 0; i < N; ++i) dv2[i] = core.self_energy_flow(i, cutoff);
    }
    Xyz core(*d, v2, dv2, v4[0], v4[1], v4[2], v4[3]);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        Xyz::Scratch sc(Nl);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int it = 0; it < FN; ++it) {
            float *out[4];
            for (int c = 0; c < 4; ++c) out[c] = dv4[c] + (long long)it * Nl;
            core.vertex_flow(it, cutoff, sc, out);
        }
    }
    return 0;
}

// Static susceptibility chi[c][Nl] per component at the given cutoff.
int oracle_xyz_correlation_f32(const XyzOracleDesc *d, float cutoff, const float *v2, const float *const *v4,
                               float *const *chi) {
    if (!d) return -2;
    Xyz core(*d, v2, nullptr, v4[0], v4[1], v4[2], v4[3]);
    core.correlation(cutoff, chi);
    return 0;
}

// Complete flow over a cutoff list, as the SU(2) oracle's flow: measurement at every cutoff
// before the Euler step, stop at a NaN.  chi[c] receives n_cutoffs * Nl values; returns the
// number of measurements.
int oracle_xyz_flow_f32(const XyzOracleDesc *d, const float *cutoffs, int n_cutoffs, float *v2, float *const *v4,
                        float *const *chi, int nthreads) {
    if (!d || n_cutoffs < 2) return -2;
    const int N = d->n_freq, Nl = d->n_sites;
    const long long size = (long long)N * N * (N + 1) / 2 * Nl;
    std::vector<float> dv2(N), dstore(4 * size);
    float *dv4[4] = {dstore.data(), dstore.data() + size, dstore.data() + 2 * size, dstore.data() + 3 * size};
    int k = 0;
    float cutoff = cutoffs[0];
    auto measure = [&](int idx) {
        float *c[4];
        for (int q = 0; q < 4; ++q) c[q] = chi[q] + (long long)idx * Nl;
        oracle_xyz_correlation_f32(d, cutoff, v2, v4, c);
    };
    for (; k < n_cutoffs - 1; ++k) {
        oracle_xyz_rhs_f32(d, cutoff, v2, v4, dv2.data(), dv4, nthreads);
        measure(k);
        bool nan = false;
        for (int i = 0; i < N && !nan; ++i) nan = std::isnan(dv2[i]);
        for (long long i = 0; i < 4 * size && !nan; ++i) nan = std::isnan(dstore[i]);
        if (nan) break;
        const float next = cutoffs[k + 1];
        const float step = next - cutoff;  // XYZFrgCore.cpp:128-159
        for (int i = 0; i < N; ++i) v2[i] += step * dv2[i];
        for (int q : {3, 0, 1, 2})
            for (long long i = 0; i < size; ++i) v4[q][i] += step * dv4[q][i];
        cutoff = next;
    }
    measure(k);
    return k + 1;
}

}  // extern "C"
