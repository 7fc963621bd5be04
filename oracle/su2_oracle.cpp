// ORACLE — test infrastructure only.  This file is the CPU checker for the GB300 SU(2)
// pf-FRG flow right-hand side; nothing in the product links or calls it.  Only the tests,
// the smoke check and the CPU-baseline leg of bench.py load it.
//
// It restates, in plain C++, the arithmetic of SpinParser's SU(2) core so that a CUDA
// result can be compared element by element with what the reference computes:
//   FrequencyDiscretization::{offset, interpolateOffset, lesser, greater}
//                                          src/FrequencyDiscretization.hpp:253-356
//   SU2VertexSingleParticle::getValue      src/SU2/SU2VertexSingleParticle.hpp:73-87
//   SU2VertexTwoParticle::getValue (None)  src/SU2/SU2VertexTwoParticle.hpp:185-297
//   generateAccessBuffer<4>, <8>           src/SU2/SU2VertexTwoParticle.hpp:399-557
//   getValueLocal / getValueSuperbundle    src/SU2/SU2VertexTwoParticle.hpp:347-387
//   _generateAccessBufferOffset            src/SU2/SU2VertexTwoParticle.hpp:616-632
//   ImplicitIntegrator::*                  src/lib/Integrator.hpp:137-287
//   SU2FrgCore::_calculateVertexSingleParticle   src/SU2/SU2FrgCore.cpp:139-169
//   SU2FrgCore::_calculateVertexTwoParticle      src/SU2/SU2FrgCore.cpp:171-431
//   SU2FrgCore::finalizeStep (Euler)             src/SU2/SU2FrgCore.cpp:111-137
//   SU2MeasurementCorrelation::_calculateCorrelation  src/SU2/SU2MeasurementCorrelation.cpp:77-177
//   SU2EffectiveAction initial condition         src/SU2/SU2EffectiveAction.hpp:38-60
//
// Instantiated for float (operation order of the reference; build with
// -ffp-contract=off so no fused multiply-add changes a rounding) and for double (the
// FP64 oracle used for precision studies).  Lattice tables come in through OracleDesc.
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
typedef struct {
    int n_freq;                  // N positive frequencies
    const float *freq;           // [N] ascending, > 0
    int n_sites;                 // Nl representatives
    const int *sites_rid;        // [Nl] getSites()[j].rid
    const int *inv_sites_rid;    // [Nl] getInvertedSites()[j].rid
    const int *overlap_ptr;      // [Nl+1]
    const int *overlap_rid1;     // [sum]
    const int *overlap_rid2;     // [sum]
    int n_range;                 // sites in range of the origin
    const int *range_rid;        // [n_range] symmetryTransform(origin, j)
    const int *range_inv_rid;    // [n_range] symmetryTransform(j, origin)
    float spin_length;           // S
} OracleDesc;
}

namespace {

// The reference mixes float(M_PI), float(2*M_PI) and float(4*M_PI*M_PI) literals; the
// float instantiation reproduces those roundings, the double one uses exact pi.
template <class R> struct Pi;
template <> struct Pi<float> {
    static float pi() { return float(M_PI); }
    static float two_pi_cast() { return float(2.0f * M_PI); }
    static float four_pi2_cast() { return float(4.0f * M_PI * M_PI); }
    static float two_pi_prod() { return 2.0f * float(M_PI); }
};
template <> struct Pi<double> {
    static double pi() { return M_PI; }
    static double two_pi_cast() { return 2.0 * M_PI; }
    static double four_pi2_cast() { return 4.0 * M_PI * M_PI; }
    static double two_pi_prod() { return 2.0 * M_PI; }
};

template <class R>
struct Mesh {
    int n;
    std::vector<R> full;  // 2N values: -w[N-1] .. -w[0], w[0] .. w[N-1]
    const R *pos;         // &full[N]
    explicit Mesh(const OracleDesc &d) : n(d.n_freq), full(2 * d.n_freq) {
        for (int i = 0; i < n; ++i) {
            full[n + i] = R(d.freq[i]);
            full[n - 1 - i] = -R(d.freq[i]);
        }
        pos = full.data() + n;
    }
    // Indices below are into `full` (0 = most negative point, N = smallest positive point).
    int lesser(R w) const {
        if (w < 0) return n - (greater(-w) - n + 1);
        if (w <= pos[0]) return n;
        for (int i = 1; i < n; ++i)
            if (pos[i] > w) return n + i - 1;
        return n + n - 1;
    }
    int greater(R w) const {
        if (w < 0) return n - (lesser(-w) - n + 1);
        if (w <= pos[0]) return n;
        for (int i = 1; i < n; ++i)
            if (pos[i] > w) return n + i;
        return n + n - 1;
    }
    int offset(R w) const {
        if (w <= pos[0]) return 0;
        for (int i = 1; i < n; ++i)
            if (pos[i] >= w) return i;
        return n - 1;
    }
    void interpolate(R w, int &lo, int &hi, R &bias) const {
        if (w <= pos[0]) {
            lo = hi = 0;
            bias = R(0);
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
        bias = R(0);
    }
};

template <class R, int K>
struct AccessBuffer {
    int off[K];
    R wgt[K];
    int sgn[K];
    bool exch = false;
};

// Length-Nl pair of site bundles (spin, density): ValueSuperbundle<float,2>.
template <class R>
struct Bundle2 {
    std::vector<R> s, d;
    explicit Bundle2(int nl = 0) : s(nl, R(0)), d(nl, R(0)) {}
    void reset() {
        std::fill(s.begin(), s.end(), R(0));
        std::fill(d.begin(), d.end(), R(0));
    }
};

template <class R>
struct Su2 {
    const OracleDesc &dsc;
    Mesh<R> mesh;
    int N, Nl;
    long long stepLat, stepLatT;
    const R *v2;    // self-energy state [N]
    const R *dv2;   // self-energy flow  [N]
    const R *ss;    // vertex spin     [F_N * Nl]
    const R *dd;    // vertex density  [F_N * Nl]
    R spin;

    Su2(const OracleDesc &d, const R *v2_, const R *dv2_, const R *ss_, const R *dd_)
        : dsc(d), mesh(d), N(d.n_freq), Nl(d.n_sites), stepLat(d.n_sites), stepLatT((long long)d.n_sites * d.n_freq),
          v2(v2_), dv2(dv2_), ss(ss_), dd(dd_), spin(R(d.spin_length)) {}

    R sigma(const R *data, R w) const {
        R sign = R(1);
        if (w < 0) {
            w = -w;
            sign = R(-1);
        }
        int lo, hi;
        R b;
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

    static void fold(R &s, R &t, R &u, bool &exch) {
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

    // channel: 0 = S, 1 = T, 2 = U (one frequency lies exactly on the mesh)
    AccessBuffer<R, 4> access4(R s, R t, R u, int channel) const {
        AccessBuffer<R, 4> ab;
        fold(s, t, u, ab.exch);
        int e, la, ua, lb, ub;
        R ba, bb;
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

    AccessBuffer<R, 8> access8(R s, R t, R u) const {
        AccessBuffer<R, 8> ab;
        fold(s, t, u, ab.exch);
        int ls, us, lt, ut, lu, uu;
        R bs, bt, bu;
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

    template <int K>
    void superbundle(const AccessBuffer<R, K> &ab, Bundle2<R> &out) const {
        out.reset();
        const int *sites = ab.exch ? dsc.inv_sites_rid : dsc.sites_rid;
        for (int i = 0; i < K; ++i) {
            R w = ab.wgt[i];
            R sw = R(ab.sgn[i]) * ab.wgt[i];
            int o = ab.off[i];
            for (int j = 0; j < Nl; ++j) {
                out.s[j] += w * ss[o + sites[j]];
                out.d[j] += sw * dd[o + sites[j]];
            }
        }
    }

    template <int K>
    R local(bool spin_channel, const AccessBuffer<R, K> &ab) const {
        R v = R(0);
        if (spin_channel)
            for (int i = 0; i < K; ++i) v += ab.wgt[i] * ss[ab.off[i]];
        else
            for (int i = 0; i < K; ++i) v += R(ab.sgn[i]) * ab.wgt[i] * dd[ab.off[i]];
        return v;
    }

    R direct(int site, int so, int to, int uo, bool spin_channel) const {
        if (so >= uo) {
            long long idx = stepLatT * (so * (so + 1) / 2 + uo) + stepLat * to + site;
            return spin_channel ? ss[idx] : dd[idx];
        }
        long long idx = stepLatT * (uo * (uo + 1) / 2 + so) + stepLat * to + site;
        return spin_channel ? ss[idx] : -dd[idx];
    }

    // getValue(i1, i2, s, t, u, symmetry, FrequencyChannel::None); the site pair enters
    // only through its rid (`rid12` for (i1,i2), `rid21` for the swapped pair).
    R value_none(int rid12, int rid21, R s, R t, R u, bool spin_channel) const {
        bool swapped = false;
        fold(s, t, u, swapped);
        int site = swapped ? rid21 : rid12;
        int ls, us, lt, ut, lu, uu;
        R bs, bt, bu;
        mesh.interpolate(s, ls, us, bs);
        mesh.interpolate(t, lt, ut, bt);
        mesh.interpolate(u, lu, uu, bu);
        auto D = [&](int a, int b, int c) { return direct(site, a, b, c, spin_channel); };
        return (1 - bu) * ((1 - bt) * ((1 - bs) * D(ls, lt, lu) + bs * D(us, lt, lu)) +
                           bt * ((1 - bs) * D(ls, ut, lu) + bs * D(us, ut, lu))) +
               bu * ((1 - bt) * ((1 - bs) * D(ls, lt, uu) + bs * D(us, lt, uu)) +
                     bt * ((1 - bs) * D(ls, ut, uu) + bs * D(us, ut, uu)));
    }

    // ---- trapezoid rules on the mesh with off-mesh boundaries ----
    // f(wp, buffer) fills buffer; result receives the integral.
    template <class F>
    void int_left(R min, F &&f, Bundle2<R> &ib, Bundle2<R> &res) const {
        res.reset();
        const int maxi = 2 * N - 1;
        int um = mesh.greater(min);
        const R *fl = mesh.full.data();
        if (um != maxi) {
            f(min, ib); axpy(res, fl[um] - min, ib);
            f(fl[um], ib); axpy(res, fl[um + 1] - min, ib);
            while (++um != maxi) {
                f(fl[um], ib);
                axpy(res, fl[um + 1] - fl[um - 1], ib);
            }
            f(fl[um], ib); axpy(res, fl[um] - fl[um - 1], ib);
            scale(res, R(0.5));
        } else {
            f(min, ib); add(res, ib);
            f(fl[um], ib); add(res, ib);
            scale(res, R(0.5) * (fl[um] - min));
        }
    }

    template <class F>
    void int_right(R max, F &&f, Bundle2<R> &ib, Bundle2<R> &res) const {
        res.reset();
        const R *fl = mesh.full.data();
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
            scale(res, R(0.5));
        } else {
            f(max, ib); add(res, ib);
            f(fl[um], ib); add(res, ib);
            scale(res, R(0.5) * (max - fl[um]));
        }
    }

    template <class F>
    void int_both(R min, R max, F &&f, Bundle2<R> &ib, Bundle2<R> &res) const {
        res.reset();
        const R *fl = mesh.full.data();
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
            scale(res, R(0.5));
        } else {
            f(max, ib); add(res, ib);
            f(min, ib); add(res, ib);
            scale(res, R(0.5) * (max - min));
        }
    }

    static void axpy(Bundle2<R> &y, R a, const Bundle2<R> &x) {
        for (size_t i = 0; i < y.s.size(); ++i) y.s[i] += a * x.s[i];
        for (size_t i = 0; i < y.d.size(); ++i) y.d[i] += a * x.d[i];
    }
    static void add(Bundle2<R> &y, const Bundle2<R> &x) {
        for (size_t i = 0; i < y.s.size(); ++i) y.s[i] += x.s[i];
        for (size_t i = 0; i < y.d.size(); ++i) y.d[i] += x.d[i];
    }
    static void scale(Bundle2<R> &y, R a) {
        for (auto &v : y.s) v *= a;
        for (auto &v : y.d) v *= a;
    }

    // ---- self-energy flow, one frequency (SU2FrgCore.cpp:139-169) ----
    R self_energy_flow(int i, R cutoff) const {
        R w = mesh.pos[i];
        R val = R(0);
        R sum = R(0);
        for (int j = 0; j < dsc.n_range; ++j) {
            sum += value_none(dsc.range_rid[j], dsc.range_inv_rid[j], w + cutoff, R(0), w - cutoff, false);
            sum -= value_none(dsc.range_rid[j], dsc.range_inv_rid[j], w - cutoff, R(0), w + cutoff, false);
        }
        val -= R(4) * spin * sum;
        val += R(0.75) * (value_none(0, 0, w + cutoff, w - cutoff, R(0), true) - value_none(0, 0, w - cutoff, w + cutoff, R(0), true));
        val += (value_none(0, 0, w + cutoff, w - cutoff, R(0), false) - value_none(0, 0, w - cutoff, w + cutoff, R(0), false));
        val /= (Pi<R>::two_pi_prod() * (cutoff + sigma(v2, cutoff)));
        return val;
    }

    // ---- two-particle vertex flow, one frequency triple (SU2FrgCore.cpp:171-431) ----
    struct Scratch {
        Bundle2<R> b1, b2, rpa, acc, st[4];
        explicit Scratch(int nl) : b1(nl), b2(nl), rpa(nl), acc(nl), st{Bundle2<R>(nl), Bundle2<R>(nl), Bundle2<R>(nl), Bundle2<R>(nl)} {}
    };

    void vertex_flow(int it, R cutoff, Scratch &sc, R *out_s, R *out_d) const {
        int su = it / N;
        R t = mesh.pos[it % N], s = R(0), u = R(0);
        for (int so = 0; so <= su; ++so)
            for (int uo = 0; uo <= so; ++uo)
                if (su == so * (so + 1) / 2 + uo) {
                    s = mesh.pos[so];
                    u = mesh.pos[uo];
                }
        const R w1p = R(0.5) * (s + t + u);
        const R w1 = R(0.5) * (s - t + u);
        const R w2p = R(0.5) * (s - t - u);
        const R w2 = R(0.5) * (s + t - u);
        Bundle2<R> *stb = sc.st;

        auto kernelS = [&](R wp, Bundle2<R> &r) {
            superbundle(access4(s, -w1 - wp, -w2 - wp, 0), stb[0]);
            superbundle(access4(s, w1p + wp, -w2p - wp, 0), stb[1]);
            superbundle(access4(s, w2 + wp, w1 + wp, 0), stb[2]);
            superbundle(access4(s, -w2p - wp, w1p + wp, 0), stb[3]);
            r.reset();
            for (int j = 0; j < Nl; ++j) {
                R S0 = stb[0].s[j], S1 = stb[1].s[j], S2 = stb[2].s[j], S3 = stb[3].s[j];
                R D0 = stb[0].d[j], D1 = stb[1].d[j], D2 = stb[2].d[j], D3 = stb[3].d[j];
                R &rs = r.s[j], &rd = r.d[j];
                rs -= R(0.5) * S0 * S1;
                rs -= R(0.5) * S2 * S3;
                rs += D0 * S1;
                rs += D2 * S3;
                rs += S0 * D1;
                rs += S2 * D3;
                rd += R(3.0f / 16.0f) * S0 * S1;
                rd += R(3.0f / 16.0f) * S2 * S3;
                rd += D0 * D1;
                rd += D2 * D3;
            }
        };
        auto kernelT = [&](R wp, Bundle2<R> &r) {
            superbundle(access4(w1 - wp, t, w1p + wp, 1), stb[0]);
            superbundle(access4(w2p - wp, t, -w2 - wp, 1), stb[1]);
            superbundle(access4(w1p + wp, t, w1 - wp, 1), stb[2]);
            superbundle(access4(w2 + wp, t, wp - w2p, 1), stb[3]);
            r.reset();
            sc.rpa.reset();
            for (int rid = 0; rid < Nl; ++rid) {
                for (int i = dsc.overlap_ptr[rid]; i < dsc.overlap_ptr[rid + 1]; ++i)
                    sc.rpa.s[rid] += stb[2].s[dsc.overlap_rid1[i]] * stb[3].s[dsc.overlap_rid2[i]];
                for (int i = dsc.overlap_ptr[rid]; i < dsc.overlap_ptr[rid + 1]; ++i)
                    sc.rpa.d[rid] += stb[2].d[dsc.overlap_rid1[i]] * stb[3].d[dsc.overlap_rid2[i]];
            }
            for (int j = 0; j < Nl; ++j) r.s[j] += R(2) * spin * sc.rpa.s[j];
            for (int j = 0; j < Nl; ++j) r.d[j] += R(8) * spin * sc.rpa.d[j];
            AccessBuffer<R, 4> a4 = access4(w2p - wp, -w2 - wp, t, 2);
            AccessBuffer<R, 4> a5 = access4(w1 - wp, -w1p - wp, -t, 2);
            AccessBuffer<R, 4> a6 = access4(w2 + wp, wp - w2p, t, 2);
            AccessBuffer<R, 4> a7 = access4(w1p + wp, wp - w1, -t, 2);
            const R cbs = local(true, a4), cbd = local(false, a4);
            const R icas = local(true, a5), icad = local(false, a5);
            const R cbs2 = local(true, a6), cbd2 = local(false, a6);
            const R icas2 = local(true, a7), icad2 = local(false, a7);
            for (int j = 0; j < Nl; ++j) {
                R &rs = r.s[j];
                rs -= cbd * stb[0].s[j];
                rs += (R(0.25) * cbs) * stb[0].s[j];
                rs -= icad * stb[1].s[j];
                rs += (R(0.25) * icas) * stb[1].s[j];
                rs -= cbd2 * stb[2].s[j];
                rs += (R(0.25) * cbs2) * stb[2].s[j];
                rs -= icad2 * stb[3].s[j];
                rs += (R(0.25) * icas2) * stb[3].s[j];
            }
            for (int j = 0; j < Nl; ++j) {
                R &rd = r.d[j];
                rd -= cbd * stb[0].d[j];
                rd -= (R(0.75) * cbs) * stb[0].d[j];
                rd -= icad * stb[1].d[j];
                rd -= (R(0.75) * icas) * stb[1].d[j];
                rd -= cbd2 * stb[2].d[j];
                rd -= (R(0.75) * cbs2) * stb[2].d[j];
                rd -= icad2 * stb[3].d[j];
                rd -= (R(0.75) * icas2) * stb[3].d[j];
            }
        };
        auto kernelU = [&](R wp, Bundle2<R> &r) {
            superbundle(access4(w1 + wp, wp - w2p, u, 2), stb[0]);
            superbundle(access4(w1p + wp, w2 - wp, u, 2), stb[1]);
            superbundle(access4(w2p - wp, -w1 - wp, u, 2), stb[2]);
            superbundle(access4(w2 - wp, w1p + wp, u, 2), stb[3]);
            r.reset();
            for (int j = 0; j < Nl; ++j) {
                R S0 = stb[0].s[j], S1 = stb[1].s[j], S2 = stb[2].s[j], S3 = stb[3].s[j];
                R D0 = stb[0].d[j], D1 = stb[1].d[j], D2 = stb[2].d[j], D3 = stb[3].d[j];
                R &rs = r.s[j], &rd = r.d[j];
                rs += R(0.5) * S0 * S1;
                rs += R(0.5) * S2 * S3;
                rs += S0 * D1;
                rs += S2 * D3;
                rs += D0 * S1;
                rs += D2 * S3;
                rd += R(3.0f / 16.0f) * S0 * S1;
                rd += R(3.0f / 16.0f) * S2 * S3;
                rd += D0 * D1;
                rd += D2 * D3;
            }
        };
        auto p = [&](R a, R b) { return R(1) / ((a + sigma(v2, a)) * (b + sigma(v2, b))); };
        auto pK = [&](R a, R b) {
            R den = a + sigma(v2, a);
            return sigma(dv2, a) / (den * den * (b + sigma(v2, b)));
        };

        Bundle2<R> &acc = sc.acc;
        acc.reset();
        kernelS(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + s), sc.b1);
        if (s > R(2) * cutoff) { kernelS(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - s), sc.b1); }
        kernelT(cutoff, sc.b1); axpy(acc, p(cutoff, cutoff + t), sc.b1);
        if (t > R(2) * cutoff) { kernelT(-cutoff, sc.b1); axpy(acc, p(cutoff, cutoff - t), sc.b1); }
        kernelU(cutoff, sc.b1); axpy(acc, -p(cutoff, cutoff + u), sc.b1);
        if (u > R(2) * cutoff) { kernelU(-cutoff, sc.b1); axpy(acc, -p(cutoff, cutoff - u), sc.b1); }

        auto kS = [&](R wp, Bundle2<R> &r) { kernelS(wp, r); scale(r, pK(wp, s + wp)); };
        auto kT = [&](R wp, Bundle2<R> &r) { kernelT(wp, r); scale(r, pK(wp, t + wp)); };
        auto kU = [&](R wp, Bundle2<R> &r) { kernelU(wp, r); scale(r, -pK(wp, u + wp)); };
        const R wmax = mesh.pos[N - 1];
        const R wneg = mesh.full[0];
        auto katanin = [&](R x, auto &kern) {
            if (-(x + cutoff) > wneg) { int_right(-(x + cutoff), kern, sc.b1, sc.b2); add(acc, sc.b2); }
            if (x - cutoff > cutoff) { int_both(cutoff - x, -cutoff, kern, sc.b1, sc.b2); add(acc, sc.b2); }
            if (cutoff < wmax) { int_left(cutoff, kern, sc.b1, sc.b2); add(acc, sc.b2); }
        };
        katanin(s, kS);
        katanin(t, kT);
        katanin(u, kU);

        const R twopi = Pi<R>::two_pi_prod();
        for (int j = 0; j < Nl; ++j) {
            out_s[j] = acc.s[j] / twopi;
            out_d[j] = acc.d[j] / twopi;
        }
    }

    // ---- static susceptibility at nu = 0 (SU2MeasurementCorrelation.cpp:77-177) ----
    void correlation(R cut, R *chi_s, R *chi_d) const {
        const R nu = R(0);
        Bundle2<R> sus(Nl), stk(Nl), b1(Nl), b2(Nl), b3(Nl), b4(Nl);
        const R wmax = mesh.pos[N - 1];
        const R wneg = mesh.full[0];
        auto outer = [&](R w, Bundle2<R> &ret) {
            ret.reset();
            R term1 = R(1) / ((w + sigma(v2, w)) * (w + nu + sigma(v2, w + nu)));
            ret.s[0] += spin * term1 / Pi<R>::two_pi_cast();
            ret.d[0] += R(2) * spin * term1 / Pi<R>::pi();
            auto inner = [&](R wp, Bundle2<R> &r) {
                r.reset();
                superbundle(access8(w + wp + nu, nu, w - wp), stk);
                R vs = value_none(0, 0, w + wp + nu, w - wp, nu, true);
                R vd = value_none(0, 0, w + wp + nu, w - wp, nu, false);
                for (int j = 0; j < Nl; ++j) r.s[j] -= spin * spin * stk.s[j];
                for (int j = 0; j < Nl; ++j) r.d[j] -= R(16) * spin * spin * stk.d[j];
                r.s[0] += spin * (-vs / R(4) + vd);
                r.d[0] += spin * (R(3) * vs + R(4) * vd);
                R norm = R(1) / ((w + sigma(v2, w)) * (w + nu + sigma(v2, w + nu)) * (wp + sigma(v2, wp)) *
                                 (wp + nu + sigma(v2, wp + nu)) * Pi<R>::four_pi2_cast());
                scale(r, norm);
            };
            if (-(nu + cut) > wneg) { int_right(-cut - nu, inner, b3, b4); add(ret, b4); }
            if (nu - cut > cut) { int_both(-nu + cut, -cut, inner, b3, b4); add(ret, b4); }
            if (cut < wmax) { int_left(cut, inner, b3, b4); add(ret, b4); }
        };
        if (-(nu + cut) > wneg) { int_right(-cut - nu, outer, b1, b2); add(sus, b2); }
        if (nu - cut > cut) { int_both(-nu + cut, -cut, outer, b1, b2); add(sus, b2); }
        if (cut < wmax) { int_left(cut, outer, b1, b2); add(sus, b2); }
        for (int j = 0; j < Nl; ++j) {
            chi_s[j] = sus.s[j];
            chi_d[j] = sus.d[j];
        }
    }
};

template <class R>
int rhs_impl(const OracleDesc *d, R cutoff, const R *v2, const R *ss, const R *dd, R *dv2, R *dss, R *ddd, int nthreads) {
    if (!d || d->n_freq < 2 || d->n_sites < 1) return -2;
    const int N = d->n_freq, Nl = d->n_sites;
    const int FN = N * N * (N + 1) / 2;
    {
        Su2<R> core(*d, v2, nullptr, ss, dd);
        for (int i = 0; i < N; ++i) dv2[i] = core.self_energy_flow(i, cutoff);
    }
    Su2<R> core(*d, v2, dv2, ss, dd);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        typename Su2<R>::Scratch sc(Nl);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int it = 0; it < FN; ++it) core.vertex_flow(it, cutoff, sc, dss + (long long)it * Nl, ddd + (long long)it * Nl);
    }
    return 0;
}

template <class R>
int rhs_range_impl(const OracleDesc *d, R cutoff, const R *v2, const R *dv2, const R *ss, const R *dd, int it0, int it1,
                   R *dss, R *ddd) {
    if (!d) return -2;
    Su2<R> core(*d, v2, dv2, ss, dd);
    typename Su2<R>::Scratch sc(d->n_sites);
    for (int it = it0; it < it1; ++it)
        core.vertex_flow(it, cutoff, sc, dss + (long long)(it - it0) * d->n_sites, ddd + (long long)(it - it0) * d->n_sites);
    return 0;
}

}  // namespace

extern "C" {

// One flow right-hand side: self-energy flow dv2[N], then vertex flow dss/ddd[F_N*Nl].
int oracle_su2_rhs_f32(const OracleDesc *d, float cutoff, const float *v2, const float *ss, const float *dd, float *dv2,
                       float *dss, float *ddd, int nthreads) {
    return rhs_impl<float>(d, cutoff, v2, ss, dd, dv2, dss, ddd, nthreads);
}
int oracle_su2_rhs_f64(const OracleDesc *d, double cutoff, const double *v2, const double *ss, const double *dd,
                       double *dv2, double *dss, double *ddd, int nthreads) {
    return rhs_impl<double>(d, cutoff, v2, ss, dd, dv2, dss, ddd, nthreads);
}

// Self-energy flow only.
int oracle_su2_self_energy_f32(const OracleDesc *d, float cutoff, const float *v2, const float *ss, const float *dd,
                               float *dv2) {
    if (!d) return -2;
    Su2<float> core(*d, v2, nullptr, ss, dd);
    for (int i = 0; i < d->n_freq; ++i) dv2[i] = core.self_energy_flow(i, cutoff);
    return 0;
}

// Vertex flow for triples [it0, it1) given an already computed self-energy flow (used to
// time a bounded sample on the CPU and to check subsets of large configurations).
int oracle_su2_vertex_range_f32(const OracleDesc *d, float cutoff, const float *v2, const float *dv2, const float *ss,
                                const float *dd, int it0, int it1, float *dss, float *ddd) {
    return rhs_range_impl<float>(d, cutoff, v2, dv2, ss, dd, it0, it1, dss, ddd);
}
int oracle_su2_vertex_range_f64(const OracleDesc *d, double cutoff, const double *v2, const double *dv2,
                                const double *ss, const double *dd, int it0, int it1, double *dss, double *ddd) {
    return rhs_range_impl<double>(d, cutoff, v2, dv2, ss, dd, it0, it1, dss, ddd);
}

// Vertex flow of an arbitrary list of triples, OpenMP-parallel (bounded CPU samples).
int oracle_su2_vertex_sample_f32(const OracleDesc *d, float cutoff, const float *v2, const float *dv2, const float *ss,
                                 const float *dd, const int *its, int n_its, float *dss, float *ddd, int nthreads) {
    if (!d) return -2;
    Su2<float> core(*d, v2, dv2, ss, dd);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        Su2<float>::Scratch sc(d->n_sites);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int k = 0; k < n_its; ++k)
            core.vertex_flow(its[k], cutoff, sc, dss + (long long)k * d->n_sites, ddd + (long long)k * d->n_sites);
    }
    return 0;
}

// Static susceptibility chi[Nl] (spin, density) at the given cutoff.
int oracle_su2_correlation_f32(const OracleDesc *d, float cutoff, const float *v2, const float *ss, const float *dd,
                               float *chi_s, float *chi_d) {
    if (!d) return -2;
    Su2<float> core(*d, v2, nullptr, ss, dd);
    core.correlation(cutoff, chi_s, chi_d);
    return 0;
}
int oracle_su2_correlation_f64(const OracleDesc *d, double cutoff, const double *v2, const double *ss,
                               const double *dd, double *chi_s, double *chi_d) {
    if (!d) return -2;
    Su2<double> core(*d, v2, nullptr, ss, dd);
    core.correlation(cutoff, chi_s, chi_d);
    return 0;
}

// Explicit Euler update x += (new - old) * dx, in float as the reference does.
void oracle_su2_euler_f32(float old_cutoff, float new_cutoff, long long n, float *x, const float *dx) {
    float step = new_cutoff - old_cutoff;
    for (long long i = 0; i < n; ++i) x[i] += step * dx[i];
}

// Complete flow over a cutoff list: measurement at every cutoff (before the Euler step),
// RHS + Euler between consecutive cutoffs, stopping early if the flow contains a NaN
// (SpinParser::runCore, src/SpinParser.cpp:126-187).  State arrays are updated in place;
// chi_s/chi_d receive n_cutoffs * Nl values; returns the number of measurements taken.
int oracle_su2_flow_f32(const OracleDesc *d, const float *cutoffs, int n_cutoffs, float *v2, float *ss, float *dd,
                        float *chi_s, float *chi_d, int nthreads) {
    if (!d || n_cutoffs < 2) return -2;
    const int N = d->n_freq, Nl = d->n_sites;
    const long long size = (long long)N * N * (N + 1) / 2 * Nl;
    std::vector<float> dv2(N), dss(size), ddd(size);
    int k = 0;
    float cutoff = cutoffs[0];
    for (; k < n_cutoffs - 1; ++k) {
        rhs_impl<float>(d, cutoff, v2, ss, dd, dv2.data(), dss.data(), ddd.data(), nthreads);
        oracle_su2_correlation_f32(d, cutoff, v2, ss, dd, chi_s + (long long)k * Nl, chi_d + (long long)k * Nl);
        bool nan = false;
        for (int i = 0; i < N && !nan; ++i) nan = std::isnan(dv2[i]);
        for (long long i = 0; i < size && !nan; ++i) nan = std::isnan(dss[i]) || std::isnan(ddd[i]);
        if (nan) break;
        float next = cutoffs[k + 1];
        oracle_su2_euler_f32(cutoff, next, N, v2, dv2.data());
        oracle_su2_euler_f32(cutoff, next, size, dd, ddd.data());
        oracle_su2_euler_f32(cutoff, next, size, ss, dss.data());
        cutoff = next;
    }
    oracle_su2_correlation_f32(d, cutoff, v2, ss, dd, chi_s + (long long)k * Nl, chi_d + (long long)k * Nl);
    return k + 1;
}

// The same flow entirely in double precision (the FP64 oracle of the precision study): the
// cutoff list is the float list of the task, every operation after that is FP64.
int oracle_su2_flow_f64(const OracleDesc *d, const float *cutoffs, int n_cutoffs, double *v2, double *ss, double *dd,
                        double *chi_s, double *chi_d, int nthreads) {
    if (!d || n_cutoffs < 2) return -2;
    const int N = d->n_freq, Nl = d->n_sites;
    const long long size = (long long)N * N * (N + 1) / 2 * Nl;
    std::vector<double> dv2(N), dss(size), ddd(size);
    int k = 0;
    double cutoff = cutoffs[0];
    auto euler = [](double step, long long n, double *x, const double *dx) {
        for (long long i = 0; i < n; ++i) x[i] += step * dx[i];
    };
    for (; k < n_cutoffs - 1; ++k) {
        rhs_impl<double>(d, cutoff, v2, ss, dd, dv2.data(), dss.data(), ddd.data(), nthreads);
        oracle_su2_correlation_f64(d, cutoff, v2, ss, dd, chi_s + (long long)k * Nl, chi_d + (long long)k * Nl);
        bool nan = false;
        for (int i = 0; i < N && !nan; ++i) nan = std::isnan(dv2[i]);
        for (long long i = 0; i < size && !nan; ++i) nan = std::isnan(dss[i]) || std::isnan(ddd[i]);
        if (nan) break;
        const double next = cutoffs[k + 1];
        euler(next - cutoff, N, v2, dv2.data());
        euler(next - cutoff, size, dd, ddd.data());
        euler(next - cutoff, size, ss, dss.data());
        cutoff = next;
    }
    oracle_su2_correlation_f64(d, cutoff, v2, ss, dd, chi_s + (long long)k * Nl, chi_d + (long long)k * Nl);
    return k + 1;
}

}  // extern "C"
