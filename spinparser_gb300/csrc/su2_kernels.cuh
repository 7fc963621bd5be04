// Device bodies of the SU(2) flow kernels besides the vertex flow: self-energy flow, loop-
// frequency node tables, correlation measurement and the Euler update.  The single-flow
// kernels (su2_flow.cu) and the batched kernels (su2_batch.cu) call the same bodies, so a
// flow's numbers do not depend on whether it runs alone or in a batch.
#pragma once
#include "su2_common.cuh"
#include "su2_device.cuh"

namespace spn {
namespace dev {

constexpr double kPiD = 3.14159265358979323846;
constexpr int kCorrWarps = 4;  // the correlation kernels run 128-thread blocks

// ------------------------------------------------------------------------------------
// 1. self-energy flow
// ------------------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void self_energy_body(const FlowArgsT<T> &a, int blk) {
    __shared__ T pos[kMaxFreq];
    __shared__ double red[4];
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    const int i = blk;
    const T w = pos[i], L = T(a.cutoff);
    const T wpl = w + L, wml = w - L;
    const PairedState<T> st{a.sd};
    double part = 0.0;
    for (int j = threadIdx.x; j < a.n_range; j += blockDim.x) {
        const int r12 = a.range_rid[j], r21 = a.range_inv[j];
        T x1 = value_none(pos, a.n, a.nl, st, true, r12, r21, wpl, T(0), wml);
        T x2 = value_none(pos, a.n, a.nl, st, true, r12, r21, wml, T(0), wpl);
        part += double(x1) - double(x2);
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int k = 0; k < int(blockDim.x >> 5); ++k) sum += red[k];
        double val = -4.0 * double(a.spin) * sum;
        val += 0.75 * (double(value_none(pos, a.n, a.nl, st, false, 0, 0, wpl, wml, T(0))) -
                       double(value_none(pos, a.n, a.nl, st, false, 0, 0, wml, wpl, T(0))));
        val += (double(value_none(pos, a.n, a.nl, st, true, 0, 0, wpl, wml, T(0))) -
                double(value_none(pos, a.n, a.nl, st, true, 0, 0, wml, wpl, T(0))));
        const double sig = a.fp64_sigma ? odd_interp(pos, a.n, a.v2d, L) : odd_interp(pos, a.n, a.v2, L);
        val /= (2.0 * kPiD * (double(L) + sig));
        T out = T(val);
        a.dv2[i] = out;
        if (a.fp64_sigma) a.dv2d[i] = val;
        if (isnan(out)) atomicOr(a.status, kStatusNaN);
    }
}

// ------------------------------------------------------------------------------------
// 2. loop-frequency node tables
// ------------------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void node_table_body(const FlowArgsT<T> &a, int blk) {
    __shared__ T pos[kMaxFreq];
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    const int xi = blk * blockDim.x + threadIdx.x;
    if (xi >= a.n) return;
    const int n = a.n;
    const T x = pos[xi], L = T(a.cutoff);
    T *wp_out = a.node_wp + size_t(xi) * a.max_nodes;
    T *c_out = a.node_c + size_t(xi) * a.max_nodes;
    int cnt = 0;
    bool overflow = false;
    auto put = [&](T wp, double c) {
        if (cnt < a.max_nodes) {
            wp_out[cnt] = wp;
            c_out[cnt] = T(c);
            ++cnt;
        } else {
            overflow = true;
        }
    };
    auto sig = [&](T w) { return a.fp64_sigma ? odd_interp(pos, n, a.v2d, w) : odd_interp(pos, n, a.v2, w); };
    auto dsig = [&](T w) { return a.fp64_sigma ? odd_interp(pos, n, a.dv2d, w) : odd_interp(pos, n, a.dv2, w); };
    auto p = [&](T w1, T w2) { return 1.0 / ((double(w1) + sig(w1)) * (double(w2) + sig(w2))); };
    auto pk = [&](T w1, T w2) {
        double d1 = double(w1) + sig(w1);
        return dsig(w1) / (d1 * d1 * (double(w2) + sig(w2)));
    };
    // conventional contribution (SU2FrgCore.cpp:351-371)
    put(L, p(L, L + x));
    if (x > T(2) * L) put(-L, p(L, L - x));
    // Katanin contribution (SU2FrgCore.cpp:374-424)
    auto kat = [&](T wp, double weight) { put(wp, weight * pk(wp, x + wp)); };
    if (-(x + L) > -pos[n - 1]) nodes_right(pos, n, -(x + L), kat);
    if (x - L > L) nodes_both(pos, n, L - x, -L, kat);
    if (L < pos[n - 1]) nodes_left(pos, n, L, kat);
    a.node_cnt[xi] = cnt;
    if (overflow) atomicOr(a.status, kStatusNodeOverflow);
}

// ------------------------------------------------------------------------------------
// Euler update of one element, x + step * dx, rounded like the reference (product, then sum;
// SU2FrgCore.cpp:111-137)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ float euler_update(float x, float dx, float step) { return __fadd_rn(x, __fmul_rn(step, dx)); }
// FP64 self-energy (SPN_SU2_FP64_SELF_ENERGY) and the FP64 flow: the same update in double.
__device__ __forceinline__ double euler_update_f64(double x, double dx, double step) {
    return __dadd_rn(x, __dmul_rn(step, dx));
}

// ------------------------------------------------------------------------------------
// correlation measurement (nu = 0), SU2MeasurementCorrelation.cpp:77-177
// ------------------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ double corr_sigma(const CorrArgsT<T> &a, const T *pos, T w) {
    return a.v2d ? odd_interp(pos, a.n, a.v2d, w) : odd_interp(pos, a.n, a.v2, w);
}

// Loop-frequency nodes of the measurement's trapezoid rules at nu = 0 (outer and inner
// integrals use the same ranges): (-inf, -cutoff] and [cutoff, inf).
template <class T>
__device__ inline int corr_nodes(const T *pos, int n, T cut, T *wp, double *w) {
    int cnt = 0;
    auto put = [&](T x, double c) {
        wp[cnt] = x;
        w[cnt] = c;
        ++cnt;
    };
    if (-(T(0) + cut) > -pos[n - 1]) nodes_right(pos, n, -cut - T(0), put);
    if (cut < pos[n - 1]) nodes_left(pos, n, cut, put);
    return cnt;
}

constexpr int kMaxCorrNodes = 2 * kMaxFreq + 8;

// `st`: the state (PairedState of a flow, or SplitState of an allocation-free call).
template <int SPT, class T, class View>
__device__ __forceinline__ void corr_inner_body(const CorrArgsT<T> &a, const View &st, int blk) {
    __shared__ T pos[kMaxFreq];
    __shared__ T nwp[kMaxCorrNodes];
    __shared__ double nw[kMaxCorrNodes];
    __shared__ int ncnt;
    __shared__ double red[4][2][32 * SPT];
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    if (threadIdx.x == 0) ncnt = corr_nodes(pos, a.n, T(a.cutoff), nwp, nw);
    __syncthreads();
    const int ia = blk;
    if (ia >= ncnt) return;
    const T w = nwp[ia];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = (SPT == 1) ? a.wsite : 32;
    const int G = 32 / W;
    const int g = lane / W, jl = lane - g * W;
    const int nl = a.nl;
    int site[SPT], isite[SPT];
    bool valid[SPT];
    for (int k = 0; k < SPT; ++k) {
        const int j = jl + k * W;
        valid[k] = j < nl;
        site[k] = valid[k] ? a.sites[j] : 0;
        isite[k] = valid[k] ? a.inv_sites[j] : 0;
    }
    const double S = a.spin;
    auto sig = [&](T x) { return corr_sigma(a, pos, x); };
    const double dw = double(w) + sig(w);
    double acc_s[SPT], acc_d[SPT];
    for (int k = 0; k < SPT; ++k) acc_s[k] = acc_d[k] = 0.0;
    const int groups = kCorrWarps * G;
    const int gid = warp * G + g;
    for (int b = gid; b < ncnt; b += groups) {
        const T wp = nwp[b];
        AB8T<T> ab;
        access8(pos, a.n, nl, w + wp + T(0), T(0), w - wp, ab);
        const T vs = value_none(pos, a.n, nl, st, false, 0, 0, w + wp + T(0), w - wp, T(0));
        const T vd = value_none(pos, a.n, nl, st, true, 0, 0, w + wp + T(0), w - wp, T(0));
        const double dwp = double(wp) + sig(wp);
        const double norm = 1.0 / (dw * dw * dwp * dwp * (4.0 * kPiD * kPiD));
        const double cw = nw[b] * norm;
        for (int k = 0; k < SPT; ++k) {
            const int site_k = ab.exch ? isite[k] : site[k];
            T gs = T(0), gd = T(0);
            for (int q = 0; q < 8; ++q) {
                const pair_t<T> p = st.both(ab.off[q] + site_k);
                gs += ab.w[q] * p.x;
                gd += ab.sw[q] * p.y;
            }
            double rs = -S * S * double(gs);
            double rd = -16.0 * S * S * double(gd);
            if (jl + k * W == 0) {
                rs += S * (-double(vs) / 4.0 + double(vd));
                rd += S * (3.0 * double(vs) + 4.0 * double(vd));
            }
            if (valid[k]) {
                acc_s[k] += cw * rs;
                acc_d[k] += cw * rd;
            }
        }
    }
    for (int k = 0; k < SPT; ++k) {
        for (int o = W; o < 32; o <<= 1) {
            acc_s[k] += __shfl_xor_sync(0xffffffffu, acc_s[k], o);
            acc_d[k] += __shfl_xor_sync(0xffffffffu, acc_d[k], o);
        }
        if (g == 0) {
            red[warp][0][jl + k * W] = acc_s[k];
            red[warp][1][jl + k * W] = acc_d[k];
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nl; j += blockDim.x) {
        double s = 0.0, d = 0.0;
        for (int q = 0; q < kCorrWarps; ++q) {
            s += red[q][0][j];
            d += red[q][1][j];
        }
        a.partial[(size_t(ia) * 2 + 0) * nl + j] = s;
        a.partial[(size_t(ia) * 2 + 1) * nl + j] = d;
    }
}

template <class T>
__device__ __forceinline__ void corr_final_body(const CorrArgsT<T> &a) {
    __shared__ T pos[kMaxFreq];
    __shared__ T nwp[kMaxCorrNodes];
    __shared__ double nw[kMaxCorrNodes];
    __shared__ int ncnt;
    extern __shared__ double chi[];  // [2][nl]
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    if (threadIdx.x == 0) ncnt = corr_nodes(pos, a.n, T(a.cutoff), nwp, nw);
    __syncthreads();
    const double S = a.spin;
    for (int j = threadIdx.x; j < a.nl; j += blockDim.x) {
        double cs = 0.0, cd = 0.0;
        for (int ia = 0; ia < ncnt; ++ia) {
            double ls = a.partial[(size_t(ia) * 2 + 0) * a.nl + j];
            double ld = a.partial[(size_t(ia) * 2 + 1) * a.nl + j];
            if (j == 0) {
                const T w = nwp[ia];
                const double dw = double(w) + corr_sigma(a, pos, w);
                const double t1 = 1.0 / (dw * dw);
                ls += S * t1 / (2.0 * kPiD);
                ld += 2.0 * S * t1 / kPiD;
            }
            cs += nw[ia] * ls;
            cd += nw[ia] * ld;
        }
        chi[j] = cs;
        chi[a.nl + j] = cd;
        a.out[2 * a.n_corr + j] = T(cs);
        a.out[2 * a.n_corr + a.nl + j] = T(cd);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < a.n_corr; q += blockDim.x) {
        const int r = a.corr_rid[q];
        // an entry outside [0, nl) (possible only with caller-owned device tables) reads
        // nothing and yields NaN
        double zz = __longlong_as_double(0x7ff8000000000000LL), dd = zz;
        if (r >= 0 && r < a.nl) {
            zz = chi[r];
            dd = chi[a.nl + r];
        }
        a.out[q] = T(zz);
        a.out[a.n_corr + q] = T(dd);
    }
}


}  // namespace dev
}  // namespace spn
