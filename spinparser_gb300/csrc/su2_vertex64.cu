// Two-particle vertex flow in double precision (flows created with SPN_SU2_FP64): the
// reference's right-hand side (SU2FrgCore::_calculateVertexTwoParticle,
// src/SU2/SU2FrgCore.cpp:171-431) evaluated entirely in FP64 on the GPU, the precision
// reference for the FP32 flows of the same task.
//
// Written for clarity rather than speed: a persistent grid whose warps take one (s,t,u)
// triple at a time from a device counter; the lanes hold the sites (up to four each); the
// loop-frequency nodes of each channel are visited in order; every lane builds the node's
// access buffers itself; the t channel's RPA sum runs over each rid's own overlap pair list
// in the reference's order (SU2FrgCore.cpp:249-266).  The node tables (conventional and
// Katanin terms with their quadrature weights) come from the same node-table body as the
// FP32 flow, instantiated in double.
#include "su2_common.cuh"
#include "su2_device.cuh"

namespace spn {
namespace {

using namespace spn::dev;

constexpr int kThreads64 = 128;
constexpr int kWarps64 = kThreads64 / 32;
constexpr int kSitesPerLane64 = 4;  // Nl <= 128
constexpr double kPi64 = 3.14159265358979323846;

struct Freqs {
    double s, t, u, w1p, w1, w2p, w2;
};

// Interpolated slab of one access buffer for the lane's sites (getValueSuperbundle).
__device__ __forceinline__ void gather64(const FlowArgsT<double> &a, const AB4T<double> &ab, const int *site,
                                         const int *isite, const bool *valid, double *vs, double *vd) {
#pragma unroll
    for (int k = 0; k < kSitesPerLane64; ++k) {
        double gs = 0.0, gd = 0.0;
        if (valid[k]) {
            const int st = ab.exch ? isite[k] : site[k];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const double2 p = a.sd[ab.off[q] + st];
                gs += ab.w[q] * p.x;
                gd += ab.sw[q] * p.y;
            }
        }
        vs[k] = gs;
        vd[k] = gd;
    }
}

// Site-local (rid 0) value pair of an access buffer.
__device__ __forceinline__ void local64(const FlowArgsT<double> &a, const AB4T<double> &ab, double &vs, double &vd) {
    double gs = 0.0, gd = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double2 p = a.sd[ab.off[q]];
        gs += ab.w[q] * p.x;
        gd += ab.sw[q] * p.y;
    }
    vs = gs;
    vd = gd;
}

__global__ void __launch_bounds__(kThreads64) su2_vertex_flow_f64_kernel(FlowArgsT<double> a) {
    __shared__ double pos[kMaxFreq];
    extern __shared__ double xs[];  // per warp: As, Ad, Bs, Bd [nl each]
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) pos[i] = a.freq[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = a.n, nl = a.nl;
    double *As = xs + size_t(warp) * 4 * nl, *Ad = As + nl, *Bs = Ad + nl, *Bd = Bs + nl;
    int site[kSitesPerLane64], isite[kSitesPerLane64], jj[kSitesPerLane64];
    bool valid[kSitesPerLane64];
#pragma unroll
    for (int k = 0; k < kSitesPerLane64; ++k) {
        jj[k] = lane + 32 * k;
        valid[k] = jj[k] < nl;
        site[k] = valid[k] ? a.sites[jj[k]] : 0;
        isite[k] = valid[k] ? a.inv_sites[jj[k]] : 0;
    }
    const double s2 = 2.0 * double(a.spin), s8 = 8.0 * double(a.spin);

    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.work_counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= a.fn) break;
        const int su = it / n, ti = it - su * n;
        int si = int((sqrt(8.0 * double(su) + 1.0) - 1.0) * 0.5);
        while (si * (si + 1) / 2 > su) --si;
        while ((si + 1) * (si + 2) / 2 <= su) ++si;
        const int ui = su - si * (si + 1) / 2;
        Freqs f;
        f.s = pos[si];
        f.t = pos[ti];
        f.u = pos[ui];
        f.w1p = 0.5 * (f.s + f.t + f.u);
        f.w1 = 0.5 * (f.s - f.t + f.u);
        f.w2p = 0.5 * (f.s - f.t - f.u);
        f.w2 = 0.5 * (f.s + f.t - f.u);

        double acc_s[kSitesPerLane64] = {}, acc_d[kSitesPerLane64] = {};
        for (int ch = 0; ch < 3; ++ch) {
            const int xi = ch == 0 ? si : (ch == 1 ? ti : ui);
            const int cnt = a.node_cnt[xi];
            const double *nwp = a.node_wp + size_t(xi) * a.max_nodes;
            const double *nc = a.node_c + size_t(xi) * a.max_nodes;
            for (int b = 0; b < cnt; ++b) {
                const double wp = nwp[b];
                const double c = ch == 2 ? -nc[b] : nc[b];
                AB4T<double> ab[4];
                double S0[kSitesPerLane64], S1[kSitesPerLane64], S2[kSitesPerLane64], S3[kSitesPerLane64];
                double D0[kSitesPerLane64], D1[kSitesPerLane64], D2[kSitesPerLane64], D3[kSitesPerLane64];
                double xv[kSitesPerLane64], yv[kSitesPerLane64];
                if (ch == 0) {  // integralKernelS, SU2FrgCore.cpp:199-227
                    access4<kS>(pos, n, nl, f.s, -f.w1 - wp, -f.w2 - wp, ab[0]);
                    access4<kS>(pos, n, nl, f.s, f.w1p + wp, -f.w2p - wp, ab[1]);
                    access4<kS>(pos, n, nl, f.s, f.w2 + wp, f.w1 + wp, ab[2]);
                    access4<kS>(pos, n, nl, f.s, -f.w2p - wp, f.w1p + wp, ab[3]);
                } else if (ch == 1) {  // integralKernelT, SU2FrgCore.cpp:229-303
                    access4<kT>(pos, n, nl, f.w1 - wp, f.t, f.w1p + wp, ab[0]);
                    access4<kT>(pos, n, nl, f.w2p - wp, f.t, -f.w2 - wp, ab[1]);
                    access4<kT>(pos, n, nl, f.w1p + wp, f.t, f.w1 - wp, ab[2]);
                    access4<kT>(pos, n, nl, f.w2 + wp, f.t, wp - f.w2p, ab[3]);
                } else {  // integralKernelU, SU2FrgCore.cpp:305-334
                    access4<kU>(pos, n, nl, f.w1 + wp, wp - f.w2p, f.u, ab[0]);
                    access4<kU>(pos, n, nl, f.w1p + wp, f.w2 - wp, f.u, ab[1]);
                    access4<kU>(pos, n, nl, f.w2p - wp, -f.w1 - wp, f.u, ab[2]);
                    access4<kU>(pos, n, nl, f.w2 - wp, f.w1p + wp, f.u, ab[3]);
                }
                gather64(a, ab[0], site, isite, valid, S0, D0);
                gather64(a, ab[1], site, isite, valid, S1, D1);
                gather64(a, ab[2], site, isite, valid, S2, D2);
                gather64(a, ab[3], site, isite, valid, S3, D3);
                if (ch != 1) {
#pragma unroll
                    for (int k = 0; k < kSitesPerLane64; ++k) {
                        double x = 0.0, y = 0.0;
                        if (ch == 0) {
                            x -= 0.5 * S0[k] * S1[k];
                            x -= 0.5 * S2[k] * S3[k];
                            x += D0[k] * S1[k];
                            x += D2[k] * S3[k];
                            x += S0[k] * D1[k];
                            x += S2[k] * D3[k];
                        } else {
                            x += 0.5 * S0[k] * S1[k];
                            x += 0.5 * S2[k] * S3[k];
                            x += S0[k] * D1[k];
                            x += S2[k] * D3[k];
                            x += D0[k] * S1[k];
                            x += D2[k] * S3[k];
                        }
                        y += (3.0 / 16.0) * S0[k] * S1[k];
                        y += (3.0 / 16.0) * S2[k] * S3[k];
                        y += D0[k] * D1[k];
                        y += D2[k] * D3[k];
                        xv[k] = x;
                        yv[k] = y;
                    }
                } else {
                    // exchange the third and fourth slabs, then the RPA sum per rid
#pragma unroll
                    for (int k = 0; k < kSitesPerLane64; ++k)
                        if (valid[k]) {
                            As[jj[k]] = S2[k];
                            Ad[jj[k]] = D2[k];
                            Bs[jj[k]] = S3[k];
                            Bd[jj[k]] = D3[k];
                        }
                    __syncwarp();
                    AB4T<double> lb;
                    double cbs, cbd, icas, icad, cbs2, cbd2, icas2, icad2;
                    access4<kU>(pos, n, nl, f.w2p - wp, -f.w2 - wp, f.t, lb);
                    local64(a, lb, cbs, cbd);
                    access4<kU>(pos, n, nl, f.w1 - wp, -f.w1p - wp, -f.t, lb);
                    local64(a, lb, icas, icad);
                    access4<kU>(pos, n, nl, f.w2 + wp, wp - f.w2p, f.t, lb);
                    local64(a, lb, cbs2, cbd2);
                    access4<kU>(pos, n, nl, f.w1p + wp, wp - f.w1, -f.t, lb);
                    local64(a, lb, icas2, icad2);
#pragma unroll
                    for (int k = 0; k < kSitesPerLane64; ++k) {
                        double rpa_s = 0.0, rpa_d = 0.0;
                        if (valid[k]) {
                            const int r = jj[k];
                            for (int i = a.ov_ptr[r]; i < a.ov_ptr[r + 1]; ++i) {
                                const int r1 = a.ov_r1[i], r2 = a.ov_r2[i];
                                rpa_s += As[r1] * Bs[r2];
                                rpa_d += Ad[r1] * Bd[r2];
                            }
                        }
                        double x = 0.0 + s2 * rpa_s;  // SU2FrgCore.cpp:265, 286-293
                        x -= cbd * S0[k];
                        x += (0.25 * cbs) * S0[k];
                        x -= icad * S1[k];
                        x += (0.25 * icas) * S1[k];
                        x -= cbd2 * S2[k];
                        x += (0.25 * cbs2) * S2[k];
                        x -= icad2 * S3[k];
                        x += (0.25 * icas2) * S3[k];
                        double y = 0.0 + s8 * rpa_d;  // SU2FrgCore.cpp:266, 295-302
                        y -= cbd * D0[k];
                        y -= (0.75 * cbs) * D0[k];
                        y -= icad * D1[k];
                        y -= (0.75 * icas) * D1[k];
                        y -= cbd2 * D2[k];
                        y -= (0.75 * cbs2) * D2[k];
                        y -= icad2 * D3[k];
                        y -= (0.75 * icas2) * D3[k];
                        xv[k] = x;
                        yv[k] = y;
                    }
                    __syncwarp();
                }
#pragma unroll
                for (int k = 0; k < kSitesPerLane64; ++k) {
                    acc_s[k] += c * xv[k];
                    acc_d[k] += c * yv[k];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kSitesPerLane64; ++k)
            if (valid[k]) {
                const double os = acc_s[k] / (2.0 * kPi64), od = acc_d[k] / (2.0 * kPi64);
                a.dsd[size_t(it) * nl + jj[k]] = make_double2(os, od);
                if (isnan(os) || isnan(od)) atomicOr(a.status, kStatusNaN);
            }
    }
}

}  // namespace

int vertex_flow_f64_blocks_per_sm(int nl) {
    const size_t smem = size_t(kWarps64) * 4 * nl * sizeof(double);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, su2_vertex_flow_f64_kernel, kThreads64, smem) != cudaSuccess)
        return -1;
    return per_sm;
}

void launch_vertex_flow_f64(const FlowArgsT<double> &a, int grid, cudaStream_t stream) {
    const size_t smem = size_t(kWarps64) * 4 * a.nl * sizeof(double);
    su2_vertex_flow_f64_kernel<<<grid, kThreads64, smem, stream>>>(a);
}

}  // namespace spn
