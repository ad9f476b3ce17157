// Top eigenvectors of M_c = Q S_c Q for all clusters by power iteration
// (get_class_centers, shapeExtract.cuh:269-360, :577-630; the sign rule and store
// of get_center, :217-264).
//
// M v = S v - (1.v/m) r - (r.v/m) 1 + (tot 1.v/m^2) 1 with r = S 1 and tot = 1^T S 1,
// so M is never formed.  Step t: v_t = u_t/|u_t|, u_{t+1} = M v_t.  Where the
// repeated squaring (power_sq.cu) produced M^e v_0, the iteration starts from that
// vector instead, with its own step cap.
//
// One thread-block cluster of CL CTAs per k-Shape cluster c.  CTA `rank` owns rows
// [rank*m/CL, (rank+1)*m/CL) of S_c and streams them (float4, row pitch ld) from
// L2/HBM every step.  Each CTA keeps the whole current vector in shared memory;
// the new entries and the per-CTA partial sums are stored straight into every
// CTA's shared memory (distributed shared memory), and one hardware cluster
// barrier per step makes them visible.  Every CTA sums the partials in rank order,
// so all CTAs hold bit-identical norms and take the same stop decision; clusters
// stop independently.  Rank 0 finishes: Rayleigh quotient, sign rule, store.
//
// Arithmetic: row dot products are compensated FP32 (per lane, each float4's FMA
// chain Kahan-added; TwoSum across lanes); the norm, the sums and the step difference are accumulated as
// FP32 pairs (TwoSum, products split exactly by FMA: about 44 bits), so rounding
// noise in |v_t - v_{t-1}| stays well below the tolerance; FP64 only for the
// final per-step norm and corrections (one thread).
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tc_internal.h"

namespace tc {

constexpr int PC_THREADS = 512;
constexpr int PC_UNROLL = 4;  // rows in flight per warp

struct PowerClusterParams {
    const float* S;
    int ld;
    const double* r;
    const double* tot;
    const int32_t* counts;
    const int32_t* offsets;
    const float* seg;  // members in cluster order, or (lead_rows) the first member of each cluster
    int lead_rows;
    float* C;
    int k, m, tmax, mode;
    double tol2;   // squared step difference below which the stop test applies
    double tail2;  // squared bound on the movement still to come (geometric tail)
    int* steps;  // per cluster: the step T whose vector was stored (diagnostics)
    // start vectors from the repeated squaring (k x ld, any scale) where vok[c];
    // such clusters run at most tmax_sq steps
    const float* vinit;
    const int32_t* vok;
    int tmax_sq;
    const uint8_t* skip;  // clusters whose centroid is kept (may be null)
};

// (s, c) += (s2, c2) where a pair means s - c; the two leading parts are added
// error-free (TwoSum) and the rounding error folded into c.
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float s2, float c2) {
    const float t = s + s2;
    const float bp = t - s;
    const float err = (s - (t - bp)) + (s2 - bp);
    s = t;
    c = c + c2 - err;
}

// 1/sqrt(x) to double precision: FP32 estimate and two Newton steps.
__device__ __forceinline__ double rsqrt_d(double x) {
    double y = (double)rsqrtf((float)x);
    y = y * (1.5 - 0.5 * x * y * y);
    y = y * (1.5 - 0.5 * x * y * y);
    return y;
}

// BPL > 0: rows of at most 32*BPL float4 (loads unrolled); 0: any length.
// RES: the CTA's rows of S_c are copied into shared memory once and every step reads
// them there (when they fit: m <= ~600 with 8 CTAs per cluster), else from L2.
// HOLD (BPL <= 4, at most one group of rows per warp: m <= 512 with 8 CTAs): each
// warp loads its rows into registers once and keeps them for every step, so a step
// reads only the vector from shared memory (the rows are 128 KB per CTA a step).
template <int CL, int BPL, bool RES, bool HOLD>
__global__ void __launch_bounds__(PC_THREADS, 1) k_power_cluster(PowerClusterParams p) {
    static_assert(!HOLD || (BPL > 0 && BPL <= 4 && !RES), "HOLD keeps at most 4 x 4 float4 rows per lane");
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char dsm[];
    const int m = p.m, ld = p.ld;
    const int rank = CL == 1 ? 0 : (int)cluster.block_rank();
    // one CTA per k-Shape cluster: plain shared memory and CTA barriers
    auto cluster_sync = [&]() {
        if constexpr (CL == 1) __syncthreads();
        else cluster.sync();
    };
    const int c = blockIdx.x / CL;
    if (p.counts[c] == 0 || (p.skip && p.skip[c])) return;  // every CTA of this cluster leaves together
    const int a0 = (int)((int64_t)rank * m / CL), a1 = (int)((int64_t)(rank + 1) * m / CL);
    const int nrow = a1 - a0;
    // shared memory: v[ld] | y[2][ld] | part[2][CL][warps][4] float pairs | vprev[nrow] | r_own[nrow]
    //                | (RES) rows[nrow][ld]
    auto a16 = [](size_t x) { return (x + 15) & ~size_t(15); };
    float* v = reinterpret_cast<float*>(dsm);
    float* ybuf = reinterpret_cast<float*>(dsm + a16((size_t)ld * 4));
    constexpr int NWARP = PC_THREADS / 32;
    // per-step partial sums of every warp of every CTA: part[parity][rank][warp][4]
    float2* part = reinterpret_cast<float2*>(dsm + a16((size_t)ld * 4) + a16((size_t)2 * ld * 4));
    float* vprev = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(part) +
                                            a16((size_t)2 * CL * NWARP * 4 * 8));
    float* r_own = vprev + a16((size_t)nrow * 4) / 4;
    __shared__ double red[PC_THREADS / 32][4];
    __shared__ float sh_corr[2];
    __shared__ float sh_inv;
    __shared__ int sh_done;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = PC_THREADS / 32;
    const double* rc = p.r + (size_t)c * m;
    const float* Sc = p.S + (size_t)c * m * ld;
    const double inv_m = 1.0 / (double)m, totc = p.tot[c];
    const float finv_m = (float)inv_m, totf = (float)totc, tol2f = (float)p.tol2, tail2f = (float)p.tail2;
    float ddp = 0.f;  // the previous step's squared difference (warp 0, lane 0)
    for (int i = threadIdx.x; i < nrow; i += PC_THREADS) r_own[i] = (float)rc[a0 + i];
    const int nv4 = ld / 4;
    float4* srows = reinterpret_cast<float4*>(r_own + a16((size_t)nrow * 4) / 4);
    if constexpr (RES) {
        const float4* g = reinterpret_cast<const float4*>(Sc + (size_t)a0 * ld);
        for (int e = threadIdx.x; e < nrow * nv4; e += PC_THREADS) srows[e] = __ldg(g + e);
        // published by the barriers of the start-vector block below
    }

    // v_0 = [1, .5, 1, .5, ...] / |.| (or the squaring's vector, normalised), with its
    // sum and r.v (identical in every CTA)
    const float* vi = (p.vinit && p.vok[c]) ? p.vinit + (size_t)c * ld : nullptr;
    int tmax = p.tmax;
    {
        double s2 = 0, s1 = 0, sr = 0;
        for (int a = threadIdx.x; a < m; a += PC_THREADS) {
            const double x = vi ? (double)vi[a] : ((a % 2 == 0) ? 1.0 : 0.5);
            s2 += x * x;
            s1 += x;
            sr += rc[a] * x;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
        }
        if (lane == 0) { red[wid][0] = s2; red[wid][1] = s1; red[wid][2] = sr; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double t2 = 0, t1 = 0, tr = 0;
            for (int w = 0; w < nw; ++w) { t2 += red[w][0]; t1 += red[w][1]; tr += red[w][2]; }
            const bool use = vi && t2 > 0 && t2 < 1e300;  // a zero or non-finite product: start from v0
            if (vi && !use) {
                t2 = 0;
                t1 = 0;
                tr = 0;
                for (int a = 0; a < m; ++a) {
                    const double x = (a % 2 == 0) ? 1.0 : 0.5;
                    t2 += x * x;
                    t1 += x;
                    tr += rc[a] * x;
                }
            }
            const double inv = rsqrt_d(t2), sv = t1 * inv, rv = tr * inv;
            sh_corr[0] = (float)(-sv * inv_m);
            sh_corr[1] = (float)(-rv * inv_m + totc * sv * inv_m * inv_m);
            sh_inv = (float)inv;
            sh_done = use;
        }
        __syncthreads();
        const float finv = (float)sh_inv;
        if (!sh_done) vi = nullptr;
        else tmax = p.tmax_sq;
        for (int a = threadIdx.x; a < ld; a += PC_THREADS)
            v[a] = a < m ? (vi ? vi[a] : ((a % 2 == 0) ? 1.0f : 0.5f)) * finv : 0.f;
        for (int a = threadIdx.x; a < 2 * ld; a += PC_THREADS) ybuf[a] = 0.f;  // padding stays zero
        __syncthreads();
    }
    // lane q < CL stores into CTA q: one remote address per lane
    float* yre = CL == 1 ? ybuf : cluster.map_shared_rank(ybuf, lane < CL ? lane : 0);
    float2* pre = CL == 1 ? part : cluster.map_shared_rank(part, lane < CL ? lane : 0);
    constexpr int U = BPL >= 8 ? 2 : PC_UNROLL;  // rows in flight per warp
    constexpr int XU = HOLD ? U : 1, XB = HOLD ? BPL : 1;
    float4 xh[XU][XB];  // HOLD: this warp's rows wid*U.., loaded once
    if constexpr (HOLD) {
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < BPL; ++j) {
                const int i = wid * U + u, b = lane + 32 * j;
                xh[u][j] = (i < nrow && b < nv4)
                               ? __ldg(reinterpret_cast<const float4*>(Sc + (size_t)(a0 + i) * ld) + b)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
            }
    }
    cluster_sync();  // every CTA initialised before remote stores start
    int T = tmax;
    float fsc = 1.f;  // v_t = ybuf[(t-1)&1] * fsc for t >= 1 (the FP32 product the update stored before)
    for (int t = 0;; ++t) {
        const int par = t & 1;
        const float cr = sh_corr[0], cc = sh_corr[1];
        const float* vt = t == 0 ? v : ybuf + (par ^ 1) * ld;  // u_t, scaled by fsc below
        const float4* vt4 = reinterpret_cast<const float4*>(vt);
        // per-step sums as FP32 pairs (value = s - c), exact products by FMA: GB300's
        // FP64 pipe is too narrow for per-row double arithmetic
        float accs[4] = {0.f, 0.f, 0.f, 0.f}, accc[4] = {0.f, 0.f, 0.f, 0.f};
        auto add_prod = [&](int q, float a, float b) {
            const float pr = a * b, e = fmaf(a, b, -pr);  // a*b = pr + e exactly
            two_sum_acc(accs[q], accc[q], pr, -e);
        };
        for (int i0 = wid * U; i0 < nrow; i0 += nw * U) {
            float s[U], cp[U];
            const float4* rowp[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                s[u] = 0.f;
                cp[u] = 0.f;
                rowp[u] = RES ? srows + (size_t)min(i0 + u, nrow - 1) * nv4
                              : reinterpret_cast<const float4*>(Sc + (size_t)(a0 + min(i0 + u, nrow - 1)) * ld);
            }
            // a float4's four products as one FMA chain (a few ulp of a 4-term partial),
            // Kahan-added to the lane's sum: 8 operations where four Kahan additions take 20
            auto kahan4 = [&](int u, const float4& x, const float4& w) {
                const float pr = fmaf(x.w, w.w, fmaf(x.z, w.z, fmaf(x.y, w.y, x.x * w.x)));
                const float yk = pr - cp[u], tt = s[u] + yk;
                cp[u] = (tt - s[u]) - yk;
                s[u] = tt;
            };
            if constexpr (HOLD) {
#pragma unroll
                for (int j = 0; j < BPL; ++j) {
                    const int b = lane + 32 * j;
                    if (b < nv4) {
                        float4 w = vt4[b];
                        w.x *= fsc;
                        w.y *= fsc;
                        w.z *= fsc;
                        w.w *= fsc;
#pragma unroll
                        for (int u = 0; u < U; ++u) kahan4(u, xh[u][j], w);
                    }
                }
            } else if constexpr (BPL > 0) {
                // every load of the U rows in flight at once: one L2 round trip per step
                float4 x[U][BPL];
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int j = 0; j < BPL; ++j) {
                        const int b = lane + 32 * j;
                        x[u][j] = b < nv4 ? (RES ? rowp[u][b] : __ldg(rowp[u] + b)) : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
#pragma unroll
                for (int j = 0; j < BPL; ++j) {
                    const int b = lane + 32 * j;
                    if (b < nv4) {
                        float4 w = vt4[b];
                        w.x *= fsc;
                        w.y *= fsc;
                        w.z *= fsc;
                        w.w *= fsc;
#pragma unroll
                        for (int u = 0; u < U; ++u) kahan4(u, x[u][j], w);
                    }
                }
            } else {
                for (int b = lane; b < nv4; b += 32) {
                    float4 w = vt4[b];
                    w.x *= fsc;
                    w.y *= fsc;
                    w.z *= fsc;
                    w.w *= fsc;
                    float4 x[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) x[u] = RES ? rowp[u][b] : __ldg(rowp[u] + b);
#pragma unroll
                    for (int u = 0; u < U; ++u) kahan4(u, x[u], w);
                }
            }
            // a warp's U = 4 rows are consecutive: one 16-byte store per CTA instead of
            // four (the remote stores of a step are what its cluster barrier waits for)
            float yq[U];
            const bool vec4 = U == 4 && (a0 & 3) == 0 && i0 + U <= nrow;
#pragma unroll
            for (int u = 0; u < U; ++u) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float s2 = __shfl_xor_sync(0xffffffffu, s[u], o);
                    const float c2 = __shfl_xor_sync(0xffffffffu, cp[u], o);
                    two_sum_acc(s[u], cp[u], s2, c2);
                }
                const int i = i0 + u;
                if (i < nrow) {
                    const int a = a0 + i;
                    const float ra = r_own[i];
                    const float yf = (s[u] - cp[u]) + fmaf(cr, ra, cc);
                    yq[u] = yf;
                    // into every CTA of the cluster (four rows at once below when they can)
                    if (lane < CL && !vec4) yre[par * ld + a] = yf;
                    if (lane == 0) {
                        add_prod(0, yf, yf);
                        two_sum_acc(accs[1], accc[1], yf, 0.f);
                        add_prod(2, ra, yf);
                        const float va = vt[a] * fsc;
                        if (t >= 1) {
                            const float d = va - vprev[i];
                            add_prod(3, d, d);
                        }
                        vprev[i] = va;
                    }
                }
            }
            if constexpr (U == 4) {
                if (vec4 && lane < CL)
                    *reinterpret_cast<float4*>(yre + par * ld + a0 + i0) = make_float4(yq[0], yq[1], yq[2], yq[3]);
            }
        }
        // every warp's partial (held by lane 0) straight into every CTA, lane q storing into
        // CTA q: no CTA barrier before the exchange
        float2 mine[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            mine[q] = make_float2(__shfl_sync(0xffffffffu, accs[q], 0), __shfl_sync(0xffffffffu, accc[q], 0));
        if (lane < CL) {  // 32 bytes at a 32-byte offset: two 16-byte stores
            float4* dst = reinterpret_cast<float4*>(pre + ((size_t)(par * CL + rank) * NWARP + wid) * 4);
            dst[0] = make_float4(mine[0].x, mine[0].y, mine[1].x, mine[1].y);
            dst[1] = make_float4(mine[2].x, mine[2].y, mine[3].x, mine[3].y);
        }
        cluster_sync();  // y and partials of step t visible in every CTA
        if (wid == 0) {  // the same fixed order in every CTA, so all take the same decision
            float ts[4] = {0.f, 0.f, 0.f, 0.f}, tcm[4] = {0.f, 0.f, 0.f, 0.f};
            const float2* pp = part + (size_t)par * CL * NWARP * 4;
            for (int e = lane; e < CL * NWARP; e += 32)
#pragma unroll
                for (int q = 0; q < 4; ++q) two_sum_acc(ts[q], tcm[q], pp[e * 4 + q].x, pp[e * 4 + q].y);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float s2 = __shfl_xor_sync(0xffffffffu, ts[q], o);
                    const float c2 = __shfl_xor_sync(0xffffffffu, tcm[q], o);
                    two_sum_acc(ts[q], tcm[q], s2, c2);
                }
            if (lane == 0) {  // FP32 (GB300's FP64 pipe is narrow and this is the step's critical path)
                const float n2 = ts[0] - tcm[0], sy = ts[1] - tcm[1], ry = ts[2] - tcm[2], dd = ts[3] - tcm[3];
                float inv = rsqrtf(n2);
                inv = inv * fmaf(-0.5f * n2 * inv, inv, 1.5f);  // one Newton step: correctly rounded or 1 ulp
                const float sv = sy * inv, rv = ry * inv;
                sh_corr[0] = -sv * finv_m;
                sh_corr[1] = fmaf(totf * finv_m * finv_m, sv, -rv * finv_m);
                sh_inv = inv;
                // Stop test, once the step difference d_t = |v_t - v_{t-1}| is below tol:
                // the iteration contracts by rho = d_t/d_{t-1} per step, so the movement
                // still to come is about d_t rho/(1 - rho); stop when that is below the
                // tail bound, or when d_t no longer shrinks (rounding level).  A cluster
                // whose top eigenvalues nearly tie (rho near 1) runs on towards tmax.
                bool conv = false;
                if (t >= 2 && dd < tol2f) {
                    if (!(dd < ddp)) {
                        conv = true;
                    } else {
                        const float r = sqrtf(dd / ddp), q = 1.f - r;
                        conv = dd * r * r < tail2f * q * q;
                    }
                }
                ddp = dd;
                sh_done = t >= tmax || conv || !(n2 > 0.f);
            }
        }
        __syncthreads();
        if (sh_done) {
            T = t;
            break;
        }
        fsc = sh_inv;  // v_{t+1} = u_{t+1} * fsc, read from ybuf[par] in the next step
    }
    if (T >= 1) {  // materialise v_T = ybuf[(T-1)&1] * (its scale) for the final step
        const float* yv = ybuf + ((T - 1) & 1) * ld;
        __syncthreads();
        for (int a = threadIdx.x; a < m; a += PC_THREADS) v[a] = yv[a] * fsc;
        __syncthreads();
    }
    // v = v_T (unit), y = u_{T+1} = M v_T in ybuf[T&1]
    if (rank == 0) {
        const float* y = ybuf + (T & 1) * ld;
        const float* am = p.seg + (size_t)(p.lead_rows ? c : p.offsets[c]) * m;
        double lam = 0;
        for (int a = threadIdx.x; a < m; a += PC_THREADS) lam += (double)v[a] * (double)y[a];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lam += __shfl_xor_sync(0xffffffffu, lam, o);
        if (lane == 0) red[wid][0] = lam;
        __syncthreads();
        lam = 0;
        for (int w = 0; w < nw; ++w) lam += red[w][0];
        __syncthreads();
        const bool nan = !(lam > 0) && !(lam <= 0);
        const bool degenerate = !(lam > 0);
        if (!nan) {  // NaN: neither branch of shapeExtract.cuh:638-649 fires, the centroid stays
            auto vec = [&](int a) -> double { return degenerate ? (a == m - 1 ? 1.0 : 0.0) : (double)v[a]; };
            double d1 = 0, d2 = 0, sum = 0;
            for (int a = threadIdx.x; a < m; a += PC_THREADS) {
                const double va = vec(a), ai = am[a];
                d1 += (ai - va) * (ai - va);
                d2 += (ai + va) * (ai + va);
                sum += va;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                d1 += __shfl_xor_sync(0xffffffffu, d1, o);
                d2 += __shfl_xor_sync(0xffffffffu, d2, o);
                sum += __shfl_xor_sync(0xffffffffu, sum, o);
            }
            if (lane == 0) { red[wid][0] = d1; red[wid][1] = d2; red[wid][2] = sum; }
            __syncthreads();
            double a1s = 0, a2s = 0, ss = 0;
            for (int w = 0; w < nw; ++w) { a1s += red[w][0]; a2s += red[w][1]; ss += red[w][2]; }
            __syncthreads();
            const double sgn = (sqrt(a1s) >= sqrt(a2s)) ? -1.0 : 1.0;  // get_center
            double mean = 0, inv = 1;
            if (p.mode == TC_MODE_CANONICAL) {
                mean = sgn * ss * inv_m;
                double sq = 0;
                for (int a = threadIdx.x; a < m; a += PC_THREADS) {
                    const double x = sgn * vec(a) - mean;
                    sq += x * x;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
                if (lane == 0) red[wid][0] = sq;
                __syncthreads();
                double tq = 0;
                for (int w = 0; w < nw; ++w) tq += red[w][0];
                const double sd = sqrt(tq / (m - 1));
                inv = sd > 0 ? 1.0 / sd : 0.0;
            }
            float* out = p.C + (size_t)c * m;
            for (int a = threadIdx.x; a < m; a += PC_THREADS) out[a] = (float)((sgn * vec(a) - mean) * inv);
        }
        if (threadIdx.x == 0 && p.steps) p.steps[c] = T;
    }
    cluster_sync();  // no CTA leaves while another may still touch its shared memory
}

// ---------------------------------------------------------------- host
template <int CL, int BPL, bool RES, bool HOLD = false>
static void launch_cluster(const PowerClusterParams& pp, int k, size_t smem, cudaStream_t s) {
    auto kern = k_power_cluster<CL, BPL, RES, HOLD>;
    allow_max_dynamic_smem(kern);
    if (CL > 8) TC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)k * CL);
    cfg.blockDim = dim3(PC_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TC_CUDA(cudaLaunchKernelEx(&cfg, kern, pp));
    TC_CHECK_LAUNCH();
}

template <int CL>
static size_t cluster_smem(int m, int ld, bool res) {
    auto a16 = [](size_t x) { return (x + 15) & ~size_t(15); };
    const int nrow = (m + CL - 1) / CL;
    constexpr int NWARP = PC_THREADS / 32;
    return a16((size_t)ld * 4) + a16((size_t)2 * ld * 4) + a16((size_t)2 * CL * NWARP * 4 * 8) + a16((size_t)nrow * 4) +
           a16((size_t)nrow * 4) + (res ? (size_t)nrow * ld * 4 : 0);
}

void power_eigvecs(tc_ctx* ctx, const float* S, int ld, const double* r, const double* tot, const int32_t* counts,
                   const int32_t* offsets, const float* seg, bool lead_rows, int k, int m, int mode, int tmax,
                   double tol, const float* vinit, const int32_t* vok, int tmax_sq, float* C, cudaStream_t s,
                   const uint8_t* skip) {
    int* steps = ctx->ws.pstats.as<int>((size_t)k);
    const double tail = 3e-8;  // movement still to come, L2 norm of a unit vector
    PowerClusterParams pp{S,     ld,          r,     tot,   counts, offsets, seg,  lead_rows ? 1 : 0, C, k, m, tmax,
                          mode,  tol * tol,   tail * tail,  steps,  vinit,   vok,  tmax_sq, skip};
    // long series stream tens of MB per step from HBM: spread each over 16 SMs
    if (m > 1024) {
        const size_t smem = cluster_smem<16>(m, ld, false);
        TC_REQUIRE(smem + 4096 <= ctx->smem_optin, TC_ERR_UNSUPPORTED, "power iteration: series too long");
        launch_cluster<16, 0, false>(pp, k, smem, s);
    } else {
        const int nv4 = ld / 4;
        // rows in registers when every warp holds at most one group of 4 rows of at most
        // 128 float4 (m <= 512); else resident in shared memory when they fit (4 KB left
        // for the static arrays)
        const bool hold = (m + 7) / 8 <= (PC_THREADS / 32) * PC_UNROLL && nv4 <= 128;
        const bool res = cluster_smem<8>(m, ld, true) + 4096 <= ctx->smem_optin && !std::getenv("TIMESC_POWER_L2");
        const size_t smem = cluster_smem<8>(m, ld, res && !hold);
        // with rows in registers, the smallest cluster whose CTAs hold them (64 rows a
        // CTA): a step's exchange and cluster barrier then span fewer CTAs
        constexpr int HOLD_ROWS = (PC_THREADS / 32) * PC_UNROLL;
        if (hold && m <= HOLD_ROWS && nv4 <= 32) {
            launch_cluster<1, 1, false, true>(pp, k, cluster_smem<1>(m, ld, false), s);
        } else if (hold && m <= 2 * HOLD_ROWS && nv4 <= 32) {
            launch_cluster<2, 1, false, true>(pp, k, cluster_smem<2>(m, ld, false), s);
        } else if (hold && m <= 4 * HOLD_ROWS && nv4 <= 64) {
            launch_cluster<4, 2, false, true>(pp, k, cluster_smem<4>(m, ld, false), s);
        } else if (hold) {
            if (nv4 <= 32) launch_cluster<8, 1, false, true>(pp, k, smem, s);
            else if (nv4 <= 64) launch_cluster<8, 2, false, true>(pp, k, smem, s);
            else launch_cluster<8, 4, false, true>(pp, k, smem, s);
        } else if (res) {
            if (nv4 <= 32) launch_cluster<8, 1, true>(pp, k, smem, s);
            else if (nv4 <= 64) launch_cluster<8, 2, true>(pp, k, smem, s);
            else if (nv4 <= 128) launch_cluster<8, 4, true>(pp, k, smem, s);
            else launch_cluster<8, 8, true>(pp, k, smem, s);
        } else {
            if (nv4 <= 32) launch_cluster<8, 1, false>(pp, k, smem, s);
            else if (nv4 <= 64) launch_cluster<8, 2, false>(pp, k, smem, s);
            else if (nv4 <= 128) launch_cluster<8, 4, false>(pp, k, smem, s);
            else launch_cluster<8, 8, false>(pp, k, smem, s);
        }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    TC_CUDA(cudaStreamIsCapturing(s, &cap));
    if (std::getenv("TIMESC_TRACE") && cap == cudaStreamCaptureStatusNone) {
        std::vector<int> h(k);
        TC_CUDA(cudaMemcpyAsync(h.data(), steps, sizeof(int) * k, cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaStreamSynchronize(s));
        int mx = 0, mn = 1 << 30;
        for (int j = 0; j < k; ++j) { mx = std::max(mx, h[j]); mn = std::min(mn, h[j]); }
        std::fprintf(stderr, "timesc: power iteration k=%d m=%d steps %d..%d of %d\n", k, m, mn, mx, tmax);
    }
}

}  // namespace tc
