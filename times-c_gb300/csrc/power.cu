// Top eigenvectors of M_c = Q S_c Q for all clusters by power iteration
// (get_class_centers, shapeExtract.cuh:269-360, :577-630; the sign rule and store
// of get_center, :217-264).
//
// M v = S v - (1.v/m) r - (r.v/m) 1 + (tot 1.v/m^2) 1 with r = S 1 and tot = 1^T S 1,
// so M is never formed.  Step t: v_t = u_t/|u_t|, u_{t+1} = M v_t: compensated FP32
// dot products summed across lanes in FP64; norms, sums, the step difference and
// the Rayleigh quotient in FP64.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tc_internal.h"

namespace tc {

// ---------------------------------------------------------------- cluster kernel
// One thread-block cluster of CL CTAs per k-Shape cluster c.  CTA `rank` owns rows
// [rank*m/CL, (rank+1)*m/CL) of S_c and streams them from L2/HBM every step.  Each
// CTA keeps the whole current vector v_t in shared memory; the new entries y_a and
// the per-CTA partial sums are stored straight into every CTA's shared memory
// (distributed shared memory), and one hardware cluster barrier per step makes
// them visible.  Every CTA then sums the partials in rank order, so all CTAs hold
// bit-identical norms and make the same stop decision.  Clusters stop
// independently.  Rank 0 finishes: lambda, sign rule, store.
constexpr int PC_THREADS = 512;
constexpr int PC_UNROLL = 4;  // rows in flight per warp

struct PowerClusterParams {
    const float* S;
    const double* r;
    const double* tot;
    const int32_t* counts;
    const int32_t* offsets;
    const float* seg;
    float* C;
    int k, m, tmax, mode;
    double tol2;
    int* steps;  // per cluster: the step T whose vector was stored (diagnostics)
};

template <int CL>
__global__ void __launch_bounds__(PC_THREADS) k_power_cluster(PowerClusterParams p) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char dsm[];
    const int m = p.m;
    const int rank = (int)cluster.block_rank();
    const int c = blockIdx.x / CL;
    if (p.counts[c] == 0) return;  // every CTA of this cluster leaves together
    const int a0 = (int)((int64_t)rank * m / CL), a1 = (int)((int64_t)(rank + 1) * m / CL);
    const int nrow = a1 - a0;
    // shared memory: v[m] | y[2][m] | part[2][CL][4] doubles | vprev[nrow] | r_own[nrow] doubles
    auto a16 = [](size_t x) { return (x + 15) & ~size_t(15); };
    float* v = reinterpret_cast<float*>(dsm);
    float* ybuf = reinterpret_cast<float*>(dsm + a16((size_t)m * 4));
    double* part = reinterpret_cast<double*>(dsm + a16((size_t)m * 4) + a16((size_t)2 * m * 4));
    float* vprev = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(part) + a16((size_t)2 * CL * 4 * 8));
    double* r_own = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(vprev) + a16((size_t)nrow * 4));
    __shared__ double red[PC_THREADS / 32][4];
    __shared__ double sh_corr[2];
    __shared__ int sh_done;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = PC_THREADS / 32;
    const double* rc = p.r + (size_t)c * m;
    const float* Sc = p.S + (size_t)c * m * m;
    const double mm = (double)m, totc = p.tot[c];
    for (int i = threadIdx.x; i < nrow; i += PC_THREADS) r_own[i] = rc[a0 + i];

    // v_0 = [1, .5, 1, .5, ...] / |.|, with its sum and r.v (identical in every CTA)
    {
        double s2 = 0, s1 = 0, sr = 0;
        for (int a = threadIdx.x; a < m; a += PC_THREADS) {
            const double x = (a % 2 == 0) ? 1.0 : 0.5;
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
            const double inv = 1.0 / sqrt(t2);
            sh_corr[0] = -(t1 * inv) / mm;
            sh_corr[1] = -(tr * inv) / mm + totc * (t1 * inv) / (mm * mm);
            red[0][3] = inv;
        }
        __syncthreads();
        const float finv = (float)red[0][3];
        for (int a = threadIdx.x; a < m; a += PC_THREADS) v[a] = ((a % 2 == 0) ? 1.0f : 0.5f) * finv;
        __syncthreads();
    }
    float* yrem[CL];
    double* prem[CL];
    for (int q = 0; q < CL; ++q) {
        yrem[q] = cluster.map_shared_rank(ybuf, q);
        prem[q] = cluster.map_shared_rank(part, q);
    }
    cluster.sync();  // every CTA initialised before remote stores start
    int T = p.tmax;
    for (int t = 0;; ++t) {
        const int par = t & 1;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        // own rows, PC_UNROLL rows per warp in flight
        for (int i0 = wid * PC_UNROLL; i0 < nrow; i0 += nw * PC_UNROLL) {
            float s[PC_UNROLL], cp[PC_UNROLL];
#pragma unroll
            for (int u = 0; u < PC_UNROLL; ++u) { s[u] = 0.f; cp[u] = 0.f; }
            if ((m & 3) == 0) {
                const float4* v4 = reinterpret_cast<const float4*>(v);
                for (int b = lane; b < m / 4; b += 32) {
                    const float4 w = v4[b];
                    float4 x[PC_UNROLL];
#pragma unroll
                    for (int u = 0; u < PC_UNROLL; ++u)
                        x[u] = (i0 + u < nrow) ? __ldg(reinterpret_cast<const float4*>(Sc + (size_t)(a0 + i0 + u) * m) + b)
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                    for (int u = 0; u < PC_UNROLL; ++u) {
                        const float pr[4] = {x[u].x * w.x, x[u].y * w.y, x[u].z * w.z, x[u].w * w.w};
#pragma unroll
                        for (int e = 0; e < 4; ++e) {  // Kahan
                            const float yk = pr[e] - cp[u], tt = s[u] + yk;
                            cp[u] = (tt - s[u]) - yk;
                            s[u] = tt;
                        }
                    }
                }
            } else {
                for (int b = lane; b < m; b += 32) {
                    const float w = v[b];
#pragma unroll
                    for (int u = 0; u < PC_UNROLL; ++u) {
                        const float x = (i0 + u < nrow) ? __ldg(Sc + (size_t)(a0 + i0 + u) * m + b) : 0.f;
                        const float yk = x * w - cp[u], tt = s[u] + yk;
                        cp[u] = (tt - s[u]) - yk;
                        s[u] = tt;
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < PC_UNROLL; ++u) {
                double ds = (double)s[u] - (double)cp[u];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) ds += __shfl_xor_sync(0xffffffffu, ds, o);
                const int i = i0 + u;
                if (i < nrow) {
                    const int a = a0 + i;
                    const double ra = r_own[i];
                    const float yf = (float)(ds + sh_corr[0] * ra + sh_corr[1]);
                    if (lane < CL) yrem[lane][par * m + a] = yf;  // into every CTA of the cluster
                    if (lane == 0) {
                        acc[0] += (double)yf * yf;
                        acc[1] += (double)yf;
                        acc[2] += ra * (double)yf;
                        const float va = v[a];
                        if (t >= 1) {
                            const double d = (double)va - (double)vprev[i];
                            acc[3] += d * d;
                        }
                        vprev[i] = va;
                    }
                }
            }
        }
        if (lane == 0)
            for (int q = 0; q < 4; ++q) red[wid][q] = acc[q];
        __syncthreads();
        if (threadIdx.x < 4) {
            double sum = 0;
            for (int w = 0; w < nw; ++w) sum += red[w][threadIdx.x];
            for (int q = 0; q < CL; ++q) prem[q][(par * CL + rank) * 4 + threadIdx.x] = sum;
        }
        cluster.sync();  // y and partials of step t visible in every CTA
        // identical reductions in every CTA (rank order)
        if (threadIdx.x == 0) {
            double n2 = 0, sy = 0, ry = 0, dd = 0;
            for (int q = 0; q < CL; ++q) {
                const double* pq = part + (par * CL + q) * 4;
                n2 += pq[0]; sy += pq[1]; ry += pq[2]; dd += pq[3];
            }
            const double inv = 1.0 / sqrt(n2);
            sh_corr[0] = -(sy * inv) / mm;
            sh_corr[1] = -(ry * inv) / mm + totc * (sy * inv) / (mm * mm);
            red[0][0] = inv;
            sh_done = t >= p.tmax || (t >= 1 && dd < p.tol2);
        }
        __syncthreads();
        if (sh_done) {
            T = t;
            break;
        }
        const float finv = (float)red[0][0];
        const float* y = ybuf + par * m;
        for (int a = threadIdx.x; a < m; a += PC_THREADS) v[a] = y[a] * finv;
        __syncthreads();
    }
    // v = v_T (unit), y = u_{T+1} = M v_T in ybuf[T&1]
    if (rank == 0) {
        const float* y = ybuf + (T & 1) * m;
        const float* am = p.seg + (size_t)p.offsets[c] * m;
        double lam = 0, d1 = 0, d2 = 0, sum = 0;
        for (int a = threadIdx.x; a < m; a += PC_THREADS) {
            lam += (double)v[a] * (double)y[a];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lam += __shfl_xor_sync(0xffffffffu, lam, o);
        if (lane == 0) red[wid][0] = lam;
        __syncthreads();
        if (threadIdx.x == 0) {
            double l = 0;
            for (int w = 0; w < nw; ++w) l += red[w][0];
            red[0][3] = l;
        }
        __syncthreads();
        lam = red[0][3];
        __syncthreads();
        const bool nan = !(lam > 0) && !(lam <= 0);
        const bool degenerate = !(lam > 0);
        if (!nan) {  // NaN: neither branch of shapeExtract.cuh:638-649 fires, the centroid stays
            auto vec = [&](int a) -> double { return degenerate ? (a == m - 1 ? 1.0 : 0.0) : (double)v[a]; };
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
            if (threadIdx.x == 0) {
                double a1s = 0, a2s = 0, ss = 0;
                for (int w = 0; w < nw; ++w) { a1s += red[w][0]; a2s += red[w][1]; ss += red[w][2]; }
                const double sgn = (sqrt(a1s) >= sqrt(a2s)) ? -1.0 : 1.0;  // get_center
                sh_corr[0] = sgn;
                sh_corr[1] = sgn * ss / mm;  // mean of the signed vector
            }
            __syncthreads();
            const double sgn = sh_corr[0];
            double mean = 0, inv = 1;
            if (p.mode == TC_MODE_CANONICAL) {
                mean = sh_corr[1];
                double sq = 0;
                for (int a = threadIdx.x; a < m; a += PC_THREADS) {
                    const double x = sgn * vec(a) - mean;
                    sq += x * x;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
                __syncthreads();
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
    cluster.sync();  // no CTA leaves while another may still touch its shared memory
}

// ---------------------------------------------------------------- host
template <int CL>
static void launch_cluster(const PowerClusterParams& pp, int k, size_t smem, cudaStream_t s) {
    TC_CUDA(cudaFuncSetAttribute(k_power_cluster<CL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
    TC_CUDA(cudaLaunchKernelEx(&cfg, k_power_cluster<CL>, pp));
    TC_CHECK_LAUNCH();
}

void power_eigvecs(tc_ctx* ctx, const float* S, const double* r, const double* tot, const int32_t* counts,
                   const int32_t* offsets, const float* seg, int k, int m, int mode, int tmax, double tol, float* C,
                   cudaStream_t s) {
    constexpr int CL = 8;  // CTAs per k-Shape cluster (portable cluster size)
    int* steps = ctx->ws.pstats.as<int>((size_t)k);
    auto a16 = [](size_t x) { return (x + 15) & ~size_t(15); };
    const int nrow = (m + CL - 1) / CL;
    const size_t smem = a16((size_t)m * 4) + a16((size_t)2 * m * 4) + a16((size_t)2 * CL * 4 * 8) +
                        a16((size_t)nrow * 4) + (size_t)nrow * 8;
    TC_REQUIRE(smem + 4096 <= ctx->smem_optin, TC_ERR_UNSUPPORTED, "power iteration: series too long");
    PowerClusterParams pp{S, r, tot, counts, offsets, seg, C, k, m, tmax, mode, tol * tol, steps};
    launch_cluster<CL>(pp, k, smem, s);
    if (std::getenv("TIMESC_TRACE")) {
        std::vector<int> h(k);
        TC_CUDA(cudaMemcpyAsync(h.data(), steps, sizeof(int) * k, cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaStreamSynchronize(s));
        int mx = 0, mn = 1 << 30;
        for (int j = 0; j < k; ++j) { mx = std::max(mx, h[j]); mn = std::min(mn, h[j]); }
        std::fprintf(stderr, "timesc: power iteration k=%d m=%d steps %d..%d of %d\n", k, m, mn, mx, tmax);
    }
}

}  // namespace tc
