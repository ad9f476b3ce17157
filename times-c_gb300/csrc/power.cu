// Top eigenvectors of M_c = Q S_c Q for all clusters by power iteration
// (get_class_centers, shapeExtract.cuh:269-360, :577-630; the sign rule and store
// of get_center, :217-264).
//
// M v = S v - (1.v/m) r - (r.v/m) 1 + (tot 1.v/m^2) 1 with r = S 1 and tot = 1^T S 1,
// so M is never formed.  Step t: v_t = u_t/|u_t|, u_{t+1} = M v_t (FP32 dot
// products, FP64 norms, sums and step differences).
//
// One cooperative launch runs every step of every cluster.  Block b owns the
// contiguous rows [b*R/G, (b+1)*R/G) of the stacked k*m row space.  When they fit,
// the block copies its rows of S into shared memory once and keeps them there for
// all steps (RES); otherwise it streams them from L2/HBM each step.  After a step
// a bounded grid barrier publishes u_{t+1} and the statistics; each block then
// loads v_{t+1} of its clusters together with every cluster's step difference,
// and all blocks leave at the same t: when every non-empty cluster moved less
// than tol, or at t = tmax.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "tc_internal.h"

namespace tc {

constexpr int PST = 4;  // per slot, per cluster: |u|^2, sum u, r.u, |v_t - v_{t-1}|^2

__device__ __forceinline__ double* pst(double* st, int k, int t, int c) { return st + ((size_t)(t & 3) * k + c) * PST; }

__device__ __forceinline__ double block_sum_pw(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0;
    for (int w = 0; w < nw; ++w) s += red[w];
    return s;
}

__global__ void k_power_prep(const double* __restrict__ r, int k, int m, float* __restrict__ u,
                             double* __restrict__ st) {
    __shared__ double red[32];
    const int c = blockIdx.x;
    double s = 0, sy = 0, ry = 0;
    for (int a = threadIdx.x; a < m; a += blockDim.x) {
        float v = (a % 2 == 0) ? 1.0f : 0.5f;  // init_vec (shapeExtract.cuh:269-283)
        u[(size_t)c * m + a] = v;
        s += (double)v * v;
        sy += v;
        ry += r[(size_t)c * m + a] * (double)v;
    }
    s = block_sum_pw(s, red);
    sy = block_sum_pw(sy, red);
    ry = block_sum_pw(ry, red);
    if (threadIdx.x < 4 * PST) {
        int slot = threadIdx.x / PST, q = threadIdx.x % PST;
        double v = 0;
        if (slot == 0) v = q == 0 ? s : (q == 1 ? sy : (q == 2 ? ry : 0.0));
        st[((size_t)slot * k + c) * PST + q] = v;
    }
}

struct PowerParams {
    const float* S;
    const double* r;
    const double* tot;
    const int32_t* counts;
    int k, m, tmax, rows_max, ncl_max;
    double tol2;
    float* u;
    double* st;
    unsigned* bar;  // [0] arrivals, [1] generation
    int* status;    // [0] barrier timeout, [1] final T
};

constexpr unsigned long long BAR_SPIN_LIMIT = 1ull << 22;

// Grid-wide barrier of a cooperative launch (all blocks co-resident).  The wait is
// bounded: after BAR_SPIN_LIMIT polls it records a timeout in *err and returns.
__device__ __forceinline__ void grid_barrier(unsigned* bar, unsigned nblocks, unsigned& gen, int* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned arrived = atomicAdd(&bar[0], 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            unsigned long long spins = 0;
            while (*(volatile unsigned*)&bar[1] == gen) {
                __nanosleep(40);
                if (++spins > BAR_SPIN_LIMIT) {
                    atomicExch(err, 1);
                    break;
                }
            }
        }
        ++gen;
        __threadfence();
    }
    __syncthreads();
}

// Dynamic shared memory of the persistent kernel, 16-byte aligned sections:
// [S rows (RES only)] [v of the block's clusters] [v_{t-1} at own rows] [per-warp sums]
// [r at own rows] [cluster sizes]
struct PowerLayout {
    size_t sv, vprev, wacc, rown, cnt, total;
    __host__ __device__ PowerLayout(bool res, int rows_max, int ncl_max, int m, int k) {
        auto a16 = [](size_t x) { return (x + 15) & ~size_t(15); };
        sv = res ? a16((size_t)rows_max * m * 4) : 0;
        vprev = sv + a16((size_t)ncl_max * m * 4);
        wacc = vprev + a16((size_t)rows_max * 4);
        rown = wacc + a16((size_t)32 * ncl_max * PST * 8);
        cnt = rown + a16((size_t)rows_max * 8);
        total = cnt + a16((size_t)k * 4);
    }
};

template <bool RES>
__global__ void __launch_bounds__(1024, 1) k_power_persistent(PowerParams p) {
    extern __shared__ __align__(16) unsigned char dsm[];
    const int k = p.k, m = p.m;
    const PowerLayout L(RES, p.rows_max, p.ncl_max, m, k);
    float* S_res = reinterpret_cast<float*>(dsm);
    float* sv = reinterpret_cast<float*>(dsm + L.sv);        // v of the block's clusters
    float* vprev = reinterpret_cast<float*>(dsm + L.vprev);  // v_{t-1} at the block's own rows
    double* wacc = reinterpret_cast<double*>(dsm + L.wacc);  // [warp][lc][PST]
    double* r_own = reinterpret_cast<double*>(dsm + L.rown); // r at the block's own rows
    int* cnt = reinterpret_cast<int*>(dsm + L.cnt);          // cluster sizes
    __shared__ double sh_stat[8][4];  // per local cluster: |u|^2, sum u, r.u of the loaded step; tot
    __shared__ double sh_corr[8][2];
    __shared__ float sh_inv[8];
    __shared__ double red[32];
    __shared__ int sh_done, sh_status;
    const int64_t R = (int64_t)k * m;
    const unsigned G = gridDim.x;
    const int64_t r0 = R * blockIdx.x / G, r1 = R * (blockIdx.x + 1) / G;
    const int c_lo = (int)(r0 / m);
    const int ncl = r1 > r0 ? (int)((r1 - 1) / m) - c_lo + 1 : 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned gen = 0;

    // constants of the whole iteration live in shared memory (L1 is tiny next to them)
    for (int e = threadIdx.x; e < k; e += blockDim.x) cnt[e] = p.counts[e];
    for (int64_t e = threadIdx.x; e < r1 - r0; e += blockDim.x) r_own[e] = p.r[r0 + e];  // r is [c][a] = row order
    if (threadIdx.x < ncl) sh_stat[threadIdx.x][3] = p.tot[c_lo + threadIdx.x];
    if (RES) {
        const int64_t nval = (r1 - r0) * m;
        const float* src = p.S + (size_t)r0 * m;
        for (int64_t e = threadIdx.x; e < nval; e += blockDim.x) S_res[e] = __ldg(src + e);
    }
    __syncthreads();

    // Loads v_t (from u slot t%3 and stats slot t&3) for the block's clusters and,
    // in the same round trip, every cluster's step difference stored in that slot.
    // Returns the largest difference (0 when want_delta is false).
    auto load_step = [&](int t, bool want_delta) -> double {
        const int ncm = ncl * m;
        for (int e = threadIdx.x; e < ncm; e += blockDim.x) {
            const int lc = e / m, c = c_lo + lc;
            sv[e] = cnt[c] ? __ldcg(p.u + ((size_t)(t % 3) * k + c) * m + (e - lc * m)) : 0.f;
        }
        if (threadIdx.x < ncl * 3) {
            const int lc = threadIdx.x / 3, q = threadIdx.x % 3;
            sh_stat[lc][q] = __ldcg(pst(p.st, k, t, c_lo + lc) + q);
        }
        if (threadIdx.x == 0) sh_status = __ldcg(p.status);
        double mx = 0;
        if (want_delta)
            for (int c = threadIdx.x; c < k; c += blockDim.x)
                if (cnt[c] != 0) mx = fmax(mx, __ldcg(pst(p.st, k, t, c) + 3));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) red[wid] = mx;
        __syncthreads();
        if (threadIdx.x < ncl) {
            const int lc = threadIdx.x;
            const double inv = 1.0 / sqrt(sh_stat[lc][0]);
            const double s1 = sh_stat[lc][1] * inv, s2 = sh_stat[lc][2] * inv, mm = (double)m;
            sh_inv[lc] = (float)inv;
            sh_corr[lc][0] = -s1 / mm;
            sh_corr[lc][1] = -s2 / mm + sh_stat[lc][3] * s1 / (mm * mm);
        }
        double all = 0;
        for (int w = 0; w < nw; ++w) all = fmax(all, red[w]);
        __syncthreads();
        for (int e = threadIdx.x; e < ncm; e += blockDim.x) sv[e] *= sh_inv[e / m];
        __syncthreads();
        return all;
    };
    load_step(0, false);
    for (int t = 0;; ++t) {
        const int un = (t + 1) % 3;
        for (int e = threadIdx.x; e < nw * p.ncl_max * PST; e += blockDim.x) wacc[e] = 0.0;
        __syncthreads();
        double acc[PST] = {0.0, 0.0, 0.0, 0.0};
        int acc_lc = -1;
        for (int64_t row = r0 + wid; row < r1; row += nw) {
            const int c = (int)(row / m), a = (int)(row % m), lc = c - c_lo;
            if (cnt[c] == 0) continue;
            const float* Srow = RES ? S_res + (size_t)(row - r0) * m : p.S + (size_t)row * m;
            const float* v = sv + (size_t)lc * m;
            // compensated (Kahan) lane sums, FP64 across lanes: rounding noise well
            // below the convergence tolerance
            float s = 0.f, comp = 0.f;
            auto add = [&](float x) {
                const float y = x - comp, tt = s + y;
                comp = (tt - s) - y;
                s = tt;
            };
            if ((m & 3) == 0) {
                const float4* S4 = reinterpret_cast<const float4*>(Srow);
                const float4* v4 = reinterpret_cast<const float4*>(v);
                for (int b = lane; b < m / 4; b += 32) {
                    const float4 x = RES ? S4[b] : __ldg(S4 + b), w = v4[b];
                    add(x.x * w.x);
                    add(x.y * w.y);
                    add(x.z * w.z);
                    add(x.w * w.w);
                }
            } else {
                for (int b = lane; b < m; b += 32) add((RES ? Srow[b] : __ldg(Srow + b)) * v[b]);
            }
            double ds = (double)s - (double)comp;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ds += __shfl_xor_sync(0xffffffffu, ds, o);
            if (lane == 0) {
                if (lc != acc_lc) {
                    if (acc_lc >= 0)
                        for (int q = 0; q < PST; ++q) wacc[((size_t)wid * p.ncl_max + acc_lc) * PST + q] += acc[q];
                    acc_lc = lc;
                    for (int q = 0; q < PST; ++q) acc[q] = 0.0;
                }
                const double ra = r_own[row - r0];
                const float yf = (float)(ds + sh_corr[lc][0] * ra + sh_corr[lc][1]);
                p.u[((size_t)un * k + c) * m + a] = yf;
                acc[0] += (double)yf * yf;
                acc[1] += (double)yf;
                acc[2] += ra * (double)yf;
                const float va = v[a];
                if (t >= 1) {
                    const double d = (double)va - (double)vprev[row - r0];
                    acc[3] += d * d;
                }
                vprev[row - r0] = va;
            }
        }
        if (lane == 0 && acc_lc >= 0)
            for (int q = 0; q < PST; ++q) wacc[((size_t)wid * p.ncl_max + acc_lc) * PST + q] += acc[q];
        __syncthreads();
        if (threadIdx.x < ncl * PST) {
            const int lc = threadIdx.x / PST, q = threadIdx.x % PST;
            const int c = c_lo + lc;
            double sum = 0.0;
            for (int w = 0; w < nw; ++w) sum += wacc[((size_t)w * p.ncl_max + lc) * PST + q];
            if (cnt[c] != 0) atomicAdd(pst(p.st, k, t + 1, c) + q, sum);
        }
        grid_barrier(p.bar, G, gen, p.status);
        const double dmax = load_step(t + 1, t >= 1);
        if (threadIdx.x == 0) sh_done = t >= p.tmax || sh_status != 0 || (t >= 1 && dmax < p.tol2);
        __syncthreads();
        if (sh_done) {
            if (blockIdx.x == 0 && threadIdx.x == 0) p.status[1] = t;
            break;
        }
        // the slot step t+2 accumulates into; its last reader finished before this step's barrier
        if (blockIdx.x == 0)
            for (int e = threadIdx.x; e < k * PST; e += blockDim.x) p.st[(size_t)((t + 3) & 3) * k * PST + e] = 0.0;
    }
}

// v = u_T/|u_T|, lambda = v . u_{T+1} (FP64).  lambda > 0: sign rule against the
// cluster's first member a (flip when |a - v| >= |a + v|) and store (canonical:
// re-z-normalised, ddof=1).  lambda <= 0 (M numerically zero): the last basis
// vector - the last column of a symmetric eigensolver's identity basis - with the
// same sign rule.  NaN: the centroid is left unchanged (neither branch of
// shapeExtract.cuh:638-649 fires).
__global__ void k_power_final(const float* __restrict__ u, const double* __restrict__ st,
                              const int32_t* __restrict__ counts, const int32_t* __restrict__ offsets,
                              const float* __restrict__ seg, int k, int m, int T, int mode,
                              float* __restrict__ C) {
    __shared__ double red[32];
    __shared__ double sh_lam;
    const int c = blockIdx.x;
    if (counts[c] == 0) return;
    const float* uT = u + ((size_t)(T % 3) * k + c) * m;
    const float* uN = u + ((size_t)((T + 1) % 3) * k + c) * m;
    const double invT = 1.0 / sqrt(st[((size_t)(T & 3) * k + c) * PST]);
    const float finv = (float)invT;
    const float* a = seg + (size_t)offsets[c] * m;
    double lam = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) lam += (double)(uT[i] * finv) * (double)uN[i];
    lam = block_sum_pw(lam, red);
    if (threadIdx.x == 0) sh_lam = lam;
    __syncthreads();
    lam = sh_lam;
    if (!(lam > 0) && !(lam <= 0)) return;  // NaN
    const bool degenerate = !(lam > 0);
    auto vec = [&](int i) -> double { return degenerate ? (i == m - 1 ? 1.0 : 0.0) : (double)(uT[i] * finv); };
    double d1 = 0, d2 = 0, sum = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const double v = vec(i), ai = a[i];
        d1 += (ai - v) * (ai - v);
        d2 += (ai + v) * (ai + v);
        sum += v;
    }
    d1 = block_sum_pw(d1, red);
    d2 = block_sum_pw(d2, red);
    sum = block_sum_pw(sum, red);
    const double sgn = (sqrt(d1) >= sqrt(d2)) ? -1.0 : 1.0;
    double mean = 0, inv = 1;
    if (mode == TC_MODE_CANONICAL) {
        mean = sgn * sum / m;
        double ss = 0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const double v = sgn * vec(i);
            ss += (v - mean) * (v - mean);
        }
        ss = block_sum_pw(ss, red);
        const double sd = sqrt(ss / (m - 1));
        inv = sd > 0 ? 1.0 / sd : 0.0;
    }
    float* out = C + (size_t)c * m;
    for (int i = threadIdx.x; i < m; i += blockDim.x) out[i] = (float)((sgn * vec(i) - mean) * inv);
}

// ---------------------------------------------------------------- host
template <bool RES>
static void launch_power(tc_ctx* ctx, PowerParams& pp, int G, size_t smem, cudaStream_t s) {
    void* args[] = {&pp};
    TC_CUDA(cudaLaunchCooperativeKernel((const void*)k_power_persistent<RES>, dim3(G), dim3(1024), args, smem, s));
    TC_CHECK_LAUNCH();
}

void power_eigvecs(tc_ctx* ctx, const float* S, const double* r, const double* tot, const int32_t* counts,
                   const int32_t* offsets, const float* seg, int k, int m, int mode, int tmax, double tol, float* C,
                   cudaStream_t s) {
    Workspace& ws = ctx->ws;
    float* u = ws.piter.as<float>((size_t)3 * k * m);
    double* st = ws.pstats.as<double>((size_t)4 * PST * k);
    k_power_prep<<<k, 256, 0, s>>>(r, k, m, u, st);
    TC_CHECK_LAUNCH();

    const int G = ctx->sm_count;  // one 1024-thread block per SM
    const int64_t R = (int64_t)k * m;
    int rows_max = 0, ncl_max = 0;
    for (int b = 0; b < G; ++b) {
        int64_t r0 = R * b / G, r1 = R * (b + 1) / G;
        rows_max = std::max(rows_max, (int)(r1 - r0));
        if (r1 > r0) ncl_max = std::max(ncl_max, (int)((r1 - 1) / m - r0 / m + 1));
    }
    TC_REQUIRE(ncl_max <= 8, TC_ERR_UNSUPPORTED, "power iteration: more than 8 clusters per block");
    const size_t res_bytes = PowerLayout(true, rows_max, ncl_max, m, k).total;
    const bool res = res_bytes + 2048 <= ctx->smem_optin;
    const size_t smem = PowerLayout(res, rows_max, ncl_max, m, k).total;
    TC_REQUIRE(smem + 2048 <= ctx->smem_optin, TC_ERR_UNSUPPORTED, "power iteration: k*m too large");
    int per_sm = 0;
    if (res) {
        TC_CUDA(cudaFuncSetAttribute(k_power_persistent<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_power_persistent<true>, 1024, smem));
    } else {
        TC_CUDA(cudaFuncSetAttribute(k_power_persistent<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_power_persistent<false>, 1024, smem));
    }
    TC_REQUIRE(per_sm >= 1, TC_ERR_UNSUPPORTED, "power iteration kernel does not fit on an SM");
    int32_t* status = reinterpret_cast<int32_t*>(ws.aux.as<char>(64) + 32);
    unsigned* bar = reinterpret_cast<unsigned*>(status + 2);
    TC_CUDA(cudaMemsetAsync(status, 0, 16, s));
    PowerParams pp{S, r, tot, counts, k, m, tmax, rows_max, ncl_max, tol * tol, u, st, bar, status};
    if (res) launch_power<true>(ctx, pp, G, smem, s);
    else launch_power<false>(ctx, pp, G, smem, s);
    int32_t h[2];
    TC_CUDA(cudaMemcpyAsync(h, status, sizeof(h), cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaStreamSynchronize(s));
    TC_REQUIRE(h[0] == 0, TC_ERR_TIMEOUT, "power iteration: grid barrier wait ran out");
    if (std::getenv("TIMESC_TRACE"))
        std::fprintf(stderr, "timesc: power iteration k=%d m=%d steps=%d of %d (%s)\n", k, m, h[1], tmax,
                     res ? "S in shared memory" : "S streamed");
    k_power_final<<<k, 256, 0, s>>>(u, st, counts, offsets, seg, k, m, h[1], mode, C);
    TC_CHECK_LAUNCH();
}

}  // namespace tc
