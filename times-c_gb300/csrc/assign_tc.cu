// SBD assignment on the tensor cores (tcgen05, BF16 operands, FP32 accumulation):
// the mixed-precision form of NCC_3D + get_pos_idx (ncc.cuh:469-517,
// kshape.cuh:35-96) for series of up to 512 samples.
//
// The circular correlation at lag t of the zero-padded length F is
//   r[t] = sum_{u < m} x[u] * c_pad[(u - t) mod F],
// a GEMM of the series (M = series, K = samples) with a Toeplitz matrix
// (N = lags).  The Toeplitz operand is never built: for b in 0..7 one shifted
// copy buf_b[e] = c_pad[(e - b) mod F] of the centroid is enough, because a
// K-major no-swizzle UMMA descriptor with 16-byte core-matrix strides (LBO 16,
// SBO 128) reads row n, element u from buf_b[8n + u] - row n is lag b - 8n.
// Eight copies (F/8 rows each) cover all F lags.
//
// Persistent, warp-specialised CTA (192 threads), one per SM:
//   warp 0  producer: TMA of a 128-series BF16 tile (resident for all
//           centroids) and bulk copies of each centroid's 8 shifted copies into a
//           double buffer;
//   warp 1  one thread issues M=128, N=F/8, K=16 MMAs into two 256-column TMEM
//           slots (b-groups of 256 lags), so MMAs fill one slot while the
//           epilogue drains the other;
//   warps 2-5 epilogue: tcgen05.ld of the row's 256 lags, max over valid lags,
//           NCC = max / (|x||c|) with FP32 norms of the original data, and the
//           running argmin over centroids - only (label, distance) reach HBM.
// All waits are bounded and report through an error word.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "sm100.cuh"
#include "tc_internal.h"

namespace tc {

CUtensorMap make_tmap_2d(const void* base, CUtensorMapDataType dt, int esize, uint64_t rows, uint64_t cols,
                         uint32_t box_rows);

constexpr int AT_THREADS = 192;
constexpr int AT_TILE = 128;        // series per tile (UMMA M)
constexpr int AT_SLOT_COLS = 256;   // TMEM columns per accumulator slot

struct AtGeom {
    int m, mp, F, NB, lnb, Gb, G, KS, Lb, bsz, nch;
    // mp: padded K (multiple of 64), NB = F/8 lags per shifted copy, Gb copies per
    // TMEM slot, G groups, KS = mp/16 K steps, Lb = elements per copy, bsz = bytes
    // of one centroid's 8 copies, nch = 64-column chunks of the series tile
    __host__ __device__ AtGeom(int m_, int F_) : m(m_), F(F_) {
        mp = (m + 63) / 64 * 64;
        NB = F / 8;
        lnb = 0;
        while ((1 << lnb) < NB) ++lnb;
        Gb = AT_SLOT_COLS / NB < 8 ? AT_SLOT_COLS / NB : 8;
        G = 8 / Gb;
        KS = mp / 16;
        Lb = (F + mp + 7) / 8 * 8;
        bsz = 8 * Lb * 2;
        nch = mp / 64;
    }
    // at least 116 KB so that one CTA (and one 512-column TMEM allocation) fits an SM
    size_t smem() const {
        const size_t s = (size_t)nch * 16384 + 2 * (size_t)bsz + 1024;
        return s > 116 * 1024 ? s : 116 * 1024;
    }
};

// Series -> BF16 [n][mp] (zero padded) and FP32 norms (compensated).
__global__ void k_series_bf16(const float* __restrict__ x, int64_t n, int m, int mp, __nv_bfloat16* __restrict__ xb,
                              float* __restrict__ xnorm) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < n; i += nw) {
        const float* r = x + (size_t)i * m;
        __nv_bfloat16* o = xb + (size_t)i * mp;
        float s = 0.f, c = 0.f;
        for (int t = lane; t < mp; t += 32) {
            const float v = t < m ? r[t] : 0.f;
            o[t] = __float2bfloat16_rn(v);
            const float y = v * v - c, tt = s + y;
            c = (tt - s) - y;
            s = tt;
        }
        double d = (double)s - (double)c;
#pragma unroll
        for (int q = 16; q > 0; q >>= 1) d += __shfl_xor_sync(0xffffffffu, d, q);
        if (lane == 0) xnorm[i] = (float)sqrt(d);
    }
}

// Centroid j -> 8 shifted BF16 copies buf_b[e] = c_pad[(e - b) mod F], e < Lb, and its norm.
__global__ void k_centroid_toeplitz(const float* __restrict__ C, int m, int F, int Lb,
                                    __nv_bfloat16* __restrict__ B, float* __restrict__ cnorm) {
    __shared__ double red[32];
    const int j = blockIdx.x;
    const float* c = C + (size_t)j * m;
    double s = 0;
    for (int t = threadIdx.x; t < m; t += blockDim.x) s += (double)c[t] * c[t];
#pragma unroll
    for (int q = 16; q > 0; q >>= 1) s += __shfl_xor_sync(0xffffffffu, s, q);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        cnorm[j] = (float)sqrt(t);
    }
    __nv_bfloat16* o = B + (size_t)j * 8 * Lb;
    for (int e = threadIdx.x; e < 8 * Lb; e += blockDim.x) {
        const int b = e / Lb, q = e % Lb;
        const int u = ((q - b) % F + F) % F;
        o[e] = __float2bfloat16_rn(u < m ? c[u] : 0.f);
    }
}

struct AtParams {
    const __nv_bfloat16* B;  // [k][8][Lb]
    const float* xnorm;
    const float* cnorm;
    int64_t n;
    int m, k, F, clamp2, mask;
    int32_t* labels;
    float* dist;
    const int32_t* old_labels;
    int32_t* changed;
    double* dist_sum;
    int* err;
};

__global__ void __launch_bounds__(AT_THREADS, 1) k_assign_tc(const __grid_constant__ CUtensorMap tmapX, AtParams p) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t a_full, a_empty, b_full[2], b_empty[2], t_full[2], t_empty[2], fin;
    __shared__ uint32_t tmem_base;
    const AtGeom g(p.m, p.F);
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* Atile = base;                                    // nch x 16 KB, 128B-swizzled K-major
    uint8_t* Bslot = base + (size_t)g.nch * 16384;            // 2 x bsz
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t ntiles = (p.n + AT_TILE - 1) / AT_TILE;
    if (threadIdx.x == 0) {
        sm100::mbar_init(&a_full, 1);
        sm100::mbar_init(&a_empty, 1);
        for (int s = 0; s < 2; ++s) {
            sm100::mbar_init(&b_full[s], 1);
            sm100::mbar_init(&b_empty[s], 1);
            sm100::mbar_init(&t_full[s], 1);
            sm100::mbar_init(&t_empty[s], 4);
        }
        sm100::mbar_init(&fin, 1);
        sm100::fence_mbar_init();
        sm100::prefetch_tmap(&tmapX);
    }
    if (warp == 0) {
        sm100::tmem_alloc(&tmem_base, 2 * AT_SLOT_COLS);
        sm100::tmem_relinquish();
    }
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = tmem_base;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {  // producer
            int64_t q = 0;
            int lt = 0;
            for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++lt) {
                if (lt > 0) ok = sm100::mbar_wait(&a_empty, (lt - 1) & 1, p.err);
                if (!ok) break;
                sm100::mbar_expect_tx(&a_full, (uint32_t)g.nch * 16384);
                for (int c = 0; c < g.nch; ++c)
                    sm100::tma_load_2d(Atile + (size_t)c * 16384, &tmapX, 64 * c, (int)(tile * AT_TILE), &a_full);
                for (int j = 0; j < p.k; ++j, ++q) {
                    const int s = (int)(q & 1), u = (int)(q >> 1);
                    if (u > 0) ok = sm100::mbar_wait(&b_empty[s], (u - 1) & 1, p.err);
                    if (!ok) break;
                    sm100::mbar_expect_tx(&b_full[s], (uint32_t)g.bsz);
                    sm100::bulk_load(Bslot + (size_t)s * g.bsz, p.B + (size_t)j * 8 * g.Lb, (uint32_t)g.bsz, &b_full[s]);
                }
            }
            // copies still in flight land before the CTA can exit: wait for the last
            // phase issued on each barrier (already complete on the normal path)
            if (lt > 0) sm100::mbar_wait(&a_full, (lt - 1) & 1, p.err);
            for (int s = 0; s < 2; ++s) {
                const int64_t uses = (q + 1 - s) / 2;  // loads issued into slot s
                if (uses > 0) sm100::mbar_wait(&b_full[s], (int)((uses - 1) & 1), p.err);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            const uint32_t ID = sm100::idesc(1, AT_TILE, g.NB);
            int64_t q = 0, w = 0;
            int lt = 0;
            for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++lt) {
                ok = sm100::mbar_wait(&a_full, lt & 1, p.err);
                if (!ok) break;
                sm100::tc_fence_after();
                for (int j = 0; j < p.k && ok; ++j, ++q) {
                    const int s = (int)(q & 1);
                    ok = sm100::mbar_wait(&b_full[s], (int)(q >> 1) & 1, p.err);
                    if (!ok) break;
                    sm100::tc_fence_after();
                    const uint8_t* Bs = Bslot + (size_t)s * g.bsz;
                    for (int gi = 0; gi < g.G && ok; ++gi, ++w) {
                        const int s2 = (int)(w & 1);
                        if (w >= 2) ok = sm100::mbar_wait(&t_empty[s2], (int)((w >> 1) - 1) & 1, p.err);
                        if (!ok) break;
                        sm100::tc_fence_after();
                        for (int bb = 0; bb < g.Gb; ++bb) {
                            const int b = gi * g.Gb + bb;
                            const uint32_t d = tmem + s2 * AT_SLOT_COLS + bb * g.NB;
                            const uint8_t* buf = Bs + (size_t)b * g.Lb * 2;
                            for (int kk = 0; kk < g.KS; ++kk) {
                                const uint64_t da = sm100::desc_k_sw128(Atile + (size_t)(kk >> 2) * 16384) + 2 * (kk & 3);
                                const uint64_t db = sm100::desc_k_none(buf + 32 * kk, 16, 128);
                                sm100::mma_f16(d, da, db, ID, kk > 0);
                            }
                        }
                        sm100::mma_commit(&t_full[s2]);
                    }
                    sm100::mma_commit(&b_empty[s]);
                }
                sm100::mma_commit(&a_empty);
            }
            // every MMA issued completes before TMEM is released
            sm100::mma_commit(&fin);
            sm100::mbar_wait(&fin, 0, p.err);
        }
        __syncwarp();
    } else {
        // epilogue: TMEM lane quarter warp%4 = series rows 32*(warp%4) + lane
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        double dsum = 0.0;
        int nchg = 0;
        int64_t w = 0;
        const int slot_chunks = (g.Gb * g.NB) / 32;
        for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
            const int64_t i = tile * AT_TILE + row;
            const float xn = i < p.n ? p.xnorm[i] : 0.f;
            float bestd = 1e10f;  // get_pos_idx: min_val = 1e10, pos = 0
            int bestj = 0;
            for (int j = 0; j < p.k && ok; ++j) {
                float mx = -3.0e38f;
                for (int gi = 0; gi < g.G && ok; ++gi, ++w) {
                    const int s2 = (int)(w & 1);
                    ok = __all_sync(0xffffffffu, sm100::mbar_wait(&t_full[s2], (int)(w >> 1) & 1, p.err));
                    if (!ok) break;
                    sm100::tc_fence_after();
                    for (int ch = 0; ch < slot_chunks; ++ch) {
                        float r[32];
                        sm100::tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + s2 * AT_SLOT_COLS + ch * 32, r);
                        sm100::tmem_ld_wait();
                        if (!p.mask) {
#pragma unroll
                            for (int e = 0; e < 32; ++e) mx = fmaxf(mx, r[e]);
                        } else {
#pragma unroll
                            for (int e = 0; e < 32; ++e) {
                                const int col = ch * 32 + e;
                                const int b = gi * g.Gb + (col >> g.lnb), nn = col & (g.NB - 1);
                                const int t = (b - 8 * nn) & (g.F - 1);  // lag of this column
                                if (t <= p.m - 1 || t >= g.F - p.m + 1) mx = fmaxf(mx, r[e]);
                            }
                        }
                    }
                    sm100::tc_fence_before();
                    __syncwarp();
                    if (lane == 0) sm100::mbar_arrive(&t_empty[s2]);
                }
                const float den = xn * p.cnorm[j];
                const float ncc = den > 0.f ? mx / den : 0.f;  // a zero norm gives NCC 0 (ncc.cuh:89)
                float d = 1.0f - ncc;
                if (p.clamp2 && d > 2.0f) d = 2.0f;
                if (d < bestd) {
                    bestd = d;
                    bestj = j;
                }
            }
            if (ok && i < p.n) {
                if (p.labels) p.labels[i] = bestj;
                if (p.dist) p.dist[i] = bestd;
                dsum += (double)bestd;
                if (p.old_labels && p.old_labels[i] != bestj) ++nchg;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
            nchg += __shfl_xor_sync(0xffffffffu, nchg, o);
        }
        if (lane == 0) {
            if (p.dist_sum) atomicAdd(p.dist_sum, dsum);
            if (p.changed && nchg) atomicAdd(p.changed, nchg);
        }
    }
    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 0) sm100::tmem_dealloc(tmem, 2 * AT_SLOT_COLS);
}

// ---------------------------------------------------------------- host
bool tc_assign_supported(int m, int F, int k, int precision) {
    return precision == TC_PREC_BF16 && m >= 2 && m <= 512 && F >= 128 && F <= 1024 && k >= 1;
}

void launch_assign_tc(tc_ctx* ctx, const AssignArgs& a, int precision, cudaStream_t s) {
    TC_REQUIRE(tc_assign_supported(a.m, a.F, a.k, precision), TC_ERR_UNSUPPORTED, "tensor-core correlation shape");
    if (a.n == 0) return;
    Workspace& ws = ctx->ws;
    const AtGeom g(a.m, a.F);
    TC_REQUIRE(g.smem() <= ctx->smem_optin, TC_ERR_UNSUPPORTED, "tensor-core correlation: shared memory");
    __nv_bfloat16* xb = ws.xbf.as<__nv_bfloat16>((size_t)a.n * g.mp);
    float* xnorm = ws.xbf_norm.as<float>((size_t)a.n);
    __nv_bfloat16* B = ws.toeplitz.as<__nv_bfloat16>((size_t)a.k * 8 * g.Lb);
    float* cnorm = ws.toeplitz_norm.as<float>((size_t)a.k);
    const int wgrid = (int)std::min<int64_t>(ceil_div(a.n, 8), (int64_t)ctx->sm_count * 16);
    k_series_bf16<<<wgrid, 256, 0, s>>>(a.x, a.n, a.m, g.mp, xb, xnorm);
    TC_CHECK_LAUNCH();
    k_centroid_toeplitz<<<a.k, 256, 0, s>>>(a.centroids, a.m, a.F, g.Lb, B, cnorm);
    TC_CHECK_LAUNCH();
    CUtensorMap map = make_tmap_2d(xb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)a.n, (uint64_t)g.mp, AT_TILE);
    int* err = reinterpret_cast<int*>(ws.aux.as<char>(64) + 52);
    TC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    AtParams p{};
    p.B = B;
    p.xnorm = xnorm;
    p.cnorm = cnorm;
    p.n = a.n;
    p.m = a.m;
    p.k = a.k;
    p.F = a.F;
    p.clamp2 = a.clamp2;
    p.mask = a.F >= 2 * a.m ? 1 : 0;  // lags m..F-m fall outside the 2m-1 valid ones
    p.labels = a.labels;
    p.dist = a.dist;
    p.old_labels = a.old_labels;
    p.changed = a.changed;
    p.dist_sum = a.dist_sum;
    p.err = err;
    const size_t smem = g.smem();
    TC_CUDA(cudaFuncSetAttribute(k_assign_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t ntiles = (a.n + AT_TILE - 1) / AT_TILE;
    const int grid = (int)std::min<int64_t>(ntiles, ctx->sm_count);
    k_assign_tc<<<grid, AT_THREADS, smem, s>>>(map, p);
    TC_CHECK_LAUNCH();
    int h_err = 0;
    TC_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaStreamSynchronize(s));
    TC_REQUIRE(h_err == 0, TC_ERR_TIMEOUT, "tensor-core correlation: a pipeline wait ran out");
}

}  // namespace tc
