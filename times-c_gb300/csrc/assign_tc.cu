// SBD assignment on the tensor cores (tcgen05, BF16 operands, FP32 accumulation):
// the mixed-precision form of NCC_3D + get_pos_idx (ncc.cuh:469-517,
// kshape.cuh:35-96) for series of up to 512 samples.
//
// The circular correlation at lag t of the zero-padded length F is
//   r[t] = sum_{u < m} x[u] * c_pad[(u - t) mod F],
// a GEMM of the series (M = series, K = samples) with a Toeplitz matrix
// (N = lags).  The Toeplitz operand is never built.  A K-major, no-swizzle UMMA
// descriptor reads 8-row core matrices whose rows are 16 bytes (8 elements)
// apart; with LBO = 16 bytes, row r of a core matrix reads q = 8r + u of one
// buffer, and SBO (the distance between 8-row groups) is set to the length of
// a buffer, so each 8-row group reads its own buffer.  Buffer G holds the
// centroid shifted by T_G = 64 (G / 8) + G % 8, buf_G[q] = c_pad[(q - T_G) mod F],
// and its rows give the 8 lags T_G - 8r; the F/8 buffers cover every lag once.
// One MMA takes 32 buffers: N = 256 lags per instruction (F/8 buffers, N = F,
// when F = 128), the shape at which the tensor core runs at full rate.
//
// Persistent, warp-specialised CTA (192 threads), one per SM:
//   warp 0  producer: TMA of a 128-series BF16 tile (resident in shared memory
//           for all centroids) and bulk copies of 32-buffer groups into a
//           two-stage ring;
//   warp 1  one thread issues M=128, N=256, K=16 MMAs into two 256-column TMEM
//           accumulator slots, so MMAs fill one slot while the epilogue drains
//           the other;
//   warps 2-5 epilogue: tcgen05.ld of the row's 256 lags, max over valid lags,
//           NCC = max / (|x||c|) with FP32 norms of the unrounded data, and the
//           running argmin over centroids - only (label, distance) reach HBM.
// All waits are bounded and report through an error word.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
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
    int m, mp, F, NBT, CPG, NG, H, KS, Lq, gsz, nch;
    // mp: padded K (multiple of 64); NBT = F/8 shifted buffers per centroid; CPG
    // buffers per MMA group, NG = 8*CPG lags per MMA (N), H groups per centroid;
    // KS = mp/16 K steps; Lq = elements per buffer (reads reach 8*7 + mp - 1);
    // gsz = bytes of one group; nch = 64-column chunks of the series tile
    __host__ __device__ AtGeom(int m_, int F_) : m(m_), F(F_) {
        mp = (m + 63) / 64 * 64;
        NBT = F / 8;
        CPG = NBT < 32 ? NBT : 32;
        NG = 8 * CPG;
        H = NBT / CPG;
        KS = mp / 16;
        Lq = mp + 56;
        gsz = CPG * Lq * 2;
        nch = mp / 64;
    }
    // at least 116 KB so that one CTA (and one 512-column TMEM allocation) fits an SM
    size_t smem() const {
        const size_t s = (size_t)nch * 16384 + 2 * (size_t)gsz + 1024;
        return s > 116 * 1024 ? s : 116 * 1024;
    }
};

// lag of buffer G's row r: T_G - 8r (mod F)
__host__ __device__ inline int at_lag(int G, int r, int F) { return (64 * (G >> 3) + (G & 7) - 8 * r) & (F - 1); }

// Series -> BF16 [n][mp] (zero padded) and FP32 norms (compensated), one warp
// per row; V4: rows of float4 (m % 4 == 0 and a 16-byte aligned base).
template <bool V4>
__global__ void k_series_bf16(const float* __restrict__ x, int64_t n, int m, int mp, __nv_bfloat16* __restrict__ xb,
                              float* __restrict__ xnorm) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < n; i += nw) {
        const float* r = x + (size_t)i * m;
        __nv_bfloat16* o = xb + (size_t)i * mp;
        float s = 0.f, c = 0.f;
        auto acc = [&](float v) {
            const float y = v * v - c, tt = s + y;
            c = (tt - s) - y;
            s = tt;
        };
        if constexpr (V4) {
            for (int t = lane; t < mp / 4; t += 32) {
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (4 * t < m) v = __ldg(reinterpret_cast<const float4*>(r) + t);
                acc(v.x);
                acc(v.y);
                acc(v.z);
                acc(v.w);
                __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
                uint2 pk;
                pk.x = *reinterpret_cast<uint32_t*>(&lo);
                pk.y = *reinterpret_cast<uint32_t*>(&hi);
                reinterpret_cast<uint2*>(o)[t] = pk;
            }
        } else {
            for (int t = lane; t < mp; t += 32) {
                const float v = t < m ? r[t] : 0.f;
                o[t] = __float2bfloat16_rn(v);
                acc(v);
            }
        }
        double d = (double)s - (double)c;
#pragma unroll
        for (int q = 16; q > 0; q >>= 1) d += __shfl_xor_sync(0xffffffffu, d, q);
        if (lane == 0) xnorm[i] = (float)sqrt(d);
    }
}

// Centroid j -> F/8 shifted BF16 buffers buf_G[q] = c_pad[(q - T_G) mod F], q < Lq,
// and its norm.
__global__ void k_centroid_toeplitz(const float* __restrict__ C, int m, int F, int Lq,
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
    const int nb = F / 8;
    __nv_bfloat16* o = B + (size_t)j * nb * Lq;
    for (int e = threadIdx.x; e < nb * Lq; e += blockDim.x) {
        const int G = e / Lq, q = e % Lq;
        const int u = (q - at_lag(G, 0, F)) & (F - 1);
        o[e] = __float2bfloat16_rn(u < m ? c[u] : 0.f);
    }
}

struct AtParams {
    const __nv_bfloat16* B;  // [k][F/8][Lq] shifted buffers
    const float* xnorm;
    const float* cnorm;
    int64_t n;
    int m, k, F, clamp2;
    int32_t* labels;
    float* dist;
    const int32_t* old_labels;
    int32_t* changed;
    double* dist_sum;
    int* err;
    // screening (labels etc. unused): per series the centroids with d <= best + thr,
    // ascending, at most SCREEN_CAP (count -1: more, evaluate all)
    int32_t* cand;
    int32_t* ncand;
    float thr;
    // lower bounds d - lb_d16 on the exact distance of every pair, [n][k] (or null)
    float* lb_out;
    float lb_d16;
    // per series: an upper bound (best + lb_d16) on the exact distance of its best
    // centroid, and that centroid (the bounded BF16 pass reads and rewrites them)
    float* ubd;
    int32_t* jb;
    // per series best * k + second best (the group key of the next grouping)
    int32_t* gkey;
    unsigned long long* moved;  // series whose best centroid differs from jb's old value
    // tile-bounded pass: the tiles hold cluster-grouped positions (perm maps a position
    // to its series, for the outputs and bounds); only the centroids of tmask[tile]
    // are evaluated, and the other bounds of the tile's series are carried down by
    // delta (in place in lb_out)
    const unsigned long long* tmask;
    const int32_t* perm;
    const float* delta;
    unsigned long long* evals;  // (tile, centroid) pairs evaluated
};

// The centroids a tile evaluates, in ascending order: all k, or (tile-bounded pass,
// k <= 64) the bits of its mask.  next_centroid(p, mask, -1) is the first; p.k ends.
__device__ __forceinline__ unsigned long long tile_mask(const AtParams& p, int64_t tile) {
    return p.tmask ? p.tmask[tile] : 0ull;
}
__device__ __forceinline__ int next_centroid(const AtParams& p, unsigned long long mask, int j) {
    if (!p.tmask) return j + 1;
    const unsigned long long rest = j + 1 >= 64 ? 0ull : mask >> (j + 1);
    return rest ? j + __ffsll((long long)rest) : p.k;
}

// Keep the list entries with distance <= lim (NaN kept), in order; returns the count.
// Unrolled with constant indices so the lists stay in registers.
__device__ __forceinline__ int screen_compact(int (&cj)[SCREEN_CAP], float (&cd)[SCREEN_CAP], int nc, float lim) {
    int w = 0;
#pragma unroll
    for (int t = 0; t < SCREEN_CAP; ++t) {
        const bool keep = t < nc && !(cd[t] > lim);
#pragma unroll
        for (int u = 0; u <= t; ++u)
            if (keep && u == w) {
                cj[u] = cj[t];
                cd[u] = cd[t];
            }
        w += keep ? 1 : 0;
    }
    return w;
}

__global__ void __launch_bounds__(AT_THREADS, 1) k_assign_tc(const __grid_constant__ CUtensorMap tmapX, AtParams p) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t a_full, a_empty, b_full[2], b_empty[2], t_full[2], t_empty[2], fin;
    __shared__ uint32_t tmem_base;
    __shared__ uint32_t lagmask[32];  // valid-lag bits per (group, 32-column chunk)
    const AtGeom g(p.m, p.F);
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* Atile = base;                                    // nch x 16 KB, 128B-swizzled K-major
    uint8_t* Bring = base + (size_t)g.nch * 16384;            // 2 x gsz
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
    if (threadIdx.x < 32) {
        // column col of group h is row col of the MMA: buffer h*CPG + col/8, row col%8.
        // Valid lags are t <= m-1 and t >= F-m+1 (all of them when F <= 2m-1).
        const int h = threadIdx.x >> 3, ch = threadIdx.x & 7;
        uint32_t bits = 0;
        for (int e = 0; e < 32; ++e) {
            const int col = ch * 32 + e;
            const int t = at_lag(h * g.CPG + (col >> 3), col & 7, g.F);
            if (col < g.NG && (t <= p.m - 1 || t >= g.F - p.m + 1)) bits |= 1u << e;
        }
        lagmask[threadIdx.x] = bits;
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
            const size_t cent = (size_t)g.NBT * g.Lq;  // elements per centroid
            for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++lt) {
                if (lt > 0) ok = sm100::mbar_wait(&a_empty, (lt - 1) & 1, p.err);
                if (!ok) break;
                sm100::mbar_expect_tx(&a_full, (uint32_t)g.nch * 16384);
                for (int c = 0; c < g.nch; ++c)
                    sm100::tma_load_2d(Atile + (size_t)c * 16384, &tmapX, 64 * c, (int)(tile * AT_TILE), &a_full);
                const unsigned long long tmask = tile_mask(p, tile);
                for (int j = next_centroid(p, tmask, -1); j < p.k && ok; j = next_centroid(p, tmask, j)) {
                    for (int h = 0; h < g.H; ++h, ++q) {
                        const int s = (int)(q & 1), u = (int)(q >> 1);
                        if (u > 0) ok = sm100::mbar_wait(&b_empty[s], (u - 1) & 1, p.err);
                        if (!ok) break;
                        sm100::mbar_expect_tx(&b_full[s], (uint32_t)g.gsz);
                        sm100::bulk_load(Bring + (size_t)s * g.gsz, p.B + j * cent + (size_t)h * g.CPG * g.Lq,
                                         (uint32_t)g.gsz, &b_full[s]);
                    }
                }
            }
            // copies still in flight land before the CTA can exit: wait for the last
            // phase issued on each barrier (already complete on the normal path)
            if (lt > 0) sm100::mbar_wait(&a_full, (lt - 1) & 1, p.err);
            for (int s = 0; s < 2; ++s) {
                const int64_t uses = (q + 1 - s) / 2;  // loads issued into stage s
                if (uses > 0) sm100::mbar_wait(&b_full[s], (int)((uses - 1) & 1), p.err);
            }
            // likewise the MMA thread's last commits (they arrive when their MMAs end):
            // no arrival may land in this CTA's shared memory after it has left, when
            // another kernel's CTA may own it
            if (ok) {
                for (int s = 0; s < 2; ++s) {
                    const int64_t uses = (q + 1 - s) / 2;
                    if (uses > 0) sm100::mbar_wait(&b_empty[s], (int)((uses - 1) & 1), p.err);
                }
                if (lt > 0) sm100::mbar_wait(&a_empty, (lt - 1) & 1, p.err);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            const uint32_t ID = sm100::idesc(1, AT_TILE, g.NG);
            // descriptors advance by adding to their 14-bit address field (bytes >> 4):
            // +2 per 16 K elements, +1024 per 16 KB A chunk, gsz/16 per ring stage
            const uint64_t da0 = sm100::desc_k_sw128(Atile);
            const uint64_t db0 = sm100::desc_k_none(Bring, 16, (uint32_t)g.Lq * 2);
            int64_t q = 0;
            int lt = 0;
            for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++lt) {
                ok = sm100::mbar_wait(&a_full, lt & 1, p.err);
                if (!ok) break;
                sm100::tc_fence_after();
                const unsigned long long tmask = tile_mask(p, tile);
                for (int j = next_centroid(p, tmask, -1); j < p.k && ok; j = next_centroid(p, tmask, j))
                    for (int h = 0; h < g.H; ++h, ++q) {
                        // ring stage and accumulator slot both follow the group counter
                        const int s = (int)(q & 1);
                        ok = sm100::mbar_wait(&b_full[s], (int)(q >> 1) & 1, p.err);
                        if (ok && q >= 2) ok = sm100::mbar_wait(&t_empty[s], (int)((q >> 1) - 1) & 1, p.err);
                        if (!ok) break;
                        sm100::tc_fence_after();
                        const uint32_t d = tmem + s * AT_SLOT_COLS;
                        const uint64_t db = db0 + (uint64_t)((s * g.gsz) >> 4);
                        for (int kc = 0; kc < g.nch; ++kc) {
                            const uint64_t da = da0 + (uint64_t)(kc * 1024);
#pragma unroll
                            for (int u = 0; u < 4; ++u)
                                sm100::mma_f16(d, da + 2 * u, db + 2 * (4 * kc + u), ID, (kc | u) != 0);
                        }
                        sm100::mma_commit(&t_full[s]);
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
        const uint32_t tq = tmem + ((uint32_t)(quarter * 32) << 16);
        const int nchunk = g.NG / 32;  // 4 or 8
        double dsum = 0.0;
        int nchg = 0, nmov = 0;
        int64_t q = 0;
        for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
            const int64_t pos = tile * AT_TILE + row;  // the tile row (a series position)
            const int64_t i = pos < p.n ? (p.perm ? (int64_t)p.perm[pos] : pos) : pos;  // its series
            const float xn = pos < p.n ? p.xnorm[pos] : 0.f;
            const unsigned long long tmask = tile_mask(p, tile);
            if (p.evals && p.tmask && warp == 2 && lane == 0)
                atomicAdd(p.evals, (unsigned long long)__popcll((long long)tmask));
            float bestd = 1e10f;  // get_pos_idx: min_val = 1e10, pos = 0
            int bestj = 0;
            float secd = 1e10f;  // the second best (group key of a full pass)
            int secj = 0;
            int cj[SCREEN_CAP];
            float cd[SCREEN_CAP];
#pragma unroll
            for (int t = 0; t < SCREEN_CAP; ++t) {
                cj[t] = 0;
                cd[t] = 0.f;
            }
            int nc = 0;  // -1: the list overflowed
            for (int j = next_centroid(p, tmask, -1); j < p.k && ok; j = next_centroid(p, tmask, j)) {
                float mx = -3.0e38f;
                for (int h = 0; h < g.H && ok; ++h, ++q) {
                    const int s = (int)(q & 1);
                    ok = __all_sync(0xffffffffu, sm100::mbar_wait(&t_full[s], (int)(q >> 1) & 1, p.err));
                    if (!ok) break;
                    sm100::tc_fence_after();
                    for (int c0 = 0; c0 < nchunk; c0 += 4) {
                        float r[4][32];
#pragma unroll
                        for (int ch = 0; ch < 4; ++ch)
                            sm100::tmem_ld32(tq + s * AT_SLOT_COLS + (c0 + ch) * 32, r[ch]);
                        sm100::tmem_ld_wait();
                        if (c0 + 4 >= nchunk) {  // the slot is free once its last columns are in registers
                            sm100::tc_fence_before();
                            __syncwarp();
                            if (lane == 0) sm100::mbar_arrive(&t_empty[s]);
                        }
#pragma unroll
                        for (int ch = 0; ch < 4; ++ch) {
                            const uint32_t vm = lagmask[h * 8 + c0 + ch];  // bit e: column valid
                            float m0 = -3.0e38f, m1 = -3.0e38f;
#pragma unroll
                            for (int e = 0; e < 32; e += 2) {
                                m0 = fmaxf(m0, (vm >> e) & 1u ? r[ch][e] : -3.0e38f);
                                m1 = fmaxf(m1, (vm >> (e + 1)) & 1u ? r[ch][e + 1] : -3.0e38f);
                            }
                            mx = fmaxf(mx, fmaxf(m0, m1));
                        }
                    }
                }
                const float den = xn * p.cnorm[j];
                const float ncc = den > 0.f ? mx / den : 0.f;  // a zero norm gives NCC 0 (ncc.cuh:89)
                float d = 1.0f - ncc;
                if (p.clamp2 && d > 2.0f) d = 2.0f;
                if (p.lb_out && pos < p.n) p.lb_out[(size_t)i * p.k + j] = __fsub_rd(d, p.lb_d16);
                if (d < bestd) {
                    secd = bestd;
                    secj = bestj;
                    bestd = d;
                    bestj = j;
                } else if (d < secd) {
                    secd = d;
                    secj = j;
                }
                if (p.cand && nc >= 0 && !(d > bestd + p.thr)) {
                    if (nc == SCREEN_CAP) nc = screen_compact(cj, cd, nc, bestd + p.thr);
                    if (nc == SCREEN_CAP) {
                        nc = -1;
                    } else {
#pragma unroll
                        for (int t = 0; t < SCREEN_CAP; ++t)
                            if (t == nc) {
                                cj[t] = j;
                                cd[t] = d;
                            }
                        ++nc;
                    }
                }
            }
            if (ok && pos < p.n) {
                if (p.tmask) {  // the centroids the tile skipped: bounds carried down
                    float* lr = p.lb_out + (size_t)i * p.k;
                    const unsigned long long all = p.k >= 64 ? ~0ull : ((1ull << p.k) - 1ull);
                    const unsigned long long skipm = all & ~tmask;
                    if ((p.k & 3) == 0) {
                        // the row as float4s (rows are 16-byte aligned), 8 at a time: every
                        // load of a batch is issued before its updates, instead of one
                        // dependent read-modify-write per skipped centroid
                        float4* l4 = reinterpret_cast<float4*>(lr);
                        const int n4 = p.k >> 2;
                        for (int b0 = 0; b0 < n4; b0 += 8) {
                            float4 v[8];
#pragma unroll
                            for (int e = 0; e < 8; ++e)
                                if (b0 + e < n4 && ((skipm >> (4 * (b0 + e))) & 0xFull)) v[e] = l4[b0 + e];
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                const int q4 = b0 + e;
                                const unsigned bits = q4 < n4 ? (unsigned)(skipm >> (4 * q4)) & 0xFu : 0u;
                                if (!bits) continue;
                                const float* dl = p.delta + 4 * q4;
                                if (bits & 1u) v[e].x = __fsub_rd(v[e].x, __ldg(dl));
                                if (bits & 2u) v[e].y = __fsub_rd(v[e].y, __ldg(dl + 1));
                                if (bits & 4u) v[e].z = __fsub_rd(v[e].z, __ldg(dl + 2));
                                if (bits & 8u) v[e].w = __fsub_rd(v[e].w, __ldg(dl + 3));
                                l4[q4] = v[e];
                            }
                        }
                    } else {
                        for (unsigned long long mk = skipm; mk; mk &= mk - 1) {
                            const int j = __ffsll((long long)mk) - 1;
                            lr[j] = __fsub_rd(lr[j], __ldg(p.delta + j));
                        }
                    }
                }
                if (p.ubd) {
                    if (p.moved && p.jb[i] != bestj) ++nmov;
                    p.ubd[i] = __fadd_ru(bestd, p.lb_d16);
                    p.jb[i] = bestj;
                }
                if (p.gkey) p.gkey[i] = bestj * p.k + secj;
                if (p.cand) {
                    if (nc >= 0) nc = screen_compact(cj, cd, nc, bestd + p.thr);
                    int4* o = reinterpret_cast<int4*>(p.cand + (size_t)i * SCREEN_CAP);
                    o[0] = make_int4(cj[0], cj[1], cj[2], cj[3]);
                    o[1] = make_int4(cj[4], cj[5], cj[6], cj[7]);
                    p.ncand[i] = nc;
                } else {
                    if (p.labels) p.labels[i] = bestj;
                    if (p.dist) p.dist[i] = bestd;
                    dsum += (double)bestd;
                    if (p.old_labels && p.old_labels[i] != bestj) ++nchg;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
            nchg += __shfl_xor_sync(0xffffffffu, nchg, o);
            nmov += __shfl_xor_sync(0xffffffffu, nmov, o);
        }
        if (lane == 0) {
            if (p.dist_sum) atomicAdd(p.dist_sum, dsum);
            if (p.changed && nchg) atomicAdd(p.changed, nchg);
            if (p.moved && nmov) atomicAdd(p.moved, (unsigned long long)nmov);
        }
    }
    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 0) sm100::tmem_dealloc(tmem, 2 * AT_SLOT_COLS);
}

// ---------------------------------------------------------------- tile-bounded BF16 pass
// The series are grouped by the centroid they were last assigned (jb), so that a
// 128-row tile mostly shares one best centroid and few others can come near it; a
// tile evaluates a centroid only if one of its series' bounds allows it.  Within a
// group the order follows the atomics (any order gives the same results).

// a stored best centroid, kept inside [0, k) whatever the buffer holds
__device__ __forceinline__ int group_of(int j, int k) { return (j >= 0 && j < k) ? j : 0; }

// per-key counts: block histogram in shared memory, one global add per key
__global__ void k_group_count(const int32_t* __restrict__ key, int64_t n, int nb, int32_t* __restrict__ cnt) {
    extern __shared__ int32_t hist[];
    for (int j = threadIdx.x; j < nb; j += blockDim.x) hist[j] = 0;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&hist[group_of(key[i], nb)], 1);
    __syncthreads();
    for (int j = threadIdx.x; j < nb; j += blockDim.x)
        if (hist[j]) atomicAdd(&cnt[j], hist[j]);
}

// cursor[j] = start of group j (exclusive scan of the counts; one block, chunks of
// 1024 keys scanned in shared memory)
__global__ void __launch_bounds__(1024) k_group_offsets(const int32_t* __restrict__ cnt, int nb,
                                                        int32_t* __restrict__ cursor) {
    __shared__ int32_t buf[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    for (int b0 = 0; b0 < nb; b0 += 1024) {
        const int j = b0 + threadIdx.x;
        const int v = j < nb ? cnt[j] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
            const int add = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += add;
            __syncthreads();
        }
        if (j < nb) cursor[j] = carry + buf[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += buf[1023];
        __syncthreads();
    }
}

// perm[position] = series: each block reserves a range per key, then places its series
__global__ void k_group_scatter(const int32_t* __restrict__ key, int64_t n, int nb, int32_t* __restrict__ cursor,
                                int32_t* __restrict__ perm) {
    extern __shared__ int32_t hist[];  // [nb] counts, then [nb] reserved starts
    for (int j = threadIdx.x; j < 2 * nb; j += blockDim.x) hist[j] = 0;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int lab = 0, rank = 0;
    if (i < n) {
        lab = group_of(key[i], nb);
        rank = atomicAdd(&hist[lab], 1);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nb; j += blockDim.x)
        if (hist[j]) hist[nb + j] = atomicAdd(&cursor[j], hist[j]);
    __syncthreads();
    if (i < n) perm[hist[nb + lab] + rank] = (int32_t)i;
}

// the BF16 rows and norms in position order (one warp per row, 16-byte copies)
__global__ void k_permute_bf16(const __nv_bfloat16* __restrict__ xb, const float* __restrict__ xnorm,
                               const int32_t* __restrict__ perm, int64_t n, int mp, __nv_bfloat16* __restrict__ xbp,
                               float* __restrict__ normp) {
    const int lane = threadIdx.x & 31;
    const int64_t pos = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (pos >= n) return;
    const int64_t i = perm[pos];
    const int4* src = reinterpret_cast<const int4*>(xb + (size_t)i * mp);
    int4* dst = reinterpret_cast<int4*>(xbp + (size_t)pos * mp);
    for (int e = lane; e < mp / 8; e += 32) dst[e] = __ldg(src + e);
    if (lane == 0) normp[pos] = xnorm[i];
}

// tmask[tile]: the centroids some series of the tile may have as its minimum.  For
// series i with best centroid j0, ub = ubd + delta[j0] + D bounds its new BF16
// distance to j0 from above; centroid j is left out only if lb - delta[j] - D > ub,
// i.e. its BF16 distance is certainly larger.  j0 is always in.
__global__ void __launch_bounds__(128) k_tile_masks(const int32_t* __restrict__ perm, const float* __restrict__ lb,
                                                    const float* __restrict__ ubd, const int32_t* __restrict__ jb,
                                                    const float* __restrict__ delta, float D, int64_t n, int k,
                                                    unsigned long long* __restrict__ tmask,
                                                    unsigned long long* __restrict__ series_pairs) {
    __shared__ unsigned long long part[4];
    const int64_t pos = (int64_t)blockIdx.x * 128 + threadIdx.x;
    unsigned long long mask = 0;
    if (pos < n) {
        const int64_t i = perm[pos];
        const int j0 = group_of(jb[i], k);
        const float ub = __fadd_ru(__fadd_ru(ubd[i], __ldg(delta + j0)), D);
        mask = 1ull << j0;
        const float* lr = lb + (size_t)i * k;
        auto test = [&](int j, float b) {
            const float l = __fsub_rd(__fsub_rd(b, __ldg(delta + j)), D);
            if (!(l > ub)) mask |= 1ull << j;
        };
        if ((k & 3) == 0) {  // the row as float4s, all loads issued before the tests (rows are 16-byte aligned)
            const float4* l4 = reinterpret_cast<const float4*>(lr);
            for (int j = 0; j < k; j += 32) {
                float4 v[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (j + 4 * q < k) v[q] = __ldg(l4 + j / 4 + q);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (j + 4 * q < k) {
                        test(j + 4 * q, v[q].x);
                        test(j + 4 * q + 1, v[q].y);
                        test(j + 4 * q + 2, v[q].z);
                        test(j + 4 * q + 3, v[q].w);
                    }
            }
        } else {
            for (int j = 0; j < k; ++j) test(j, lr[j]);
        }
    }
    if (series_pairs) {  // the pairs the series themselves need (what a per-series pass would evaluate)
        const unsigned c = __reduce_add_sync(0xffffffffu, (unsigned)__popcll((long long)mask));
        if ((threadIdx.x & 31) == 0 && c) atomicAdd(series_pairs, (unsigned long long)c);
    }
    const unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)mask);
    const unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(mask >> 32));
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = ((unsigned long long)hi << 32) | lo;
    __syncthreads();
    if (threadIdx.x == 0) tmask[blockIdx.x] = part[0] | part[1] | part[2] | part[3];
}

// The grouped layout in the workspace: positions -> series, and the BF16 rows and
// norms in position order.
static TileBounds tile_layout(tc_ctx* ctx, int64_t n, int m, int k) {
    Workspace& ws = ctx->ws;
    const int mp = (m + 63) / 64 * 64;
    TileBounds t;
    t.perm = ws.bperm.as<int32_t>((size_t)n + 2 * (size_t)k * k);  // + group counts and cursors
    char* xp = static_cast<char*>(ws.xbfp.get((size_t)n * mp * 2 + (size_t)n * 4 + 16));
    t.xbf = xp;
    t.xbf_norm = reinterpret_cast<const float*>(xp + (size_t)n * mp * 2);
    t.tmask = ws.tmask.as<unsigned long long>((size_t)((n + AT_TILE - 1) / AT_TILE));
    return t;
}

void launch_tile_group(tc_ctx* ctx, int64_t n, int m, int k, const int32_t* gkey, cudaStream_t s) {
    Workspace& ws = ctx->ws;
    const int mp = (m + 63) / 64 * 64;
    const TileBounds t = tile_layout(ctx, n, m, k);
    const int nb = k * k;  // groups: (best, second best)
    int32_t* perm = const_cast<int32_t*>(t.perm);
    int32_t* cnt = perm + n;
    int32_t* cursor = cnt + nb;
    __nv_bfloat16* xbp = static_cast<__nv_bfloat16*>(const_cast<void*>(t.xbf));
    float* normp = const_cast<float*>(t.xbf_norm);
    const __nv_bfloat16* xb = ws.xbf.as<__nv_bfloat16>((size_t)n * mp);
    const float* xnorm = ws.xbf_norm.as<float>((size_t)n);
    TC_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * nb, s));
    const int gb = ceil_div(n, 1024);
    k_group_count<<<gb, 1024, sizeof(int32_t) * nb, s>>>(gkey, n, nb, cnt);
    TC_CHECK_LAUNCH();
    k_group_offsets<<<1, 1024, 0, s>>>(cnt, nb, cursor);
    TC_CHECK_LAUNCH();
    k_group_scatter<<<gb, 1024, sizeof(int32_t) * 2 * nb, s>>>(gkey, n, nb, cursor, perm);
    TC_CHECK_LAUNCH();
    k_permute_bf16<<<ceil_div(n * 32, 256), 256, 0, s>>>(xb, xnorm, perm, n, mp, xbp, normp);
    TC_CHECK_LAUNCH();
}

void launch_tile_masks(tc_ctx* ctx, int64_t n, int m, int k, const float* lb, const float* ubd, const int32_t* jb,
                       const float* delta, float D, TileBounds& out, cudaStream_t s,
                       unsigned long long* series_pairs) {
    out = tile_layout(ctx, n, m, k);
    const int64_t ntiles = (n + AT_TILE - 1) / AT_TILE;
    k_tile_masks<<<(unsigned)ntiles, 128, 0, s>>>(out.perm, lb, ubd, jb, delta, D, n, k,
                                                  const_cast<unsigned long long*>(out.tmask), series_pairs);
    TC_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- host
void prepare_series_bf16_reserve(tc_ctx* ctx, int64_t n, int m) {
    const int mp = (m + 63) / 64 * 64;
    ctx->ws.xbf.as<__nv_bfloat16>((size_t)n * mp);
    ctx->ws.xbf_norm.as<float>((size_t)n);
    ctx->prep_x = nullptr;
}

void prepare_series_bf16_rows(tc_ctx* ctx, const float* x, int64_t n, int m, int64_t r0, int64_t rows,
                              cudaStream_t s) {
    const int mp = (m + 63) / 64 * 64;
    __nv_bfloat16* xb = ctx->ws.xbf.as<__nv_bfloat16>((size_t)n * mp) + (size_t)r0 * mp;
    float* xnorm = ctx->ws.xbf_norm.as<float>((size_t)n) + r0;
    const float* xr = x + (size_t)r0 * m;
    if (rows <= 0) return;
    const int wgrid = (int)std::min<int64_t>(ceil_div(rows, 8), (int64_t)ctx->sm_count * 16);
    if (m % 4 == 0 && reinterpret_cast<uintptr_t>(xr) % 16 == 0)
        k_series_bf16<true><<<wgrid, 256, 0, s>>>(xr, rows, m, mp, xb, xnorm);
    else
        k_series_bf16<false><<<wgrid, 256, 0, s>>>(xr, rows, m, mp, xb, xnorm);
    TC_CHECK_LAUNCH();
}

void prepare_series_bf16_done(tc_ctx* ctx, const float* x, int64_t n, int m) {
    ctx->prep_x = x;
    ctx->prep_n = n;
    ctx->prep_m = m;
    ctx->bounds.valid = false;  // new series contents: bounds on old distances no longer hold
    memo_invalidate(ctx);       // and the extraction memo's outputs neither
}

void prepare_series_bf16(tc_ctx* ctx, const float* x, int64_t n, int m, cudaStream_t s) {
    prepare_series_bf16_reserve(ctx, n, m);
    prepare_series_bf16_rows(ctx, x, n, m, 0, n, s);
    prepare_series_bf16_done(ctx, x, n, m);
}

bool tc_assign_supported(int m, int F, int k, int precision) {
    return precision == TC_PREC_BF16 && m >= 2 && m <= 512 && F >= 128 && F <= 1024 && k >= 1;
}

bool screen_supported(int m, int F, int k) {
    return !std::getenv("TIMESC_NO_SCREEN") && k >= 2 && tc_assign_supported(m, F, k, TC_PREC_BF16);
}

// Bound on |d_BF16 - d_FP32| for one (series, centroid) pair.  With x~ = x(1+e1),
// c~ = c(1+e2), |e| <= 2^-9 (BF16 rounding), every lag's |x~.c~ - x.c| <= (2^-8 + 2^-18)
// sum |x_i c_j| <= (2^-8 + 2^-18) |x||c| (Cauchy-Schwarz); the norms are FP32 in both
// kernels.  Allowances: the tensor cores' FP32 accumulation over mp terms (mp * 2^-21,
// with room for truncating adders) and the FP32 FFT kernel's own error (fft_error).  A
// max over lags and the clamp at 2 do not widen it.  If d32(j*) is the FP32 minimum and
// d16(jb) the BF16 one, d16(j*) <= d32(j*) + D <= d32(jb) + D <= d16(jb) + 2D: every
// centroid that can be the FP32 first minimum (ties included) has d16 <= min d16 + 2D.
//
// fft_error: a worst-case bound on one lag of the FP32 FFT correlation of unit-norm x
// and c.  Per transform of length F, the computed spectrum satisfies
// |y^ - y|_2 <= L eta |y|_2 (1 + O(L eta)), L = log2 F, eta = mu + gamma_4 (sqrt 2 + mu),
// gamma_4 = 4u/(1 - 4u), u = 2^-24, mu the twiddles' error (<= 2^-24: FP64 sincospi
// rounded to float) - the radix-2 result of Higham, Accuracy and Stability of Numerical
// Algorithms (2nd ed.), Thm 24.2, taken per level (a radix-4 or radix-8 pass counts as
// two or three levels).  |X|_2 = sqrt(F) for the series, |C|_inf <= |c|_1 <= sqrt(m) for
// the centroid, so the errors of the two forward transforms and of the product
// (sqrt 2 gamma_2 per bin) reach the correlation as at most (2 L eta + 3u) sqrt(m) in
// 2-norm after the 1/F-scaled inverse, whose own error adds L eta |r|_2 <= L eta sqrt(m)
// (|r|_2 <= |x|_1 |c|_2 <= sqrt(m), Young).  A lag's error is at most the 2-norm; the
// bound is doubled for the normalisation's few roundings and the O(L eta) terms.
double fft_error(int m, int F) {
    const double u = std::ldexp(1.0, -24), g4 = 4 * u / (1 - 4 * u);
    const double eta = u + g4 * (std::sqrt(2.0) + u);
    const double L = std::log2((double)F);
    return 2.0 * (3.0 * L * eta + 3.0 * u) * std::sqrt((double)m);
}

double bf16_error(int m, int F) {
    const int mp = (m + 63) / 64 * 64;
    return std::ldexp(1.0, -8) + std::ldexp(1.0, -18) + mp * std::ldexp(1.0, -21) + fft_error(m, F);
}

static float screen_threshold(int m, int F) { return (float)(2.0 * bf16_error(m, F) * (1.0 + 1e-3)); }

void launch_assign_tc(tc_ctx* ctx, const AssignArgs& a, int precision, cudaStream_t s) {
    TC_REQUIRE(tc_assign_supported(a.m, a.F, a.k, precision), TC_ERR_UNSUPPORTED, "tensor-core correlation shape");
    if (a.n == 0) return;
    Workspace& ws = ctx->ws;
    const AtGeom g(a.m, a.F);
    TC_REQUIRE(g.smem() <= ctx->smem_optin, TC_ERR_UNSUPPORTED, "tensor-core correlation: shared memory");
    if (!(ctx->prep_x == a.x && ctx->prep_n == a.n && ctx->prep_m == a.m)) {
        prepare_series_bf16(ctx, a.x, a.n, a.m, s);
        ctx->prep_x = nullptr;  // converted for this call only: the caller may change x
    }
    const __nv_bfloat16* xb = a.xbf ? static_cast<const __nv_bfloat16*>(a.xbf)
                                    : ws.xbf.as<__nv_bfloat16>((size_t)a.n * g.mp);
    const float* xnorm = a.xbf ? a.xbf_norm : ws.xbf_norm.as<float>((size_t)a.n);
    __nv_bfloat16* B = ws.toeplitz.as<__nv_bfloat16>((size_t)a.k * g.NBT * g.Lq);
    float* cnorm = ws.toeplitz_norm.as<float>((size_t)a.k);
    k_centroid_toeplitz<<<a.k, 256, 0, s>>>(a.centroids, a.m, a.F, g.Lq, B, cnorm);
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
    p.labels = a.labels;
    p.dist = a.dist;
    p.old_labels = a.old_labels;
    p.changed = a.changed;
    p.dist_sum = a.dist_sum;
    p.err = err;
    p.lb_out = a.lb_out;
    p.lb_d16 = a.lb_d16;
    p.ubd = a.ubd;
    p.jb = a.jb;
    p.gkey = a.gkey;
    p.moved = a.moved;
    p.tmask = a.tmask;
    p.perm = a.perm;
    p.delta = a.delta;
    p.evals = a.evals;
    if (a.cand) {
        p.cand = a.cand;
        p.ncand = a.ncand;
        p.thr = screen_threshold(a.m, a.F);
        p.labels = nullptr;
        p.dist = nullptr;
        p.old_labels = nullptr;
        p.changed = nullptr;
        p.dist_sum = nullptr;
    }
    const size_t smem = g.smem();
    allow_max_dynamic_smem(k_assign_tc);
    const int64_t ntiles = (a.n + AT_TILE - 1) / AT_TILE;
    const int grid = (int)std::min<int64_t>(ntiles, ctx->sm_count);
    k_assign_tc<<<grid, AT_THREADS, smem, s>>>(map, p);
    TC_CHECK_LAUNCH();
    // no synchronisation here: a pipeline wait that ran out leaves the error word at
    // aux+52 set, and the caller reads it with its other results
}

}  // namespace tc
