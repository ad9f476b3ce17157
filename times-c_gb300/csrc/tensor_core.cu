// Tensor-core (tcgen05) Gram matrices for the shape extraction.
//
// S_c = Y_c^T Y_c (shapeExtract.cuh:532-537, a cuBLAS SGEMM per cluster with
// k CUDA streams in the reference) becomes one launch over all clusters and the
// 128x128 upper-triangle tiles of every S_c:
//   * the aligned members are transposed into YT[a][p'] (BF16, or FP32 rounded
//     to TF32) with each cluster's positions padded to a multiple of 64, so a
//     cluster is a contiguous, 128-byte aligned K range;
//   * per CTA a TMA producer thread streams 128-row x 128-byte K-major tiles of
//     YT (rows a0.. and b0..) through a 4-stage mbarrier pipeline with the
//     128-byte swizzle; one thread issues tcgen05.mma (M=128, N=128) into a
//     128-column FP32 TMEM accumulator;
//   * four warps read TMEM back (tcgen05.ld 32x32b) and write the tile and its
//     mirror image.
// All waits are bounded and report through an error word.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "gram_strips.h"
#include "sm100.cuh"
#include "tc_internal.h"

namespace tc {

constexpr int GT_TILE = 128;                       // rows per operand tile
constexpr int GT_TILE_BYTES = GT_TILE * 128;       // 128 rows x 128 bytes
constexpr int GT_PAD = 64;                          // cluster K padding (elements)

// FMT 1 = BF16, 2 = TF32, 3 = 3xTF32: x = hi + lo with hi, lo TF32, and
// S = hi*hi + hi*lo + lo*hi (the dropped lo*lo is below FP32 rounding), FP32-class
// products on the tensor cores for the plain FP32 form.
//
// A CTA computes a strip of one row tile: 128 rows (tile r) against w column tiles,
// one 128-column TMEM accumulator each, so every operand tile it loads serves w
// products (a 128 x 128 tile per CTA loads two tiles per product).  A strip that
// starts at the diagonal (q0 = r) holds up to W0 tiles and its A is its first B
// tile; the rest of the row goes in strips of up to W0 - 1 tiles plus the A tile.
// At m = 512 (4 row tiles, BF16) that is 4 strips of 4, 3, 2, 1 tiles: 10 tile loads
// per K slab of a cluster against 16 for tile pairs.  A strip of w tiles is split
// into w * base shares of its K range, so every CTA does the same work (its share's
// K blocks times w products); the shares' partials are summed in a fixed order.
template <int FMT>
struct GtCfg {
    static constexpr int PLANES = FMT == 3 ? 2 : 1;   // hi and lo planes (3xTF32)
    static constexpr int W0 = FMT == 3 ? 2 : 4;        // tiles per stage and plane
    static constexpr int STAGES = 3;
    static constexpr int STAGE_BYTES = W0 * PLANES * GT_TILE_BYTES;  // 64 KB
    static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;         // + alignment slack
    static constexpr int TMEM_COLS = W0 * 128;                        // a power of two
    static constexpr int KE = FMT == 1 ? 64 : 32;   // K elements per 128-byte slab
};

// ---------------------------------------------------------------- TMA descriptor
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        TC_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        TC_REQUIRE(q == cudaDriverEntryPointSuccess && p, TC_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// 2-D row-major tensor [rows][cols] of esize-byte elements; box = 128 bytes x box_rows.
CUtensorMap make_tmap_2d(const void* base, CUtensorMapDataType dt, int esize, uint64_t rows, uint64_t cols,
                                uint32_t box_rows) {
    CUtensorMap map;
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {cols * (uint64_t)esize};
    cuuint32_t box[2] = {(cuuint32_t)(128 / esize), box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(&map, dt, 2, const_cast<void*>(base), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    TC_REQUIRE(r == CUDA_SUCCESS, TC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return map;
}

// ---------------------------------------------------------------- transpose
__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
template <class TO>
__device__ __forceinline__ TO convert_out(float v);
template <>
__device__ __forceinline__ __nv_bfloat16 convert_out<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <>
__device__ __forceinline__ float convert_out<float>(float v) { return to_tf32(v); }

// YT[a][p'] = seg[pos][a], p' = pos - offsets[c] + poff[c] for the cluster c holding pos.
// With YTlo (3xTF32): YT gets tf32(x) and YTlo gets tf32(x - tf32(x)).
template <class TO>
__global__ void k_seg_transpose(const float* __restrict__ seg, int64_t n, int m, const int32_t* __restrict__ offsets,
                                const int32_t* __restrict__ counts, const int64_t* __restrict__ poff, int k,
                                TO* __restrict__ YT, float* __restrict__ YTlo, int64_t Pp) {
    __shared__ float tile[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t pos0 = (int64_t)blockIdx.x * 32;
    const int a0 = blockIdx.y * 32;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t pos = pos0 + ty + 8 * i;
        const int a = a0 + tx;
        tile[ty + 8 * i][tx] = (pos < n && a < m) ? seg[pos * m + a] : 0.f;
    }
    __syncthreads();
    const int64_t pos = pos0 + tx;
    if (pos >= n) return;
    int lo = 0, hi = k - 1;  // last cluster whose offset <= pos (non-empty)
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= pos) lo = mid;
        else hi = mid - 1;
    }
    while (counts[lo] == 0 && lo > 0) --lo;
    const int64_t pp = pos - offsets[lo] + poff[lo];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int a = a0 + ty + 8 * i;
        if (a < m) {
            const float x = tile[tx][ty + 8 * i];
            const TO hi = convert_out<TO>(x);
            YT[(int64_t)a * Pp + pp] = hi;
            if (YTlo) YTlo[(int64_t)a * Pp + pp] = to_tf32(x - (float)hi);
        }
    }
}

// ---------------------------------------------------------------- Gram kernel
template <int FMT>
__global__ void __launch_bounds__(128, 1) k_gram_tc(const __grid_constant__ CUtensorMap tmap,
                                                    const __grid_constant__ CUtensorMap tmap_lo,
                                                    const int32_t* __restrict__ counts,
                                                    const int64_t* __restrict__ poff, int m, int ld, int nt,
                                                    int nsplit, size_t part_stride, float* __restrict__ S,
                                                    int* __restrict__ err, const uint8_t* __restrict__ skip) {
    extern __shared__ uint8_t smem_raw[];
    typedef GtCfg<FMT> G;
    __shared__ __align__(8) uint64_t full[G::STAGES], empty[G::STAGES], done;
    __shared__ uint32_t tmem_base;
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int c = blockIdx.y;
    const int cnt = counts[c];
    if (cnt == 0 || (skip && skip[c])) return;
    int r, q0, w;
    bool diag;
    gram_strip(nt, G::W0, blockIdx.x, r, q0, w, diag);
    const int ns = nsplit > 0 ? w * nsplit : 1, z = blockIdx.z;  // this strip's shares (0: one)
    if (z >= ns) return;
    const int nload = diag ? w : w + 1;  // operand tiles per stage and plane
    constexpr int KE = G::KE;
    // this CTA's share of the cluster's K blocks, into partial buffer z
    const int nk_all = (cnt + KE - 1) / KE;
    const int kb0 = (int)((int64_t)z * nk_all / ns), nk = (int)((int64_t)(z + 1) * nk_all / ns) - kb0;
    if (nk == 0) return;  // the sum kernel skips empty shares
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < G::STAGES; ++s) {
            sm100::mbar_init(&full[s], 1);
            sm100::mbar_init(&empty[s], 1);
        }
        sm100::mbar_init(&done, 1);
        sm100::fence_mbar_init();
        sm100::prefetch_tmap(&tmap);
        if (FMT == 3) sm100::prefetch_tmap(&tmap_lo);
    }
    if (warp == 0) {
        sm100::tmem_alloc(&tmem_base, G::TMEM_COLS);
        sm100::tmem_relinquish();
    }
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = tmem_base;
    const int x0 = (int)poff[c];
    // stage layout: [plane][slot] tiles of 16 KB; slot 0 = A (= B tile 0 on the diagonal)
    auto slot_ptr = [&](uint8_t* st, int plane, int slot) {
        return st + (size_t)(plane * G::W0 + slot) * GT_TILE_BYTES;
    };
    bool ok = true;
    if (warp == 0 && lane == 0) {
        // TMA producer
        for (int kb = 0; kb < nk && ok; ++kb) {
            const int s = kb % G::STAGES, u = kb / G::STAGES;
            if (u > 0) ok = sm100::mbar_wait(&empty[s], (u - 1) & 1, err);
            if (!ok) break;
            uint8_t* st = base + (size_t)s * G::STAGE_BYTES;
            sm100::mbar_expect_tx(&full[s], (uint32_t)(nload * G::PLANES * GT_TILE_BYTES));
            const int xk = x0 + (kb0 + kb) * KE;
            for (int l = 0; l < nload; ++l) {
                const int tile = diag ? q0 + l : (l == 0 ? r : q0 + l - 1);
                sm100::tma_load_2d(slot_ptr(st, 0, l), &tmap, xk, tile * GT_TILE, &full[s]);
                if (FMT == 3) sm100::tma_load_2d(slot_ptr(st, 1, l), &tmap_lo, xk, tile * GT_TILE, &full[s]);
            }
        }
        // the MMA thread's last commits to empty[] arrive when their MMAs end: wait for
        // them, so no arrival lands in this CTA's shared memory after it has left
        // (another kernel's CTA may own it by then)
        if (ok)
            for (int kb = nk > G::STAGES ? nk - G::STAGES : 0; kb < nk; ++kb)
                sm100::mbar_wait(&empty[kb % G::STAGES], (kb / G::STAGES) & 1, err);
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: one 128 x 128 accumulator per column tile of the strip
        constexpr uint32_t ID = sm100::idesc(FMT == 1 ? 1 : 2, 128, 128);
        for (int kb = 0; kb < nk && ok; ++kb) {
            const int s = kb % G::STAGES, u = kb / G::STAGES;
            ok = sm100::mbar_wait(&full[s], u & 1, err);
            if (!ok) break;
            sm100::tc_fence_after();
            uint8_t* st = base + (size_t)s * G::STAGE_BYTES;
            const uint64_t da = sm100::desc_k_sw128(slot_ptr(st, 0, 0));
            const uint64_t dal = FMT == 3 ? sm100::desc_k_sw128(slot_ptr(st, 1, 0)) : 0;
            for (int i = 0; i < w; ++i) {
                const int bs = diag ? i : i + 1;
                const uint64_t db = sm100::desc_k_sw128(slot_ptr(st, 0, bs));
                const uint32_t acc = tmem + (uint32_t)(i * 128);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {  // 4 x 32 bytes of K per slab
                    if (FMT == 1) {
                        sm100::mma_f16(acc, da + 2 * kk, db + 2 * kk, ID, (kb | kk) != 0);
                    } else {
                        sm100::mma_tf32(acc, da + 2 * kk, db + 2 * kk, ID, (kb | kk) != 0);
                        if (FMT == 3) {
                            const uint64_t dbl = sm100::desc_k_sw128(slot_ptr(st, 1, bs));
                            sm100::mma_tf32(acc, da + 2 * kk, dbl + 2 * kk, ID, 1);
                            sm100::mma_tf32(acc, dal + 2 * kk, db + 2 * kk, ID, 1);
                        }
                    }
                }
            }
            sm100::mma_commit(&empty[s]);
        }
        sm100::mma_commit(&done);
    }
    __syncwarp();
    // epilogue: warp w owns TMEM lanes 32w..32w+31 = rows r*128 + 32w + lane
    const bool fin = __syncthreads_and(sm100::mbar_wait(&done, 0, err)) != 0;
    sm100::tc_fence_after();
    if (fin) {
        const int a = r * GT_TILE + warp * 32 + lane;
        float* Sc = S + (size_t)z * part_stride + (size_t)c * m * ld;
        for (int i = 0; i < w; ++i) {
            const int q = q0 + i;
            for (int cb = 0; cb < 4; ++cb) {
                float v[32];
                sm100::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(i * 128 + cb * 32), v);
                sm100::tmem_ld_wait();
                const int b0 = q * GT_TILE + cb * 32;
                if (a < m) {  // the row's 32 values as float4 (columns m..ld-1 are products with zero rows: 0)
                    float4* row4 = reinterpret_cast<float4*>(Sc + (size_t)a * ld + b0);
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (b0 + 4 * e < ld) row4[e] = make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
                }
                if (q != r) {  // the mirror image below the diagonal
#pragma unroll
                    for (int e = 0; e < 32; ++e)
                        if (b0 + e < m && a < m) Sc[(size_t)(b0 + e) * ld + a] = v[e];
                }
            }
        }
    } else if (threadIdx.x == 0) {
        // the pipeline stopped early: let copies already issued land before the CTA leaves
        for (int s = 0; s < G::STAGES; ++s) sm100::mbar_wait(&full[s], 0, nullptr);
    }
    sm100::tc_fence_before();
    __syncthreads();
    if (warp == 0) sm100::tmem_dealloc(tmem, G::TMEM_COLS);
}

// S_c = sum of the K shares' partial Grams, in share order (deterministic): the
// region of tile (lo, hi) comes from the strip holding it, split in width * base
// shares; shares with no K blocks wrote nothing and are skipped.  Rows a < m,
// columns < ld (the padding columns are zeros in every partial).
__global__ void k_gram_sum(const float* __restrict__ P, int base, int w0, int nt, size_t part_stride,
                           const int32_t* __restrict__ counts, int KE, int m, int ld, float* __restrict__ S,
                           const uint8_t* __restrict__ skip) {
    const int c = blockIdx.y;
    const int cnt = counts[c];
    if (cnt == 0 || (skip && skip[c])) return;
    const int nk = (cnt + KE - 1) / KE;
    const int ld4 = ld / 4;
    const size_t n4 = (size_t)m * ld4, off = (size_t)c * m * ld / 4;
    const float4* P4 = reinterpret_cast<const float4*>(P);
    float4* S4 = reinterpret_cast<float4*>(S);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += (size_t)gridDim.x * blockDim.x) {
        const int ta = (int)(e / ld4) / GT_TILE;
        const int tb = min((int)(e % ld4) * 4 / GT_TILE, nt - 1);
        const int ns = base > 0 ? gram_strip_width(nt, w0, min(ta, tb), max(ta, tb)) * base : 1;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int z = 0; z < ns; ++z) {
            if ((int64_t)(z + 1) * nk / ns == (int64_t)z * nk / ns) continue;
            const float4 q = P4[z * (part_stride / 4) + off + e];
            v.x += q.x;
            v.y += q.y;
            v.z += q.z;
            v.w += q.w;
        }
        S4[off + e] = v;
    }
}

// ---------------------------------------------------------------- host
// FP32 runs as 3xTF32 unless TIMESC_SIMT_GRAM is set (the SIMT kernel stays available).
bool gram_tc_supported(int m, int precision) {
    if (precision == TC_PREC_FP32 && std::getenv("TIMESC_SIMT_GRAM")) return false;
    return m >= 2;
}

// Zero the padding columns of cluster c: [poff + count, poff + roundup(count, 64)), every row.
template <class TO>
__global__ void k_zero_pads(const int32_t* __restrict__ counts, const int64_t* __restrict__ poff, int m, int64_t Pp,
                            TO* __restrict__ YT, float* __restrict__ YTlo) {
    const int c = blockIdx.x;
    const int cnt = counts[c];
    const int pad = (cnt + GT_PAD - 1) / GT_PAD * GT_PAD - cnt;
    const int64_t c0 = poff[c] + cnt;
    for (int e = threadIdx.x; e < pad * m; e += blockDim.x) {
        const int a = e / pad, q = e % pad;
        YT[(int64_t)a * Pp + c0 + q] = TO(0.f);
        if (YTlo) YTlo[(int64_t)a * Pp + c0 + q] = 0.f;
    }
}

// Columns of the transposed, cluster-padded member matrix: every cluster padded
// to a multiple of 64 members fits in n + 63 k (the padded offsets themselves
// are computed on the device, so the layout needs no host read-back).
int64_t gram_padded_cols(int64_t n, int k) {
    return std::max<int64_t>((n + 63 * (int64_t)k + GT_PAD - 1) / GT_PAD * GT_PAD, GT_PAD);
}

// The transposed, cluster-padded operand of the tensor-core Gram in the workspace:
// BF16 (precision BF16), TF32 (TF32), or TF32 hi and lo planes (FP32: 3xTF32).
size_t gram_operand_bytes(int64_t n, int k, int m, int precision) {
    const int fmt = precision == TC_PREC_BF16 ? 1 : (precision == TC_PREC_TF32 ? 2 : 3);
    return (size_t)m * gram_padded_cols(n, k) * (fmt == 1 ? 2 : 4) * (fmt == 3 ? 2 : 1);
}

GramOperand gram_tc_operand(tc_ctx* ctx, int64_t n, int k, int m, int precision) {
    GramOperand o;
    o.Pp = gram_padded_cols(n, k);
    o.fmt = precision == TC_PREC_BF16 ? 1 : (precision == TC_PREC_TF32 ? 2 : 3);
    const int esize = o.fmt == 1 ? 2 : 4;
    const size_t plane = (size_t)m * o.Pp * esize;
    char* YT = static_cast<char*>(ctx->ws.gram_yt.get(gram_operand_bytes(n, k, m, precision)));
    o.YT = YT;
    o.YTlo = o.fmt == 3 ? reinterpret_cast<float*>(YT + plane) : nullptr;
    return o;
}

// No host synchronisation: a pipeline wait that runs out sets *err (the caller reads it).
// seg == nullptr: the operand was already written by the fused gather.
void launch_gram_tc(tc_ctx* ctx, const float* seg, const int32_t* counts, const int32_t* offsets,
                    const int64_t* poff, int64_t n, int k, int m, int ld, int precision, float* S, int* err,
                    cudaStream_t s, const uint8_t* skip) {
    const GramOperand op = gram_tc_operand(ctx, n, k, m, precision);
    const int64_t Pp = op.Pp;
    const int fmt = op.fmt;
    const int esize = fmt == 1 ? 2 : 4;
    char* YT = static_cast<char*>(op.YT);
    float* YTlo = op.YTlo;
    // only the padding needs zeros: the transpose writes every member column
    if (fmt == 1)
        k_zero_pads<__nv_bfloat16><<<k, 256, 0, s>>>(counts, poff, m, Pp, (__nv_bfloat16*)YT, nullptr);
    else
        k_zero_pads<float><<<k, 256, 0, s>>>(counts, poff, m, Pp, (float*)YT, YTlo);
    TC_CHECK_LAUNCH();
    dim3 tg(ceil_div(n, 32), ceil_div(m, 32)), tb(32, 8);
    if (n > 0 && seg) {
        if (fmt == 1)
            k_seg_transpose<__nv_bfloat16><<<tg, tb, 0, s>>>(seg, n, m, offsets, counts, poff, k,
                                                             (__nv_bfloat16*)YT, nullptr, Pp);
        else
            k_seg_transpose<float><<<tg, tb, 0, s>>>(seg, n, m, offsets, counts, poff, k, (float*)YT, YTlo, Pp);
        TC_CHECK_LAUNCH();
    }
    const CUtensorMapDataType dt = fmt == 1 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    CUtensorMap map = make_tmap_2d(YT, dt, esize, (uint64_t)m, (uint64_t)Pp, GT_TILE);
    CUtensorMap map_lo = fmt == 3 ? make_tmap_2d(YTlo, dt, esize, (uint64_t)m, (uint64_t)Pp, GT_TILE) : map;
    const int nt = ceil_div(m, GT_TILE);
    // A strip of w tiles runs as w * base CTAs over shares of its K range, so every
    // CTA does the same work; base (1..W0 / 2 ... 2 shares per tile product) is the
    // count that best fills the launch's last wave (one CTA per SM: the operand ring
    // takes most of the shared memory) while every share keeps at least 64 K blocks of
    // a tile product on average (with fewer, a CTA's fixed costs - setup, pipeline
    // fill, the strip and mirror stores, its partial's share of the sum - outweigh the
    // fuller wave).  The partials are summed in a fixed order.
    const int KE = fmt == 1 ? GtCfg<1>::KE : GtCfg<3>::KE;
    const int w0 = fmt == 1 ? GtCfg<1>::W0 : (fmt == 2 ? GtCfg<2>::W0 : GtCfg<3>::W0);
    const int strips = gram_strips(nt, w0);
    const int units = nt * (nt + 1) / 2 * k;  // CTAs per unit of base: one per tile product
    const int64_t avg_kb = std::max<int64_t>(1, n / std::max(k, 1) / KE);
    auto occupancy = [&](int b) {
        const double x = (double)units * b / ctx->sm_count;
        return x / std::ceil(x);
    };
    int nsplit = 1;  // base
    for (int b = 2; b * w0 <= 8 && avg_kb / b >= 64; ++b)
        if (occupancy(b) > occupancy(nsplit) + 0.02) nsplit = b;
    if (std::getenv("TIMESC_GRAM_NOSPLIT")) nsplit = 0;  // one share per strip (for comparison)
    const int shares = nsplit > 0 ? w0 * nsplit : 1;
    const size_t part_stride = (size_t)k * m * ld;
    float* out = ctx->ws.gram_part.as<float>((size_t)shares * part_stride);
    dim3 grid(strips, k, shares);
    if (fmt == 1) {
        allow_max_dynamic_smem(k_gram_tc<1>);
        k_gram_tc<1><<<grid, 128, GtCfg<1>::SMEM, s>>>(map, map_lo, counts, poff, m, ld, nt, nsplit, part_stride,
                                                        out, err, skip);
    } else if (fmt == 2) {
        allow_max_dynamic_smem(k_gram_tc<2>);
        k_gram_tc<2><<<grid, 128, GtCfg<2>::SMEM, s>>>(map, map_lo, counts, poff, m, ld, nt, nsplit, part_stride,
                                                        out, err, skip);
    } else {
        allow_max_dynamic_smem(k_gram_tc<3>);
        k_gram_tc<3><<<grid, 128, GtCfg<3>::SMEM, s>>>(map, map_lo, counts, poff, m, ld, nt, nsplit, part_stride,
                                                        out, err, skip);
    }
    TC_CHECK_LAUNCH();
    k_gram_sum<<<dim3(ceil_div((int64_t)m * ld / 4, 256 * 4), k), 256, 0, s>>>(out, nsplit, w0, nt, part_stride,
                                                                              counts, KE, m, ld, S, skip);
    TC_CHECK_LAUNCH();
}

}  // namespace tc
