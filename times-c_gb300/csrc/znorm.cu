// Row z-normalisation: x <- (x - mean) / sqrt(sum (x-mean)^2 / (m - ddof)).
//
// Replaces z_norm_gpu_x (normalization.cuh:150-177: a cuBLAS row-mean GEMM, a
// rank-1 subtract, then a 1024-thread block per row).  Here one warp owns one
// row held in registers (one block per row for m > 1024): a single HBM read and
// write per value, FP32 lane partials combined in FP64 across the warp/block.
// The GATHER variant is the extraction's fused pass: it reads row perm[pos]
// shifted by its alignment shift (out[t] = x[t - shift], zero fill, SBD.cuh:14-29)
// and writes the normalised row to position pos of the cluster-ordered buffer
// (block_alloc2D + sbd3D + z_norm_gpu_x of shapeExtract.cuh:1117-1141).
#include <cuda_bf16.h>

#include <type_traits>

#include "tc_internal.h"

namespace tc {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct RowSrc {
    const float* x;
    int shift;
};

template <bool GATHER>
__device__ __forceinline__ RowSrc row_source(const float* src, int64_t row, int64_t n, int m, const int32_t* perm,
                                             const int32_t* labels, const int32_t* shift, const uint8_t* gate) {
    RowSrc r;
    if (GATHER) {
        int64_t i = perm[row];
        // an entry the scatter did not fill (labels outside [0, k), reported as an
        // error by the host) reads row 0 instead of an arbitrary address
        if (i < 0 || i >= n) i = 0;
        r.x = src + (size_t)i * m;
        r.shift = (gate && shift && gate[labels[i]]) ? shift[i] : 0;
    } else {
        r.x = src + (size_t)row * m;
        r.shift = 0;
    }
    return r;
}

// Compensated FP32 sums: Kahan within a lane, TwoSum across lanes; every lane
// gets the total.  (GB300 retires few FP64 lane-operations per clock, so the
// per-row path stays in FP32.)
struct KSum {
    float s = 0.f, c = 0.f;  // value = s - c
    __device__ __forceinline__ void add(float x) {
        const float y = x - c, t = s + y;
        c = (t - s) - y;
        s = t;
    }
};
__device__ __forceinline__ float warp_sum_comp(KSum k) {
    float s = k.s, c = k.c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o), c2 = __shfl_xor_sync(0xffffffffu, c, o);
        const float t = s + s2, bp = t - s;
        const float err = (s - (t - bp)) + (s2 - bp);
        s = t;
        c = c + c2 - err;
    }
    return s - c;
}

template <int VPL, bool GATHER>
__global__ void __launch_bounds__(256) k_norm_rows_warp(const float* __restrict__ src, float* dst, int64_t n, int m,
                                                        int ddof, const int32_t* __restrict__ perm,
                                                        const int32_t* __restrict__ labels,
                                                        const int32_t* __restrict__ shift,
                                                        const uint8_t* __restrict__ gate) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = w0; row < n; row += nw) {
        RowSrc rs = row_source<GATHER>(src, row, n, m, perm, labels, shift, gate);
        float v[VPL];
        KSum s;
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
            int t = lane + 32 * q;
            int a = t - rs.shift;
            v[q] = (t < m && a >= 0 && a < m) ? rs.x[a] : 0.f;
            s.add(v[q]);
        }
        const float mean = warp_sum_comp(s) / (float)m;
        KSum ss;
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
            int t = lane + 32 * q;
            float d = t < m ? v[q] - mean : 0.f;
            v[q] = d;
            ss.add(d * d);
        }
        const float var = warp_sum_comp(ss) / (float)(m - ddof);
        const float sd = sqrtf(var);
        const float inv = (sd > 0.f && isfinite(sd)) ? 1.0f / sd : 0.f;
        float* y = dst + (size_t)row * m;
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
            int t = lane + 32 * q;
            if (t < m) y[t] = v[q] * inv;
        }
    }
}

template <int VPT, bool GATHER>
__global__ void __launch_bounds__(256) k_norm_rows_block(const float* __restrict__ src, float* dst, int64_t n, int m,
                                                         int ddof, const int32_t* __restrict__ perm,
                                                         const int32_t* __restrict__ labels,
                                                         const int32_t* __restrict__ shift,
                                                         const uint8_t* __restrict__ gate) {
    __shared__ double red[8];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int64_t row = blockIdx.x; row < n; row += gridDim.x) {
        RowSrc rs = row_source<GATHER>(src, row, n, m, perm, labels, shift, gate);
        float v[VPT];
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < VPT; ++q) {
            int t = tid + 256 * q;
            int a = t - rs.shift;
            v[q] = (t < m && a >= 0 && a < m) ? rs.x[a] : 0.f;
            s += v[q];
        }
        double ds = warp_sum_d((double)s);
        if (lane == 0) red[wid] = ds;
        __syncthreads();
        ds = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) ds += red[w];
        __syncthreads();
        const float mean = (float)(ds / m);
        float ss = 0.f;
#pragma unroll
        for (int q = 0; q < VPT; ++q) {
            int t = tid + 256 * q;
            float d = t < m ? v[q] - mean : 0.f;
            v[q] = d;
            ss += d * d;
        }
        double dss = warp_sum_d((double)ss);
        if (lane == 0) red[wid] = dss;
        __syncthreads();
        dss = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) dss += red[w];
        __syncthreads();
        const double sd = sqrt(dss / (double)(m - ddof));
        const float inv = (sd > 0.0 && isfinite(sd)) ? (float)(1.0 / sd) : 0.f;
        float* y = dst + (size_t)row * m;
#pragma unroll
        for (int q = 0; q < VPT; ++q) {
            int t = tid + 256 * q;
            if (t < m) y[t] = v[q] * inv;
        }
    }
}

template <bool GATHER>
static void norm_rows(const float* src, float* dst, int64_t n, int m, int ddof, const int32_t* perm,
                      const int32_t* labels, const int32_t* shift, const uint8_t* gate, int sm_count,
                      cudaStream_t s) {
    if (n == 0) return;
    TC_REQUIRE(m >= 2 && m <= 8192, TC_ERR_UNSUPPORTED, "series length must be in [2, 8192]");
    const int wgrid = (int)std::min<int64_t>(ceil_div(n, 8), (int64_t)sm_count * 16);
    const int bgrid = (int)std::min<int64_t>(n, (int64_t)sm_count * 8);
#define WARP(VPL) k_norm_rows_warp<VPL, GATHER><<<wgrid, 256, 0, s>>>(src, dst, n, m, ddof, perm, labels, shift, gate)
#define BLOCK(VPT) k_norm_rows_block<VPT, GATHER><<<bgrid, 256, 0, s>>>(src, dst, n, m, ddof, perm, labels, shift, gate)
    if (m <= 64) WARP(2);
    else if (m <= 128) WARP(4);
    else if (m <= 256) WARP(8);
    else if (m <= 512) WARP(16);
    else if (m <= 1024) WARP(32);
    else if (m <= 2048) BLOCK(8);
    else if (m <= 4096) BLOCK(16);
    else BLOCK(32);
#undef WARP
#undef BLOCK
    TC_CHECK_LAUNCH();
}

void launch_znorm(float* x, int64_t n, int m, int ddof, int sm_count, cudaStream_t s) {
    norm_rows<false>(x, x, n, m, ddof, nullptr, nullptr, nullptr, nullptr, sm_count, s);
}

void launch_gather_norm(const float* x, const int32_t* perm, const int32_t* labels, const int32_t* shift,
                        const uint8_t* gate, int64_t n, int m, float* seg, int sm_count, cudaStream_t s) {
    norm_rows<true>(x, seg, n, m, 1, perm, labels, shift, gate, sm_count, s);
}

}  // namespace tc

// ---------------------------------------------------------------- fused gather + transpose
namespace tc {

template <class TO>
__device__ __forceinline__ TO to_operand(float v);
template <>
__device__ __forceinline__ __nv_bfloat16 to_operand<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <>
__device__ __forceinline__ float to_operand<float>(float v) {  // TF32 rounding (the 3xTF32 hi part)
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

// The extraction's gather (align + re-normalise, as k_norm_rows_warp<VPL, true>,
// with the same arithmetic) for 32 cluster-ordered positions per block, written
// transposed into the tensor-core Gram's operand YT[a][pp] (pp: the position in
// the cluster-padded layout) instead of row-major: the row-major copy and the
// separate transpose pass are never made.  The first member of each cluster also
// goes to first[c][*] (the sign rule's reference row).  With YTlo (3xTF32) the lo
// plane gets x - tf32(x) rounded to TF32.  Rows are staged in shared memory with
// pitch m+1 so the transposed reads are free of bank conflicts.
template <int VPL, class TO>
__global__ void __launch_bounds__(256) k_gather_norm_t(const float* __restrict__ src, int64_t n, int m,
                                                       const int32_t* __restrict__ perm,
                                                       const int32_t* __restrict__ labels,
                                                       const int32_t* __restrict__ shift,
                                                       const uint8_t* __restrict__ gate,
                                                       const int32_t* __restrict__ offsets,
                                                       const int32_t* __restrict__ counts, int k,
                                                       const int64_t* __restrict__ poff, TO* __restrict__ YT,
                                                       float* __restrict__ YTlo, int64_t Pp,
                                                       float* __restrict__ first, const uint8_t* __restrict__ skip) {
    extern __shared__ float tile[];  // [32][m + 1]
    const int pitch = m + 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t pos0 = (int64_t)blockIdx.x * 32;
    // positions the scatter filled (fewer than n when some labels were outside [0, k):
    // the host reports that as an error, and nothing here reads the unfilled ones)
    const int64_t placed = (int64_t)offsets[k - 1] + counts[k - 1];
    for (int r = wid; r < 32; r += 8) {
        const int64_t pos = pos0 + r;
        if (pos >= placed) break;
        const int64_t i = perm[pos];
        const int c = labels[i];
        if (skip && skip[c]) continue;  // uniform over the warp: one row per warp
        const float* x = src + (size_t)i * m;
        const int sh = (gate && shift && gate[c]) ? shift[i] : 0;
        float v[VPL];
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
            const int t = lane + 32 * q, a = t - sh;
            v[q] = (t < m && a >= 0 && a < m) ? x[a] : 0.f;
        }
        float mean, var;
        if constexpr (std::is_same<TO, float>::value) {
            // FP32 operand (its 3xTF32 low plane keeps FP32 accuracy): compensated sums
            KSum s;
#pragma unroll
            for (int q = 0; q < VPL; ++q) s.add(v[q]);
            mean = warp_sum_comp(s) / (float)m;
            KSum ss;
#pragma unroll
            for (int q = 0; q < VPL; ++q) {
                const int t = lane + 32 * q;
                const float d = t < m ? v[q] - mean : 0.f;
                v[q] = d;
                ss.add(d * d);
            }
            var = warp_sum_comp(ss) / (float)(m - 1);
        } else {
            // BF16 operand: plain FP32 sums (relative error ~1e-5 in the scale, far below
            // BF16's 4e-3 rounding step), a third of the compensated form's instructions
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < VPL; ++q) s += v[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            mean = s / (float)m;
            float ss = 0.f;
#pragma unroll
            for (int q = 0; q < VPL; ++q) {
                const int t = lane + 32 * q;
                const float d = t < m ? v[q] - mean : 0.f;
                v[q] = d;
                ss = fmaf(d, d, ss);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
            var = ss / (float)(m - 1);
        }
        const float sd = sqrtf(var);
        const float inv = (sd > 0.f && isfinite(sd)) ? 1.0f / sd : 0.f;
        const bool lead = pos == offsets[c];
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
            const int t = lane + 32 * q;
            if (t < m) {
                const float y = v[q] * inv;
                tile[r * pitch + t] = y;
                if (lead) first[(size_t)c * m + t] = y;
            }
        }
    }
    __syncthreads();
    const int r = lane;
    const int64_t pos = pos0 + r;
    if (pos >= placed) return;
    const int c = labels[perm[pos]];
    if (skip && skip[c]) return;  // its row was not staged
    const int64_t pp = pos - offsets[c] + poff[c];
    for (int a = wid; a < m; a += 8) {
        const float y = tile[r * pitch + a];
        const TO hi = to_operand<TO>(y);
        YT[(int64_t)a * Pp + pp] = hi;
        if (YTlo) YTlo[(int64_t)a * Pp + pp] = to_operand<float>(y - (float)hi);
    }
}

bool gather_transposed_supported(int m) { return m >= 2 && m <= 1024; }

void launch_gather_norm_t(const float* x, const int32_t* perm, const int32_t* labels, const int32_t* shift,
                          const uint8_t* gate, const int32_t* offsets, const int32_t* counts, int k,
                          const int64_t* poff, int64_t n, int m, bool bf16, void* YT, float* YTlo, int64_t Pp,
                          float* first, cudaStream_t s, const uint8_t* skip) {
    if (n == 0) return;
    TC_REQUIRE(gather_transposed_supported(m), TC_ERR_UNSUPPORTED, "fused gather: m must be in [2, 1024]");
    const size_t smem = (size_t)32 * (m + 1) * sizeof(float);
    const int grid = ceil_div(n, 32);
#define GT(VPL)                                                                                                 \
    do {                                                                                                        \
        if (bf16) {                                                                                             \
            allow_max_dynamic_smem(k_gather_norm_t<VPL, __nv_bfloat16>);                                        \
            k_gather_norm_t<VPL, __nv_bfloat16><<<grid, 256, smem, s>>>(x, n, m, perm, labels, shift, gate,     \
                                                                        offsets, counts, k, poff,               \
                                                                        (__nv_bfloat16*)YT,                     \
                                                                        nullptr, Pp, first, skip);             \
        } else {                                                                                                \
            allow_max_dynamic_smem(k_gather_norm_t<VPL, float>);                                                \
            k_gather_norm_t<VPL, float><<<grid, 256, smem, s>>>(x, n, m, perm, labels, shift, gate, offsets,    \
                                                                counts, k, poff, (float*)YT, YTlo, Pp, first,   \
                                                                skip);                                          \
        }                                                                                                       \
    } while (0)
    if (m <= 64) GT(2);
    else if (m <= 128) GT(4);
    else if (m <= 256) GT(8);
    else if (m <= 512) GT(16);
    else GT(32);
#undef GT
    TC_CHECK_LAUNCH();
}

}  // namespace tc
