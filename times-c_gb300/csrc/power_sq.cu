// Power iteration by repeated squaring on the tensor cores, for the forms that
// converge to the top eigenvector (canonical mode, cal_select = 1).
//
// The power iteration (shapeExtract.cuh:269-283, :577-630) steps v <- Mv/|Mv| from
// v0 = [1, .5, 1, .5, ...] on the centred matrix M = S - (r 1^T + 1 r^T)/m + tot 11^T/m^2,
// so after e steps v ~ M^e v0.  Here the e sequential matrix-vector steps (each a
// cluster-wide barrier) become floor(log2 e) squarings and one matrix-vector product
// per set bit of e:
//   P_0 = M / trace(M),  P_{j+1} = P_j^2 / trace(P_j^2),  v <- P_j v for bit j of e.
// M is symmetric, so P_j^2 = P_j P_j^T is a Gram matrix: the 3xTF32 tensor-core
// Gram kernel computes it with the rows of P_j as the "members" of cluster c
// (P_j in the transposed operand at columns poff[c] .. poff[c] + m).  The trace
// normalisation keeps every P_j's largest eigenvalue in [1/m, 1], so nothing
// overflows or underflows on the way.  The power-iteration kernel then starts
// from the product, steps on until its convergence test passes, and applies the
// eigenvalue, sign and centring rules as before.  (The compat form's fixed m steps
// stay plain steps: an error in the j-th square is applied e/2^j times.)
#include <cuda_runtime.h>

#include <cstdlib>

#include "tc_internal.h"

namespace tc {

namespace {

constexpr int SQ_THREADS = 256;
constexpr int SQ_ROWS = 32;  // rows of P per block

__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ double sum_block_d(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0;
    for (int w = 0; w < SQ_THREADS / 32; ++w) s += red[w];
    return s;
}

__device__ __forceinline__ void put_split(float* YT, float* YTlo, int64_t idx, float x) {
    const float hi = tf32_round(x);
    YT[idx] = hi;
    YTlo[idx] = tf32_round(x - hi);
}

// P_0 = M / trace(M) into the operand planes; flags and padded offsets per cluster.
__global__ void __launch_bounds__(SQ_THREADS) k_sq_first(const float* __restrict__ S, int ld,
                                                         const double* __restrict__ r,
                                                         const double* __restrict__ tot,
                                                         const int32_t* __restrict__ counts, int m, int mp,
                                                         int64_t Pp, float* __restrict__ YT, float* __restrict__ YTlo,
                                                         int32_t* __restrict__ cnt_sq, int32_t* __restrict__ ok,
                                                         int64_t* __restrict__ poff) {
    __shared__ double red[SQ_THREADS / 32];
    const int c = blockIdx.y;
    const float* Sc = S + (size_t)c * m * ld;
    const double* rc = r + (size_t)c * m;
    const double inv_m = 1.0 / m, tm = tot[c] * inv_m * inv_m;
    double tr = 0;
    if (counts[c] > 0)
        for (int a = threadIdx.x; a < m; a += SQ_THREADS) tr += (double)Sc[(size_t)a * ld + a] - 2.0 * rc[a] * inv_m + tm;
    tr = sum_block_d(tr, red);
    const bool good = counts[c] > 0 && tr > 0 && isfinite(tr);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ok[c] = good ? 1 : 0;
        cnt_sq[c] = good ? m : 0;
        poff[c] = (int64_t)c * mp;
    }
    if (!good) return;
    const double inv = 1.0 / tr;
    const int64_t x0 = (int64_t)c * mp;
    const int a0 = blockIdx.x * SQ_ROWS, a1 = min(a0 + SQ_ROWS, m);
    for (int a = a0; a < a1; ++a) {
        const double ra = rc[a] * inv_m;
        for (int b = threadIdx.x; b < m; b += SQ_THREADS) {
            const double x = ((double)Sc[(size_t)a * ld + b] - ra - rc[b] * inv_m + tm) * inv;
            put_split(YT, YTlo, (int64_t)a * Pp + x0 + b, (float)x);
        }
    }
}

// P_{j+1} = Q / trace(Q) with Q = P_j^2 from the Gram kernel.
__global__ void __launch_bounds__(SQ_THREADS) k_sq_next(const float* __restrict__ Q, int ld, int m, int mp,
                                                        int64_t Pp, float* __restrict__ YT, float* __restrict__ YTlo,
                                                        int32_t* __restrict__ cnt_sq, int32_t* __restrict__ ok) {
    __shared__ double red[SQ_THREADS / 32];
    const int c = blockIdx.y;
    if (!ok[c]) return;  // block-uniform: every block of the cluster reads the same flag
    const float* Qc = Q + (size_t)c * m * ld;
    double tr = 0;
    for (int a = threadIdx.x; a < m; a += SQ_THREADS) tr += (double)Qc[(size_t)a * ld + a];
    tr = sum_block_d(tr, red);
    if (!(tr > 0 && isfinite(tr))) {  // every block of the cluster sees the same trace
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ok[c] = 0;
            cnt_sq[c] = 0;
        }
        return;
    }
    const float inv = (float)(1.0 / tr);
    const int64_t x0 = (int64_t)c * mp;
    const int a0 = blockIdx.x * SQ_ROWS, a1 = min(a0 + SQ_ROWS, m);
    for (int a = a0; a < a1; ++a)
        for (int b = threadIdx.x; b < m; b += SQ_THREADS)
            put_split(YT, YTlo, (int64_t)a * Pp + x0 + b, Qc[(size_t)a * ld + b] * inv);
}

// vout = P_j (vin / |vin|); vin == nullptr means v0 = [1, .5, 1, .5, ...].
// Compensated FP32 sums per row (the operand is hi + lo).
__global__ void __launch_bounds__(SQ_THREADS) k_sq_apply(const float* __restrict__ YT, const float* __restrict__ YTlo,
                                                         int64_t Pp, int m, int mp, const int32_t* __restrict__ ok,
                                                         const float* __restrict__ vin, float* __restrict__ vout,
                                                         int ldv) {
    extern __shared__ float vs[];
    __shared__ double red[SQ_THREADS / 32];
    const int c = blockIdx.y;
    if (!ok[c]) return;
    double q = 0;
    for (int a = threadIdx.x; a < m; a += SQ_THREADS) {
        const float x = vin ? vin[(size_t)c * ldv + a] : ((a % 2 == 0) ? 1.f : 0.5f);
        vs[a] = x;
        q += (double)x * x;
    }
    q = sum_block_d(q, red);  // its barriers also publish vs
    const float sc = (float)(1.0 / sqrt(q));
    const int64_t x0 = (int64_t)c * mp;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int a0 = blockIdx.x * SQ_ROWS, a1 = min(a0 + SQ_ROWS, m);
    for (int a = a0 + wid; a < a1; a += SQ_THREADS / 32) {
        const float* hr = YT + (int64_t)a * Pp + x0;
        const float* lr = YTlo + (int64_t)a * Pp + x0;
        float s = 0.f, cp = 0.f;
        for (int b = lane; b < m; b += 32) {
            const float pr = (hr[b] + lr[b]) * vs[b];
            const float y = pr - cp, t = s + y;
            cp = (t - s) - y;
            s = t;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
            const float c2 = __shfl_xor_sync(0xffffffffu, cp, o);
            const float t = s + s2;  // TwoSum of the leading parts, errors folded into cp
            const float bp = t - s;
            const float err = (s - (t - bp)) + (s2 - bp);
            s = t;
            cp = cp + c2 - err;
        }
        if (lane == 0) vout[(size_t)c * ldv + a] = (s - cp) * sc;
    }
}

}  // namespace

// Used where the squares' Gram launch (k x tiles CTAs, one per SM) fits in one wave:
// measured on GB300 (canonical and cal_select forms, whole extraction), squaring ran
// 1.3-2.2x faster than stepping at m = 128..512 with k = 8..32 in one wave, and
// slower once the launch took three waves (m = 512, k = 32: 11 squares of ~0.25 ms
// against ~1.9 ms of early-stopping steps).
bool power_squaring_supported(int m, int k, int sm_count) {
    if (std::getenv("TIMESC_NO_SQUARING")) return false;
    const int nt = (m + 127) / 128;
    return m >= 2 && m <= 1024 && (int64_t)k * nt * (nt + 1) / 2 <= sm_count &&
           gram_tc_supported(m, TC_PREC_FP32);
}

size_t power_squaring_operand_bytes(int k, int m) {
    return gram_operand_bytes((int64_t)k * ((m + 63) / 64 * 64), k, m, TC_PREC_FP32);
}

// v_c ~ M_c^e v0 for every cluster whose matrix has a positive trace (ok[c] = 1).
// Returns the vectors (k x ld, not normalised) and the flags.
SquaringResult power_squaring(tc_ctx* ctx, const float* S, int ld, const double* r, const double* tot,
                              const int32_t* counts, int k, int m, int64_t e, int* err, cudaStream_t s) {
    Workspace& ws = ctx->ws;
    const int mp = (m + 63) / 64 * 64;
    const int64_t nsq = (int64_t)k * mp;  // operand columns: cluster c at c * mp
    const GramOperand op = gram_tc_operand(ctx, nsq, k, m, TC_PREC_FP32);
    float* YT = static_cast<float*>(op.YT);
    float* YTlo = op.YTlo;
    float* Q = ws.gram_sq.as<float>((size_t)k * m * ld);
    float* vec = ws.piter.as<float>((size_t)2 * k * ld);
    char* meta = ws.sq_meta.as<char>((size_t)k * 16);
    int64_t* poff = reinterpret_cast<int64_t*>(meta);
    int32_t* cnt_sq = reinterpret_cast<int32_t*>(meta + (size_t)k * 8);
    int32_t* ok = cnt_sq + k;
    const dim3 grid(ceil_div(m, SQ_ROWS), k);
    k_sq_first<<<grid, SQ_THREADS, 0, s>>>(S, ld, r, tot, counts, m, mp, op.Pp, YT, YTlo, cnt_sq, ok, poff);
    TC_CHECK_LAUNCH();
    int J = 0;
    while ((e >> (J + 1)) > 0) ++J;
    const float* vin = nullptr;
    int cur = 0;
    for (int j = 0; j <= J; ++j) {
        if ((e >> j) & 1) {
            float* vout = vec + (size_t)cur * k * ld;
            k_sq_apply<<<grid, SQ_THREADS, (size_t)m * sizeof(float), s>>>(YT, YTlo, op.Pp, m, mp, ok, vin, vout, ld);
            TC_CHECK_LAUNCH();
            vin = vout;
            cur ^= 1;
        }
        if (j < J) {
            launch_gram_tc(ctx, nullptr, cnt_sq, nullptr, poff, nsq, k, m, ld, TC_PREC_FP32, Q, err, s);
            k_sq_next<<<grid, SQ_THREADS, 0, s>>>(Q, ld, m, mp, op.Pp, YT, YTlo, cnt_sq, ok);
            TC_CHECK_LAUNCH();
        }
    }
    return SquaringResult{vin, ok};
}

}  // namespace tc
