// Shape extraction (extract_shape, shapeExtract.cuh:1058-1181).
//
//   segment   stable counting sort of series by label: chunk histograms, a scan
//             per cluster over chunks, a scan over clusters, and a stable scatter
//             (warp match + per-warp counts) - replaces class_count/get_loc2
//             (a single-thread loop for n < 1e6) and block_alloc2D (:21-188).
//   gate      per-cluster alignment gate (:1129-1135).
//   gather    align + re-z-normalise members into cluster order (znorm.cu);
//             with the tensor-core Gram (m <= 1024) written straight into its
//             transposed, cluster-padded operand.
//   Gram      S_c = sum_{i in c} y_i y_i^T (:532-537): tcgen05 (tensor_core.cu,
//             3xTF32 for the FP32 form) or SIMT FP32 here.
//   centring  M = Q S Q is never formed: M v = S v - (1.v/m) r - (r.v/m) 1
//             + (tot 1.v/m^2) 1 with r = S 1, tot = 1^T S 1 (replaces get_matQ and
//             two in-place m^3 GEMMs, :204-214, :551-570).
//   power     power.cu: one thread-block cluster per k-Shape cluster, all in one
//             launch (:269-360, :577-630); the Rayleigh quotient, the sign rule and
//             the store are fused into its last step (get_center, :217-264).
#include <algorithm>
#include <cmath>

#include "tc_internal.h"

namespace tc {

void launch_gather_norm(const float* x, const int32_t* perm, const int32_t* labels, const int32_t* shift,
                        const uint8_t* gate, int64_t n, int m, float* seg, int sm_count, cudaStream_t s);

constexpr int SEG_CHUNK = 4096;
constexpr int SEG_BLOCK = 256;
constexpr int MAX_K = 1024;

__device__ __forceinline__ double block_sum_d(double v, double* red) {
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

// ---------------------------------------------------------------- segment
// Labels outside [0, k) are not counted; they raise *bad, which the host checks
// before anything indexes by label.
__global__ void k_seg_count(const int32_t* __restrict__ labels, int64_t n, int k, int32_t* __restrict__ chunk_cnt,
                            int32_t* __restrict__ bad) {
    extern __shared__ int hist[];
    for (int j = threadIdx.x; j < k; j += blockDim.x) hist[j] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * SEG_CHUNK;
    for (int t = threadIdx.x; t < SEG_CHUNK; t += blockDim.x) {
        int64_t i = base + t;
        if (i < n) {
            int l = labels[i];
            if (l >= 0 && l < k) atomicAdd(&hist[l], 1);
            else atomicOr(bad, 1);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < k; j += blockDim.x) chunk_cnt[(size_t)blockIdx.x * k + j] = hist[j];
}

// one block per cluster: exclusive scan of its per-chunk counts, total -> counts[j]
__global__ void k_seg_scan_chunks(int32_t* __restrict__ chunk_cnt, int nchunks, int k, int32_t* __restrict__ counts) {
    __shared__ int red[32];
    const int j = blockIdx.x;
    int carry = 0;
    for (int c0 = 0; c0 < nchunks; c0 += blockDim.x) {
        int c = c0 + threadIdx.x;
        int v = c < nchunks ? chunk_cnt[(size_t)c * k + j] : 0;
        // block inclusive scan
        int x = v;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) red[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int w = lane < (int)(blockDim.x >> 5) ? red[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            red[lane] = w;
        }
        __syncthreads();
        int incl = x + (wid > 0 ? red[wid - 1] : 0);
        if (c < nchunks) chunk_cnt[(size_t)c * k + j] = carry + incl - v;
        int total = red[(blockDim.x >> 5) - 1];
        __syncthreads();
        carry += total;
    }
    if (threadIdx.x == 0) counts[j] = carry;
}

// offsets, sum_class and (for the tensor-core Gram) offsets of the clusters
// padded to multiples of 64 members.
__global__ void k_seg_offsets(const int32_t* __restrict__ counts, int k, int32_t* __restrict__ offsets,
                              int32_t* __restrict__ sum_class, int64_t* __restrict__ poff) {
    if (threadIdx.x == 0) {
        int acc = 0, nz = 0;
        int64_t pacc = 0;
        for (int j = 0; j < k; ++j) {
            offsets[j] = acc;
            if (poff) poff[j] = pacc;
            acc += counts[j];
            pacc += (counts[j] + 63) / 64 * 64;
            nz += counts[j] != 0;
        }
        *sum_class = nz;
    }
}

__global__ void __launch_bounds__(SEG_BLOCK) k_seg_scatter(const int32_t* __restrict__ labels, int64_t n, int k,
                                                           const int32_t* __restrict__ chunk_base,
                                                           const int32_t* __restrict__ offsets,
                                                           int32_t* __restrict__ perm) {
    extern __shared__ int sm[];
    int* running = sm;              // k
    int* wcnt = sm + k;             // 8 * k
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * SEG_CHUNK;
    for (int j = tid; j < k; j += SEG_BLOCK) running[j] = offsets[j] + chunk_base[(size_t)blockIdx.x * k + j];
    const unsigned lt = (1u << lane) - 1u;
    for (int r0 = 0; r0 < SEG_CHUNK; r0 += SEG_BLOCK) {
        for (int e = tid; e < 8 * k; e += SEG_BLOCK) wcnt[e] = 0;
        __syncthreads();
        const int64_t i = base + r0 + tid;
        int lab = i < n ? labels[i] : -1;
        if (lab >= k) lab = -1;
        const unsigned peers = __match_any_sync(0xffffffffu, lab);
        const int rank = __popc(peers & lt);
        if (lab >= 0 && rank == 0) wcnt[wid * k + lab] = __popc(peers);
        __syncthreads();
        if (lab >= 0) {
            int pos = running[lab] + rank;
            for (int w = 0; w < wid; ++w) pos += wcnt[w * k + lab];
            perm[pos] = (int32_t)i;
        }
        __syncthreads();
        for (int j = tid; j < k; j += SEG_BLOCK) {
            int add = 0;
#pragma unroll
            for (int w = 0; w < 8; ++w) add += wcnt[w * k + j];
            running[j] += add;
        }
        // the next pass zeroes wcnt: every thread must have read it first
        __syncthreads();
    }
}

// ---------------------------------------------------------------- gate
// compat: thrust::reduce(c, c+m, 0) accumulates in int, truncating each value
// (shapeExtract.cuh:1131), gate = |sum| > 1e-16; canonical: any non-zero value.
__global__ void k_gate(const float* __restrict__ C, int m, int mode, uint8_t* __restrict__ gate) {
    __shared__ double red[32];
    const float* c = C + (size_t)blockIdx.x * m;
    double s = 0;
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        float v = c[t];
        if (mode == TC_MODE_COMPAT) s += (double)(long long)(int)v;  // cvt.rzi saturates
        else s += (v != 0.f) ? 1.0 : 0.0;
    }
    s = block_sum_d(s, red);
    if (threadIdx.x == 0) gate[blockIdx.x] = (mode == TC_MODE_COMPAT) ? (fabs(s) > 1e-16) : (s > 0);
}

// ---------------------------------------------------------------- SIMT Gram
// 64x64 output tiles of the upper triangle, 256 threads x 4x4 outputs, K in
// 32-row slabs; FP32 sums of 256 rows are folded into a compensated total.
__global__ void __launch_bounds__(256) k_gram_simt(const float* __restrict__ Y, const int32_t* __restrict__ counts,
                                                   const int32_t* __restrict__ offsets, int m, int ld, int nt,
                                                   float* __restrict__ S, const uint8_t* __restrict__ skip) {
    __shared__ __align__(16) float As[32][64];
    __shared__ __align__(16) float Bs[32][64];
    const int c = blockIdx.y;
    const int cnt = counts[c];
    if (cnt == 0 || (skip && skip[c])) return;
    int t = blockIdx.x, ta = 0;
    while (t >= nt - ta) { t -= nt - ta; ++ta; }
    const int tb = ta + t;
    const int a0 = ta * 64, b0 = tb * 64;
    const float* Yc = Y + (size_t)offsets[c] * m;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    float acc[4][4], tot[4][4], cmp[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = tot[i][j] = cmp[i][j] = 0.f;
    int slab = 0;
    for (int k0 = 0; k0 < cnt; k0 += 32, ++slab) {
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            int idx = tid + e * 256;
            int kk = idx >> 6, ii = idx & 63;
            int row = k0 + kk;
            bool ok = row < cnt;
            As[kk][ii] = (ok && a0 + ii < m) ? Yc[(size_t)row * m + a0 + ii] : 0.f;
            Bs[kk][ii] = (ok && b0 + ii < m) ? Yc[(size_t)row * m + b0 + ii] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; ++kk) {
            float4 av = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
            float4 bv = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
            float a[4] = {av.x, av.y, av.z, av.w}, b[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
        if ((slab & 7) == 7 || k0 + 32 >= cnt) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {  // Kahan: tot += acc
                    float y = acc[i][j] - cmp[i][j];
                    float tt = tot[i][j] + y;
                    cmp[i][j] = (tt - tot[i][j]) - y;
                    tot[i][j] = tt;
                    acc[i][j] = 0.f;
                }
        }
    }
    float* Sc = S + (size_t)c * m * ld;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int a = a0 + ty * 4 + i, b = b0 + tx * 4 + j;
            if (a < m && b < m) {
                Sc[(size_t)a * ld + b] = tot[i][j];
                Sc[(size_t)b * ld + a] = tot[i][j];
            }
        }
}

// ---------------------------------------------------------------- centring terms
// r[c][a] = sum_b S[c][a][b] (FP64), tot[c] = sum_a r[c][a]
__global__ void k_rowsum(const float* __restrict__ S, const int32_t* __restrict__ counts, int m, int ld,
                         double* __restrict__ r, double* __restrict__ tot) {
    const int c = blockIdx.y;
    if (counts[c] == 0) return;
    const int lane = threadIdx.x & 31;
    const int a = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (a >= m) return;
    const float* row = S + ((size_t)c * m + a) * ld;
    float s = 0.f;
    for (int b = lane; b < m; b += 32) s += row[b];
    double d = s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) r[(size_t)c * m + a] = d;
}

// tot[c] = sum_a r[c][a] in a fixed order (no atomics: the result, and the
// power iteration that uses it, is the same on every run)
__global__ void k_rowsum_total(const double* __restrict__ r, const int32_t* __restrict__ counts, int m,
                               double* __restrict__ tot) {
    __shared__ double red[32];
    const int c = blockIdx.x;
    if (counts[c] == 0) {
        if (threadIdx.x == 0) tot[c] = 0.0;
        return;
    }
    double s = 0.0;
    for (int a = threadIdx.x; a < m; a += blockDim.x) s += r[(size_t)c * m + a];
    s = block_sum_d(s, red);
    if (threadIdx.x == 0) tot[c] = s;
}

// ---------------------------------------------------------------- memo of unchanged clusters
// Every stage of the extraction is deterministic per cluster: a centroid depends
// only on the cluster's members (the set, taken in series order by the stable
// segment), their alignment shifts (computed against the centroid given) and that
// centroid.  So on the same series, a cluster whose members and input centroid equal
// those of the previous extraction gets that extraction's output again, bit for bit:
// its shifts, gather, Gram and power iteration are left out and the output is copied.
// The previous extraction's labels and its input and output centroids stay in the
// workspace, and the comparison runs on the device, so a replayed CUDA graph of the
// extraction keeps working.  Once the loop settles, most clusters keep their members
// from one iteration to the next.

// dirty[c] = 1 where a series entered or left cluster c since the previous extraction
__global__ void k_memo_dirty(const int32_t* __restrict__ L, const int32_t* __restrict__ Lm, int64_t n, int k,
                             uint8_t* __restrict__ dirty) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int a = L[i], b = Lm[i];
        if (a != b) {  // every writer stores 1
            if ((unsigned)a < (unsigned)k) dirty[a] = 1;
            if ((unsigned)b < (unsigned)k) dirty[b] = 1;
        }
    }
}

// One block per cluster: skip[c] when the previous extraction is complete, c kept its
// members and its input centroid is bitwise the previous one; the shift pass's gate
// closes for skipped clusters.  The input centroids are kept in cin_now.
__global__ void k_memo_skip(const float* __restrict__ C, float* __restrict__ cin_now,
                            const float* __restrict__ cin_prev, int m, const uint8_t* __restrict__ dirty,
                            const int* __restrict__ valid, const uint8_t* __restrict__ gate,
                            uint8_t* __restrict__ skip, uint8_t* __restrict__ gate_shift,
                            unsigned long long* __restrict__ count) {
    const int c = blockIdx.x;
    const uint32_t* a = reinterpret_cast<const uint32_t*>(C) + (size_t)c * m;
    const uint32_t* b = reinterpret_cast<const uint32_t*>(cin_prev) + (size_t)c * m;
    bool same = true;
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        const uint32_t v = a[t];
        cin_now[(size_t)c * m + t] = __uint_as_float(v);
        same = same && v == b[t];
    }
    same = __syncthreads_and(same) != 0;
    if (threadIdx.x == 0) {
        const bool sk = *valid != 0 && !dirty[c] && same;
        skip[c] = sk;
        gate_shift[c] = gate[c] && !sk;
        if (c == 0) atomicAdd(count, 1ull);
        atomicAdd(count + 1, 1ull);
        if (sk) atomicAdd(count + 2, 1ull);
    }
}

// After the extraction: skipped clusters get the previous output; the memo takes
// this extraction's input and output centroids and is marked complete (the labels
// are copied after this kernel).
__global__ void k_memo_finish(float* __restrict__ C, float* __restrict__ cout_prev, float* __restrict__ cin_prev,
                              const float* __restrict__ cin_now, const uint8_t* __restrict__ skip, int m,
                              int* __restrict__ valid) {
    const int c = blockIdx.x;
    const bool sk = skip[c] != 0;
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        const size_t e = (size_t)c * m + t;
        if (sk) C[e] = cout_prev[e];
        else cout_prev[e] = C[e];
        cin_prev[e] = cin_now[e];
    }
    if (c == 0 && threadIdx.x == 0) *valid = 1;
}

struct MemoBuffers {
    int32_t* labels;
    float *cin_prev, *cout_prev, *cin_now;
    uint8_t *dirty, *skip, *gate_shift;
    int* valid;
    unsigned long long* count;
};

static MemoBuffers memo_buffers(tc_ctx* ctx, int64_t n, int k, int m, cudaStream_t s) {
    Workspace& ws = ctx->ws;
    MemoBuffers b;
    b.labels = ws.memo_labels.as<int32_t>(std::max<int64_t>(n, 1));
    float* c = ws.memo_c.as<float>((size_t)3 * k * m);
    b.cin_prev = c;
    b.cout_prev = c + (size_t)k * m;
    b.cin_now = c + (size_t)2 * k * m;
    const size_t fb = ((size_t)3 * k + 15) / 16 * 16;
    uint8_t* f = ws.memo_flags.as<uint8_t>(fb + 16);
    b.dirty = f;
    b.skip = f + k;
    b.gate_shift = f + 2 * k;
    b.valid = reinterpret_cast<int*>(f + fb);
    if (!ctx->memo.counters || !ws.memo_count.p) {  // outside graph capture (memo_prepare comes first)
        b.count = ws.memo_count.as<unsigned long long>(3);
        TC_CUDA(cudaMemsetAsync(b.count, 0, 3 * sizeof(unsigned long long), s));
        ctx->memo.counters = true;
    }
    b.count = static_cast<unsigned long long*>(ws.memo_count.p);
    return b;
}

static bool memo_keyed_for(const tc_ctx* ctx, const ExtractArgs& a) {
    const MemoState& ms = ctx->memo;
    return ms.keyed && ms.x == a.x && ms.n == a.n && ms.m == a.m && ms.k == a.k && ms.mode == a.mode &&
           ms.precision == a.precision && ms.cal_select == a.cal_select;
}

void memo_prepare(tc_ctx* ctx, const ExtractArgs& a, cudaStream_t s) {
    if (!a.memo || a.n <= 0) return;
    const MemoBuffers b = memo_buffers(ctx, a.n, a.k, a.m, s);  // allocated here, before any capture
    if (memo_keyed_for(ctx, a)) return;
    MemoState& ms = ctx->memo;
    TC_CUDA(cudaMemsetAsync(b.valid, 0, sizeof(int), s));
    ms.x = a.x;
    ms.n = a.n;
    ms.m = a.m;
    ms.k = a.k;
    ms.mode = a.mode;
    ms.precision = a.precision;
    ms.cal_select = a.cal_select;
    ms.keyed = true;
}

void power_eigvecs(tc_ctx* ctx, const float* S, int ld, const double* r, const double* tot, const int32_t* counts,
                   const int32_t* offsets, const float* seg, bool lead_rows, int k, int m, int mode, int tmax,
                   double tol, const float* vinit, const int32_t* vok, int tmax_sq, float* C, cudaStream_t s,
                   const uint8_t* skip);

// ---------------------------------------------------------------- driver
// Everything on the stream, with no host synchronisation (capturable in a CUDA
// graph): the alignment shifts are computed for every series whose centroid's
// gate is open (the kernel skips the others), and the flags stay on the device:
// scal[0] = sum_class, scal[1] = a label outside [0, k), Gram error word at aux+48.
void extract_async(tc_ctx* ctx, const ExtractArgs& a, cudaStream_t s) {
    Workspace& ws = ctx->ws;
    const int64_t n = a.n;
    const int m = a.m, k = a.k;
    TC_REQUIRE(k >= 1 && k <= MAX_K, TC_ERR_UNSUPPORTED, "k must be in [1, 1024]");
    TC_REQUIRE(m >= 2 && m <= 8192, TC_ERR_UNSUPPORTED, "series length must be in [2, 8192]");
    const int nchunks = ceil_div(n, SEG_CHUNK);
    int32_t* perm = ws.perm.as<int32_t>(std::max<int64_t>(n, 1));
    int32_t* chunk = ws.chunk_counts.as<int32_t>((size_t)std::max(nchunks, 1) * k);
    int32_t* counts = a.counts ? a.counts : ws.counts.as<int32_t>(k);
    int32_t* offsets = ws.offsets.as<int32_t>(k);
    int64_t* poff = ws.gram_poff.as<int64_t>(k);
    uint8_t* gate = ws.gate.as<uint8_t>(k);
    int32_t* scal = ws.scal.as<int32_t>(16);
    float* seg = nullptr;  // row-major members in cluster order (only without the fused gather)
    const int ld = (m + 3) & ~3;  // Gram row pitch: rows stream as float4
    float* S = ws.gram.as<float>((size_t)k * m * ld);
    double* rs = ws.rowsum.as<double>((size_t)k * m + k);
    double* tot = rs + (size_t)k * m;
    int* gram_err = reinterpret_cast<int*>(ws.aux.as<char>(64) + 48);

    TC_CUDA(cudaMemsetAsync(scal, 0, sizeof(int32_t) * 16, s));
    if (n > 0) {
        k_seg_count<<<nchunks, SEG_BLOCK, k * sizeof(int), s>>>(a.labels, n, k, chunk, scal + 1);
        TC_CHECK_LAUNCH();
    } else {
        TC_CUDA(cudaMemsetAsync(chunk, 0, sizeof(int32_t) * k, s));
    }
    k_seg_scan_chunks<<<k, 256, 0, s>>>(chunk, std::max(nchunks, 1), k, counts);
    TC_CHECK_LAUNCH();
    k_seg_offsets<<<1, 32, 0, s>>>(counts, k, offsets, scal, poff);
    TC_CHECK_LAUNCH();
    if (n > 0) {
        size_t smem = (size_t)9 * k * sizeof(int);
        allow_max_dynamic_smem(k_seg_scatter);
        k_seg_scatter<<<nchunks, SEG_BLOCK, smem, s>>>(a.labels, n, k, chunk, offsets, perm);
        TC_CHECK_LAUNCH();
    }
    k_gate<<<k, 256, 0, s>>>(a.C, m, a.mode, gate);
    TC_CHECK_LAUNCH();

    // memo of unchanged clusters: only on fixed series without caller shifts, and not
    // with the repeated squaring (its launches cover all clusters together)
    const bool squaring =
        (a.cal_select || a.mode == TC_MODE_CANONICAL) && power_squaring_supported(m, k, ctx->sm_count);
    const bool memo = a.memo && !a.shift && !squaring && n > 0 && !std::getenv("TIMESC_NO_MEMO") &&
                      memo_keyed_for(ctx, a);  // memo_prepare sized and keyed it
    MemoBuffers mb{};
    const uint8_t* skip = nullptr;
    const uint8_t* gate_shift = gate;
    if (memo) {
        mb = memo_buffers(ctx, n, k, m, s);
        TC_CUDA(cudaMemsetAsync(mb.dirty, 0, k, s));
        const int g = (int)std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->sm_count * 8);
        k_memo_dirty<<<g, 256, 0, s>>>(a.labels, mb.labels, n, k, mb.dirty);
        TC_CHECK_LAUNCH();
        k_memo_skip<<<k, 128, 0, s>>>(a.C, mb.cin_now, mb.cin_prev, m, mb.dirty, mb.valid, gate, mb.skip,
                                      mb.gate_shift, mb.count);
        TC_CHECK_LAUNCH();
        skip = mb.skip;
        gate_shift = mb.gate_shift;
    }

    const int32_t* shift = a.shift;
    if (!shift && n > 0) {
        // alignment shifts of each series against its own centroid (sbd3D, SBD.cuh:69-85)
        const int F = fft_size(m, a.mode);
        float2* spec = ws.spectra.as<float2>((size_t)k * (F / 2 + 1));
        launch_centroid_spectra(ctx, a.C, k, m, F, spec, s);
        int32_t* sh = ws.shift.as<int32_t>(std::max<int64_t>(n, 1));
        AssignArgs aa{};
        aa.x = a.x;
        aa.spec = spec;
        aa.n = n;
        aa.m = m;
        aa.k = k;
        aa.F = F;
        aa.clamp2 = 0;
        aa.fixed = a.labels;
        aa.gate = gate_shift;  // skipped clusters need no shifts
        aa.shift = sh;
        launch_assign_fft(ctx, aa, s);
        shift = sh;
    }
    // gather + align + re-normalise: straight into the tensor-core Gram's transposed
    // operand when it is used (m <= 1024), else into the row-major segment buffer
    const bool tc_gram = gram_tc_supported(m, a.precision);
    const bool fused = tc_gram && gather_transposed_supported(m);
    if (tc_gram && squaring)  // one operand buffer for both uses, sized before either is written
        ws.gram_yt.get(std::max(gram_operand_bytes(n, k, m, a.precision), power_squaring_operand_bytes(k, m)));
    const float* lead = nullptr;
    if (fused) {
        const GramOperand op = gram_tc_operand(ctx, n, k, m, a.precision);
        float* first = ws.first.as<float>((size_t)k * m);
        launch_gather_norm_t(a.x, perm, a.labels, shift, gate_shift, offsets, counts, k, poff, n, m, op.fmt == 1,
                             op.YT, op.YTlo, op.Pp, first, s, skip);
        lead = first;
    } else {
        seg = ws.seg.as<float>((size_t)std::max<int64_t>(n, 1) * m);
        // skipped clusters' rows are gathered unaligned (their shifts were not computed) and not used
        launch_gather_norm(a.x, perm, a.labels, shift, gate_shift, n, m, seg, ctx->sm_count, s);
        lead = seg;
    }

    // Gram (padding columns b in [m, ld) stay zero)
    if (ld != m) TC_CUDA(cudaMemsetAsync(S, 0, sizeof(float) * (size_t)k * m * ld, s));
    TC_CUDA(cudaMemsetAsync(gram_err, 0, sizeof(int), s));
    const int nt = ceil_div(m, 64);
    if (tc_gram) {
        launch_gram_tc(ctx, fused ? nullptr : seg, counts, offsets, poff, n, k, m, ld, a.precision, S, gram_err, s,
                       skip);
    } else {
        dim3 g(nt * (nt + 1) / 2, k);
        k_gram_simt<<<g, 256, 0, s>>>(seg, counts, offsets, m, ld, nt, S, skip);
        TC_CHECK_LAUNCH();
    }
    k_rowsum<<<dim3(ceil_div(m, 8), k), 256, 0, s>>>(S, counts, m, ld, rs, tot);
    TC_CHECK_LAUNCH();
    k_rowsum_total<<<k, 256, 0, s>>>(rs, counts, m, tot);
    TC_CHECK_LAUNCH();

    // power iteration: compat runs at most m steps (the reference's fixed count),
    // stopping early only once a cluster's vector will move by less than 3e-8 in the
    // steps left (geometric tail of the measured contraction) or has reached rounding
    // level; cal_select=1 / canonical converge fully (the reference's syevd result).
    const bool full = a.cal_select || a.mode == TC_MODE_CANONICAL;
    const int tmax = full ? std::max(4 * m, 200) : m;
    const double tol = full ? 5e-7 : 1e-6;
    // The converging forms start from M^e v_0, e = 2^J >= tmax, by repeated squaring on
    // the tensor cores, and step on until the convergence test passes.  The compat form
    // keeps its m plain steps: an error eps in the j-th square is applied m/2^j times, so
    // with FP32 accumulation (eps ~ 1e-6) a cluster whose top two eigenvalues nearly tie
    // would drift by ~m*eps from the m-step vector, which the steps themselves hold to
    // ~1e-7 per step.
    SquaringResult sq;
    int tmax_sq = 0;
    if (squaring) {
        int64_t e = 1;
        while (e < tmax) e <<= 1;
        tmax_sq = tmax;
        sq = power_squaring(ctx, S, ld, rs, tot, counts, k, m, e, gram_err, s);
    }
    power_eigvecs(ctx, S, ld, rs, tot, counts, offsets, lead, fused, k, m, a.mode, tmax, tol, sq.vec, sq.ok, tmax_sq,
                  a.C, s, skip);
    if (memo) {
        k_memo_finish<<<k, 128, 0, s>>>(a.C, mb.cout_prev, mb.cin_prev, mb.cin_now, mb.skip, m, mb.valid);
        TC_CHECK_LAUNCH();
        TC_CUDA(cudaMemcpyAsync(mb.labels, a.labels, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
    }
}

int run_extract(tc_ctx* ctx, const ExtractArgs& a, cudaStream_t s) {
    memo_prepare(ctx, a, s);
    extract_async(ctx, a, s);
    int32_t h_sc[2] = {0, 0};
    int h_err = 0;
    TC_CUDA(cudaMemcpyAsync(h_sc, ctx->ws.scal.p, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaMemcpyAsync(&h_err, static_cast<char*>(ctx->ws.aux.p) + 48, sizeof(int), cudaMemcpyDeviceToHost, s));
    TC_CUDA(cudaStreamSynchronize(s));
    if (h_sc[1] || h_err) memo_invalidate(ctx);  // this extraction's outputs are not complete
    TC_REQUIRE(h_sc[1] == 0, TC_ERR_ARG, "a label is outside [0, k)");
    TC_REQUIRE(h_err == 0, TC_ERR_TIMEOUT, "tensor-core Gram: a pipeline wait ran out");
    return h_sc[0];
}

}  // namespace tc
