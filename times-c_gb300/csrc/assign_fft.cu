// Fused SBD assignment on SIMT FP32 (the "plain FP32" form).
//
// Replaces NCC_3D + get_pos_idx (ncc.cuh:469-517, kshape.cuh:35-96).  The
// reference materialises n*k*F complex products and n*k*(2m-1) correlations in
// HBM; here one team of threads per series keeps the series spectrum in
// registers, multiplies it by each centroid spectrum (resident in shared memory
// when they fit), runs the inverse transform in registers + shared memory and
// reduces the max NCC over the valid lags on the fly.  Only (label, distance,
// shift) per series reach HBM.
#include <curand_kernel.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "sbd_core.cuh"
#include "tc_internal.h"

using namespace tcfft;

namespace tc {

// ------------------------------------------------------------------ tables
// twN[e] = exp(-2 pi i e/N), twF[e] = exp(-2 pi i e/(2N)), e in [0, N), from the
// FP64 sincospi rounded to float.  The context's tables and the allocation-free
// entry point's both come from this kernel, so the two paths transform with
// identical twiddles.
__global__ void k_twiddles(float2* twN, float2* twF, int N) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < N) {
        double s, c;
        sincospi(-2.0 * (double)e / (double)N, &s, &c);
        twN[e] = make_float2((float)c, (float)s);
        sincospi(-(double)e / (double)N, &s, &c);
        twF[e] = make_float2((float)c, (float)s);
    }
}

const FftTables& fft_tables(tc_ctx* ctx, int F) {
    for (auto* t : ctx->fft)
        if (t->F == F) return *t;
    auto* t = new FftTables();
    t->F = F;
    const int N = F / 2;
    // built once per context and length, finished before the first use on any
    // stream (the legacy stream, as a synchronous copy would be; not while
    // another thread captures a graph)
    std::lock_guard<std::recursive_mutex> lk(capture_mutex());
    float2* dN = t->twN.as<float2>(N);
    float2* dF = t->twF.as<float2>(N);
    k_twiddles<<<ceil_div(N, 256), 256, 0, 0>>>(dN, dF, N);
    TC_CHECK_LAUNCH();
    TC_CUDA(cudaStreamSynchronize(0));
    ctx->fft.push_back(t);
    return *t;
}

// ------------------------------------------------------------------ team primitives
// Lanes of the calling thread's team inside its warp (all lanes for T >= 32).
template <int T>
__device__ __forceinline__ unsigned team_mask() {
    if constexpr (T >= 32) return 0xffffffffu;
    else return ((1u << T) - 1u) << ((threadIdx.x & 31) & ~(T - 1));
}

template <int T>
__device__ __forceinline__ void team_sync(int team) {
    if constexpr (T <= 32) {
        __syncwarp(team_mask<T>());
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(team + 1), "r"(T) : "memory");
    }
}

struct TeamScratch {
    double sum[16];
    float val[16];
    int u[16];
};

// Sum over the team (compensated FP32 within warps, FP64 across warps); every
// thread gets the result.
template <int T>
__device__ __forceinline__ double team_sum(float x, int team, int tid, TeamScratch* scr) {
    constexpr int W = T < 32 ? T : 32;
    float s = x, c = 0.f;  // value = s - c
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(team_mask<T>(), s, o, W), c2 = __shfl_xor_sync(team_mask<T>(), c, o, W);
        const float t = s + s2, bp = t - s;
        const float err = (s - (t - bp)) + (s2 - bp);
        s = t;
        c = c + c2 - err;
    }
    double v = (double)s - (double)c;
    if constexpr (T > 32) {
        if ((tid & 31) == 0) scr->sum[tid >> 5] = v;
        team_sync<T>(team);
        v = 0;
#pragma unroll
        for (int w = 0; w < T / 32; ++w) v += scr->sum[w];
        team_sync<T>(team);
    }
    return v;
}

// (val, u) max over the team (larger u wins ties); every thread of the team gets it.
template <int T>
__device__ __forceinline__ LagMax team_max(LagMax lm, int team, int tid, TeamScratch* scr) {
    constexpr int W = T < 32 ? T : 32;
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
        float ov = __shfl_xor_sync(team_mask<T>(), lm.val, o, W);
        int ou = __shfl_xor_sync(team_mask<T>(), lm.u, o, W);
        lm.take(ov, ou);
    }
    if constexpr (T > 32) {
        if ((tid & 31) == 0) {
            scr->val[tid >> 5] = lm.val;
            scr->u[tid >> 5] = lm.u;
        }
        team_sync<T>(team);
        lm.val = scr->val[0];
        lm.u = scr->u[0];
        for (int w = 1; w < T / 32; ++w) lm.take(scr->val[w], scr->u[w]);
    }
    return lm;
}

// Stockham passes PS..NPASS-1 over the team buffer.
template <int N, int PS, bool INV, bool STORE_LAST, class Out>
__device__ __forceinline__ void run_passes(float2* buf, int tid, int team, const float2* __restrict__ twN, Out& out) {
    typedef Core<N> C;
    typename C::template Pass<PS> st;
    st.load(buf, tid);
    constexpr bool last = PS + 1 >= Plan<N>::NPASS;
    if constexpr (!last || STORE_LAST) {
        team_sync<C::T>(team);
        st.template compute<INV>(tid, twN);
        st.store(buf, tid);
        team_sync<C::T>(team);
    } else {
        st.template compute<INV>(tid, twN);
        out(st, tid);
    }
    if constexpr (!last) run_passes<N, PS + 1, INV, STORE_LAST>(buf, tid, team, twN, out);
}

struct NoOut {
    template <class P>
    __device__ void operator()(const P&, int) const {}
};

// Forward transform of one row into the thread's spectrum registers.
template <int N>
__device__ __forceinline__ void forward_row(const float* __restrict__ x, int m, float2* buf, int tid, int team,
                                            const float2* __restrict__ twN, const float2* __restrict__ twF,
                                            TeamScratch* scr, double extra, float2 (&xh)[2][Plan<N>::R0],
                                            float& xhN, double& nrm2) {
    typedef Core<N> C;
    float2 v[2][C::R0];
    float ss = C::fwd_load(x, m, tid, v);
    nrm2 = team_sum<C::T>(ss, team, tid, scr);
    C::template pass0_store<false>(v, tid, buf);
    team_sync<C::T>(team);
    NoOut no;
    run_passes<N, 1, false, true>(buf, tid, team, twN, no);
    float s = nrm2 > 0 ? (float)(1.0 / (std::sqrt(nrm2) * extra)) : 0.f;
    C::post(buf, tid, twF, s, xh, xhN);
    team_sync<C::T>(team);
}

template <int N>
struct Cfg {
    static constexpr int T = Plan<N>::T;
    static constexpr int BLOCK = T > 512 ? T : 512;
    static constexpr int TEAMS = BLOCK / T;
    static constexpr size_t BUF_BYTES = (size_t)BufSize<N>::value * sizeof(float2);
    static size_t smem(int k, bool csmem) {
        size_t s = (size_t)TEAMS * (BUF_BYTES + sizeof(TeamScratch));
        if (csmem) s += ((size_t)k * (N + 1) * sizeof(float2) + 15) / 16 * 16;  // as laid out in the kernel
        return s;
    }
};

// ------------------------------------------------------------------ centroid spectra
template <int N>
__global__ void __launch_bounds__(Plan<N>::T) k_centroid_spectra(const float* __restrict__ C, int m,
                                                                 const float2* __restrict__ twN,
                                                                 const float2* __restrict__ twF,
                                                                 float2* __restrict__ spec) {
    typedef Core<N> Co;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* buf = reinterpret_cast<float2*>(smem);
    TeamScratch* scr = reinterpret_cast<TeamScratch*>(smem + Cfg<N>::BUF_BYTES);
    const int tid = threadIdx.x, j = blockIdx.x;
    float2 xh[2][Co::R0];
    float xhN = 0.f;
    double nrm2;
    forward_row<N>(C + (size_t)j * m, m, buf, tid, 0, twN, twF, scr, 2.0 * N, xh, xhN, nrm2);
    float2* S = spec + (size_t)j * (N + 1);
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int r = 0; r < Co::R0; ++r) S[Co::j_of(tid, b) + r * Co::NB0] = xh[b][r];
    if (tid == 0) S[N] = make_float2(xhN, 0.f);
}

// ------------------------------------------------------------------ assignment
struct AssignParams {
    const float* x;
    const float2* spec;
    const float2* twN;
    const float2* twF;
    int64_t n;
    int m, k, F, clamp2;
    const int32_t* fixed;
    const uint8_t* gate;  // with fixed: series whose centroid's gate is closed get shift 0, no work
    int32_t* labels;
    float* dist;
    int32_t* shift;
    const int32_t* old_labels;
    int32_t* changed;
    double* dist_sum;
    // screened assignment: only centroids cand[i][0 .. ncand[i]) (ascending; -1: all)
    const int32_t* cand;
    const int32_t* ncand;
    // lower bounds [n][k] on the exact distances: d32 - lb_eps for every pair evaluated
    float* lb_out;
    float lb_eps;
    // per series the label and distance this pass leaves (written when set); with
    // reuse, a series whose only candidate is that label, of a centroid unchanged
    // (same[j]) since, keeps that distance without being transformed
    float* prev_dist;
    int32_t* prev_label;
    const uint8_t* same;
    int reuse;
};

// Max NCC over the valid lags with the lag of the first maximum in sbd3D's order
// (needed for alignment shifts).
struct LagOut {
    LagMax lm;
    int m, F;
    template <class P>
    __device__ void operator()(const P& st, int tid) {
        st.each_output(tid, [this](int o, float2 v) {
            lag_take(lm, 2 * o, v.x, m, F);
            lag_take(lm, 2 * o + 1, v.y, m, F);
        });
    }
};

// Max NCC only: the thread's valid outputs are a fixed bit mask of its slots.
struct MaxOut {
    float val;
    unsigned mask;
    template <class P>
    __device__ void operator()(const P& st, int tid) {
        st.each_output_slot(tid, [this](int e, float2 v) {
            if (mask & (1u << (2 * e))) val = fmaxf(val, v.x);
            if (mask & (2u << (2 * e))) val = fmaxf(val, v.y);
        });
    }
};

template <int N, bool CSMEM, bool SHIFT>
__global__ void __launch_bounds__(Cfg<N>::BLOCK, 1) k_assign_fft(AssignParams p) {
    typedef Core<N> Co;
    constexpr int T = Co::T, TEAMS = Cfg<N>::TEAMS;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* cur = smem;
    float2* cspec = reinterpret_cast<float2*>(cur);
    if (CSMEM) cur += ((size_t)p.k * (N + 1) * sizeof(float2) + 15) / 16 * 16;
    const int team = threadIdx.x / T, tid = threadIdx.x % T;
    float2* buf = reinterpret_cast<float2*>(cur) + (size_t)team * BufSize<N>::value;
    TeamScratch* scr = reinterpret_cast<TeamScratch*>(cur + (size_t)TEAMS * Cfg<N>::BUF_BYTES) + team;

    if (CSMEM) {
        const size_t nv = (size_t)p.k * (N + 1);
        for (size_t e = threadIdx.x; e < nv; e += blockDim.x) cspec[e] = p.spec[e];
        __syncthreads();
    }

    const unsigned vmask = Co::template Pass<Plan<N>::NPASS - 1>::valid_mask(tid, p.m, p.F);
    double dsum = 0.0;
    int nchg = 0;
    const int64_t stride = (int64_t)gridDim.x * TEAMS;
    for (int64_t i = (int64_t)blockIdx.x * TEAMS + team; i < p.n; i += stride) {
        if (p.fixed && p.gate && !p.gate[p.fixed[i]]) {  // uniform over the team
            if (tid == 0 && p.shift) p.shift[i] = 0;
            continue;
        }
        if (p.reuse) {  // uniform over the team: every thread reads the same values
            const int32_t* cl = p.cand + (size_t)i * SCREEN_CAP;
            const int j = cl[0];
            if (screen_list_len(cl, p.ncand[i], p.k) == 1 && j == p.prev_label[i] && p.same[j]) {
                if (tid == 0) {  // the distance the same kernel computed for this series and centroid
                    const float d = p.prev_dist[i];
                    if (p.labels) p.labels[i] = j;
                    if (p.dist) p.dist[i] = d;
                    if (p.lb_out) p.lb_out[(size_t)i * p.k + j] = __fsub_rd(d, p.lb_eps);
                    dsum += (double)d;
                    if (p.old_labels && p.old_labels[i] != j) ++nchg;
                }
                continue;
            }
        }
        float2 xh[2][Co::R0];
        float xhN = 0.f;
        double nrm2;
        forward_row<N>(p.x + (size_t)i * p.m, p.m, buf, tid, team, p.twN, p.twF, scr, 1.0, xh, xhN, nrm2);
        // max NCC of this series against centroid c (every thread of the team gets it)
        auto eval = [&](int c) -> LagMax {
            float2 v[2][Co::R0];
            if (CSMEM) {
                const float2* S = cspec + (size_t)c * (N + 1);
                Co::product(xh, xhN, [S](int f) { return S[f]; }, tid, p.twF, v);
            } else {
                const float2* S = p.spec + (size_t)c * (N + 1);
                Co::product(xh, xhN, [S](int f) { return __ldg(S + f); }, tid, p.twF, v);
            }
            Co::template pass0_store<true>(v, tid, buf);
            team_sync<T>(team);
            LagMax lm;
            if constexpr (SHIFT) {
                LagOut out;
                out.lm.init();
                out.m = p.m;
                out.F = p.F;
                run_passes<N, 1, true, false>(buf, tid, team, p.twN, out);
                lm = team_max<T>(out.lm, team, tid, scr);
            } else {
                MaxOut out;
                out.val = -3.0e38f;
                out.mask = vmask;
                run_passes<N, 1, true, false>(buf, tid, team, p.twN, out);
                lm.val = out.val;
                lm.u = 0;
                lm = team_max<T>(lm, team, tid, scr);
            }
            team_sync<T>(team);
            return lm;
        };
        auto distance = [&](const LagMax& lm) {
            float d = 1.0f - lm.val;
            if (p.clamp2 && d > 2.0f) d = 2.0f;
            return d;
        };
        float bestd = 1e10f;  // get_pos_idx: min_val = 1e10, pos = 0
        int bestj = 0, bests = 0;
        int c0 = 0, c1 = p.k;
        if (p.fixed) {
            c0 = p.fixed[i];
            c1 = c0 + 1;
        }
        // screened: the candidates in ascending order (every centroid that can be the
        // first minimum), so the first strict minimum below is the unscreened one
        const int32_t* cl = nullptr;
        int ncl = -1;
        if (p.cand) {
            cl = p.cand + (size_t)i * SCREEN_CAP;
            ncl = screen_list_len(cl, p.ncand[i], p.k);
        }
        const int iters = ncl >= 0 ? ncl : c1 - c0;
        for (int it = 0; it < iters; ++it) {
            const int c = ncl >= 0 ? cl[it] : c0 + it;
            const LagMax lm = eval(c);
            const float d = distance(lm);
            if (tid == 0 && p.lb_out) p.lb_out[(size_t)i * p.k + c] = __fsub_rd(d, p.lb_eps);
            if (d < bestd) {
                bestd = d;
                bestj = c;
                bests = -lm.u;
            }
        }
        if (tid == 0) {
            if (p.labels) p.labels[i] = bestj;
            if (p.dist) p.dist[i] = bestd;
            if (p.prev_dist) {
                p.prev_dist[i] = bestd;
                p.prev_label[i] = bestj;
            }
            if (p.shift) p.shift[i] = bests;
            dsum += (double)bestd;
            if (p.old_labels && p.old_labels[i] != bestj) ++nchg;
        }
    }
    if (tid == 0) {
        if (p.dist_sum) atomicAdd(p.dist_sum, dsum);
        if (p.changed && nchg) atomicAdd(p.changed, nchg);
    }
}

// ------------------------------------------------------------------ dispatch
template <int N>
static void centroid_spectra_n(tc_ctx* ctx, const float* C, int k, int m, float2* spec, cudaStream_t s) {
    const FftTables& tb = fft_tables(ctx, 2 * N);
    size_t sm = Cfg<N>::BUF_BYTES + sizeof(TeamScratch);
    allow_max_dynamic_smem(k_centroid_spectra<N>);
    k_centroid_spectra<N><<<k, Plan<N>::T, sm, s>>>(C, m, (const float2*)tb.twN.p, (const float2*)tb.twF.p, spec);
    TC_CHECK_LAUNCH();
}

// A launch plan of the fused assignment: centroid spectra staged in shared memory
// or read through L1, and how many blocks per SM the grid is sized for (the
// kernel loops over series, so fewer blocks means fewer, longer-lived teams).
struct AssignPlan {
    bool csmem;
    int blocks_per_sm;  // 0: the occupancy maximum
};

template <int N, bool CSMEM, bool SHIFT>
static void launch_variant(tc_ctx* ctx, const AssignParams& p, int blocks_per_sm, cudaStream_t s) {
    auto fn = k_assign_fft<N, CSMEM, SHIFT>;
    allow_max_dynamic_smem(fn);
    const size_t sm = Cfg<N>::smem(p.k, CSMEM);
    int per_sm = 0;
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, Cfg<N>::BLOCK, sm));
    per_sm = std::max(per_sm, 1);
    if (blocks_per_sm > 0) per_sm = std::min(per_sm, blocks_per_sm);
    const int64_t teams_needed = (p.n + Cfg<N>::TEAMS - 1) / Cfg<N>::TEAMS;
    const int grid = (int)std::min<int64_t>(teams_needed, (int64_t)ctx->sm_count * per_sm);
    fn<<<grid, Cfg<N>::BLOCK, sm, s>>>(p);
}

template <int N, bool SHIFT>
static void launch_plan(tc_ctx* ctx, const AssignParams& p, const AssignPlan& pl, cudaStream_t s) {
    if (pl.csmem) launch_variant<N, true, SHIFT>(ctx, p, pl.blocks_per_sm, s);
    else launch_variant<N, false, SHIFT>(ctx, p, pl.blocks_per_sm, s);
}

// Autotuner: the first assignment of a shape (FFT length, k, shift output) on a
// context times every candidate plan on a sample of its own series (outputs for the
// sample rows are overwritten by the real launch that follows; no counters are
// touched) and keeps the fastest for the context's later launches, graph captures
// included.  Candidates: spectra in shared memory (when they fit) or not, times
// the occupancy maximum, half of it and one block per SM.  Off with TIMESC_AUTOTUNE=0,
// and never inside a stream capture (the default plan is used then).
template <int N, bool SHIFT>
static AssignPlan tuned_plan(tc_ctx* ctx, const AssignParams& p, cudaStream_t s) {
    const bool fits = Cfg<N>::smem(p.k, true) <= ctx->smem_optin;
    const AssignPlan dflt{fits, 0};
    const uint64_t key = ((uint64_t)N << 40) | ((uint64_t)p.k << 8) | (SHIFT ? 1u : 0u) | (p.cand ? 2u : 0u);
    for (const auto& t : ctx->tuned)
        if (t.first == key) return AssignPlan{(t.second & 1u) != 0, (int)(t.second >> 1)};
    const char* env = std::getenv("TIMESC_AUTOTUNE");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    TC_CUDA(cudaStreamIsCapturing(s, &cap));
    const int64_t sample = std::min<int64_t>(p.n, (int64_t)ctx->sm_count * Cfg<N>::TEAMS * 8);
    if ((env && env[0] == '0') || cap != cudaStreamCaptureStatusNone || sample < (int64_t)ctx->sm_count * 4)
        return dflt;
    AssignParams q = p;
    q.n = sample;
    q.changed = nullptr;
    q.dist_sum = nullptr;
    std::vector<AssignPlan> cands;
    for (int cs = fits ? 1 : 0; cs >= 0; --cs)
        for (int b : {0, -2, 1}) cands.push_back(AssignPlan{cs != 0, b});
    cudaEvent_t e0, e1;
    TC_CUDA(cudaEventCreate(&e0));
    TC_CUDA(cudaEventCreate(&e1));
    float best = 3.0e38f;
    AssignPlan pick = dflt;
    for (AssignPlan c : cands) {
        if (c.blocks_per_sm == -2) {  // half the occupancy maximum
            int per_sm = 0;
            if (c.csmem)
                TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, k_assign_fft<N, true, SHIFT>, Cfg<N>::BLOCK, Cfg<N>::smem(p.k, true)));
            else
                TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, k_assign_fft<N, false, SHIFT>, Cfg<N>::BLOCK, Cfg<N>::smem(p.k, false)));
            if (per_sm < 2) continue;
            c.blocks_per_sm = per_sm / 2;
        }
        launch_plan<N, SHIFT>(ctx, q, c, s);  // warm
        TC_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 2; ++r) launch_plan<N, SHIFT>(ctx, q, c, s);
        TC_CUDA(cudaEventRecord(e1, s));
        TC_CUDA(cudaEventSynchronize(e1));
        TC_CUDA(cudaGetLastError());
        float ms = 0.f;
        TC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            pick = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->tuned.emplace_back(key, (uint32_t)(pick.csmem ? 1 : 0) | ((uint32_t)pick.blocks_per_sm << 1));
    if (std::getenv("TIMESC_TRACE"))
        std::fprintf(stderr, "timesc: autotune assignment F=%d k=%d shift=%d -> spectra %s, %d blocks/SM\n", 2 * N,
                     p.k, (int)SHIFT, pick.csmem ? "in shared memory" : "through L1", pick.blocks_per_sm);
    return pick;
}

template <int N>
static void assign_n(tc_ctx* ctx, const AssignArgs& a, cudaStream_t s) {
    const FftTables& tb = fft_tables(ctx, 2 * N);
    AssignParams p{};
    p.x = a.x;
    p.spec = a.spec;
    p.twN = (const float2*)tb.twN.p;
    p.twF = (const float2*)tb.twF.p;
    p.n = a.n;
    p.m = a.m;
    p.k = a.k;
    p.F = a.F;
    p.clamp2 = a.clamp2;
    p.fixed = a.fixed;
    p.gate = a.gate;
    p.labels = a.labels;
    p.dist = a.dist;
    p.shift = a.shift;
    p.old_labels = a.old_labels;
    p.changed = a.changed;
    p.dist_sum = a.dist_sum;
    p.cand = a.cand;
    p.ncand = a.ncand;
    p.lb_out = a.lb_out;
    p.lb_eps = a.lb_eps;
    p.prev_dist = a.prev_dist;
    p.prev_label = a.prev_label;
    p.same = a.same;
    p.reuse = a.reuse;
    TC_REQUIRE(!a.reuse || (a.cand && a.prev_dist && a.same), TC_ERR_ARG, "assignment reuse: arguments");
    const bool want_shift = a.shift != nullptr || a.fixed != nullptr;
    if (want_shift) launch_plan<N, true>(ctx, p, tuned_plan<N, true>(ctx, p, s), s);
    else launch_plan<N, false>(ctx, p, tuned_plan<N, false>(ctx, p, s), s);
    TC_CHECK_LAUNCH();
}

// ------------------------------------------------------------------ centroid movement
// delta[j] >= |c_j/|c_j| - cprev_j| (FP64 sums, rounded up with a margin for the FP32
// storage of cprev), +inf where exactly one of the two is zero; then cprev_j <- the
// unit centroid (zeros for a zero centroid).  The NCC of a series with c_j moves by
// at most delta[j] at every lag (the lags are norm-preserving or norm-reducing
// shifts of the unit centroid, Cauchy-Schwarz), and so does its distance.
// With craw: same[j] = 1 where centroid j equals craw_j bitwise, then craw_j <- c_j.
__global__ void __launch_bounds__(256) k_centroid_delta(const float* __restrict__ C, int m, float* __restrict__ cprev,
                                                        float* __restrict__ delta, float* __restrict__ craw,
                                                        uint8_t* __restrict__ same) {
    __shared__ double red[8][2];
    __shared__ double sh[2];
    const int j = blockIdx.x, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const float* c = C + (size_t)j * m;
    float* cp = cprev + (size_t)j * m;
    double a = 0, b = 0;
    bool eq = true;
    for (int t = threadIdx.x; t < m; t += 256) {
        a += (double)c[t] * c[t];
        b += (double)cp[t] * cp[t];
        if (craw) {
            const float v = c[t];
            eq = eq && __float_as_uint(v) == __float_as_uint(craw[(size_t)j * m + t]);
            craw[(size_t)j * m + t] = v;  // this thread's own element: read before written
        }
    }
    eq = __syncthreads_and(eq) != 0;
    if (craw && threadIdx.x == 0) same[j] = eq;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) { red[wid][0] = a; red[wid][1] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0, sb = 0;
        for (int w = 0; w < 8; ++w) { sa += red[w][0]; sb += red[w][1]; }
        sh[0] = sqrt(sa);
        sh[1] = sqrt(sb);
    }
    __syncthreads();
    const double nc = sh[0], np = sh[1];
    double dd = 0;
    if (nc > 0 && np > 0)
        for (int t = threadIdx.x; t < m; t += 256) {
            const double e = (double)c[t] / nc - (double)cp[t] / np;
            dd += e * e;
        }
    for (int o = 16; o > 0; o >>= 1) dd += __shfl_xor_sync(0xffffffffu, dd, o);
    __syncthreads();
    if (lane == 0) red[wid][0] = dd;
    __syncthreads();
    if (threadIdx.x == 0) {
        float dl;
        if (nc > 0 && np > 0) {
            double s2 = 0;
            for (int w = 0; w < 8; ++w) s2 += red[w][0];
            dl = __double2float_ru(sqrt(s2) * (1.0 + 1e-6) + 1e-6);
        } else {
            dl = (nc > 0) != (np > 0) ? __int_as_float(0x7f800000) : 0.f;  // +inf / unchanged zero
        }
        delta[j] = dl;
    }
    __syncthreads();  // every read of cprev is done
    for (int t = threadIdx.x; t < m; t += 256) cp[t] = nc > 0 ? (float)((double)c[t] / nc) : 0.f;
}

void launch_centroid_delta(const float* C, int k, int m, float* cprev, float* delta, cudaStream_t s, float* craw,
                           uint8_t* same) {
    k_centroid_delta<<<k, 256, 0, s>>>(C, m, cprev, delta, craw, same);
    TC_CHECK_LAUNCH();
}

#define TC_FOR_EACH_N(X) X(4) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(8192)

void launch_centroid_spectra(tc_ctx* ctx, const float* C, int k, int m, int F, float2* spec, cudaStream_t s) {
    switch (F / 2) {
#define X(n) \
    case n: centroid_spectra_n<n>(ctx, C, k, m, spec, s); return;
        TC_FOR_EACH_N(X)
#undef X
    }
    throw TcError{TC_ERR_UNSUPPORTED, "FFT length " + std::to_string(F) + " not supported (8..16384)"};
}

void launch_assign_fft(tc_ctx* ctx, const AssignArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    switch (a.F / 2) {
#define X(n) \
    case n: assign_n<n>(ctx, a, s); return;
        TC_FOR_EACH_N(X)
#undef X
    }
    throw TcError{TC_ERR_UNSUPPORTED, "FFT length " + std::to_string(a.F) + " not supported (8..16384)"};
}

// ------------------------------------------------------------------ curand label init
// kshape.cuh:16-32: curand_init(seed = series index, subsequence 0, offset 0),
// label = curand() % k (+1 in the reference; stored 0-based here).
__global__ void k_init_labels(int32_t* labels, int64_t n, int k) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        curandState_t st;
        curand_init((unsigned int)i, 0, 0, &st);
        labels[i] = (int32_t)(curand(&st) % (unsigned int)k);
    }
}

void launch_init_labels(int32_t* labels, int64_t n, int k, cudaStream_t s) {
    if (n == 0) return;
    k_init_labels<<<ceil_div(n, 256), 256, 0, s>>>(labels, n, k);
    TC_CHECK_LAUNCH();
}

}  // namespace tc

// ------------------------------------------------------------------ allocation-free assignment
// tc_sbd_assign_noalloc: the same fused SBD assignment for callers that must not
// allocate device memory on the call path (a serving loop that reserved all HBM
// up front, or a thread that cannot take cudaMalloc's implicit synchronisation).
// Its scratch (twiddle tables and centroid spectra) lives in one file-scope
// device array instead of context buffers.  No counterpart in the reference.
namespace tc {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)4 << 20;  // TC_NOALLOC_SCRATCH_BYTES
static __device__ __align__(256) float2 g_noalloc_scratch[NOALLOC_SCRATCH_BYTES / sizeof(float2)];

struct NoallocDevice {
    float2* scratch = nullptr;  // device address of g_noalloc_scratch on that device
    int sm_count = 0;
    size_t smem_optin = 0;
};
static std::mutex g_noalloc_mu;
static NoallocDevice g_noalloc_dev[256];

// Once per device, with that device current: the scratch array's device address
// (a host-side reference to the symbol is not a device address).
static NoallocDevice noalloc_setup(int dev) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    TC_REQUIRE(dev >= 0 && dev < 256, TC_ERR_ARG, "device index out of range");
    NoallocDevice& d = g_noalloc_dev[dev];
    if (!d.scratch) {
        void* p = nullptr;
        TC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        int sm = 0, optin = 0;
        TC_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
        TC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        d.sm_count = sm;
        d.smem_optin = (size_t)optin;
        d.scratch = static_cast<float2*>(p);
    }
    return d;
}

template <int N>
static void noalloc_n(const NoallocDevice& d, const float* x, const float* C, int64_t n, int m, int k, int F,
                      int clamp2, int32_t* labels, float* dist, cudaStream_t s) {
    float2* twN = d.scratch;
    float2* twF = twN + N;
    float2* spec = twF + N;
    k_twiddles<<<ceil_div(N, 256), 256, 0, s>>>(twN, twF, N);
    TC_CHECK_LAUNCH();
    const size_t ssm = Cfg<N>::BUF_BYTES + sizeof(TeamScratch);
    allow_max_dynamic_smem(k_centroid_spectra<N>);
    k_centroid_spectra<N><<<k, Plan<N>::T, ssm, s>>>(C, m, twN, twF, spec);
    TC_CHECK_LAUNCH();
    AssignParams p{};
    p.x = x;
    p.spec = spec;
    p.twN = twN;
    p.twF = twF;
    p.n = n;
    p.m = m;
    p.k = k;
    p.F = F;
    p.clamp2 = clamp2;
    p.labels = labels;
    p.dist = dist;
    const bool csmem = Cfg<N>::smem(k, true) <= d.smem_optin;
    const size_t sm = Cfg<N>::smem(k, csmem);
    auto fn = csmem ? k_assign_fft<N, true, false> : k_assign_fft<N, false, false>;
    allow_max_dynamic_smem(fn);
    int per_sm = 0;
    TC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, Cfg<N>::BLOCK, sm));
    const int64_t teams = (n + Cfg<N>::TEAMS - 1) / Cfg<N>::TEAMS;
    const int grid = (int)std::min<int64_t>(teams, (int64_t)d.sm_count * std::max(per_sm, 1));
    fn<<<grid, Cfg<N>::BLOCK, sm, s>>>(p);
    TC_CHECK_LAUNCH();
}

}  // namespace tc

extern "C" int tc_sbd_assign_noalloc(const float* d_x, const float* d_centroids, int64_t n, int m, int k, int mode,
                                     int32_t* d_labels, float* d_dist, tc_stream stream, char* err, int err_len) {
    using namespace tc;
    auto fail = [&](int code, const std::string& msg) {
        if (err && err_len > 0) std::snprintf(err, (size_t)err_len, "%s", msg.c_str());
        return code;
    };
    try {
        TC_REQUIRE(mode == TC_MODE_COMPAT || mode == TC_MODE_CANONICAL, TC_ERR_ARG, "unknown mode");
        TC_REQUIRE(n >= 0 && n <= (int64_t)INT32_MAX, TC_ERR_ARG, "n must be in [0, 2^31)");
        TC_REQUIRE(m >= 2 && m <= 8192, TC_ERR_UNSUPPORTED, "series length m must be in [2, 8192]");
        TC_REQUIRE(k >= 1 && k <= 1024, TC_ERR_UNSUPPORTED, "k must be in [1, 1024]");
        TC_REQUIRE((d_x && d_centroids && d_labels) || n == 0, TC_ERR_ARG, "null pointer");
        const int F = fft_size(m, mode), N = F / 2;
        TC_REQUIRE(F >= 8 && F <= 16384, TC_ERR_UNSUPPORTED, "FFT length outside [8, 16384]");
        const size_t need = ((size_t)2 * N + (size_t)k * (N + 1)) * sizeof(float2);
        TC_REQUIRE(need <= NOALLOC_SCRATCH_BYTES, TC_ERR_UNSUPPORTED,
                   "scratch of " + std::to_string(need) + " bytes needed (2*(F/2) + k*(F/2+1) complex values), the "
                   "static array holds " + std::to_string(NOALLOC_SCRATCH_BYTES));
        int dev = 0;
        TC_CUDA(cudaGetDevice(&dev));
        const NoallocDevice d = noalloc_setup(dev);
        if (n == 0) return TC_OK;
        const int clamp2 = (mode == TC_MODE_COMPAT && 2 * m - 1 < 512) ? 1 : 0;
        cudaStream_t s = (cudaStream_t)stream;
        switch (N) {
#define X(nn) \
    case nn: noalloc_n<nn>(d, d_x, d_centroids, n, m, k, F, clamp2, d_labels, d_dist, s); break;
            TC_FOR_EACH_N(X)
#undef X
            default:
                return fail(TC_ERR_UNSUPPORTED, "FFT length not supported");
        }
        return TC_OK;
    } catch (const TcError& e) {
        return fail(e.code, e.msg);
    }
}
