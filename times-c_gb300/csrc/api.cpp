// C ABI entry points and the host side of the k-Shape loop.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>

#include "loop_graph.h"
#include "tc_internal.h"

std::recursive_mutex& capture_mutex() {
    static std::recursive_mutex mu;
    return mu;
}

size_t guard_bytes(size_t need) {
    static const bool on = std::getenv("TIMESC_GUARD") != nullptr;
    // a multiple of 4 KB: the buffer after the front zone keeps cudaMalloc's alignment
    return on ? (((size_t)1 << 20) + need / 4 + 4095) / 4096 * 4096 : 0;
}

namespace tc {

std::atomic<uint64_t> g_launches{0};

// ncc.cuh:12-16 and :473: 1 << (int)ceil(my_log2(2m-1)) with my_log2 returning a
// truncated int, i.e. the largest power of two <= 2m-1.  Canonical k-Shape pads to
// 1 << bit_length(2m-1) (test_timesC.py:88), a power of two >= 2m-1.
int fft_size(int m, int mode) {
    int x = 2 * m - 1;
    if (mode == TC_MODE_COMPAT) {
        int lg = (int)(std::log((double)x) / std::log(2.0));
        return 1 << lg;
    }
    int bl = 0;
    while ((1 << bl) <= x) ++bl;
    return 1 << bl;
}

void launch_gather_norm(const float*, const int32_t*, const int32_t*, const int32_t*, const uint8_t*, int64_t,
                        int, float*, int, cudaStream_t);

static void check_shape(int64_t n, int m, int k, int mode) {
    TC_REQUIRE(n >= 0, TC_ERR_ARG, "n must be >= 0");
    TC_REQUIRE(n <= (int64_t)INT32_MAX, TC_ERR_UNSUPPORTED, "n must fit in int32");
    TC_REQUIRE(m >= 2 && m <= 8192, TC_ERR_UNSUPPORTED, "series length m must be in [2, 8192]");
    TC_REQUIRE(k >= 1 && k <= 1024, TC_ERR_UNSUPPORTED, "k must be in [1, 1024]");
    TC_REQUIRE(mode == TC_MODE_COMPAT || mode == TC_MODE_CANONICAL, TC_ERR_ARG, "unknown mode");
    int F = fft_size(m, mode);
    TC_REQUIRE(F >= 8 && F <= 16384, TC_ERR_UNSUPPORTED,
               "FFT length " + std::to_string(F) + " outside [8, 16384] (series too short or too long for this mode)");
}

// The bounded assignment across iterations (both forms, at the lengths the tensor-core
// correlation takes): lower bounds on every (series, centroid) distance, carried from
// one assignment to the next with each centroid's movement, let the tensor-core pass
// skip, per 128-series tile, the centroids that cannot be any of the tile's series'
// first minimum.  Bounds are kept only for series that stay fixed across calls - those
// prepared by tc_prepare_series (or the whole loop's own normalised copy).
//   * A full pass (BOUNDS_REFRESH) evaluates every pair, writes fresh bounds and
//     groups the series by best and second-best centroid.
//   * A bounded pass (BOUNDS_USE) evaluates the tiles' masks; BOUNDS_USE_REGROUP first
//     groups the series anew by the keys the previous pass left, which the next pass
//     does once more than 1/20 of the series changed their best centroid since the
//     last grouping (a moved series widens its old tile's mask).
//   * Every evaluated pair gets a fresh bound, so only the skipped ones loosen; a full
//     pass is run again once the bounded passes since the last one have cost, beyond
//     the cheapest of them, about one full pass (in units of a full tensor-core pass:
//     sum of evaluated fractions - passes x their minimum >= BOUNDS_REFRESH_COST).
// (BOUNDS_* modes and the two constants: loop_graph.h, whose control kernels restate
// the same rule on the device.)

static bool bounded_mode(int use) { return use == BOUNDS_USE || use == BOUNDS_USE_REGROUP; }

// The regroup threshold's denominator (BOUNDS_REGROUP_SHARE, or TIMESC_REGROUP_SHARE).
static int64_t regroup_share() {
    const char* e = std::getenv("TIMESC_REGROUP_SHARE");
    const long long v = e ? std::atoll(e) : 0;
    return v > 0 ? (int64_t)v : BOUNDS_REGROUP_SHARE;
}

// Bounds are kept for the FP32 form where the screened pass runs, and for the BF16
// form where the tensor-core correlation runs with k <= 64 (one mask word per tile).
static bool bounds_usable(const tc_ctx* ctx, const float* x, int64_t n, int m, int k, int mode, int precision) {
    const int F = fft_size(m, mode);
    // both forms bound through the tensor-core pass's 64-bit tile masks
    const bool form = (precision == TC_PREC_FP32 ? screen_supported(m, F, k)
                                                 : tc_assign_supported(m, F, k, precision)) &&
                      k >= 2 && k <= 64;
    return form && !std::getenv("TIMESC_NO_BOUNDS") && ctx->prep_x == x && ctx->prep_n == n && ctx->prep_m == m;
}

// The bounds state for these series and shape (reset when any of them changes).
static BoundsState& bounds_for(tc_ctx* ctx, const float* x, int64_t n, int m, int k, int mode, int precision) {
    BoundsState& b = ctx->bounds;
    if (!(b.x == x && b.n == n && b.m == m && b.k == k && b.mode == mode && b.precision == precision)) {
        const uint64_t sc = b.screened, bd = b.bounded, bp = b.bounded_pairs;
        b = BoundsState{};
        b.x = x;
        b.n = n;
        b.m = m;
        b.k = k;
        b.mode = mode;
        b.precision = precision;
        b.screened = sc;
        b.bounded = bd;
        b.bounded_pairs = bp;
    }
    return b;
}

// The mode an assignment with bounds runs in (bmode AUTO: from the state).
static int bounds_mode(const BoundsState& b, int bmode) {
    int use = bmode;
    if (bmode == BOUNDS_AUTO) use = b.refresh ? BOUNDS_REFRESH : (b.regroup ? BOUNDS_USE_REGROUP : BOUNDS_USE);
    if (bounded_mode(use) && !b.valid) use = BOUNDS_REFRESH;
    return use;
}

// The bound fields of one tensor-core pass and what runs before it: centroid
// movements, counters, and for a bounded pass the (new) grouping and the tile masks.
static void bounds_setup(tc_ctx* ctx, AssignArgs& a, int use, const float* C, cudaStream_t s, bool fp32) {
    Workspace& ws = ctx->ws;
    const int64_t n = a.n;
    const int m = a.m, k = a.k;
    float* cprev = ws.cprev.as<float>((size_t)k * m + k);
    float* delta = cprev + (size_t)k * m;
    float* craw = nullptr;
    uint8_t* same = nullptr;
    if (fp32) {  // the FFT pass's labels and distances, and the raw centroids they belong to
        char* f = static_cast<char*>(ws.fprev.get((size_t)n * 8 + (size_t)k * m * 4 + k));
        a.prev_dist = reinterpret_cast<float*>(f);
        a.prev_label = reinterpret_cast<int32_t*>(f + (size_t)n * 4);
        craw = reinterpret_cast<float*>(f + (size_t)n * 8);
        same = reinterpret_cast<uint8_t*>(f + (size_t)n * 8 + (size_t)k * m * 4);
        a.same = same;
        a.reuse = bounded_mode(use);  // after a full pass every series has its label and distance
    }
    launch_centroid_delta(C, k, m, cprev, delta, s, craw, same);  // cprev (and craw) <- these centroids
    char* st = static_cast<char*>(ws.bstate.get((size_t)n * 12));
    a.ubd = reinterpret_cast<float*>(st);
    a.jb = reinterpret_cast<int32_t*>(st + (size_t)n * 4);
    a.gkey = reinterpret_cast<int32_t*>(st + (size_t)n * 8);
    a.lb_out = ws.bounds.as<float>((size_t)k * n);  // the BF16 pass d16 - D, an FP32 pass d32 - eps
    a.lb_d16 = (float)bf16_error(m, a.F);
    a.lb_eps = (float)(fft_error(m, a.F) + 1e-6);
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(ws.aux.as<char>(64) + 24);
    TC_CUDA(cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned long long), s));  // evaluated tiles, moved series, series pairs
    a.moved = cnt + 1;
    if (bounded_mode(use)) {
        if (use == BOUNDS_USE_REGROUP) launch_tile_group(ctx, n, m, k, a.gkey, s);
        TileBounds tb;
        launch_tile_masks(ctx, n, m, k, a.lb_out, a.ubd, a.jb, delta, a.lb_d16, tb, s, cnt + 2);
        a.perm = tb.perm;
        a.xbf = tb.xbf;
        a.xbf_norm = tb.xbf_norm;
        a.tmask = tb.tmask;
        a.delta = delta;
        a.evals = cnt;
    }
}

// One assignment against the current centroids.  Returns the bounds mode it ran.
static int assign(tc_ctx* ctx, const float* x, const float* C, int64_t n, int m, int k, int mode, int precision,
                  int32_t* labels, float* dist, int32_t* shift, const int32_t* old, int32_t* changed,
                  double* dsum, cudaStream_t s, int bmode = BOUNDS_AUTO) {
    const int F = fft_size(m, mode);
    AssignArgs a{};
    a.x = x;
    a.n = n;
    a.m = m;
    a.k = k;
    a.F = F;
    a.clamp2 = (mode == TC_MODE_COMPAT && 2 * m - 1 < 512) ? 1 : 0;  // get_pos_idx pads with 2
    a.labels = labels;
    a.dist = dist;
    a.shift = shift;
    a.old_labels = old;
    a.changed = changed;
    a.dist_sum = dsum;
    if (precision == TC_PREC_FP32 && !shift && screen_supported(m, F, k)) {
        // exact screening: the BF16 pass keeps every centroid whose FP32 distance can be
        // the minimum, the FP32 pass evaluates those (same labels and distances as the
        // unscreened FP32 kernel).  With bounds, the BF16 pass is the tile-bounded one
        // (as in the BF16 form): a centroid its tile leaves out has an exact distance
        // above the series' best by more than 2D >= 2 eps, so it is not the FP32 first
        // minimum either, and among the centroids it evaluates the screen keeps that
        // minimum as before.
        Workspace& ws = ctx->ws;
        const bool usable = bmode != BOUNDS_OFF && bounds_usable(ctx, x, n, m, k, mode, precision);
        BoundsState& b = usable ? bounds_for(ctx, x, n, m, k, mode, precision) : ctx->bounds;
        const int use = usable ? bounds_mode(b, bmode) : BOUNDS_OFF;
        a.centroids = C;
        a.cand = ws.screen.as<int32_t>((size_t)n * (SCREEN_CAP + 1));
        a.ncand = a.cand + (size_t)n * SCREEN_CAP;
        if (use != BOUNDS_OFF) bounds_setup(ctx, a, use, C, s, true);
        // -1 (all centroids) for every series the tensor-core pass does not reach,
        // e.g. after one of its bounded waits ran out
        TC_CUDA(cudaMemsetAsync(a.ncand, 0xFF, (size_t)n * sizeof(int32_t), s));
        launch_assign_tc(ctx, a, TC_PREC_BF16, s);
        if (use == BOUNDS_REFRESH) launch_tile_group(ctx, n, m, k, a.gkey, s);
        float2* spec = ws.spectra.as<float2>((size_t)k * (F / 2 + 1));
        launch_centroid_spectra(ctx, C, k, m, F, spec, s);
        a.spec = spec;
        launch_assign_fft(ctx, a, s);
        if (use == BOUNDS_REFRESH) {
            b.valid = true;
            b.refresh = false;
        }
        return use;
    }
    if (precision == TC_PREC_FP32 || shift || !tc_assign_supported(m, F, k, precision)) {
        float2* spec = ctx->ws.spectra.as<float2>((size_t)k * (F / 2 + 1));
        launch_centroid_spectra(ctx, C, k, m, F, spec, s);
        a.spec = spec;
        launch_assign_fft(ctx, a, s);
        return BOUNDS_OFF;
    }
    a.centroids = C;
    const bool usable = bmode != BOUNDS_OFF && bounds_usable(ctx, x, n, m, k, mode, precision);
    if (!usable) {
        launch_assign_tc(ctx, a, precision, s);
        return BOUNDS_OFF;
    }
    // BF16 form with bounds: a full pass leaves a lower bound d16 - D on every pair and
    // per series an upper bound on its best, and groups the series by that best; the
    // tile-bounded passes then evaluate, per 128-row tile of that grouping, only the
    // centroids whose bounds do not rule them out for every series of the tile
    BoundsState& b = bounds_for(ctx, x, n, m, k, mode, precision);
    const int use = bounds_mode(b, bmode);
    bounds_setup(ctx, a, use, C, s, false);
    launch_assign_tc(ctx, a, precision, s);
    if (use == BOUNDS_REFRESH) {
        launch_tile_group(ctx, n, m, k, a.gkey, s);  // by best and second best: similar masks
        b.valid = true;
        b.refresh = false;
    }
    return use;
}

// After an assignment that kept bounds: count it, and decide whether the next one
// regroups the series or runs a full pass (see BOUNDS_REFRESH_COST).
static void bounds_feedback(tc_ctx* ctx, int used, unsigned long long evals, unsigned long long moved,
                            unsigned long long spairs, int64_t n, int k) {
    BoundsState& b = ctx->bounds;
    if (used == BOUNDS_REFRESH) {
        ++b.screened;
        b.moved = 0;  // grouped by this pass's keys
        b.regroup = false;
        b.sum_f = 0;
        b.min_f = 2;
        b.passes = 0;
    } else if (bounded_mode(used)) {
        // the tensor-core pass counts (tile, centroid) pairs of its 128-row tiles
        evals *= 128;
        ++b.bounded;
        b.bounded_pairs += evals;
        b.series_pairs += spairs;
        if (std::getenv("TIMESC_TRACE"))
            std::fprintf(stderr, "timesc: bounded pass%s: tiles evaluate %.3f of the pairs, the series need %.3f\n",
                         used == BOUNDS_USE_REGROUP ? " (regrouped)" : "", (double)evals / ((double)n * k),
                         (double)spairs / ((double)n * k));
        b.moved = (used == BOUNDS_USE_REGROUP ? 0 : b.moved) + moved;
        b.regroup = (int64_t)b.moved * regroup_share() > n;
        const double f = (double)evals / ((double)n * k);
        b.sum_f += f;
        b.min_f = std::min(b.min_f, f);
        ++b.passes;
        b.refresh = b.sum_f - b.passes * b.min_f >= BOUNDS_REFRESH_COST;
    }
}

// Error words the asynchronous stages leave in aux: Gram at +48, tensor-core
// correlation at +52.
static void check_async_errors(const int* words) {
    TC_REQUIRE(words[0] == 0, TC_ERR_TIMEOUT, "tensor-core Gram: a pipeline wait ran out");
    TC_REQUIRE(words[1] == 0, TC_ERR_TIMEOUT, "tensor-core correlation: a pipeline wait ran out");
}

// One stage of an iteration (extraction, or assignment) as a CUDA graph: the
// first run issues the launches directly (workspace buffers, FFT tables and
// kernel attributes get set up), the second captures them and later runs replay
// the graph.  The stages hold no host synchronisation, and their buffers and
// arguments are the same every iteration.  If capture or instantiation fails
// the stage keeps issuing its launches directly.
struct StageGraph {
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;  // kept for the loop graph, which embeds it
    bool warm = false, failed = false;
    uint64_t kernels = 0;  // kernel launches recorded in the graph
    StageGraph() = default;
    StageGraph(const StageGraph&) = delete;
    StageGraph& operator=(const StageGraph&) = delete;
    ~StageGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
    template <class F>
    void run(bool enabled, cudaStream_t s, F&& issue) {
        if (!enabled || failed || !warm) {
            issue();
            warm = true;
            return;
        }
        if (!exec) capture(s, issue);
        if (exec) {
            TC_CUDA(cudaGraphLaunch(exec, s));
            g_launches.fetch_add(kernels, std::memory_order_relaxed);  // the kernels the replay runs
        } else {
            issue();
        }
    }
    template <class F>
    void capture(cudaStream_t s, F&& issue) {
        std::lock_guard<std::recursive_mutex> lk(capture_mutex());
        cudaGraph_t gr = nullptr;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            cudaGetLastError();
            failed = true;
            return;
        }
        bool ok = true;
        const uint64_t before = g_launches.load();
        try {
            issue();
        } catch (const TcError&) {
            ok = false;
        }
        kernels = g_launches.load() - before;
        g_launches.fetch_sub(kernels);  // captured, not launched
        const cudaError_t e = cudaStreamEndCapture(s, &gr);
        if (!ok || e != cudaSuccess || !gr || cudaGraphInstantiate(&exec, gr, 0) != cudaSuccess) {
            exec = nullptr;
            failed = true;
        }
        if (exec) graph = gr;
        else if (gr) cudaGraphDestroy(gr);
        cudaGetLastError();
    }
};

struct LoopState {
    int iterations = 0;
    int sum_class = 0;
    double inertia = 0;
};

// kshape.cuh:197-324 (k_shape) and :332-474 (k_shape_tsl) on device-resident state.
static LoopState run_loop(tc_ctx* ctx, const tc_job* job, const float* x, int k, int order_tsl, int cal_select,
                          int cap, cudaStream_t s) {
    Workspace& ws = ctx->ws;
    const int64_t n = job->n;
    const int m = job->m;
    int32_t* labels = ws.labels.as<int32_t>(n);
    int32_t* old = ws.old_labels.as<int32_t>(n);
    float* dist = ws.dist.as<float>(n);
    float* C = ws.centroids.as<float>((size_t)k * m);
    char* aux = ws.aux.as<char>(64);
    int32_t* changed = reinterpret_cast<int32_t*>(aux);
    double* dsum = reinterpret_cast<double*>(aux + 8);

    // initial labels: idx_init (curand) or the caller's
    if (job->h_init_labels)
        TC_CUDA(cudaMemcpyAsync(labels, job->h_init_labels, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    else
        launch_init_labels(labels, n, k, s);
    TC_CUDA(cudaMemcpyAsync(old, labels, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
    TC_CUDA(cudaMemsetAsync(C, 0, sizeof(float) * k * m, s));
    if (order_tsl) {
        // k distinct raw rows (kshape.cuh:159-191, :345-352), before normalisation
        std::vector<int32_t> pick(k);
        TC_REQUIRE(tc_random_select(n, k, job->seed, pick.data()) == TC_OK, TC_ERR_ARG, "k > n");
        for (int j = 0; j < k; ++j) {
            if (job->h_data)
                TC_CUDA(cudaMemcpyAsync(C + (size_t)j * m, job->h_data + (size_t)pick[j] * m, sizeof(float) * m,
                                        cudaMemcpyHostToDevice, s));
            else
                TC_CUDA(cudaMemcpyAsync(C + (size_t)j * m, job->d_data + (size_t)pick[j] * m, sizeof(float) * m,
                                        cudaMemcpyDeviceToDevice, s));
        }
    }
    LoopState st;
    st.sum_class = k;
    st.iterations = cap;
    double old_inertia = 1e10;
    int countIter = 0;
    // what the stages leave in aux: changed (+0), dist sum (+8), sum_class and the
    // bad-label flag (+16), the bounded pass's counters (+24, +32), error words of the
    // Gram and the correlation (+48)
    struct {
        int32_t changed;
        int32_t pad;
        double dsum;
        int32_t sum_class, bad_label;
        unsigned long long evals;   // (tile, centroid) pairs the bounded pass evaluated (+24)
        unsigned long long moved;   // series whose best centroid changed (+32)
        unsigned long long spairs;  // pairs the series' own masks hold (+40)
        int32_t err[2];
    } h;
    static_assert(sizeof(h) == 56, "aux layout");
    StageGraph g_extract, g_assign, g_assign_bounded, g_assign_regroup;
    const bool bnd = bounds_usable(ctx, x, n, m, k, job->mode, job->precision);
    const bool graphs = ctx->graphs && !std::getenv("TIMESC_NO_GRAPHS");
    auto readback = [&]() {
        TC_CUDA(cudaMemcpyAsync(&h, aux, sizeof(h), cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaStreamSynchronize(s));
        if (h.err[0] || h.err[1]) {  // a pass that stopped early left no bounds, no complete extraction
            ctx->bounds.valid = false;
            memo_invalidate(ctx);
        }
        check_async_errors(h.err);
    };
    TC_CUDA(cudaMemsetAsync(aux, 0, 64, s));
    auto issue_assign = [&](int bmode) {
        TC_CUDA(cudaMemsetAsync(aux, 0, 16, s));
        // no shifts here: the extraction computes its own where the gate is open
        assign(ctx, x, C, n, m, k, job->mode, job->precision, labels, dist, nullptr, old, changed, dsum, s, bmode);
    };
    ExtractArgs e{};
    e.x = x;
    e.labels = labels;
    e.shift = nullptr;
    e.C = C;
    e.n = n;
    e.m = m;
    e.k = k;
    e.mode = job->mode;
    e.cal_select = cal_select;
    e.precision = job->precision;
    e.counts = nullptr;
    e.memo = 1;  // the run's own copy of the series, fixed for the run
    memo_invalidate(ctx);  // the copy was rewritten for this run
    memo_prepare(ctx, e, s);  // before the extraction graph is captured
    auto issue_extract = [&]() {
        extract_async(ctx, e, s);
        TC_CUDA(cudaMemcpyAsync(aux + 16, ws.scal.p, 2 * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    };
    auto do_assign = [&]() -> bool {
        // a full pass (or no bounds), a bounded pass, or a bounded pass on a new
        // grouping, as the bounds state asks - one graph for each
        const int use = bnd ? bounds_mode(ctx->bounds, BOUNDS_AUTO) : BOUNDS_OFF;
        if (use == BOUNDS_USE) g_assign_bounded.run(graphs, s, [&]() { issue_assign(BOUNDS_USE); });
        else if (use == BOUNDS_USE_REGROUP) g_assign_regroup.run(graphs, s, [&]() { issue_assign(BOUNDS_USE_REGROUP); });
        else g_assign.run(graphs, s, [&]() { issue_assign(BOUNDS_REFRESH); });
        readback();
        if (bnd) {
            if (use == BOUNDS_REFRESH) {
                ctx->bounds.valid = true;
                ctx->bounds.refresh = false;
            }
            bounds_feedback(ctx, use, h.evals, h.moved, h.spairs, n, k);
        }
        check_guards(ctx, "assignment");
        st.inertia = h.dsum / (double)n;
        return h.changed == 0;
    };
    auto converge = [&](int i, bool flag) -> bool {
        if (flag || countIter > 20) {
            st.iterations = i + 1;
            return true;
        }
        if (st.inertia < old_inertia || std::fabs(old_inertia - st.inertia) < 1e-6) {
            TC_CUDA(cudaMemcpyAsync(old, labels, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
            old_inertia = st.inertia;
            countIter = 0;
        } else {
            ++countIter;
        }
        return false;
    };
    auto extract = [&]() {
        g_extract.run(graphs, s, issue_extract);
        readback();
        check_guards(ctx, "extraction");
        if (h.bad_label) memo_invalidate(ctx);
        TC_REQUIRE(h.bad_label == 0, TC_ERR_ARG, "a label is outside [0, k)");
        if (!cal_select) st.sum_class = h.sum_class;  // get_class_centers_a leaves sum_class alone
    };
    // With TIMESC_DEVICE_LOOP=1: the whole loop as one graph (loop_graph.h) once the
    // extraction and the assignment variant an iteration needs are captured; until then,
    // and whenever the graph returns for a variant it does not hold yet, the host runs
    // the iteration.  Off by default: on a GB300 host the two read-backs an iteration
    // takes cost a few microseconds, about what the graph's conditional nodes and
    // control kernels cost, and building the graph (twice per run) cost more than that.
    const char* dl_env = std::getenv("TIMESC_DEVICE_LOOP");
    const bool dev_loop = graphs && dl_env && std::strcmp(dl_env, "0") != 0 && !ctx->loop_graph_failed &&
                          !guard_bytes(1) && !std::getenv("TIMESC_TRACE");
    StageGraph* variants[3] = {&g_assign, &g_assign_bounded, &g_assign_regroup};
    struct LoopExec {
        cudaGraphExec_t exec = nullptr;
        int avail = -1;  // the variants it holds
        ~LoopExec() {
            if (exec) cudaGraphExecDestroy(exec);
        }
    } lx;
    LoopCtl* dctl = dev_loop ? ws.loopctl.as<LoopCtl>(1) : nullptr;
    // true once the loop has ended on the device; otherwise i is the iteration the host runs
    auto device_loop = [&](int& i) -> bool {
        if (!dev_loop || !g_extract.graph) return false;
        const int mode = bnd ? bounds_mode(ctx->bounds, BOUNDS_AUTO) : BOUNDS_OFF;
        int avail = 0;
        for (int v = 0; v < 3; ++v)
            if (variants[v]->graph) avail |= 1 << v;
        if (!((avail >> assign_variant(mode)) & 1)) return false;
        if (lx.avail != avail) {
            if (lx.exec) cudaGraphExecDestroy(lx.exec);
            LoopGraphSpec sp;
            sp.extract = g_extract.graph;
            for (int v = 0; v < 3; ++v) sp.assign[v] = variants[v]->graph;
            sp.order_tsl = order_tsl;
            sp.ctl = dctl;
            sp.aux = aux;
            sp.labels = labels;
            sp.old_labels = old;
            sp.n = n;
            lx.exec = build_loop_graph(sp);
            lx.avail = avail;
            ++ctx->loop.builds;
            if (!lx.exec) {
                ctx->loop_graph_failed = true;  // the runtime refused it: iterations stay on the host
                return false;
            }
        }
        const BoundsState& b = ctx->bounds;
        LoopCtl c{};
        c.n = n;
        c.regroup_share = regroup_share();
        c.k = k;
        c.cap = cap;
        c.cal_select = cal_select;
        c.bnd = bnd;
        c.avail = avail;
        c.kern_extract = (int)g_extract.kernels;
        for (int v = 0; v < 3; ++v) c.kern_assign[v] = (int)variants[v]->kernels;
        c.i = i;
        c.count_iter = countIter;
        c.sum_class = st.sum_class;
        c.iterations = cap;
        c.stop = LOOP_RUN;
        c.mode = mode;
        c.old_inertia = old_inertia;
        c.inertia = st.inertia;
        c.valid = b.valid;
        c.refresh = b.refresh;
        c.regroup = b.regroup;
        c.passes = b.passes;
        c.moved = b.moved;
        c.sum_f = b.sum_f;
        c.min_f = b.min_f;
        c.screened = b.screened;
        c.bounded = b.bounded;
        c.bounded_pairs = b.bounded_pairs;
        c.series_pairs = b.series_pairs;
        TC_CUDA(cudaMemcpyAsync(dctl, &c, sizeof(c), cudaMemcpyHostToDevice, s));
        TC_CUDA(cudaGraphLaunch(lx.exec, s));
        TC_CUDA(cudaMemcpyAsync(&c, dctl, sizeof(c), cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaMemcpyAsync(&h, aux, sizeof(h), cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaStreamSynchronize(s));
        g_launches.fetch_add(c.launched, std::memory_order_relaxed);
        ctx->loop.device_iterations += (uint64_t)((c.stop == LOOP_DONE ? c.iterations : c.i) - i);
        BoundsState& bw = ctx->bounds;
        bw.valid = c.valid != 0;
        bw.refresh = c.refresh != 0;
        bw.regroup = c.regroup != 0;
        bw.passes = c.passes;
        bw.moved = c.moved;
        bw.sum_f = c.sum_f;
        bw.min_f = c.min_f;
        bw.screened = c.screened;
        bw.bounded = c.bounded;
        bw.bounded_pairs = c.bounded_pairs;
        bw.series_pairs = c.series_pairs;
        countIter = c.count_iter;
        old_inertia = c.old_inertia;
        st.inertia = c.inertia;
        st.sum_class = c.sum_class;
        if (c.stop == LOOP_ERROR) {  // the host's checks, in its order
            if (h.err[0] || h.err[1]) {
                ctx->bounds.valid = false;
                memo_invalidate(ctx);
            }
            check_async_errors(h.err);
            if (h.bad_label) memo_invalidate(ctx);
            TC_REQUIRE(h.bad_label == 0, TC_ERR_ARG, "a label is outside [0, k)");
            throw TcError{TC_ERR_CUDA, "the loop graph stopped without a reason"};
        }
        if (c.stop == LOOP_DONE) {
            st.iterations = c.iterations;
            return true;
        }
        i = c.i;
        return false;
    };
    for (int i = 0; i < cap; ++i) {
        if (device_loop(i)) break;
        ++ctx->loop.host_iterations;
        if (!order_tsl) {
            extract();
            if (st.sum_class == 1 || st.sum_class <= k / 2) {
                st.iterations = i + 1;
                break;
            }
            if (converge(i, do_assign())) break;
        } else {
            if (converge(i, do_assign())) break;
            extract();
            if (st.sum_class == 1 || st.sum_class <= k / 2) {
                st.iterations = i + 1;
                break;
            }
        }
    }
    return st;
}

static const char* const WS_NAMES[] = {"x", "labels", "old_labels", "shift", "dist", "centroids", "spectra",
                                       "seg", "perm", "chunk_counts", "counts", "offsets", "gate", "scal",
                                       "gram", "rowsum", "gram_yt", "gram_poff", "piter", "pstats", "aux",
                                       "toeplitz", "toeplitz_norm", "xbf", "xbf_norm", "first", "gram_sq", "sq_meta", "screen", "gram_part",
                                       "bounds", "cprev", "bstate", "bperm", "xbfp", "tmask", "memo_labels", "memo_c",
                                       "memo_flags", "memo_count", "fprev", "loopctl"};

static std::vector<DevBuf*> workspace_buffers(tc_ctx* ctx);

void check_guards(tc_ctx* ctx, const char* where) {
    if (!guard_bytes(1)) return;
    TC_CUDA(cudaStreamSynchronize(ctx->own_stream));
    auto check = [&](const DevBuf* b, const std::string& name) {
        if (!b->p) return;
        const size_t g = guard_bytes(b->bytes);
        std::vector<unsigned char> h(g);
        for (int side = 0; side < 2; ++side) {
            const char* z = side ? static_cast<const char*>(b->p) + b->bytes : static_cast<const char*>(b->base());
            TC_CUDA(cudaMemcpy(h.data(), z, g, cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < g; ++i)
                if (h[i] != GUARD_BYTE) {
                    std::fprintf(stderr, "timesc guard: buffer %s (%zu bytes) overwritten %s at %zu after %s\n",
                                 name.c_str(), b->bytes, side ? "after its end" : "before its start",
                                 side ? i : g - i, where);
                    throw TcError{TC_ERR_CUDA, "guard of buffer " + name + " overwritten after " + where};
                }
        }
    };
    const auto bufs = workspace_buffers(ctx);
    for (size_t i = 0; i < bufs.size(); ++i) check(bufs[i], WS_NAMES[i]);
    for (const FftTables* t : ctx->fft) {
        check(&t->twN, "twN" + std::to_string(t->F));
        check(&t->twF, "twF" + std::to_string(t->F));
    }
}

static std::vector<DevBuf*> workspace_buffers(tc_ctx* ctx) {
    Workspace& w = ctx->ws;
    return {&w.x,    &w.labels,  &w.old_labels, &w.shift,   &w.dist,      &w.centroids, &w.spectra,
            &w.seg,  &w.perm,    &w.chunk_counts, &w.counts, &w.offsets,  &w.gate,      &w.scal,
            &w.gram, &w.rowsum,  &w.gram_yt,    &w.gram_poff, &w.piter,   &w.pstats,    &w.aux,
            &w.toeplitz, &w.toeplitz_norm, &w.xbf, &w.xbf_norm, &w.first, &w.gram_sq, &w.sq_meta, &w.screen, &w.gram_part,
            &w.bounds, &w.cprev, &w.bstate, &w.bperm, &w.xbfp, &w.tmask, &w.memo_labels, &w.memo_c,
            &w.memo_flags, &w.memo_count, &w.fprev, &w.loopctl};
}

void release_workspace(tc_ctx* ctx) {
    for (DevBuf* b : workspace_buffers(ctx)) b->release();
    ctx->prep_x = nullptr;
    ctx->bounds.valid = false;
    ctx->memo.keyed = false;
    ctx->memo.counters = false;
}

size_t workspace_bytes(tc_ctx* ctx) {
    size_t t = 0;
    for (DevBuf* b : workspace_buffers(ctx)) t += b->bytes;
    return t;
}

}  // namespace tc

using namespace tc;

#define TC_API_BEGIN try {
#define TC_API_END(ctx)                                           \
    }                                                             \
    catch (const TcError& e) {                                    \
        if (ctx) (ctx)->last_error = e.msg;                       \
        return e.code;                                            \
    }                                                             \
    catch (const std::bad_alloc&) {                               \
        if (ctx) (ctx)->last_error = "host allocation failed";    \
        return TC_ERR_NOMEM;                                      \
    }                                                             \
    catch (const std::exception& e) {                             \
        if (ctx) (ctx)->last_error = e.what();                    \
        return TC_ERR_ARG;                                        \
    }                                                             \
    return TC_OK;

extern "C" {

int tc_version(void) { return TC_ABI_VERSION; }

int tc_create(int device, tc_ctx** out) {
    if (!out) return TC_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return TC_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return TC_ERR_CUDA;
    tc_ctx* c = new (std::nothrow) tc_ctx();
    if (!c) return TC_ERR_NOMEM;
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    c->smem_optin = (size_t)optin;
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return TC_ERR_CUDA;
    }
    if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(c->own_stream);
        delete c;
        return TC_ERR_CUDA;
    }
    *out = c;
    return TC_OK;
}

int tc_destroy(tc_ctx* ctx) {
    if (!ctx) return TC_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->own_stream);
    tc::release_workspace(ctx);
    for (auto* t : ctx->fft) {
        t->twN.release();
        t->twF.release();
        delete t;
    }
    cudaStreamDestroy(ctx->own_stream);
    cudaStreamDestroy(ctx->copy_stream);
    delete ctx;
    return TC_OK;
}

const char* tc_last_error(const tc_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

uint64_t tc_launch_count(void) { return g_launches.load(); }

int tc_fft_size(int m, int mode) {
    if (m < 1) return 0;
    return fft_size(m, mode);
}

int tc_znorm(tc_ctx* ctx, float* d_x, int64_t n, int m, int ddof, tc_stream stream) {
    if (!ctx) return TC_ERR_ARG;
    TC_API_BEGIN
    TC_REQUIRE(d_x || n == 0, TC_ERR_ARG, "null data");
    TC_REQUIRE(ddof >= 0 && ddof < m, TC_ERR_ARG, "ddof must be in [0, m)");
    TC_CUDA(cudaSetDevice(ctx->device));
    launch_znorm(d_x, n, m, ddof, ctx->sm_count, (cudaStream_t)stream);
    TC_API_END(ctx)
}

int tc_init_labels(tc_ctx* ctx, int32_t* d_labels, int64_t n, int k, tc_stream stream) {
    if (!ctx) return TC_ERR_ARG;
    TC_API_BEGIN
    TC_REQUIRE(d_labels || n == 0, TC_ERR_ARG, "null labels");
    TC_REQUIRE(k >= 1, TC_ERR_ARG, "k must be >= 1");
    TC_CUDA(cudaSetDevice(ctx->device));
    launch_init_labels(d_labels, n, k, (cudaStream_t)stream);
    TC_API_END(ctx)
}

int tc_sbd_assign(tc_ctx* ctx, const float* d_x, const float* d_centroids, int64_t n, int m, int k, int mode,
                  int precision, int32_t* d_labels, float* d_dist, int32_t* d_shift, const int32_t* d_old_labels,
                  int32_t* d_changed, double* d_dist_sum, tc_stream stream) {
    if (!ctx) return TC_ERR_ARG;
    TC_API_BEGIN
    check_shape(n, m, k, mode);
    TC_REQUIRE((d_x && d_centroids && d_labels) || n == 0, TC_ERR_ARG, "null pointer");
    TC_REQUIRE(precision >= TC_PREC_FP32 && precision <= TC_PREC_TF32, TC_ERR_ARG, "unknown precision");
    TC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    char* aux = ctx->ws.aux.as<char>(64);
    TC_CUDA(cudaMemsetAsync(aux + 48, 0, 2 * sizeof(int), s));
    const int used = assign(ctx, d_x, d_centroids, n, m, k, mode, precision, d_labels, d_dist, d_shift,
                            d_old_labels, d_changed, d_dist_sum, s);
    const bool tc_used = precision != TC_PREC_FP32 || (!d_shift && screen_supported(m, fft_size(m, mode), k));
    if (tc_used) {  // the tensor-core pass reports through an error word; the bounded pass counts its pairs
        struct {
            unsigned long long evals, moved, spairs;
            int32_t err[2];
        } h;
        static_assert(sizeof(h) == 32, "aux layout");
        TC_CUDA(cudaMemcpyAsync(&h, aux + 24, sizeof(h), cudaMemcpyDeviceToHost, s));
        TC_CUDA(cudaStreamSynchronize(s));
        if (h.err[0] || h.err[1]) ctx->bounds.valid = false;  // a pass that stopped early left no bounds
        check_async_errors(h.err);
        bounds_feedback(ctx, used, h.evals, h.moved, h.spairs, n, k);
    }
    TC_API_END(ctx)
}

int tc_assign_stats(const tc_ctx* ctx, uint64_t* screened, uint64_t* bounded, uint64_t* bounded_pairs) {
    if (!ctx) return TC_ERR_ARG;
    if (screened) *screened = ctx->bounds.screened;
    if (bounded) *bounded = ctx->bounds.bounded;
    if (bounded_pairs) *bounded_pairs = ctx->bounds.bounded_pairs;
    return TC_OK;
}

int tc_loop_stats(const tc_ctx* ctx, uint64_t* device_iterations, uint64_t* host_iterations,
                  uint64_t* graphs_built) {
    if (!ctx) return TC_ERR_ARG;
    if (device_iterations) *device_iterations = ctx->loop.device_iterations;
    if (host_iterations) *host_iterations = ctx->loop.host_iterations;
    if (graphs_built) *graphs_built = ctx->loop.builds;
    return TC_OK;
}

int tc_extract_stats(tc_ctx* ctx, uint64_t* extractions, uint64_t* clusters, uint64_t* reused) {
    if (!ctx) return TC_ERR_ARG;
    TC_API_BEGIN
    uint64_t h[3] = {0, 0, 0};
    if (ctx->memo.counters && ctx->ws.memo_count.p) {
        TC_CUDA(cudaSetDevice(ctx->device));
        TC_CUDA(cudaDeviceSynchronize());
        TC_CUDA(cudaMemcpy(h, ctx->ws.memo_count.p, sizeof(h), cudaMemcpyDeviceToHost));
    }
    if (extractions) *extractions = h[0];
    if (clusters) *clusters = h[1];
    if (reused) *reused = h[2];
    TC_API_END(ctx)
}

int tc_prepare_series(tc_ctx* ctx, const float* d_x, int64_t n, int m, tc_stream stream) {
    if (!ctx) return TC_ERR_ARG;
    TC_API_BEGIN
    TC_REQUIRE(n >= 0 && m >= 2 && m <= 512, TC_ERR_ARG, "tc_prepare_series: n >= 0 and 2 <= m <= 512");
    TC_REQUIRE(d_x || n == 0, TC_ERR_ARG, "null pointer");
    TC_CUDA(cudaSetDevice(ctx->device));
    prepare_series_bf16(ctx, d_x, n, m, (cudaStream_t)stream);
    TC_API_END(ctx)
}

int tc_extract_shapes(tc_ctx* ctx, const float* d_x, const int32_t* d_labels, const int32_t* d_shift,
                      float* d_centroids, int64_t n, int m, int k, int mode, int cal_select, int precision,
                      int32_t* d_counts, int* h_sum_class, tc_stream stream) {
    if (!ctx) return TC_ERR_ARG;
    TC_API_BEGIN
    check_shape(n, m, k, mode);
    TC_REQUIRE((d_x && d_labels) || n == 0, TC_ERR_ARG, "null pointer");
    TC_REQUIRE(d_centroids, TC_ERR_ARG, "null centroids");
    TC_CUDA(cudaSetDevice(ctx->device));
    ExtractArgs e{};
    e.x = d_x;
    e.labels = d_labels;
    e.shift = d_shift;
    e.C = d_centroids;
    e.n = n;
    e.m = m;
    e.k = k;
    e.mode = mode;
    e.cal_select = cal_select ? 1 : 0;
    e.precision = precision;
    e.counts = d_counts;
    // prepared series are fixed until prepared again: clusters that kept their members
    // and centroid reuse the previous extraction's output
    e.memo = ctx->prep_x == d_x && ctx->prep_n == n && ctx->prep_m == m && !d_shift;
    int sc = run_extract(ctx, e, (cudaStream_t)stream);
    if (h_sum_class) *h_sum_class = sc;
    TC_API_END(ctx)
}

int tc_kshape_run(tc_ctx* ctx, const tc_job* job, tc_result* res) {
    if (!ctx) return TC_ERR_ARG;
    TC_API_BEGIN
    auto t0 = std::chrono::steady_clock::now();
    TC_REQUIRE(job && res, TC_ERR_ARG, "null job/result");
    TC_REQUIRE(job->n >= 1, TC_ERR_ARG, "n must be >= 1");
    check_shape(job->n, job->m, job->k, job->mode);
    TC_REQUIRE((job->h_data != nullptr) != (job->d_data != nullptr), TC_ERR_ARG, "give exactly one of h_data/d_data");
    TC_REQUIRE(job->init_chose == 0 || job->init_chose == 1, TC_ERR_ARG, "init_chose must be 0 or 1");
    TC_REQUIRE(job->init_chose == 0 || job->k <= job->n, TC_ERR_ARG, "init_chose=1 needs k <= n");
    TC_REQUIRE(job->precision >= TC_PREC_FP32 && job->precision <= TC_PREC_TF32, TC_ERR_ARG, "unknown precision");
    TC_REQUIRE(res->h_labels, TC_ERR_ARG, "null label output");
    if (job->h_init_labels)
        for (int64_t i = 0; i < job->n; ++i)
            TC_REQUIRE(job->h_init_labels[i] >= 0 && job->h_init_labels[i] < job->k, TC_ERR_ARG,
                       "initial label out of range");
    TC_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->own_stream;
    const int64_t n = job->n;
    const int m = job->m, k = job->k;
    float* x = ctx->ws.x.as<float>((size_t)n * m);
    // the series stay fixed for the whole run: their BF16 copy is made once
    const int F = fft_size(m, job->mode);
    const bool bf16 = (job->precision != TC_PREC_FP32 && tc_assign_supported(m, F, k, job->precision)) ||
                      (job->precision == TC_PREC_FP32 && screen_supported(m, F, k));
    if (bf16) prepare_series_bf16_reserve(ctx, n, m);
    // upload, z-norm (test_kshape.cu:37 / :99) and BF16 copy in row chunks: the copy
    // stream uploads chunk i+1 while this stream normalises chunk i (rows are independent)
    const int64_t chunk = std::max<int64_t>((n + 7) / 8, std::max<int64_t>(1, (16 << 20) / (4 * (int64_t)m)));
    struct Events {  // destroyed on every exit; each is released once its recorded work completes
        std::vector<cudaEvent_t> v;
        ~Events() {
            for (cudaEvent_t e : v) cudaEventDestroy(e);
        }
    } ev;
    for (int64_t r0 = 0; r0 < n; r0 += chunk) {
        const int64_t rows = std::min(chunk, n - r0);
        const size_t off = (size_t)r0 * m, bytes = sizeof(float) * (size_t)rows * m;
        if (job->h_data) {
            cudaEvent_t e;
            TC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            ev.v.push_back(e);
            TC_CUDA(cudaMemcpyAsync(x + off, job->h_data + off, bytes, cudaMemcpyHostToDevice, ctx->copy_stream));
            TC_CUDA(cudaEventRecord(e, ctx->copy_stream));
            TC_CUDA(cudaStreamWaitEvent(s, e, 0));
        } else {
            TC_CUDA(cudaMemcpyAsync(x + off, job->d_data + off, bytes, cudaMemcpyDeviceToDevice, s));
        }
        launch_znorm(x + off, rows, m, 1, ctx->sm_count, s);
        if (bf16) prepare_series_bf16_rows(ctx, x, n, m, r0, rows, s);
    }
    if (bf16) prepare_series_bf16_done(ctx, x, n, m);
    const int cap = job->max_iter > 0 ? job->max_iter : 20;
    LoopState st = run_loop(ctx, job, x, k, job->init_chose == 1, 0, cap, s);
    res->restarted = 0;
    // test_kshape.cu:54-59 / :112-117: too few clusters survived -> rerun k_shape
    // from the random-label start with the full eigensolver.
    if (job->restart && (st.sum_class == 1 || st.sum_class < k / 2)) {
        res->restarted = 1;
        st = run_loop(ctx, job, x, k, 0, 1, cap, s);
    }
    TC_CUDA(cudaMemcpyAsync(res->h_labels, ctx->ws.labels.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    if (res->h_centroids)
        TC_CUDA(cudaMemcpyAsync(res->h_centroids, ctx->ws.centroids.p, sizeof(float) * k * m, cudaMemcpyDeviceToHost,
                                s));
    TC_CUDA(cudaStreamSynchronize(s));
    ctx->prep_x = nullptr;
    res->iterations = st.iterations;
    res->sum_class = st.sum_class;
    res->inertia = st.inertia;
    res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    TC_API_END(ctx)
}

}  // extern "C"
