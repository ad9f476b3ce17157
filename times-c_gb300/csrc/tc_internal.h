// Internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "timesc.h"
#include "screen.cuh"

// ---------------------------------------------------------------- errors
struct TcError {
    int code;
    std::string msg;
};

#define TC_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            throw TcError{TC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

namespace tc {
extern std::atomic<uint64_t> g_launches;  // kernel launches issued by this library
}
// after a kernel launch: counts it, and names the launch site in the error
#define TC_CHECK_LAUNCH()                                                                        \
    do {                                                                                         \
        ::tc::g_launches.fetch_add(1);                                                           \
        cudaError_t e_ = cudaGetLastError();                                                     \
        if (e_ != cudaSuccess)                                                                   \
            throw TcError{TC_ERR_CUDA, std::string("kernel launch at ") + __FILE__ + ":" +        \
                                           std::to_string(__LINE__) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

#define TC_REQUIRE(cond, code, text)                         \
    do {                                                     \
        if (!(cond)) throw TcError{(code), std::string(text)}; \
    } while (0)

// Raise a kernel's dynamic shared memory limit to the device maximum.  Every call
// sets the same value: host threads that launch one kernel with different sizes
// must never lower the limit under a launch, or a replayed CUDA graph, that
// needs more (a kernel run with less shared memory than it addresses faults).
template <class K>
inline void allow_max_dynamic_smem(K kernel) {
    cudaFuncAttributes fa;
    TC_CUDA(cudaFuncGetAttributes(&fa, kernel));
    int dev = 0, optin = 0;
    TC_CUDA(cudaGetDevice(&dev));
    TC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    TC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa.sharedSizeBytes));
}

// ---------------------------------------------------------------- device buffers
// Serialises device allocation and release with CUDA graph capture across the
// host threads of a process: cudaFree synchronises the device, which must not
// happen while another thread captures a stream.
std::recursive_mutex& capture_mutex();

// Diagnostics (TIMESC_GUARD set): every buffer gets a guard zone after its end,
// filled with GUARD_BYTE, which check_guards() verifies - a kernel writing past
// a buffer then changes the guard instead of another allocation.
constexpr unsigned char GUARD_BYTE = 0xA5;
size_t guard_bytes(size_t need);  // 0 unless diagnostics are on

// A grow-only device allocation owned by a context.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void* get(size_t need) {
        if (need <= bytes) return p;
        std::lock_guard<std::recursive_mutex> lk(capture_mutex());
        if (p) cudaFree(base());
        p = nullptr;
        bytes = 0;
        if (need == 0) return nullptr;
        const size_t g = guard_bytes(need);
        cudaError_t e = cudaMalloc(&p, need + 2 * g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            throw TcError{TC_ERR_NOMEM, "cudaMalloc of " + std::to_string(need) + " bytes failed"};
        }
        if (g) {  // guard zones before and after the buffer; the buffer itself poisoned
            cudaMemset(p, GUARD_BYTE, g);
            p = static_cast<char*>(p) + g;
            cudaMemset(static_cast<char*>(p) + need, GUARD_BYTE, g);
            cudaMemset(p, 0xFF, need);  // NaN floats, -1 integers: reads before writes show up
            // cudaMemset runs on the legacy stream, which does not order with the
            // contexts' non-blocking streams: finish the fills before the buffer is used
            cudaDeviceSynchronize();
        }
        bytes = need;
        return p;
    }
    void* base() const { return p ? static_cast<char*>(p) - guard_bytes(bytes) : nullptr; }
    template <class T>
    T* as(size_t count) { return static_cast<T*>(get(count * sizeof(T))); }
    void release() {
        if (!p) return;
        std::lock_guard<std::recursive_mutex> lk(capture_mutex());
        cudaFree(base());
        p = nullptr;
        bytes = 0;
    }
};

// Twiddle tables for one FFT length F (N = F/2 complex points):
//   twN[e] = exp(-2 pi i e / N), twF[f] = exp(-2 pi i f / F), e, f in [0, N)
struct FftTables {
    int F = 0;
    DevBuf twN, twF;
};

// Per-iteration working set of the k-Shape loop and the stage entry points.
struct Workspace {
    DevBuf x;            // normalised series, n*m f32 (whole-loop runs)
    DevBuf labels, old_labels, shift, dist;
    DevBuf centroids, spectra;  // k*m f32; k*(N+1) float2
    DevBuf seg;          // aligned, re-normalised members in cluster order, n*m (f32 or bf16)
    DevBuf perm, chunk_counts, counts, offsets, gate, scal;
    DevBuf gram;         // k*m*m f32
    DevBuf gram_yt;      // transposed, cluster-padded members for the tensor-core Gram
    DevBuf gram_poff;    // padded cluster offsets (int64)
    DevBuf first;        // k*m f32: first aligned member of each cluster (fused gather)
    DevBuf rowsum;       // k*m f64 + k f64
    DevBuf piter;        // power-by-squaring vectors 2*k*ld f32
    DevBuf gram_sq;      // k*m*ld f32: squares of the power-by-squaring matrices
    DevBuf gram_part;    // up to 8 x k*m*ld f32: the Gram's K-share partials
    DevBuf sq_meta;      // k int64 padded offsets + 2k int32 (column counts, flags)
    DevBuf pstats;       // 3*k*4 f64
    DevBuf aux;          // small scalars (changed count, dist sum, sum_class, flags)
    DevBuf toeplitz;     // bf16 shifted centroid copies for the tensor-core correlation
    DevBuf toeplitz_norm;  // k f32 centroid norms
    DevBuf xbf;          // bf16 copy of the series for the tensor-core correlation
    DevBuf xbf_norm;     // n f32 series norms
    DevBuf screen;       // n x SCREEN_CAP candidate centroids + n counts (screened FP32 assignment)
    DevBuf bounds;       // n x k f32: distance lower bounds (bounded assignment)
    DevBuf cprev;        // k x m f32 unit centroids the bounds refer to, + k f32 movements
    DevBuf bstate;       // n f32 + 2n i32: per series the best centroid's upper bound and index, and group key
    DevBuf bperm;        // n i32 positions -> series, + 2k i32 group counts and cursors
    DevBuf xbfp;         // n x mp bf16 + n f32: the BF16 series and norms in position order
    DevBuf tmask;        // one u64 centroid mask per 128-row tile
    DevBuf fprev;        // FP32 form with bounds: n f32 + n i32 (label and distance left) + k x m raw centroids + k u8
    DevBuf memo_labels;  // n i32: the labels of the previous extraction (memo of unchanged clusters)
    DevBuf memo_c;       // 3 x k x m f32: that extraction's input and output centroids, this one's input
    DevBuf memo_flags;   // 3k u8 (dirty, skip, gate for the shift pass) + an i32 valid word
    DevBuf memo_count;   // 3 u64: extractions with the memo, clusters they covered, clusters skipped
    DevBuf loopctl;      // the loop graph's state (LoopCtl)
};

// The extraction's memo (extract.cu): the key of the previous extraction whose
// labels and centroids the workspace holds; the device word `valid` says whether
// those are complete.
struct MemoState {
    const float* x = nullptr;
    int64_t n = -1;
    int m = 0, k = 0, mode = -1, precision = -1, cal_select = -1;
    bool keyed = false;
    bool counters = false;  // memo_count allocated and zeroed
};

// State of the bounded assignment across iterations: the bounds in ws.bounds are
// valid for these series and the unit centroids in ws.cprev.
struct BoundsState {
    const float* x = nullptr;
    int64_t n = 0;
    int m = 0, k = 0, mode = -1, precision = -1;
    bool valid = false;
    bool refresh = true;   // next assignment: a full pass (new bounds)
    bool regroup = false;  // next bounded pass: group the series anew first
    uint64_t moved = 0;    // series whose best centroid changed since the last grouping
    // bounded passes since the last full pass: their evaluated fractions' sum, count, minimum
    double sum_f = 0, min_f = 2;
    int passes = 0;
    // totals for tc_assign_stats; series_pairs: the pairs the bounded passes' series
    // themselves needed (their tiles evaluate bounded_pairs)
    uint64_t screened = 0, bounded = 0, bounded_pairs = 0, series_pairs = 0;
};

struct tc_ctx {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;
    std::string last_error;
    std::vector<FftTables*> fft;  // cached per F
    Workspace ws;
    cudaStream_t own_stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host uploads overlapped with own_stream's work
    // iteration stages replayed from CUDA graphs
    bool graphs = true;
    // launch plans picked by the autotuner, per kernel shape (see assign_fft.cu)
    std::vector<std::pair<uint64_t, uint32_t>> tuned;
    // series whose BF16 copy and norms sit in ws.xbf / ws.xbf_norm (tc_prepare_series)
    const float* prep_x = nullptr;
    int64_t prep_n = 0;
    int prep_m = 0;
    // bounded assignment (used for prepared series and inside tc_kshape_run)
    BoundsState bounds;
    // memo of unchanged clusters in the extraction (same series: prepared, or the run's own)
    MemoState memo;
    // iterations of tc_kshape_run run by the loop graph and by the host, graphs built
    struct {
        uint64_t device_iterations = 0, host_iterations = 0, builds = 0;
    } loop;
    bool loop_graph_failed = false;  // the runtime refused a loop graph: the host runs iterations
};

namespace tc {

// ---------------------------------------------------------------- launch helpers (defined in .cu files)
const FftTables& fft_tables(tc_ctx* ctx, int F);

void launch_znorm(float* x, int64_t n, int m, int ddof, int sm_count, cudaStream_t s);
void launch_init_labels(int32_t* labels, int64_t n, int k, cudaStream_t s);

// centroid spectra: spec[j][f] = conj-free spectrum of c_j scaled by 1/(2N |c_j|), f in [0, N]
void launch_centroid_spectra(tc_ctx* ctx, const float* C, int k, int m, int F, float2* spec, cudaStream_t s);

struct AssignArgs {
    const float* x;
    const float* centroids;    // k*m (tensor-core correlation)
    const float2* spec;        // k*(N+1) (FFT correlation)
    int64_t n;
    int m, k, F;
    int clamp2;                // pad value 2 of get_pos_idx (compat, 2m-1 < 512)
    const int32_t* fixed;      // if set: evaluate only centroid fixed[i] (alignment shifts)
    const uint8_t* gate;       // with fixed: skip series whose centroid's gate is closed (shift 0)
    int32_t* labels;
    float* dist;
    int32_t* shift;
    const int32_t* old_labels;
    int32_t* changed;
    double* dist_sum;
    // exact screening of the FP32 assignment: the tensor-core pass writes, per series,
    // up to SCREEN_CAP candidate centroids in ascending order (ncand -1: all), and the
    // FFT pass evaluates only those
    int32_t* cand;
    int32_t* ncand;
    // lower bounds on the exact distance of every (series, centroid) pair, series-major
    // [n][k] (the bounded assignment across iterations, both forms; see assign_tc.cu):
    //   lb_out  the tensor-core pass writes d16 - lb_d16 for every pair it evaluates
    //           and, in a tile-bounded pass, lowers the bounds of the pairs its tile
    //           skips by delta[j] >= |c_j/|c_j| - c'_j/|c'_j|| (centroid j's movement);
    //           the FFT pass writes d32 - lb_eps for every pair it evaluates
    float* lb_out;
    const float* delta;
    float lb_eps;   // bound on |d32 - d| of the FFT kernel (fft_error)
    float lb_d16;   // bound on |d16 - d| of the tensor-core pass
    unsigned long long* evals;  // tile-bounded pass: (tile, centroid) pairs evaluated (accumulated)
    // tensor-core pass with bounds: per series an upper bound on the exact distance of
    // its best centroid and that centroid; the tile-bounded pass also takes the series
    // in position order (xbf, xbf_norm, perm) and a centroid mask per 128-row tile
    float* ubd;
    int32_t* jb;
    int32_t* gkey;  // per series best * k + second best: the key of the next grouping
    unsigned long long* moved;  // series whose best centroid changed (accumulated)
    const void* xbf;
    const float* xbf_norm;
    const int32_t* perm;
    const unsigned long long* tmask;
    // FFT pass of the FP32 form with bounds: the label and distance it leaves per
    // series; with reuse, a series whose only candidate is that label, of a centroid
    // bitwise unchanged since (same[j]), keeps that distance without a transform
    float* prev_dist;
    int32_t* prev_label;
    const uint8_t* same;
    int reuse;
};
void launch_assign_fft(tc_ctx* ctx, const AssignArgs& a, cudaStream_t s);
// movement of every centroid since cprev (unit vectors, k x m), then cprev <- the unit
// centroids; delta[j] is rounded up, and +inf where one of the two is zero and the
// other not
// With craw (k x m, the raw centroids of the previous call): same[j] = centroid j is
// bitwise unchanged, and craw <- C.
void launch_centroid_delta(const float* C, int k, int m, float* cprev, float* delta, cudaStream_t s,
                           float* craw = nullptr, uint8_t* same = nullptr);
// worst-case |d32 - d| of the FP32 FFT correlation for unit-norm series and centroids
double fft_error(int m, int F);
// worst-case |d16 - d32| of the BF16 tensor-core correlation (the screen's half-width)
double bf16_error(int m, int F);

// tensor-core correlation (tcgen05); returns false when the shape is not supported
bool tc_assign_supported(int m, int F, int k, int precision);
// the FP32 assignment screened by the BF16 tensor-core pass (TIMESC_NO_SCREEN turns it off)
bool screen_supported(int m, int F, int k);
void launch_assign_tc(tc_ctx* ctx, const AssignArgs& a, int precision, cudaStream_t s);
// BF16 copy and norms of the series into the context's workspace, marked as prepared for x
void prepare_series_bf16(tc_ctx* ctx, const float* x, int64_t n, int m, cudaStream_t s);
// the same in row ranges: reserve for n rows, convert [r0, r0 + rows), then mark x prepared
void prepare_series_bf16_reserve(tc_ctx* ctx, int64_t n, int m);
void prepare_series_bf16_rows(tc_ctx* ctx, const float* x, int64_t n, int m, int64_t r0, int64_t rows,
                              cudaStream_t s);
void prepare_series_bf16_done(tc_ctx* ctx, const float* x, int64_t n, int m);
// The tile-bounded BF16 pass's inputs: series grouped by their best centroid jb as of
// the last full pass (perm: position -> series), their BF16 rows and norms in that
// order, and per 128-row tile the centroids a series of the tile may have as its
// minimum (k <= 64).
struct TileBounds {
    const int32_t* perm = nullptr;
    const void* xbf = nullptr;
    const float* xbf_norm = nullptr;
    const unsigned long long* tmask = nullptr;
};
// after a full pass: group the series by the best and second best centroids it found
// (gkey = best * k + second, so groups of one best centroid are adjacent) and copy
// their BF16 rows in that order; the grouping is kept until the next full pass
void launch_tile_group(tc_ctx* ctx, int64_t n, int m, int k, const int32_t* gkey, cudaStream_t s);
// before a bounded pass: the centroid mask of every tile of the kept grouping
// (series_pairs, if set, accumulates the pairs the series' own masks hold)
void launch_tile_masks(tc_ctx* ctx, int64_t n, int m, int k, const float* lb, const float* ubd, const int32_t* jb,
                       const float* delta, float D, TileBounds& out, cudaStream_t s,
                       unsigned long long* series_pairs = nullptr);

// extraction
struct ExtractArgs {
    const float* x;
    const int32_t* labels;
    const int32_t* shift;      // may be null when no gate is set
    float* C;
    int64_t n;
    int m, k, mode, cal_select, precision;
    int32_t* counts;           // k
    // the series stay fixed across calls (prepared, or the run's own copy): clusters
    // whose members and centroid equal the previous extraction's reuse its output
    int memo;
};
// Starts the memo for extractions with these arguments: forgets the previous
// extraction unless it had the same series and shape.  Called outside graph capture
// (run_extract calls it; the loop calls it once before its captured iterations).
void memo_prepare(tc_ctx* ctx, const ExtractArgs& a, cudaStream_t s);
// Forgets the previous extraction (its outputs may be incomplete, or the series changed).
inline void memo_invalidate(tc_ctx* ctx) { ctx->memo.keyed = false; }
// no host synchronisation: sum_class and the bad-label flag stay in ws.scal[0..1],
// the Gram error word at aux+48
void extract_async(tc_ctx* ctx, const ExtractArgs& a, cudaStream_t s);
// extract_async, then reads and checks the flags; returns sum_class
int run_extract(tc_ctx* ctx, const ExtractArgs& a, cudaStream_t s);

// operand of the tensor-core Gram (transposed, cluster-padded members)
struct GramOperand {
    void* YT = nullptr;
    float* YTlo = nullptr;  // 3xTF32 lo plane
    int64_t Pp = 0;         // columns (padded positions)
    int fmt = 0;            // 1 BF16, 2 TF32, 3 3xTF32
};
GramOperand gram_tc_operand(tc_ctx* ctx, int64_t n, int k, int m, int precision);
size_t gram_operand_bytes(int64_t n, int k, int m, int precision);
bool gram_tc_supported(int m, int precision);
int64_t gram_padded_cols(int64_t n, int k);
// S_c = YT_c YT_c^T for every cluster (seg == nullptr: the operand is already in place)
// skip (may be null): clusters whose Gram is not needed (their S is left as it was)
void launch_gram_tc(tc_ctx* ctx, const float* seg, const int32_t* counts, const int32_t* offsets,
                    const int64_t* poff, int64_t n, int k, int m, int ld, int precision, float* S, int* err,
                    cudaStream_t s, const uint8_t* skip = nullptr);
// power iteration by repeated squaring (power_sq.cu): vec[c] ~ M_c^e v0 where ok[c]
struct SquaringResult {
    const float* vec = nullptr;  // k x ld, not normalised
    const int32_t* ok = nullptr;  // k flags
};
bool power_squaring_supported(int m, int k, int sm_count);
size_t power_squaring_operand_bytes(int k, int m);
SquaringResult power_squaring(tc_ctx* ctx, const float* S, int ld, const double* r, const double* tot,
                              const int32_t* counts, int k, int m, int64_t e, int* err, cudaStream_t s);
// the extraction's gather written straight into that operand (m <= 1024), plus the
// first member row of every cluster into first[k][m]
bool gather_transposed_supported(int m);
void launch_gather_norm_t(const float* x, const int32_t* perm, const int32_t* labels, const int32_t* shift,
                          const uint8_t* gate, const int32_t* offsets, const int32_t* counts, int k,
                          const int64_t* poff, int64_t n, int m, bool bf16, void* YT, float* YTlo, int64_t Pp,
                          float* first, cudaStream_t s, const uint8_t* skip = nullptr);

// workspace of a context: free every buffer (the context must be idle) / bytes held
void release_workspace(tc_ctx* ctx);
size_t workspace_bytes(tc_ctx* ctx);
// with TIMESC_GUARD: synchronise the context's stream and throw if a buffer's
// guard zone changed (names the buffer and `where`)
void check_guards(tc_ctx* ctx, const char* where);

// helpers
inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
int fft_size(int m, int mode);

}  // namespace tc
