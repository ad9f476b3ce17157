/*
 * timesc.h - C ABI of the GB300 k-Shape engine (drop-in for the Times-C
 * `./test -d dev path k flag init_chose` path).
 *
 * All entry points return a tc_status (0 = success) and never exit the process.
 * Device buffers passed in are owned by the caller and used in stream order on
 * the given stream (NULL = the legacy default stream).  A context owns its
 * scratch (spectra, Gram matrices, segment buffers) and reuses it across calls;
 * one context must be driven from one host thread at a time.
 *
 * Reference interfaces replaced (paths inside the Times-C project):
 *   tc_znorm            z_norm_gpu_x<T>        Code/include/normalization.cuh:150-177
 *   tc_init_labels      idx_init / rand_init   Code/include/kshape.cuh:16-32
 *   tc_sbd_assign       NCC_3D + get_pos_idx   Code/include/ncc.cuh:469-517, Code/include/kshape.cuh:35-96
 *   tc_extract_shapes   extract_shape<T>       Code/include/shapeExtract.cuh:1058-1181 (+ sbd3D, SBD.cuh:69-85)
 *   tc_kshape_run       k_shape / k_shape_tsl + the driver restart
 *                                              Code/include/kshape.cuh:197-474, Code/test/test_kshape.cu:13-137
 *   tc_read_file        readFile / read_unlabeled_File   Code/include/readfile.cuh:13-116
 *   tc_write_labels     writeFile<int>         Code/include/readfile.cuh:121-129
 *   tc_random_select    randomSelectK          Code/include/kshape.cuh:159-176
 *   tc_k_from_labels    k from the label column  Code/test/test_kshape.cu:24-30
 *   tc_fft_size         fft_size rule          Code/include/ncc.cuh:12-16, :473
 */
#ifndef TIMESC_H
#define TIMESC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TC_ABI_VERSION 1

typedef struct tc_ctx tc_ctx;
typedef struct CUstream_st* tc_stream; /* the same type as cudaStream_t */

typedef enum {
    TC_OK = 0,
    TC_ERR_ARG = 1,         /* invalid argument (sizes, pointers, alignment) */
    TC_ERR_CUDA = 2,        /* a CUDA runtime call or a kernel launch failed */
    TC_ERR_NOMEM = 3,       /* device or host allocation failed */
    TC_ERR_IO = 4,          /* file could not be read/written or parsed */
    TC_ERR_TIMEOUT = 5,     /* a bounded device wait ran out; the context stays usable */
    TC_ERR_UNSUPPORTED = 6, /* size or mode not supported by this build */
    TC_ERR_REJECTED = 7     /* job refused by admission control */
} tc_status;

typedef enum {
    TC_MODE_COMPAT = 0,    /* the reference GPU build: FFT size rounded down, int-truncated gate, unit-norm centroids */
    TC_MODE_CANONICAL = 1  /* k-Shape as published: FFT size >= 2m-1, real gate, re-z-normalised centroids */
} tc_mode;

typedef enum {
    TC_PREC_FP32 = 0,      /* FP32 FFT correlation; Gram matrices in 3xTF32 on the tensor cores.  Where
                              the BF16 correlation applies (FFT length 128..1024, k >= 2, no shift
                              requested) a BF16 tensor-core pass first keeps, per series, only the
                              centroids whose FP32 distance can be the minimum (a rigorous bound on
                              the BF16 error); the FP32 pass evaluates those: same labels and
                              distances as evaluating all (TIMESC_NO_SCREEN=1 turns it off) */
    TC_PREC_BF16 = 1,      /* BF16 operands, FP32 accumulation, on the tensor cores (tcgen05): the
                              correlation when FFT length is 128..1024 (m <= 512) and no shift is
                              requested (the FP32 FFT correlation otherwise), and the Gram matrices */
    TC_PREC_TF32 = 2       /* TF32 Gram matrices on the tensor cores; FP32 FFT correlation */
} tc_precision;

/* ---------------------------------------------------------------- context */
int tc_version(void);
int tc_create(int device, tc_ctx** out);
int tc_destroy(tc_ctx* ctx);
/* Message of the last failed call on this context ("" if none). */
const char* tc_last_error(const tc_ctx* ctx);
/* Number of kernel launches this library has issued in this process (all
 * contexts); for accounting in benchmarks.  No reference counterpart. */
uint64_t tc_launch_count(void);

/* ---------------------------------------------------------------- stages (device pointers) */
/* FFT length the mode uses for series length m. */
int tc_fft_size(int m, int mode);

/* In place: each of n rows of length m becomes (x - mean) / std(ddof).  Rows with
 * zero spread become zeros. */
int tc_znorm(tc_ctx* ctx, float* d_x, int64_t n, int m, int ddof, tc_stream stream);

/* Initial labels of init_chose=0: label_i = curand(XORWOW seeded with i) % k,
 * written 0-based (the reference stores it +1). */
int tc_init_labels(tc_ctx* ctx, int32_t* d_labels, int64_t n, int k, tc_stream stream);

/* SBD assignment.  For every series (z-normalised row of d_x) and centroid: the
 * normalised cross-correlation over all lags of the mode's FFT length; the series
 * gets the centroid with the smallest 1 - max NCC (first centroid on ties).
 * Outputs (any may be NULL except d_labels): d_labels (0-based), d_dist (that
 * smallest distance), d_shift (the shift that aligns the series to its centroid:
 * out[t] = x[t - shift]).  If d_old_labels is not NULL, *d_changed receives the
 * number of labels that differ from it; d_dist_sum receives the FP64 sum of
 * d_dist (both accumulated: zero them first).  On prepared series (tc_prepare_series)
 * a call may use the distance bounds kept from earlier calls (tc_assign_stats), with
 * the same results. */
int tc_sbd_assign(tc_ctx* ctx, const float* d_x, const float* d_centroids, int64_t n, int m, int k,
                  int mode, int precision, int32_t* d_labels, float* d_dist, int32_t* d_shift,
                  const int32_t* d_old_labels, int32_t* d_changed, double* d_dist_sum,
                  tc_stream stream);

/* Keeps a BF16 copy of the series d_x (n rows of length m <= 512) and their FP32
 * norms in the context for the tensor-core correlation: later tc_sbd_assign calls
 * with TC_PREC_BF16 (or TC_PREC_FP32, whose screening pass uses it) and the same
 * d_x, n and m use it instead of converting the series again.  The copy is taken now: call again after changing d_x.  Any
 * tc_sbd_assign on other series, and tc_kshape_run, drop it.  No counterpart in
 * the reference (NCC_3D transforms the series on every iteration). */
int tc_prepare_series(tc_ctx* ctx, const float* d_x, int64_t n, int m, tc_stream stream);

/* Work of the assignments on this context since its creation.  On series kept
 * fixed across calls (tc_prepare_series, and inside tc_kshape_run) the assignment
 * keeps lower bounds on every (series, centroid) distance, in both precision forms
 * at FFT lengths 128..1024 (m <= 512): a full call builds them (in TC_PREC_FP32 the
 * screened call: the BF16 tensor-core pass and the FP32 pass over its candidates),
 * and later calls carry them over with each centroid's movement and evaluate only
 * the pairs whose bound does not rule them out, per 128-series tile of series
 * grouped by their best centroid (in TC_PREC_FP32 that tile-bounded BF16 pass is the
 * screen, and the FP32 pass evaluates its candidates) - with labels and distances
 * equal to evaluating every pair.  A full call runs again once the bounded calls
 * since the last one have cost about one full call more than the cheapest of them
 * would have.  screened: calls that built
 * bounds; bounded: calls that used them; bounded_pairs: pairs those evaluated (out
 * of n*k each, counted in whole 128-series tiles).  Any output may be NULL.
 * TIMESC_NO_BOUNDS=1 in the environment turns the bounds off; TIMESC_REGROUP_SHARE=s
 * groups the series anew once 1/s of them changed best centroid (default 20).  No
 * counterpart in the reference. */
int tc_assign_stats(const tc_ctx* ctx, uint64_t* screened, uint64_t* bounded, uint64_t* bounded_pairs);

/* Work the extraction memo saved on this context since its creation: extractions
 * that compared their clusters with the previous call's (prepared series, and
 * every extraction inside tc_kshape_run except the repeated-squaring forms),
 * clusters they covered, and clusters whose output was reused instead of
 * recomputed.  Synchronises the device.  Any output may be NULL.  No counterpart in
 * the reference. */
int tc_extract_stats(tc_ctx* ctx, uint64_t* extractions, uint64_t* clusters, uint64_t* reused);

/* Allocation-free SBD assignment.  No counterpart in the reference.
 * For callers that must not allocate device memory on the call path: a serving
 * loop that reserved all HBM for resident jobs up front, or a latency-critical
 * host thread that cannot take cudaMalloc's implicit device synchronisation.
 * Same kernels and results as tc_sbd_assign with precision TC_PREC_FP32 (labels
 * 0-based, d_dist may be NULL), but no context: the scratch (twiddle tables and
 * centroid spectra, 2*(F/2) + k*(F/2+1) complex values, F = tc_fft_size(m, mode))
 * lives in one static device array of TC_NOALLOC_SCRATCH_BYTES that every GPU
 * loading the library holds until the process exits.  Larger requests return
 * TC_ERR_UNSUPPORTED with a message in err (may be NULL).  Calls no cudaMalloc or
 * cudaFree.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  All
 * calls share the array: calls that overlap on the GPU (other streams, other host
 * threads) race on it - serialise them. */
#define TC_NOALLOC_SCRATCH_BYTES (4u << 20)
int tc_sbd_assign_noalloc(const float* d_x, const float* d_centroids, int64_t n, int m, int k, int mode,
                          int32_t* d_labels, float* d_dist, tc_stream stream, char* err, int err_len);

/* Shape extraction: groups the rows by label (stable), aligns the members of each
 * cluster whose centroid passes the mode's gate (using d_shift if given, else
 * computing the shifts against d_centroids), re-z-normalises them, and replaces
 * each non-empty cluster's centroid by the top eigenvector of Q S Q (S = the
 * members' Gram matrix, Q = I - 11^T/m) with the reference's sign rule.
 * cal_select = 1 takes the fully converged top eigenvector (the reference's
 * syevd path).  Empty clusters keep their centroid.  d_counts (k, may be NULL)
 * receives the cluster sizes and *h_sum_class (may be NULL) the number of
 * non-empty clusters (this synchronises the stream).  On prepared series
 * (tc_prepare_series) without d_shift, a cluster whose members and centroid equal
 * those of the previous call on this context gets that call's output again
 * without being recomputed - the same bits, as every stage is deterministic per
 * cluster (tc_extract_stats; TIMESC_NO_MEMO=1 turns it off). */
int tc_extract_shapes(tc_ctx* ctx, const float* d_x, const int32_t* d_labels, const int32_t* d_shift,
                      float* d_centroids, int64_t n, int m, int k, int mode, int cal_select,
                      int precision, int32_t* d_counts, int* h_sum_class, tc_stream stream);

/* ---------------------------------------------------------------- whole loop */
typedef struct {
    const float* h_data;          /* n*m raw values on the host (row-major), or NULL */
    const float* d_data;          /* or the same on the device (not modified); one of the two */
    int64_t n;
    int m;
    int k;
    int mode;                     /* tc_mode */
    int precision;                /* tc_precision */
    int init_chose;               /* 0: random labels (curand), 1: k random raw rows as centroids */
    uint32_t seed;                /* mt19937 seed of the init_chose=1 draw */
    int max_iter;                 /* iteration cap; <= 0 means 20 (the reference's unlabelled cap) */
    int restart;                  /* 1: rerun with cal_select=1 when <= k/2 clusters survive */
    const int32_t* h_init_labels; /* optional 0-based initial labels instead of the curand draw */
} tc_job;

typedef struct {
    int32_t* h_labels;            /* out: n labels, 0-based (host) */
    float* h_centroids;           /* out: k*m centroids (host), may be NULL */
    int iterations;               /* iterations of the last loop */
    int sum_class;                /* non-empty clusters after the last extraction */
    int restarted;                /* 1 if the cal_select=1 rerun happened */
    double inertia;               /* mean distance of the last assignment */
    double seconds;               /* wall time of the call */
} tc_result;

/* The reference's whole path after parsing: copy in (if h_data), z-normalise,
 * initialise, iterate (extract/assign/converge in the reference's loop order for
 * init_chose), apply the restart rule, copy labels/centroids out.  Synchronous.
 * Each iteration's stages are replayed from CUDA graphs.  With TIMESC_DEVICE_LOOP=1
 * in the environment, once those are captured the remaining iterations run as one
 * graph launch: a conditional WHILE node over the stages, with the convergence test,
 * the class-count stop and the assignment's bounds rule evaluated on the device (no
 * host round trip per iteration; the same results as the host-driven loop). */
int tc_kshape_run(tc_ctx* ctx, const tc_job* job, tc_result* result);

/* Iterations of tc_kshape_run on this context since its creation that ran inside
 * the loop graph and on the host, and loop graphs built.  Any output may be NULL.
 * No counterpart in the reference. */
int tc_loop_stats(const tc_ctx* ctx, uint64_t* device_iterations, uint64_t* host_iterations,
                  uint64_t* graphs_built);

/* ---------------------------------------------------------------- many jobs: batch and serving */
/* No counterpart in the reference, which runs one job per process.  A pool owns
 * `workers` contexts (each a stream and a workspace) and host threads that run
 * tc_kshape_run on them, so the iterations of different jobs overlap on the
 * device.  Admission: the device memory held by the workers' workspaces, plus
 * the footprint (tc_job_footprint) reserved for each running job, stays within
 * hbm_budget_bytes; a job starts when a worker is free and its footprint fits,
 * idle workers give their workspaces back when a job needs the room, and a job
 * larger than the budget is rejected (TC_ERR_REJECTED). */
typedef struct {
    int workers;                  /* jobs in flight at once; <= 0 means 8 */
    uint64_t hbm_budget_bytes;    /* 0 means 80% of the device memory free at creation */
} tc_pool_opts;

typedef struct tc_pool tc_pool;

int tc_pool_create(int device, const tc_pool_opts* opts, tc_pool** out);
/* Waits for every submitted job, then frees the workers. */
int tc_pool_destroy(tc_pool* pool);
/* Upper estimate of the device bytes a worker's workspace grows by for job. */
uint64_t tc_job_footprint(const tc_job* job);

/* Batch: runs jobs[0..njobs) to completion, largest estimated work first;
 * statuses[i] (if not NULL) gets job i's tc_status.  Returns TC_OK, or the first
 * failing status.  The job's host buffers and result stay the caller's. */
int tc_pool_run_batch(tc_pool* pool, const tc_job* jobs, int njobs, tc_result* results, int* statuses);

/* Serving: queue one job (FIFO; a job that does not fit the memory left lets
 * smaller queued jobs start first).  *job and *result must stay valid until the
 * job is waited for.  Returns TC_ERR_REJECTED at once for a job larger than the
 * budget. */
int tc_pool_submit(tc_pool* pool, const tc_job* job, tc_result* result, uint64_t* ticket);
/* Blocks until the job is done; *status = its tc_status, *queued_s = seconds from
 * submission to start, *latency_s = seconds from submission to completion (any
 * output pointer may be NULL). */
int tc_pool_wait(tc_pool* pool, uint64_t ticket, int* status, double* queued_s, double* latency_s);
/* Jobs running and queued now, and the bytes held or reserved by the workers. */
int tc_pool_stats(tc_pool* pool, int* running, int* queued, uint64_t* held_bytes);

/* ---------------------------------------------------------------- host I/O */
/* Parse a text file: one series per line, values separated by commas (a line
 * with a comma is split on commas only) or else by spaces/tabs.  labeled=1: the
 * first token is an integer label.  *data (n*m) and *labels (n, or NULL) are
 * malloc'ed and released with tc_free_host. */
int tc_read_file(const char* path, int labeled, float** data, int32_t** labels, int64_t* n, int* m,
                 char* err, int err_len);
void tc_free_host(void* p);
/* Writes "l0,l1,...,l(n-1)," on one line (labels as given). */
int tc_write_labels(const char* path, const int32_t* labels, int64_t n);
/* Writes k lines of m comma-separated values. */
int tc_write_centroids(const char* path, const float* centroids, int k, int m);
int tc_random_select(int64_t n, int k, uint32_t seed, int32_t* out);
int tc_k_from_labels(const int32_t* labels, int64_t n);

/* ---------------------------------------------------------------- synthetic workloads */
typedef struct {
    int64_t n;
    int m;
    int classes;          /* number of prototypes */
    double noise;         /* noise sigma as a fraction of the prototype std */
    double dirichlet;     /* > 0: class sizes ~ Dirichlet(alpha); 0: equal sizes */
    uint64_t seed;
} tc_gen_spec;
/* Fills data (n*m) and labels (n, 0-based, may be NULL). */
int tc_generate(const tc_gen_spec* spec, float* data, int32_t* labels);

#ifdef __cplusplus
}
#endif
#endif
