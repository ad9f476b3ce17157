/*
 * Times-C k-Shape oracle: a CPU FP64 restatement of the reference's k-Shape path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only as
 * the checker or the timed CPU baseline.  The product (times-c_gb300/) never
 * links, loads or calls it.
 *
 * Three semantic modes:
 *   OR_MODE_COMPAT    the reference GPU build (Code/test/test_kshape.cu + Code/include/*.cuh)
 *                     with its intended arithmetic: FFT size rounded down
 *                     (ncc.cuh:12-16, :473), circular lag slots (ncc.cuh:230-245),
 *                     int-truncating alignment gate (shapeExtract.cuh:1131),
 *                     m power iterations from [1,.5,1,.5,...] (shapeExtract.cuh:269-283,
 *                     :590-606), unit-norm centroid with the get_center sign rule
 *                     (shapeExtract.cuh:217-264), loop orders and convergence of
 *                     kshape.cuh:197-474 and the driver restart of test_kshape.cu:54-59.
 *   OR_MODE_CANONICAL k-Shape as published: FFT size >= 2m-1, alignment whenever the
 *                     centroid is non-zero, exact top eigenvector, re-z-normalised
 *                     centroid (ddof=1); same loop control as COMPAT.
 *   OR_MODE_PYREF     the reference's numpy CPU path Code/test/test_timesC.py
 *                     (reversed alignment :127-133, ddof=0 initial z-score :214,
 *                     eigh fallback test :159-192, re-z-scored centroid :204,
 *                     label-equality stop :262).  Used only to pin this oracle
 *                     against the reference's own runnable code.
 */
#ifndef TC_ORACLE_H
#define TC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_MODE_COMPAT = 0, OR_MODE_CANONICAL = 1, OR_MODE_PYREF = 2 };

typedef struct {
    const float* data;          /* n*m raw values as parsed (not normalised) */
    int64_t n;
    int m;
    int k;
    int mode;                   /* OR_MODE_* */
    int init_chose;             /* 0: random labels, 1: random raw rows as centroids */
    const int32_t* init_labels; /* n labels, 0-based (the curand draw of kshape.cuh:16-32) */
    uint32_t seed;              /* mt19937 seed of the init_chose=1 row draw */
    int max_iter;               /* iteration cap (reference: 10 labelled, 20 unlabelled) */
    int restart;                /* 1: apply the sum_class restart of test_kshape.cu:54-59 */
} or_job;

typedef struct {
    int32_t* labels;            /* out: n labels, 0-based */
    double* centroids;          /* out: k*m */
    int iterations;             /* iterations run by the last loop */
    int sum_class;              /* non-empty clusters after the last extraction */
    int restarted;              /* 1 if the cal_select=1 rerun happened */
    double inertia;             /* mean best distance of the last assignment */
    double min_margin;          /* smallest (second-best - best) distance seen in any assignment */
} or_result;

/* FFT length used by a mode for series length m. */
int or_fft_size(int m, int mode);

/* In-place z-normalisation of n rows of length m (FP64).  zero_std: rows whose
 * standard deviation is zero become all zeros. */
void or_znorm(double* x, int64_t n, int m, int ddof);

/* Normalised cross-correlation slots of NCC_3D for one pair (ncc.cuh:469-517):
 * out[j] = circcorr_F(x, y)[(j-m+1) mod F] / (|x||y|), j in [0, 2m-1); a zero
 * norm product gives 0 (the 1e10 rule of ncc.cuh:89). */
void or_ncc(const double* x, const double* y, int m, int F, double* out);
/* Same by direct summation (for cross-checking the FFT). */
void or_ncc_naive(const double* x, const double* y, int m, int F, double* out);

/* Alignment of one member to a centroid (sbd3D + maxAndShift, SBD.cuh:49-85):
 * shift = first argmax of NCC(center, member) + 1 - m; out = member shifted with
 * zero fill (out[t] = member[t - shift]).  Returns the shift. */
int or_align(const double* center, const double* member, int m, int F, double* out);
/* zeroShift (SBD.cuh:14-29) / roll_zeropad (test_timesC.py:55-77). */
void or_shift_row(const double* x, int m, int shift, double* out);

/* Assignment (NCC_3D + get_pos_idx, kshape.cuh:35-96).  labels 0-based; dist =
 * min over slots of 1-ncc for the chosen centroid; shift = the alignment shift
 * sbd3D would apply to the series against its chosen centroid (SBD.cuh:49-65);
 * margin = second-best minus best distance.  clamp2: pad value 2 of get_pos_idx
 * when 2m-1 < 512 (kshape.cuh:55-60). */
void or_assign(const double* X, const double* C, int64_t n, int m, int k, int F, int clamp2,
               int32_t* labels, double* dist, int32_t* shift, double* margin);

/* One shape extraction (shapeExtract.cuh:1058-1181 for COMPAT/CANONICAL,
 * test_timesC.py:127-204 for PYREF).  X: n*m normalised rows; labels 0-based;
 * C: k*m centroids in/out; counts: k out.  cal_select=1 takes the top
 * eigenvector from a full eigensolver (get_class_centers_a).  Returns sum_class. */
int or_extract(const double* X, const int32_t* labels, double* C, int64_t n, int m, int k,
               int mode, int cal_select, int32_t* counts);

/* Top eigenvector of a symmetric m*m matrix by cyclic Jacobi: the eigenvector of
 * the largest eigenvalue (ties: the largest index), as the last column of an
 * ascending eigendecomposition. Returns the eigenvalue. */
double or_top_eig_jacobi(const double* A, int m, double* vec);

/* k distinct row indices by mt19937(seed) + uniform_int_distribution<>(0,n-1) with
 * rejection of repeats (kshape.cuh:159-176, with the random_device seed replaced). */
void or_random_select(int64_t n, int k, uint32_t seed, int32_t* out);

/* The whole k-Shape loop. Returns 0 on success. */
int or_kshape(const or_job* job, or_result* res);

/* Adjusted Rand index of two labelings. */
double or_ari(const int32_t* a, const int32_t* b, int64_t n);

/* Label parsing of the reference: k from labels (test_kshape.cu:24-30). */
int or_k_from_labels(const int32_t* labels, int64_t n);

// The engine's synthetic workloads (times-c_gb300/csrc/gen_core.h): data n*m,
// labels n (may be null).  Returns 0, or 1 for invalid parameters.
int or_generate(int64_t n, int m, int classes, double noise, double dirichlet, uint64_t seed, float* data,
                int32_t* labels);

#ifdef __cplusplus
}
#endif
#endif
