// Times-C k-Shape oracle: CPU FP64 restatement of the reference path.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
// CPU legs of bench.py as the checker / timed CPU baseline.  Never part of the
// product.  Every function cites the reference file:line it restates (paths
// relative to the Times-C project root).
#include "oracle.h"

#include "gen_core.h"  // the synthetic workloads (header-only; the engine library is not linked)

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <random>
#include <set>
#include <vector>

typedef std::complex<double> cd;

// ---------------------------------------------------------------------------
// FFT (textbook iterative radix-2 Cooley-Tukey, FP64).  Twiddles come from a
// directly evaluated root table, so error stays at a few ulp of log2(F).
// ---------------------------------------------------------------------------
namespace {

struct FftPlan {
    int n = 0;
    std::vector<cd> roots;      // exp(-2 pi i j / n)
    std::vector<cd> iroots;     // their conjugates (inverse transform)
    std::vector<int> rev;
    void init(int n_) {
        n = n_;
        roots.resize(n);
        for (int j = 0; j < n; ++j) {
            double a = -2.0 * M_PI * (double)j / (double)n;
            roots[j] = cd(std::cos(a), std::sin(a));
        }
        iroots.resize(n);
        for (int j = 0; j < n; ++j) iroots[j] = std::conj(roots[j]);
        rev.assign(n, 0);
        int lg = 0;
        while ((1 << lg) < n) ++lg;
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < lg; ++b)
                if (i & (1 << b)) r |= 1 << (lg - 1 - b);
            rev[i] = r;
        }
    }
    // forward: sign -1; inverse (unnormalised): conj twiddles
    void run(cd* a, bool inverse) const {
        for (int i = 0; i < n; ++i)
            if (i < rev[i]) std::swap(a[i], a[rev[i]]);
        const cd* rt = inverse ? iroots.data() : roots.data();
        for (int len = 2; len <= n; len <<= 1) {
            int half = len >> 1, step = n / len;
            for (int i = 0; i < n; i += len)
                for (int j = 0; j < half; ++j) {
                    const cd w = rt[j * step];
                    cd u = a[i + j], v = a[i + j + half] * w;
                    a[i + j] = u + v;
                    a[i + j + half] = u - v;
                }
        }
    }
};

double norm2(const double* x, int m) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += x[i] * x[i];
    return std::sqrt(s);
}

// r[tau] = sum_t x[(t+tau) mod F] * y[t]  for tau in [0,F)   (ncc.cuh:124-145 + C2R :358)
void circ_corr_spec(const std::vector<cd>& X, const std::vector<cd>& Y, const FftPlan& p,
                    std::vector<cd>& work, double* r) {
    int F = p.n;
    for (int f = 0; f < F; ++f) work[f] = X[f] * std::conj(Y[f]);
    p.run(work.data(), true);
    for (int f = 0; f < F; ++f) r[f] = work[f].real() / F;
}

// The same correlation through a complex transform of half the length (Z = X conj(Y)
// is Hermitian, so r is real): with N = F/2, A[k] = Z[k] + Z[k+N] and
// B[k] = (Z[k] - Z[k+N]) exp(2 pi i k/F), the inverse transform of A + iB holds
// r[2t] in its real and r[2t+1] in its imaginary parts.  pF: length F, pN: F/2.
void circ_corr_half(const std::vector<cd>& X, const std::vector<cd>& Y, const FftPlan& pF, const FftPlan& pN,
                    std::vector<cd>& work, double* r) {
    const int F = pF.n, N = F / 2;
    for (int f = 0; f <= N; ++f) work[f] = X[f] * std::conj(Y[f]);  // Z[0..N]
    cd* c = work.data() + N + 1;                                    // N values after Z[0..N]
    for (int q = 0; q < N; ++q) {
        const cd z0 = work[q], z1 = std::conj(work[N - q]);  // Z[q], Z[q+N]
        c[q] = (z0 + z1) + cd(0, 1) * ((z0 - z1) * pF.iroots[q]);
    }
    pN.run(c, true);
    for (int t = 0; t < N; ++t) {
        r[2 * t] = c[t].real() / F;
        r[2 * t + 1] = c[t].imag() / F;
    }
}

void spectrum(const double* x, int m, const FftPlan& p, std::vector<cd>& out) {
    out.assign(p.n, cd(0, 0));
    for (int i = 0; i < m; ++i) out[i] = cd(x[i], 0);
    p.run(out.data(), false);
}

inline int slot_to_circ(int j, int m, int F) {  // copy_result2D (ncc.cuh:241)
    long v = (long)j - m + 1;
    v %= F;
    if (v < 0) v += F;
    return (int)v;
}

}  // namespace

extern "C" {

// ncc.cuh:12-16 and :473: fft_size = 1 << (int)ceil(my_log2(2m-1)) where my_log2
// returns an int (truncated), so the size is rounded DOWN.  test_timesC.py:88:
// 1 << (2m-1).bit_length().  Canonical k-Shape uses the Python form.
int or_fft_size(int m, int mode) {
    int x = 2 * m - 1;
    if (mode == OR_MODE_COMPAT) {
        int lg = (int)(std::log((double)x) / std::log(2.0));
        return 1 << (int)std::ceil((double)lg);
    }
    int bl = 0;
    while ((1 << bl) <= x) ++bl;  // bit_length
    return 1 << bl;
}

// normalization.cuh:94-118 (row mean via GEMM, subtract) and :30-64
// (x /= sqrt(sum x^2 / (m - ddof))).  A row with zero spread becomes zeros
// (the reference divides 0/0; test_timesC.py:52 maps that NaN to 0).
void or_znorm(double* x, int64_t n, int m, int ddof) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double* r = x + i * (int64_t)m;
        double mean = 0;
        for (int t = 0; t < m; ++t) mean += r[t];
        mean /= m;
        double ss = 0;
        for (int t = 0; t < m; ++t) {
            r[t] -= mean;
            ss += r[t] * r[t];
        }
        double sd = std::sqrt(ss / (double)(m - ddof));
        if (!(sd > 0) || !std::isfinite(sd)) {
            for (int t = 0; t < m; ++t) r[t] = 0;
        } else {
            for (int t = 0; t < m; ++t) r[t] /= sd;
        }
    }
}

// NCC_3D for a single pair (ncc.cuh:469-517): norms (:19-71), den 0 -> 1e10
// (:76-101, so the result is 0), zero pad to F (:249-259), R2C, X*conj(Y)/(F*den)
// (:124-145), C2R (:358), lag reorder (:230-245).
void or_ncc(const double* x, const double* y, int m, int F, double* out) {
    FftPlan p;
    p.init(F);
    std::vector<cd> X, Y, work(F);
    spectrum(x, m, p, X);
    spectrum(y, m, p, Y);
    std::vector<double> r(F);
    circ_corr_spec(X, Y, p, work, r.data());
    double den = norm2(x, m) * norm2(y, m);
    for (int j = 0; j < 2 * m - 1; ++j) out[j] = den == 0 ? 0.0 : r[slot_to_circ(j, m, F)] / den;
}

void or_ncc_naive(const double* x, const double* y, int m, int F, double* out) {
    std::vector<double> xp(F, 0.0), yp(F, 0.0);
    for (int i = 0; i < m; ++i) { xp[i] = x[i]; yp[i] = y[i]; }
    double den = norm2(x, m) * norm2(y, m);
    for (int j = 0; j < 2 * m - 1; ++j) {
        int tau = slot_to_circ(j, m, F);
        double s = 0;
        for (int t = 0; t < F; ++t) s += xp[(t + tau) % F] * yp[t];
        out[j] = den == 0 ? 0.0 : s / den;
    }
}

// NCC_3D(d_mat, d_centers) + get_pos_idx (kshape.cuh:35-96): per series the min
// over lag slots of 1-ncc for each centroid (pad value 2 when 2m-1 < 512 because
// the 512-thread block pads with 2, :55-60), argmin over centroids with strict <
// (first centroid wins ties, :82-86).
void or_assign(const double* X, const double* C, int64_t n, int m, int k, int F, int clamp2,
               int32_t* labels, double* dist, int32_t* shift, double* margin) {
    FftPlan p, ph;
    p.init(F);
    ph.init(F / 2);
    std::vector<std::vector<cd>> Cs(k);
    std::vector<double> cn(k);
    for (int j = 0; j < k; ++j) {
        spectrum(C + (int64_t)j * m, m, p, Cs[j]);
        cn[j] = norm2(C + (int64_t)j * m, m);
    }
    const int L = 2 * m - 1;
    const bool pad2 = clamp2 && L < 512;
    std::vector<int> slot(L);
    for (int s = 0; s < L; ++s) slot[s] = slot_to_circ(s, m, F);
#pragma omp parallel
    {
        std::vector<cd> Xs, work(F + 2);
        std::vector<double> r(F);
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < n; ++i) {
            const double* x = X + i * (int64_t)m;
            spectrum(x, m, p, Xs);
            double xn = norm2(x, m);
            double best = 1e300, second = 1e300;
            int bj = 0, bshift = 0;
            for (int j = 0; j < k; ++j) {
                circ_corr_half(Xs, Cs[j], p, ph, work, r.data());
                double den = xn * cn[j];
                double dmin = 1e300;
                int last_arg = 0;
                double vmax = -1e300;
                for (int s = 0; s < L; ++s) {
                    double v = den == 0 ? 0.0 : r[slot[s]] / den;
                    double d = 1.0 - v;
                    if (d < dmin) dmin = d;
                    if (v >= vmax) { vmax = v; last_arg = s; }
                }
                if (pad2 && dmin > 2.0) dmin = 2.0;
                if (dmin < best) {
                    second = best;
                    best = dmin;
                    bj = j;
                    // first argmax of NCC(center, series) = reversed slots (SBD.cuh:33-45, :61)
                    bshift = m - 1 - last_arg;
                } else if (dmin < second) {
                    second = dmin;
                }
            }
            labels[i] = bj;
            if (dist) dist[i] = best;
            if (shift) shift[i] = bshift;
            if (margin) margin[i] = second - best;
        }
    }
}

// cyclic Jacobi eigen-solver (stands in for cusolverDnSsyevd, shapeExtract.cuh:434-445).
// Top eigenpair of a symmetric matrix (stands in for the last column of
// cusolverDnSsyevd, shapeExtract.cuh:434-445 and :658-689): Householder
// reduction to tridiagonal form (Golub & Van Loan, Matrix Computations, Alg.
// 8.3.1), the largest eigenvalue of the tridiagonal matrix by Sturm-sequence
// bisection, its eigenvector by inverse iteration (tridiagonal elimination with
// partial pivoting), transformed back by the Householder reflectors.  A zero
// matrix gives the last basis vector, the last column of the identity
// eigenbasis a symmetric eigensolver returns for it.
double or_top_eig_jacobi(const double* Ain, int m, double* vec) {
    std::vector<double> A(Ain, Ain + (size_t)m * m);
    double fro = 0;
    for (double a : A) fro += a * a;
    if (!(fro > 0)) {
        for (int r = 0; r < m; ++r) vec[r] = r == m - 1 ? 1.0 : 0.0;
        return 0.0;
    }
    // reflectors H_k = I - 2 v_k v_k^T on indices k+1..m-1, stored in V (row k)
    std::vector<double> V((size_t)m * m, 0.0), p(m), w(m);
    for (int k = 0; k + 2 < m; ++k) {
        const int n = m - k - 1;
        double xn = 0;
        for (int i = 0; i < n; ++i) xn += A[(size_t)(k + 1 + i) * m + k] * A[(size_t)(k + 1 + i) * m + k];
        xn = std::sqrt(xn);
        if (xn == 0) continue;
        const double x0 = A[(size_t)(k + 1) * m + k];
        const double alpha = x0 > 0 ? -xn : xn;
        double* v = &V[(size_t)k * m];
        for (int i = 0; i < n; ++i) v[i] = A[(size_t)(k + 1 + i) * m + k];
        v[0] -= alpha;
        double vn = 0;
        for (int i = 0; i < n; ++i) vn += v[i] * v[i];
        vn = std::sqrt(vn);
        if (vn == 0) continue;
        for (int i = 0; i < n; ++i) v[i] /= vn;
        // B = A[k+1:, k+1:]:  p = 2 B v, q = p - (v.p) v, B -= v q^T + q v^T
        for (int i = 0; i < n; ++i) {
            const double* Bi = &A[(size_t)(k + 1 + i) * m + k + 1];
            double s2 = 0;
            for (int j = 0; j < n; ++j) s2 += Bi[j] * v[j];
            p[i] = 2 * s2;
        }
        double K = 0;
        for (int i = 0; i < n; ++i) K += v[i] * p[i];
        for (int i = 0; i < n; ++i) w[i] = p[i] - K * v[i];
        for (int i = 0; i < n; ++i) {
            double* Bi = &A[(size_t)(k + 1 + i) * m + k + 1];
            for (int j = 0; j < n; ++j) Bi[j] -= v[i] * w[j] + w[i] * v[j];
        }
        A[(size_t)(k + 1) * m + k] = alpha;
        A[(size_t)k * m + k + 1] = alpha;
        for (int i = 1; i < n; ++i) {
            A[(size_t)(k + 1 + i) * m + k] = 0;
            A[(size_t)k * m + k + 1 + i] = 0;
        }
    }
    std::vector<double> d(m), e(m, 0.0);
    for (int i = 0; i < m; ++i) d[i] = A[(size_t)i * m + i];
    for (int i = 0; i + 1 < m; ++i) e[i] = A[(size_t)(i + 1) * m + i];
    // largest eigenvalue: eigenvalues below x = negative pivots of T - x I
    auto below = [&](double x) {
        int c = 0;
        double q = 1;
        for (int i = 0; i < m; ++i) {
            q = (d[i] - x) - (i > 0 ? e[i - 1] * e[i - 1] / q : 0.0);
            if (q == 0) q = -1e-300;
            if (q < 0) ++c;
        }
        return c;
    };
    double lo = d[0], hi = d[0];
    for (int i = 0; i < m; ++i) {
        const double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(e[i]) : 0.0);
        lo = std::min(lo, d[i] - r);
        hi = std::max(hi, d[i] + r);
    }
    for (int it = 0; it < 200 && hi - lo > 4e-16 * std::max(std::fabs(lo), std::fabs(hi)); ++it) {
        const double mid = 0.5 * (lo + hi);
        if (below(mid) < m) lo = mid;
        else hi = mid;
    }
    const double lam = hi;
    // inverse iteration: (T - lam I) y = x, Gaussian elimination with row swaps (the
    // upper factor gains a second superdiagonal)
    const double tiny = 1e-300 + 2.2e-16 * std::sqrt(fro);
    std::vector<double> x(m, 1.0), u0(m), u1(m), u2(m), l(m);
    std::vector<char> swp(m);
    for (int i = 0; i < m; ++i) {
        u0[i] = d[i] - lam;
        u1[i] = i + 1 < m ? e[i] : 0.0;
        u2[i] = 0.0;
    }
    for (int i = 0; i + 1 < m; ++i) {
        const double sub = e[i];  // row i+1, column i
        if (std::fabs(sub) > std::fabs(u0[i])) {  // swap rows i and i+1
            swp[i] = 1;
            const double r0 = u0[i], r1 = u1[i], r2 = u2[i];
            u0[i] = sub;
            u1[i] = d[i + 1] - lam;
            u2[i] = i + 2 < m ? e[i + 1] : 0.0;
            l[i] = r0 / u0[i];
            u0[i + 1] = r1 - l[i] * u1[i];
            u1[i + 1] = r2 - l[i] * u2[i];
        } else {
            swp[i] = 0;
            if (u0[i] == 0) u0[i] = tiny;
            l[i] = sub / u0[i];
            u0[i + 1] = (d[i + 1] - lam) - l[i] * u1[i];
            u1[i + 1] = (i + 2 < m ? e[i + 1] : 0.0) - l[i] * u2[i];
        }
        u2[i + 1] = 0.0;
    }
    if (u0[m - 1] == 0) u0[m - 1] = tiny;
    for (int it = 0; it < 3; ++it) {
        for (int i = 0; i + 1 < m; ++i) {  // apply the row operations
            if (swp[i]) std::swap(x[i], x[i + 1]);
            x[i + 1] -= l[i] * x[i];
        }
        for (int i = m - 1; i >= 0; --i) {  // back substitution
            double sacc = x[i];
            if (i + 1 < m) sacc -= u1[i] * x[i + 1];
            if (i + 2 < m) sacc -= u2[i] * x[i + 2];
            x[i] = sacc / (u0[i] != 0 ? u0[i] : tiny);
        }
        double nn = 0;
        for (double t : x) nn += t * t;
        nn = std::sqrt(nn);
        for (double& t : x) t /= nn;
    }
    // back to A's basis: vec = H_0 H_1 ... H_{m-3} x
    for (int k = m - 3; k >= 0; --k) {
        const int n = m - k - 1;
        const double* v = &V[(size_t)k * m];
        double dot = 0;
        for (int i = 0; i < n; ++i) dot += v[i] * x[k + 1 + i];
        for (int i = 0; i < n; ++i) x[k + 1 + i] -= 2 * dot * v[i];
    }
    for (int r = 0; r < m; ++r) vec[r] = x[r];
    return lam;
}

void or_random_select(int64_t n, int k, uint32_t seed, int32_t* out) {
    std::mt19937 gen(seed);
    std::uniform_int_distribution<> dis(0, (int)n - 1);
    std::set<int> sel;
    for (int i = 0; i < k; ++i) {
        int num;
        do {
            num = dis(gen);
        } while (sel.find(num) != sel.end());
        sel.insert(num);
        out[i] = num;
    }
}

int or_k_from_labels(const int32_t* labels, int64_t n) {  // test_kshape.cu:24-30
    int mx = labels[0], mn = labels[0];
    for (int64_t i = 1; i < n; ++i) {
        mx = std::max(mx, (int)labels[i]);
        mn = std::min(mn, (int)labels[i]);
    }
    int k = mx;
    if (mn == 0) k += 1;
    else if (mn == -1) k = 2;
    return k;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// shape extraction
// ---------------------------------------------------------------------------
namespace {

// zeroShift (SBD.cuh:14-29): out[t] = x[t - shift], zero fill.
// roll_zeropad (test_timesC.py:55-77) is the same map for |shift| <= m.
void zero_shift(const double* x, double* out, int shift, int m) {
    for (int t = 0; t < m; ++t) out[t] = 0;
    int a = shift > 0 ? shift : -shift;
    if (a >= m) return;
    for (int t = 0; t < m; ++t) {
        int s = t - shift;
        if (s >= 0 && s < m) out[t] = x[s];
    }
}

// first argmax with strict < against an initial -1e10 (SBD.cuh:33-45); numpy argmax
// also returns the first maximum.
int first_argmax(const double* a, int len) {
    double v = -1e10;
    int pos = 0;
    for (int i = 0; i < len; ++i)
        if (v < a[i]) { pos = i; v = a[i]; }
    return pos;
}

void gram_centered(const std::vector<double>& Y, int cnt, int m, std::vector<double>& M) {
    // S = Y^T Y (shapeExtract.cuh:532-537); M = Q S Q with Q = I - 11^T/m (:204-214, :551-570).
    // Upper triangle, rows of Y in blocks that stay in cache, each S row a contiguous
    // axpy per member row.
    std::vector<double> S((size_t)m * m, 0.0);
    const int RB = 128;
    for (int i0 = 0; i0 < cnt; i0 += RB) {
        const int i1 = std::min(cnt, i0 + RB);
#pragma omp parallel for schedule(dynamic, 4)
        for (int a = 0; a < m; ++a) {
            double* Sa = &S[(size_t)a * m];
            for (int i = i0; i < i1; ++i) {
                const double* y = &Y[(size_t)i * m];
                const double ya = y[a];
                for (int b = a; b < m; ++b) Sa[b] += ya * y[b];
            }
        }
    }
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < a; ++b) S[(size_t)a * m + b] = S[(size_t)b * m + a];
    std::vector<double> rs(m, 0.0);
    double tot = 0;
    for (int a = 0; a < m; ++a) {
        double s = 0;
        for (int b = 0; b < m; ++b) s += S[(size_t)a * m + b];
        rs[a] = s;
        tot += s;
    }
    M.resize((size_t)m * m);
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b)
            M[(size_t)a * m + b] = S[(size_t)a * m + b] - rs[a] / m - rs[b] / m + tot / ((double)m * m);
}

void matvec(const std::vector<double>& M, const double* v, double* out, int m) {
    for (int a = 0; a < m; ++a) {
        double s = 0;
        const double* row = &M[(size_t)a * m];
        for (int b = 0; b < m; ++b) s += row[b] * v[b];
        out[a] = s;
    }
}

// get_center (shapeExtract.cuh:217-264): flip when |a-v| >= |a+v|.
void sign_rule(const double* a, double* v, int m) {
    double d1 = 0, d2 = 0;
    for (int t = 0; t < m; ++t) {
        d1 += (a[t] - v[t]) * (a[t] - v[t]);
        d2 += (a[t] + v[t]) * (a[t] + v[t]);
    }
    if (std::sqrt(d1) >= std::sqrt(d2))
        for (int t = 0; t < m; ++t) v[t] = -v[t];
}

void zscore_vec(double* v, int m, int ddof) {
    double mean = 0;
    for (int t = 0; t < m; ++t) mean += v[t];
    mean /= m;
    double ss = 0;
    for (int t = 0; t < m; ++t) ss += (v[t] - mean) * (v[t] - mean);
    double sd = std::sqrt(ss / (m - ddof));
    for (int t = 0; t < m; ++t) v[t] = sd > 0 ? (v[t] - mean) / sd : 0.0;
}

// power iteration of get_class_centers (shapeExtract.cuh:269-283, :577-630):
// v0 = [1, .5, 1, .5, ...], `iters` steps of v <- Mv/|Mv|, lambda = v.(Mv).
double power_iter(const std::vector<double>& M, int m, int iters, double tol, double* v) {
    std::vector<double> w(m);
    for (int t = 0; t < m; ++t) v[t] = (t % 2 == 0) ? 1.0 : 0.5;
    for (int it = 0; it < iters; ++it) {
        matvec(M, v, w.data(), m);
        double nn = 0;
        for (int t = 0; t < m; ++t) nn += w[t] * w[t];
        nn = std::sqrt(nn);
        double diff = 0;
        for (int t = 0; t < m; ++t) {
            double nv = w[t] / nn;
            diff += (nv - v[t]) * (nv - v[t]);
            v[t] = nv;
        }
        if (tol > 0 && std::sqrt(diff) < tol) break;
    }
    matvec(M, v, w.data(), m);
    double lam = 0;
    for (int t = 0; t < m; ++t) lam += v[t] * w[t];
    return lam;
}

}  // namespace

extern "C" int or_align(const double* center, const double* member, int m, int F, double* out) {
    std::vector<double> ncc(2 * m - 1);
    or_ncc(center, member, m, F, ncc.data());
    int shift = first_argmax(ncc.data(), 2 * m - 1) + 1 - m;
    zero_shift(member, out, shift, m);
    return shift;
}

extern "C" void or_shift_row(const double* x, int m, int shift, double* out) { zero_shift(x, out, shift, m); }

extern "C" int or_extract(const double* X, const int32_t* labels, double* C, int64_t n, int m, int k,
                          int mode, int cal_select, int32_t* counts) {
    // stable group-by-cluster (class_count + get_loc2 + exclusive_scan + block_alloc2D,
    // shapeExtract.cuh:21-188, :1062-1122; test_timesC.py:228-243)
    std::vector<std::vector<int64_t>> members(k);
    for (int64_t i = 0; i < n; ++i) members[labels[i]].push_back(i);
    int sum_class = 0;
    for (int j = 0; j < k; ++j) {
        counts[j] = (int32_t)members[j].size();
        if (counts[j]) ++sum_class;
    }
    const int Fal = mode == OR_MODE_COMPAT ? or_fft_size(m, OR_MODE_COMPAT) : or_fft_size(m, OR_MODE_CANONICAL);
    // per non-empty cluster: the centred Gram M and the sign reference a, kept for
    // the eigenvector phase, which runs the clusters in parallel
    std::vector<std::vector<double>> Ms(k), As(k);
    for (int j = 0; j < k; ++j) {
        int cnt = counts[j];
        double* cj = C + (int64_t)j * m;
        if (cnt == 0) {
            if (mode == OR_MODE_PYREF)  // test_timesC.py:139-140
                for (int t = 0; t < m; ++t) cj[t] = 0;
            continue;  // the GPU path keeps the old centroid (shapeExtract.cuh:638-649)
        }
        std::vector<double> Y((size_t)cnt * m);
        for (int i = 0; i < cnt; ++i)
            std::memcpy(&Y[(size_t)i * m], X + members[j][i] * (int64_t)m, sizeof(double) * m);
        // alignment gate
        bool gate;
        if (mode == OR_MODE_COMPAT) {
            // thrust::reduce(..., 0) accumulates with plus<int>: each value truncated (:1131-1135)
            long long s = 0;
            for (int t = 0; t < m; ++t) s += (long long)(int)cj[t];
            gate = std::fabs((double)s) > 1e-16;
        } else if (mode == OR_MODE_CANONICAL) {
            gate = false;
            for (int t = 0; t < m; ++t) gate |= cj[t] != 0;
        } else {
            double s = 0;  // cur_center.sum() != 0 (test_timesC.py:128)
            for (int t = 0; t < m; ++t) s += cj[t];
            gate = s != 0;
        }
        if (gate) {
#pragma omp parallel
            {
            std::vector<double> tmp(m), ncc(2 * m - 1);
#pragma omp for schedule(dynamic, 64)
            for (int i = 0; i < cnt; ++i) {
                double* row = &Y[(size_t)i * m];
                int shift;
                if (mode == OR_MODE_PYREF) {
                    or_ncc(row, cj, m, Fal, ncc.data());  // _ncc_c_2dim(x, center) (:129)
                } else {
                    or_ncc(cj, row, m, Fal, ncc.data());  // NCC_3D(center, members) (SBD.cuh:78)
                }
                shift = first_argmax(ncc.data(), 2 * m - 1) + 1 - m;
                zero_shift(row, tmp.data(), shift, m);
                std::memcpy(row, tmp.data(), sizeof(double) * m);
            }
            }
        }
        std::vector<double> a(m);
        if (mode == OR_MODE_PYREF) {
            std::memcpy(a.data(), &Y[0], sizeof(double) * m);  // a[0] before z-scoring (:163)
            or_znorm(Y.data(), cnt, m, 1);                      // zscore(a, ddof=1) (:142)
        } else {
            or_znorm(Y.data(), cnt, m, 1);                      // z_norm_gpu_x(seg, ddof=1) (:1141)
            std::memcpy(a.data(), &Y[0], sizeof(double) * m);  // val_copy: first member (:192-200)
        }
        gram_centered(Y, cnt, m, Ms[j]);
        As[j] = std::move(a);
    }
    // eigenvector, sign rule and store of every non-empty cluster (independent)
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = 0; j < k; ++j) {
        if (counts[j] == 0) continue;
        double* cj = C + (int64_t)j * m;
        const std::vector<double>& M = Ms[j];
        std::vector<double>& a = As[j];
        std::vector<double> v(m), w(m);
        if (mode == OR_MODE_COMPAT) {
            if (cal_select) {  // get_class_centers_a: syevd top eigenvector (:367-468)
                or_top_eig_jacobi(M.data(), m, v.data());
                sign_rule(a.data(), v.data(), m);
                std::memcpy(cj, v.data(), sizeof(double) * m);
            } else {
                double lam = power_iter(M, m, m, 0.0, v.data());
                if (lam > 0) {
                    sign_rule(a.data(), v.data(), m);
                    std::memcpy(cj, v.data(), sizeof(double) * m);
                } else if (lam <= 0) {  // syevd fallback (:649-692); NaN keeps the old centroid
                    or_top_eig_jacobi(M.data(), m, v.data());
                    sign_rule(a.data(), v.data(), m);
                    std::memcpy(cj, v.data(), sizeof(double) * m);
                }
            }
        } else if (mode == OR_MODE_CANONICAL) {
            double lam = power_iter(M, m, 200 * m + 1000, 1e-13, v.data());
            if (!(lam > 0) && m <= 1024) or_top_eig_jacobi(M.data(), m, v.data());
            sign_rule(a.data(), v.data(), m);
            zscore_vec(v.data(), m, 1);
            std::memcpy(cj, v.data(), sizeof(double) * m);
        } else {
            // _extract_shape (test_timesC.py:136-204)
            int iters = std::min(m, 1000);
            double lam = power_iter(M, m, iters, 0.0, v.data());
            std::vector<double> vr(m), vl(m);
            bool have = lam != 0;
            if (have) {
                sign_rule(a.data(), v.data(), m);
                for (int t = 0; t < m; ++t) vr[t] = lam * v[t];
                matvec(M, v.data(), vl.data(), m);
                int pos = 0;
                for (int t = 0; t < m; ++t)
                    if (vl[t] != 0 && vr[t] != 0) { pos = t; break; }
                if (vl[pos] < 0 && vr[pos] > 0) {
                    lam = -lam;
                    for (int t = 0; t < m; ++t) vr[t] = -vl[t];
                }
            }
            double sumdiff = 0;
            for (int t = 0; t < m; ++t) sumdiff += vr[t] - vl[t];
            sumdiff = std::fabs(sumdiff);
            if (lam <= 0 || sumdiff > m * 0.01) {
                or_top_eig_jacobi(M.data(), m, v.data());
                sign_rule(a.data(), v.data(), m);
            }
            zscore_vec(v.data(), m, 1);
            std::memcpy(cj, v.data(), sizeof(double) * m);
        }
    }
    return sum_class;
}

// ---------------------------------------------------------------------------
// the loop
// ---------------------------------------------------------------------------
namespace {

struct Loop {
    const or_job* job;
    std::vector<double> X;   // normalised data
    int64_t n;
    int m, k, F;
    double min_margin = 1e300;
    std::vector<int32_t> labels;
    std::vector<double> C;
    std::vector<double> dist, margin;
    std::vector<int32_t> counts;
    int iterations = 0;
    int sum_class = 0;
    double inertia = 0;

    void assign() {
        or_assign(X.data(), C.data(), n, m, k, F, job->mode == OR_MODE_COMPAT, labels.data(), dist.data(),
                  nullptr, margin.data());
        double s = 0;
        for (int64_t i = 0; i < n; ++i) {
            s += dist[i];
            if (k > 1) min_margin = std::min(min_margin, margin[i]);
        }
        inertia = s / (double)n;
    }

    // k_shape (kshape.cuh:197-324): extract -> assign -> converge
    void k_shape(int cal_select, int iter_cap, int sum_class_in) {
        labels.assign(job->init_labels, job->init_labels + n);
        C.assign((size_t)k * m, 0.0);
        std::vector<int32_t> old = labels;
        double old_inertia = 1e10;
        int countIter = 0;
        sum_class = sum_class_in;
        iterations = iter_cap;
        for (int i = 0; i < iter_cap; ++i) {
            int sc = or_extract(X.data(), labels.data(), C.data(), n, m, k, job->mode, cal_select, counts.data());
            if (!cal_select) sum_class = sc;  // get_class_centers_a leaves sum_class alone
            if (sum_class == 1 || sum_class <= k / 2) { iterations = i + 1; break; }
            assign();
            bool flag = old == labels;
            if (flag || countIter > 20) { iterations = i + 1; break; }
            if (inertia < old_inertia || std::fabs(old_inertia - inertia) < 1e-6) {
                old = labels;
                old_inertia = inertia;
                countIter = 0;
            } else {
                ++countIter;
            }
        }
    }

    // k_shape_tsl (kshape.cuh:332-474): assign -> converge -> extract
    void k_shape_tsl(int iter_cap) {
        labels.assign(job->init_labels, job->init_labels + n);
        std::vector<int32_t> old = labels;
        std::vector<int32_t> pick(k);
        or_random_select(n, k, job->seed, pick.data());
        C.assign((size_t)k * m, 0.0);
        for (int j = 0; j < k; ++j)  // raw (un-normalised) rows: center_select (:178-191)
            for (int t = 0; t < m; ++t) C[(size_t)j * m + t] = (double)job->data[(int64_t)pick[j] * m + t];
        double old_inertia = 1e10;
        int countIter = 0;
        iterations = iter_cap;
        for (int i = 0; i < iter_cap; ++i) {
            assign();
            bool flag = old == labels;
            if (flag || countIter > 20) { iterations = i + 1; break; }
            if (inertia < old_inertia || std::fabs(old_inertia - inertia) < 1e-6) {
                old = labels;
                old_inertia = inertia;
                countIter = 0;
            } else {
                ++countIter;
            }
            sum_class = or_extract(X.data(), labels.data(), C.data(), n, m, k, job->mode, 0, counts.data());
            if (sum_class == 1 || sum_class <= k / 2) { iterations = i + 1; break; }
        }
    }

    // _kshape (test_timesC.py:213-265)
    void py_kshape(int iter_cap) {
        labels.assign(job->init_labels, job->init_labels + n);
        C.assign((size_t)k * m, 0.0);
        iterations = iter_cap;
        for (int i = 0; i < iter_cap; ++i) {
            std::vector<int32_t> old = labels;
            sum_class = or_extract(X.data(), labels.data(), C.data(), n, m, k, OR_MODE_PYREF, 0, counts.data());
            assign();
            if (old == labels) { iterations = i + 1; break; }
        }
    }
};

}  // namespace

extern "C" int or_kshape(const or_job* job, or_result* res) {
    if (!job || !res || job->n <= 0 || job->m <= 1 || job->k <= 0) return 1;
    if (job->init_chose == 1 && job->k > job->n) return 1;
    Loop L;
    L.job = job;
    L.n = job->n;
    L.m = job->m;
    L.k = job->k;
    L.F = or_fft_size(job->m, job->mode == OR_MODE_COMPAT ? OR_MODE_COMPAT : OR_MODE_CANONICAL);
    L.X.resize((size_t)L.n * L.m);
    for (size_t i = 0; i < L.X.size(); ++i) L.X[i] = (double)job->data[i];
    or_znorm(L.X.data(), L.n, L.m, job->mode == OR_MODE_PYREF ? 0 : 1);  // test_kshape.cu:37 / test_timesC.py:214
    L.dist.resize(L.n);
    L.margin.resize(L.n);
    L.counts.resize(L.k);
    res->restarted = 0;
    if (job->mode == OR_MODE_PYREF) {
        L.py_kshape(job->max_iter);
    } else {
        if (job->init_chose == 1) L.k_shape_tsl(job->max_iter);
        else L.k_shape(0, job->max_iter, job->k);
        // test_kshape.cu:54-59 / :112-117
        if (job->restart && (L.sum_class == 1 || L.sum_class < job->k / 2)) {
            res->restarted = 1;
            L.k_shape(1, job->max_iter, job->k);
        }
    }
    std::memcpy(res->labels, L.labels.data(), sizeof(int32_t) * L.n);
    std::memcpy(res->centroids, L.C.data(), sizeof(double) * (size_t)L.k * L.m);
    res->iterations = L.iterations;
    res->sum_class = L.sum_class;
    res->inertia = L.inertia;
    res->min_margin = L.min_margin;
    return 0;
}

extern "C" double or_ari(const int32_t* a, const int32_t* b, int64_t n) {
    std::map<std::pair<int, int>, int64_t> nij;
    std::map<int, int64_t> ai, bj;
    for (int64_t i = 0; i < n; ++i) {
        nij[{a[i], b[i]}]++;
        ai[a[i]]++;
        bj[b[i]]++;
    }
    auto c2 = [](double x) { return x * (x - 1) / 2; };
    double sij = 0, sa = 0, sb = 0;
    for (auto& kv : nij) sij += c2((double)kv.second);
    for (auto& kv : ai) sa += c2((double)kv.second);
    for (auto& kv : bj) sb += c2((double)kv.second);
    double tot = c2((double)n);
    double expected = sa * sb / tot;
    double mx = 0.5 * (sa + sb);
    if (mx == expected) return 1.0;
    return (sij - expected) / (mx - expected);
}

// The engine's synthetic workloads (gen_core.h), so that the CPU baseline runs on
// the same series without loading the engine's library.
extern "C" int or_generate(int64_t n, int m, int classes, double noise, double dirichlet, uint64_t seed,
                           float* data, int32_t* labels) {
    const tcgen::Params p{n, m, classes, noise, dirichlet, seed};
    return tcgen::generate(&p, data, labels) ? 0 : 1;
}
