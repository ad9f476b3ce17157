// Per-thread phases of the fused SBD correlation (one "team" of Plan<N>::T
// threads per transform; the caller synchronises the team between phases).
// The same functions run in the CUDA kernels and in a CPU emulation of a team.
//
// Scaling: the series spectrum is X/|x|, the centroid spectrum is C/(2N|c|), so
// the inverse transform's outputs are directly the normalised cross-correlation
// ncc(t) = sum_s x[(s+t) mod F] c[s] / (|x||c|)  (ncc.cuh:124-145, :358).
#pragma once
#include "fft.cuh"

namespace tcfft {

// Read-only cached load on the device, plain load on the host.
template <class V>
TC_HD V ldg(const V* p) {
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}
#define TC_LDG(p) ::tcfft::ldg(p)

template <int N>
struct Core {
    typedef Plan<N> P;
    static constexpr int R0 = P::R0, T = P::T, NB0 = P::NB0;

    TC_HD static int j_of(int tid, int b) { return b == 0 ? tid : (tid == 0 ? NB0 / 2 : NB0 - tid); }

    // forward: pass-0 inputs z[f] = x[2f] + i x[2f+1] (zero beyond m); also the
    // thread's partial sum of squares.
    TC_HD static float fwd_load(const float* x, int m, int tid, float2 (&v)[2][R0]) {
        float ss = 0.f;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int j = j_of(tid, b);
#pragma unroll
            for (int r = 0; r < R0; ++r) {
                int f = j + r * NB0;
                int a = 2 * f;
                float re = a < m ? x[a] : 0.f;
                float im = a + 1 < m ? x[a + 1] : 0.f;
                ss += re * re + im * im;
                v[b][r] = mk(re, im);
            }
        }
        return ss;
    }

    // pass 0 (Ns = 1, no twiddles): DFT and store.
    template <bool INV>
    TC_HD static void pass0_store(float2 (&v)[2][R0], int tid, float2* buf) {
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int j = j_of(tid, b);
            dft<R0, INV>(v[b]);
#pragma unroll
            for (int q = 0; q < R0; ++q) buf[pad(j * R0 + q)] = v[b][q];
        }
    }

    // generic pass p >= 1
    template <int PS>
    struct Pass {
        static constexpr int R = P::radix(PS);
        static constexpr int NS = P::ns(PS);
        static constexpr int NB = N / R;
        static constexpr int PER = (NB + T - 1) / T;
        float2 v[PER][R];

        TC_HD void load(const float2* buf, int tid) {
#pragma unroll
            for (int b = 0; b < PER; ++b) {
                int j = tid + b * T;
                if (j < NB) {
#pragma unroll
                    for (int r = 0; r < R; ++r) v[b][r] = buf[pad(in_index(j, r, N, R))];
                }
            }
        }
        template <bool INV>
        TC_HD void compute(int tid, const float2* twN) {
#pragma unroll
            for (int b = 0; b < PER; ++b) {
                int j = tid + b * T;
                if (j < NB) {
                    float2 w = TC_LDG(twN + tw_step(j, NS, N, R));
                    if (INV) w = conj(w);
                    twiddle<R>(v[b], w);
                    dft<R, INV>(v[b]);
                }
            }
        }
        TC_HD void store(float2* buf, int tid) const {
#pragma unroll
            for (int b = 0; b < PER; ++b) {
                int j = tid + b * T;
                if (j < NB) {
#pragma unroll
                    for (int q = 0; q < R; ++q) buf[pad(out_index(j, q, NS, R))] = v[b][q];
                }
            }
        }
        // outputs of this (last) pass: complex index o, value
        template <class F>
        TC_HD void each_output(int tid, F&& fn) const {
#pragma unroll
            for (int b = 0; b < PER; ++b) {
                int j = tid + b * T;
                if (j < NB) {
#pragma unroll
                    for (int q = 0; q < R; ++q) fn(out_index(j, q, NS, R), v[b][q]);
                }
            }
        }
        // outputs with their slot e = b*R + q in this thread (constant after unrolling)
        template <class F>
        TC_HD void each_output_slot(int tid, F&& fn) const {
#pragma unroll
            for (int b = 0; b < PER; ++b) {
                if (tid + b * T < NB) {
#pragma unroll
                    for (int q = 0; q < R; ++q) fn(b * R + q, v[b][q]);
                }
            }
        }
        // bit 2e / 2e+1: the two real outputs of slot e are valid lags (t <= m-1 or
        // t >= F-m+1) of an existing butterfly.  Every plan has PER*R <= 16.
        TC_HD static unsigned valid_mask(int tid, int m, int F) {
            unsigned mask = 0;
#pragma unroll
            for (int b = 0; b < PER; ++b) {
                const int j = tid + b * T;
#pragma unroll
                for (int q = 0; q < R; ++q) {
                    const int t = 2 * out_index(j, q, NS, R);
                    const bool ok = j < NB;
                    const unsigned b0 = (ok && (t <= m - 1 || t >= F - m + 1)) ? 1u : 0u;
                    const unsigned b1 = (ok && (t + 1 <= m - 1 || t + 1 >= F - m + 1)) ? 2u : 0u;
                    mask |= (b0 | b1) << (2 * (b * R + q));
                }
            }
            return mask;
        }
    };

    // Real-to-complex post-processing of the forward transform (natural-order Z in
    // buf): the thread's spectrum bins X[f]*s for its pass-0 f set, plus X[N]*s on
    // thread 0.  X[f] = (Z[f] + conj Z[N-f])/2 - i W_F^f (Z[f] - conj Z[N-f])/2.
    TC_HD static void post(const float2* buf, int tid, const float2* twF, float s, float2 (&xh)[2][R0],
                           float& xhN) {
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int j = j_of(tid, b);
#pragma unroll
            for (int r = 0; r < R0; ++r) {
                int f = j + r * NB0;
                int fm = (N - f) & (N - 1);
                float2 zf = buf[pad(f)], zm = conj(buf[pad(fm)]);
                float2 e = scale(add(zf, zm), 0.5f);
                float2 o = mul_ni(scale(sub(zf, zm), 0.5f));
                float2 w = TC_LDG(twF + f);
                xh[b][r] = scale(add(e, mul(w, o)), s);
                if (f == 0) xhN = (e.x - o.x) * s;  // X[N] is real: Re Z0 - Im Z0
            }
        }
    }

    // Spectral product with a centroid spectrum S (N+1 bins) and the
    // complex-to-real pre-processing of the inverse, straight into pass-0 inputs.
    // For a mirror pair (f, N-f): P = X[f] conj S[f], Pm = X[N-f] conj S[N-f],
    // E = P + conj Pm, D = P - conj Pm, O = D conj W_F^f,
    // Z[f] = E + iO, Z[N-f] = conj E + i conj O.
    TC_HD static void pair(float2 xa, float2 sa, float2 xb, float2 sb, float2 wa, float2& za, float2& zb) {
        float2 p = mulc(xa, sa), pm = mulc(xb, sb);
        float2 e = add(p, conj(pm)), d = sub(p, conj(pm));
        float2 o = mulc(d, wa);
        za = add(e, mul_i(o));
        zb = add(conj(e), mul_i(conj(o)));
    }

    template <class SpecPtr>
    TC_HD static void product(const float2 (&xh)[2][R0], float xhN, SpecPtr S, int tid, const float2* twF,
                              float2 (&v)[2][R0]) {
        if (tid != 0) {
            const int j0 = tid, j1 = NB0 - tid;
#pragma unroll
            for (int r = 0; r < R0; ++r) {
                int f = j0 + r * NB0, fm = j1 + (R0 - 1 - r) * NB0;
                pair(xh[0][r], S(f), xh[1][R0 - 1 - r], S(fm), TC_LDG(twF + f), v[0][r], v[1][R0 - 1 - r]);
            }
        } else {
            // b = 0, r = 0 pairs with bin N
            {
                float2 sN = S(N);
                float2 dummy;
                pair(xh[0][0], S(0), mk(xhN, 0.f), sN, mk(1.f, 0.f), v[0][0], dummy);
            }
#pragma unroll
            for (int r = 1; r <= R0 / 2; ++r) {
                int f = r * NB0, fm = (R0 - r) * NB0;
                float2 za, zb;
                pair(xh[0][r], S(f), xh[0][R0 - r], S(fm), TC_LDG(twF + f), za, zb);
                v[0][r] = za;
                if (R0 - r != r) v[0][R0 - r] = zb;
            }
            const int j1 = NB0 / 2;
#pragma unroll
            for (int r = 0; r < R0 / 2; ++r) {
                int f = j1 + r * NB0, fm = j1 + (R0 - 1 - r) * NB0;
                pair(xh[1][r], S(f), xh[1][R0 - 1 - r], S(fm), TC_LDG(twF + f), v[1][r], v[1][R0 - 1 - r]);
            }
        }
    }
};

// Lag bookkeeping of the max: circular index t in [0, F) is a valid lag when it is
// one of the 2m-1 slots of copy_result2D (ncc.cuh:230-245): t <= m-1 or
// t >= F-m+1.  Its lag u (largest representative <= m-1) is t or t-F.  Among equal
// values the larger u wins: that is the first maximum sbd3D's get_maxpos finds in
// NCC(center, member) (SBD.cuh:33-45), whose shift is -u (SBD.cuh:61).
struct LagMax {
    float val;
    int u;
    TC_HD void init() { val = -3.0e38f; u = -2147483647; }
    TC_HD void take(float v, int uu) {
        if (v > val || (v == val && uu > u)) { val = v; u = uu; }
    }
};

TC_HD void lag_take(LagMax& lm, int t, float v, int m, int F) {
    if (t <= m - 1) lm.take(v, t);
    else if (t >= F - m + 1) lm.take(v, t - F);
}

}  // namespace tcfft
