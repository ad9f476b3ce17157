// Radix-2/4/8 DFT butterflies and the Stockham pass plan used by the fused SBD
// kernels.  Host-compilable (TC_HD) so the same plan can be checked on a CPU.
//
// A length-F real correlation is computed with an N = F/2 point complex FFT:
// z[n] = x[2n] + i x[2n+1].  The plan for N:
//   pass 0 has radix R0 and N/R0 = 2T butterflies, T = threads per transform
//   ("team"); thread t owns butterflies t and (2T - t) mod 2T (thread 0 owns 0 and
//   T), so it holds every input bin f together with its mirror N - f.  That lets
//   the spectral product and the real-to-complex pre-processing run in registers.
//   later passes use radix <= min(8, 2*R0); the last one may be smaller.
#pragma once

#if defined(__CUDACC__)
#define TC_HD __host__ __device__ __forceinline__
#else
#include <vector_types.h>
#define TC_HD inline
#endif

namespace tcfft {

TC_HD float2 mk(float a, float b) { float2 r; r.x = a; r.y = b; return r; }
TC_HD float2 add(float2 a, float2 b) { return mk(a.x + b.x, a.y + b.y); }
TC_HD float2 sub(float2 a, float2 b) { return mk(a.x - b.x, a.y - b.y); }
TC_HD float2 mul(float2 a, float2 b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
TC_HD float2 mulc(float2 a, float2 b) { return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
TC_HD float2 conj(float2 a) { return mk(a.x, -a.y); }
TC_HD float2 scale(float2 a, float s) { return mk(a.x * s, a.y * s); }
TC_HD float2 mul_i(float2 a) { return mk(-a.y, a.x); }   // i * a
TC_HD float2 mul_ni(float2 a) { return mk(a.y, -a.x); }  // -i * a

// In-register DFT of size R. INV: e^{+2 pi i rq/R} kernel, else e^{-2 pi i rq/R}.
template <int R, bool INV>
TC_HD void dft(float2* v);

template <>
TC_HD void dft<2, false>(float2* v) { float2 t = v[0]; v[0] = add(t, v[1]); v[1] = sub(t, v[1]); }
template <>
TC_HD void dft<2, true>(float2* v) { float2 t = v[0]; v[0] = add(t, v[1]); v[1] = sub(t, v[1]); }

template <bool INV>
TC_HD void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
    float2 s0 = add(a0, a2), d0 = sub(a0, a2), s1 = add(a1, a3), d1 = sub(a1, a3);
    a0 = add(s0, s1);
    a2 = sub(s0, s1);
    if (INV) {
        a1 = add(d0, mul_i(d1));
        a3 = sub(d0, mul_i(d1));
    } else {
        a1 = add(d0, mul_ni(d1));
        a3 = sub(d0, mul_ni(d1));
    }
}
template <>
TC_HD void dft<4, false>(float2* v) { dft4<false>(v[0], v[1], v[2], v[3]); }
template <>
TC_HD void dft<4, true>(float2* v) { dft4<true>(v[0], v[1], v[2], v[3]); }

template <bool INV>
TC_HD void dft8(float2* v) {
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    const float c = 0.70710678118654752440f;
    // W8^q (forward: e^{-i pi q/4}); inverse uses the conjugates
    o1 = INV ? mk(c * (o1.x - o1.y), c * (o1.x + o1.y)) : mk(c * (o1.x + o1.y), c * (o1.y - o1.x));
    o2 = INV ? mul_i(o2) : mul_ni(o2);
    o3 = INV ? mk(-c * (o3.x + o3.y), c * (o3.x - o3.y)) : mk(c * (o3.y - o3.x), -c * (o3.x + o3.y));
    v[0] = add(e0, o0); v[4] = sub(e0, o0);
    v[1] = add(e1, o1); v[5] = sub(e1, o1);
    v[2] = add(e2, o2); v[6] = sub(e2, o2);
    v[3] = add(e3, o3); v[7] = sub(e3, o3);
}
template <>
TC_HD void dft<8, false>(float2* v) { dft8<false>(v); }
template <>
TC_HD void dft<8, true>(float2* v) { dft8<true>(v); }

// Shared-memory padding: one extra slot every 8 keeps the stride-R stores of the
// early passes free of bank conflicts.
TC_HD int pad(int i) { return i + (i >> 3); }
template <int N>
struct BufSize { static constexpr int value = N + N / 8; };

constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

// Pass plan for an N-point transform.
template <int N>
struct Plan {
    static constexpr int R0 = N >= 512 ? 8 : (N == 256 ? 4 : 2);
    static constexpr int T = N >= 1024 ? N / 16 : N / (2 * R0);  // threads per transform
    static constexpr int NB0 = N / R0;                           // = 2T
    static constexpr int RMAX = (2 * R0 < 8) ? 2 * R0 : 8;
    static constexpr int REST_LG = ilog2(N / R0);
    static constexpr int LG_MAX = ilog2(RMAX);
    static constexpr int NFULL = REST_LG / LG_MAX;               // passes of radix RMAX
    static constexpr int TAIL = 1 << (REST_LG % LG_MAX);         // last radix if > 1
    static constexpr int NPASS = 1 + NFULL + (TAIL > 1 ? 1 : 0);
    // radix of pass p (p >= 1)
    static constexpr int radix(int p) { return p <= NFULL ? RMAX : TAIL; }
    // product of the radices before pass p
    static constexpr int ns(int p) {
        return p == 0 ? 1 : (p == 1 ? R0 : ns(p - 1) * radix(p - 1));
    }
};

// Stockham index maps (butterfly j of a radix-R pass over N points, Ns = product
// of the earlier radices): inputs j + r*N/R, outputs (j - j%Ns)*R + j%Ns + q*Ns,
// twiddle of input r: W_N^(r * (j%Ns) * N/(Ns*R)).
TC_HD int in_index(int j, int r, int N, int R) { return j + r * (N / R); }
TC_HD int out_index(int j, int q, int Ns, int R) {
    int k = j & (Ns - 1);
    return (j - k) * R + k + q * Ns;
}
TC_HD int tw_step(int j, int Ns, int N, int R) { return (j & (Ns - 1)) * (N / (Ns * R)); }

// Apply twiddles w^r (r = 1..R-1) given w = W_N^e from the table (conjugated for
// the inverse): powers by repeated products (at most 3 roundings deep).
template <int R>
TC_HD void twiddle(float2* v, float2 w) {
    if (R == 2) {
        v[1] = mul(v[1], w);
    } else if (R == 4) {
        float2 w2 = mul(w, w), w3 = mul(w2, w);
        v[1] = mul(v[1], w); v[2] = mul(v[2], w2); v[3] = mul(v[3], w3);
    } else {
        float2 w2 = mul(w, w), w3 = mul(w2, w), w4 = mul(w2, w2);
        float2 w5 = mul(w4, w), w6 = mul(w4, w2), w7 = mul(w4, w3);
        v[1] = mul(v[1], w); v[2] = mul(v[2], w2); v[3] = mul(v[3], w3); v[4] = mul(v[4], w4);
        v[5] = mul(v[5], w5); v[6] = mul(v[6], w6); v[7] = mul(v[7], w7);
    }
}

}  // namespace tcfft
