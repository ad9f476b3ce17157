// CPU emulation of one team running the fused SBD phases of sbd_core.cuh for
// every supported transform size; compares the normalised correlation and the
// lag bookkeeping against direct FP64 sums.  Prints one line per N and exits
// non-zero on a mismatch.  Built and run by tests/test_fft_plan.py (no GPU).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "sbd_core.cuh"

using namespace tcfft;

template <int N, int PS, bool INV>
struct Runner {
    // runs passes PS..NPASS-1; the last one stores when STORE_LAST
    template <class OutFn>
    static void run(std::vector<float2>& buf, const std::vector<float2>& twN, bool store_last, OutFn&& out) {
        typedef Core<N> C;
        typedef typename C::template Pass<PS> PassT;
        const int T = C::T;
        std::vector<PassT> st(T);
        for (int t = 0; t < T; ++t) st[t].load(buf.data(), t);
        for (int t = 0; t < T; ++t) st[t].template compute<INV>(t, twN.data());
        constexpr bool last = PS + 1 >= Plan<N>::NPASS;
        if (!last || store_last) {
            for (int t = 0; t < T; ++t) st[t].store(buf.data(), t);
        }
        if constexpr (!last) {
            Runner<N, PS + 1, INV>::run(buf, twN, store_last, out);
        } else {
            if (!store_last)
                for (int t = 0; t < T; ++t) st[t].each_output(t, out);
        }
    }
};

template <int N>
int check(std::mt19937& g) {
    typedef Core<N> C;
    const int T = C::T, R0 = C::R0, F = 2 * N;
    std::vector<float2> twN(N), twF(N);
    for (int e = 0; e < N; ++e) {
        double a = -2.0 * M_PI * e / N, b = -2.0 * M_PI * e / F;
        twN[e] = mk((float)cos(a), (float)sin(a));
        twF[e] = mk((float)cos(b), (float)sin(b));
    }
    int worst = 0;
    for (int trial = 0; trial < 3; ++trial) {
        // m: the largest compat length for this F, a canonical length, a short one
        int ms[3] = {F <= 4 ? 3 : F / 2 + F / 4, N, N / 2 + 1};
        int m = ms[trial];
        if (m < 2) m = 2;
        if (m > F) m = F;
        std::normal_distribution<double> nd;
        std::vector<float> x(m), c(m);
        for (int i = 0; i < m; ++i) { x[i] = (float)nd(g); c[i] = (float)nd(g); }
        struct V { float2 v[2][R0]; };
        struct X { float2 xh[2][R0]; float xhN = 0; };
        std::vector<float2> buf(BufSize<N>::value);
        auto forward = [&](const std::vector<float>& s, std::vector<X>& xs, double extra) {
            std::vector<V> v(T);
            double ss = 0;
            for (int t = 0; t < T; ++t) ss += C::fwd_load(s.data(), m, t, v[t].v);
            for (int t = 0; t < T; ++t) C::template pass0_store<false>(v[t].v, t, buf.data());
            Runner<N, 1, false>::run(buf, twN, true, [](int, float2) {});
            float sc = (float)(1.0 / (sqrt(ss) * extra));
            xs.resize(T);
            for (int t = 0; t < T; ++t) C::post(buf.data(), t, twF.data(), sc, xs[t].xh, xs[t].xhN);
        };
        std::vector<X> xs, cs;
        forward(x, xs, 1.0);
        forward(c, cs, 2.0 * N);
        // assemble the centroid spectrum S[0..N]
        std::vector<float2> S(N + 1);
        for (int t = 0; t < T; ++t)
            for (int b = 0; b < 2; ++b)
                for (int r = 0; r < R0; ++r) S[C::j_of(t, b) + r * C::NB0] = cs[t].xh[b][r];
        S[N] = mk(cs[0].xhN, 0.f);
        std::vector<V> v(T);
        auto sp = [&](int f) { return S[f]; };
        for (int t = 0; t < T; ++t) C::product(xs[t].xh, xs[t].xhN, sp, t, twF.data(), v[t].v);
        for (int t = 0; t < T; ++t) C::template pass0_store<true>(v[t].v, t, buf.data());
        std::vector<double> got(F, 1e300);
        LagMax lm;
        lm.init();
        Runner<N, 1, true>::run(buf, twN, false, [&](int o, float2 val) {
            got[2 * o] = val.x;
            got[2 * o + 1] = val.y;
            lag_take(lm, 2 * o, val.x, m, F);
            lag_take(lm, 2 * o + 1, val.y, m, F);
        });
        // direct reference
        double nx = 0, nc = 0;
        for (int i = 0; i < m; ++i) { nx += (double)x[i] * x[i]; nc += (double)c[i] * c[i]; }
        double den = sqrt(nx) * sqrt(nc), maxerr = 0, bestv = -1e300;
        int bestu = 0;
        for (int tt = 0; tt < F; ++tt) {
            double s = 0;
            for (int i = 0; i < m; ++i) {
                int a = (i + tt) % F;
                if (a < m) s += (double)x[a] * c[i];
            }
            s /= den;
            if (got[tt] > 1e299) { printf("N=%d: output %d never written\n", N, tt); return 1; }
            maxerr = std::max(maxerr, fabs(s - got[tt]));
            bool valid = tt <= m - 1 || tt >= F - m + 1;
            int u = tt <= m - 1 ? tt : tt - F;
            if (valid && (s > bestv + 1e-5 || (fabs(s - bestv) <= 1e-5 && u > bestu))) { bestv = s; bestu = u; }
        }
        double tol = 2e-6 * log2((double)F) + 1e-6;
        bool ok = maxerr < tol && fabs(bestv - lm.val) < 1e-5;
        if (!ok || (trial == 0)) printf("N=%d T=%d R0=%d passes=%d m=%d maxerr=%.3g best=%.6f/%.6f u=%d/%d %s\n", N, T,
                                        R0, Plan<N>::NPASS, m, maxerr, bestv, lm.val, bestu, lm.u, ok ? "ok" : "FAIL");
        if (!ok) worst = 1;
    }
    return worst;
}

int main() {
    std::mt19937 g(12345);
    int bad = 0;
    bad |= check<4>(g);
    bad |= check<8>(g);
    bad |= check<16>(g);
    bad |= check<32>(g);
    bad |= check<64>(g);
    bad |= check<128>(g);
    bad |= check<256>(g);
    bad |= check<512>(g);
    bad |= check<1024>(g);
    bad |= check<2048>(g);
    bad |= check<4096>(g);
    bad |= check<8192>(g);
    printf(bad ? "FAIL\n" : "ALL OK\n");
    return bad;
}
