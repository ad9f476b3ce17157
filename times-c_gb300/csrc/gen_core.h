// Synthetic k-Shape workloads (the stand-in for the UCR/UEA archives, which are
// not available): each class prototype is a sum of 3-6 sinusoids (1-8 cycles
// over the series, N(0,1) amplitudes, U(0, 2pi) phases) plus one Gaussian bump
// (amplitude +-U(1,3), centre U(0,m), width U(m/40, m/10)).  A series is its
// class prototype circularly shifted by an integer U[-m/10, m/10], scaled by
// U(0.5, 2), offset by N(0, 5), plus i.i.d. N(0, (noise * std(prototype))^2).
// Class sizes are equal (labels i mod classes) or drawn from a Dirichlet(alpha)
// mixture.  Every series has its own counter-based stream, so the output does
// not depend on the number of threads.
//
// Header-only so that the engine's tc_generate and the oracle's CPU baseline
// (which must not load the engine's library) make the same series bit for bit.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace tcgen {

inline uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed, uint64_t stream) {
        uint64_t x = seed * 0x2545F4914F6CDD1Dull ^ (stream + 0x632BE59BD9B4E019ull);
        for (auto& v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {  // xoshiro256**
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uni(double a, double b) { return a + (b - a) * uni(); }
    double normal() {
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }
    double gamma(double a) {  // Marsaglia-Tsang, a >= 1
        double d = a - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
        for (;;) {
            double x = normal(), v = 1 + c * x;
            if (v <= 0) continue;
            v = v * v * v;
            double u = uni();
            if (u < 1 - 0.0331 * x * x * x * x) return d * v;
            if (std::log(u) < 0.5 * x * x + d * (1 - v + std::log(v))) return d * v;
        }
    }
};

struct Params {
    int64_t n;
    int m;
    int classes;
    double noise;
    double dirichlet;
    uint64_t seed;
};

// Fills data (n*m) and labels (n, may be null); false for invalid parameters.
inline bool generate(const Params* sp, float* data, int32_t* labels) {
    if (!sp || !data || sp->n < 0 || sp->m < 2 || sp->classes < 1) return false;
    const int64_t n = sp->n;
    const int m = sp->m, K = sp->classes;
    // prototypes
    std::vector<double> proto((size_t)K * m), pstd(K);
    for (int c = 0; c < K; ++c) {
        Rng r(sp->seed, 0xC1A55000ull + (uint64_t)c);
        double* p = &proto[(size_t)c * m];
        std::fill(p, p + m, 0.0);
        int ns = 3 + (int)(r.next() % 4);
        for (int q = 0; q < ns; ++q) {
            double cyc = r.uni(1.0, 8.0), amp = r.normal(), ph = r.uni(0.0, 2.0 * M_PI);
            for (int t = 0; t < m; ++t) p[t] += amp * std::sin(2.0 * M_PI * cyc * t / m + ph);
        }
        double bamp = r.uni(1.0, 3.0) * ((r.next() & 1) ? 1.0 : -1.0);
        double bc = r.uni(0.0, (double)m), bw = r.uni(m / 40.0, m / 10.0);
        if (bw < 0.5) bw = 0.5;
        for (int t = 0; t < m; ++t) p[t] += bamp * std::exp(-0.5 * ((t - bc) / bw) * ((t - bc) / bw));
        double mu = 0, ss = 0;
        for (int t = 0; t < m; ++t) mu += p[t];
        mu /= m;
        for (int t = 0; t < m; ++t) ss += (p[t] - mu) * (p[t] - mu);
        pstd[c] = std::sqrt(ss / m);
    }
    // class weights
    std::vector<double> cdf(K);
    if (sp->dirichlet > 0) {
        Rng r(sp->seed, 0xD1A1C4E7ull);
        double a = std::max(1.0, sp->dirichlet), tot = 0;
        for (int c = 0; c < K; ++c) tot += (cdf[c] = r.gamma(a));
        double acc = 0;
        for (int c = 0; c < K; ++c) cdf[c] = (acc += cdf[c] / tot);
    }
    const int maxshift = m / 10;
    auto work = [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            Rng r(sp->seed, 0x5E41E5000000ull + (uint64_t)i);
            int c;
            if (sp->dirichlet > 0) {
                double u = r.uni();
                c = 0;
                while (c < K - 1 && u >= cdf[c]) ++c;
            } else {
                c = (int)(i % K);
            }
            int sh = (int)(r.next() % (uint64_t)(2 * maxshift + 1)) - maxshift;
            double sc = r.uni(0.5, 2.0), off = 5.0 * r.normal(), sig = sp->noise * pstd[c];
            const double* p = &proto[(size_t)c * m];
            float* x = data + (size_t)i * m;
            for (int t = 0; t < m; ++t) {
                int src = ((t - sh) % m + m) % m;
                x[t] = (float)(sc * p[src] + off + sig * r.normal());
            }
            if (labels) labels[i] = c;
        }
    };
    unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < 2048) nth = 1;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t) th.emplace_back(work, n * t / nth, n * (t + 1) / nth);
    for (auto& t : th) t.join();
    return true;
}

}  // namespace tcgen
