// Text input/output of the reference's CLI path (readfile.cuh:13-129) and the
// random centroid-row draw (kshape.cuh:159-176).
//
// Parsing follows readFile / read_unlabeled_File: one series per line; a line
// that contains a comma is split on commas (getline(ss, s, ',')), so a trailing
// comma adds no value and an empty field between two commas reads as 0 (atof);
// other lines are split on runs of spaces/tabs.  With a label column the first
// field is read like std::stoi (leading integer, "1.0" -> 1).  Differences, all
// on inputs where the reference reads garbage: '\r' line ends are stripped,
// blank lines are skipped, and ragged rows are an error instead of UB.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "timesc.h"

namespace {

struct Line {
    const char* b;
    const char* e;
};

inline bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Splits one line into fields. Returns false on a malformed label.
bool parse_line(const Line& L, bool labeled, std::vector<float>& vals, int32_t& label, std::string& why) {
    vals.clear();
    const char* p = L.b;
    const char* e = L.e;
    while (e > p && is_ws(e[-1])) --e;
    const bool comma = e > p && std::memchr(p, ',', (size_t)(e - p)) != nullptr;
    std::vector<std::pair<const char*, const char*>> fields;
    if (comma) {
        const char* s = p;
        for (const char* q = p;; ++q) {
            if (q == e || *q == ',') {
                fields.push_back({s, q});
                if (q == e) break;
                s = q + 1;
            }
        }
        // getline(ss, s, ',') yields nothing after a final comma
        if (!fields.empty() && e > p && e[-1] == ',') fields.pop_back();
    } else {
        const char* q = p;
        while (q < e) {
            while (q < e && is_ws(*q)) ++q;
            if (q >= e) break;
            const char* s = q;
            while (q < e && !is_ws(*q)) ++q;
            fields.push_back({s, q});
        }
    }
    size_t start = 0;
    if (labeled) {
        if (fields.empty()) {
            why = "missing label";
            return false;
        }
        std::string t(fields[0].first, fields[0].second);
        char* end = nullptr;
        errno = 0;
        long v = std::strtol(t.c_str(), &end, 10);
        if (end == t.c_str() || errno == ERANGE || v < INT32_MIN || v > INT32_MAX) {
            why = "label '" + t + "' is not an integer";
            return false;
        }
        label = (int32_t)v;
        start = 1;
    }
    char tmp[128];
    for (size_t f = start; f < fields.size(); ++f) {
        size_t len = (size_t)(fields[f].second - fields[f].first);
        if (len >= sizeof(tmp)) len = sizeof(tmp) - 1;
        std::memcpy(tmp, fields[f].first, len);
        tmp[len] = 0;
        vals.push_back((float)std::atof(tmp));  // atof: no digits -> 0
    }
    return true;
}

}  // namespace

extern "C" {

int tc_read_file(const char* path, int labeled, float** data, int32_t** labels, int64_t* n_out, int* m_out,
                 char* err, int err_len) {
    auto fail = [&](int code, const std::string& msg) {
        if (err && err_len > 0) {
            std::snprintf(err, (size_t)err_len, "%s", msg.c_str());
        }
        return code;
    };
    if (!path || !data || !n_out || !m_out) return fail(TC_ERR_ARG, "null argument");
    *data = nullptr;
    if (labels) *labels = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(TC_ERR_IO, std::string("cannot open ") + path);
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<char> buf((size_t)std::max(sz, 0L) + 1);
    size_t got = sz > 0 ? std::fread(buf.data(), 1, (size_t)sz, f) : 0;
    std::fclose(f);
    buf[got] = 0;
    std::vector<Line> lines;
    const char* p = buf.data();
    const char* end = p + got;
    while (p < end) {
        const char* q = (const char*)std::memchr(p, '\n', (size_t)(end - p));
        if (!q) q = end;
        const char* a = p;
        while (a < q && is_ws(*a)) ++a;
        if (a < q) lines.push_back({p, q});
        p = q + 1;
    }
    if (lines.empty()) return fail(TC_ERR_IO, "no data rows");
    const int64_t n = (int64_t)lines.size();
    // the first row fixes m
    std::vector<float> v0;
    int32_t l0 = 0;
    std::string why;
    if (!parse_line(lines[0], labeled != 0, v0, l0, why)) return fail(TC_ERR_IO, "row 1: " + why);
    const int m = (int)v0.size();
    if (m < 1) return fail(TC_ERR_IO, "row 1 has no values");
    float* D = (float*)std::malloc(sizeof(float) * (size_t)n * m);
    int32_t* Lb = labeled ? (int32_t*)std::malloc(sizeof(int32_t) * (size_t)n) : nullptr;
    if (!D || (labeled && !Lb)) {
        std::free(D);
        std::free(Lb);
        return fail(TC_ERR_NOMEM, "out of host memory");
    }
    unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096) nth = 1;
    std::vector<int64_t> bad(nth, -1);
    std::vector<std::string> bad_why(nth);
    auto work = [&](unsigned t) {
        std::vector<float> vals;
        int64_t lo = n * t / nth, hi = n * (t + 1) / nth;
        for (int64_t i = lo; i < hi; ++i) {
            int32_t lab = 0;
            std::string w;
            if (!parse_line(lines[i], labeled != 0, vals, lab, w)) {
                bad[t] = i;
                bad_why[t] = w;
                return;
            }
            if ((int)vals.size() != m) {
                bad[t] = i;
                bad_why[t] = "has " + std::to_string(vals.size()) + " values, expected " + std::to_string(m);
                return;
            }
            std::memcpy(D + (size_t)i * m, vals.data(), sizeof(float) * m);
            if (Lb) Lb[i] = lab;
        }
    };
    if (nth == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nth; ++t) th.emplace_back(work, t);
        for (auto& t : th) t.join();
    }
    for (unsigned t = 0; t < nth; ++t)
        if (bad[t] >= 0) {
            std::free(D);
            std::free(Lb);
            return fail(TC_ERR_IO, "row " + std::to_string(bad[t] + 1) + ": " + bad_why[t]);
        }
    *data = D;
    if (labels) *labels = Lb;
    else std::free(Lb);
    *n_out = n;
    *m_out = m;
    return TC_OK;
}

void tc_free_host(void* p) { std::free(p); }

// writeFile<int> (readfile.cuh:121-129): "v," per value, no newline.
int tc_write_labels(const char* path, const int32_t* labels, int64_t n) {
    if (!path || (!labels && n > 0)) return TC_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return TC_ERR_IO;
    std::string out;
    out.reserve((size_t)n * 4);
    char tmp[16];
    for (int64_t i = 0; i < n; ++i) {
        int len = std::snprintf(tmp, sizeof(tmp), "%d,", labels[i]);
        out.append(tmp, (size_t)len);
    }
    bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    ok &= std::fclose(f) == 0;
    return ok ? TC_OK : TC_ERR_IO;
}

int tc_write_centroids(const char* path, const float* C, int k, int m) {
    if (!path || !C || k < 1 || m < 1) return TC_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return TC_ERR_IO;
    for (int j = 0; j < k; ++j)
        for (int t = 0; t < m; ++t) std::fprintf(f, t + 1 < m ? "%.9g," : "%.9g\n", (double)C[(size_t)j * m + t]);
    return std::fclose(f) == 0 ? TC_OK : TC_ERR_IO;
}

// randomSelectK (kshape.cuh:159-176) with the random_device seed replaced by `seed`:
// mt19937 + uniform_int_distribution<int>(0, n-1), rejecting repeats.
int tc_random_select(int64_t n, int k, uint32_t seed, int32_t* out) {
    if (!out || k < 0 || n < 1 || k > n || n > INT32_MAX) return TC_ERR_ARG;
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
    return TC_OK;
}

// test_kshape.cu:24-30
int tc_k_from_labels(const int32_t* labels, int64_t n) {
    if (!labels || n < 1) return 0;
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
