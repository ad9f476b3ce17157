// `test` - drop-in for the reference CLI (Code/test/test_kshape.cu:150-214):
//
//   test -d <dev> <path> <k> <flag> <init_chose> [options]
//
// flag 0: the first column is an integer label and k is derived from it
// (test_kshape.cu:24-30, iteration cap 10); flag 1: no label column, k from the
// command line (cap 20).  init_chose 0: random labels, 1: k random rows as
// centroids.  Labels are written 1-based as "l1,l2,...," (readfile.cuh:121-129).
// Options (after the positional arguments):
//   --labels-out P      label file (default ../out/cukshape/result.txt)
//   --centroids-out P   also write the k centroids, one per line
//   --max-iter N        iteration cap instead of 10 / 20
//   --mode compat|canonical
//   --precision fp32|bf16|tf32
//   --seed S            seed of the init_chose=1 row draw (default 0)
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "timesc.h"

static int usage() {
    std::fprintf(stderr,
                 "usage: test -d <dev> <path> <k> <flag> <init_chose> [--labels-out P] [--centroids-out P]\n"
                 "            [--max-iter N] [--mode compat|canonical] [--precision fp32|bf16|tf32] [--seed S]\n");
    return 2;
}

int main(int argc, char** argv) {
    if (argc < 2 || std::strcmp(argv[1], "-d") != 0) return 0;  // the reference returns 0 without -d
    if (argc < 7) return usage();
    const int dev = std::atoi(argv[2]);
    const std::string path = argv[3];
    int k = std::atoi(argv[4]);
    const int flag = std::atoi(argv[5]);
    const int init_chose = std::atoi(argv[6]);
    std::string labels_out = "../out/cukshape/result.txt", centroids_out;
    int max_iter = 0, mode = TC_MODE_COMPAT, prec = TC_PREC_FP32;
    unsigned seed = 0;
    for (int i = 7; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() -> const char* { return i + 1 < argc ? argv[++i] : nullptr; };
        const char* v = nullptr;
        if (a == "--labels-out" && (v = next())) labels_out = v;
        else if (a == "--centroids-out" && (v = next())) centroids_out = v;
        else if (a == "--max-iter" && (v = next())) max_iter = std::atoi(v);
        else if (a == "--seed" && (v = next())) seed = (unsigned)std::strtoul(v, nullptr, 10);
        else if (a == "--mode" && (v = next())) {
            if (!std::strcmp(v, "compat")) mode = TC_MODE_COMPAT;
            else if (!std::strcmp(v, "canonical")) mode = TC_MODE_CANONICAL;
            else return usage();
        } else if (a == "--precision" && (v = next())) {
            if (!std::strcmp(v, "fp32")) prec = TC_PREC_FP32;
            else if (!std::strcmp(v, "bf16")) prec = TC_PREC_BF16;
            else if (!std::strcmp(v, "tf32")) prec = TC_PREC_TF32;
            else return usage();
        } else {
            return usage();
        }
    }
    if ((flag != 0 && flag != 1) || (init_chose != 0 && init_chose != 1)) return usage();
    std::printf("device_id = %i\n", dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        std::fprintf(stderr, "no CUDA device %d\n", dev);
        return 1;
    }
    std::printf("---------------------------------------------------------------\n");
    std::printf("Device [ %i ] %s\n", dev, prop.name);
    std::printf("-------------- %s --------------\n", path.c_str());

    float* data = nullptr;
    int32_t* lab = nullptr;
    int64_t n = 0;
    int m = 0;
    char err[512] = {0};
    int rc = tc_read_file(path.c_str(), flag == 0, &data, flag == 0 ? &lab : nullptr, &n, &m, err, sizeof err);
    if (rc != TC_OK) {
        std::fprintf(stderr, "read failed: %s\n", err);
        return 1;
    }
    std::printf("mat_rows%lld mat_cols%d\n", (long long)n, m);
    if (flag == 0) k = tc_k_from_labels(lab, n);
    if (k < 1) {
        std::fprintf(stderr, "k must be >= 1\n");
        return 1;
    }
    tc_ctx* ctx = nullptr;
    if ((rc = tc_create(dev, &ctx)) != TC_OK) {
        std::fprintf(stderr, "tc_create failed (%d)\n", rc);
        return 1;
    }
    tc_job job{};
    job.h_data = data;
    job.n = n;
    job.m = m;
    job.k = k;
    job.mode = mode;
    job.precision = prec;
    job.init_chose = init_chose;
    job.seed = seed;
    job.max_iter = max_iter > 0 ? max_iter : (flag == 0 ? 10 : 20);
    job.restart = 1;
    std::vector<int32_t> out((size_t)n);
    std::vector<float> cents((size_t)k * m);
    tc_result res{};
    res.h_labels = out.data();
    res.h_centroids = cents.data();
    std::printf(init_chose == 1 ? "exec k_shape_tsl\n" : "exec k_shape\n");
    rc = tc_kshape_run(ctx, &job, &res);
    if (rc != TC_OK) {
        std::fprintf(stderr, "k-Shape failed (%d): %s\n", rc, tc_last_error(ctx));
        tc_destroy(ctx);
        return 1;
    }
    std::printf("iterations: %d  sum_class: %d  restarted: %d  inertia: %lf\n", res.iterations, res.sum_class,
                res.restarted, res.inertia);
    std::printf("total time run on GPU: %f msecs.\n", res.seconds * 1e3);
    for (auto& v : out) v += 1;  // 1-based like the reference
    if (tc_write_labels(labels_out.c_str(), out.data(), n) != TC_OK)
        std::fprintf(stderr, "cannot write %s\n", labels_out.c_str());
    if (!centroids_out.empty() && tc_write_centroids(centroids_out.c_str(), cents.data(), k, m) != TC_OK)
        std::fprintf(stderr, "cannot write %s\n", centroids_out.c_str());
    tc_destroy(ctx);
    tc_free_host(data);
    tc_free_host(lab);
    std::printf("\n");
    return 0;
}
