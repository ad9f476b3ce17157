// Driver around the reference's own GPU code (test infrastructure).
//
// Compiled by oracle/build.py (build_ref_gpu) against a git-ignored copy of the
// reference headers staged under oracle/_ref/src/include, with the seeded
// random_device shim force-included.  No reference source is edited.  It calls
// the reference's templates exactly as its CLI driver does, with float data
// (Code/test/test_kshape.cu:9), and writes raw little-endian outputs:
//
//   ref_gpu init    n k out.i32                           idx_init (kshape.cuh:16-32): 1-based labels
//   ref_gpu znorm   n m x.f32 out.f32                     z_norm_gpu_x, ddof 1 (normalization.cuh:150-177)
//   ref_gpu assign  n m k x.f32 c.f32 out                 NCC_3D + get_pos_idx (ncc.cuh:469-517, kshape.cuh:35-96)
//                                                         out: int32 labels[n] (1-based), float dist[n]
//   ref_gpu extract n m k cal_select x.f32 l.i32 c.f32 out
//                                                         extract_shape (shapeExtract.cuh:1058-1181)
//                                                         l: 1-based labels; out: float centroids[k*m],
//                                                         int32 counts[k], int32 sum_class
//   ref_gpu loop    n m k init_chose iternum seed x.f32 out
//                                                         the driver's path after parsing
//                                                         (test_kshape.cu:13-137): copy in, z_norm_gpu_x,
//                                                         k_shape / k_shape_tsl, the cal_select=1 restart;
//                                                         out: int32 labels[n] (1-based), int32 iterations,
//                                                         int32 sum_class, int32 restarted,
//                                                         float norm_ms, float loop_ms
//
// x.f32 holds n*m floats: raw values for znorm and loop, z-normalised rows for
// assign and extract.  The reference's maxAndShift calls device malloc(m*4)
// per thread (SBD.cuh:55) and never raises the device heap; the harness raises
// it first so that every such malloc succeeds on the sizes it is given.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kshape.cuh"

unsigned int tc_ref_seed = 0;

static bool read_exact(const char* path, void* dst, size_t bytes) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    size_t got = fread(dst, 1, bytes, f);
    fclose(f);
    return got == bytes;
}

static bool write_parts(const char* path, const std::vector<std::pair<const void*, size_t>>& parts) {
    FILE* f = fopen(path, "wb");
    if (!f) return false;
    bool ok = true;
    for (const auto& p : parts) ok = ok && fwrite(p.first, 1, p.second, f) == p.second;
    fclose(f);
    return ok;
}

static int fail(const char* what) {
    fprintf(stderr, "ref_gpu: %s\n", what);
    return 3;
}

static bool cuda_ok(const char* where) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "ref_gpu: CUDA error after %s: %s\n", where, cudaGetErrorString(e));
        return false;
    }
    return true;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string cmd = argv[1];
    // 1 GiB device heap: maxAndShift holds cnt * m * 4 bytes at once for a
    // cluster of cnt members (SBD.cuh:55-63).
    if (cudaDeviceSetLimit(cudaLimitMallocHeapSize, size_t(1) << 30) != cudaSuccess)
        return fail("cannot raise the device heap");

    if (cmd == "init" && argc == 5) {
        const int n = atoi(argv[2]), k = atoi(argv[3]);
        int* d = nullptr;
        CHECK(cudaMalloc(&d, (size_t)n * 4));
        // the launch of the loop (kshape.cuh:217-222)
        idx_init<<<(n + 31) / 32, 32>>>(d, k, n);
        if (!cuda_ok("idx_init")) return 4;
        std::vector<int> lab(n);
        CHECK(cudaMemcpy(lab.data(), d, (size_t)n * 4, cudaMemcpyDeviceToHost));
        cudaFree(d);
        return write_parts(argv[4], {{lab.data(), (size_t)n * 4}}) ? 0 : fail("write");
    }

    if (cmd == "znorm" && argc == 6) {
        const int n = atoi(argv[2]), m = atoi(argv[3]);
        std::vector<float> x((size_t)n * m);
        if (!read_exact(argv[4], x.data(), x.size() * 4)) return fail("read x");
        float* d = nullptr;
        CHECK(cudaMalloc(&d, x.size() * 4));
        CHECK(cudaMemcpy(d, x.data(), x.size() * 4, cudaMemcpyHostToDevice));
        z_norm_gpu_x(d, n, m, 1);
        if (!cuda_ok("z_norm_gpu_x")) return 4;
        CHECK(cudaMemcpy(x.data(), d, x.size() * 4, cudaMemcpyDeviceToHost));
        cudaFree(d);
        return write_parts(argv[5], {{x.data(), x.size() * 4}}) ? 0 : fail("write");
    }

    if (cmd == "assign" && argc == 8) {
        const int n = atoi(argv[2]), m = atoi(argv[3]), k = atoi(argv[4]);
        std::vector<float> x((size_t)n * m), c((size_t)k * m);
        if (!read_exact(argv[5], x.data(), x.size() * 4)) return fail("read x");
        if (!read_exact(argv[6], c.data(), c.size() * 4)) return fail("read c");
        const int ncc_len = 2 * m - 1;
        float *d_x, *d_c, *d_ncc, *d_part;
        int* d_idx;
        CHECK(cudaMalloc(&d_x, x.size() * 4));
        CHECK(cudaMalloc(&d_c, c.size() * 4));
        CHECK(cudaMalloc(&d_ncc, (size_t)n * k * ncc_len * 4));
        CHECK(cudaMalloc(&d_part, (size_t)n * 4));
        CHECK(cudaMalloc(&d_idx, (size_t)n * 4));
        CHECK(cudaMemcpy(d_x, x.data(), x.size() * 4, cudaMemcpyHostToDevice));
        CHECK(cudaMemcpy(d_c, c.data(), c.size() * 4, cudaMemcpyHostToDevice));
        cudaMemset(d_ncc, 0, (size_t)n * k * ncc_len * 4);
        // As in the loop (kshape.cuh:257, :265): one 512-thread block per series.
        NCC_3D(d_x, d_c, d_ncc, n, k, m);
        get_pos_idx<<<n, 512, sizeof(float) * 512>>>(d_ncc, d_idx, d_part, k, ncc_len, n);
        if (!cuda_ok("NCC_3D/get_pos_idx")) return 4;
        std::vector<int> lab(n);
        std::vector<float> dist(n);
        CHECK(cudaMemcpy(lab.data(), d_idx, (size_t)n * 4, cudaMemcpyDeviceToHost));
        CHECK(cudaMemcpy(dist.data(), d_part, (size_t)n * 4, cudaMemcpyDeviceToHost));
        cudaFree(d_x); cudaFree(d_c); cudaFree(d_ncc); cudaFree(d_part); cudaFree(d_idx);
        return write_parts(argv[7], {{lab.data(), (size_t)n * 4}, {dist.data(), (size_t)n * 4}}) ? 0 : fail("write");
    }

    if (cmd == "extract" && argc == 10) {
        const int n = atoi(argv[2]), m = atoi(argv[3]), k = atoi(argv[4]), cal_select = atoi(argv[5]);
        std::vector<float> x((size_t)n * m), c((size_t)k * m);
        std::vector<int> lab(n);
        if (!read_exact(argv[6], x.data(), x.size() * 4)) return fail("read x");
        if (!read_exact(argv[7], lab.data(), lab.size() * 4)) return fail("read labels");
        if (!read_exact(argv[8], c.data(), c.size() * 4)) return fail("read c");
        for (int i = 0; i < n; ++i)
            if (lab[i] < 1 || lab[i] > k) return fail("labels must be 1..k");
        float *d_x, *d_c;
        int *d_idx, *d_kcount;
        CHECK(cudaMalloc(&d_x, x.size() * 4));
        CHECK(cudaMalloc(&d_c, c.size() * 4));
        CHECK(cudaMalloc(&d_idx, (size_t)n * 4));
        CHECK(cudaMalloc(&d_kcount, (size_t)k * 4));
        CHECK(cudaMemcpy(d_x, x.data(), x.size() * 4, cudaMemcpyHostToDevice));
        CHECK(cudaMemcpy(d_c, c.data(), c.size() * 4, cudaMemcpyHostToDevice));
        CHECK(cudaMemcpy(d_idx, lab.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
        cudaMemset(d_kcount, 0, (size_t)k * 4);
        int sum_class = k;
        // The call of the loop (kshape.cuh:245, :451).
        extract_shape(d_idx, d_x, d_kcount, d_c, k, n, n, m, sum_class, cal_select);
        if (!cuda_ok("extract_shape")) return 4;
        std::vector<int> counts(k);
        CHECK(cudaMemcpy(c.data(), d_c, c.size() * 4, cudaMemcpyDeviceToHost));
        CHECK(cudaMemcpy(counts.data(), d_kcount, (size_t)k * 4, cudaMemcpyDeviceToHost));
        cudaFree(d_x); cudaFree(d_c); cudaFree(d_idx); cudaFree(d_kcount);
        return write_parts(argv[9], {{c.data(), c.size() * 4}, {counts.data(), (size_t)k * 4},
                                     {&sum_class, 4}}) ? 0 : fail("write");
    }

    if (cmd == "loop" && argc == 10) {
        const int n = atoi(argv[2]), m = atoi(argv[3]), k = atoi(argv[4]);
        const int init_chose = atoi(argv[5]);
        int iternum = atoi(argv[6]);
        tc_ref_seed = (unsigned int)strtoul(argv[7], nullptr, 10);
        std::vector<float> x((size_t)n * m);
        if (!read_exact(argv[8], x.data(), x.size() * 4)) return fail("read x");
        cudaEvent_t e0, e1, e2;
        cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventCreate(&e2);
        std::vector<int> idx(n);
        float* d_mat = nullptr;
        // test_kshape.cu:34-38 (labelled) / :95-99 (unlabelled).
        cudaEventRecord(e0);
        CHECK(cudaMalloc(&d_mat, x.size() * 4));
        CHECK(cudaMemcpy(d_mat, x.data(), x.size() * 4, cudaMemcpyHostToDevice));
        z_norm_gpu_x(d_mat, n, m, 1);
        cudaEventRecord(e1);
        // test_kshape.cu:41-60 / :100-116.  sum_class starts at k (the labelled
        // driver leaves it unset; it is assigned by the first extraction).
        int sum_class = k, cal_select = 0, iternum2 = iternum, restarted = 0;
        if (init_chose == 1) k_shape_tsl(d_mat, x.data(), idx.data(), n, m, k, iternum, sum_class, cal_select);
        else k_shape(d_mat, idx.data(), n, m, k, iternum, sum_class, cal_select);
        if (sum_class == 1 || sum_class < (k / 2)) {
            cal_select = 1;
            sum_class = k;
            restarted = 1;
            k_shape(d_mat, idx.data(), n, m, k, iternum2, sum_class, cal_select);
            iternum = iternum2;
        }
        cudaEventRecord(e2);
        cudaEventSynchronize(e2);
        if (!cuda_ok("k_shape")) return 4;
        float norm_ms = 0.f, loop_ms = 0.f;
        cudaEventElapsedTime(&norm_ms, e0, e1);
        cudaEventElapsedTime(&loop_ms, e1, e2);
        cudaFree(d_mat);
        return write_parts(argv[9], {{idx.data(), (size_t)n * 4}, {&iternum, 4}, {&sum_class, 4},
                                     {&restarted, 4}, {&norm_ms, 4}, {&loop_ms, 4}}) ? 0 : fail("write");
    }
    return 2;
}
