// Driver around the reference's own host-side code (test infrastructure).
// Compiled by oracle/build.py against the reference headers where they lie.
// It only calls host functions, so it runs without a GPU:
//   ref_harness read <path> <labeled 0|1> <out.bin>   readFile / read_unlabeled_File (readfile.cuh:13-116)
//   ref_harness write <out_path> <l0> <l1> ...         writeFile<int> (readfile.cuh:121-129)
//   ref_harness select <n> <k> <seed>                  randomSelectK (kshape.cuh:159-176)
//   ref_harness fftsize <m>                             the fft_size expression of ncc.cuh:473
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kshape.cuh"
#include "readfile.cuh"

unsigned int tc_ref_seed = 0;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::string cmd = argv[1];
    if (cmd == "read" && argc == 5) {
        int rows = 0, cols = 0;
        std::vector<int> label;
        float* mat;
        if (atoi(argv[3])) mat = readFile<float>(argv[2], label, rows, cols);
        else mat = read_unlabeled_File<float>(argv[2], rows, cols);
        FILE* f = fopen(argv[4], "wb");
        if (!f) return 3;
        int nl = (int)label.size();
        fwrite(&rows, 4, 1, f);
        fwrite(&cols, 4, 1, f);
        fwrite(&nl, 4, 1, f);
        if (nl) fwrite(label.data(), 4, nl, f);
        fwrite(mat, 4, (size_t)rows * cols, f);
        fclose(f);
        delete[] mat;
        return 0;
    }
    if (cmd == "write" && argc >= 3) {
        std::vector<int> v;
        for (int i = 3; i < argc; ++i) v.push_back(atoi(argv[i]));
        writeFile<int>(argv[2], v.data(), (int)v.size());
        return 0;
    }
    if (cmd == "select" && argc == 5) {
        tc_ref_seed = (unsigned int)strtoul(argv[4], nullptr, 10);
        std::vector<int> r = randomSelectK(atoi(argv[2]), atoi(argv[3]));
        for (size_t i = 0; i < r.size(); ++i) printf("%d%c", r[i], i + 1 == r.size() ? '\n' : ' ');
        return 0;
    }
    if (cmd == "fftsize" && argc == 3) {
        int mat_col = atoi(argv[2]);
        const int fft_size = 1 << (int)ceil(my_log2((2 * mat_col - 1)));
        printf("%d\n", fft_size);
        return 0;
    }
    return 2;
}
