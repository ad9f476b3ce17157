// CPU check of the tensor-core Gram's strip enumeration (gram_strips.h): for every
// tile grid up to 64 x 64 and both strip widths, the strips cover each upper-triangle
// tile exactly once, the sum kernel's width lookup names the strip that covers a
// tile, and a strip loads at most w0 tiles per K slab.
#include <cstdio>
#include <vector>

#include "gram_strips.h"

int main() {
    int bad = 0;
    for (int w0 : {2, 4}) {
        for (int nt = 1; nt <= 64; ++nt) {
            std::vector<int> cover(nt * nt, 0), width(nt * nt, 0);
            const int S = tc::gram_strips(nt, w0);
            int loads = 0;
            for (int t = 0; t < S; ++t) {
                int r, q0, w;
                bool diag;
                tc::gram_strip(nt, w0, t, r, q0, w, diag);
                if (w < 1 || (diag && w > w0) || (!diag && w > w0 - 1) || (diag && q0 != r) || (!diag && q0 <= r) ||
                    q0 + w > nt || r >= nt) {
                    std::printf("bad strip nt=%d w0=%d t=%d: r=%d q0=%d w=%d diag=%d\n", nt, w0, t, r, q0, w, diag);
                    ++bad;
                    continue;
                }
                loads += diag ? w : w + 1;
                for (int q = q0; q < q0 + w; ++q) {
                    ++cover[r * nt + q];
                    width[r * nt + q] = w;
                }
            }
            for (int r = 0; r < nt; ++r)
                for (int q = 0; q < nt; ++q) {
                    const int want = q >= r ? 1 : 0;
                    if (cover[r * nt + q] != want) {
                        std::printf("nt=%d w0=%d tile (%d,%d) covered %d times\n", nt, w0, r, q, cover[r * nt + q]);
                        ++bad;
                    }
                    if (q >= r && tc::gram_strip_width(nt, w0, r, q) != width[r * nt + q]) {
                        std::printf("nt=%d w0=%d tile (%d,%d): width %d, lookup %d\n", nt, w0, r, q,
                                    width[r * nt + q], tc::gram_strip_width(nt, w0, r, q));
                        ++bad;
                    }
                }
            const int pairs = nt * (nt + 1) / 2, pair_loads = nt + 2 * (pairs - nt);  // tile pairs: 1 or 2 loads
            if (loads > pair_loads) {
                std::printf("nt=%d w0=%d: %d tile loads per slab against %d for tile pairs\n", nt, w0, loads,
                            pair_loads);
                ++bad;
            }
            if (nt == 4 && w0 == 4 && loads != 10) {
                std::printf("nt=4 w0=4: %d tile loads per slab, expected 10\n", loads);
                ++bad;
            }
        }
    }
    if (bad) {
        std::printf("%d problems\n", bad);
        return 1;
    }
    std::printf("ALL OK\n");
    return 0;
}
