// The strips of the tensor-core Gram (tensor_core.cu): the upper triangle of an
// nt x nt grid of 128 x 128 tiles, cut row by row into strips of column tiles.  A
// strip that starts at the diagonal holds up to w0 tiles (its A tile is its first B
// tile); the rest of the row goes in strips of up to w0 - 1 tiles plus the A tile, so
// every strip loads at most w0 tiles per K slab.  Host and device code, checked on the
// CPU by tests/native/gram_strips_check.cpp.
#pragma once

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace tc {

// Strips of the upper triangle of nt x nt tiles, row by row (widest first in each row).
__host__ __device__ inline int gram_row_strips(int nt, int r, int w0) {
    const int rest = nt - r - w0;
    return 1 + (rest > 0 ? (rest + w0 - 2) / (w0 - 1) : 0);
}
__host__ __device__ inline int gram_strips(int nt, int w0) {
    int s = 0;
    for (int r = 0; r < nt; ++r) s += gram_row_strips(nt, r, w0);
    return s;
}
// strip t -> row tile r, first column tile q0, width w, diagonal (A is B tile 0)
__host__ __device__ inline void gram_strip(int nt, int w0, int t, int& r, int& q0, int& w, bool& diag) {
    r = 0;
    while (t >= gram_row_strips(nt, r, w0)) t -= gram_row_strips(nt, r++, w0);
    if (t == 0) {
        q0 = r;
        w = nt - r < w0 ? nt - r : w0;
        diag = true;
    } else {
        q0 = r + w0 + (t - 1) * (w0 - 1);
        w = nt - q0 < w0 - 1 ? nt - q0 : w0 - 1;
        diag = false;
    }
}
// width of the strip holding tile (lo, hi), lo <= hi
__host__ __device__ inline int gram_strip_width(int nt, int w0, int lo, int hi) {
    if (hi < lo + w0) return nt - lo < w0 ? nt - lo : w0;
    const int q0 = lo + w0 + (hi - lo - w0) / (w0 - 1) * (w0 - 1);
    return nt - q0 < w0 - 1 ? nt - q0 : w0 - 1;
}

}  // namespace tc
