// Candidate lists of the screened FP32 assignment.
//
// The BF16 tensor-core pass writes, per series, the centroids whose FP32 distance
// can be the minimum: at most SCREEN_CAP of them, in ascending order, and a count
// (-1: evaluate all).  The FFT pass reads them.  A list is used only if it is
// well formed; anything else - a count the tensor-core pass never wrote because
// one of its bounded waits ran out, stale workspace from a call with another k -
// makes the FFT pass evaluate every centroid, so it never indexes centroid
// spectra with a value outside [0, k).
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace tc {

constexpr int SCREEN_CAP = 8;

// Number of candidates to evaluate from list cl of count ncl, or -1 for all k.
__host__ __device__ inline int screen_list_len(const int32_t* cl, int ncl, int k) {
    if (ncl <= 0 || ncl > SCREEN_CAP) return -1;  // the pass always keeps at least one
    int prev = -1;
    for (int i = 0; i < ncl; ++i) {
        const int c = cl[i];
        if (c <= prev || c >= k) return -1;
        prev = c;
    }
    return ncl;
}

}  // namespace tc
