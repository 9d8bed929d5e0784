// Rectangle sums of the mirror-symmetric cartesian PSF grid from its quadrant
// summed-area table (see psf.cu for the table and splat.cu for the use).
#pragma once

#include "sc_common.cuh"

namespace sc {

// Python slice semantics of grid[lo:hi] on an axis of length n.
__device__ __forceinline__ void slice_bounds(int &lo, int &hi, int n) {
    if (lo < 0) lo = max(lo + n, 0);
    else if (lo > n) lo = n;
    if (hi < 0) hi = max(hi + n, 0);
    else if (hi > n) hi = n;
}

// Quadrant-table terms of a grid interval [a0, a1) on the (2n-1) grid with
// centre c = n-1: sum_{x in [a0,a1)} f(|x - c|) = sum_k sign_k * F(u_k) with F
// the exclusive prefix over |x - c|.  At most three terms; F(0) = 0 is dropped.
__device__ __forceinline__ int fold(int a0, int a1, int n, int *u, float *sg) {
    const int c = n - 1;
    int m = 0;
    if (a1 <= n) {
        u[m] = n - a0; sg[m++] = 1.f;
        if (n - a1 > 0) { u[m] = n - a1; sg[m++] = -1.f; }
    } else if (a0 >= c) {
        u[m] = a1 - c; sg[m++] = 1.f;
        if (a0 - c > 0) { u[m] = a0 - c; sg[m++] = -1.f; }
    } else {
        u[m] = n - a0; sg[m++] = 1.f;
        u[m] = a1 - c; sg[m++] = 1.f;
        u[m] = 1; sg[m++] = -1.f;
    }
    return m;
}

}  // namespace sc
