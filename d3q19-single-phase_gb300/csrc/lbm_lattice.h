// D3Q19 lattice tables shared by host and device code.
//
// Population order and velocities follow d'Humieres et al. (2002), the order
// the reference fixes in Channel-Flow/para.f90:176-203 (cix/ciy/ciz at
// :201-203, opposite directions ipopp at :206, weights ww0/ww1/ww2 at
// :172-174).  Axes are the reference's: x wall-normal, y streamwise,
// z spanwise.
//
// Device layout (GPU axes): the populations live in HBM as 19 planes of
// N = nx*ny*nz values (SoA).  Inside a plane the node index is
//     n = X + NX*(Y + NY*Z),   X = ref y (streamwise, periodic, contiguous)
//                              Y = ref z (spanwise, periodic)
//                              Z = ref x (wall-normal, bounce-back walls)
// so that rows along the longest periodic axis are contiguous and the two
// walls are whole planes (no divergence at the walls inside a thread block).
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace lbm {

constexpr int Q = 19;

// velocity components in reference axes (functions so that device code can
// use them; after loop unrolling every call folds to a constant)
__host__ __device__ constexpr int CXf(int i) {
    constexpr int t[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
    return t[i];
}
__host__ __device__ constexpr int CYf(int i) {
    constexpr int t[Q] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
    return t[i];
}
__host__ __device__ constexpr int CZf(int i) {
    constexpr int t[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    return t[i];
}
__host__ __device__ constexpr int OPPf(int i) {
    constexpr int t[Q] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
    return t[i];
}

constexpr double W0 = 1.0 / 3.0, W1 = 1.0 / 18.0, W2 = 1.0 / 36.0;
__host__ __device__ constexpr double weight(int i) { return i == 0 ? W0 : (i <= 6 ? W1 : W2); }

// GPU-axis offsets of population i: (dX, dY, dZ) = (cy, cz, cx)
__host__ __device__ constexpr int DXg(int i) { return CYf(i); }
__host__ __device__ constexpr int DYg(int i) { return CZf(i); }
__host__ __device__ constexpr int DZg(int i) { return CXf(i); }

}  // namespace lbm
