// Shared-memory staging of stencil tiles.
//
// A block computes a TX x TZ tile of outputs.  The 8th-order operator needs
// a 4-point halo along x for the P-type field and along z for the F-type
// field only (the stencil is a cross, never a corner), so each field is
// staged as either an x-halo tile [TZ][TX+8] or a z-halo tile [TZ+8][TX].
// Points outside the grid read as zero; the grid's own 4-point frame is
// zero by construction, so no other edge handling is needed.
#pragma once

#include "common.cuh"

namespace fwi {

template <int TX, int TZ> struct TileShape {
    static constexpr int XH_W = TX + 2 * kRad;  // x-halo tile width
    static constexpr int ZH_H = TZ + 2 * kRad;  // z-halo tile height
};

// Cooperative load of rows [z0, z0+TZ) x cols [x0-4, x0+TX+4).
template <typename T, int TX, int TZ>
__device__ __forceinline__ void load_xhalo(T (*s)[TX + 2 * kRad], const T *__restrict__ g, int x0,
                                           int z0, int nx, int nz, long pitch)
{
    constexpr int W = TX + 2 * kRad;
    const int nthr = blockDim.x * blockDim.y;
    for (int k = threadIdx.y * blockDim.x + threadIdx.x; k < TZ * W; k += nthr) {
        int r = k / W, c = k - r * W;
        int gx = x0 - kRad + c, gz = z0 + r;
        s[r][c] = (gx >= 0 && gx < nx && gz < nz) ? g[(long)gz * pitch + gx] : T(0);
    }
}

// Cooperative load of rows [z0-4, z0+TZ+4) x cols [x0, x0+TX).
template <typename T, int TX, int TZ>
__device__ __forceinline__ void load_zhalo(T (*s)[TX], const T *__restrict__ g, int x0, int z0,
                                           int nx, int nz, long pitch)
{
    constexpr int H = TZ + 2 * kRad;
    const int nthr = blockDim.x * blockDim.y;
    for (int k = threadIdx.y * blockDim.x + threadIdx.x; k < H * TX; k += nthr) {
        int r = k / TX, c = k - r * TX;
        int gx = x0 + c, gz = z0 - kRad + r;
        s[r][c] = (gx < nx && gz >= 0 && gz < nz) ? g[(long)gz * pitch + gx] : T(0);
    }
}

// Second-derivative taps (unnormalised) from staged tiles.  (r, c) is the
// output's position inside the tile.  The weights sum to zero, so the taps
// are applied to differences from the centre value: for a smooth field the
// neighbour differences are small and exact, and the sum no longer cancels
// (the plain form loses about 7 bits in FP32 at 20-40 points per wavelength).
template <typename T, int W>
__device__ __forceinline__ T d2x_tile(const T (*s)[W], int r, int c)
{
    using C = Coef<T>;
    const T *q = &s[r][c + kRad];
    const T o = q[0];
    return C::d2_1 * ((q[1] - o) + (q[-1] - o)) - C::d2_2 * ((q[2] - o) + (q[-2] - o)) +
           C::d2_3 * ((q[3] - o) + (q[-3] - o)) - C::d2_4 * ((q[4] - o) + (q[-4] - o));
}

template <typename T, int TX>
__device__ __forceinline__ T d2z_tile(const T (*s)[TX], int r, int c)
{
    using C = Coef<T>;
    const int rr = r + kRad;
    const T o = s[rr][c];
    return C::d2_1 * ((s[rr + 1][c] - o) + (s[rr - 1][c] - o)) -
           C::d2_2 * ((s[rr + 2][c] - o) + (s[rr - 2][c] - o)) +
           C::d2_3 * ((s[rr + 3][c] - o) + (s[rr - 3][c] - o)) -
           C::d2_4 * ((s[rr + 4][c] - o) + (s[rr - 4][c] - o));
}

}  // namespace fwi
