// Shared device-side definitions of the sm_103a FWI library.
//
// Grid convention (the reference's, include/parallelcalls.h:5): arrays are
// [iz][ix] with x fastest; the 4-point frame at every edge is never updated
// (Dirichlet zeros) and the CPML layers cover the left, right and bottom
// edges (src/parallelcalls.cu:55).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace fwi {

// 8th-order central coefficients, first and second derivative
// (src/parallelcalls.cu:57, 127).
template <typename T> struct Coef {
    static constexpr T d1_1 = T(4.0 / 5.0), d1_2 = T(1.0 / 5.0), d1_3 = T(4.0 / 105.0),
                       d1_4 = T(1.0 / 280.0);
    static constexpr T d2_0 = T(-205.0 / 72.0), d2_1 = T(8.0 / 5.0), d2_2 = T(1.0 / 5.0),
                       d2_3 = T(8.0 / 315.0), d2_4 = T(1.0 / 560.0);
};

// Stencil radius and the frame width that stays zero.
constexpr int kRad = 4;

__host__ __device__ inline bool interior(int ix, int iz, int nx, int nz)
{
    return ix > 3 && ix < nx - 4 && iz > 3 && iz < nz - 4;
}

// Points where the CPML memory variables are updated (src/parallelcalls.cu:55).
__host__ __device__ inline bool in_strip(int ix, int iz, int nx, int nz, int cpml)
{
    return interior(ix, iz, nx, nz) && (ix < cpml || ix > nx - cpml - 1 || iz > nz - cpml - 1);
}

// Second derivative (unnormalised) of a strided array, `s` = 1 for x and the
// row pitch for z, on differences from the centre value (the weights sum to
// zero; see d2x_tile).
template <typename T>
__device__ __forceinline__ T d2_strided(const T *__restrict__ f, long i, long s)
{
    using C = Coef<T>;
    const T o = f[i];
    return C::d2_1 * ((f[i + s] - o) + (f[i - s] - o)) - C::d2_2 * ((f[i + 2 * s] - o) + (f[i - 2 * s] - o)) +
           C::d2_3 * ((f[i + 3 * s] - o) + (f[i - 3 * s] - o)) - C::d2_4 * ((f[i + 4 * s] - o) + (f[i - 4 * s] - o));
}

template <typename T>
__device__ __forceinline__ T d1_strided(const T *__restrict__ f, long i, long s)
{
    using C = Coef<T>;
    return C::d1_1 * (f[i + s] - f[i - s]) - C::d1_2 * (f[i + 2 * s] - f[i - 2 * s]) +
           C::d1_3 * (f[i + 3 * s] - f[i - 3 * s]) - C::d1_4 * (f[i + 4 * s] - f[i - 4 * s]);
}

// Enumerates the strip points of an nx x nz grid as one flat index space:
// left columns [4, cpml), right columns [nx-cpml, nx-4), both over rows
// [4, nz-4), then the bottom rows [nz-cpml, nz-4) between them.  x runs
// fastest inside each region so that a warp touches consecutive addresses.
struct StripMap {
    int nx, nz, cpml;
    int wl, wr, wb, hb, h;  // widths of left/right/bottom regions, bottom height, side height
    int x_r0, x_b0, z_b0;   // first column of the right region and of the bottom region, first bottom row
    long nl, nr, nb;        // points per region

    __host__ __device__ static StripMap make(int nx, int nz, int cpml)
    {
        StripMap m;
        m.nx = nx; m.nz = nz; m.cpml = cpml;
        const int lo = 4, hi_x = nx - 4, hi_z = nz - 4;
        m.h = hi_z > lo ? hi_z - lo : 0;
        int l1 = cpml < hi_x ? cpml : hi_x;           // left region: [4, l1)
        if (l1 < lo) l1 = lo;
        int r0 = nx - cpml;                           // right region: [r0, hi_x)
        if (r0 < l1) r0 = l1;
        if (r0 > hi_x) r0 = hi_x;
        m.wl = l1 - lo;
        m.wr = hi_x - r0;
        m.x_r0 = r0;
        m.x_b0 = l1;                                  // bottom region: [l1, r0) x [z_b0, hi_z)
        m.wb = r0 - l1;
        int b0 = nz - cpml;
        if (b0 < lo) b0 = lo;
        if (b0 > hi_z) b0 = hi_z;
        m.z_b0 = b0;
        m.hb = hi_z - b0;
        if (m.h <= 0 || hi_x <= lo) { m.wl = m.wr = m.wb = m.hb = m.h = 0; }
        m.nl = (long)m.wl * m.h;
        m.nr = (long)m.wr * m.h;
        m.nb = (long)m.wb * m.hb;
        return m;
    }
    __host__ __device__ long count() const { return nl + nr + nb; }
    __host__ __device__ void point(long k, int &ix, int &iz) const
    {
        if (k < nl) { ix = 4 + (int)(k % wl); iz = 4 + (int)(k / wl); return; }
        k -= nl;
        if (k < nr) { ix = x_r0 + (int)(k % wr); iz = 4 + (int)(k / wr); return; }
        k -= nr;
        ix = x_b0 + (int)(k % wb);
        iz = z_b0 + (int)(k / wb);
    }
};

}  // namespace fwi

#define FWI_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t e_ = (expr);                             \
        if (e_ != cudaSuccess) return fwi_status_from_cuda(e_); \
    } while (0)
