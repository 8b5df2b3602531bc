// Boundary storage (FWI_STORE_BOUNDARY): the forward keeps, every step, the
// ring of the state around the region R the CPML layers do not touch,
// R = [cpml, nx - cpml) x [4, nz - cpml) of each shot's window; the adjoint
// then runs the forward step backwards inside R to rebuild the state step by
// step, and takes the images from it.
//
// Forward step g (increment form, R has no CPML term):
//   v^{g+1} = v^g + (v_hor Dxx P^g + v_po Dzz F^g) + w_g [source],  P^{g+1} = P^g + v^{g+1}
// (and F with v_nmo).  Backwards:
//   P^g = P^{g+1} - v^{g+1},  v^g = v^{g+1} - (v_hor Dxx P^g + v_po Dzz F^g) - w_g.
// Dxx P^g at R's first and last 4 columns reads P^g in the 4 columns beside
// R, Dzz F^g at R's last 4 rows reads F^g in the 4 rows below R (above R is
// the zero frame): that ring is what the forward saves.  The images of R's
// points are the forward's (no CPML term in R, so G = Dxx P and H = Dzz F in
// both modes); the images of the layer points are zero, so the gradient in
// the layers is zero in this mode.  The reconstruction repeats the
// forward's arithmetic backwards; FP rounding makes it approximate (the
// difference to FWI_STORE_FULL is measured in the tests).
#pragma once

#include <algorithm>

#include "prop.cuh"

namespace fwi {

// ring[s][g][k] <- the state P^g, F^g of the ring points, for the shots active at
// global step g (called before step g).
template <typename T>
__global__ void k_save_ring(Batch<T> b, int g, int ntb, int cur, T *ring, long ring_len)
{
    const int s = blockIdx.y;
    const DevShot sh = b.shots[s];
    if (g - (ntb - sh.nt) < 0) return;
    const Ring R = Ring::make(sh.nx, b.nz, b.cpml);
    const long so = (long)s * b.slot;
    T *out = ring + ((long)s * b.nt_max + g) * ring_len;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < R.count(); k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        bool isF;
        R.point(k, ix, iz, isF);
        out[k] = b.lvl[isF ? 2 + cur : cur][so + (long)iz * b.pitch + ix];
    }
}

// Level `lev` of the rebuild state gets the ring of step g.
template <typename T>
__global__ void k_load_ring(Batch<T> b, int g, int ntb, int lev, const T *ring, long ring_len)
{
    const int s = blockIdx.y;
    const DevShot sh = b.shots[s];
    if (g < 0 || g - (ntb - sh.nt) < 0) return;
    const Ring R = Ring::make(sh.nx, b.nz, b.cpml);
    const long so = (long)s * b.slot;
    const T *in = ring + ((long)s * b.nt_max + g) * ring_len;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < R.count(); k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        bool isF;
        R.point(k, ix, iz, isF);
        b.lvl[isF ? 2 + lev : lev][so + (long)iz * b.pitch + ix] = in[k];
    }
}

__host__ __device__ inline bool in_rebuild_region(int ix, int iz, int nx, int nz, int cpml)
{
    return ix >= cpml && ix < nx - cpml && iz >= 4 && iz < nz - cpml;
}

// P^g = P^{g+1} - v^{g+1} (and F) in R: from level `src` (P^{g+1}, with v^{g+1} in
// the increments) to level 1 - src.
template <typename T>
__global__ void k_rebuild_begin(Batch<T> b, int g, int ntb, int src)
{
    const int s = blockIdx.z;
    const DevShot sh = b.shots[s];
    if (g - (ntb - sh.nt) < 0) return;
    const int ix = b.cpml + blockIdx.x * blockDim.x + threadIdx.x, iz = 4 + blockIdx.y * blockDim.y + threadIdx.y;
    if (!in_rebuild_region(ix, iz, sh.nx, b.nz, b.cpml)) return;
    const long i = (long)s * b.slot + (long)iz * b.pitch + ix;
    b.lvl[1 - src][i] = b.lvl[src][i] - b.lvl[4][i];
    b.lvl[3 - src][i] = b.lvl[2 + src][i] - b.lvl[5][i];
}

// One backward step at global step g: level `cur` holds P^g, F^g (R and the
// ring), the increments v^{g+1}.  Writes the images of step g to image slot
// `img_slot` (R only), v^g in place, and P^{g-1} = P^g - v^g into level
// 1 - cur (R only; k_load_ring fills its ring).
template <typename T, int ST>
__global__ void __launch_bounds__(256) k_rebuild_step(Batch<T> b, int g, int ntb, int cur, int img_slot)
{
    using Cd = Codec<T, ST>;
    const int s = blockIdx.z;
    const DevShot sh = b.shots[s];
    const int it = g - (ntb - sh.nt);
    if (it < 0) return;
    const int nx = sh.nx, nz = b.nz, pitch = b.pitch;
    const int ix = b.cpml + blockIdx.x * blockDim.x + threadIdx.x, iz = 4 + blockIdx.y * blockDim.y + threadIdx.y;
    float sc = 1.f;
    if (Cd::scaled) {
        sc = image_scale(b.amax[(long)s * (b.nt_max + 1) + g], (float)b.inv_dh2);
        if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
            b.scale[(long)s * b.nt_max + g] = sc;
    }
    if (!in_rebuild_region(ix, iz, nx, nz, b.cpml)) return;
    const long so = (long)s * b.slot, i = so + (long)iz * pitch + ix;
    const T *P = b.lvl[cur], *F = b.lvl[2 + cur];
    const T G = d2_strided(P, i, 1) * b.inv_dh2;
    const T H = d2_strided(F, i, (long)pitch) * b.inv_dh2;
    typename Cd::S *img = (typename Cd::S *)b.store + ((long)s * b.n_img + img_slot) * 2 * b.slot;
    img[i - so] = Cd::enc(G, sc, b.status);
    img[b.slot + i - so] = Cd::enc(H, sc, b.status);
    const long mi = (long)iz * b.mpitch + sh.x0 + ix;
    const T mpH = b.mp[mi] * H;
    T vp = b.lvl[4][i], vf = b.lvl[5][i];
    if (ix == sh.sx && iz == sh.sz) {
        const T w = b.wavelet[it];
        vp -= w;
        vf -= w;
    }
    vp -= (b.mh[mi] * G + mpH);
    vf -= (b.mn[mi] * G + mpH);
    b.lvl[4][i] = vp;
    b.lvl[5][i] = vf;
    b.lvl[1 - cur][i] = P[i] - vp;
    b.lvl[3 - cur][i] = F[i] - vf;
}

template <typename T> void launch_save_ring(const Batch<T> &b, int nx_max, int g, int ntb, int cur, T *ring,
                                            long ring_len, cudaStream_t st)
{
    const long n = Ring::make(nx_max, b.nz, b.cpml).count();
    const dim3 grid((unsigned)std::max(1L, (n + 255) / 256), b.B);
    k_save_ring<T><<<grid, 256, 0, st>>>(b, g, ntb, cur, ring, ring_len);
}

template <typename T> void launch_rebuild_begin(const Batch<T> &rb, int nx_max, int g, int ntb, int src,
                                                const T *ring, long ring_len, cudaStream_t st)
{
    const dim3 blk(32, 8), grid((nx_max + 31) / 32, (rb.nz + 7) / 8, rb.B);
    k_rebuild_begin<T><<<grid, blk, 0, st>>>(rb, g, ntb, src);
    const long n = Ring::make(nx_max, rb.nz, rb.cpml).count();
    k_load_ring<T><<<dim3((unsigned)std::max(1L, (n + 255) / 256), rb.B), 256, 0, st>>>(rb, g, ntb, 1 - src, ring,
                                                                                       ring_len);
}

template <typename T> void launch_rebuild_step(const Batch<T> &rb, int nx_max, int g, int ntb, int cur,
                                               const T *ring, long ring_len, int img_slot, cudaStream_t st)
{
    const dim3 blk(32, 8), grid((nx_max + 31) / 32, (rb.nz + 7) / 8, rb.B);
    switch (rb.store_type) {
    case kStoreHalf: k_rebuild_step<T, kStoreHalf><<<grid, blk, 0, st>>>(rb, g, ntb, cur, img_slot); break;
    case kStoreBf16: k_rebuild_step<T, kStoreBf16><<<grid, blk, 0, st>>>(rb, g, ntb, cur, img_slot); break;
    default: k_rebuild_step<T, kStoreNative><<<grid, blk, 0, st>>>(rb, g, ntb, cur, img_slot); break;
    }
    const long n = Ring::make(nx_max, rb.nz, rb.cpml).count();
    k_load_ring<T><<<dim3((unsigned)std::max(1L, (n + 255) / 256), rb.B), 256, 0, st>>>(rb, g - 1, ntb, 1 - cur, ring,
                                                                                       ring_len);
}

}  // namespace fwi
