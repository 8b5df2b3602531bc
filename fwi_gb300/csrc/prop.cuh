// Batched forward and adjoint time steps of the native path (templated on
// the compute type T; instantiated by prop_f32.cu and prop_f64.cu).
//
// Per step and batch: one pass over the CPML strip points (memory variables
// whose x/z derivatives the main pass needs), then one tiled main pass over
// every (shot, 32x32 tile).  The main pass stages the two stencil fields in
// shared memory with the halo only along the axis their operator needs (P
// and the adjoint's x-combination along x, F and the z-combination along z),
// and does all point-wise work of the step in registers: CPML zeta terms,
// leapfrog update, source, receivers, image store (forward) or residual
// injection and the imaging condition (adjoint).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "prop.h"
#include "tile.cuh"

namespace fwi {

constexpr int PTX = 32, PTZ = 32, PBY = 8;  // tile and block of the main passes
constexpr int PXW = PTX + 2 * kRad, PZH = PTZ + 2 * kRad;
constexpr int kStripBlock = 256;

// CPML coefficient of column ix / row iz of a grid (src/parallelcalls.cu:23-33, 41-45),
// looked up by distance into the layer.
template <typename T>
__device__ __forceinline__ T coef_x(const T *tab, int ix, int nx, int cpml)
{
    if (ix < cpml) return tab[cpml - ix];
    if (ix > nx - cpml - 1) return tab[ix - nx + cpml + 1];
    return T(0);
}
template <typename T>
__device__ __forceinline__ T coef_z(const T *tab, int iz, int nz, int cpml)
{
    return iz > nz - cpml - 1 ? tab[iz - nz + cpml + 1] : T(0);
}

// ---------------------------------------------------------------- image store codecs

template <typename T, int ST> struct Codec;
// enc(v, sc, status) reports saturation at once; enc_flag(v, sc, sat) only
// sets `sat` (NaN included), for callers that report once per thread.
template <typename T> struct Codec<T, kStoreNative> {
    using S = T;
    static constexpr bool scaled = false;
    static __device__ __forceinline__ S enc(T v, float, unsigned *) { return v; }
    static __device__ __forceinline__ S enc_flag(T v, float, bool &) { return v; }
    static __device__ __forceinline__ T dec(S v, float) { return v; }  // second argument: inverse scale
};
template <typename T> struct Codec<T, kStoreHalf> {
    using S = __half;
    static constexpr bool scaled = true;
    static __device__ __forceinline__ S enc(T v, float sc, unsigned *status)
    {
        float x = (float)v * sc;
        if (fabsf(x) > 65504.f) {  // saturate instead of storing inf, and report it
            x = copysignf(65504.f, x);
            atomicOr(status, 1u);
        }
        return __float2half_rn(x);
    }
    static __device__ __forceinline__ S enc_flag(T v, float sc, bool &sat)
    {
        const float x = (float)v * sc;
        sat |= !(fabsf(x) <= 65504.f);
        return __float2half_rn(fminf(fmaxf(x, -65504.f), 65504.f));
    }
    static __device__ __forceinline__ T dec(S v, float inv_sc) { return (T)(__half2float(v) * inv_sc); }
};
template <typename T> struct Codec<T, kStoreBf16> {
    using S = __nv_bfloat16;
    static constexpr bool scaled = true;
    static __device__ __forceinline__ S enc(T v, float sc, unsigned *) { return __float2bfloat16_rn((float)v * sc); }
    static __device__ __forceinline__ S enc_flag(T v, float sc, bool &) { return __float2bfloat16_rn((float)v * sc); }
    static __device__ __forceinline__ T dec(S v, float inv_sc) { return (T)(__bfloat162float(v) * inv_sc); }
};

// Per-snapshot scale: a power of two that maps the largest possible image
// value of the step to about 2^14.  |G|, |H| <= 32 max(|P|,|F|) / dh^2 for
// the 8th-order operator plus the CPML terms (|a| / (1 - b) <= 1), so the
// bound comes from the state's max, which the previous step recorded.  Made
// with ldexpf so that it and its inverse are exact powers of two: decoding
// multiplies by the inverse and gets the same value a division would.
__device__ __forceinline__ float image_scale(float amax, float inv_dh2)
{
    const float bound = 32.f * amax * inv_dh2;
    if (!(bound > 0.f) || !isfinite(bound)) return 1.f;
    const float e = floorf(log2f(16384.f / bound));
    return ldexpf(1.f, (int)fminf(fmaxf(e, -120.f), 120.f));
}

__device__ __forceinline__ void block_max_to(float v, float *dst)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ float wmax[32];
    const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
    const int warp = (threadIdx.y * blockDim.x + threadIdx.x) >> 5;
    const int nw = (blockDim.x * blockDim.y + 31) >> 5;
    if (lane == 0) wmax[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nw ? wmax[lane] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.f) atomicMax((unsigned *)dst, __float_as_uint(v));  // v >= 0
    }
}

// ---------------------------------------------------------------- forward

template <typename T>
__global__ void __launch_bounds__(kStripBlock) k_fwd_strip(Batch<T> b, int g, int ntb, int cur)
{
    const int s = blockIdx.y;
    const DevShot sh = b.shots[s];
    const int it = g - (ntb - sh.nt);
    if (it < 0) return;
    const StripMap sm = StripMap::make(sh.nx, b.nz, b.cpml);
    const long so = (long)s * b.slot;
    const T *P = b.lvl[cur] + so, *F = b.lvl[2 + cur] + so;
    T *psx = b.cp[0] + so, *psz = b.cp[1] + so;
    const int pitch = b.pitch, cpml = b.cpml, nz = b.nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < sm.count();
         k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        sm.point(k, ix, iz);
        const long i = (long)iz * pitch + ix;
        if (ix < cpml || ix > sh.nx - cpml - 1)
            psx[i] = coef_x(b.cpb, ix, sh.nx, cpml) * psx[i] +
                     coef_x(b.cpa, ix, sh.nx, cpml) * (d1_strided(P, i, 1) * b.inv_dh);
        if (iz > nz - cpml - 1)
            psz[i] = coef_z(b.cpb, iz, nz, cpml) * psz[i] +
                     coef_z(b.cpa, iz, nz, cpml) * (d1_strided(F, i, pitch) * b.inv_dh);
    }
}

// `img_slot` < 0: no images this step.  A runtime flag, not a template
// parameter, so that passes with and without images execute the same
// arithmetic (a checkpointed segment must recompute the state bit for bit).
template <typename T, int ST, bool EXACT>
__global__ void __launch_bounds__(PTX * PBY)
k_fwd_main(Batch<T> b, int g, int ntb, int cur, int img_slot)
{
    const bool STORE = img_slot >= 0;
    using Cd = Codec<T, ST>;
    const int s = blockIdx.z;
    const DevShot sh = b.shots[s];
    const int it = g - (ntb - sh.nt);
    const int x0 = blockIdx.x * PTX, z0 = blockIdx.y * PTZ;
    if (it < 0 || x0 >= sh.nx) return;
    const int nx = sh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    const long so = (long)s * b.slot;
    const T *P = b.lvl[cur] + so, *F = b.lvl[2 + cur] + so;
    T *Pn = b.lvl[1 - cur] + so, *Fn = b.lvl[3 - cur] + so;
    T *Pv = b.lvl[4] + so, *Fv = b.lvl[5] + so;

    __shared__ T sP[PTZ][PXW];
    __shared__ T sF[PZH][PTX];
    load_xhalo<T, PTX, PTZ>(sP, P, x0, z0, nx, nz, pitch);
    load_zhalo<T, PTX, PTZ>(sF, F, x0, z0, nx, nz, pitch);
    __syncthreads();

    float sc = 1.f;
    typename Cd::S *img = nullptr;
    if (STORE) {
        img = (typename Cd::S *)b.store + ((long)s * b.n_img + img_slot) * 2 * b.slot;
        if (Cd::scaled) {
            sc = image_scale(b.amax[(long)s * (b.nt_max + 1) + g], (float)b.inv_dh2);
            if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
                b.scale[(long)s * b.nt_max + g] = sc;
        }
    }
    const T w = b.wavelet[it];
    const int c = threadIdx.x, ix = x0 + c;
    const int nrec = sh.rx1 - sh.rx0;
    float lmax = 0.f;
    if (ix < nx) {
        const T *psx = b.cp[0] + so, *psz = b.cp[1] + so;
        T *zx = b.cp[2] + so, *zz = b.cp[3] + so;
        for (int r = threadIdx.y; r < PTZ; r += PBY) {
            const int iz = z0 + r;
            if (iz >= nz) break;
            if (!interior(ix, iz, nx, nz)) continue;
            const long i = (long)iz * pitch + ix;
            const T p2 = d2x_tile<T, PXW>(sP, r, c) * b.inv_dh2;
            const T r2 = d2z_tile<T, PTX>(sF, r, c) * b.inv_dh2;
            T G = p2, H = r2;
            if (in_strip(ix, iz, nx, nz, cpml)) {
                const T tx = d1_strided(psx, i, 1) * b.inv_dh;
                const T tz = d1_strided(psz, i, pitch) * b.inv_dh;
                const T zxn = coef_x(b.cpb, ix, nx, cpml) * zx[i] + coef_x(b.cpa, ix, nx, cpml) * (p2 + tx);
                const T zzn = coef_z(b.cpb, iz, nz, cpml) * zz[i] + coef_z(b.cpa, iz, nz, cpml) * (r2 + tz);
                zx[i] = zxn;
                zz[i] = zzn;
                G = p2 + (tx + zxn);
                H = r2 + (tz + zzn);
            }
            const long mi = (long)iz * b.mpitch + sh.x0 + ix;
            const T mpH = b.mp[mi] * H;
            T vp = Pv[i] + (b.mh[mi] * G + mpH);
            T vf = Fv[i] + (b.mn[mi] * G + mpH);
            if (ix == sh.sx && iz == sh.sz) { vp += w; vf += w; }
            Pv[i] = vp;
            Fv[i] = vf;
            const T pn = sP[r][c + kRad] + vp;
            const T fn = sF[r + kRad][c] + vf;
            Pn[i] = pn;
            Fn[i] = fn;
            if (iz == sh.rz && ix >= sh.rx0 && ix < sh.rx1)
                b.rec[sh.rec_off + (long)it * nrec + (ix - sh.rx0)] = pn + fn;
            if (STORE) {
                img[i] = Cd::enc(EXACT ? G : p2, sc, b.status);
                img[b.slot + i] = Cd::enc(EXACT ? H : r2, sc, b.status);
            }
            if (Cd::scaled) lmax = fmaxf(lmax, fmaxf(fabsf((float)pn), fabsf((float)fn)));
        }
    }
    // the state's max bounds the next step's images (image_scale); recorded on every
    // pass so that a segment recomputed from a checkpoint finds it
    if (Cd::scaled) block_max_to(lmax, &b.amax[(long)s * (b.nt_max + 1) + g + 1]);
}

// ---------------------------------------------------------------- adjoint

// dt^2 (v_hor lP + v_nmo lF) and dt^2 v_po (lP + lF) at one point (zero off the interior).
template <typename T>
__device__ __forceinline__ void adj_sources(const Batch<T> &b, const DevShot &sh, const T *lP,
                                            const T *lF, int ix, int iz, T &gx, T &hz)
{
    if (!interior(ix, iz, sh.nx, b.nz)) { gx = hz = T(0); return; }
    const long i = (long)iz * b.pitch + ix, mi = (long)iz * b.mpitch + sh.x0 + ix;
    const T p = lP[i], f = lF[i];
    gx = b.mh[mi] * p + b.mn[mi] * f;
    hz = b.mp[mi] * (p + f);
}

// Exact adjoint, strip pass.  With g = dt^2 (v_hor lP + v_nmo lF) of lambda^{m+1}:
//   Zx' = S (g + bx Zx),  Yx' = S (-Dx[S (g + ax Zx')] + bx Yx)   (and the same in z).
// Z is ping-ponged (neighbours read the old half), Y is updated in place.
template <typename T>
__global__ void __launch_bounds__(kStripBlock) k_adj_strip_exact(Batch<T> b, int j, int cur, int zsel)
{
    const int s = blockIdx.y;
    const DevShot sh = b.shots[s];
    if (j >= sh.nt) return;
    const StripMap sm = StripMap::make(sh.nx, b.nz, b.cpml);
    const long so = (long)s * b.slot;
    const T *lP = b.lvl[cur] + so, *lF = b.lvl[2 + cur] + so;
    T *Yx = b.cp[0] + so, *Yz = b.cp[1] + so;
    const T *Zx0 = b.cp[2 + zsel] + so, *Zz0 = b.cp[4 + zsel] + so;
    T *Zx1 = b.cp[3 - zsel] + so, *Zz1 = b.cp[5 - zsel] + so;
    const int nx = sh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    using C = Coef<T>;
    const T c1[4] = {C::d1_1, -C::d1_2, C::d1_3, -C::d1_4};
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < sm.count();
         k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        sm.point(k, ix, iz);
        const long i = (long)iz * pitch + ix;
        if (ix < cpml || ix > nx - cpml - 1) {
            T acc = T(0);
            for (int q = 1; q <= 4; q++) {
                T wv[2];
                for (int sgn = 0; sgn < 2; sgn++) {
                    const int jx = sgn ? ix - q : ix + q;
                    T w = T(0);
                    if (in_strip(jx, iz, nx, nz, cpml)) {
                        T gx, hz;
                        adj_sources(b, sh, lP, lF, jx, iz, gx, hz);
                        const T zn = gx + coef_x(b.cpb, jx, nx, cpml) * Zx0[i - ix + jx];
                        w = gx + coef_x(b.cpa, jx, nx, cpml) * zn;
                    }
                    wv[sgn] = w;
                }
                acc += c1[q - 1] * (wv[0] - wv[1]);
            }
            T gx, hz;
            adj_sources(b, sh, lP, lF, ix, iz, gx, hz);
            const T bx = coef_x(b.cpb, ix, nx, cpml);
            Zx1[i] = gx + bx * Zx0[i];
            Yx[i] = -acc * b.inv_dh + bx * Yx[i];
        }
        if (iz > nz - cpml - 1) {
            T acc = T(0);
            for (int q = 1; q <= 4; q++) {
                T wv[2];
                for (int sgn = 0; sgn < 2; sgn++) {
                    const int jz = sgn ? iz - q : iz + q;
                    T w = T(0);
                    if (in_strip(ix, jz, nx, nz, cpml)) {
                        T gx, hz;
                        adj_sources(b, sh, lP, lF, ix, jz, gx, hz);
                        const T zn = hz + coef_z(b.cpb, jz, nz, cpml) * Zz0[(long)jz * pitch + ix];
                        w = hz + coef_z(b.cpa, jz, nz, cpml) * zn;
                    }
                    wv[sgn] = w;
                }
                acc += c1[q - 1] * (wv[0] - wv[1]);
            }
            T gx, hz;
            adj_sources(b, sh, lP, lF, ix, iz, gx, hz);
            const T bz = coef_z(b.cpb, iz, nz, cpml);
            Zz1[i] = hz + bz * Zz0[i];
            Yz[i] = -acc * b.inv_dh + bz * Yz[i];
        }
    }
}

// Reference adjoint, strip pass (src/parallelcalls.cu:179-198) on the
// dt^2-scaled model-weighted adjoint fields.
template <typename T>
__global__ void __launch_bounds__(kStripBlock) k_adj_strip_ref(Batch<T> b, int j, int cur)
{
    const int s = blockIdx.y;
    const DevShot sh = b.shots[s];
    if (j >= sh.nt) return;
    const StripMap sm = StripMap::make(sh.nx, b.nz, b.cpml);
    const long so = (long)s * b.slot;
    const T *lP = b.lvl[cur] + so, *lF = b.lvl[2 + cur] + so;
    T *psixcx = b.cp[0] + so, *psixcz = b.cp[1] + so, *psizdx = b.cp[2] + so, *psizcz = b.cp[3] + so;
    const int nx = sh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml, mp = b.mpitch;
    using C = Coef<T>;
    const T c1[4] = {C::d1_1, -C::d1_2, C::d1_3, -C::d1_4};
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < sm.count();
         k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        sm.point(k, ix, iz);
        const long i = (long)iz * pitch + ix, mi = (long)iz * mp + sh.x0 + ix;
        if (ix < cpml || ix > nx - cpml - 1) {
            T d1 = T(0), d3 = T(0);
            for (int q = 1; q <= 4; q++) {
                d1 += c1[q - 1] * (b.mh[mi + q] * lP[i + q] - b.mh[mi - q] * lP[i - q]);
                d3 += c1[q - 1] * (b.mn[mi + q] * lF[i + q] - b.mn[mi - q] * lF[i - q]);
            }
            const T bx = coef_x(b.cpb, ix, nx, cpml), ax = coef_x(b.cpa, ix, nx, cpml);
            psixcx[i] = bx * psixcx[i] + ax * (d1 * b.inv_dh);
            psizdx[i] = bx * psizdx[i] + ax * (d3 * b.inv_dh);
        }
        if (iz > nz - cpml - 1) {
            T d2 = T(0), d4 = T(0);
            for (int q = 1; q <= 4; q++) {
                const long up = i + (long)q * pitch, dn = i - (long)q * pitch;
                const long mup = mi + (long)q * mp, mdn = mi - (long)q * mp;
                d2 += c1[q - 1] * (b.mp[mup] * lP[up] - b.mp[mdn] * lP[dn]);
                d4 += c1[q - 1] * (b.mp[mup] * lF[up] - b.mp[mdn] * lF[dn]);
            }
            const T bz = coef_z(b.cpb, iz, nz, cpml), az = coef_z(b.cpa, iz, nz, cpml);
            psixcz[i] = bz * psixcz[i] + az * (d2 * b.inv_dh);
            psizcz[i] = bz * psizcz[i] + az * (d4 * b.inv_dh);
        }
    }
}

// Adjoint main pass.  Tiles: U = dt^2 (v_hor lP + v_nmo lF) with an x-halo,
// V = dt^2 v_po (lP + lF) with a z-halo (lambda^{m+1}).  Interior update
//   lP^m = 2 lP - lP_old + Dxx U + (strip terms),  lF^m = 2 lF - lF_old + Dzz V + (strip terms)
// then the residual injection and the imaging condition.
template <typename T, int ST, bool EXACT>
__global__ void __launch_bounds__(PTX * PBY)
k_adj_main(Batch<T> b, int j, int ntb, int cur, int zsel, int img_base)
{
    using Cd = Codec<T, ST>;
    const int s = blockIdx.z;
    const DevShot sh = b.shots[s];
    const int x0 = blockIdx.x * PTX, z0 = blockIdx.y * PTZ;
    if (j >= sh.nt || x0 >= sh.nx) return;
    const int nx = sh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    const long so = (long)s * b.slot;
    const T *lP = b.lvl[cur] + so, *lF = b.lvl[2 + cur] + so;
    T *lPn = b.lvl[1 - cur] + so, *lFn = b.lvl[3 - cur] + so;
    T *lPw = b.lvl[4] + so, *lFw = b.lvl[5] + so;
    const int m = sh.nt - j;

    __shared__ T sU[PTZ][PXW];
    __shared__ T sV[PZH][PTX];
    {
        const int nthr = PTX * PBY;
        const int tid = threadIdx.y * PTX + threadIdx.x;
        for (int k = tid; k < PTZ * PXW; k += nthr) {
            int r = k / PXW, cc = k - r * PXW;
            T gx, hz;
            adj_sources(b, sh, lP, lF, x0 - kRad + cc, z0 + r, gx, hz);
            sU[r][cc] = gx;
        }
        for (int k = tid; k < PZH * PTX; k += nthr) {
            int r = k / PTX, cc = k - r * PTX;
            T gx, hz;
            adj_sources(b, sh, lP, lF, x0 + cc, z0 - kRad + r, gx, hz);
            sV[r][cc] = hz;
        }
    }
    __syncthreads();

    // image of global step ntb - 1 - lag - j (local step m - 1 - lag)
    const int lag = EXACT ? 0 : 1;
    const int img_local = m - 1 - lag;
    const int img_g = ntb - 1 - lag - j;
    const typename Cd::S *img = nullptr;
    float inv_sc = 1.f;
    if (img_local >= 0) {
        img = (const typename Cd::S *)b.store + ((long)s * b.n_img + (img_g - img_base)) * 2 * b.slot;
        if (Cd::scaled) inv_sc = 1.f / b.scale[(long)s * b.nt_max + img_g];
    }
    const int nrec = sh.rx1 - sh.rx0;
    const T *res_row = b.rec + sh.rec_off + (long)(m - 1) * nrec;
    const int c = threadIdx.x, ix = x0 + c;
    if (ix >= nx) return;
    T *g0 = b.g[0] + so, *g1 = b.g[1] + so, *g2 = b.g[2] + so;
    const bool near_x = ix < cpml + kRad || ix > nx - cpml - 1 - kRad;
    for (int r = threadIdx.y; r < PTZ; r += PBY) {
        const int iz = z0 + r;
        if (iz >= nz) break;
        if (!interior(ix, iz, nx, nz)) continue;
        const long i = (long)iz * pitch + ix;
        T ex = d2x_tile<T, PXW>(sU, r, c) * b.inv_dh2;
        T ez = d2z_tile<T, PTX>(sV, r, c) * b.inv_dh2;
        if (EXACT) {
            // + Dxx(S ax Zx') - Dx(S ax Yx')  (near the side layers), and the same in z
            if (near_x) {
                const T *Zx = b.cp[3 - zsel] + so, *Yx = b.cp[0] + so;
                using C = Coef<T>;
                const T c2[5] = {C::d2_0, C::d2_1, -C::d2_2, C::d2_3, -C::d2_4};
                const T c1[4] = {C::d1_1, -C::d1_2, C::d1_3, -C::d1_4};
                T a2 = c2[0] * coef_x(b.cpa, ix, nx, cpml) * Zx[i], a1 = T(0);
                for (int q = 1; q <= 4; q++) {
                    const T ap = coef_x(b.cpa, ix + q, nx, cpml), am = coef_x(b.cpa, ix - q, nx, cpml);
                    a2 += c2[q] * (ap * Zx[i + q] + am * Zx[i - q]);
                    a1 += c1[q - 1] * (ap * Yx[i + q] - am * Yx[i - q]);
                }
                ex += a2 * b.inv_dh2 - a1 * b.inv_dh;
            }
            if (iz > nz - cpml - 1 - kRad) {
                const T *Zz = b.cp[5 - zsel] + so, *Yz = b.cp[1] + so;
                using C = Coef<T>;
                const T c2[5] = {C::d2_0, C::d2_1, -C::d2_2, C::d2_3, -C::d2_4};
                const T c1[4] = {C::d1_1, -C::d1_2, C::d1_3, -C::d1_4};
                T a2 = c2[0] * coef_z(b.cpa, iz, nz, cpml) * Zz[i], a1 = T(0);
                for (int q = 1; q <= 4; q++) {
                    const long up = i + (long)q * pitch, dn = i - (long)q * pitch;
                    const T ap = coef_z(b.cpa, iz + q, nz, cpml), am = coef_z(b.cpa, iz - q, nz, cpml);
                    a2 += c2[q] * (ap * Zz[up] + am * Zz[dn]);
                    a1 += c1[q - 1] * (ap * Yz[up] - am * Yz[dn]);
                }
                ez += a2 * b.inv_dh2 - a1 * b.inv_dh;
            }
        } else if (in_strip(ix, iz, nx, nz, cpml)) {
            // reference ZETA_R (src/parallelcalls.cu:216-243) on dt^2-scaled fields
            const long mi = (long)iz * b.mpitch + sh.x0 + ix;
            const int mpp = b.mpitch;
            using C = Coef<T>;
            const T c2[5] = {C::d2_0, C::d2_1, -C::d2_2, C::d2_3, -C::d2_4};
            T p2cx = c2[0] * b.mh[mi] * lP[i], r2dx = c2[0] * b.mn[mi] * lF[i];
            T p2cz = c2[0] * b.mp[mi] * lP[i], r2cz = c2[0] * b.mp[mi] * lF[i];
            for (int q = 1; q <= 4; q++) {
                p2cx += c2[q] * (b.mh[mi + q] * lP[i + q] + b.mh[mi - q] * lP[i - q]);
                r2dx += c2[q] * (b.mn[mi + q] * lF[i + q] + b.mn[mi - q] * lF[i - q]);
                const long up = i + (long)q * pitch, dn = i - (long)q * pitch;
                const long mup = mi + (long)q * mpp, mdn = mi - (long)q * mpp;
                p2cz += c2[q] * (b.mp[mup] * lP[up] + b.mp[mdn] * lP[dn]);
                r2cz += c2[q] * (b.mp[mup] * lF[up] + b.mp[mdn] * lF[dn]);
            }
            p2cx *= b.inv_dh2; r2dx *= b.inv_dh2; p2cz *= b.inv_dh2; r2cz *= b.inv_dh2;
            const T *psixcx = b.cp[0] + so, *psixcz = b.cp[1] + so, *psizdx = b.cp[2] + so, *psizcz = b.cp[3] + so;
            T *zxcx = b.cp[4] + so, *zxcz = b.cp[5] + so, *zzdx = b.cp[6] + so, *zzcz = b.cp[7] + so;
            const T dxcx = d1_strided(psixcx, i, 1) * b.inv_dh;
            const T dxcz = d1_strided(psixcz, i, pitch) * b.inv_dh;
            const T dzdx = d1_strided(psizdx, i, 1) * b.inv_dh;
            const T dzcz = d1_strided(psizcz, i, pitch) * b.inv_dh;
            const T bx = coef_x(b.cpb, ix, nx, cpml), ax = coef_x(b.cpa, ix, nx, cpml);
            const T bz = coef_z(b.cpb, iz, nz, cpml), az = coef_z(b.cpa, iz, nz, cpml);
            const T n1 = bx * zxcx[i] + ax * (dxcx + p2cx);
            const T n2 = bz * zxcz[i] + az * (dxcz + p2cz);
            const T n3 = bx * zzdx[i] + ax * (dzdx + r2dx);
            const T n4 = bz * zzcz[i] + az * (dzcz + r2cz);
            zxcx[i] = n1; zxcz[i] = n2; zzdx[i] = n3; zzcz[i] = n4;
            ex += (n1 + dxcx) + (n3 + dzdx);
            ez += (n2 + dxcz) + (n4 + dzcz);
        }
        T wp = lPw[i] + ex;
        T wf = lFw[i] + ez;
        if (iz == sh.rz && ix >= sh.rx0 && ix < sh.rx1) {
            const T d = res_row[ix - sh.rx0];
            wp += d;
            wf += d;
        }
        lPw[i] = wp;
        lFw[i] = wf;
        const T pn = lP[i] + wp;
        const T fn = lF[i] + wf;
        lPn[i] = pn;
        lFn[i] = fn;
        if (img) {
            const T G = Cd::dec(img[i], inv_sc), H = Cd::dec(img[b.slot + i], inv_sc);
            const T k = b.img_scale;
            g0[i] += k * G * pn;
            g1[i] += k * H * (pn + fn);
            g2[i] += k * G * fn;
        }
    }
}

// ---------------------------------------------------------------- launchers

template <typename T>
inline dim3 main_grid(const Batch<T> &b, int nx_max)
{
    return dim3((nx_max + PTX - 1) / PTX, (b.nz + PTZ - 1) / PTZ, b.B);
}

template <typename T>
inline dim3 strip_grid(const Batch<T> &b, int nx_max)
{
    const StripMap sm = StripMap::make(nx_max, b.nz, b.cpml);
    long n = sm.count();
    long blocks = (n + kStripBlock - 1) / kStripBlock;
    if (blocks < 1) blocks = 1;
    return dim3((unsigned)blocks, b.B);
}

template <typename T, int ST>
inline void fwd_dispatch(const Batch<T> &b, int nx_max, int g, int ntb, int cur, int slot, bool exact, cudaStream_t st)
{
    if (exact) k_fwd_main<T, ST, true><<<main_grid(b, nx_max), dim3(PTX, PBY), 0, st>>>(b, g, ntb, cur, slot);
    else k_fwd_main<T, ST, false><<<main_grid(b, nx_max), dim3(PTX, PBY), 0, st>>>(b, g, ntb, cur, slot);
}

template <typename T>
void launch_forward_step(const Batch<T> &b, int nx_max, int g, int ntb, int cur, int img_slot,
                         bool exact, const StepStreams &ss)
{
    cudaStream_t st = ss.main;
    k_fwd_strip<T><<<strip_grid(b, nx_max), kStripBlock, 0, st>>>(b, g, ntb, cur);
    switch (b.store_type) {
    case kStoreHalf: fwd_dispatch<T, kStoreHalf>(b, nx_max, g, ntb, cur, img_slot, exact, st); break;
    case kStoreBf16: fwd_dispatch<T, kStoreBf16>(b, nx_max, g, ntb, cur, img_slot, exact, st); break;
    default: fwd_dispatch<T, kStoreNative>(b, nx_max, g, ntb, cur, img_slot, exact, st); break;
    }
}

template <typename T, int ST>
inline void adj_dispatch(const Batch<T> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact,
                         int img_base, cudaStream_t st)
{
    if (exact)
        k_adj_main<T, ST, true><<<main_grid(b, nx_max), dim3(PTX, PBY), 0, st>>>(b, j, ntb, cur, zsel, img_base);
    else
        k_adj_main<T, ST, false><<<main_grid(b, nx_max), dim3(PTX, PBY), 0, st>>>(b, j, ntb, cur, zsel, img_base);
}

template <typename T>
void launch_adjoint_step(const Batch<T> &b, int nx_max, int j, int ntb, int cur, int zsel,
                         bool exact, int img_base, const StepStreams &ss)
{
    cudaStream_t st = ss.main;
    if (exact) k_adj_strip_exact<T><<<strip_grid(b, nx_max), kStripBlock, 0, st>>>(b, j, cur, zsel);
    else k_adj_strip_ref<T><<<strip_grid(b, nx_max), kStripBlock, 0, st>>>(b, j, cur);
    switch (b.store_type) {
    case kStoreHalf: adj_dispatch<T, kStoreHalf>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st); break;
    case kStoreBf16: adj_dispatch<T, kStoreBf16>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st); break;
    default: adj_dispatch<T, kStoreNative>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st); break;
    }
}

}  // namespace fwi
