// Small shots resident on chip (FP32, exact adjoint, every step's images
// kept): one thread-block cluster per shot, sm_103a.
//
// A shot whose grid fits the cluster's shared memory (C1: 209 x 209) gains
// nothing from the tile passes' per-step launches: one step of one small shot
// is a few microseconds of work, less than the launch and dependency latency
// of the two tile passes.  Here a cluster of kClusterCtas CTAs (16: a
// non-portable cluster size, enabled per kernel) takes one shot through all
// its time steps in a single launch.  CTA k owns the interior rows
// [4 + k h, 4 + (k + 1) h) of the shot's window, every column, and keeps the
// state of its rows in its own shared memory; the stencils read the 4 rows
// beyond its own from the neighbouring CTAs' shared memory (distributed
// shared memory, map_shared_rank), and the phases of a step are separated by
// cluster barriers (barrier.cluster: hardware, with release / acquire
// semantics over the cluster's shared memory).  No other wait exists, and
// every thread of every CTA runs the same number of steps and barriers.
//
// Forward step (2 barriers): psi of the band points from the current level;
// barrier; everything else (zeta, the increment update, the next level into
// the other half of a ping-pong pair, receivers, images) and the CTA's max of
// |P|, |F|; barrier; every CTA reads all CTAs' maxima (the next step's image
// scale).  Exact adjoint step (3 barriers): g, h, Z and the fields u of the
// Laplacian terms; barrier; Y of the band points from the neighbours' u;
// barrier; the increment and lambda update, residual injection and imaging;
// barrier.  The arithmetic is the tile passes' (difference-form Laplacian,
// increment-form leapfrog, the same CPML recursions), evaluated in another
// order: results agree with them to FP32 rounding.
#pragma once

#include <cooperative_groups.h>

#include "prop_tma.cuh"

namespace fwi {

namespace cg = cooperative_groups;

constexpr int kClusterCtas = 16;
constexpr int kClusterThreads = 1024;
constexpr int kClusterFwdArrays = 13;  // P0 P1 F0 F1 PSX PSZ VP VF ZX ZZ MH MP MN
constexpr int kClusterAdjArrays = 16;  // LP LF WP WF UX UZ ZX ZZ YX YZ MH MP MN GH GP GN

// Rows per CTA and shared-memory row pitch of a window nx wide on an nz-row grid.
struct ClusterPlan {
    int h = 0, pitch = 0;
    size_t smem_fwd = 0, smem_adj = 0;
};

inline bool cluster_plan(int nx, int nz, size_t smem_limit, ClusterPlan &p)
{
    const int nzi = nz - 8;
    if (nzi <= 0 || nx < 9) return false;
    p.h = (nzi + kClusterCtas - 1) / kClusterCtas;
    p.pitch = (nx + 3) / 4 * 4;
    p.smem_fwd = sizeof(float) * (size_t)kClusterFwdArrays * p.h * p.pitch + 64;
    p.smem_adj = sizeof(float) * (size_t)kClusterAdjArrays * p.h * p.pitch + 64;
    // the z-stencils reach 4 rows: one neighbour on either side
    return p.h >= kRad && p.smem_adj <= smem_limit && p.smem_fwd <= smem_limit;
}

// Rows of one shared array: this CTA's own, and the neighbours' above and below.
struct ClRows {
    float *own;
    const float *up, *down;
    int h, pitch, k, nz;
    // value at own-relative row lr (-4 .. h + 3), column ix; zero on the frame rows
    __device__ __forceinline__ float at(int lr, int ix) const
    {
        const int iz = 4 + k * h + lr;
        if (iz < 4 || iz >= nz - 4) return 0.f;
        if (lr < 0) return up[(lr + h) * pitch + ix];
        if (lr >= h) return down[(lr - h) * pitch + ix];
        return own[lr * pitch + ix];
    }
};

__device__ __forceinline__ ClRows cl_rows(cg::cluster_group &cl, float *own, int h, int pitch, int k, int ncta, int nz)
{
    ClRows r;
    r.own = own;
    r.up = k > 0 ? cl.map_shared_rank(own, k - 1) : own;
    r.down = k + 1 < ncta ? cl.map_shared_rank(own, k + 1) : own;
    r.h = h;
    r.pitch = pitch;
    r.k = k;
    r.nz = nz;
    return r;
}

// 8th-order derivatives (unnormalised) at (lr, ix): along x from the CTA's own row, along z
// through ClRows.  Difference form for the second derivative, as the tile passes.
__device__ __forceinline__ float cl_d2x(const float *row, int ix)
{
    using C = Coef<float>;
    const float o = row[ix];
    return C::d2_1 * ((row[ix + 1] - o) + (row[ix - 1] - o)) - C::d2_2 * ((row[ix + 2] - o) + (row[ix - 2] - o)) +
           C::d2_3 * ((row[ix + 3] - o) + (row[ix - 3] - o)) - C::d2_4 * ((row[ix + 4] - o) + (row[ix - 4] - o));
}
__device__ __forceinline__ float cl_d1x(const float *row, int ix)
{
    using C = Coef<float>;
    return C::d1_1 * (row[ix + 1] - row[ix - 1]) - C::d1_2 * (row[ix + 2] - row[ix - 2]) +
           C::d1_3 * (row[ix + 3] - row[ix - 3]) - C::d1_4 * (row[ix + 4] - row[ix - 4]);
}
__device__ __forceinline__ float cl_d2z(const ClRows &a, int lr, int ix)
{
    using C = Coef<float>;
    const float o = a.at(lr, ix);
    return C::d2_1 * ((a.at(lr + 1, ix) - o) + (a.at(lr - 1, ix) - o)) -
           C::d2_2 * ((a.at(lr + 2, ix) - o) + (a.at(lr - 2, ix) - o)) +
           C::d2_3 * ((a.at(lr + 3, ix) - o) + (a.at(lr - 3, ix) - o)) -
           C::d2_4 * ((a.at(lr + 4, ix) - o) + (a.at(lr - 4, ix) - o));
}
__device__ __forceinline__ float cl_d1z(const ClRows &a, int lr, int ix)
{
    using C = Coef<float>;
    return C::d1_1 * (a.at(lr + 1, ix) - a.at(lr - 1, ix)) - C::d1_2 * (a.at(lr + 2, ix) - a.at(lr - 2, ix)) +
           C::d1_3 * (a.at(lr + 3, ix) - a.at(lr - 3, ix)) - C::d1_4 * (a.at(lr + 4, ix) - a.at(lr - 4, ix));
}

// CPML coefficient of column ix / row iz of an nx x nz window (0 outside the layers).
__device__ __forceinline__ float cl_coef_x(const float *tab, int ix, int nx, int cpml)
{
    return ix < cpml ? tab[cpml - ix] : ix > nx - cpml - 1 ? tab[ix - nx + cpml + 1] : 0.f;
}
__device__ __forceinline__ float cl_coef_z(const float *tab, int iz, int nz, int cpml)
{
    return iz > nz - cpml - 1 ? tab[iz - nz + cpml + 1] : 0.f;
}

// Max over the CTA into *slot (values >= 0).
__device__ __forceinline__ void cl_block_max(float v, float *slot)
{
    __shared__ float wm[kClusterThreads / 32];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, wm[w]);
        *slot = m;
    }
}

// Forward of shot blockIdx.x / kClusterCtas of the batch through all its steps (global steps
// ntb - nt .. ntb - 1); every step's images (img != 0) to slot g of the image store.
template <int ST>
__global__ void __launch_bounds__(kClusterThreads, 1)
k_cluster_fwd(Batch<float> b, int ntb, int h, int pitch, int img)
{
    using Cd = Codec<float, ST>;
    using SI = typename Cd::S;
    extern __shared__ __align__(16) float csm[];
    __shared__ float s_max;
    cg::cluster_group cl = cg::this_cluster();
    const int k = (int)cl.block_rank(), ncta = (int)cl.num_blocks();
    const int s = blockIdx.x / ncta;
    const DevShot sh = b.shots[s];
    const int nx = sh.nx, nz = b.nz, cpml = b.cpml;
    const size_t plane = (size_t)h * pitch;
    float *const P0 = csm, *const P1 = csm + plane, *const F0 = csm + 2 * plane, *const F1 = csm + 3 * plane;
    float *PSX = csm + 4 * plane, *PSZ = csm + 5 * plane, *VP = csm + 6 * plane, *VF = csm + 7 * plane;
    float *ZX = csm + 8 * plane, *ZZ = csm + 9 * plane, *MH = csm + 10 * plane, *MP = csm + 11 * plane,
          *MN = csm + 12 * plane;
    const int iz0 = 4 + k * h;
    const int nrows = max(0, min(h, nz - 4 - iz0));  // own interior rows
    const int nxi = nx - 8, npts = nrows * nxi;
    for (size_t i = threadIdx.x; i < (size_t)kClusterFwdArrays * plane; i += blockDim.x) csm[i] = 0.f;
    __syncthreads();
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
        const int lr = q / nxi, ix = 4 + q - lr * nxi;
        const long mi = (long)(iz0 + lr) * b.mpitch + sh.x0 + ix;
        MH[lr * pitch + ix] = b.mh[mi];
        MP[lr * pitch + ix] = b.mp[mi];
        MN[lr * pitch + ix] = b.mn[mi];
    }
    if (threadIdx.x == 0) s_max = 0.f;
    cl.sync();  // every CTA's state zeroed before any neighbour reads it
    const ClRows fz0 = cl_rows(cl, F0, h, pitch, k, ncta, nz), fz1 = cl_rows(cl, F1, h, pitch, k, ncta, nz);
    const ClRows psz = cl_rows(cl, PSZ, h, pitch, k, ncta, nz);
    const float inv_dh = b.inv_dh, inv_dh2 = b.inv_dh2;
    const int nrec = sh.rx1 - sh.rx0;
    float amax = 0.f;  // max |P|, |F| after the previous step, over the shot
    int cur = 0;
    for (int it = 0; it < sh.nt; it++) {
        const int g = it + ntb - sh.nt;
        // the current level and the next (selected, not indexed: no local-memory arrays)
        float *const Pc = cur ? P1 : P0, *const Fc = cur ? F1 : F0;
        float *const Pn = cur ? P0 : P1, *const Fn = cur ? F0 : F1;
        const ClRows fzc = cur ? fz1 : fz0;
        // psi of the band points from the current level (src/parallelcalls.cu:48-63)
        for (int q = threadIdx.x; q < npts; q += blockDim.x) {
            const int lr = q / nxi, ix = 4 + q - lr * nxi, iz = iz0 + lr, i = lr * pitch + ix;
            if (!layer_point(ix, iz, nx, nz, cpml)) continue;
            if (ix < cpml || ix > nx - cpml - 1)
                PSX[i] = cl_coef_x(b.cpb, ix, nx, cpml) * PSX[i] +
                         cl_coef_x(b.cpa, ix, nx, cpml) * (cl_d1x(Pc + lr * pitch, ix) * inv_dh);
            if (iz > nz - cpml - 1)
                PSZ[i] = cl_coef_z(b.cpb, iz, nz, cpml) * PSZ[i] +
                         cl_coef_z(b.cpa, iz, nz, cpml) * (cl_d1z(fzc, lr, ix) * inv_dh);
        }
        cl.sync();
        const float sc = Cd::scaled ? image_scale(amax, inv_dh2) : 1.f;
        if (img && Cd::scaled && k == 0 && threadIdx.x == 0) b.scale[(long)s * b.nt_max + g] = sc;
        const float w = b.wavelet[it];
        SI *imgp = img ? (SI *)b.store + ((long)s * b.n_img + g) * 2 * b.slot : nullptr;
        float lmax = 0.f;
        bool sat = false;
        for (int q = threadIdx.x; q < npts; q += blockDim.x) {
            const int lr = q / nxi, ix = 4 + q - lr * nxi, iz = iz0 + lr, i = lr * pitch + ix;
            const float *prow = Pc + lr * pitch;
            const float gP = cl_d2x(prow, ix) * inv_dh2, gF = cl_d2z(fzc, lr, ix) * inv_dh2;
            float G = gP, H = gF;
            if (layer_point(ix, iz, nx, nz, cpml)) {
                const float tx = cl_d1x(PSX + lr * pitch, ix) * inv_dh, tz = cl_d1z(psz, lr, ix) * inv_dh;
                float nzx = 0.f, nzz = 0.f;
                if (ix < cpml || ix > nx - cpml - 1) {
                    nzx = cl_coef_x(b.cpb, ix, nx, cpml) * ZX[i] + cl_coef_x(b.cpa, ix, nx, cpml) * (gP + tx);
                    ZX[i] = nzx;
                }
                if (iz > nz - cpml - 1) {
                    nzz = cl_coef_z(b.cpb, iz, nz, cpml) * ZZ[i] + cl_coef_z(b.cpa, iz, nz, cpml) * (gF + tz);
                    ZZ[i] = nzz;
                }
                G = gP + (tx + nzx);
                H = gF + (tz + nzz);
            }
            const float mpH = MP[i] * H;
            float vp = VP[i] + (MH[i] * G + mpH), vf = VF[i] + (MN[i] * G + mpH);
            if (iz == sh.sz && ix == sh.sx) {
                vp += w;
                vf += w;
            }
            VP[i] = vp;
            VF[i] = vf;
            const float nP = prow[ix] + vp, nF = Fc[i] + vf;
            Pn[i] = nP;
            Fn[i] = nF;
            if (Cd::scaled) lmax = fmaxf(lmax, fmaxf(fabsf(nP), fabsf(nF)));
            if (iz == sh.rz && ix >= sh.rx0 && ix < sh.rx1)
                b.rec[sh.rec_off + (long)it * nrec + ix - sh.rx0] = nP + nF;
            if (img) {
                const long o = (long)iz * b.pitch + ix;
                imgp[o] = Cd::enc_flag(G, sc, sat);
                imgp[b.slot + o] = Cd::enc_flag(H, sc, sat);
            }
        }
        if (sat) atomicOr(b.status, kStatusSaturated);
        if (Cd::scaled) cl_block_max(lmax, &s_max);
        cl.sync();  // the new level, and every CTA's max, complete
        if (Cd::scaled) {
            float m = 0.f;
            for (int r = 0; r < ncta; r++) m = fmaxf(m, *cl.map_shared_rank(&s_max, r));
            amax = m;
            if (k == 0 && threadIdx.x == 0) b.amax[(long)s * (b.nt_max + 1) + g + 1] = m;
        }
        cur ^= 1;
    }
    cl.sync();  // no CTA leaves while a neighbour may still read its shared memory
}

// Exact adjoint of shot blockIdx.x / kClusterCtas with imaging from the image store (slot of
// each global step), the residual in b.rec; the shot's gradient to its slot s of b.g.
template <int ST>
__global__ void __launch_bounds__(kClusterThreads, 1) k_cluster_adj(Batch<float> b, int ntb, int h, int pitch)
{
    using Cd = Codec<float, ST>;
    using SI = typename Cd::S;
    extern __shared__ __align__(16) float csm[];
    cg::cluster_group cl = cg::this_cluster();
    const int k = (int)cl.block_rank(), ncta = (int)cl.num_blocks();
    const int s = blockIdx.x / ncta;
    const DevShot sh = b.shots[s];
    const int nx = sh.nx, nz = b.nz, cpml = b.cpml;
    const size_t plane = (size_t)h * pitch;
    float *LP = csm, *LF = csm + plane, *WP = csm + 2 * plane, *WF = csm + 3 * plane;
    float *UX = csm + 4 * plane, *UZ = csm + 5 * plane, *ZX = csm + 6 * plane, *ZZ = csm + 7 * plane;
    float *YX = csm + 8 * plane, *YZ = csm + 9 * plane, *MH = csm + 10 * plane, *MP = csm + 11 * plane,
          *MN = csm + 12 * plane, *GH = csm + 13 * plane, *GP = csm + 14 * plane, *GN = csm + 15 * plane;
    const int iz0 = 4 + k * h;
    const int nrows = max(0, min(h, nz - 4 - iz0));
    const int nxi = nx - 8, npts = nrows * nxi;
    for (size_t i = threadIdx.x; i < (size_t)kClusterAdjArrays * plane; i += blockDim.x) csm[i] = 0.f;
    __syncthreads();
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
        const int lr = q / nxi, ix = 4 + q - lr * nxi;
        const long mi = (long)(iz0 + lr) * b.mpitch + sh.x0 + ix;
        MH[lr * pitch + ix] = b.mh[mi];
        MP[lr * pitch + ix] = b.mp[mi];
        MN[lr * pitch + ix] = b.mn[mi];
    }
    cl.sync();
    const ClRows uz = cl_rows(cl, UZ, h, pitch, k, ncta, nz), yz = cl_rows(cl, YZ, h, pitch, k, ncta, nz);
    const float inv_dh = b.inv_dh, inv_dh2 = b.inv_dh2, kk = b.img_scale;
    const int nrec = sh.rx1 - sh.rx0;
    for (int j = 0; j < sh.nt; j++) {
        const int m = sh.nt - j;
        const int g_img = ntb - 1 - j;  // global step of the image this iteration pairs with
        // g = dt^2 (v_hor lP + v_nmo lF), h = dt^2 v_po (lP + lF); Z and the fields u of the Laplacian terms
        for (int q = threadIdx.x; q < npts; q += blockDim.x) {
            const int lr = q / nxi, ix = 4 + q - lr * nxi, iz = iz0 + lr, i = lr * pitch + ix;
            const float lp = LP[i], lf = LF[i];
            const float gx = MH[i] * lp + MN[i] * lf, hz = MP[i] * (lp + lf);
            float ux = gx, uzv = hz;
            if (layer_point(ix, iz, nx, nz, cpml)) {
                const float zx = gx + cl_coef_x(b.cpb, ix, nx, cpml) * ZX[i];
                const float zz = hz + cl_coef_z(b.cpb, iz, nz, cpml) * ZZ[i];
                ZX[i] = zx;
                ZZ[i] = zz;
                ux = gx + cl_coef_x(b.cpa, ix, nx, cpml) * zx;
                uzv = hz + cl_coef_z(b.cpa, iz, nz, cpml) * zz;
            }
            UX[i] = ux;
            UZ[i] = uzv;
        }
        cl.sync();
        // Y of the band points: Yx' = -Dx(wx) + bx Yx with wx = u at band points, 0 elsewhere
        for (int q = threadIdx.x; q < npts; q += blockDim.x) {
            const int lr = q / nxi, ix = 4 + q - lr * nxi, iz = iz0 + lr, i = lr * pitch + ix;
            if (!layer_point(ix, iz, nx, nz, cpml)) continue;
            using C = Coef<float>;
            auto wxv = [&](int dx) {
                const int x2 = ix + dx;
                return (x2 > 3 && x2 < nx - 4 && layer_point(x2, iz, nx, nz, cpml)) ? UX[lr * pitch + x2] : 0.f;
            };
            auto wzv = [&](int dz) {
                const int z2 = iz + dz;
                return (z2 > 3 && z2 < nz - 4 && layer_point(ix, z2, nx, nz, cpml)) ? uz.at(lr + dz, ix) : 0.f;
            };
            const float dwx = C::d1_1 * (wxv(1) - wxv(-1)) - C::d1_2 * (wxv(2) - wxv(-2)) +
                              C::d1_3 * (wxv(3) - wxv(-3)) - C::d1_4 * (wxv(4) - wxv(-4));
            const float dwz = C::d1_1 * (wzv(1) - wzv(-1)) - C::d1_2 * (wzv(2) - wzv(-2)) +
                              C::d1_3 * (wzv(3) - wzv(-3)) - C::d1_4 * (wzv(4) - wzv(-4));
            YX[i] = -(dwx * inv_dh) + cl_coef_x(b.cpb, ix, nx, cpml) * YX[i];
            YZ[i] = -(dwz * inv_dh) + cl_coef_z(b.cpb, iz, nz, cpml) * YZ[i];
        }
        cl.sync();
        // lambda^m: increments += Dxx(u) - Dx(a Y) (and z), residual at the receivers; imaging
        float inv_sc = 1.f;
        if (Cd::scaled) inv_sc = 1.f / b.scale[(long)s * b.nt_max + g_img];
        const SI *imgp = (const SI *)b.store + ((long)s * b.n_img + g_img) * 2 * b.slot;
        for (int q = threadIdx.x; q < npts; q += blockDim.x) {
            const int lr = q / nxi, ix = 4 + q - lr * nxi, iz = iz0 + lr, i = lr * pitch + ix;
            using C = Coef<float>;
            const float *urow = UX + lr * pitch, *yrow = YX + lr * pitch;
            auto vx = [&](int dx) { return cl_coef_x(b.cpa, ix + dx, nx, cpml) * yrow[ix + dx]; };
            auto vz = [&](int dz) { return cl_coef_z(b.cpa, iz + dz, nz, cpml) * yz.at(lr + dz, ix); };
            const float dvx = C::d1_1 * (vx(1) - vx(-1)) - C::d1_2 * (vx(2) - vx(-2)) + C::d1_3 * (vx(3) - vx(-3)) -
                              C::d1_4 * (vx(4) - vx(-4));
            const float dvz = C::d1_1 * (vz(1) - vz(-1)) - C::d1_2 * (vz(2) - vz(-2)) + C::d1_3 * (vz(3) - vz(-3)) -
                              C::d1_4 * (vz(4) - vz(-4));
            float wp = WP[i] + (cl_d2x(urow, ix) * inv_dh2 - dvx * inv_dh);
            float wf = WF[i] + (cl_d2z(uz, lr, ix) * inv_dh2 - dvz * inv_dh);
            if (iz == sh.rz && ix >= sh.rx0 && ix < sh.rx1) {
                const float d = b.rec[sh.rec_off + (long)(m - 1) * nrec + ix - sh.rx0];
                wp += d;
                wf += d;
            }
            WP[i] = wp;
            WF[i] = wf;
            const float lp = LP[i] + wp, lf = LF[i] + wf;
            LP[i] = lp;
            LF[i] = lf;
            const long o = (long)iz * b.pitch + ix;
            const float Gv = Cd::dec(imgp[o], inv_sc), Hv = Cd::dec(imgp[b.slot + o], inv_sc);
            GH[i] += kk * Gv * lp;
            GP[i] += kk * Hv * (lp + lf);
            GN[i] += kk * Gv * lf;
        }
        cl.sync();  // u and Y of this step read by every neighbour before the next step rewrites them
    }
    // the shot's gradient to its own slot
    const long so = (long)s * b.slot;
    for (int q = threadIdx.x; q < npts; q += blockDim.x) {
        const int lr = q / nxi, ix = 4 + q - lr * nxi, iz = iz0 + lr, i = lr * pitch + ix;
        const long o = so + (long)iz * b.pitch + ix;
        b.g[0][o] = GH[i];
        b.g[1][o] = GP[i];
        b.g[2][o] = GN[i];
    }
}

}  // namespace fwi
