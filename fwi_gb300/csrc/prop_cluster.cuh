// Small shots resident on chip (FP32, exact adjoint, every step's images
// kept): one thread-block cluster per shot, sm_103a.
//
// A shot whose grid fits the cluster's shared memory (e.g. 209 x 209) gains
// nothing from the tile passes' per-step launches: one step of one small shot
// is a few microseconds of work, less than the launch and dependency latency
// of the two tile passes.  Here a cluster of up to 16 CTAs (a non-portable
// cluster size, enabled per kernel) takes one shot through all its time steps
// in a single launch.  CTA k owns a band of interior rows of the shot's window
// (at least 8; the partition balances a cost model of the CPML work, so the
// CTAs at the bottom layer hold fewer rows), every column, and keeps the state
// of its rows in its own shared memory.  The one field the next step's
// z-stencils need from other CTAs is written, for the 8 rows next to each
// edge, straight into the neighbours' halo rows as it is computed (stores to
// distributed shared memory), and each CTA recomputes the CPML auxiliary field
// of the 4 rows either side of its own itself, so that a step needs a single
// cluster barrier (barrier.cluster: hardware, release / acquire over the
// cluster's shared memory) and no copy.  No other wait exists, and every
// thread of every CTA runs the same number of steps and barriers.
//
// Forward step: the previous step's staged images and receiver values out to
// global memory; psi_x of the band points of the own rows, psi_z of the band
// points of the own rows and 4 either side; zeta, the increment update, the
// next level into the other half of a ping-pong pair (and the neighbours'
// halos), receivers and images into shared staging, the CTA's max of |P|,
// |F| pushed to every CTA; barrier; the next step's image scale from the
// maxima.  Exact adjoint step: the next step's images prefetched (cp.async);
// Y_x of the own band points, Y_z of the band points of the own rows and 4
// either side; the increment and lambda update, residual injection, imaging
// (reductions into the gradient, fire-and-forget), and then at once the next
// step's g, h, Z and fields u from the new lambda (into the other half of a
// ping-pong pair, and the neighbours' halos); barrier.  Both fields with halos
// are double-buffered, so that a neighbour's write of step t + 1 never meets
// the owner's reads of step t.  Global stores and reductions are issued early
// in a step or spread over it, not at its end, so that the barrier's release
// seldom waits for them.  The arithmetic is the tile passes' (difference-form
// Laplacian, increment-form leapfrog, the same CPML recursions), evaluated in
// another order: results agree with them to FP32 rounding; the recomputed
// CPML rows are bit-identical to the owner's (same inputs, same operations).
#pragma once

#include <cooperative_groups.h>

#include "cluster_plan.h"
#include "prop_tma.cuh"

namespace fwi {

namespace cg = cooperative_groups;

// Geometry of one CTA and its walk: point q = threadIdx.x + n blockDim.x of the own rows x
// interior columns, stepped by carries instead of divisions.
struct ClGeom {
    int k, ncta, h, pitch, nx, nz, iz0, nrows, nup, nxi, npts;
    int dlr, dix;  // blockDim.x = dlr rows + dix columns
    __device__ void init(int k_, int ncta_, int h_, int pitch_, int nx_, int nz_, const ClRows &rows)
    {
        k = k_;
        ncta = ncta_;
        h = h_;
        pitch = pitch_;
        nx = nx_;
        nz = nz_;
        iz0 = 4 + rows.start[k];
        nrows = rows.start[k + 1] - rows.start[k];
        nup = k > 0 ? rows.start[k] - rows.start[k - 1] : 0;
        nxi = nx - 8;
        npts = nrows * nxi;
        dlr = (int)blockDim.x / nxi;
        dix = (int)blockDim.x - dlr * nxi;
    }
};

// Each thread's walk: for (ClWalk w(g); w.on(); w.next()) { w.lr, w.ix }
struct ClWalk {
    int q, lr, ix;
    const ClGeom &g;
    __device__ explicit ClWalk(const ClGeom &g_) : g(g_)
    {
        q = threadIdx.x;
        lr = q / g.nxi;
        ix = 4 + q - lr * g.nxi;
    }
    __device__ bool on() const { return q < g.npts; }
    __device__ void next()
    {
        q += blockDim.x;
        lr += g.dlr;
        ix += g.dix;
        if (ix >= g.nx - 4) {
            ix -= g.nxi;
            lr++;
        }
    }
};

// 8th-order derivatives (unnormalised) from the centre o and the values k = 1..4 points after
// (pk) and before (mk).  Difference form for the second derivative, as the tile passes.  Every
// stencil of this file goes through these two, so that the scalar and the 4-column forms give
// the same results.
__device__ __forceinline__ float cl_d2v(float o, float p1, float m1, float p2, float m2, float p3, float m3, float p4,
                                        float m4)
{
    using C = Coef<float>;
    return C::d2_1 * ((p1 - o) + (m1 - o)) - C::d2_2 * ((p2 - o) + (m2 - o)) + C::d2_3 * ((p3 - o) + (m3 - o)) -
           C::d2_4 * ((p4 - o) + (m4 - o));
}
__device__ __forceinline__ float cl_d1v(float p1, float m1, float p2, float m2, float p3, float m3, float p4, float m4)
{
    using C = Coef<float>;
    return C::d1_1 * (p1 - m1) - C::d1_2 * (p2 - m2) + C::d1_3 * (p3 - m3) - C::d1_4 * (p4 - m4);
}
// the same at c along stride st (1: x, the pitch: z)
__device__ __forceinline__ float cl_d2(const float *c, int st)
{
    return cl_d2v(c[0], c[st], c[-st], c[2 * st], c[-2 * st], c[3 * st], c[-3 * st], c[4 * st], c[-4 * st]);
}
__device__ __forceinline__ float cl_d1(const float *c, int st)
{
    return cl_d1v(c[st], c[-st], c[2 * st], c[-2 * st], c[3 * st], c[-3 * st], c[4 * st], c[-4 * st]);
}

// Four consecutive floats (16-byte aligned) to and from registers.
__device__ __forceinline__ void cl_ld4(float (&v)[4], const float *p)
{
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
}
__device__ __forceinline__ void cl_st4(float *p, const float (&v)[4])
{
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
// x window of 12 values around the 4 columns at p (p[-4] .. p[7])
__device__ __forceinline__ void cl_ld12(float (&w)[12], const float *p)
{
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float4 t = *reinterpret_cast<const float4 *>(p - 4 + 4 * c);
        w[4 * c] = t.x;
        w[4 * c + 1] = t.y;
        w[4 * c + 2] = t.z;
        w[4 * c + 3] = t.w;
    }
}
// derivatives of column j (0..3) of a window (centre w[4 + j])
__device__ __forceinline__ float cl_d2w(const float (&w)[12], int j)
{
    return cl_d2v(w[4 + j], w[5 + j], w[3 + j], w[6 + j], w[2 + j], w[7 + j], w[1 + j], w[8 + j], w[j]);
}
__device__ __forceinline__ float cl_d1w(const float (&w)[12], int j)
{
    return cl_d1v(w[5 + j], w[3 + j], w[6 + j], w[2 + j], w[7 + j], w[1 + j], w[8 + j], w[j]);
}
// z derivatives of 4 columns at p (stride the pitch), into d[0..3]
__device__ __forceinline__ void cl_d2z4(float (&d)[4], const float *p, int st)
{
    float o[4], a[4], b2[4], c[4], e[4], f[4], g[4], h[4], k[4];
    cl_ld4(o, p);
    cl_ld4(a, p + st);
    cl_ld4(b2, p - st);
    cl_ld4(c, p + 2 * st);
    cl_ld4(e, p - 2 * st);
    cl_ld4(f, p + 3 * st);
    cl_ld4(g, p - 3 * st);
    cl_ld4(h, p + 4 * st);
    cl_ld4(k, p - 4 * st);
#pragma unroll
    for (int j = 0; j < 4; j++) d[j] = cl_d2v(o[j], a[j], b2[j], c[j], e[j], f[j], g[j], h[j], k[j]);
}
__device__ __forceinline__ void cl_d1z4(float (&d)[4], const float *p, int st)
{
    float a[4], b2[4], c[4], e[4], f[4], g[4], h[4], k[4];
    cl_ld4(a, p + st);
    cl_ld4(b2, p - st);
    cl_ld4(c, p + 2 * st);
    cl_ld4(e, p - 2 * st);
    cl_ld4(f, p + 3 * st);
    cl_ld4(g, p - 3 * st);
    cl_ld4(h, p + 4 * st);
    cl_ld4(k, p - 4 * st);
#pragma unroll
    for (int j = 0; j < 4; j++) d[j] = cl_d1v(a[j], b2[j], c[j], e[j], f[j], g[j], h[j], k[j]);
}

// Four image values to a 16-byte-or-8-byte aligned staging slot.
__device__ __forceinline__ void cl_st4_img(float *p, float a, float b, float c, float d)
{
    *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}
template <typename S> __device__ __forceinline__ void cl_st4_img(S *p, S a, S b, S c, S d)
{
    static_assert(sizeof(S) == 2, "2-byte image type");
    unsigned short u[4];
    memcpy(&u[0], &a, 2);
    memcpy(&u[1], &b, 2);
    memcpy(&u[2], &c, 2);
    memcpy(&u[3], &d, 2);
    *reinterpret_cast<uint2 *>(p) = make_uint2(u[0] | ((uint32_t)u[1] << 16), u[2] | ((uint32_t)u[3] << 16));
}
// Four image values from a staging slot.
__device__ __forceinline__ void cl_ld4_img(float (&v)[4], const float *p) { cl_ld4(v, p); }
template <typename S> __device__ __forceinline__ void cl_ld4_img(S (&v)[4], const S *p)
{
    static_assert(sizeof(S) == 2, "2-byte image type");
    const uint2 t = *reinterpret_cast<const uint2 *>(p);
    const unsigned short u[4] = {(unsigned short)(t.x & 0xffffu), (unsigned short)(t.x >> 16),
                                 (unsigned short)(t.y & 0xffffu), (unsigned short)(t.y >> 16)};
#pragma unroll
    for (int j = 0; j < 4; j++) memcpy(&v[j], &u[j], 2);
}

// CPML coefficient tables of the CTA: by column (0 outside the side layers) and by banded row
// (row r of the table: global row iz0 - 4 + r; 0 outside the bottom layer).
__device__ __forceinline__ void cl_tables(const Batch<float> &b, const ClGeom &g, float *ax, float *bx, float *az,
                                          float *bz)
{
    const int cp = b.cpml;
    for (int ix = threadIdx.x; ix < g.pitch; ix += blockDim.x) {
        const int d = ix >= g.nx ? 0 : ix < cp ? cp - ix : ix > g.nx - cp - 1 ? ix - g.nx + cp + 1 : 0;
        ax[ix] = d ? b.cpa[d] : 0.f;
        bx[ix] = d ? b.cpb[d] : 0.f;
    }
    for (int r = threadIdx.x; r < g.h + 2 * kRad; r += blockDim.x) {
        const int iz = g.iz0 - kRad + r;
        const int d = (iz > g.nz - cp - 1 && iz < g.nz) ? iz - g.nz + cp + 1 : 0;
        az[r] = d ? b.cpa[d] : 0.f;
        bz[r] = d ? b.cpb[d] : 0.f;
    }
}

// 16-byte copies global -> shared that complete asynchronously (cp.async, waited with
// cp.async.wait_group: a hardware wait, no polling)
__device__ __forceinline__ void cl_cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cl_cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cl_cp_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Max over the CTA of v >= 0, pushed by thread 0 into slot k of every CTA's table (no remote
// read after the barrier: each CTA reduces its own copy).
__device__ __forceinline__ void cl_push_max(cg::cluster_group &cl, const ClGeom &g, float v, float *table)
{
    __shared__ float wm[kClusterThreads / 32];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if ((int)threadIdx.x < g.ncta) *cl.map_shared_rank(table + g.k, (int)threadIdx.x) = v;
    }
}

// The banded rows of the CTA in z-band (bottom layer) that lie inside the interior: rows
// r in [-4, h + 4) with global row iz0 + r in [max(4, zb), nz - 4); walked as r0 + q / nxi.
struct ClBand {
    int r0, nrows, npts;
    __device__ ClBand(const ClGeom &g, int zb)
    {
        const int lo = max(max(4, zb), g.iz0 - kRad), hi = min(g.nz - 4, g.iz0 + g.nrows + kRad);
        r0 = lo - g.iz0;
        nrows = hi > lo ? hi - lo : 0;
        npts = nrows * g.nxi;
    }
};

// Staged images of one step (own rows, G then H, rows of ip elements) <-> the image store:
// the 16-byte chunks of the CTA, one per thread and pass.  to_store: generic stores; else
// cp.async loads (the caller commits and waits).
template <typename SI, bool to_store>
__device__ __forceinline__ void cl_stage_copy(const Batch<float> &b, const ClGeom &g, int ip, SI *stage, SI *imgp)
{
    const int nch = ip * (int)sizeof(SI) / 16, per = g.nrows * nch, n = 2 * per;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int arr = e >= per, r = e - arr * per, lr = r / nch, c = r - lr * nch;
        uint4 *sp = reinterpret_cast<uint4 *>(stage + ((long)arr * g.h + lr) * ip) + c;
        uint4 *gp = reinterpret_cast<uint4 *>(imgp + arr * b.slot + (long)(g.iz0 + lr) * b.pitch) + c;
        if (to_store)
            *gp = *sp;
        else
            cl_cp_async16(sp, gp);
    }
}

// Forward of shot blockIdx.x / ncta of the batch through all its steps (global steps ntb - nt
// .. ntb - 1); every step's images (img != 0) to slot g of the image store.  Global stores of a
// step (images, receivers) are staged in shared memory and issued at the start of the next
// step, so that they are complete long before the release of the next cluster barrier.
template <int ST>
__global__ void __launch_bounds__(kClusterThreads, 1)
k_cluster_fwd(Batch<float> b, const __grid_constant__ ClRows rows, int ntb, int h, int pitch, int img)
{
    using Cd = Codec<float, ST>;
    using SI = typename Cd::S;
    extern __shared__ __align__(16) float csm[];
    __shared__ float s_all[2][kClusterMaxCtas];
    __shared__ float s_sc;  // the next step's image scale, from every CTA's max (thread 0 computes it)
    cg::cluster_group cl = cg::this_cluster();
    const int ncta = (int)cl.num_blocks();
    const int s = blockIdx.x / ncta;
    const DevShot sh = b.shots[s];
    ClGeom G;
    G.init((int)cl.block_rank(), ncta, h, pitch, sh.nx, b.nz, rows);
    const int nx = sh.nx, nz = b.nz, cpml = b.cpml;
    const size_t hp = (size_t)(h + 2 * kClHalo) * pitch, bp = (size_t)(h + 2 * kRad) * pitch,
                 op = (size_t)h * pitch;
    float *const F0 = csm, *const F1 = csm + hp, *const PSZ = csm + 2 * hp;
    float *const base = PSZ + bp;
    float *const P0 = base, *const P1 = base + op, *const PSX = base + 2 * op, *const VP = base + 3 * op,
                 *const VF = base + 4 * op, *const ZX = base + 5 * op, *const ZZ = base + 6 * op,
                 *const MH = base + 7 * op, *const MP = base + 8 * op, *const MN = base + 9 * op;
    float *const RB = base + 10 * op;  // the receiver row (own rows holding it)
    float *const AX = RB + pitch, *const BX = AX + pitch, *const AZ = BX + pitch, *const BZ = AZ + h + 2 * kRad;
    const size_t nfl = cluster_floats(h, pitch, kClFwdHaloed, kClFwdOwn, 1);
    const int ip = cluster_img_pitch(nx, (int)sizeof(SI));
    SI *const IMG = reinterpret_cast<SI *>(csm + nfl);
    const size_t stage_words = (size_t)2 * h * ip * sizeof(SI) / 4;
    for (size_t i = threadIdx.x; i < nfl + stage_words; i += blockDim.x) csm[i] = 0.f;
    __syncthreads();
    cl_tables(b, G, AX, BX, AZ, BZ);
    for (ClWalk w(G); w.on(); w.next()) {
        const long mi = (long)(G.iz0 + w.lr) * b.mpitch + sh.x0 + w.ix;
        const int i = w.lr * pitch + w.ix;
        MH[i] = b.mh[mi];
        MP[i] = b.mp[mi];
        MN[i] = b.mn[mi];
    }
    cl.sync();  // every CTA's state zeroed before any neighbour reads it
    const float inv_dh = b.inv_dh, inv_dh2 = b.inv_dh2;
    const int nrec = sh.rx1 - sh.rx0;
    const bool has_rec = sh.rz >= G.iz0 && sh.rz < G.iz0 + G.nrows;
    const int zb = nz - cpml;  // first row of the bottom layer
    const ClBand band(G, zb);
    const int nbx = cpml > 4 ? min(2 * (cpml - 4), G.nxi) : 0;  // side-band columns of a row
    const int nq = (G.nxi + 3) / 4;                               // groups of 4 columns of a row
    SI *const imgb = img ? (SI *)b.store + (long)s * b.n_img * 2 * b.slot : nullptr;
    if (threadIdx.x == 0) s_sc = Cd::scaled ? image_scale(0.f, b.inv_dh2) : 1.f;  // read after the psi barrier
    float wv_next = sh.nt > 0 ? b.wavelet[0] : 0.f;
    int cur = 0;
    for (int it = 0; it < sh.nt; it++) {
        const int g = it + ntb - sh.nt;
        // the current level and the next (selected, not indexed: no local-memory arrays)
        float *const Pc = cur ? P1 : P0, *const Fc = cur ? F1 : F0;
        float *const Pn = cur ? P0 : P1, *const Fn = cur ? F0 : F1;
        // the neighbours' copies of the next level's rows next to this CTA's (their halo rows)
        float *const Fn_up = G.k > 0 ? cl.map_shared_rank(Fn, G.k - 1) : nullptr;
        float *const Fn_dn = G.k + 1 < G.ncta ? cl.map_shared_rank(Fn, G.k + 1) : nullptr;
        const float wv = wv_next;
        if (it + 1 < sh.nt) wv_next = b.wavelet[it + 1];
        // the previous step's images and receiver values, staged, to global memory (the staging
        // area is rewritten only after the barrier that ends phase A)
        if (it > 0) {
            if (img) cl_stage_copy<SI, true>(b, G, ip, IMG, imgb + (long)(g - 1) * 2 * b.slot);
            if (has_rec)
                for (int t = threadIdx.x; t < nrec; t += blockDim.x)
                    b.rec[sh.rec_off + (long)(it - 1) * nrec + t] = RB[sh.rx0 + t];
        }
        // psi (src/parallelcalls.cu:48-63): x of the side-band points of the own rows ...
        for (int q = threadIdx.x; q < G.nrows * nbx; q += blockDim.x) {
            const int lr = q / nbx, c = q - lr * nbx;
            const int ix = c < nbx / 2 ? 4 + c : nx - 4 - nbx + c;
            const int i = lr * pitch + ix;
            PSX[i] = BX[ix] * PSX[i] + AX[ix] * (cl_d1(Pc + i, 1) * inv_dh);
        }
        // ... z of the bottom-band points of the own rows and 4 either side, 4 columns a thread
        for (int q = threadIdx.x; q < band.nrows * nq; q += blockDim.x) {
            const int rr = q / nq, r = band.r0 + rr, ix = 4 + 4 * (q - rr * nq);
            const int ib = (r + kRad) * pitch + ix, ih = (r + kClHalo) * pitch + ix;
            const int nval = min(4, nx - 4 - ix);  // columns inside the interior
            float d[4], ps[4];
            cl_d1z4(d, Fc + ih, pitch);
            cl_ld4(ps, PSZ + ib);
            const float bz = BZ[r + kRad], az = AZ[r + kRad];
#pragma unroll
            for (int j = 0; j < 4; j++) ps[j] = j < nval ? bz * ps[j] + az * (d[j] * inv_dh) : 0.f;
            cl_st4(PSZ + ib, ps);
        }
        __syncthreads();
        const float sc = Cd::scaled ? s_sc : 1.f;
        if (img && Cd::scaled && G.k == 0 && threadIdx.x == 0) b.scale[(long)s * b.nt_max + g] = sc;
        float lmax = 0.f;
        bool sat = false;
        // 4 columns a thread (16-byte shared loads and stores; the last group of a row may reach
        // the frame, whose values stay zero)
        for (int q = threadIdx.x; q < G.nrows * nq; q += blockDim.x) {
            const int lr = q / nq, ix = 4 + 4 * (q - lr * nq), iz = G.iz0 + lr;
            const int i = lr * pitch + ix, ih = (lr + kClHalo) * pitch + ix, rb = lr + kRad;
            const int nval = min(4, nx - 4 - ix);
            float pw[12], gP[4], gF[4], Gv[4], Hv[4];
            cl_ld12(pw, Pc + i);
            cl_d2z4(gF, Fc + ih, pitch);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                gP[j] = cl_d2w(pw, j) * inv_dh2;
                gF[j] *= inv_dh2;
                Gv[j] = gP[j];
                Hv[j] = gF[j];
            }
            const bool zl = iz >= zb;
            if (zl || ix < cpml || ix + 3 > nx - cpml - 1) {  // a point of the CPML layers
                // psi_x is zero beyond 4 columns of the side bands, psi_z above 4 rows of the bottom
                float tx[4] = {0.f, 0.f, 0.f, 0.f}, tz[4] = {0.f, 0.f, 0.f, 0.f};
                if (ix < cpml + 4 || ix + 3 > nx - cpml - 5) {
                    float sw[12];
                    cl_ld12(sw, PSX + i);
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (ix + j < cpml + 4 || ix + j > nx - cpml - 5) tx[j] = cl_d1w(sw, j) * inv_dh;
                }
                if (iz >= zb - 4) {
                    cl_d1z4(tz, PSZ + rb * pitch + ix, pitch);
#pragma unroll
                    for (int j = 0; j < 4; j++) tz[j] *= inv_dh;
                }
                float zx[4], zz[4], ax[4], bx[4];
                cl_ld4(zx, ZX + i);
                cl_ld4(zz, ZZ + i);
                cl_ld4(ax, AX + ix);
                cl_ld4(bx, BX + ix);
                const float az = AZ[rb], bz = BZ[rb];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const bool xl = ix + j < cpml || ix + j > nx - cpml - 1;
                    if (j < nval && (xl || zl)) {
                        float nzx = 0.f, nzz = 0.f;
                        if (xl) {
                            nzx = bx[j] * zx[j] + ax[j] * (gP[j] + tx[j]);
                            zx[j] = nzx;
                        }
                        if (zl) {
                            nzz = bz * zz[j] + az * (gF[j] + tz[j]);
                            zz[j] = nzz;
                        }
                        Gv[j] = gP[j] + (tx[j] + nzx);
                        Hv[j] = gF[j] + (tz[j] + nzz);
                    }
                }
                cl_st4(ZX + i, zx);
                cl_st4(ZZ + i, zz);
            }
            float mh[4], mp[4], mn[4], vp[4], vf[4], fc[4], nP[4], nF[4];
            cl_ld4(fc, Fc + ih);
            cl_ld4(mh, MH + i);
            cl_ld4(mp, MP + i);
            cl_ld4(mn, MN + i);
            cl_ld4(vp, VP + i);
            cl_ld4(vf, VF + i);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float mpH = mp[j] * Hv[j];
                vp[j] = vp[j] + (mh[j] * Gv[j] + mpH);
                vf[j] = vf[j] + (mn[j] * Gv[j] + mpH);
                if (iz == sh.sz && ix + j == sh.sx) {
                    vp[j] += wv;
                    vf[j] += wv;
                }
                nP[j] = pw[4 + j] + vp[j];
                nF[j] = fc[j] + vf[j];
                if (j >= nval) vp[j] = vf[j] = nP[j] = nF[j] = Gv[j] = Hv[j] = 0.f;
                if (Cd::scaled) lmax = fmaxf(lmax, fmaxf(fabsf(nP[j]), fabsf(nF[j])));
            }
            cl_st4(VP + i, vp);
            cl_st4(VF + i, vf);
            cl_st4(Pn + i, nP);
            cl_st4(Fn + ih, nF);
            // rows within 8 of the CTA's edges into the neighbours' halo rows
            if (lr < kClHalo && Fn_up) cl_st4(Fn_up + (G.nup + kClHalo + lr) * pitch + ix, nF);
            if (lr >= G.nrows - kClHalo && Fn_dn) cl_st4(Fn_dn + (lr - G.nrows + kClHalo) * pitch + ix, nF);
            if (iz == sh.rz) {
                const float r4[4] = {nP[0] + nF[0], nP[1] + nF[1], nP[2] + nF[2], nP[3] + nF[3]};
                cl_st4(RB + ix, r4);
            }
            if (img) {
                cl_st4_img(IMG + lr * ip + ix, Cd::enc_flag(Gv[0], sc, sat), Cd::enc_flag(Gv[1], sc, sat),
                           Cd::enc_flag(Gv[2], sc, sat), Cd::enc_flag(Gv[3], sc, sat));
                cl_st4_img(IMG + (h + lr) * ip + ix, Cd::enc_flag(Hv[0], sc, sat), Cd::enc_flag(Hv[1], sc, sat),
                           Cd::enc_flag(Hv[2], sc, sat), Cd::enc_flag(Hv[3], sc, sat));
            }
        }
        if (sat) atomicOr(b.status, kStatusSaturated);
        if (Cd::scaled) cl_push_max(cl, G, lmax, s_all[it & 1]);
        cl.sync();  // the new level, and every CTA's max, complete
        if (Cd::scaled && threadIdx.x == 0) {  // read by every thread after the next step's psi barrier
            float m = 0.f;
            for (int r = 0; r < G.ncta; r++) m = fmaxf(m, s_all[it & 1][r]);
            s_sc = image_scale(m, inv_dh2);
            if (G.k == 0) b.amax[(long)s * (b.nt_max + 1) + g + 1] = m;
        }
        cur ^= 1;
    }
    if (sh.nt > 0) {  // the last step's staged images and receiver values
        if (img) cl_stage_copy<SI, true>(b, G, ip, IMG, imgb + (long)(ntb - 1) * 2 * b.slot);
        if (has_rec)
            for (int t = threadIdx.x; t < nrec; t += blockDim.x)
                b.rec[sh.rec_off + (long)(sh.nt - 1) * nrec + t] = RB[sh.rx0 + t];
    }
    cl.sync();  // no CTA leaves while a neighbour may still read its shared memory
}

// Exact adjoint of shot blockIdx.x / ncta with imaging from the image store (slot of each
// global step), the residual in b.rec; the shot's gradient added into its slot s of b.g (zeroed
// by the caller) with reductions.  Each step's images are prefetched into shared memory with
// cp.async (one step ahead when two staging buffers fit).
template <int ST>
__global__ void __launch_bounds__(kClusterThreads, 1)
k_cluster_adj(Batch<float> b, const __grid_constant__ ClRows rows, int ntb, int h, int pitch, int abuf)
{
    using Cd = Codec<float, ST>;
    using SI = typename Cd::S;
    extern __shared__ __align__(16) float csm[];
    cg::cluster_group cl = cg::this_cluster();
    const int ncta = (int)cl.num_blocks();
    const int s = blockIdx.x / ncta;
    const DevShot sh = b.shots[s];
    ClGeom G;
    G.init((int)cl.block_rank(), ncta, h, pitch, sh.nx, b.nz, rows);
    const int nx = sh.nx, nz = b.nz, cpml = b.cpml;
    const size_t hp = (size_t)(h + 2 * kClHalo) * pitch, bp = (size_t)(h + 2 * kRad) * pitch,
                 op = (size_t)h * pitch;
    float *const UZ0 = csm, *const UZ1 = csm + hp, *const YZ = csm + 2 * hp;
    float *const base = YZ + bp;
    float *const LP = base, *const LF = base + op, *const WP = base + 2 * op, *const WF = base + 3 * op,
                 *const UX0 = base + 4 * op, *const UX1 = base + 5 * op, *const ZX = base + 6 * op,
                 *const ZZ = base + 7 * op, *const YX = base + 8 * op, *const MH = base + 9 * op,
                 *const MP = base + 10 * op, *const MN = base + 11 * op;
    float *const AX = base + 12 * op, *const BX = AX + pitch, *const AZ = BX + pitch, *const BZ = AZ + h + 2 * kRad;
    const size_t nfl = cluster_floats(h, pitch, kClAdjHaloed, kClAdjOwn, 0);
    const int ip = cluster_img_pitch(nx, (int)sizeof(SI));
    const long stage = (long)2 * h * ip;  // elements of one staging buffer
    SI *const IMG = reinterpret_cast<SI *>(csm + nfl);
    for (size_t i = threadIdx.x; i < nfl; i += blockDim.x) csm[i] = 0.f;
    __syncthreads();
    cl_tables(b, G, AX, BX, AZ, BZ);
    for (ClWalk w(G); w.on(); w.next()) {
        const long mi = (long)(G.iz0 + w.lr) * b.mpitch + sh.x0 + w.ix;
        const int i = w.lr * pitch + w.ix;
        MH[i] = b.mh[mi];
        MP[i] = b.mp[mi];
        MN[i] = b.mn[mi];
    }
    const SI *const imgb = (const SI *)b.store + (long)s * b.n_img * 2 * b.slot;
    // the image of adjoint step j (global step ntb - 1 - j) into buffer j % abuf
    auto prefetch = [&](int j) {
        if (j < sh.nt)
            cl_stage_copy<SI, false>(b, G, ip, IMG + (j % abuf) * stage,
                                     const_cast<SI *>(imgb) + (long)(ntb - 1 - j) * 2 * b.slot);
        cl_cp_commit();
    };
    if (abuf == 2) prefetch(0);
    cl.sync();
    const float inv_dh = b.inv_dh, inv_dh2 = b.inv_dh2, kk = b.img_scale;
    const int nrec = sh.rx1 - sh.rx0;
    const int zb = nz - cpml;
    const ClBand band(G, zb);
    const int nbx = cpml > 4 ? min(2 * (cpml - 4), G.nxi) : 0;
    const int nq = (G.nxi + 3) / 4;
    float *const g0 = b.g[0] + (long)s * b.slot, *const g1 = b.g[1] + (long)s * b.slot,
                 *const g2 = b.g[2] + (long)s * b.slot;
    using C = Coef<float>;
    // band membership of a point (x side layers or the bottom layer)
    auto in_band = [&](int ix, int iz) { return ix < cpml || ix > nx - cpml - 1 || iz >= zb; };
    int cur = 0;  // u of this step in UX0 / UZ0 (cur 0) or UX1 / UZ1; zero before the first step
    for (int j = 0; j < sh.nt; j++) {
        const int m = sh.nt - j;
        const int g_img = ntb - 1 - j;  // global step of the image this iteration pairs with
        const float inv_sc = Cd::scaled ? 1.f / b.scale[(long)s * b.nt_max + g_img] : 1.f;
        float *const UXc = cur ? UX1 : UX0, *const UZc = cur ? UZ1 : UZ0;
        float *const UXn = cur ? UX0 : UX1, *const UZn = cur ? UZ0 : UZ1;
        float *const UZn_up = G.k > 0 ? cl.map_shared_rank(UZn, G.k - 1) : nullptr;
        float *const UZn_dn = G.k + 1 < G.ncta ? cl.map_shared_rank(UZn, G.k + 1) : nullptr;
        // the next staging buffer was last read by the previous step's phase C
        prefetch(j + abuf - 1);
        // Y of the band points: Y' = -D(w) + b Y with w = u at band points, 0 elsewhere; x of the
        // side-band points of the own rows ...
        for (int q = threadIdx.x; q < G.nrows * nbx; q += blockDim.x) {
            const int lr = q / nbx, c = q - lr * nbx;
            const int ix = c < nbx / 2 ? 4 + c : nx - 4 - nbx + c, iz = G.iz0 + lr;
            const int i = lr * pitch + ix;
            float dwx;
            if (iz >= zb || ix < cpml - 4 || ix > nx - cpml + 3) {  // every tap a band point (or frame, 0)
                dwx = cl_d1(UXc + i, 1);
            } else {
                auto wxv = [&](int dx) {
                    const int x2 = ix + dx;
                    return (x2 < cpml || x2 > nx - cpml - 1) ? UXc[i + dx] : 0.f;
                };
                dwx = cl_d1v(wxv(1), wxv(-1), wxv(2), wxv(-2), wxv(3), wxv(-3), wxv(4), wxv(-4));
            }
            YX[i] = -(dwx * inv_dh) + BX[ix] * YX[i];
        }
        // ... z of the bottom-band points of the own rows and 4 either side, 4 columns a thread
        for (int q = threadIdx.x; q < band.nrows * nq; q += blockDim.x) {
            const int rr = q / nq, r = band.r0 + rr, ix = 4 + 4 * (q - rr * nq), iz = G.iz0 + r;
            const int ib = (r + kRad) * pitch + ix, ih = (r + kClHalo) * pitch + ix;
            const int nval = min(4, nx - 4 - ix);
            float dwz[4], yz[4];
            if (iz >= zb + 4) {  // every tap a band point (or frame, 0)
                cl_d1z4(dwz, UZc + ih, pitch);
            } else {  // taps above the bottom layer count only in the side layers
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const bool side = ix + j < cpml || ix + j > nx - cpml - 1;
                    auto wzv = [&](int dz) { return (side || iz + dz >= zb) ? UZc[ih + dz * pitch + j] : 0.f; };
                    dwz[j] = cl_d1v(wzv(1), wzv(-1), wzv(2), wzv(-2), wzv(3), wzv(-3), wzv(4), wzv(-4));
                }
            }
            cl_ld4(yz, YZ + ib);
            const float bz = BZ[r + kRad];
#pragma unroll
            for (int j = 0; j < 4; j++) yz[j] = j < nval ? -(dwz[j] * inv_dh) + bz * yz[j] : 0.f;
            cl_st4(YZ + ib, yz);
        }
        if (abuf == 2) cl_cp_wait<1>();  // this step's images (the next step's may still fly)
        else cl_cp_wait<0>();
        __syncthreads();
        const SI *const Gs = IMG + (j % abuf) * stage, *const Hs = Gs + (long)h * ip;
        // lambda^m: increments += Dxx(u) - Dx(a Y) (and z), residual at the receivers; then g, h,
        // Z and u of the next step from the new lambda
        for (int q = threadIdx.x; q < G.nrows * nq; q += blockDim.x) {
            const int lr = q / nq, ix = 4 + 4 * (q - lr * nq), iz = G.iz0 + lr;
            const int i = lr * pitch + ix, ih = (lr + kClHalo) * pitch + ix, rb = lr + kRad, ib = rb * pitch + ix;
            const int nval = min(4, nx - 4 - ix);
            float uw[12], dxx[4], dzz[4], wp[4], wf[4];
            cl_ld12(uw, UXc + i);
            cl_d2z4(dzz, UZc + ih, pitch);
            cl_ld4(wp, WP + i);
            cl_ld4(wf, WF + i);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                dxx[j] = cl_d2w(uw, j) * inv_dh2;
                dzz[j] *= inv_dh2;
            }
            // a Y . a term only within reach of a CPML coefficient (a = 0 outside the layers)
            float dvx[4] = {0.f, 0.f, 0.f, 0.f}, dvz[4] = {0.f, 0.f, 0.f, 0.f};
            if (ix < cpml + 4 || ix + 3 > nx - cpml - 5) {
                float aw[12], yw[12];
                cl_ld12(aw, AX + ix);
                cl_ld12(yw, YX + i);
#pragma unroll
                for (int c = 0; c < 12; c++) yw[c] *= aw[c];
#pragma unroll
                for (int j = 0; j < 4; j++) dvx[j] = cl_d1w(yw, j);
            }
            if (iz >= zb - 4) {
                float yv[9][4];
#pragma unroll
                for (int dz = -4; dz <= 4; dz++) {
                    cl_ld4(yv[dz + 4], YZ + ib + dz * pitch);
                    const float a = AZ[rb + dz];
#pragma unroll
                    for (int j = 0; j < 4; j++) yv[dz + 4][j] *= a;
                }
#pragma unroll
                for (int j = 0; j < 4; j++)
                    dvz[j] = cl_d1v(yv[5][j], yv[3][j], yv[6][j], yv[2][j], yv[7][j], yv[1][j], yv[8][j], yv[0][j]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c = ix + j;
                wp[j] = (c < cpml + 4 || c > nx - cpml - 5) ? wp[j] + (dxx[j] - dvx[j] * inv_dh) : wp[j] + dxx[j];
                wf[j] = iz >= zb - 4 ? wf[j] + (dzz[j] - dvz[j] * inv_dh) : wf[j] + dzz[j];
                if (iz == sh.rz && c >= sh.rx0 && c < sh.rx1) {
                    const float d = b.rec[sh.rec_off + (long)(m - 1) * nrec + c - sh.rx0];
                    wp[j] += d;
                    wf[j] += d;
                }
            }
            float lp[4], lf[4], gi[4], hi[4];
            cl_ld4(lp, LP + i);
            cl_ld4(lf, LF + i);
            {
                SI gs[4], hs[4];
                cl_ld4_img(gs, Gs + lr * ip + ix);
                cl_ld4_img(hs, Hs + lr * ip + ix);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    gi[j] = Cd::dec(gs[j], inv_sc);
                    hi[j] = Cd::dec(hs[j], inv_sc);
                }
            }
            float a0[4], a1[4], a2[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (j >= nval) wp[j] = wf[j] = 0.f;
                lp[j] = lp[j] + wp[j];
                lf[j] = lf[j] + wf[j];
                // imaging
                a0[j] = kk * gi[j] * lp[j];
                a1[j] = kk * hi[j] * (lp[j] + lf[j]);
                a2[j] = kk * gi[j] * lf[j];
            }
            cl_st4(WP + i, wp);
            cl_st4(WF + i, wf);
            cl_st4(LP + i, lp);
            cl_st4(LF + i, lf);
            const long o = (long)iz * b.pitch + ix;  // 16-byte aligned: the pitch is a multiple of 32
            atomicAdd(reinterpret_cast<float4 *>(g0 + o), make_float4(a0[0], a0[1], a0[2], a0[3]));
            atomicAdd(reinterpret_cast<float4 *>(g1 + o), make_float4(a1[0], a1[1], a1[2], a1[3]));
            atomicAdd(reinterpret_cast<float4 *>(g2 + o), make_float4(a2[0], a2[1], a2[2], a2[3]));
            // u of the next step: g = v_hor lP + v_nmo lF, h = v_po (lP + lF) (dt^2 folded in)
            float mh[4], mp[4], mn[4], ux[4], uz[4];
            cl_ld4(mh, MH + i);
            cl_ld4(mp, MP + i);
            cl_ld4(mn, MN + i);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                ux[j] = mh[j] * lp[j] + mn[j] * lf[j];
                uz[j] = mp[j] * (lp[j] + lf[j]);
            }
            if (iz >= zb || ix < cpml || ix + 3 > nx - cpml - 1) {
                float zx[4], zz[4], ax[4], bx[4];
                cl_ld4(zx, ZX + i);
                cl_ld4(zz, ZZ + i);
                cl_ld4(ax, AX + ix);
                cl_ld4(bx, BX + ix);
                const float az = AZ[rb], bz = BZ[rb];
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (j < nval && in_band(ix + j, iz)) {
                        const float gx = ux[j], hz = uz[j];
                        zx[j] = gx + bx[j] * zx[j];
                        zz[j] = hz + bz * zz[j];
                        ux[j] = gx + ax[j] * zx[j];
                        uz[j] = hz + az * zz[j];
                    }
                cl_st4(ZX + i, zx);
                cl_st4(ZZ + i, zz);
            }
            cl_st4(UXn + i, ux);
            cl_st4(UZn + ih, uz);
            if (lr < kClHalo && UZn_up) cl_st4(UZn_up + (G.nup + kClHalo + lr) * pitch + ix, uz);
            if (lr >= G.nrows - kClHalo && UZn_dn) cl_st4(UZn_dn + (lr - G.nrows + kClHalo) * pitch + ix, uz);
        }
        cl.sync();  // lambda and u of the next step complete in every CTA
        cur ^= 1;
    }
    cl_cp_wait<0>();  // nothing in flight at exit (an empty group when the prefetch ran past the end)
    cl.sync();  // no CTA leaves while a neighbour may still read its shared memory
}

}  // namespace fwi
