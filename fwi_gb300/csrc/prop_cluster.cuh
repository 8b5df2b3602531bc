// Small shots resident on chip (FP32, exact adjoint, every step's images
// kept): one thread-block cluster per shot, sm_103a.
//
// A shot whose grid fits the cluster's shared memory (C1: 209 x 209) gains
// nothing from the tile passes' per-step launches: one step of one small shot
// is a few microseconds of work, less than the launch and dependency latency
// of the two tile passes.  Here a cluster of up to 16 CTAs (a non-portable
// cluster size, enabled per kernel) takes one shot through all its time steps
// in a single launch.  CTA k owns the interior rows [4 + k h, 4 + (k + 1) h)
// of the shot's window (h >= 8), every column, and keeps the state of its rows
// in its own shared memory.  After each step's cluster barrier (barrier.cluster:
// hardware, release / acquire over the cluster's shared memory) it copies the
// 8 rows above and below its own of the one field the next step's z-stencils
// need from the neighbours' shared memory (distributed shared memory) and
// recomputes the CPML auxiliary field of the 4 rows either side itself, so
// that a step needs a single cluster barrier.  No other wait exists, and
// every thread of every CTA runs the same number of steps and barriers.
//
// Forward step: copy the 8-row halo of F; psi_x of the band points of the own
// rows, psi_z of the band points of the own rows and 4 either side; zeta, the
// increment update, the next level into the other half of a ping-pong pair,
// receivers, images and the CTA's max of |P|, |F|; barrier; every CTA reads
// all CTAs' maxima (the next step's image scale).  Exact adjoint step: copy
// the 8-row halo of u_z; Y_x of the own band points, Y_z of the band points of
// the own rows and 4 either side; the increment and lambda update, residual
// injection, imaging, and then at once the next step's g, h, Z and fields u
// from the new lambda (into the other half of a ping-pong pair); barrier.
// Both fields the halos come from are double-buffered, so a neighbour's copy
// of step t and the owner's writes of step t + 1 never meet.  The arithmetic
// is the tile passes' (difference-form Laplacian, increment-form leapfrog, the
// same CPML recursions), evaluated in another order: results agree with them
// to FP32 rounding; the recomputed halo values are bit-identical to the
// owner's (same inputs, same operations).
#pragma once

#include <cooperative_groups.h>

#include "prop_tma.cuh"

namespace fwi {

namespace cg = cooperative_groups;

constexpr int kClusterMaxCtas = 16;
constexpr int kClusterThreads = 1024;
constexpr int kClHalo = 2 * kRad;  // halo rows of the copied fields

// CTAs, rows per CTA and shared-memory row pitch of a window nx wide on an nz-row grid, for
// images of elem bytes.  Shared arrays: "haloed" ones carry kClHalo rows above and below the
// own rows, "banded" ones kRad rows (the recomputed CPML fields), the rest only the own rows;
// the CPML coefficients sit in shared tables by column and by banded row.  Each step's images
// pass through a staging area of the own rows (rows of whole 16-byte chunks): the forward
// writes one and copies it out at the start of the next step, the adjoint prefetches into one
// or two (abuf; two when they fit).
struct ClusterPlan {
    int ncta = 0, h = 0, pitch = 0, abuf = 0;
    size_t smem_fwd = 0, smem_adj = 0;
};

// forward: F0 F1 haloed; PSZ banded; P0 P1 PSX VP VF ZX ZZ MH MP MN own; the receiver row
// adjoint: UZ0 UZ1 haloed; YZ banded; LP LF WP WF UX0 UX1 ZX ZZ YX MH MP MN own
constexpr int kClFwdHaloed = 2, kClFwdOwn = 10;
constexpr int kClAdjHaloed = 2, kClAdjOwn = 12;

// floats of the arrays and tables (rounded to 16 bytes), then the image staging
__host__ __device__ inline size_t cluster_floats(int h, int pitch, int haloed, int own, int extra_rows)
{
    const size_t rows = (size_t)haloed * (h + 2 * kClHalo) + (h + 2 * kRad) + (size_t)own * h + extra_rows;
    return (rows * pitch + 2 * (size_t)pitch + 2 * (size_t)(h + 2 * kRad) + 3) / 4 * 4;
}
// elements of a staged image row: whole 16-byte chunks covering nx
__host__ __device__ inline int cluster_img_pitch(int nx, int elem) { return (nx * elem + 15) / 16 * 16 / elem; }

inline bool cluster_plan(int nx, int nz, int elem, size_t smem_limit, ClusterPlan &p)
{
    const int nzi = nz - 8;
    if (nzi < kClHalo || nx < 9) return false;
    // a halo comes from one neighbour only: h >= 8
    p.ncta = nzi / kClHalo < kClusterMaxCtas ? nzi / kClHalo : kClusterMaxCtas;
    p.h = (nzi + p.ncta - 1) / p.ncta;
    p.pitch = (nx + 3) / 4 * 4;
    const size_t stage = (size_t)2 * p.h * cluster_img_pitch(nx, elem) * elem;  // G and H of one step
    p.smem_fwd = sizeof(float) * cluster_floats(p.h, p.pitch, kClFwdHaloed, kClFwdOwn, 1) + stage;
    const size_t adj = sizeof(float) * cluster_floats(p.h, p.pitch, kClAdjHaloed, kClAdjOwn, 0);
    p.abuf = adj + 2 * stage <= smem_limit ? 2 : 1;
    p.smem_adj = adj + p.abuf * stage;
    return p.smem_adj <= smem_limit && p.smem_fwd <= smem_limit;
}

// Geometry of one CTA's rows and the thread's walk over its points: point q = threadIdx.x +
// n blockDim.x of the own rows x interior columns, stepped by carries instead of divisions.
struct ClGeom {
    int k, ncta, h, pitch, nx, nz, iz0, nrows, nxi, npts;
    int dlr, dix;  // blockDim.x = dlr rows + dix columns
    __device__ void init(int k_, int ncta_, int h_, int pitch_, int nx_, int nz_)
    {
        k = k_;
        ncta = ncta_;
        h = h_;
        pitch = pitch_;
        nx = nx_;
        nz = nz_;
        iz0 = 4 + k * h;
        nrows = max(0, min(h, nz - 4 - iz0));
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

// The kClHalo rows above and below the CTA's own of a haloed array (own row r at row
// r + kClHalo) from the neighbours' own rows after a cluster barrier; frame rows read zero.
__device__ __forceinline__ void cl_fill_halo(cg::cluster_group &cl, const ClGeom &g, float *a)
{
    const int p4 = g.pitch / 4, n = 2 * kClHalo * p4;
    const float4 *up = g.k > 0 ? reinterpret_cast<const float4 *>(cl.map_shared_rank(a, g.k - 1)) : nullptr;
    const float4 *down = g.k + 1 < g.ncta ? reinterpret_cast<const float4 *>(cl.map_shared_rank(a, g.k + 1)) : nullptr;
    float4 *a4 = reinterpret_cast<float4 *>(a);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int hr = e / p4, c = e - hr * p4;
        if (hr < kClHalo) {  // global row iz0 - 8 + hr: the upper neighbour's own row h - 8 + hr
            const int iz = g.iz0 - kClHalo + hr;
            a4[hr * p4 + c] = (iz >= 4 && up) ? up[(g.h + hr) * p4 + c] : z;
        } else {  // global row iz0 + h + hr - 8: the lower neighbour's own row hr - 8
            const int iz = g.iz0 + g.h + hr - kClHalo;
            a4[(g.h + hr) * p4 + c] = (iz < g.nz - 4 && down) ? down[hr * p4 + c] : z;
        }
    }
}

// 8th-order derivatives (unnormalised) at c along stride st (1: x, the pitch: z).  Difference
// form for the second derivative, as the tile passes.
__device__ __forceinline__ float cl_d2(const float *c, int st)
{
    using C = Coef<float>;
    const float o = c[0];
    return C::d2_1 * ((c[st] - o) + (c[-st] - o)) - C::d2_2 * ((c[2 * st] - o) + (c[-2 * st] - o)) +
           C::d2_3 * ((c[3 * st] - o) + (c[-3 * st] - o)) - C::d2_4 * ((c[4 * st] - o) + (c[-4 * st] - o));
}
__device__ __forceinline__ float cl_d1(const float *c, int st)
{
    using C = Coef<float>;
    return C::d1_1 * (c[st] - c[-st]) - C::d1_2 * (c[2 * st] - c[-2 * st]) + C::d1_3 * (c[3 * st] - c[-3 * st]) -
           C::d1_4 * (c[4 * st] - c[-4 * st]);
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
template <int N> __device__ __forceinline__ void cl_cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

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
    int r0, npts;
    __device__ ClBand(const ClGeom &g, int zb)
    {
        const int lo = max(max(4, zb), g.iz0 - kRad), hi = min(g.nz - 4, g.iz0 + g.h + kRad);
        r0 = lo - g.iz0;
        npts = hi > lo ? (hi - lo) * g.nxi : 0;
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
k_cluster_fwd(Batch<float> b, int ntb, int h, int pitch, int img)
{
    using Cd = Codec<float, ST>;
    using SI = typename Cd::S;
    extern __shared__ __align__(16) float csm[];
    __shared__ float s_all[2][kClusterMaxCtas];
    cg::cluster_group cl = cg::this_cluster();
    const int ncta = (int)cl.num_blocks();
    const int s = blockIdx.x / ncta;
    const DevShot sh = b.shots[s];
    ClGeom G;
    G.init((int)cl.block_rank(), ncta, h, pitch, sh.nx, b.nz);
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
    SI *const imgb = img ? (SI *)b.store + (long)s * b.n_img * 2 * b.slot : nullptr;
    float amax = 0.f;  // max |P|, |F| after the previous step, over the shot
    float wv_next = sh.nt > 0 ? b.wavelet[0] : 0.f;
    int cur = 0;
    for (int it = 0; it < sh.nt; it++) {
        const int g = it + ntb - sh.nt;
        // the current level and the next (selected, not indexed: no local-memory arrays)
        float *const Pc = cur ? P1 : P0, *const Fc = cur ? F1 : F0;
        float *const Pn = cur ? P0 : P1, *const Fn = cur ? F0 : F1;
        const float wv = wv_next;
        if (it + 1 < sh.nt) wv_next = b.wavelet[it + 1];
        cl_fill_halo(cl, G, Fc);
        // the previous step's images and receiver values, staged, to global memory
        if (it > 0) {
            if (img) cl_stage_copy<SI, true>(b, G, ip, IMG, imgb + (long)(g - 1) * 2 * b.slot);
            if (has_rec)
                for (int t = threadIdx.x; t < nrec; t += blockDim.x)
                    b.rec[sh.rec_off + (long)(it - 1) * nrec + t] = RB[sh.rx0 + t];
        }
        __syncthreads();
        // psi (src/parallelcalls.cu:48-63): x of the side-band points of the own rows ...
        for (int q = threadIdx.x; q < G.nrows * nbx; q += blockDim.x) {
            const int lr = q / nbx, c = q - lr * nbx;
            const int ix = c < nbx / 2 ? 4 + c : nx - 4 - nbx + c;
            const int i = lr * pitch + ix;
            PSX[i] = BX[ix] * PSX[i] + AX[ix] * (cl_d1(Pc + i, 1) * inv_dh);
        }
        // ... z of the bottom-band points of the own rows and 4 either side
        for (int q = threadIdx.x; q < band.npts; q += blockDim.x) {
            const int rr = q / G.nxi, r = band.r0 + rr, ix = 4 + q - rr * G.nxi;
            const int ib = (r + kRad) * pitch + ix, ih = (r + kClHalo) * pitch + ix;
            PSZ[ib] = BZ[r + kRad] * PSZ[ib] + AZ[r + kRad] * (cl_d1(Fc + ih, pitch) * inv_dh);
        }
        __syncthreads();
        const float sc = Cd::scaled ? image_scale(amax, inv_dh2) : 1.f;
        if (img && Cd::scaled && G.k == 0 && threadIdx.x == 0) b.scale[(long)s * b.nt_max + g] = sc;
        float lmax = 0.f;
        bool sat = false;
        for (ClWalk w(G); w.on(); w.next()) {
            const int ix = w.ix, iz = G.iz0 + w.lr, i = w.lr * pitch + ix, ih = (w.lr + kClHalo) * pitch + ix;
            const float gP = cl_d2(Pc + i, 1) * inv_dh2, gF = cl_d2(Fc + ih, pitch) * inv_dh2;
            float Gv = gP, Hv = gF;
            const bool xl = ix < cpml || ix > nx - cpml - 1, zl = iz >= zb;
            if (xl || zl) {
                const int ib = (w.lr + kRad) * pitch + ix;
                const float tx = cl_d1(PSX + i, 1) * inv_dh, tz = cl_d1(PSZ + ib, pitch) * inv_dh;
                float nzx = 0.f, nzz = 0.f;
                if (xl) {
                    nzx = BX[ix] * ZX[i] + AX[ix] * (gP + tx);
                    ZX[i] = nzx;
                }
                if (zl) {
                    nzz = BZ[w.lr + kRad] * ZZ[i] + AZ[w.lr + kRad] * (gF + tz);
                    ZZ[i] = nzz;
                }
                Gv = gP + (tx + nzx);
                Hv = gF + (tz + nzz);
            }
            const float mpH = MP[i] * Hv;
            float vp = VP[i] + (MH[i] * Gv + mpH), vf = VF[i] + (MN[i] * Gv + mpH);
            if (iz == sh.sz && ix == sh.sx) {
                vp += wv;
                vf += wv;
            }
            VP[i] = vp;
            VF[i] = vf;
            const float nP = Pc[i] + vp, nF = Fc[ih] + vf;
            Pn[i] = nP;
            Fn[ih] = nF;
            if (Cd::scaled) lmax = fmaxf(lmax, fmaxf(fabsf(nP), fabsf(nF)));
            if (iz == sh.rz) RB[ix] = nP + nF;
            if (img) {
                IMG[w.lr * ip + ix] = Cd::enc_flag(Gv, sc, sat);
                IMG[(h + w.lr) * ip + ix] = Cd::enc_flag(Hv, sc, sat);
            }
        }
        if (sat) atomicOr(b.status, kStatusSaturated);
        if (Cd::scaled) cl_push_max(cl, G, lmax, s_all[it & 1]);
        cl.sync();  // the new level, and every CTA's max, complete
        if (Cd::scaled) {
            float m = 0.f;
            for (int r = 0; r < G.ncta; r++) m = fmaxf(m, s_all[it & 1][r]);
            amax = m;
            if (G.k == 0 && threadIdx.x == 0) b.amax[(long)s * (b.nt_max + 1) + g + 1] = m;
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
// by the caller).  Each step's images are prefetched into shared memory with cp.async (one
// step ahead when two staging buffers fit); the imaging of a step runs at the start of the
// next one and adds into the gradient with fire-and-forget reductions, so that no global
// memory operation is pending at a cluster barrier.
template <int ST>
__global__ void __launch_bounds__(kClusterThreads, 1)
k_cluster_adj(Batch<float> b, int ntb, int h, int pitch, int abuf)
{
    using Cd = Codec<float, ST>;
    using SI = typename Cd::S;
    extern __shared__ __align__(16) float csm[];
    cg::cluster_group cl = cg::this_cluster();
    const int ncta = (int)cl.num_blocks();
    const int s = blockIdx.x / ncta;
    const DevShot sh = b.shots[s];
    ClGeom G;
    G.init((int)cl.block_rank(), ncta, h, pitch, sh.nx, b.nz);
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
    float *const g0 = b.g[0] + (long)s * b.slot, *const g1 = b.g[1] + (long)s * b.slot,
                 *const g2 = b.g[2] + (long)s * b.slot;
    using C = Coef<float>;
    // band membership of a point (x side layers or the bottom layer)
    auto in_band = [&](int ix, int iz) { return ix < cpml || ix > nx - cpml - 1 || iz >= zb; };
    // imaging of step j from its staged images and lambda of that step (in LP, LF)
    auto imaging = [&](int j, float inv_sc) {
        const SI *const Gs = IMG + (j % abuf) * stage, *const Hs = Gs + (long)h * ip;
        for (ClWalk w(G); w.on(); w.next()) {
            const int i = w.lr * pitch + w.ix, si = w.lr * ip + w.ix;
            const long o = (long)(G.iz0 + w.lr) * b.pitch + w.ix;
            const float lp = LP[i], lf = LF[i];
            const float Gv = Cd::dec(Gs[si], inv_sc), Hv = Cd::dec(Hs[si], inv_sc);
            atomicAdd(g0 + o, kk * Gv * lp);
            atomicAdd(g1 + o, kk * Hv * (lp + lf));
            atomicAdd(g2 + o, kk * Gv * lf);
        }
    };
    float inv_sc_prev = 1.f;  // image scale of the previous step, inverted
    int cur = 0;  // u of this step in UX0 / UZ0 (cur 0) or UX1 / UZ1; zero before the first step
    for (int j = 0; j < sh.nt; j++) {
        const int m = sh.nt - j;
        const int g_img = ntb - 1 - j;  // global step of the image this iteration pairs with
        const float inv_sc = Cd::scaled ? 1.f / b.scale[(long)s * b.nt_max + g_img] : 1.f;
        float *const UXc = cur ? UX1 : UX0, *const UZc = cur ? UZ1 : UZ0;
        float *const UXn = cur ? UX0 : UX1, *const UZn = cur ? UZ0 : UZ1;
        cl_fill_halo(cl, G, UZc);
        if (j > 0) imaging(j - 1, inv_sc_prev);
        __syncthreads();  // the buffer of step j - 1 free again
        prefetch(j + abuf - 1);
        // Y of the band points: Y' = -D(w) + b Y with w = u at band points, 0 elsewhere; x of the
        // side-band points of the own rows ...
        for (int q = threadIdx.x; q < G.nrows * nbx; q += blockDim.x) {
            const int lr = q / nbx, c = q - lr * nbx;
            const int ix = c < nbx / 2 ? 4 + c : nx - 4 - nbx + c, iz = G.iz0 + lr;
            const int i = lr * pitch + ix;
            auto wxv = [&](int dx) {
                const int x2 = ix + dx;
                return (x2 > 3 && x2 < nx - 4 && in_band(x2, iz)) ? UXc[i + dx] : 0.f;
            };
            const float dwx = C::d1_1 * (wxv(1) - wxv(-1)) - C::d1_2 * (wxv(2) - wxv(-2)) +
                              C::d1_3 * (wxv(3) - wxv(-3)) - C::d1_4 * (wxv(4) - wxv(-4));
            YX[i] = -(dwx * inv_dh) + BX[ix] * YX[i];
        }
        // ... z of the bottom-band points of the own rows and 4 either side
        for (int q = threadIdx.x; q < band.npts; q += blockDim.x) {
            const int rr = q / G.nxi, r = band.r0 + rr, ix = 4 + q - rr * G.nxi, iz = G.iz0 + r;
            const int ib = (r + kRad) * pitch + ix, ih = (r + kClHalo) * pitch + ix;
            auto wzv = [&](int dz) {
                const int z2 = iz + dz;
                return (z2 > 3 && z2 < nz - 4 && in_band(ix, z2)) ? UZc[ih + dz * pitch] : 0.f;
            };
            const float dwz = C::d1_1 * (wzv(1) - wzv(-1)) - C::d1_2 * (wzv(2) - wzv(-2)) +
                              C::d1_3 * (wzv(3) - wzv(-3)) - C::d1_4 * (wzv(4) - wzv(-4));
            YZ[ib] = -(dwz * inv_dh) + BZ[r + kRad] * YZ[ib];
        }
        if (abuf == 2) cl_cp_wait<1>();  // this step's images (the next step's may still fly)
        else cl_cp_wait<0>();
        __syncthreads();
        // lambda^m: increments += Dxx(u) - Dx(a Y) (and z), residual at the receivers; then g, h,
        // Z and u of the next step from the new lambda
        for (ClWalk w(G); w.on(); w.next()) {
            const int ix = w.ix, iz = G.iz0 + w.lr, i = w.lr * pitch + ix, ih = (w.lr + kClHalo) * pitch + ix;
            const int rb = w.lr + kRad, ib = rb * pitch + ix;
            const float dxx = cl_d2(UXc + i, 1) * inv_dh2, dzz = cl_d2(UZc + ih, pitch) * inv_dh2;
            float wp, wf;
            if (ix < cpml + 4 || ix > nx - cpml - 5 || iz >= zb - 4) {  // a CPML coefficient within reach
                auto vx = [&](int dx) { return AX[ix + dx] * YX[i + dx]; };
                auto vz = [&](int dz) { return AZ[rb + dz] * YZ[ib + dz * pitch]; };
                const float dvx = C::d1_1 * (vx(1) - vx(-1)) - C::d1_2 * (vx(2) - vx(-2)) +
                                  C::d1_3 * (vx(3) - vx(-3)) - C::d1_4 * (vx(4) - vx(-4));
                const float dvz = C::d1_1 * (vz(1) - vz(-1)) - C::d1_2 * (vz(2) - vz(-2)) +
                                  C::d1_3 * (vz(3) - vz(-3)) - C::d1_4 * (vz(4) - vz(-4));
                wp = WP[i] + (dxx - dvx * inv_dh);
                wf = WF[i] + (dzz - dvz * inv_dh);
            } else {
                wp = WP[i] + dxx;
                wf = WF[i] + dzz;
            }
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
            // u of the next step: g = v_hor lP + v_nmo lF, h = v_po (lP + lF) (dt^2 folded in)
            const float gx = MH[i] * lp + MN[i] * lf, hz = MP[i] * (lp + lf);
            float ux = gx, uzv = hz;
            if (in_band(ix, iz)) {
                const float zx = gx + BX[ix] * ZX[i];
                const float zz = hz + BZ[rb] * ZZ[i];
                ZX[i] = zx;
                ZZ[i] = zz;
                ux = gx + AX[ix] * zx;
                uzv = hz + AZ[rb] * zz;
            }
            UXn[i] = ux;
            UZn[ih] = uzv;
        }
        cl.sync();  // lambda and u of the next step complete in every CTA
        inv_sc_prev = inv_sc;
        cur ^= 1;
    }
    if (sh.nt > 0) imaging(sh.nt - 1, inv_sc_prev);
    cl_cp_wait<0>();  // nothing in flight at exit (an empty group when the prefetch ran past the end)
    cl.sync();  // no CTA leaves while a neighbour may still read its shared memory
}

}  // namespace fwi
