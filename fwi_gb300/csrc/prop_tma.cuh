// FP32 main passes (sm_103a): TMA tile loads, shot groups, 4-wide vectors.
//
// A 32 x 32 tile block loops over a group of shots (one window, or several:
// the MIXED instantiations).  Each shot's halo'd fields arrive by
// cp.async.bulk.tensor into one of kStages shared-memory stages while the
// block computes earlier shots (mbarrier pipeline, one issuing thread; every
// thread waits for its stage itself and the block meets where the stage is
// handed back, stage_release); the increments and images, read at each
// thread's own 4 points, are loaded into registers before the stage wait.  A
// thread owns 4 consecutive points of a row: the x-stencil is 3
// ld.shared.v4, the z-stencil 9, stores are 16-byte vectors.  The adjoint
// sums the imaging of a one-window group in registers (one gradient
// read-modify-write per group and step); a group of several windows adds
// each shot's imaging to its own slot.
//
// These kernels take the interior tiles (tile_role 1: no point the CPML
// layers touch); prop_layer.cuh takes the layer tiles.
#pragma once

#include "prop.cuh"
#include "tma.cuh"

namespace fwi {

constexpr int TT = kTileEdge;      // tile edge
constexpr int TH = TT + 2 * kRad;  // tile with a 4-point halo on every side (40)
constexpr int kTmaThreads = 256;   // 8 threads x 4 points per row, 32 rows
constexpr int kMaxGroup = 64;

// Tensor maps over one batch's per-shot arrays ([B][nz][pitch]).
struct TmaMaps {
    CUtensorMap lvl[4];  // P level 0/1, F level 0/1: 40 x 40 boxes
    CUtensorMap px[2];   // P level 0/1: 40 x 32 boxes (x-halo)
    CUtensorMap fz[2];   // F level 0/1: 32 x 40 boxes (z-halo)
    CUtensorMap mx[8];   // CPML memory variables cp[k]: 40 x 32 boxes (x-halo)
    CUtensorMap mz[8];   // the same, 32 x 40 boxes (z-halo)
    CUtensorMap inc[2];  // P and F increments (levels 4, 5): 32 x 32 boxes, no halo
};

// Only the fields read with a halo are staged; the increments and images,
// read at each thread's own 4 points, are loaded straight into registers.
// The forward operator takes Dxx of P and Dzz of F only: each is staged with
// the halo along its own axis.
struct FwdStage {
    float P[TT][TH];
    float F[TH][TT];
};

// The forward interior tiles also stage the tile's P and F increments (the
// thread's own points, no halo), so that every state read of a shot is an
// asynchronous copy issued kStages shots ahead.
struct FwdIncStage {
    float P[TT][TH];
    float F[TH][TT];
    float VP[TT][TT];
    float VF[TT][TT];
};

struct AdjStage {
    float P[TH][TH];
    float F[TH][TH];
};

// The adjoint interior tiles also stage the tile's lambda increments (own points, no halo).
struct AdjIncStage {
    float P[TH][TH];
    float F[TH][TH];
    float WP[TT][TT];
    float WF[TT][TT];
};

constexpr int kStages = 3;     // TMA pipeline depth over a group's shots (forward interior tiles)
constexpr int kAdjStages = 2;  // adjoint interior tiles: 2 stages keep 3 blocks on an SM

__device__ __forceinline__ unsigned char *aligned_dsm(unsigned char *p)
{
    const uint32_t a = smem_addr(p);
    return p + ((128u - (a & 127u)) & 127u);
}

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ float comp(const float4 &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }

// Bounded wait whose outcome every thread of the block agrees on.  Thread 0
// polls; the other threads sleep in the barrier and then observe the
// completed phase themselves with one more try_wait (which returns at once),
// so that the staged data is visible to each of them.
__device__ __forceinline__ bool stage_ready(uint64_t *bar, unsigned parity, unsigned *status)
{
    bool ok = true;
    if (threadIdx.x == 0) ok = mbar_wait(bar, parity);
    const bool any_fail = __syncthreads_or(!ok);
    if (any_fail) {
        if (threadIdx.x == 0) atomicOr(status, kStatusTimeout);
        return false;
    }
    if (threadIdx.x != 0) (void)mbar_wait(bar, parity);
    return true;
}

// After a failed wait at shot a: give the loads still in flight (shots a + 1
// .. a + nst - 1 of an nst-stage pipeline) a bounded time to land before the
// block's shared memory is released.
__device__ __forceinline__ void drain_stages_n(uint64_t *bar, int a, int na, int nst)
{
    if (threadIdx.x == 0)
        for (int k = a + 1; k < min(a + nst, na); k++) (void)mbar_wait(&bar[k % nst], (k / nst) & 1);
    __syncthreads();
}
__device__ __forceinline__ void drain_stages(uint64_t *bar, int a, int na) { drain_stages_n(bar, a, na, kStages); }

// The interior passes' pipeline: every thread waits for its stage itself
// (mbar_wait: try_wait suspends the thread in hardware, no block barrier),
// and the block meets once, at the end of the iteration, where the stage is
// handed back for its refill.  stage_release: that meeting, agreeing on
// whether any thread's wait gave up in this iteration (a thread that gave up
// skips the stage's work); then the status bit, the loads in flight (shots
// a + 1 .. a + nst - 1) get a bounded time to land, and false.
__device__ __forceinline__ bool stage_release(bool ok, uint64_t *bar, int a, int na, int nst, unsigned *status)
{
    if (!__syncthreads_or(!ok)) return true;
    if (threadIdx.x == 0) {
        atomicOr(status, kStatusTimeout);
        for (int k = a + 1; k < min(a + nst, na); k++) (void)mbar_wait(&bar[k % nst], (k / nst) & 1);
    }
    __syncthreads();
    return false;
}

// The shots of this block's group that run at this step; with aw > 0 (a
// group of several windows), only those for which the tile at (x0, z0) is an
// interior tile (tile_role 1 for width aw) of their own window.
__device__ __forceinline__ int active_shots(const Batch<float> &b, int sg, int *act, bool adjoint, int step, int ntb,
                                            int x0 = 0, int z0 = 0, int aw = 0)
{
    __shared__ int n_s;
    if (threadIdx.x == 0) {
        const int s0 = blockIdx.z * sg, s1 = min(s0 + sg, b.B);
        int n = 0;
        for (int s = s0; s < s1; s++) {
            const DevShot &d = b.shots[s];
            if (!(adjoint ? (step < d.nt) : (step - (ntb - d.nt) >= 0))) continue;
            if (aw > 0 && tile_role(x0, z0, d.nx, b.nz, aw) != 1) continue;
            act[n++] = s;
        }
        n_s = n;
    }
    __syncthreads();
    return n_s;
}

// 8th-order second derivative (unnormalised, difference form) of 4
// consecutive points from 12 values v[0..11] = f(ix0 - 4 .. ix0 + 7).
__device__ __forceinline__ float d2_row(const float *v, int q)
{
    using C = Coef<float>;
    const float o = v[4 + q];
    return C::d2_1 * ((v[5 + q] - o) + (v[3 + q] - o)) - C::d2_2 * ((v[6 + q] - o) + (v[2 + q] - o)) +
           C::d2_3 * ((v[7 + q] - o) + (v[1 + q] - o)) - C::d2_4 * ((v[8 + q] - o) + (v[q] - o));
}

// The same along z from 9 vectors f(iz - 4 .. iz + 4) of 4 columns.
__device__ __forceinline__ float d2_col(const float4 *v, int q)
{
    using C = Coef<float>;
    const float o = comp(v[4], q);
    return C::d2_1 * ((comp(v[5], q) - o) + (comp(v[3], q) - o)) -
           C::d2_2 * ((comp(v[6], q) - o) + (comp(v[2], q) - o)) +
           C::d2_3 * ((comp(v[7], q) - o) + (comp(v[1], q) - o)) -
           C::d2_4 * ((comp(v[8], q) - o) + (comp(v[0], q) - o));
}

// Origin of this block's tile: the list entry blockIdx.x of Batch::tiles[list], or grid
// position (blockIdx.x, blockIdx.y) without a list.
__device__ __forceinline__ void tile_origin(const Batch<float> &b, int list, int &x0, int &z0)
{
    const int *t = b.tiles[list];
    if (t) {
        const int v = t[blockIdx.x];
        x0 = b.xbase + (v & 0xffff) * TT;
        z0 = b.zbase + (v >> 16) * TT;
    } else {
        x0 = b.xbase + blockIdx.x * TT;
        z0 = b.zbase + blockIdx.y * TT;
    }
}

// Max over the warp, one atomic per warp (values are >= 0).
__device__ __forceinline__ void warp_max_to(float v, float *dst)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.f) atomicMax((unsigned *)dst, __float_as_uint(v));
}

template <typename S> struct Vec4Store;
template <> struct Vec4Store<float> {
    static __device__ __forceinline__ void put(float *p, const float (&v)[4])
    {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
    static __device__ __forceinline__ void get(const float *p, float (&v)[4])
    {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
};
// 16-bit image values: 4 per 8-byte access (callers keep p 8-byte aligned).
template <typename H> struct Vec4Store16 {
    static __device__ __forceinline__ void put(H *p, const H (&v)[4])
    {
        uint2 u;
        u.x = (uint32_t)__builtin_bit_cast(uint16_t, v[0]) | ((uint32_t)__builtin_bit_cast(uint16_t, v[1]) << 16);
        u.y = (uint32_t)__builtin_bit_cast(uint16_t, v[2]) | ((uint32_t)__builtin_bit_cast(uint16_t, v[3]) << 16);
        *reinterpret_cast<uint2 *>(p) = u;
    }
    static __device__ __forceinline__ void get(const H *p, H (&v)[4])
    {
        const uint2 u = *reinterpret_cast<const uint2 *>(p);
        v[0] = __builtin_bit_cast(H, (uint16_t)(u.x & 0xffffu));
        v[1] = __builtin_bit_cast(H, (uint16_t)(u.x >> 16));
        v[2] = __builtin_bit_cast(H, (uint16_t)(u.y & 0xffffu));
        v[3] = __builtin_bit_cast(H, (uint16_t)(u.y >> 16));
    }
};
template <> struct Vec4Store<__half> : Vec4Store16<__half> {};
template <> struct Vec4Store<__nv_bfloat16> : Vec4Store16<__nv_bfloat16> {};

// ------------------------------------------------------------------ forward tiles

// Per-shot scalars of a forward step, gathered once per block.
struct FwdShot {
    long so;        // shot offset in the per-shot arrays
    long rec_base;  // record index of column 0 at this step (receivers at rec_base + ix)
    long img;       // image offset, in elements of the store type
    int sx, sz, rz, rx0, rx1, wx0;  // source, receivers; wx0: model column of window column 0
    float w, sc;    // wavelet sample, image scale
};

// Interior tiles: no CPML term, so the images are the plain stencils in both modes.
// MIXED: the group's shots have several windows (one tile grid, in window
// coordinates, for all): the block keeps the shots for which its tile is an
// interior tile of their own window and reads the models at each shot's own
// columns; its interior mask depends on the row only (every column of an
// interior tile is an interior column).
template <int ST, bool MIXED>
__global__ void __launch_bounds__(kTmaThreads, 4)
k_fwd_tma(Batch<float> b, const __grid_constant__ TmaMaps maps, int g, int ntb, int cur, int img_slot, int sg)
{
    using Cd = Codec<float, ST>;
    // dynamic shared memory: the stages, then the group's per-shot scalars and active shots (sized
    // by the group, so that a small group leaves room for a fourth block on the SM)
    extern __shared__ __align__(128) unsigned char dsm_raw[];
    unsigned char *dsm = aligned_dsm(dsm_raw);
    FwdIncStage *stage = reinterpret_cast<FwdIncStage *>(dsm);
    FwdShot *ps = reinterpret_cast<FwdShot *>(dsm + kStages * sizeof(FwdIncStage));
    int *act = reinterpret_cast<int *>(ps + sg);
    __shared__ __align__(8) uint64_t bar[kStages];
    __shared__ float wmax[2][kTmaThreads / 32];  // the warps' maxima of |P|, |F| of a shot (alternate shots)
    const int tid = threadIdx.x;
    int x0, z0;
    tile_origin(b, kTilesFwdInterior, x0, z0);
    const DevShot gsh = b.shots[blockIdx.z * sg];  // unless MIXED, every shot of the group has this window
    const int nx = gsh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    if (!MIXED && tile_role(x0, z0, nx, nz, cpml) != 1) return;
    const int na = MIXED ? active_shots(b, sg, act, false, g, ntb, x0, z0, cpml) : active_shots(b, sg, act, false, g, ntb);
    if (na == 0) return;
    if (tid == 0) {
        for (int k = 0; k < kStages; k++) mbar_init(&bar[k], 1);
        mbar_init_fence();
    }
    if (tid < na) {
        const int s = act[tid];
        const DevShot sh = b.shots[s];
        const int it = g - (ntb - sh.nt);
        FwdShot q;
        q.so = (long)s * b.slot;
        q.rec_base = sh.rec_off + (long)it * (sh.rx1 - sh.rx0) - sh.rx0;
        q.img = ((long)s * b.n_img + (img_slot >= 0 ? img_slot : 0)) * 2 * b.slot;
        q.sx = sh.sx; q.sz = sh.sz; q.rz = sh.rz; q.rx0 = sh.rx0; q.rx1 = sh.rx1; q.wx0 = sh.x0;
        q.w = b.wavelet[it];
        q.sc = 1.f;
        if (img_slot >= 0 && Cd::scaled) {
            q.sc = image_scale(b.amax[(long)s * (b.nt_max + 1) + g], (float)b.inv_dh2);
            if (x0 == b.xbase && z0 == b.zbase) b.scale[(long)s * b.nt_max + g] = q.sc;  // never: a layer tile
        }
        ps[tid] = q;
    }
    __syncthreads();
    auto issue = [&](int a) {
        const int s = act[a];
        FwdIncStage &S = stage[a % kStages];
        uint64_t *br = &bar[a % kStages];
        mbar_expect_tx(br, (unsigned)sizeof(FwdIncStage));
        tma_load_3d(S.P, &maps.px[cur], br, x0 - kRad, z0, s);
        tma_load_3d(S.F, &maps.fz[cur], br, x0, z0 - kRad, s);
        tma_load_3d(S.VP, &maps.inc[0], br, x0, z0, s);
        tma_load_3d(S.VF, &maps.inc[1], br, x0, z0, s);
    };
    if (tid == 0)
        for (int k = 0; k < min(kStages, na); k++) issue(k);
    const int c4 = 4 * (tid & 7), r = tid >> 3;
    const int ix0 = x0 + c4, iz = z0 + r;
    bool m[4];  // interior points
    bool any = false, all = true;
    float mh[4], mp[4], mn[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int ix = ix0 + q;
        m[q] = MIXED ? (iz > 3 && iz < nz - 4) : (ix < nx && iz < nz && interior(ix, iz, nx, nz));
        any |= m[q];
        all &= m[q];
        const long mi = (long)iz * b.mpitch + gsh.x0 + ix;
        mh[q] = !MIXED && m[q] ? b.mh[mi] : 0.f;
        mp[q] = !MIXED && m[q] ? b.mp[mi] : 0.f;
        mn[q] = !MIXED && m[q] ? b.mn[mi] : 0.f;
    }
    const long ipt = (long)iz * pitch + ix0;
    float *const Pn0 = b.lvl[1 - cur], *const Fn0 = b.lvl[3 - cur];
    float *const Pv0 = b.lvl[4], *const Fv0 = b.lvl[5];
    for (int a = 0; a < na; a++) {
        const FwdShot &sh = ps[a];
        const long so = sh.so;
        if (MIXED && any) {  // this shot's model columns: issued before the wait, in flight during it
            const long mi = (long)iz * b.mpitch + sh.wx0 + ix0;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                mh[q] = m[q] ? b.mh[mi + q] : 0.f;
                mp[q] = m[q] ? b.mp[mi + q] : 0.f;
                mn[q] = m[q] ? b.mn[mi + q] : 0.f;
            }
        }
        const bool ok = mbar_wait(&bar[a % kStages], (a / kStages) & 1);
        const FwdIncStage &S = stage[a % kStages];
        float lmax = 0.f;
        if (any && ok) {
            const float4 vP = ld4(&S.VP[r][c4]), vF = ld4(&S.VF[r][c4]);
            float pv[12];
            {
                const float *row = &S.P[r][c4];
                const float4 a0 = ld4(row), a1 = ld4(row + 4), a2 = ld4(row + 8);
                pv[0] = a0.x; pv[1] = a0.y; pv[2] = a0.z; pv[3] = a0.w;
                pv[4] = a1.x; pv[5] = a1.y; pv[6] = a1.z; pv[7] = a1.w;
                pv[8] = a2.x; pv[9] = a2.y; pv[10] = a2.z; pv[11] = a2.w;
            }
            float4 fz[9];
#pragma unroll
            for (int k = 0; k < 9; k++) fz[k] = ld4(&S.F[r + k][c4]);
            const float w = sh.w;
            const bool src_row = iz == sh.sz;
            float gG[4], gH[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                gG[q] = d2_row(pv, q) * b.inv_dh2;
                gH[q] = d2_col(fz, q) * b.inv_dh2;
            }
            float nP[4], nF[4], iP[4], iF[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float G = gG[q], H = gH[q];
                const float mpH = mp[q] * H;
                float vp = comp(vP, q) + (mh[q] * G + mpH);
                float vf = comp(vF, q) + (mn[q] * G + mpH);
                if (src_row && ix0 + q == sh.sx) { vp += w; vf += w; }
                iP[q] = vp;
                iF[q] = vf;
                nP[q] = pv[4 + q] + vp;
                nF[q] = comp(fz[4], q) + vf;
                if (Cd::scaled && m[q]) lmax = fmaxf(lmax, fmaxf(fabsf(nP[q]), fabsf(nF[q])));
            }
            float *Pn = Pn0 + so, *Fn = Fn0 + so, *Pv = Pv0 + so, *Fv = Fv0 + so;
            if (all) {
                Vec4Store<float>::put(Pv + ipt, iP);
                Vec4Store<float>::put(Fv + ipt, iF);
                Vec4Store<float>::put(Pn + ipt, nP);
                Vec4Store<float>::put(Fn + ipt, nF);
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (m[q]) {
                        Pv[ipt + q] = iP[q];
                        Fv[ipt + q] = iF[q];
                        Pn[ipt + q] = nP[q];
                        Fn[ipt + q] = nF[q];
                    }
            }
            if (iz == sh.rz) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int ix = ix0 + q;
                    if (m[q] && ix >= sh.rx0 && ix < sh.rx1) b.rec[sh.rec_base + ix] = nP[q] + nF[q];
                }
            }
            if (img_slot >= 0) {
                using SI = typename Cd::S;
                SI *img = (SI *)b.store + sh.img;
                const float sc = sh.sc;
                SI eG[4], eH[4];
                bool sat = false;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    eG[q] = Cd::enc_flag(m[q] ? gG[q] : 0.f, sc, sat);
                    eH[q] = Cd::enc_flag(m[q] ? gH[q] : 0.f, sc, sat);
                }
                if (sat) atomicOr(b.status, kStatusSaturated);
                if (all) {
                    Vec4Store<SI>::put(img + ipt, eG);
                    Vec4Store<SI>::put(img + b.slot + ipt, eH);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (m[q]) {
                            img[ipt + q] = eG[q];
                            img[b.slot + ipt + q] = eH[q];
                        }
                }
            }
        }
        if (Cd::scaled) {
            for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            if ((tid & 31) == 0) wmax[a & 1][tid >> 5] = lmax;
        }
        if (!stage_release(ok, bar, a, na, kStages, b.status)) return;  // every thread is done with this stage
        if (Cd::scaled && tid == 0) {  // one reduction per block and shot
            float m = 0.f;
            for (int w = 0; w < kTmaThreads / 32; w++) m = fmaxf(m, wmax[a & 1][w]);
            if (m > 0.f) atomicMax((unsigned *)&b.amax[(long)act[a] * (b.nt_max + 1) + g + 1], __float_as_uint(m));
        }
        if (tid == 0 && a + kStages < na) {
            fence_proxy_async();
            issue(a + kStages);
        }
    }
}

// ------------------------------------------------------------------ adjoint tiles

// Per-shot scalars of an adjoint step, gathered once per block.
struct AdjShot {
    long so;        // shot offset in the per-shot arrays
    long res_base;  // residual index of column 0 at this step (residual at res_base + ix)
    long img;       // image offset in elements of the store type, < 0: no image this step
    int rz, rx0, rx1, wx0;  // receiver row and columns; model column of window column 0
    int nx;         // window width
    float inv_sc;   // inverse image scale
};

// MIXED (several windows in the group, see k_fwd_tma): the model tiles are
// staged per shot, at the shot's own columns, and each shot's imaging goes
// to its own gradient slot (shot s: slot s) instead of a sum per group.
template <int ST, bool EXACT, bool MIXED>
__global__ void __launch_bounds__(kTmaThreads, 3)
k_adj_tma(Batch<float> b, const __grid_constant__ TmaMaps maps, int j, int ntb, int cur, int zsel, int img_base,
          int sg)
{
    using Cd = Codec<float, ST>;
    using Stage = AdjIncStage;
    using SI = typename Cd::S;
    extern __shared__ __align__(128) unsigned char dsm_raw[];
    unsigned char *dsm = aligned_dsm(dsm_raw);
    Stage *stage = reinterpret_cast<Stage *>(dsm);
    float(*MH)[TH] = reinterpret_cast<float(*)[TH]>(dsm + kAdjStages * sizeof(Stage));  // [TT][TH]
    float(*MN)[TH] = MH + TT;                                                          // [TT][TH]
    float(*MP)[TT] = reinterpret_cast<float(*)[TT]>(MN + TT);                          // [TH][TT]
    float(*U)[TH] = reinterpret_cast<float(*)[TH]>(MP + TH);                           // [TT][TH]
    float(*V)[TT] = reinterpret_cast<float(*)[TT]>(U + TT);                            // [TH][TT]
    __shared__ __align__(8) uint64_t bar[kAdjStages];
    __shared__ int act[kMaxGroup];
    __shared__ AdjShot ps[kMaxGroup];
    const int tid = threadIdx.x;
    int x0, z0;
    tile_origin(b, kTilesAdjInterior, x0, z0);
    const int grp = blockIdx.z;
    const DevShot gsh = b.shots[grp * sg];
    const int nx = gsh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    const int aw = EXACT ? cpml + kRad : cpml;
    if (!MIXED && tile_role(x0, z0, nx, nz, aw) != 1) return;
    const int na = MIXED ? active_shots(b, sg, act, true, j, ntb, x0, z0, aw) : active_shots(b, sg, act, true, j, ntb);
    if (na == 0) return;
    const int lag = EXACT ? 0 : 1;
    const int img_g = ntb - 1 - lag - j;  // global step of the image this iteration needs
    if (tid == 0) {
        for (int k = 0; k < kAdjStages; k++) mbar_init(&bar[k], 1);
        mbar_init_fence();
    }
    if (tid < na) {
        const int s = act[tid];
        const DevShot sh = b.shots[s];
        const int mm = sh.nt - j;
        AdjShot q;
        q.so = (long)s * b.slot;
        q.res_base = sh.rec_off + (long)(mm - 1) * (sh.rx1 - sh.rx0) - sh.rx0;
        const bool im = mm - 1 - lag >= 0;
        q.img = im ? ((long)s * b.n_img + (img_g - img_base)) * 2 * b.slot : -1;
        q.rz = sh.rz; q.rx0 = sh.rx0; q.rx1 = sh.rx1; q.wx0 = sh.x0; q.nx = sh.nx;
        q.inv_sc = (im && Cd::scaled) ? 1.f / b.scale[(long)s * b.nt_max + img_g] : 1.f;
        ps[tid] = q;
    }
    __syncthreads();
    auto issue = [&](int a) {
        const int s = act[a];
        Stage &S = stage[a % kAdjStages];
        uint64_t *br = &bar[a % kAdjStages];
        mbar_expect_tx(br, (unsigned)sizeof(Stage));
        tma_load_3d(S.P, &maps.lvl[cur], br, x0 - kRad, z0 - kRad, s);
        tma_load_3d(S.F, &maps.lvl[2 + cur], br, x0 - kRad, z0 - kRad, s);
        tma_load_3d(S.WP, &maps.inc[0], br, x0, z0, s);
        tma_load_3d(S.WF, &maps.inc[1], br, x0, z0, s);
    };
    if (tid == 0)
        for (int k = 0; k < min(kAdjStages, na); k++) issue(k);
    // model tiles of a window (its first model column wx0, width wnx): v_hor, v_nmo with
    // the x-halo, v_po with the z-halo
    auto stage_models = [&](int wx0, int wnx) {
        for (int k = tid; k < TT * TH; k += kTmaThreads) {
            const int rr = k / TH, cc = k - rr * TH;
            const int gx = x0 - kRad + cc, gz = z0 + rr;
            const bool in = gx >= 0 && gx < wnx && gz >= 0 && gz < nz;
            const long mi = (long)gz * b.mpitch + wx0 + gx;
            MH[rr][cc] = in ? b.mh[mi] : 0.f;
            MN[rr][cc] = in ? b.mn[mi] : 0.f;
        }
        for (int k = tid; k < TH * TT; k += kTmaThreads) {
            const int rr = k / TT, cc = k - rr * TT;
            const int gx = x0 + cc, gz = z0 - kRad + rr;
            const bool in = gx < wnx && gz >= 0 && gz < nz;
            MP[rr][cc] = in ? b.mp[(long)gz * b.mpitch + wx0 + gx] : 0.f;
        }
    };
    if (!MIXED) {
        stage_models(gsh.x0, nx);
        __syncthreads();  // the model tiles, before any thread's first U, V (no block barrier before that)
    }
    const int c4 = 4 * (tid & 7), r = tid >> 3;
    const int ix0 = x0 + c4, iz = z0 + r;
    bool m[4];  // interior points
    bool any = false, all = true;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int ix = ix0 + q;
        m[q] = MIXED ? (iz > 3 && iz < nz - 4) : (ix < nx && iz < nz && interior(ix, iz, nx, nz));
        any |= m[q];
        all &= m[q];
    }
    const long ipt = (long)iz * pitch + ix0;
    float *const lPn0 = b.lvl[1 - cur], *const lFn0 = b.lvl[3 - cur];
    float *const lPw0 = b.lvl[4], *const lFw0 = b.lvl[5];
    float ah[4] = {0.f, 0.f, 0.f, 0.f}, ap[4] = {0.f, 0.f, 0.f, 0.f}, an[4] = {0.f, 0.f, 0.f, 0.f};
    for (int a = 0; a < na; a++) {
        // own points' images: issued before the wait, in flight during it (the increments come
        // with the stage)
        SI iG[4], iH[4];
        if (any) {
            if (ps[a].img >= 0) {
                const SI *img = (const SI *)b.store + ps[a].img;
                Vec4Store<SI>::get(img + ipt, iG);
                Vec4Store<SI>::get(img + b.slot + ipt, iH);
            }
        }
        // MIXED: this shot's model tiles (the previous shot's U, V are done: stage_release)
        if (MIXED) stage_models(ps[a].wx0, ps[a].nx);
        const bool ok = mbar_wait(&bar[a % kAdjStages], (a / kAdjStages) & 1);
        if (MIXED) __syncthreads();  // the model tiles, before U, V
        const Stage &S = stage[a % kAdjStages];
        // U = dt^2 (v_hor lP + v_nmo lF) on the x-halo tile, V = dt^2 v_po (lP + lF) on the z-halo tile
        // (from whatever the stage holds if this thread's wait gave up: the iteration is then discarded)
        for (int k = tid; k < TT * (TH / 4); k += kTmaThreads) {
            const int rr = k / (TH / 4), cc = 4 * (k - rr * (TH / 4));
            const float4 p = ld4(&S.P[rr + kRad][cc]), f = ld4(&S.F[rr + kRad][cc]);
            const float4 h = ld4(&MH[rr][cc]), n = ld4(&MN[rr][cc]);
            *reinterpret_cast<float4 *>(&U[rr][cc]) =
                make_float4(h.x * p.x + n.x * f.x, h.y * p.y + n.y * f.y, h.z * p.z + n.z * f.z, h.w * p.w + n.w * f.w);
        }
        for (int k = tid; k < TH * (TT / 4); k += kTmaThreads) {
            const int rr = k / (TT / 4), cc = 4 * (k - rr * (TT / 4));
            const float4 p = ld4(&S.P[rr][cc + kRad]), f = ld4(&S.F[rr][cc + kRad]), v = ld4(&MP[rr][cc]);
            *reinterpret_cast<float4 *>(&V[rr][cc]) =
                make_float4(v.x * (p.x + f.x), v.y * (p.y + f.y), v.z * (p.z + f.z), v.w * (p.w + f.w));
        }
        const bool bad = __syncthreads_or(!ok);  // U and V complete; any thread's wait given up
        const AdjShot &sh = ps[a];
        const long so = sh.so;
        if (any && !bad) {
            float uv[12];
            {
                const float4 a0 = ld4(&U[r][c4]), a1 = ld4(&U[r][c4 + 4]), a2 = ld4(&U[r][c4 + 8]);
                uv[0] = a0.x; uv[1] = a0.y; uv[2] = a0.z; uv[3] = a0.w;
                uv[4] = a1.x; uv[5] = a1.y; uv[6] = a1.z; uv[7] = a1.w;
                uv[8] = a2.x; uv[9] = a2.y; uv[10] = a2.z; uv[11] = a2.w;
            }
            float4 vz[9];
#pragma unroll
            for (int k = 0; k < 9; k++) vz[k] = ld4(&V[r + k][c4]);
            const float4 cP = ld4(&S.P[r + kRad][c4 + kRad]), cF = ld4(&S.F[r + kRad][c4 + kRad]);
            float e[4][2];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                e[q][0] = d2_row(uv, q) * b.inv_dh2;
                e[q][1] = d2_col(vz, q) * b.inv_dh2;
            }
                const bool rec_row = iz == sh.rz;
            const float4 wP = ld4(&S.WP[r][c4]), wF = ld4(&S.WF[r][c4]);
            float nwP[4], nwF[4], nP[4], nF[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                float wp = comp(wP, q) + e[q][0];
                float wf = comp(wF, q) + e[q][1];
                const int ix = ix0 + q;
                if (rec_row && m[q] && ix >= sh.rx0 && ix < sh.rx1) {
                    const float d = b.rec[sh.res_base + ix];
                    wp += d;
                    wf += d;
                }
                nwP[q] = wp;
                nwF[q] = wf;
                nP[q] = comp(cP, q) + wp;
                nF[q] = comp(cF, q) + wf;
            }
            float *lPn = lPn0 + so, *lFn = lFn0 + so, *lPw = lPw0 + so, *lFw = lFw0 + so;
            if (all) {
                Vec4Store<float>::put(lPw + ipt, nwP);
                Vec4Store<float>::put(lFw + ipt, nwF);
                Vec4Store<float>::put(lPn + ipt, nP);
                Vec4Store<float>::put(lFn + ipt, nF);
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (m[q]) {
                        lPw[ipt + q] = nwP[q];
                        lFw[ipt + q] = nwF[q];
                        lPn[ipt + q] = nP[q];
                        lFn[ipt + q] = nF[q];
                    }
            }
            if (sh.img >= 0) {
                const float inv_sc = sh.inv_sc;
                const float kk = b.img_scale;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float Gv = Cd::dec(iG[q], inv_sc), Hv = Cd::dec(iH[q], inv_sc);
                    ah[q] += kk * Gv * nP[q];
                    ap[q] += kk * Hv * (nP[q] + nF[q]);
                    an[q] += kk * Gv * nF[q];
                }
                if (MIXED) {
                    // this shot's slot: g[act[a]] += its imaging, as reductions that the
                    // thread does not wait for.  One add per point and launch (each slot
                    // point belongs to one block and thread), so the sum is the plain
                    // read-modify-write's, bit for bit.
                    const long gi = (long)act[a] * b.slot + ipt;
                    float *g0 = b.g[0] + gi, *g1 = b.g[1] + gi, *g2 = b.g[2] + gi;
                    if (all) {
                        atomicAdd(reinterpret_cast<float4 *>(g0), make_float4(ah[0], ah[1], ah[2], ah[3]));
                        atomicAdd(reinterpret_cast<float4 *>(g1), make_float4(ap[0], ap[1], ap[2], ap[3]));
                        atomicAdd(reinterpret_cast<float4 *>(g2), make_float4(an[0], an[1], an[2], an[3]));
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            if (m[q]) {
                                atomicAdd(g0 + q, ah[q]);
                                atomicAdd(g1 + q, ap[q]);
                                atomicAdd(g2 + q, an[q]);
                            }
                    }
#pragma unroll
                    for (int q = 0; q < 4; q++) ah[q] = ap[q] = an[q] = 0.f;
                }
            }
        }
        if (!stage_release(!bad, bar, a, na, kAdjStages, b.status)) return;  // stage, U and V are free again
        if (tid == 0 && a + kAdjStages < na) {
            fence_proxy_async();
            issue(a + kAdjStages);
        }
    }
    if (MIXED || !any) return;
    // one read-modify-write per group: g[grp] += the group's imaging
    const long gi = (long)grp * b.slot + ipt;
    float *g0 = b.g[0] + gi, *g1 = b.g[1] + gi, *g2 = b.g[2] + gi;
    if (all) {
        const float4 o0 = ld4(g0), o1 = ld4(g1), o2 = ld4(g2);
        *reinterpret_cast<float4 *>(g0) = make_float4(o0.x + ah[0], o0.y + ah[1], o0.z + ah[2], o0.w + ah[3]);
        *reinterpret_cast<float4 *>(g1) = make_float4(o1.x + ap[0], o1.y + ap[1], o1.z + ap[2], o1.w + ap[3]);
        *reinterpret_cast<float4 *>(g2) = make_float4(o2.x + an[0], o2.y + an[1], o2.z + an[2], o2.w + an[3]);
    } else {
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (m[q]) {
                g0[q] += ah[q];
                g1[q] += ap[q];
                g2[q] += an[q];
            }
    }
}

inline size_t fwd_tma_smem(int sg) { return 128 + kStages * sizeof(FwdIncStage) + sg * (sizeof(FwdShot) + sizeof(int)); }
inline size_t adj_tma_smem()
{
    return 128 + kAdjStages * sizeof(AdjIncStage) + sizeof(float) * (2 * TT * TH + TH * TT + TT * TH + TH * TT);
}

}  // namespace fwi
