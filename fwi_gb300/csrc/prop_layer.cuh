// FP32 layer tiles (tile_role 2: tiles holding points the CPML layers
// touch), on sm_103a.  Same structure as the interior tiles of
// prop_tma.cuh (a block per tile and shot group, TMA stages, 4 points per
// thread), with the CPML memory variables the strip pass advanced this step
// staged beside the fields, so that every neighbour read of the CPML terms
// is a shared-memory read and runs 4 points at a time:
//
//   forward:            P, F + psi_x (x-halo), psi_z (z-halo)
//   exact adjoint:      lP, lF + Zx', Yx' (x-halo), Zz', Yz' (z-halo)
//   reference adjoint:  lP, lF + psi_xcx, psi_zdx (x-halo), psi_xcz, psi_zcz (z-halo)
//
// The zeta variables (read and written at each point only) load into
// registers before the stage wait, like the increments.  Where the tile
// grid puts each band with the points beside it in one tile column or row
// (TileGrid::inline_strip), the INLINE instantiations advance the memory
// variables of their own band points in the tile instead of staging what the
// strip pass wrote.  A layer group's shots share one window (their bands sit
// at that window's edges); a thread polls each stage and the block meets
// there (stage_ready), which measured faster here than per-thread waits.
#pragma once

#include "prop_tma.cuh"

namespace fwi {

constexpr int kLayerStages = 2;

struct FwdLayerStage {
    float P[TT][TH];
    float F[TH][TT];
    float SX[TT][TH];  // psi_x
    float SZ[TH][TT];  // psi_z
};

struct AdjLayerStage {
    float P[TH][TH];
    float F[TH][TH];
    float A[TT][TH];  // x-halo memory variables (see the file comment)
    float B[TT][TH];
    float C[TH][TT];  // z-halo memory variables
    float D[TH][TT];
};

// 8th-order first derivative (unnormalised) at 4 consecutive points from 12
// values v[0..11] = f(ix0 - 4 .. ix0 + 7), the reference's tap order.
__device__ __forceinline__ float d1_row(const float *v, int q)
{
    using C = Coef<float>;
    return C::d1_1 * (v[5 + q] - v[3 + q]) - C::d1_2 * (v[6 + q] - v[2 + q]) + C::d1_3 * (v[7 + q] - v[1 + q]) -
           C::d1_4 * (v[8 + q] - v[q]);
}

// The same along z from 9 vectors f(iz - 4 .. iz + 4) of 4 columns.
__device__ __forceinline__ float d1_col(const float4 *v, int q)
{
    using C = Coef<float>;
    return C::d1_1 * (comp(v[5], q) - comp(v[3], q)) - C::d1_2 * (comp(v[6], q) - comp(v[2], q)) +
           C::d1_3 * (comp(v[7], q) - comp(v[1], q)) - C::d1_4 * (comp(v[8], q) - comp(v[0], q));
}

__device__ __forceinline__ void row12(const float *row, float *v)
{
    const float4 a0 = ld4(row), a1 = ld4(row + 4), a2 = ld4(row + 8);
    v[0] = a0.x; v[1] = a0.y; v[2] = a0.z; v[3] = a0.w;
    v[4] = a1.x; v[5] = a1.y; v[6] = a1.z; v[7] = a1.w;
    v[8] = a2.x; v[9] = a2.y; v[10] = a2.z; v[11] = a2.w;
}

// ------------------------------------------------------------------ forward

// Forward layer tiles (src/parallelcalls.cu:48-117 at the strip points):
// G = Dxx P + (Dx psi_x + zeta_x'), zeta_x' = b zeta_x + a (Dxx P + Dx psi_x)
// (and H along z), only at strip points; the other points of the tile as
// in the interior.  EXACT stores images of G, H; the reference's of the
// plain stencils.  INLINE (TileGrid::inline_strip): the tile advances psi
// of its own band points, psi = b psi + a Dx P, from the staged P and F
// instead of loading what the strip pass wrote.
template <int ST, bool EXACT, bool INLINE>
__global__ void __launch_bounds__(kTmaThreads, 2)
k_fwd_layer(Batch<float> b, const __grid_constant__ TmaMaps maps, int g, int ntb, int cur, int img_slot, int sg)
{
    using Cd = Codec<float, ST>;
    extern __shared__ __align__(128) unsigned char dsm_raw[];
    FwdLayerStage *stage = reinterpret_cast<FwdLayerStage *>(aligned_dsm(dsm_raw));
    __shared__ __align__(8) uint64_t bar[kLayerStages];
    __shared__ int act[kMaxGroup];
    __shared__ FwdShot ps[kMaxGroup];
    __shared__ float wmax[2][kTmaThreads / 32];  // the warps' maxima of |P|, |F| of a shot (alternate shots)
    const int tid = threadIdx.x;
    int x0, z0;
    tile_origin(b, kTilesFwdLayer, x0, z0);
    const DevShot gsh = b.shots[blockIdx.z * sg];
    const int nx = gsh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    if (tile_role(x0, z0, nx, nz, cpml) != 2) return;
    const int na = active_shots(b, sg, act, false, g, ntb);
    if (na == 0) return;
    if (tid == 0) {
        for (int k = 0; k < kLayerStages; k++) mbar_init(&bar[k], 1);
        mbar_init_fence();
    }
    if (INLINE)  // psi tiles are computed here: their halos stay zero
        for (int k = 0; k < kLayerStages; k++) {
            float *sx = &stage[k].SX[0][0], *szp = &stage[k].SZ[0][0];
            for (int i = tid; i < TT * TH; i += kTmaThreads) sx[i] = szp[i] = 0.f;
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
            if (x0 == b.xbase && z0 == b.zbase) b.scale[(long)s * b.nt_max + g] = q.sc;  // tile (0, 0)
        }
        ps[tid] = q;
    }
    __syncthreads();
    auto issue = [&](int a) {
        const int s = act[a];
        FwdLayerStage &S = stage[a % kLayerStages];
        uint64_t *br = &bar[a % kLayerStages];
        mbar_expect_tx(br, (unsigned)(INLINE ? sizeof(S.P) + sizeof(S.F) : sizeof(FwdLayerStage)));
        tma_load_3d(S.P, &maps.px[cur], br, x0 - kRad, z0, s);
        tma_load_3d(S.F, &maps.fz[cur], br, x0, z0 - kRad, s);
        if (!INLINE) {
            tma_load_3d(S.SX, &maps.mx[0], br, x0 - kRad, z0, s);
            tma_load_3d(S.SZ, &maps.mz[1], br, x0, z0 - kRad, s);
        }
    };
    if (tid == 0)
        for (int k = 0; k < min(kLayerStages, na); k++) issue(k);
    const int c4 = 4 * (tid & 7), r = tid >> 3;
    const int ix0 = x0 + c4, iz = z0 + r;
    bool m[4], S4[4], xl[4];  // interior points, strip points, x-layer points
    bool any = false, all = true, anyS = false;
    float mh[4], mp[4], mn[4], ax[4], bx[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int ix = ix0 + q;
        m[q] = ix < nx && iz < nz && interior(ix, iz, nx, nz);
        S4[q] = m[q] && layer_point(ix, iz, nx, nz, cpml);
        xl[q] = S4[q] && (ix < cpml || ix > nx - cpml - 1);
        any |= m[q];
        all &= m[q];
        anyS |= S4[q];
        const long mi = (long)iz * b.mpitch + gsh.x0 + ix;
        mh[q] = m[q] ? b.mh[mi] : 0.f;
        mp[q] = m[q] ? b.mp[mi] : 0.f;
        mn[q] = m[q] ? b.mn[mi] : 0.f;
        ax[q] = xl[q] ? coef_x(b.cpa, ix, nx, cpml) : 0.f;
        bx[q] = xl[q] ? coef_x(b.cpb, ix, nx, cpml) : 0.f;
    }
    const bool zl = iz > nz - cpml - 1 && iz < nz - 4;
    const float az = zl ? coef_z(b.cpa, iz, nz, cpml) : 0.f, bz = zl ? coef_z(b.cpb, iz, nz, cpml) : 0.f;
    const long ipt = (long)iz * pitch + ix0;
    float *const Pn0 = b.lvl[1 - cur], *const Fn0 = b.lvl[3 - cur];
    float *const Pv0 = b.lvl[4], *const Fv0 = b.lvl[5];
    float *const psx0 = b.cp[0], *const psz0 = b.cp[1], *const zx0 = b.cp[2], *const zz0 = b.cp[3];
    for (int a = 0; a < na; a++) {
        const FwdShot &sh = ps[a];
        const long so = sh.so;
        float4 vP = make_float4(0.f, 0.f, 0.f, 0.f), vF = vP, zX = vP, zZ = vP, pX = vP, pZ = vP;
        if (any) {  // own points: issued before the wait
            vP = ld4(Pv0 + so + ipt);
            vF = ld4(Fv0 + so + ipt);
            if (anyS) {
                zX = ld4(zx0 + so + ipt);
                zZ = ld4(zz0 + so + ipt);
                if (INLINE) {
                    pX = ld4(psx0 + so + ipt);
                    pZ = ld4(psz0 + so + ipt);
                }
            }
        }
        if (!stage_ready(&bar[a % kLayerStages], (a / kLayerStages) & 1, b.status)) {
            drain_stages_n(bar, a, na, kLayerStages);
            return;
        }
        FwdLayerStage &S = stage[a % kLayerStages];
        float lmax = 0.f;
        if (INLINE) {
            // psi of the own band points (src/parallelcalls.cu:48-63); other cells stay 0
            if (any && anyS) {
                float pv[12];
                row12(&S.P[r][c4], pv);
                float4 fz[9];
#pragma unroll
                for (int k = 0; k < 9; k++) fz[k] = ld4(&S.F[r + k][c4]);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    float px = 0.f, pz = 0.f;
                    if (xl[q]) px = bx[q] * comp(pX, q) + ax[q] * (d1_row(pv, q) * b.inv_dh);
                    if (S4[q] && zl) pz = bz * comp(pZ, q) + az * (d1_col(fz, q) * b.inv_dh);
                    S.SX[r][c4 + kRad + q] = px;
                    S.SZ[r + kRad][c4 + q] = pz;
                    if (xl[q]) psx0[so + ipt + q] = px;
                    if (S4[q] && zl) psz0[so + ipt + q] = pz;
                }
            }
            __syncthreads();  // the tile's psi complete
        }
        if (any) {
            float pv[12];
            row12(&S.P[r][c4], pv);
            float4 fz[9];
#pragma unroll
            for (int k = 0; k < 9; k++) fz[k] = ld4(&S.F[r + k][c4]);
            float gP[4], gF[4], G[4], H[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                gP[q] = d2_row(pv, q) * b.inv_dh2;
                gF[q] = d2_col(fz, q) * b.inv_dh2;
                G[q] = gP[q];
                H[q] = gF[q];
            }
            if (anyS) {
                float sx[12];
                row12(&S.SX[r][c4], sx);
                float4 sz[9];
#pragma unroll
                for (int k = 0; k < 9; k++) sz[k] = ld4(&S.SZ[r + k][c4]);
                float nzx[4], nzz[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float tx = d1_row(sx, q) * b.inv_dh, tz = d1_col(sz, q) * b.inv_dh;
                    nzx[q] = xl[q] ? bx[q] * comp(zX, q) + ax[q] * (gP[q] + tx) : 0.f;
                    nzz[q] = (S4[q] && zl) ? bz * comp(zZ, q) + az * (gF[q] + tz) : 0.f;
                    if (S4[q]) {
                        G[q] = gP[q] + (tx + nzx[q]);
                        H[q] = gF[q] + (tz + nzz[q]);
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (xl[q]) zx0[so + ipt + q] = nzx[q];
                    if (S4[q] && zl) zz0[so + ipt + q] = nzz[q];
                }
            }
            const float w = sh.w;
            const bool src_row = iz == sh.sz;
            float nP[4], nF[4], iP[4], iF[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float mpH = mp[q] * H[q];
                float vp = comp(vP, q) + (mh[q] * G[q] + mpH);
                float vf = comp(vF, q) + (mn[q] * G[q] + mpH);
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
                SI eG[4], eH[4];
                bool sat = false;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    eG[q] = Cd::enc_flag(m[q] ? (EXACT ? G[q] : gP[q]) : 0.f, sh.sc, sat);
                    eH[q] = Cd::enc_flag(m[q] ? (EXACT ? H[q] : gF[q]) : 0.f, sh.sc, sat);
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
        __syncthreads();  // every thread is done with this stage
        if (Cd::scaled && tid == 0) {  // one reduction per block and shot
            float m = 0.f;
            for (int w = 0; w < kTmaThreads / 32; w++) m = fmaxf(m, wmax[a & 1][w]);
            if (m > 0.f) atomicMax((unsigned *)&b.amax[(long)act[a] * (b.nt_max + 1) + g + 1], __float_as_uint(m));
        }
        if (tid == 0 && a + kLayerStages < na) {
            fence_proxy_async();
            issue(a + kLayerStages);
        }
    }
}

// ------------------------------------------------------------------ adjoint

// Adjoint layer tiles.
//  EXACT: at points within 4 of a layer, + Dxx(S ax Zx') - Dx(S ax Yx') and
//         + Dzz(S az Zz') - Dz(S az Yz') (Z', Y' from this step's strip pass);
//         the coefficients vanish away from the layers, so the terms are
//         computed for every point of the tile.
//  reference: at strip points, the four second derivatives of the
//         model-weighted fields and the zeta recursion of
//         src/parallelcalls.cu:200-243 on the psi of this step's strip pass.
// INLINE (TileGrid::inline_strip): the tile advances the memory variables
// of its own band points itself (what the strip pass would), from the
// staged fields and, for the exact adjoint, the previous Z staged with its
// halo: Zx' = g + bx Zx, Yx' = -Dx[S (g + ax (g + bx Zx))] + bx Yx (and z).
template <int ST, bool EXACT, bool INLINE>
__global__ void __launch_bounds__(kTmaThreads, 2)
k_adj_layer(Batch<float> b, const __grid_constant__ TmaMaps maps, int j, int ntb, int cur, int zsel, int img_base,
            int sg)
{
    using Cd = Codec<float, ST>;
    using SI = typename Cd::S;
    using Cf = Coef<float>;
    extern __shared__ __align__(128) unsigned char dsm_raw[];
    unsigned char *dsm = aligned_dsm(dsm_raw);
    AdjLayerStage *stage = reinterpret_cast<AdjLayerStage *>(dsm);
    float(*MH)[TH] = reinterpret_cast<float(*)[TH]>(dsm + kLayerStages * sizeof(AdjLayerStage));  // [TT][TH]
    float(*MN)[TH] = MH + TT;                                                                    // [TT][TH]
    float(*MP)[TT] = reinterpret_cast<float(*)[TT]>(MN + TT);                                    // [TH][TT]
    float(*U)[TH] = reinterpret_cast<float(*)[TH]>(MP + TH);                                     // [TT][TH]
    float(*V)[TT] = reinterpret_cast<float(*)[TT]>(U + TT);                                      // [TH][TT]
    float(*WX)[TH] = reinterpret_cast<float(*)[TH]>(V + TH);  // [TT][TH] INLINE exact: S (g + ax Zx')
    float(*WZ)[TT] = reinterpret_cast<float(*)[TT]>(WX + TT);  // [TH][TT]
    __shared__ __align__(8) uint64_t bar[kLayerStages];
    __shared__ int act[kMaxGroup];
    __shared__ AdjShot ps[kMaxGroup];
    const int tid = threadIdx.x;
    int x0, z0;
    tile_origin(b, kTilesAdjLayer, x0, z0);
    const int grp = blockIdx.z;
    const DevShot gsh = b.shots[grp * sg];
    const int nx = gsh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    const int aw = EXACT ? cpml + kRad : cpml;
    if (tile_role(x0, z0, nx, nz, aw) != 2) return;
    const int na = active_shots(b, sg, act, true, j, ntb);
    if (na == 0) return;
    const int lag = EXACT ? 0 : 1;
    const int img_g = ntb - 1 - lag - j;
    if (tid == 0) {
        for (int k = 0; k < kLayerStages; k++) mbar_init(&bar[k], 1);
        mbar_init_fence();
    }
    if (INLINE) {  // arrays computed here (not loaded): their halos stay zero
        for (int k = 0; k < kLayerStages; k++) {
            float *pb = &stage[k].B[0][0], *pd = &stage[k].D[0][0];
            float *pa = &stage[k].A[0][0], *pc = &stage[k].C[0][0];
            for (int i = tid; i < TT * TH; i += kTmaThreads) {
                pb[i] = pd[i] = 0.f;
                if (!EXACT) pa[i] = pc[i] = 0.f;
            }
        }
        float *wx = &WX[0][0], *wz = &WZ[0][0];
        for (int i = tid; i < TT * TH; i += kTmaThreads) wx[i] = wz[i] = 0.f;
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
        q.rz = sh.rz; q.rx0 = sh.rx0; q.rx1 = sh.rx1; q.wx0 = sh.x0;
        q.inv_sc = (im && Cd::scaled) ? 1.f / b.scale[(long)s * b.nt_max + img_g] : 1.f;
        ps[tid] = q;
    }
    __syncthreads();
    // EXACT: A = Zx', B = Yx, C = Zz', D = Yz;  reference: A = psi_xcx, B = psi_zdx, C = psi_xcz, D = psi_zcz
    const CUtensorMap *mA = &maps.mx[EXACT ? 3 - zsel : 0], *mB = &maps.mx[EXACT ? 0 : 2];
    const CUtensorMap *mC = &maps.mz[EXACT ? 5 - zsel : 1], *mD = &maps.mz[EXACT ? 1 : 3];
    // INLINE exact: A = Zx (old half), C = Zz (old half) staged; B = Yx', D = Yz' computed.
    // INLINE reference: A..D computed.
    if (INLINE && EXACT) {
        mA = &maps.mx[2 + zsel];
        mC = &maps.mz[4 + zsel];
    }
    auto issue = [&](int a) {
        const int s = act[a];
        AdjLayerStage &S = stage[a % kLayerStages];
        uint64_t *br = &bar[a % kLayerStages];
        const unsigned bytes = !INLINE ? (unsigned)sizeof(AdjLayerStage)
                               : EXACT ? (unsigned)(sizeof(S.P) + sizeof(S.F) + sizeof(S.A) + sizeof(S.C))
                                       : (unsigned)(sizeof(S.P) + sizeof(S.F));
        mbar_expect_tx(br, bytes);
        tma_load_3d(S.P, &maps.lvl[cur], br, x0 - kRad, z0 - kRad, s);
        tma_load_3d(S.F, &maps.lvl[2 + cur], br, x0 - kRad, z0 - kRad, s);
        if (!INLINE || EXACT) {
            tma_load_3d(S.A, mA, br, x0 - kRad, z0, s);
            tma_load_3d(S.C, mC, br, x0, z0 - kRad, s);
        }
        if (!INLINE) {
            tma_load_3d(S.B, mB, br, x0 - kRad, z0, s);
            tma_load_3d(S.D, mD, br, x0, z0 - kRad, s);
        }
    };
    if (tid == 0)
        for (int k = 0; k < min(kLayerStages, na); k++) issue(k);
    for (int k = tid; k < TT * TH; k += kTmaThreads) {
        const int rr = k / TH, cc = k - rr * TH;
        const int gx = x0 - kRad + cc, gz = z0 + rr;
        const bool in = gx >= 0 && gx < nx && gz >= 0 && gz < nz;
        const long mi = (long)gz * b.mpitch + gsh.x0 + gx;
        MH[rr][cc] = in ? b.mh[mi] : 0.f;
        MN[rr][cc] = in ? b.mn[mi] : 0.f;
    }
    for (int k = tid; k < TH * TT; k += kTmaThreads) {
        const int rr = k / TT, cc = k - rr * TT;
        const int gx = x0 + cc, gz = z0 - kRad + rr;
        const bool in = gx < nx && gz >= 0 && gz < nz;
        MP[rr][cc] = in ? b.mp[(long)gz * b.mpitch + gsh.x0 + gx] : 0.f;
    }
    const int c4 = 4 * (tid & 7), r = tid >> 3;
    const int ix0 = x0 + c4, iz = z0 + r;
    bool m[4], S4[4];  // interior points, strip points (reference mode)
    bool any = false, all = true, anyS = false;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int ix = ix0 + q;
        m[q] = ix < nx && iz < nz && interior(ix, iz, nx, nz);
        S4[q] = m[q] && layer_point(ix, iz, nx, nz, cpml);
        any |= m[q];
        all &= m[q];
        anyS |= S4[q];
    }
    // CPML coefficients of the thread's columns (EXACT: the 12-wide window
    // ix0 - 4 .. ix0 + 7) and rows (iz - 4 .. iz + 4), zero outside the layers
    float axw[12], azw[9];
    bool xnear = false, znear = false;
#pragma unroll
    for (int k = 0; k < 12; k++) {
        const int ix = ix0 - kRad + k;
        axw[k] = (ix >= 0 && ix < nx) ? coef_x(b.cpa, ix, nx, cpml) : 0.f;
        xnear |= axw[k] != 0.f;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int jz = iz - kRad + k;
        azw[k] = (jz >= 0 && jz < nz) ? coef_z(b.cpa, jz, nz, cpml) : 0.f;
        znear |= azw[k] != 0.f;
    }
    // reference mode: b at the thread's own points
    float bxq[4];
#pragma unroll
    for (int q = 0; q < 4; q++) bxq[q] = S4[q] ? coef_x(b.cpb, ix0 + q, nx, cpml) : 0.f;
    const float bzr = (iz > nz - cpml - 1 && iz < nz) ? coef_z(b.cpb, iz, nz, cpml) : 0.f;
    const long ipt = (long)iz * pitch + ix0;
    float *const lPn0 = b.lvl[1 - cur], *const lFn0 = b.lvl[3 - cur];
    float *const lPw0 = b.lvl[4], *const lFw0 = b.lvl[5];
    float ah[4] = {0.f, 0.f, 0.f, 0.f}, ap[4] = {0.f, 0.f, 0.f, 0.f}, an[4] = {0.f, 0.f, 0.f, 0.f};
    const float c2[5] = {Cf::d2_0, Cf::d2_1, -Cf::d2_2, Cf::d2_3, -Cf::d2_4};
    const float c1[4] = {Cf::d1_1, -Cf::d1_2, Cf::d1_3, -Cf::d1_4};
    for (int a = 0; a < na; a++) {
        float4 wP = make_float4(0.f, 0.f, 0.f, 0.f), wF = wP;
        float4 zt[4] = {wP, wP, wP, wP};  // reference zeta: xcx, xcz, zdx, zcz
        float4 yo[4] = {wP, wP, wP, wP};  // INLINE: old memory variables at the own points
        SI iG[4], iH[4];
        if (any) {
            const long so = ps[a].so;
            wP = ld4(lPw0 + so + ipt);
            wF = ld4(lFw0 + so + ipt);
            if (ps[a].img >= 0) {
                const SI *img = (const SI *)b.store + ps[a].img;
                Vec4Store<SI>::get(img + ipt, iG);
                Vec4Store<SI>::get(img + b.slot + ipt, iH);
            }
            if (!EXACT && anyS)
                for (int k = 0; k < 4; k++) zt[k] = ld4(b.cp[4 + k] + so + ipt);
            if (INLINE && anyS)  // EXACT: Yx, Yz; reference: the four psi (updated in place)
                for (int k = 0; k < (EXACT ? 2 : 4); k++) yo[k] = ld4(b.cp[k] + so + ipt);
        }
        if (!stage_ready(&bar[a % kLayerStages], (a / kLayerStages) & 1, b.status)) {
            drain_stages_n(bar, a, na, kLayerStages);
            return;
        }
        AdjLayerStage &S = stage[a % kLayerStages];
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
        __syncthreads();
        const AdjShot &sh = ps[a];
        const long so = sh.so;
        if (INLINE) {
            // the memory variables of the own band points, what the strip pass would
            // compute (exact: this file's comment; reference: src/parallelcalls.cu:179-198)
            if (any && anyS) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int ix = ix0 + q, c = c4 + q;
                    const bool xl = S4[q] && (ix < cpml || ix > nx - cpml - 1);
                    const bool zl = S4[q] && iz > nz - cpml - 1;
                    const float axq = axw[4 + q], bxq_ = bxq[q], az = azw[4], bz = bzr;
                    const long i = so + ipt + q;
                    if (EXACT) {
                        const float gq = U[r][c + kRad], hq = V[r + kRad][c];
                        const float zxo = S.A[r][c + kRad], zzo = S.C[r + kRad][c];
                        WX[r][c + kRad] = S4[q] ? gq + axq * (gq + bxq_ * zxo) : 0.f;
                        WZ[r + kRad][c] = S4[q] ? hq + az * (hq + bz * zzo) : 0.f;
                        const float zxn = xl ? gq + bxq_ * zxo : 0.f, zzn = zl ? hq + bz * zzo : 0.f;
                        S.A[r][c + kRad] = zxn;  // own cell: Z' replaces the old Z
                        S.C[r + kRad][c] = zzn;
                        if (xl) b.cp[3 - zsel][i] = zxn;
                        if (zl) b.cp[5 - zsel][i] = zzn;
                    } else {
                        float d1 = 0.f, d3 = 0.f, d2 = 0.f, d4 = 0.f;
#pragma unroll
                        for (int k = 1; k <= 4; k++) {
                            d1 += c1[k - 1] * (MH[r][c + kRad + k] * S.P[r + kRad][c + kRad + k] -
                                               MH[r][c + kRad - k] * S.P[r + kRad][c + kRad - k]);
                            d3 += c1[k - 1] * (MN[r][c + kRad + k] * S.F[r + kRad][c + kRad + k] -
                                               MN[r][c + kRad - k] * S.F[r + kRad][c + kRad - k]);
                            d2 += c1[k - 1] * (MP[r + kRad + k][c] * S.P[r + kRad + k][c + kRad] -
                                               MP[r + kRad - k][c] * S.P[r + kRad - k][c + kRad]);
                            d4 += c1[k - 1] * (MP[r + kRad + k][c] * S.F[r + kRad + k][c + kRad] -
                                               MP[r + kRad - k][c] * S.F[r + kRad - k][c + kRad]);
                        }
                        const float pxcx = xl ? bxq_ * comp(yo[0], q) + axq * (d1 * b.inv_dh) : 0.f;
                        const float pzdx = xl ? bxq_ * comp(yo[2], q) + axq * (d3 * b.inv_dh) : 0.f;
                        const float pxcz = zl ? bz * comp(yo[1], q) + az * (d2 * b.inv_dh) : 0.f;
                        const float pzcz = zl ? bz * comp(yo[3], q) + az * (d4 * b.inv_dh) : 0.f;
                        S.A[r][c + kRad] = pxcx;
                        S.B[r][c + kRad] = pzdx;
                        S.C[r + kRad][c] = pxcz;
                        S.D[r + kRad][c] = pzcz;
                        if (xl) {
                            b.cp[0][i] = pxcx;
                            b.cp[2][i] = pzdx;
                        }
                        if (zl) {
                            b.cp[1][i] = pxcz;
                            b.cp[3][i] = pzcz;
                        }
                    }
                }
            }
            __syncthreads();
            if (EXACT) {
                // Y' = -Dx W + b Y at the own band points (W complete now)
                if (any && anyS) {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const int ix = ix0 + q, c = c4 + q;
                        const bool xl = S4[q] && (ix < cpml || ix > nx - cpml - 1);
                        const bool zl = S4[q] && iz > nz - cpml - 1;
                        float ax_ = 0.f, az_ = 0.f;
#pragma unroll
                        for (int k = 1; k <= 4; k++) {
                            ax_ += c1[k - 1] * (WX[r][c + kRad + k] - WX[r][c + kRad - k]);
                            az_ += c1[k - 1] * (WZ[r + kRad + k][c] - WZ[r + kRad - k][c]);
                        }
                        const float yx = xl ? -ax_ * b.inv_dh + bxq[q] * comp(yo[0], q) : 0.f;
                        const float yz = zl ? -az_ * b.inv_dh + bzr * comp(yo[1], q) : 0.f;
                        S.B[r][c + kRad] = yx;
                        S.D[r + kRad][c] = yz;
                        const long i = so + ipt + q;
                        if (xl) b.cp[0][i] = yx;
                        if (zl) b.cp[1][i] = yz;
                    }
                }
                __syncthreads();
            }
        }
        if (any) {
            float e0[4], e1[4];
            {
                float uv[12];
                row12(&U[r][c4], uv);
                float4 vz[9];
#pragma unroll
                for (int k = 0; k < 9; k++) vz[k] = ld4(&V[r + k][c4]);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    e0[q] = d2_row(uv, q) * b.inv_dh2;
                    e1[q] = d2_col(vz, q) * b.inv_dh2;
                }
            }
            if (EXACT) {
                if (xnear) {
                    float za[12], ya[12];
                    row12(&S.A[r][c4], za);
                    row12(&S.B[r][c4], ya);
#pragma unroll
                    for (int k = 0; k < 12; k++) {
                        za[k] *= axw[k];
                        ya[k] *= axw[k];
                    }
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float a2 = c2[0] * za[4 + q], a1 = 0.f;
#pragma unroll
                        for (int k = 1; k <= 4; k++) {
                            a2 += c2[k] * (za[4 + q + k] + za[4 + q - k]);
                            a1 += c1[k - 1] * (ya[4 + q + k] - ya[4 + q - k]);
                        }
                        e0[q] += a2 * b.inv_dh2 - a1 * b.inv_dh;
                    }
                }
                if (znear) {
                    float4 zc[9], yd[9];
#pragma unroll
                    for (int k = 0; k < 9; k++) {
                        const float4 cz = ld4(&S.C[r + k][c4]), dz = ld4(&S.D[r + k][c4]);
                        zc[k] = make_float4(azw[k] * cz.x, azw[k] * cz.y, azw[k] * cz.z, azw[k] * cz.w);
                        yd[k] = make_float4(azw[k] * dz.x, azw[k] * dz.y, azw[k] * dz.z, azw[k] * dz.w);
                    }
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float a2 = c2[0] * comp(zc[4], q), a1 = 0.f;
#pragma unroll
                        for (int k = 1; k <= 4; k++) {
                            a2 += c2[k] * (comp(zc[4 + k], q) + comp(zc[4 - k], q));
                            a1 += c1[k - 1] * (comp(yd[4 + k], q) - comp(yd[4 - k], q));
                        }
                        e1[q] += a2 * b.inv_dh2 - a1 * b.inv_dh;
                    }
                }
            } else if (anyS) {
                // reference ZETA_R (src/parallelcalls.cu:216-243) at the strip points
#pragma unroll 1
                for (int q = 0; q < 4; q++) {
                    if (!S4[q]) continue;
                    const int c = c4 + q;
                    float p2cx = 0.f, r2dx = 0.f, p2cz = 0.f, r2cz = 0.f;
#pragma unroll
                    for (int k = -4; k <= 4; k++) {
                        const float w2 = c2[k < 0 ? -k : k];
                        p2cx += w2 * (MH[r][c + kRad + k] * S.P[r + kRad][c + kRad + k]);
                        r2dx += w2 * (MN[r][c + kRad + k] * S.F[r + kRad][c + kRad + k]);
                        p2cz += w2 * (MP[r + kRad + k][c] * S.P[r + kRad + k][c + kRad]);
                        r2cz += w2 * (MP[r + kRad + k][c] * S.F[r + kRad + k][c + kRad]);
                    }
                    p2cx *= b.inv_dh2; r2dx *= b.inv_dh2; p2cz *= b.inv_dh2; r2cz *= b.inv_dh2;
                    float dxcx = 0.f, dzdx = 0.f, dxcz = 0.f, dzcz = 0.f;
#pragma unroll
                    for (int k = 1; k <= 4; k++) {
                        dxcx += c1[k - 1] * (S.A[r][c + kRad + k] - S.A[r][c + kRad - k]);
                        dzdx += c1[k - 1] * (S.B[r][c + kRad + k] - S.B[r][c + kRad - k]);
                        dxcz += c1[k - 1] * (S.C[r + kRad + k][c] - S.C[r + kRad - k][c]);
                        dzcz += c1[k - 1] * (S.D[r + kRad + k][c] - S.D[r + kRad - k][c]);
                    }
                    dxcx *= b.inv_dh; dzdx *= b.inv_dh; dxcz *= b.inv_dh; dzcz *= b.inv_dh;
                    const float axq = axw[4 + q], bxq_ = bxq[q];
                    const float az = azw[4], bz = bzr;
                    const float n1 = bxq_ * comp(zt[0], q) + axq * (dxcx + p2cx);
                    const float n2 = bz * comp(zt[1], q) + az * (dxcz + p2cz);
                    const float n3 = bxq_ * comp(zt[2], q) + axq * (dzdx + r2dx);
                    const float n4 = bz * comp(zt[3], q) + az * (dzcz + r2cz);
                    const long i = so + ipt + q;
                    b.cp[4][i] = n1;
                    b.cp[5][i] = n2;
                    b.cp[6][i] = n3;
                    b.cp[7][i] = n4;
                    e0[q] = (p2cx + r2dx) + ((n1 + dxcx) + (n3 + dzdx));
                    e1[q] = (p2cz + r2cz) + ((n2 + dxcz) + (n4 + dzcz));
                }
            }
            const float4 cP = ld4(&S.P[r + kRad][c4 + kRad]), cF = ld4(&S.F[r + kRad][c4 + kRad]);
            const bool rec_row = iz == sh.rz;
            float nwP[4], nwF[4], nP[4], nF[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                float wp = comp(wP, q) + e0[q];
                float wf = comp(wF, q) + e1[q];
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
                const float kk = b.img_scale;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float Gv = Cd::dec(iG[q], sh.inv_sc), Hv = Cd::dec(iH[q], sh.inv_sc);
                    ah[q] += kk * Gv * nP[q];
                    ap[q] += kk * Hv * (nP[q] + nF[q]);
                    an[q] += kk * Gv * nF[q];
                }
            }
        }
        __syncthreads();  // stage, U and V are free again
        if (tid == 0 && a + kLayerStages < na) {
            fence_proxy_async();
            issue(a + kLayerStages);
        }
    }
    if (!any) return;
    const long gi = (long)grp * b.slot + ipt;
    float *g0 = b.g[0] + gi, *g1 = b.g[1] + gi, *g2 = b.g[2] + gi;
#pragma unroll
    for (int q = 0; q < 4; q++)
        if (m[q]) {
            g0[q] += ah[q];
            g1[q] += ap[q];
            g2[q] += an[q];
        }
}

inline size_t fwd_layer_smem() { return 128 + kLayerStages * sizeof(FwdLayerStage); }
inline size_t adj_layer_smem()
{
    return 128 + kLayerStages * sizeof(AdjLayerStage) +
           sizeof(float) * (2 * TT * TH + TH * TT + TT * TH + TH * TT + TT * TH + TH * TT);
}

}  // namespace fwi
