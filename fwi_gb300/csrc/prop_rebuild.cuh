// FP32 backward rebuild of the CPML-free region R for FWI_STORE_BOUNDARY
// (the scheme is described in prop_boundary.cuh), on the tile pipeline of
// prop_tma.cuh: one block per (32 x 32 tile, shot group), the rebuild
// level's P (x-halo) and F (z-halo) staged by TMA, the increments loaded
// into registers before the stage wait, 4 points per thread.  Per point of R:
// the images of step g, v^g = v^{g+1} - w - (v_hor G + v_po H) (and F), and
// P^{g-1} = P^g - v^g into the other level; per ring point: the ring of step
// g - 1 from storage into the other level (one launch per step).
#pragma once

#include "prop_boundary.cuh"
#include "prop_tma.cuh"

namespace fwi {

template <int ST>
__global__ void __launch_bounds__(kTmaThreads, 3)
k_rebuild_tma(Batch<float> b, const __grid_constant__ TmaMaps maps, int g, int ntb, int cur, const float *ring,
              long ring_len, int sg, int img_slot)
{
    using Cd = Codec<float, ST>;
    extern __shared__ __align__(128) unsigned char dsm_raw[];
    FwdStage *stage = reinterpret_cast<FwdStage *>(aligned_dsm(dsm_raw));
    __shared__ __align__(8) uint64_t bar[kStages];
    __shared__ int act[kMaxGroup];
    __shared__ FwdShot ps[kMaxGroup];
    const int tid = threadIdx.x;
    const int x0 = b.xbase + blockIdx.x * TT, z0 = b.zbase + blockIdx.y * TT;
    const DevShot gsh = b.shots[blockIdx.z * sg];
    const int nx = gsh.nx, nz = b.nz, pitch = b.pitch, cpml = b.cpml;
    if (tile_role(x0, z0, nx, nz, cpml) == 0) return;
    const int na = active_shots(b, sg, act, false, g, ntb);
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
        q.rec_base = it - 1 >= 0 ? ((long)s * b.nt_max + (g - 1)) * ring_len : -1;  // ring of step g - 1
        q.img = ((long)s * b.n_img + img_slot) * 2 * b.slot;
        q.sx = sh.sx; q.sz = sh.sz; q.rz = 0; q.rx0 = 0; q.rx1 = 0; q.wx0 = sh.x0;
        q.w = b.wavelet[it];
        q.sc = Cd::scaled ? image_scale(b.amax[(long)s * (b.nt_max + 1) + g], (float)b.inv_dh2) : 1.f;
        if (Cd::scaled && blockIdx.x == 0 && blockIdx.y == 0) b.scale[(long)s * b.nt_max + g] = q.sc;
        ps[tid] = q;
    }
    __syncthreads();
    auto issue = [&](int a) {
        const int s = act[a];
        FwdStage &S = stage[a % kStages];
        uint64_t *br = &bar[a % kStages];
        mbar_expect_tx(br, (unsigned)sizeof(FwdStage));
        tma_load_3d(S.P, &maps.px[cur], br, x0 - kRad, z0, s);
        tma_load_3d(S.F, &maps.fz[cur], br, x0, z0 - kRad, s);
    };
    if (tid == 0)
        for (int k = 0; k < min(kStages, na); k++) issue(k);
    const int c4 = 4 * (tid & 7), r = tid >> 3;
    const int ix0 = x0 + c4, iz = z0 + r;
    const Ring R = Ring::make(nx, nz, cpml);
    bool inR[4], any = false, all = true, anyRing = false;
    long rk[4];  // ring index of the point (-1: not a ring point), P ring first
    bool rF[4];
    float mh[4], mp[4], mn[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int ix = ix0 + q;
        inR[q] = in_rebuild_region(ix, iz, nx, nz, cpml);
        any |= inR[q];
        all &= inR[q];
        rk[q] = R.index(ix, iz, rF[q]);
        anyRing |= rk[q] >= 0;
        const long mi = (long)iz * b.mpitch + gsh.x0 + ix;
        mh[q] = inR[q] ? b.mh[mi] : 0.f;
        mp[q] = inR[q] ? b.mp[mi] : 0.f;
        mn[q] = inR[q] ? b.mn[mi] : 0.f;
    }
    const long ipt = (long)iz * pitch + ix0;
    float *const Pn0 = b.lvl[1 - cur], *const Fn0 = b.lvl[3 - cur];
    float *const Pv0 = b.lvl[4], *const Fv0 = b.lvl[5];
    for (int a = 0; a < na; a++) {
        const FwdShot &sh = ps[a];
        const long so = sh.so;
        float4 vP = make_float4(0.f, 0.f, 0.f, 0.f), vF = vP;
        if (any) {
            vP = ld4(Pv0 + so + ipt);
            vF = ld4(Fv0 + so + ipt);
        }
        if (!stage_ready(&bar[a % kStages], (a / kStages) & 1, b.status)) {
            drain_stages(bar, a, na);
            return;
        }
        const FwdStage &S = stage[a % kStages];
        if (any) {
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
            const bool src_row = iz == sh.sz;
            float nP[4], nF[4], iP[4], iF[4];
            using SI = typename Cd::S;
            SI eG[4], eH[4];
            bool sat = false;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float G = d2_row(pv, q) * b.inv_dh2;
                const float H = d2_col(fz, q) * b.inv_dh2;
                eG[q] = Cd::enc_flag(inR[q] ? G : 0.f, sh.sc, sat);
                eH[q] = Cd::enc_flag(inR[q] ? H : 0.f, sh.sc, sat);
                const float mpH = mp[q] * H;
                float vp = comp(vP, q), vf = comp(vF, q);
                if (src_row && ix0 + q == sh.sx) {
                    vp -= sh.w;
                    vf -= sh.w;
                }
                vp -= (mh[q] * G + mpH);
                vf -= (mn[q] * G + mpH);
                iP[q] = vp;
                iF[q] = vf;
                nP[q] = pv[4 + q] - vp;
                nF[q] = comp(fz[4], q) - vf;
            }
            if (sat) atomicOr(b.status, kStatusSaturated);
            float *Pn = Pn0 + so, *Fn = Fn0 + so, *Pv = Pv0 + so, *Fv = Fv0 + so;
            SI *img = (SI *)b.store + sh.img;
            if (all) {
                Vec4Store<float>::put(Pv + ipt, iP);
                Vec4Store<float>::put(Fv + ipt, iF);
                Vec4Store<float>::put(Pn + ipt, nP);
                Vec4Store<float>::put(Fn + ipt, nF);
                Vec4Store<SI>::put(img + ipt, eG);
                Vec4Store<SI>::put(img + b.slot + ipt, eH);
            } else {
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (inR[q]) {
                        Pv[ipt + q] = iP[q];
                        Fv[ipt + q] = iF[q];
                        Pn[ipt + q] = nP[q];
                        Fn[ipt + q] = nF[q];
                        img[ipt + q] = eG[q];
                        img[b.slot + ipt + q] = eH[q];
                    }
            }
        }
        if (anyRing && sh.rec_base >= 0) {
            const float *rg = ring + sh.rec_base;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (rk[q] >= 0) (rF[q] ? Fn0 : Pn0)[so + ipt + q] = rg[rk[q]];
        }
        __syncthreads();  // every thread is done with this stage
        if (tid == 0 && a + kStages < na) {
            fence_proxy_async();
            issue(a + kStages);
        }
    }
}

inline size_t rebuild_tma_smem() { return 128 + kStages * sizeof(FwdStage); }

}  // namespace fwi
