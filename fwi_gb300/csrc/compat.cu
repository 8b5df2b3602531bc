// Reference-compatible C-ABI (include/fwi_compat.h): danielvn/Fwi's 17 host
// entry points (include/serialcalls.h) on the library's own sm_103a kernels.
//
// Buffer semantics are the reference's: every array the reference kernels
// write is written here, and nothing else is touched.  The arithmetic is the
// reference's too, operation for operation: stencil differences and pair sums
// in FP32, the double-literal coefficients and the division by dh (dh2) in
// FP64, rounding to FP32 on assignment, everything else in FP32 in the
// reference's operand order.  This unit is compiled without multiply-add
// contraction (--fmad=false, fwi_gb300/build.py), so every operation rounds
// as C evaluates the expression, and the results equal the reference kernels
// run as C on the CPU bit for bit.  The per-step sequences of the reference
// (launchPropagation: 4 kernels; launchBackPropagation: 6 kernels) run as 2
// and 3 kernels: one pass over the CPML strip points (the memory variables
// whose derivatives the next pass needs), then one tiled pass that stages
// the x- and z-halos of the stencil fields in shared memory and does every
// point-wise update of that step.
#include "../../include/fwi_compat.h"
#include "common.cuh"
#include "tile.cuh"

#include <cmath>

namespace {

using fwi::Coef;
using fwi::in_strip;
using fwi::interior;
using fwi::StripMap;

constexpr int TX = 32, TZ = 32, BY = 8;  // 32x32 outputs per 32x8-thread block
constexpr int XW = TX + 2 * fwi::kRad, ZH = TZ + 2 * fwi::kRad;

cudaError_t g_last_error = cudaSuccess;

inline void note(cudaError_t e)
{
    if (e != cudaSuccess && g_last_error == cudaSuccess) g_last_error = e;
}
inline void note_launch() { note(cudaGetLastError()); }

inline dim3 tile_grid(int nx, int nz) { return dim3((nx + TX - 1) / TX, (nz + TZ - 1) / TZ); }

// The reference's 8th-order stencils (src/parallelcalls.cu:57, 127).  v(k) is the
// FP32 value k points from the centre along the stencil's axis.  Differences and
// pair sums of neighbours are FP32 operations; the coefficients are double
// literals, so the products, the sum and the division by dh (dh2) are FP64; the
// caller rounds the result to FP32.
template <typename V> __device__ __forceinline__ double ref_first(V v, float dh)
{
    return ((4 / 5.) * (v(1) - v(-1)) - (1 / 5.) * (v(2) - v(-2)) + (4 / 105.) * (v(3) - v(-3)) -
            (1 / 280.) * (v(4) - v(-4))) /
           dh;
}

template <typename V> __device__ __forceinline__ double ref_second(V v, float dh2)
{
    return (-(205 / 72.) * v(0) + (8 / 5.) * (v(1) + v(-1)) - (1 / 5.) * (v(2) + v(-2)) +
            (8 / 315.) * (v(3) + v(-3)) - (1 / 560.) * (v(4) + v(-4))) /
           dh2;
}

// Along x (s = 1) or z (s = nx) of a global array, at flat index i.
__device__ __forceinline__ float first_g(const float *f, long i, long s, float dh)
{
    return (float)ref_first([&](int k) { return f[i + k * s]; }, dh);
}
// From a staged x-halo tile [rows][W] (output column c, row r) or z-halo tile [rows + 8][TX].
template <int W> __device__ __forceinline__ float second_xt(const float (*t)[W], int r, int c, float dh2)
{
    return (float)ref_second([&](int k) { return t[r][c + fwi::kRad + k]; }, dh2);
}
__device__ __forceinline__ float second_zt(const float (*t)[TX], int r, int c, float dh2)
{
    return (float)ref_second([&](int k) { return t[r + fwi::kRad + k][c]; }, dh2);
}
inline unsigned blocks1d(long n, int b) { return (unsigned)((n + b - 1) / b); }

// ----------------------------------------------------------------- setup

__global__ void k_pre_variables(const float *__restrict__ vel, const float *__restrict__ eps,
                                const float *__restrict__ del, float *v_hor, float *v_po,
                                float *v_nmo, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float vp = __fmul_rn(vel[i], vel[i]);
        v_po[i] = vp;
        v_hor[i] = __fmul_rn(vp, __fadd_rn(1.0f, __fmul_rn(2.0f, eps[i])));
        v_nmo[i] = __fmul_rn(vp, __fadd_rn(1.0f, __fmul_rn(2.0f, del[i])));
    }
}

// One CPML coefficient pair at `dist` points into the layer, evaluated in
// FP64 from FP32 inputs as the reference does (src/parallelcalls.cu:25-26):
// d = d0 Vmax (dist dh / L)^2, alpha = pi f (L - dist dh) / L,
// b = exp(-(d + alpha) dt), a = d (b - 1) / (d + alpha).
__device__ void cpml_pair(float *a, float *b, int dist, float vmax, float dt, float dh, float f,
                          float d0, float L)
{
    float frac = dist * dh / L;
    double d = (double)(d0 * vmax) * ((double)frac * (double)frac);
    double alpha = 3.141592653589793 * (double)f * (double)(L - dist * dh) / (double)L;
    float bf = (float)exp(-(d + alpha) * (double)dt);
    *b = bf;
    *a = (float)(d * (double)(bf - 1.0f) / (d + alpha));
}

__global__ void k_cpml_x(float *a_x, float *b_x, int cpml, float vmax, int nx, float dt, float dh,
                         float f, float d0, float L)
{
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix < cpml && ix < nx) cpml_pair(&a_x[ix], &b_x[ix], cpml - ix, vmax, dt, dh, f, d0, L);
    if (ix > nx - cpml - 1 && ix < nx)
        cpml_pair(&a_x[ix], &b_x[ix], ix - nx + cpml + 1, vmax, dt, dh, f, d0, L);
}

__global__ void k_cpml_z(float *a_z, float *b_z, int cpml, float vmax, int nz, float dt, float dh,
                         float f, float d0, float L)
{
    int iz = blockIdx.x * blockDim.x + threadIdx.x;
    if (iz > nz - cpml - 1 && iz < nz)
        cpml_pair(&a_z[iz], &b_z[iz], iz - nz + cpml + 1, vmax, dt, dh, f, d0, L);
}

// ----------------------------------------------------------------- single kernels

__global__ void k_psi_f_strip(const float *__restrict__ P, const float *__restrict__ F,
                              const float *__restrict__ a_x, const float *__restrict__ b_x,
                              const float *__restrict__ a_z, const float *__restrict__ b_z,
                              float *psi_px, float *psi_fz, StripMap sm, float dh)
{
    const int nx = sm.nx;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < sm.count();
         k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        sm.point(k, ix, iz);
        long i = (long)iz * nx + ix;
        float tpx = first_g(P, i, 1, dh);
        float tfz = first_g(F, i, nx, dh);
        psi_px[i] = b_x[ix] * psi_px[i] + a_x[ix] * tpx;
        psi_fz[i] = b_z[iz] * psi_fz[i] + a_z[iz] * tfz;
    }
}

__global__ void k_zeta_f_strip(const float *__restrict__ p2, const float *__restrict__ r2,
                               const float *__restrict__ a_x, const float *__restrict__ b_x,
                               const float *__restrict__ a_z, const float *__restrict__ b_z,
                               const float *__restrict__ psi_px, const float *__restrict__ psi_fz,
                               float *z_px, float *z_fz, float *aten_p, float *aten_f, StripMap sm,
                               float dh)
{
    const int nx = sm.nx;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < sm.count();
         k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        sm.point(k, ix, iz);
        long i = (long)iz * nx + ix;
        float tx = first_g(psi_px, i, 1, dh);
        float tz = first_g(psi_fz, i, nx, dh);
        float zp = b_x[ix] * z_px[i] + a_x[ix] * (p2[i] + tx);
        float zf = b_z[iz] * z_fz[i] + a_z[iz] * (r2[i] + tz);
        z_px[i] = zp;
        z_fz[i] = zf;
        aten_p[i] = tx + zp;
        aten_f[i] = tz + zf;
    }
}

__global__ void k_second_p(const float *__restrict__ P, const float *__restrict__ F, float *p2,
                           float *r2, float dh2, int nx, int nz)
{
    __shared__ float sP[TZ][XW];
    __shared__ float sF[ZH][TX];
    const int x0 = blockIdx.x * TX, z0 = blockIdx.y * TZ;
    fwi::load_xhalo<float, TX, TZ>(sP, P, x0, z0, nx, nz, nx);
    fwi::load_zhalo<float, TX, TZ>(sF, F, x0, z0, nx, nz, nx);
    __syncthreads();
    const int c = threadIdx.x, ix = x0 + c;
    for (int r = threadIdx.y; r < TZ; r += BY) {
        int iz = z0 + r;
        if (!interior(ix, iz, nx, nz)) continue;
        long i = (long)iz * nx + ix;
        p2[i] = second_xt<XW>(sP, r, c, dh2);
        r2[i] = second_zt(sF, r, c, dh2);
    }
}

// propagator_F: leapfrog update, P+F, source, receivers (src/parallelcalls.cu:88-117)
__device__ __forceinline__ void propagate_point(long i, int ix, int iz, float p2v, float r2v,
                                                float atp, float atf, float *PF,
                                                const float *P_pre, const float *F_pre,
                                                float *P_past, float *F_past, const float *v_hor,
                                                const float *v_po, const float *v_nmo,
                                                const float *source, float *shot, float C,
                                                float dh2, int nx, int nz, int sx, int sz, int it,
                                                int cpml)
{
    float pn = 0.f, fn = 0.f;
    bool upd = interior(ix, iz, nx, nz);
    if (upd) {
        float tp = dh2 * (p2v + atp);
        float tf = dh2 * (r2v + atf);
        pn = 2.0f * P_pre[i] - P_past[i] + v_hor[i] * C * tp + v_po[i] * C * tf;
        fn = 2.0f * F_pre[i] - F_past[i] + v_nmo[i] * C * tp + v_po[i] * C * tf;
        PF[i] = pn + fn;
    }
    bool src = (ix == sx - 1 && iz == sz - 1);
    bool rec = (ix > cpml - 1 && ix < nx - cpml && iz == sz - 1);
    if (!upd && (src || rec)) { pn = P_past[i]; fn = F_past[i]; }
    if (src) { pn += source[it]; fn += source[it]; }
    if (upd || src) { P_past[i] = pn; F_past[i] = fn; }
    if (rec) shot[ix + (long)nx * it] = pn + fn;
}

__global__ void k_propagator(const float *__restrict__ p2, const float *__restrict__ r2, float *PF,
                             const float *P_pre, const float *F_pre, float *P_past, float *F_past,
                             const float *__restrict__ v_hor, const float *__restrict__ v_po,
                             const float *__restrict__ v_nmo, const float *__restrict__ aten_p,
                             const float *__restrict__ aten_f, const float *__restrict__ source,
                             float *shot, float C, float dh2, int nx, int nz, int sx, int sz,
                             int it, int cpml)
{
    int ix = blockIdx.x * blockDim.x + threadIdx.x;
    for (int iz = blockIdx.y * blockDim.y + threadIdx.y; iz < nz; iz += gridDim.y * blockDim.y) {
        if (ix >= nx) return;
        long i = (long)iz * nx + ix;
        bool upd = interior(ix, iz, nx, nz);
        propagate_point(i, ix, iz, upd ? p2[i] : 0.f, upd ? r2[i] : 0.f, upd ? aten_p[i] : 0.f,
                        upd ? aten_f[i] : 0.f, PF, P_pre, F_pre, P_past, F_past, v_hor, v_po,
                        v_nmo, source, shot, C, dh2, nx, nz, sx, sz, it, cpml);
    }
}

__global__ void k_res(float *Res, const float *__restrict__ shot1, const float *__restrict__ shot2,
                      long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        Res[i] = shot2[i] - shot1[i];
}

// ----------------------------------------------------------------- fused forward step

// SecondDerivate_P + ZETA_F + propagator_F of one step.  The strip pass
// (k_psi_f_strip) has already advanced psi_px/psi_fz.
__global__ void __launch_bounds__(TX * BY)
k_fwd_main(float *p2, float *r2, float *PF, const float *__restrict__ P_pre,
           const float *__restrict__ F_pre, float *P_past, float *F_past,
           const float *__restrict__ a_x, const float *__restrict__ b_x,
           const float *__restrict__ a_z, const float *__restrict__ b_z,
           const float *__restrict__ psi_px, const float *__restrict__ psi_fz, float *z_px,
           float *z_fz, float *aten_p, float *aten_f, const float *__restrict__ v_hor,
           const float *__restrict__ v_po, const float *__restrict__ v_nmo,
           const float *__restrict__ source, float *shot, float C, float dh2, float dh, int nx, int nz,
           int sx, int sz, int it, int cpml)
{
    __shared__ float sP[TZ][XW];
    __shared__ float sF[ZH][TX];
    const int x0 = blockIdx.x * TX, z0 = blockIdx.y * TZ;
    fwi::load_xhalo<float, TX, TZ>(sP, P_pre, x0, z0, nx, nz, nx);
    fwi::load_zhalo<float, TX, TZ>(sF, F_pre, x0, z0, nx, nz, nx);
    __syncthreads();
    const int c = threadIdx.x, ix = x0 + c;
    if (ix >= nx) return;
    for (int r = threadIdx.y; r < TZ; r += BY) {
        const int iz = z0 + r;
        if (iz >= nz) break;
        const long i = (long)iz * nx + ix;
        float p2v = 0.f, r2v = 0.f, atp = 0.f, atf = 0.f;
        if (interior(ix, iz, nx, nz)) {
            p2v = second_xt<XW>(sP, r, c, dh2);
            r2v = second_zt(sF, r, c, dh2);
            p2[i] = p2v;
            r2[i] = r2v;
            if (in_strip(ix, iz, nx, nz, cpml)) {
                float tx = first_g(psi_px, i, 1, dh);
                float tz = first_g(psi_fz, i, nx, dh);
                float zp = b_x[ix] * z_px[i] + a_x[ix] * (p2v + tx);
                float zf = b_z[iz] * z_fz[i] + a_z[iz] * (r2v + tz);
                z_px[i] = zp;
                z_fz[i] = zf;
                atp = tx + zp;
                atf = tz + zf;
                aten_p[i] = atp;
                aten_f[i] = atf;
            } else {
                atp = aten_p[i];  // outside the layers the reference reads what is stored (zeros)
                atf = aten_f[i];
            }
        }
        propagate_point(i, ix, iz, p2v, r2v, atp, atf, PF, P_pre, F_pre, P_past, F_past, v_hor,
                        v_po, v_nmo, source, shot, C, dh2, nx, nz, sx, sz, it, cpml);
    }
}

// ----------------------------------------------------------------- fused adjoint step

__global__ void k_entry_point(const float *__restrict__ P_pre, const float *__restrict__ F_pre,
                              float *aux1, float *aux2, float *aux3, float *aux4,
                              const float *__restrict__ v_hor, const float *__restrict__ v_po,
                              const float *__restrict__ v_nmo, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float lp = P_pre[i], lf = F_pre[i], vp = v_po[i];
        aux1[i] = v_hor[i] * lp;
        aux2[i] = vp * lp;
        aux3[i] = v_nmo[i] * lf;
        aux4[i] = vp * lf;
    }
}

__global__ void k_psi_r_strip(const float *__restrict__ aux1, const float *__restrict__ aux2,
                              const float *__restrict__ aux3, const float *__restrict__ aux4,
                              const float *__restrict__ a_x, const float *__restrict__ b_x,
                              const float *__restrict__ a_z, const float *__restrict__ b_z,
                              float *psixcx, float *psixcz, float *psizdx, float *psizcz,
                              StripMap sm, float dh)
{
    const int nx = sm.nx;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < sm.count();
         k += (long)gridDim.x * blockDim.x) {
        int ix, iz;
        sm.point(k, ix, iz);
        long i = (long)iz * nx + ix;
        float p1cx = first_g(aux1, i, 1, dh);
        float p1cz = first_g(aux2, i, nx, dh);
        float r1dx = first_g(aux3, i, 1, dh);
        float r1cz = first_g(aux4, i, nx, dh);
        psixcx[i] = b_x[ix] * psixcx[i] + a_x[ix] * p1cx;
        psixcz[i] = b_z[iz] * psixcz[i] + a_z[iz] * p1cz;
        psizdx[i] = b_x[ix] * psizdx[i] + a_x[ix] * r1dx;
        psizcz[i] = b_z[iz] * psizcz[i] + a_z[iz] * r1cz;
    }
}

struct AdjArgs {
    const float *aux1, *aux2, *aux3, *aux4;
    float *p2cx, *p2cz, *r2dx, *r2cz;
    const float *a_x, *b_x, *a_z, *b_z;
    const float *psixcx, *psixcz, *psizdx, *psizcz;
    float *zitaxcx, *zitaxcz, *zitazdx, *zitazcz;
    float *atenxcx, *atenxcz, *atenzdx, *atenzcz;
    const float *P_pre, *F_pre;
    float *P_past, *F_past;
    const float *Res;
    const float *P_snap, *F_snap;
    float *gcx, *gcz, *gdx;
    float C, dh2, dt, dh;
    int nx, nz, nt, sz, it, cpml;
};

// secondDerivate + ZETA_R + retroPropagation + GRADIENT of one adjoint step.
__global__ void __launch_bounds__(TX * BY) k_adj_main(AdjArgs a)
{
    __shared__ float s1[TZ][XW];  // aux1 = v_hor lambdaP (x-halo)
    __shared__ float s3[TZ][XW];  // aux3 = v_nmo lambdaF (x-halo)
    __shared__ float sS[TZ][XW];  // snapshot P (x-halo)
    __shared__ float s2[ZH][TX];  // aux2 = v_po lambdaP (z-halo)
    __shared__ float s4[ZH][TX];  // aux4 = v_po lambdaF (z-halo)
    __shared__ float sT[ZH][TX];  // snapshot F (z-halo)
    const int nx = a.nx, nz = a.nz;
    const int x0 = blockIdx.x * TX, z0 = blockIdx.y * TZ;
    fwi::load_xhalo<float, TX, TZ>(s1, a.aux1, x0, z0, nx, nz, nx);
    fwi::load_xhalo<float, TX, TZ>(s3, a.aux3, x0, z0, nx, nz, nx);
    fwi::load_xhalo<float, TX, TZ>(sS, a.P_snap, x0, z0, nx, nz, nx);
    fwi::load_zhalo<float, TX, TZ>(s2, a.aux2, x0, z0, nx, nz, nx);
    fwi::load_zhalo<float, TX, TZ>(s4, a.aux4, x0, z0, nx, nz, nx);
    fwi::load_zhalo<float, TX, TZ>(sT, a.F_snap, x0, z0, nx, nz, nx);
    __syncthreads();
    const int c = threadIdx.x, ix = x0 + c;
    if (ix >= nx) return;
    const float *res_row = a.Res + (long)nx * (a.nt - a.it - 1);
    for (int r = threadIdx.y; r < TZ; r += BY) {
        const int iz = z0 + r;
        if (iz >= nz) break;
        const long i = (long)iz * nx + ix;
        const bool upd = interior(ix, iz, nx, nz);
        float pn = 0.f, fn = 0.f;
        if (upd) {
            float p2cx = second_xt<XW>(s1, r, c, a.dh2);
            float r2dx = second_xt<XW>(s3, r, c, a.dh2);
            float p2cz = second_zt(s2, r, c, a.dh2);
            float r2cz = second_zt(s4, r, c, a.dh2);
            a.p2cx[i] = p2cx;
            a.r2dx[i] = r2dx;
            a.p2cz[i] = p2cz;
            a.r2cz[i] = r2cz;
            float axcx, axcz, azdx, azcz;
            if (in_strip(ix, iz, nx, nz, a.cpml)) {
                float dxcx = first_g(a.psixcx, i, 1, a.dh);
                float dxcz = first_g(a.psixcz, i, nx, a.dh);
                float dzdx = first_g(a.psizdx, i, 1, a.dh);
                float dzcz = first_g(a.psizcz, i, nx, a.dh);
                float bx = a.b_x[ix], ax = a.a_x[ix], bz = a.b_z[iz], az = a.a_z[iz];
                float zxcx = bx * a.zitaxcx[i] + ax * (dxcx + p2cx);
                float zxcz = bz * a.zitaxcz[i] + az * (dxcz + p2cz);
                float zzdx = bx * a.zitazdx[i] + ax * (dzdx + r2dx);
                float zzcz = bz * a.zitazcz[i] + az * (dzcz + r2cz);
                a.zitaxcx[i] = zxcx;
                a.zitaxcz[i] = zxcz;
                a.zitazdx[i] = zzdx;
                a.zitazcz[i] = zzcz;
                axcx = zxcx + dxcx;
                axcz = zxcz + dxcz;
                azdx = zzdx + dzdx;
                azcz = zzcz + dzcz;
                a.atenxcx[i] = axcx;
                a.atenxcz[i] = axcz;
                a.atenzdx[i] = azdx;
                a.atenzcz[i] = azcz;
            } else {
                axcx = a.atenxcx[i];
                axcz = a.atenxcz[i];
                azdx = a.atenzdx[i];
                azcz = a.atenzcz[i];
            }
            const float k = a.dh2 * a.C;
            pn = 2.0f * a.P_pre[i] - a.P_past[i] + k * (p2cx + axcx + r2dx + azdx);
            fn = 2.0f * a.F_pre[i] - a.F_past[i] + k * (p2cz + r2cz + axcz + azcz);
        }
        const bool inj = (ix > a.cpml - 1 && ix < nx - a.cpml && iz == a.sz - 1);
        if (!upd && inj) { pn = a.P_past[i]; fn = a.F_past[i]; }
        if (inj) { float d = res_row[ix]; pn += d; fn += d; }
        if (upd || inj) { a.P_past[i] = pn; a.F_past[i] = fn; }
        if (upd) {
            float p2 = second_xt<XW>(sS, r, c, a.dh2);
            float r2 = second_zt(sT, r, c, a.dh2);
            a.gcx[i] += a.dt * p2 * pn;
            a.gcz[i] += a.dt * r2 * (pn + fn);
            a.gdx[i] += a.dt * p2 * fn;
        }
    }
}

// ----------------------------------------------------------------- steepest descent, L-BFGS
// Element-wise updates use explicitly rounded multiply and add (no fused
// multiply-add), which makes them bit-identical to the reference's formulas.

constexpr int kLayer = 15;  // include/parallelcalls.h:6

__global__ void k_normal(float *gcx, float *gcz, float *gdx, int nx, int nz, float ngcx, float ngcz,
                         float ngdx)
{
    long n = (long)nx * nz, i0 = (long)nx * (kLayer + 1);
    for (long i = i0 + blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        gcx[i] = gcx[i] / ngcx;
        gcz[i] = gcz[i] / ngcz;
        gdx[i] = gdx[i] / ngdx;
    }
}

__global__ void k_update_model(const float *__restrict__ gcx, const float *__restrict__ gcz,
                               const float *__restrict__ gdx, float *v_hor, float *v_po,
                               float *v_nmo, float a1, float a2, float a3, int nx, int nz)
{
    long n = (long)nx * nz, i0 = (long)nx * (kLayer + 1);
    for (long i = i0 + blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        v_po[i] = __fsub_rn(v_po[i], __fmul_rn(a2, gcz[i]));
        float vn = __fsub_rn(v_nmo[i], __fmul_rn(a3, gdx[i]));
        float vh = __fsub_rn(v_hor[i], __fmul_rn(a1, gcx[i]));
        v_nmo[i] = vn;
        v_hor[i] = vh < vn ? vn : vh;
    }
}

__global__ void k_compute_sy(float *s_vp, float *s_vn, float *s_vh, float *y1, float *y2, float *y3,
                             const float *vp, const float *vn, const float *vh, const float *bvp,
                             const float *bvn, const float *bvh, const float *b1, const float *b2,
                             const float *b3, const float *bb1, const float *bb2, const float *bb3,
                             long n, long off)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        s_vp[i + off] = vp[i] - bvp[i];
        s_vn[i + off] = vn[i] - bvn[i];
        s_vh[i + off] = vh[i] - bvh[i];
        y1[i + off] = b1[i] - bb1[i];
        y2[i + off] = b2[i] - bb2[i];
        y3[i + off] = b3[i] - bb3[i];
    }
}

__global__ void k_axpy3(float *q1, float *q2, float *q3, const float *y1, const float *y2,
                        const float *y3, float e1, float e2, float e3, long n, long off)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        q1[i] = __fsub_rn(q1[i], __fmul_rn(e1, y1[i + off]));
        q2[i] = __fsub_rn(q2[i], __fmul_rn(e2, y2[i + off]));
        q3[i] = __fsub_rn(q3[i], __fmul_rn(e3, y3[i + off]));
    }
}

__global__ void k_scale3(float *r1, float *r2, float *r3, const float *q1, const float *q2,
                         const float *q3, float g1, float g2, float g3, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        r1[i] = g1 * q1[i];
        r2[i] = g2 * q2[i];
        r3[i] = g3 * q3[i];
    }
}

__global__ void k_update_r(float *r1, float *r2, float *r3, const float *s1, const float *s2,
                           const float *s3, float c1, float c2, float c3, long n, long off)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        r1[i] = __fadd_rn(r1[i], __fmul_rn(c1, s1[i + off]));
        r2[i] = __fadd_rn(r2[i], __fmul_rn(c2, s2[i + off]));
        r3[i] = __fadd_rn(r3[i], __fmul_rn(c3, s3[i + off]));
    }
}

// include/parallelcalls.h:7-12
__global__ void k_update_lbfgs(const float *r1, const float *r2, const float *r3, float *vp,
                               float *vn, float *vh, const float *bvp, const float *bvn,
                               const float *bvh, int nx, int nz, float av, float ad, float ae,
                               int fv, int fd, int fe, int fmin, int fmax)
{
    long n = (long)nx * nz, i0 = (long)nx * (kLayer + 1);
    for (long i = i0 + blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (fv == 1) {
            float v = __fsub_rn(bvp[i], __fmul_rn(av, r1[i]));
            if (fmax == 1 && v > 3.5e6f) v = 3.5e6f;
            if (fmin == 1 && v < 1.8e6f) v = 1.8e6f;
            vp[i] = v;
        }
        if (fd == 1) {
            float v = __fsub_rn(bvn[i], __fmul_rn(ad, r2[i]));
            if (fmax == 1 && v > 4e6f) v = 4e6f;
            if (fmin == 1 && v < 1.8e6f) v = 1.8e6f;
            vn[i] = v;
        }
        if (fe == 1) {
            float v = __fsub_rn(bvh[i], __fmul_rn(ae, r3[i]));
            if (fmax == 1 && v > 4.5e6f) v = 4.5e6f;
            if (fmin == 1 && v < 1.8e6f) v = 1.8e6f;
            float w = vn[i];
            vh[i] = v < w ? w : v;
        }
    }
}

constexpr int kEltBlock = 256;
// Grid of a grid-stride kernel: one block per kEltBlock elements, at most 16
// blocks per SM of the current device (the runtime caches the attribute).
inline unsigned elt_grid(long n)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        sms = 1;
    }
    const long cap = 16L * sms;
    long b = (n + kEltBlock - 1) / kEltBlock;
    return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

}  // namespace

extern "C" {

int fwi_compat_last_error(void)
{
    int e = (int)g_last_error;
    g_last_error = cudaSuccess;
    return e;
}

void pre_variables_h(float *vel, float *epsilon, float *delta, float *v_hor, float *v_po,
                     float *v_nmo, int nx, int nz)
{
    long n = (long)nx * nz;
    k_pre_variables<<<elt_grid(n), kEltBlock>>>(vel, epsilon, delta, v_hor, v_po, v_nmo, n);
    note_launch();
}

void CPML_x_h(float *a_x, float *b_x, int CPML, float Vmax, int nx, float dt, float dh, float f,
              float d0, float L)
{
    k_cpml_x<<<blocks1d(nx, 256), 256>>>(a_x, b_x, CPML, Vmax, nx, dt, dh, f, d0, L);
    note_launch();
}

void CPML_z_h(float *a_z, float *b_z, int CPML, float Vmax, int nz, float dt, float dh, float f,
              float d0, float L)
{
    k_cpml_z<<<blocks1d(nz, 256), 256>>>(a_z, b_z, CPML, Vmax, nz, dt, dh, f, d0, L);
    note_launch();
}

void PSI_F_h(float *P, float *F, float *a_x, float *b_x, float *a_z, float *b_z, float *psi_px,
             float *psi_fz, int nx, int nz, float dh, int CPML)
{
    StripMap sm = StripMap::make(nx, nz, CPML);
    if (sm.count() == 0) return;
    k_psi_f_strip<<<elt_grid(sm.count()), kEltBlock>>>(P, F, a_x, b_x, a_z, b_z, psi_px, psi_fz,
                                                         sm, dh);
    note_launch();
}

void ZETA_F_h(float *p2, float *r2, float *P, float *F, float *a_x, float *b_x, float *a_z,
              float *b_z, float *psi_px, float *psi_fz, float *z_px, float *z_fz, float *aten_p,
              float *aten_f, int nx, int nz, float dh, float dh2, int CPML)
{
    (void)P; (void)F; (void)dh2;  // unused by the reference kernel as well
    StripMap sm = StripMap::make(nx, nz, CPML);
    if (sm.count() == 0) return;
    k_zeta_f_strip<<<elt_grid(sm.count()), kEltBlock>>>(p2, r2, a_x, b_x, a_z, b_z, psi_px,
                                                          psi_fz, z_px, z_fz, aten_p, aten_f, sm,
                                                          dh);
    note_launch();
}

void propagator_F_h(float *p2, float *r2, float *PF, float *P_pre, float *F_pre, float *P_past,
                    float *F_past, float *v_hor, float *v_po, float *v_nmo, float *aten_p,
                    float *aten_f, float *source, float *shot, float C, float dh2, int nx, int nz,
                    int sx, int sz, int it, int CPML)
{
    dim3 block(32, 8), grid((nx + 31) / 32, (nz + 7) / 8);
    k_propagator<<<grid, block>>>(p2, r2, PF, P_pre, F_pre, P_past, F_past, v_hor, v_po, v_nmo,
                                  aten_p, aten_f, source, shot, C, dh2, nx, nz, sx, sz, it, CPML);
    note_launch();
}

void res_h(float *Res, float *shot1, float *shot2, int nx, int nz)
{
    long n = (long)nx * nz;
    k_res<<<elt_grid(n), kEltBlock>>>(Res, shot1, shot2, n);
    note_launch();
}

void SecondDerivate_P_h(float *P_pre, float *F_pre, float *p2, float *r2, float dh2, int nx,
                        int nz)
{
    k_second_p<<<tile_grid(nx, nz), dim3(TX, BY)>>>(P_pre, F_pre, p2, r2, dh2, nx, nz);
    note_launch();
}

void launchPropagation(cudaStream_t stream1, cudaStream_t stream2, float *PF_h, float *PF,
                       float *P_past, float *P_pre, float *F_past, float *F_pre, float *p2,
                       float *r2, float dh2, int nx, int nz, float *a_x, float *b_x, float *a_z,
                       float *b_z, float *psi_px, float *psi_fz, float dh, int CPML, float *z_px,
                       float *z_fz, float *aten_p, float *aten_f, float *v_hor, float *v_po,
                       float *v_nmo, float *source, float *shot2, float C, int sx, int sz, int it)
{
    // snapshot of the previous level before this step overwrites it (src/serialcalls.cu:60)
    note(cudaMemcpyAsync(PF_h, P_past, 2 * (size_t)nx * nz * sizeof(float),
                         cudaMemcpyDeviceToHost, stream1));
    StripMap sm = StripMap::make(nx, nz, CPML);
    if (sm.count() > 0)
        k_psi_f_strip<<<elt_grid(sm.count()), kEltBlock, 0, stream2>>>(
            P_pre, F_pre, a_x, b_x, a_z, b_z, psi_px, psi_fz, sm, dh);
    // legacy default stream: waits for the copy on stream1 and the strip pass on stream2
    k_fwd_main<<<tile_grid(nx, nz), dim3(TX, BY), 0, cudaStreamLegacy>>>(
        p2, r2, PF, P_pre, F_pre, P_past, F_past, a_x, b_x, a_z, b_z, psi_px, psi_fz, z_px, z_fz,
        aten_p, aten_f, v_hor, v_po, v_nmo, source, shot2, C, dh2, dh, nx, nz, sx, sz, it, CPML);
    note_launch();
}

void launchBackPropagation(cudaStream_t stream1, cudaStream_t stream2, int nx, int nz, int nt,
                           float *PF_h, float *P_pre, float *P_past, float *F_pre, float *F_past,
                           float *aux1, float *aux2, float *aux3, float *aux4, float *v_hor,
                           float *v_po, float *v_nmo, float *p2cx, float *p2cz, float *r2dx,
                           float *r2cz, float dh2, float *P_pre2, float *F_pre2, float *a_x,
                           float *b_x, float *a_z, float *b_z, float *psixcx, float *psixcz,
                           float *psizdx, float *psizcz, float dh, int CPML, float *zitaxcx,
                           float *zitaxcz, float *zitazdx, float *zitazcz, float *atenxcx,
                           float *atenxcz, float *atenzdx, float *atenzcz, float *Res, float C,
                           float *PF, int it, int sx, int sz, float dt, float *gcx, float *gcz,
                           float *gdx)
{
    (void)PF; (void)sx;  // passed by the reference but unused by its kernels
    // snapshot back to the device (src/serialcalls.cu:76); F_pre2 = P_pre2 + nx*nz
    note(cudaMemcpyAsync(P_pre2, PF_h, 2 * (size_t)nx * nz * sizeof(float),
                         cudaMemcpyHostToDevice, stream1));
    long n = (long)nx * nz;
    k_entry_point<<<elt_grid(n), kEltBlock, 0, stream2>>>(P_pre, F_pre, aux1, aux2, aux3, aux4,
                                                           v_hor, v_po, v_nmo, n);
    StripMap sm = StripMap::make(nx, nz, CPML);
    if (sm.count() > 0)
        k_psi_r_strip<<<elt_grid(sm.count()), kEltBlock, 0, stream2>>>(
            aux1, aux2, aux3, aux4, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx, psizcz, sm, dh);
    AdjArgs a;
    a.aux1 = aux1; a.aux2 = aux2; a.aux3 = aux3; a.aux4 = aux4;
    a.p2cx = p2cx; a.p2cz = p2cz; a.r2dx = r2dx; a.r2cz = r2cz;
    a.a_x = a_x; a.b_x = b_x; a.a_z = a_z; a.b_z = b_z;
    a.psixcx = psixcx; a.psixcz = psixcz; a.psizdx = psizdx; a.psizcz = psizcz;
    a.zitaxcx = zitaxcx; a.zitaxcz = zitaxcz; a.zitazdx = zitazdx; a.zitazcz = zitazcz;
    a.atenxcx = atenxcx; a.atenxcz = atenxcz; a.atenzdx = atenzdx; a.atenzcz = atenzcz;
    a.P_pre = P_pre; a.F_pre = F_pre; a.P_past = P_past; a.F_past = F_past;
    a.Res = Res; a.P_snap = P_pre2; a.F_snap = F_pre2;
    a.gcx = gcx; a.gcz = gcz; a.gdx = gdx;
    a.C = C; a.dh2 = dh2; a.dt = dt; a.dh = dh;
    a.nx = nx; a.nz = nz; a.nt = nt; a.sz = sz; a.it = it; a.cpml = CPML;
    // legacy default stream: after the H2D copy (stream1) and the strip pass (stream2)
    k_adj_main<<<tile_grid(nx, nz), dim3(TX, BY), 0, cudaStreamLegacy>>>(a);
    note_launch();
}

void NORMAL_h(float *gcx, float *gcz, float *gdx, int nx, int nz, float ngcx, float ngcz,
              float ngdx)
{
    long n = (long)nx * nz;
    k_normal<<<elt_grid(n), kEltBlock>>>(gcx, gcz, gdx, nx, nz, ngcx, ngcz, ngdx);
    note_launch();
}

void UpdateModel_h(float *gcx, float *gcz, float *gdx, float *v_hor, float *v_po, float *v_nmo,
                   float alpha1, float alpha2, float alpha3, int nx, int nz)
{
    long n = (long)nx * nz;
    k_update_model<<<elt_grid(n), kEltBlock>>>(gcx, gcz, gdx, v_hor, v_po, v_nmo, alpha1, alpha2,
                                               alpha3, nx, nz);
    note_launch();
}

void compute_sy_h(float *s_vp, float *s_vn, float *s_vh, float *y_b1, float *y_b2, float *y_b3,
                  float *vp, float *vn, float *vh, float *back_vp, float *back_vn, float *back_vh,
                  float *b1, float *b2, float *b3, float *back_b1, float *back_b2, float *back_b3,
                  int nx, int nz, int k)
{
    long n = (long)nx * nz;
    k_compute_sy<<<elt_grid(n), kEltBlock>>>(s_vp, s_vn, s_vh, y_b1, y_b2, y_b3, vp, vn, vh,
                                             back_vp, back_vn, back_vh, b1, b2, b3, back_b1,
                                             back_b2, back_b3, n, (long)k * n);
    note_launch();
}

void compute_qi_h(float *q_b1, float *q_b2, float *q_b3, float *y_b1, float *y_b2, float *y_b3,
                  float epsilon_v, float epsilon_d, float epsilon_e, int nx, int nz, int k)
{
    long n = (long)nx * nz;
    k_axpy3<<<elt_grid(n), kEltBlock>>>(q_b1, q_b2, q_b3, y_b1, y_b2, y_b3, epsilon_v, epsilon_d,
                                        epsilon_e, n, (long)k * n);
    note_launch();
}

void compute_ri_h(float *r_b1, float *r_b2, float *r_b3, float *q_b1, float *q_b2, float *q_b3,
                  float gamma_v, float gamma_d, float gamma_e, int nx, int nz)
{
    long n = (long)nx * nz;
    k_scale3<<<elt_grid(n), kEltBlock>>>(r_b1, r_b2, r_b3, q_b1, q_b2, q_b3, gamma_v, gamma_d,
                                         gamma_e, n);
    note_launch();
}

void update_r_h(float *r_b1, float *r_b2, float *r_b3, float *s_vp, float *s_vn, float *s_vh,
                float epsilon_v, float epsilon_d, float epsilon_e, float beta_v, float beta_d,
                float beta_e, int nx, int nz, int k)
{
    long n = (long)nx * nz;
    k_update_r<<<elt_grid(n), kEltBlock>>>(r_b1, r_b2, r_b3, s_vp, s_vn, s_vh, epsilon_v - beta_v,
                                           epsilon_d - beta_d, epsilon_e - beta_e, n, (long)k * n);
    note_launch();
}

void update_LBFGS_h(float *r_b1, float *r_b2, float *r_b3, float *vp, float *vn, float *vh,
                    float *back_vp, float *back_vn, float *back_vh, int nx, int nz,
                    float alpha_v, float alpha_d, float alpha_e, int flag_v, int flag_d,
                    int flag_e, int flag_min, int flag_max)
{
    long n = (long)nx * nz;
    k_update_lbfgs<<<elt_grid(n), kEltBlock>>>(r_b1, r_b2, r_b3, vp, vn, vh, back_vp, back_vn,
                                               back_vh, nx, nz, alpha_v, alpha_d, alpha_e, flag_v,
                                               flag_d, flag_e, flag_min, flag_max);
    note_launch();
}

}  // extern "C"
