// Native context of the FWI gradient library (include/fwi.h).
//
// One context = one device, one stream, one arena of device memory.  A
// gradient call runs the shots in batches of up to max_shots:
//   forward (FP32: strip pass and layer tiles on a side stream beside the
//   interior tiles, 3 launches / step; FP64: 2), images kept per the
//   storage mode
//   -> residual + FP64 misfit partials
//   -> adjoint + imaging (3 launches / step in FP32, 2 in FP64)
//   -> deterministic reduction of the per-shot gradients into the model grid.
// The L-BFGS update of src/main.c:539-800 runs on the device with FP64 dot
// products reduced by the last block to finish (no host round trip).
#include "../../include/fwi.h"
#include "common.cuh"
#include "prop.h"
#include "tma.cuh"

#include <cuda_fp16.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace fwi {

EncodeTiledFn tensor_map_encoder()
{
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

int make_tensor_map_3d(CUtensorMap *map, const void *base, CUtensorMapDataType type, int elem, long pitch,
                       long rows, long depth, int bx, int by, int bz)
{
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return FWI_ERR_NODEVICE;
    cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)rows, (cuuint64_t)depth};
    cuuint64_t strides[2] = {(cuuint64_t)(pitch * elem), (cuuint64_t)(pitch * rows * elem)};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(map, type, 3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? FWI_OK : FWI_ERR_CUDA;
}

// Mirrors the layout of fwi::TmaMaps in prop_tma.cuh (device code is not
// compiled into this unit).
struct HostTmaMaps {
    CUtensorMap lvl[4];
    CUtensorMap px[2];
    CUtensorMap fz[2];
    CUtensorMap mx[8];
    CUtensorMap mz[8];
    CUtensorMap inc[2];
};
static_assert(sizeof(HostTmaMaps) == 26 * sizeof(CUtensorMap), "HostTmaMaps mirrors TmaMaps");

}  // namespace fwi

namespace {

using fwi::Batch;
using fwi::DevShot;

int status_from_cuda(cudaError_t e)
{
    if (e == cudaSuccess) return FWI_OK;
    if (e == cudaErrorMemoryAllocation) return FWI_ERR_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
        return FWI_ERR_NODEVICE;
    return FWI_ERR_CUDA;
}

constexpr int kLayer = 15;  // near-surface rows never updated (include/parallelcalls.h:6)
constexpr int kMaxHist = 16;
constexpr int kRedThreads = 256;  // reduction grids: 2 blocks of kRedThreads per SM of the device

long round_up(long v, long m) { return (v + m - 1) / m * m; }

// ------------------------------------------------------------------ small kernels

template <typename T>
__global__ void k_scale_models(const T *vh, const T *vp, const T *vn, T *mh, T *mp, T *mn, T dt2, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        mh[i] = dt2 * vh[i];
        mp[i] = dt2 * vp[i];
        mn[i] = dt2 * vn[i];
    }
}

template <typename T>
__global__ void k_pre_variables(const T *vel, const T *eps, const T *del, T *vh, T *vp, T *vn, int nx,
                                int nz, int mpitch)
{
    long n = (long)nx * nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        long iz = k / nx, ix = k - iz * nx, i = iz * mpitch + ix;
        T v2 = vel[k] * vel[k];
        vp[i] = v2;
        vh[i] = v2 * (T(1) + T(2) * eps[k]);
        vn[i] = v2 * (T(1) + T(2) * del[k]);
    }
}

// CPML a, b by distance d = 1..cpml into the layer (src/parallelcalls.cu:25-26):
// d0 Vmax (d dh / L)^2 and pi f (L - d dh) / L in FP64 from T inputs, b
// rounded to T before a = d (b - 1) / (d + alpha) is formed, as the reference
// does with T = float.
template <typename T>
__global__ void k_cpml_table(T *a, T *b, int cpml, T vmax, T dt, T dh, T f, T d0, T L)
{
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d > cpml) return;
    if (d == 0) { a[0] = T(0); b[0] = T(0); return; }
    T frac = d * dh / L;
    double dd = (double)(d0 * vmax) * ((double)frac * (double)frac);
    double al = 3.141592653589793 * (double)f * (double)(L - d * dh) / (double)L;
    T bT = (T)exp(-(dd + al) * (double)dt);
    b[d] = bT;
    a[d] = (T)(dd * (double)(bT - T(1)) / (dd + al));
}

// rec := mask (rec - obs); per-block partial sums of rec^2 (FP64).
template <typename T>
__global__ void k_residual(T *rec, const T *obs, const unsigned char *mask, const DevShot *shots,
                           const long *mask_off, double *partial)
{
    const int s = blockIdx.y;
    const DevShot sh = shots[s];
    const int nrec = sh.rx1 - sh.rx0;
    const long n = (long)sh.nt * nrec;
    double acc = 0.0;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const long e = sh.rec_off + k;
        T d = rec[e] - obs[e];
        if (mask && !mask[mask_off[s] + (k % nrec)]) d = T(0);
        rec[e] = d;
        acc += (double)d * (double)d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += w[q];
        partial[(long)s * gridDim.x + blockIdx.x] = t;
    }
}

// misfit += 1/2 sum of partials, in a fixed order
__global__ void k_misfit_finish(const double *partial, long n, double *misfit)
{
    __shared__ double w[32];
    double acc = 0.0;
    for (long k = threadIdx.x; k < n; k += blockDim.x) acc += partial[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += w[q];
        *misfit += 0.5 * t;
    }
}

// grad[iz][X] += sum over the batch's gradient slots (fixed order); slot q
// has the window of shot q sg (callers pass sg = 1 when every slot shares
// one window).
template <typename T>
__global__ void k_accumulate_gradient(T *gh, T *gp, T *gn, const T *sh_h, const T *sh_p, const T *sh_n,
                                      const DevShot *shots, int ngroups, int sg, int nx, int nz, int mpitch,
                                      int pitch, long slot)
{
    const long n = (long)nx * nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k / nx), X = (int)(k - (long)iz * nx);
        T a = T(0), b = T(0), c = T(0);
        for (int q = 0; q < ngroups; q++) {
            const DevShot &w = shots[q * sg];
            const int lx = X - w.x0;
            if (lx < 0 || lx >= w.nx) continue;
            const long i = (long)q * slot + (long)iz * pitch + lx;
            a += sh_h[i];
            b += sh_p[i];
            c += sh_n[i];
        }
        const long o = (long)iz * mpitch + X;
        gh[o] += a;
        gp[o] += b;
        gn[o] += c;
    }
}

// ------------------------------------------------------------------ observed data kept on the device

// Per-trace scale of a compact (FP16) record store: trace r of a shot is the column r of its
// [nt][nrec] block.  scale = max |d| / 32768, so that every value maps below FP16's largest.
template <typename T>
__global__ void k_trace_scale(const T *d, long off, int nt, int nrec, float *scale)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    float m = 0.f;
    for (int t = 0; t < nt; t++) m = fmaxf(m, fabsf((float)d[off + (long)t * nrec + r]));
    scale[r] = m > 0.f ? m / 32768.f : 1.f;
}

template <typename T>
__global__ void k_trace_encode(const T *d, long in_off, int nt, int nrec, const float *scale, __half *out,
                               long out_off)
{
    const long n = (long)nt * nrec;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        out[out_off + k] = __float2half_rn((float)d[in_off + k] / scale[k % nrec]);
}

template <typename T>
__global__ void k_trace_decode(const __half *in, long off, int nt, int nrec, const float *scale, T *out, long out_off)
{
    const long n = (long)nt * nrec;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        out[out_off + k] = (T)(__half2float(in[off + k]) * scale[k % nrec]);
}

// ------------------------------------------------------------------ L-BFGS on the device

// Three-parameter dot products with a last-block-done FP64 reduction.
struct DotScratch {
    double *partial;    // [reduction blocks][4][3]
    unsigned *counter;  // one per kernel sequence position
};

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Reduces up to 4 x 3 per-thread values into partial[block], then the last
// block to arrive sums all partials in block order into out[4][3].
__device__ void reduce_last_block(double (&v)[4][3], int nv, DotScratch ds, double *out)
{
    __shared__ double sm[8][12];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int a = 0; a < nv; a++)
        for (int p = 0; p < 3; p++) {
            double t = warp_sum(v[a][p]);
            if (lane == 0) sm[warp][a * 3 + p] = t;
        }
    __syncthreads();
    if (threadIdx.x < nv * 3) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w][threadIdx.x];
        ds.partial[(long)blockIdx.x * 12 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(ds.counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x < nv * 3) {
        double t = 0.0;
        for (int bI = 0; bI < (int)gridDim.x; bI++) t += ((volatile double *)ds.partial)[(long)bI * 12 + threadIdx.x];
        out[threadIdx.x] = t;
    }
    if (threadIdx.x == 0) *ds.counter = 0u;
}

template <typename T> struct Tri {
    T *p[3];
};
template <typename T> struct CTri {
    const T *p[3];
};

// s_k = m - m_back, y_k = g - g_back (3 parameters), and the dots y.s, y.y, s.g, s.s.
template <typename T>
__global__ void k_lb_pair(Tri<T> s, Tri<T> y, CTri<T> m, CTri<T> mb, CTri<T> g, CTri<T> gb, long n,
                          DotScratch ds, double *out)
{
    double v[4][3] = {};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        for (int p = 0; p < 3; p++) {
            T sv = m.p[p][i] - mb.p[p][i], yv = g.p[p][i] - gb.p[p][i];
            s.p[p][i] = sv;
            y.p[p][i] = yv;
            v[0][p] += (double)yv * sv;
            v[1][p] += (double)yv * yv;
            v[2][p] += (double)sv * g.p[p][i];
            v[3][p] += (double)sv * sv;
        }
    reduce_last_block(v, 4, ds, out);
}

// v := w (copy) and the dots a.w for the first loop's first slot.
template <typename T>
__global__ void k_lb_copy_dot(Tri<T> dst, CTri<T> src, CTri<T> a, long n, DotScratch ds, double *out)
{
    double v[4][3] = {};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        for (int p = 0; p < 3; p++) {
            T w = src.p[p][i];
            dst.p[p][i] = w;
            v[0][p] += (double)a.p[p][i] * w;
        }
    reduce_last_block(v, 1, ds, out);
}

// x := c0 * x + c1 * u (per-parameter scalars from device memory, FP64), then
// the dots b.x for the next step (b may be null).
template <typename T>
__global__ void k_lb_axpy_dot(Tri<T> x, CTri<T> u, const double *c0, const double *c1, CTri<T> bnext,
                              int has_next, long n, DotScratch ds, double *out)
{
    double v[4][3] = {};
    double k0[3], k1[3];
    for (int p = 0; p < 3; p++) { k0[p] = c0 ? c0[p] : 1.0; k1[p] = c1 ? c1[p] : 0.0; }
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        for (int p = 0; p < 3; p++) {
            T xv = (T)(k0[p] * (double)x.p[p][i] + (u.p[p] ? k1[p] * (double)u.p[p][i] : 0.0));
            x.p[p][i] = xv;
            if (has_next) v[0][p] += (double)bnext.p[p][i] * xv;
        }
    if (has_next) reduce_last_block(v, 1, ds, out);
}

// Scalar bookkeeping of the two-loop recursion (one thread).
struct LbScalars {
    double rho[3][kMaxHist];
    double alpha[3][kMaxHist];
    double ys[3][kMaxHist], yy[3][kMaxHist];  // curvature of each slot's pair when it was formed
    double gamma[3];
    double coefA[3], coefB[3];  // scratch coefficients for the next axpy
    double dots[12];
    double pair[12];            // y.s, y.y, s.g, s.s of the newest pair
};

// History slots newest .. oldest, for the scaling of the initial matrix.
struct LbOrder {
    int n;
    int slot[kMaxHist];
};

// mode 0: newest pair formed: rho_k = 1/(y.s), first-loop alpha_k = rho_k (s_k.q) with q = g;
//         with `guard`, a pair whose y.s <= 0 (no positive curvature along s) gets rho = 0 and so
//         takes no part in either loop
// mode 1: alpha_l = rho_l (s_l.q) from dots[0..2]
// mode 3: beta = rho_l (y_l.r) from dots; coefB = alpha_l - beta
__global__ void k_lb_scalar(LbScalars *S, int mode, int slot, int guard)
{
    if (threadIdx.x != 0) return;
    for (int p = 0; p < 3; p++) {
        if (mode == 0) {
            S->ys[p][slot] = S->pair[p];
            S->yy[p][slot] = S->pair[3 + p];
            S->rho[p][slot] = (guard && !(S->pair[p] > 0.0)) ? 0.0 : 1.0 / S->pair[p];
            S->alpha[p][slot] = S->rho[p][slot] * S->pair[6 + p];
            S->coefB[p] = -S->alpha[p][slot];
        } else if (mode == 1) {
            S->alpha[p][slot] = S->rho[p][slot] * S->dots[p];
            S->coefB[p] = -S->alpha[p][slot];
        } else {
            double beta = S->rho[p][slot] * S->dots[p];
            S->coefB[p] = S->alpha[p][slot] - beta;
        }
    }
}

// Scaling of the initial matrix, coefA = gamma = (s.y)/(y.y) of the newest pair (src/main.c:622-655).
// With `guard`: of the newest pair with positive curvature; without one, |s| / |y| of the newest
// pair (a step as long as the last one, along the gradient).
__global__ void k_lb_gamma(LbScalars *S, LbOrder o, int guard)
{
    if (threadIdx.x != 0) return;
    for (int p = 0; p < 3; p++) {
        double gam = S->pair[p] / S->pair[3 + p];
        if (guard) {
            gam = sqrt(S->pair[9 + p] / S->pair[3 + p]);
            for (int a = 0; a < o.n; a++) {
                const int l = o.slot[a];
                if (S->ys[p][l] > 0.0) {
                    gam = S->ys[p][l] / S->yy[p][l];
                    break;
                }
            }
        }
        S->gamma[p] = gam;
        S->coefA[p] = gam;
    }
}

// First-iteration scale 1/|g| (src/main.c:551-561).
__global__ void k_lb_inv_norm(LbScalars *S)
{
    if (threadIdx.x != 0) return;
    for (int p = 0; p < 3; p++) S->coefA[p] = 1.0 / sqrt(S->dots[p]);
}

// v -= a_p * g * coefA_p below the layer, v_hor >= v_nmo (src/parallelcalls.cu:273-286).
template <typename T>
__global__ void k_first_update(T *vh, T *vp, T *vn, const T *gh, const T *gp, const T *gn, const LbScalars *S,
                               float a_hor, float a_po, float a_nmo, int nx, int nz, int mpitch)
{
    long n = (long)nx * (nz - kLayer - 1);
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        long iz = kLayer + 1 + k / nx, ix = k % nx, i = iz * mpitch + ix;
        vp[i] = vp[i] - (T)(a_po * (gp[i] * S->coefA[1]));
        T vnn = vn[i] - (T)(a_nmo * (gn[i] * S->coefA[2]));
        T vhn = vh[i] - (T)(a_hor * (gh[i] * S->coefA[0]));
        vn[i] = vnn;
        vh[i] = vhn < vnn ? vnn : vhn;
    }
}

// Directional derivative of the misfit along the trial step m_back - alpha r:
// out[p] = sum of g_p r_p over the rows the update changes (iz > kLayer), FP64.
template <typename T>
__global__ void k_lb_slope(CTri<T> g, CTri<T> r, int nx, int nz, int mpitch, DotScratch ds, double *out)
{
    double v[4][3] = {};
    const long n = (long)nx * (nz - kLayer - 1);
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const long iz = kLayer + 1 + k / nx, ix = k % nx, i = iz * mpitch + ix;
        for (int p = 0; p < 3; p++) v[0][p] += (double)g.p[p][i] * r.p[p][i];
    }
    reduce_last_block(v, 1, ds, out);
}

// Trial model (src/parallelcalls.cu:343-404) for all three parameters.
template <typename T>
__global__ void k_lb_update(T *vh, T *vp, T *vn, const T *bh, const T *bp, const T *bn, const T *rh,
                            const T *rp, const T *rn, float av, float ad, float ae, int fmin, int fmax,
                            int nx, int nz, int mpitch)
{
    long n = (long)nx * (nz - kLayer - 1);
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        long iz = kLayer + 1 + k / nx, ix = k % nx, i = iz * mpitch + ix;
        T p = bp[i] - (T)av * rp[i];
        if (fmax == 1 && p > T(3.5e6)) p = T(3.5e6);
        if (fmin == 1 && p < T(1.8e6)) p = T(1.8e6);
        vp[i] = p;
        T q = bn[i] - (T)ad * rn[i];
        if (fmax == 1 && q > T(4e6)) q = T(4e6);
        if (fmin == 1 && q < T(1.8e6)) q = T(1.8e6);
        vn[i] = q;
        T h = bh[i] - (T)ae * rh[i];
        if (fmax == 1 && h > T(4.5e6)) h = T(4.5e6);
        if (fmin == 1 && h < T(1.8e6)) h = T(1.8e6);
        vh[i] = h < q ? q : h;
    }
}

// dJ/dVp, dJ/deps, dJ/ddelta from the squared-velocity gradients.
template <typename T>
__global__ void k_grad_vti(const T *vh, const T *vp, const T *vn, const T *gh, const T *gp, const T *gn, T *ovp,
                           T *oeps, T *odel, int nx, int nz, int mpitch)
{
    long n = (long)nx * nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        long iz = k / nx, ix = k - iz * nx, i = iz * mpitch + ix;
        T v2 = vp[i];
        T vel = sqrt(v2);
        T ope = vh[i] / v2, opd = vn[i] / v2;  // 1 + 2 eps, 1 + 2 delta
        ovp[i] = T(2) * vel * (gp[i] + ope * gh[i] + opd * gn[i]);
        oeps[i] = T(2) * v2 * gh[i];
        odel[i] = T(2) * v2 * gn[i];
    }
}

// Steps between checkpoints: minimises checkpoint memory (8 full arrays each,
// nt / K of them) plus segment image memory (two segments in flight, 2
// arrays of the image type per step: 4 K) for nt steps.
int checkpoint_interval(const fwi_config &c)
{
    if (c.ckpt_every > 0) return std::min(c.ckpt_every, c.nt_max);
    const double img = c.store_prec == FWI_SPREC_NATIVE ? 1.0 : 0.5 * (c.precision == FWI_PREC_FP64 ? 0.5 : 1.0);
    int k = (int)std::ceil(std::sqrt(8.0 * c.nt_max / (4.0 * img)));
    return std::max(1, std::min(k, c.nt_max));
}

// Grid of a grid-stride element-wise kernel of 256-thread blocks: at most 8 blocks per SM.
inline unsigned elt_grid(long n, int n_sm)
{
    long b = (n + 255) / 256;
    return (unsigned)std::max(1L, std::min(b, 8L * n_sm));
}

// Check of the bounded pipeline wait (fwi_check_bounded_wait): one block
// waits, as the tile passes do, on an mbarrier phase that nothing completes
// (no thread arrives, no copy is in flight), gives up after `polls` polls and
// records kStatusTimeout in the status word, then returns.
__global__ void k_check_bounded_wait(unsigned *status, long polls)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        fwi::mbar_init(&bar, 1);
        fwi::mbar_init_fence();
    }
    __syncthreads();
    const bool ok = fwi::mbar_wait(&bar, 0, polls);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(status, fwi::kStatusTimeout);
}

// Host range on the profiler timelines (NVTX; nothing without a tool attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ------------------------------------------------------------------ the context

struct CtxBase {
    fwi_config cfg{};
    int last_cuda = 0;
    int n_sm = 1;        // streaming multiprocessors of the context's device
    int red_blocks = 2;  // blocks of the reduction kernels: 2 per SM
    unsigned eg(long n) const { return elt_grid(n, n_sm); }
    float timing[4] = {0, 0, 0, 0};
    long launches = 0;

    // Interior tile timing (fwi_set_tile_timing): event pairs around the
    // interior tile launches of up to kTimeSamples sampled steps per phase
    // (0 forward, 1 adjoint, 2 the forward steps of a checkpoint segment's
    // recompute, which run beside the adjoint), with the interior points each
    // launch updated; recompute_steps: forward steps the last call recomputed.
    static constexpr int kTimeSamples = 16;
    static constexpr int kPhases = 3;
    bool tile_timing = false;
    cudaEvent_t tev[kPhases][kTimeSamples][2] = {};
    double tile_ms[kPhases] = {0, 0, 0}, tile_pts[kPhases] = {0, 0, 0};
    long tile_n[kPhases] = {0, 0, 0};
    long recompute_steps = 0;
    // CUDA graphs of the batch sections (Ctx<T>::run_section): on/off, sections
    // replayed and captured
    bool graphs = true;
    long graph_replays = 0, graph_captures = 0;
    virtual void drop_sections() {}
    int set_graphs(bool on)
    {
        if (!on) drop_sections();
        graphs = on;
        return FWI_OK;
    }

    int set_tile_timing(bool on)
    {
        if (on && !tev[0][0][0])
            for (auto &ph : tev)
                for (auto &pr : ph)
                    for (auto &e : pr) {
                        const cudaError_t r = cudaEventCreate(&e);
                        if (r != cudaSuccess) return fail(r);
                    }
        tile_timing = on;
        return FWI_OK;
    }

    virtual ~CtxBase()
    {
        for (auto &ph : tev)
            for (auto &pr : ph)
                for (auto &e : pr)
                    if (e) cudaEventDestroy(e);
    }
    virtual int init() = 0;
    virtual int set_model(const void *, const void *, const void *) = 0;
    virtual int set_model_vti(const void *, const void *, const void *) = 0;
    virtual int get_model(void *, void *, void *) = 0;
    virtual int set_wavelet(const void *, int) = 0;
    virtual int set_ricker(float, int) = 0;
    virtual int set_frequency(float, int) = 0;
    virtual int run(const fwi_shot *, int, const void *, const unsigned char *, void *, void *, void *,
                    double *, void *traces, bool grad) = 0;
    virtual int autotune(const fwi_shot *, int, int, fwi_tuning *) = 0;
    virtual int store_observed(const fwi_shot *, int, const void *, int) = 0;
    virtual int model_observed(const fwi_shot *, int, const void *, const void *, const void *, int) = 0;
    virtual int free_observed() = 0;
    virtual int set_tuning(const fwi_shot *, int, const fwi_tuning *) = 0;
    virtual int check_bounded_wait(long polls) = 0;
    virtual int first_step(float, float, float) = 0;
    virtual int lbfgs_direction(int, double *) = 0;
    virtual void set_lbfgs_guard(int) = 0;
    virtual int lbfgs_update(float, float, float, int, int) = 0;
    virtual int direction_slope(double *) = 0;
    virtual int restore_model() = 0;
    virtual int gradient_vti(void *, void *, void *) = 0;
    virtual int set_gradient(const void *, const void *, const void *) = 0;
    int fail(cudaError_t e)
    {
        last_cuda = (int)e;
        cudaGetLastError();
        return status_from_cuda(e);
    }
};

#define TRY(expr)                                        \
    do {                                                 \
        cudaError_t e_ = (expr);                         \
        if (e_ != cudaSuccess) return fail(e_);          \
    } while (0)
#define TRY_LAUNCH() TRY(cudaGetLastError())

template <typename T> struct Ctx : CtxBase {
    int nx = 0, nz = 0, mpitch = 0, pitch = 0, B = 0, nt_max = 0, nrec_max = 0, n_img = 0;
    long slot = 0, mslot = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {};
    fwi::StepStreams ss{};  // st, plus the side streams of the FP32 step (prop_f32.cu)


    // Interior points of the interior tiles of a window nxw wide (tile_role 1
    // for width aw) on the tile grid from (xbase, zbase).
    long interior_tile_points(int nxw, int aw, int xbase, int zbase) const
    {
        long n = 0;
        for (int z0 = zbase; z0 < nz; z0 += fwi::kTileEdge)
            for (int x0 = xbase; x0 < nxw; x0 += fwi::kTileEdge)
                if (fwi::tile_role(x0, z0, nxw, nz, aw) == 1) {
                    const long w = std::min(x0 + fwi::kTileEdge - 1, nxw - 5) - std::max(x0, 4) + 1;
                    const long h = std::min(z0 + fwi::kTileEdge - 1, nz - 5) - std::max(z0, 4) + 1;
                    n += w * h;
                }
        return n;
    }


    std::vector<void *> allocs;
    // model and setup
    T *vh = nullptr, *vp = nullptr, *vn = nullptr, *mh = nullptr, *mp = nullptr, *mn = nullptr;
    T *cpa = nullptr, *cpb = nullptr, *wavelet = nullptr;
    bool have_model = false, have_wavelet = false, models_dirty = true;
    int wavelet_nt = 0;
    // batch
    T *lvl[6] = {}, *cp[8] = {}, *gs[3] = {};
    void *store = nullptr;
    // boundary storage: ring of every step [B][nt_max][ring_len], rebuild state in rlvl.
    T *ring = nullptr;
    long ring_len = 0;
    // Checkpoint and boundary storage rebuild images on their own streams (rss)
    // ahead of the adjoint, into two halves of the image buffer: ev_reb[h] =
    // half h rebuilt, ev_adj[h] = half h consumed by the adjoint.
    cudaStream_t rst = nullptr;
    fwi::StepStreams rss{};
    cudaEvent_t ev_rfork = nullptr, ev_reb[2] = {}, ev_adj[2] = {};
    // checkpointing: full states every ck_every steps, segment recompute buffers
    int ck_every = 0, n_ck = 0;
    T *ck = nullptr;                 // [n_ck][8][B * slot]: P, F, their increments, CPML x4
    T *rlvl[6] = {}, *rcp[4] = {};
    // TMA tensor maps of the batch buffers and of the recompute buffers (FP32 contexts)
    fwi::HostTmaMaps maps{}, rmaps{};
    bool use_tma = false;

    // CUDA graphs of the two sections of a batch (the forward steps; the
    // adjoint with its rebuild or recompute streams and the gradient sum).
    // A section is keyed by every launch parameter it bakes in; it is issued
    // directly the first time its key is seen, captured and instantiated the
    // second time, replayed after that.  Every buffer it uses lives as long
    // as the context, so a graph stays valid for its key.  FWI_GRAPHS=0:
    // always direct.
    struct Section {
        std::vector<long> key;
        cudaGraphExec_t exec = nullptr;
        long launches = 0;              // kernel launches of the section
        unsigned phases = 0;            // tile timing phases it samples (bit p: phase p) ...
        int nsamp[kPhases] = {};        // ... their sample counts and points
        double spts[kPhases][kTimeSamples] = {};
        long rsteps = 0;                // forward steps of segment recomputes it runs
        unsigned long long used = 0;
    };
    static constexpr int kSections = 6;
    std::vector<Section> sections;
    unsigned long long section_clock = 0;

    static void key_add(std::vector<long> &k, const void *p) { k.push_back((long)(uintptr_t)p); }
    static void key_add(std::vector<long> &k, long v) { k.push_back(v); }
    static void key_add(std::vector<long> &k, double v)
    {
        long bits = 0;
        std::memcpy(&bits, &v, sizeof(bits));
        k.push_back(bits);
    }

    // Every field of a batch view (the kernels take it by value).
    static void key_batch(std::vector<long> &k, const Batch<T> &b)
    {
        for (long v : {(long)b.B, (long)b.nz, (long)b.pitch, (long)b.mpitch, (long)b.cpml, (long)b.nt_max, b.slot,
                       (long)b.store_type, (long)b.n_img, (long)b.sg, (long)b.sg_layer, (long)b.xbase, (long)b.zbase,
                       (long)b.inline_strip, (long)b.mixed})
            key_add(k, v);
        for (const void *p : {(const void *)b.store, (const void *)b.scale, (const void *)b.amax,
                              (const void *)b.rec, (const void *)b.shots, (const void *)b.mh, (const void *)b.mp,
                              (const void *)b.mn, (const void *)b.cpa, (const void *)b.cpb, (const void *)b.wavelet,
                              (const void *)b.status, b.tma})
            key_add(k, p);
        for (int l = 0; l < 4; l++) {
            key_add(k, (const void *)b.tiles[l]);
            key_add(k, (long)b.ntiles[l]);
        }
        for (const T *p : b.lvl) key_add(k, (const void *)p);
        for (const T *p : b.cp) key_add(k, (const void *)p);
        for (const T *p : b.g) key_add(k, (const void *)p);
        for (double v : {(double)b.inv_dh, (double)b.inv_dh2, (double)b.img_scale}) key_add(k, v);
    }

    void drop_sections() override
    {
        for (Section &s : sections)
            if (s.exec) cudaGraphExecDestroy(s.exec);
        sections.clear();
    }

    // Issues `body` (launches on st and on streams it joins back into st) as
    // the section `key`: directly, or captured into a graph, or by replaying
    // the graph.  The section's host bookkeeping (launch count, recomputed
    // steps, timing samples of the phases in the mask `phases`: nsamp[p] and
    // the points rows spts[p]) is kept with it for the replays.
    template <typename F>
    int run_section(const std::vector<long> &key, unsigned phases, int *nsamp, double (*spts)[kTimeSamples], F body)
    {
        Section *s = nullptr;
        for (Section &c : sections)
            if (c.key == key) s = &c;
        if (s && s->exec) {
            s->used = ++section_clock;
            TRY(cudaGraphLaunch(s->exec, st));
            launches += s->launches;
            recompute_steps += s->rsteps;
            for (int p = 0; p < kPhases; p++)
                if (phases >> p & 1) {
                    nsamp[p] = s->nsamp[p];
                    std::copy(s->spts[p], s->spts[p] + kTimeSamples, spts[p]);
                }
            graph_replays++;
            return FWI_OK;
        }
        const bool capture = graphs && s != nullptr;
        if (!s) {
            if ((int)sections.size() >= kSections) {  // evict the least recently used
                auto lru = std::min_element(sections.begin(), sections.end(),
                                            [](const Section &a, const Section &c) { return a.used < c.used; });
                if (lru->exec) cudaGraphExecDestroy(lru->exec);
                sections.erase(lru);
            }
            sections.emplace_back();
            s = &sections.back();
            s->key = key;
        }
        s->used = ++section_clock;
        s->phases = phases;
        const long l0 = launches, r0 = recompute_steps;
        if (capture) TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = body();
        if (capture) {
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (rc == FWI_OK && e == cudaSuccess)
                e = cudaGraphInstantiateWithFlags(&s->exec, g, cudaGraphInstantiateFlagUseNodePriority);
            if (rc == FWI_OK && e == cudaSuccess) graph_captures++;
            if (g) cudaGraphDestroy(g);
            if (rc != FWI_OK) return rc;
            if (e != cudaSuccess) {
                s->exec = nullptr;
                return fail(e);
            }
            TRY(cudaGraphLaunch(s->exec, st));  // the captured work has not run yet
        }
        if (rc != FWI_OK) return rc;
        s->launches = launches - l0;
        s->rsteps = recompute_steps - r0;
        for (int p = 0; p < kPhases; p++)
            if (phases >> p & 1) {
                s->nsamp[p] = nsamp[p];
                std::copy(spts[p], spts[p] + kTimeSamples, s->spts[p]);
            }
        return FWI_OK;
    }
    float *scale = nullptr, *amax = nullptr;
    T *rec = nullptr, *obs = nullptr;
    unsigned char *mask = nullptr;
    long *mask_off = nullptr;
    DevShot *shots = nullptr;
    unsigned *status = nullptr;
    double *partial = nullptr, *misfit = nullptr;
    // gradient and L-BFGS
    T *grad[3] = {};
    bool have_grad = false;
    T *mb[3] = {}, *gb[3] = {}, *q[3] = {}, *r[3] = {};
    T *hs[kMaxHist][3] = {}, *hy[kMaxHist][3] = {};
    int hist_m = 0, hist_count = 0, hist_next = 0;
    bool have_back = false;
    bool have_dir = false;  // r holds an L-BFGS direction from (mb, gb)
    LbScalars *lbs = nullptr;
    int lb_guard = 0;  // fwi_set_lbfgs_guard: skip pairs without positive curvature
    DotScratch ds{};
    T *vti_out[3] = {};
    // observed data kept on the device (fwi_store_observed / fwi_model_observed): the records of
    // the shots ostore_shots, laid out as fwi_gradient takes them, in FP32 (ostore) or FP16 with
    // one scale per trace (ostore_h, ostore_scale; scale of trace r of shot k at moff[k] + r)
    std::vector<fwi_shot> ostore_shots;
    std::vector<long> ostore_off, ostore_moff;
    T *ostore = nullptr;
    __half *ostore_h = nullptr;
    float *ostore_scale = nullptr;
    T *ostore_tmp = nullptr, *model_keep[3] = {};

    ~Ctx() override
    {
        if (st) cudaStreamSynchronize(st);
        drop_sections();
        for (void *p : allocs) cudaFree(p);
        for (const TileListEntry &e : tile_lists) cudaFree(e.dev);
        free_observed();  // (the store's scratch and the kept model are among allocs)
        if (ss.side) cudaStreamSynchronize(ss.side);
        if (rst) cudaStreamSynchronize(rst);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        for (int k = 0; k < 2; k++) {
            if (ev_reb[k]) cudaEventDestroy(ev_reb[k]);
            if (ev_adj[k]) cudaEventDestroy(ev_adj[k]);
        }
        if (ev_rfork) cudaEventDestroy(ev_rfork);
        if (rss.side) cudaStreamSynchronize(rss.side);
        for (cudaEvent_t e : {rss.fork, rss.join})
            if (e) cudaEventDestroy(e);
        if (rss.side) cudaStreamDestroy(rss.side);
        if (rst) cudaStreamDestroy(rst);
        for (cudaEvent_t e : {ss.fork, ss.join})
            if (e) cudaEventDestroy(e);
        if (ss.side) cudaStreamDestroy(ss.side);
        if (st) cudaStreamDestroy(st);
    }

    template <typename U> cudaError_t alloc(U **p, size_t count)
    {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(U));
        if (e == cudaSuccess) allocs.push_back(q);
        *p = (U *)q;
        return e;
    }

    int store_type() const
    {
        if (cfg.store_prec == FWI_SPREC_FP16) return fwi::kStoreHalf;
        if (cfg.store_prec == FWI_SPREC_BF16) return fwi::kStoreBf16;
        return fwi::kStoreNative;
    }
    size_t store_elem() const { return store_type() == fwi::kStoreNative ? sizeof(T) : 2; }

    int init() override
    {
        nx = cfg.nx;
        nz = cfg.nz;
        mpitch = (int)round_up(nx, 32);
        const int win = cfg.max_window > 0 ? cfg.max_window : nx;
        pitch = (int)round_up(win, 32);
        B = cfg.max_shots;
        nt_max = cfg.nt_max;
        nrec_max = cfg.max_receivers > 0 ? cfg.max_receivers : win;
        slot = (long)nz * pitch;
        mslot = (long)nz * mpitch;
        n_img = nt_max;
        TRY(cudaSetDevice(cfg.device));
        TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, cfg.device));
        red_blocks = 2 * n_sm;
        if (const char *e = getenv("FWI_GRAPHS")) graphs = atoi(e) != 0;
        TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        for (auto &e : ev) TRY(cudaEventCreate(&e));
        ss.main = st;
        if (sizeof(T) == 4) {
            // the side stream carries the step's critical path (strip pass -> layer
            // tiles): the highest priority, so that its blocks take SM slots ahead
            // of the interior tiles' as those free up
            int lo = 0, hi = 0;
            TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            TRY(cudaStreamCreateWithPriority(&ss.side, cudaStreamNonBlocking, hi));
            TRY(cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming));
            TRY(cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming));
        }
        for (T **p : {&vh, &vp, &vn, &mh, &mp, &mn}) TRY(alloc(p, mslot));
        TRY(alloc(&cpa, cfg.cpml + 1));
        TRY(alloc(&cpb, cfg.cpml + 1));
        TRY(alloc(&wavelet, nt_max));
        for (auto &p : lvl) TRY(alloc(&p, (size_t)B * slot));
        for (auto &p : cp) TRY(alloc(&p, (size_t)B * slot));
        for (auto &p : gs) TRY(alloc(&p, (size_t)B * slot));
        if (cfg.store == FWI_STORE_CHECKPOINT) {
            ck_every = checkpoint_interval(cfg);
            n_ck = (nt_max + ck_every - 1) / ck_every;
            n_img = 2 * ck_every;  // two segments' images: one rebuilt while the other is consumed
            TRY(alloc(&ck, (size_t)n_ck * 8 * B * slot));
            for (auto &p : rlvl) TRY(alloc(&p, (size_t)B * slot));
            for (auto &p : rcp) TRY(alloc(&p, (size_t)B * slot));
        }
        if (cfg.store == FWI_STORE_BOUNDARY) {
            ring_len = fwi::boundary_ring_len(win, nz, cfg.cpml);
            n_img = 2;  // the images of the last two steps rebuilt
            TRY(alloc(&ring, (size_t)B * nt_max * ring_len));
            for (auto &p : rlvl) TRY(alloc(&p, (size_t)B * slot));
        }
        if (cfg.store != FWI_STORE_FULL) {
            TRY(cudaStreamCreateWithFlags(&rst, cudaStreamNonBlocking));
            TRY(cudaEventCreateWithFlags(&ev_rfork, cudaEventDisableTiming));
            for (int k = 0; k < 2; k++) {
                TRY(cudaEventCreateWithFlags(&ev_reb[k], cudaEventDisableTiming));
                TRY(cudaEventCreateWithFlags(&ev_adj[k], cudaEventDisableTiming));
            }
            rss.main = rst;
            if (ss.side) {  // the recompute's forward steps fork like the main ones
                int lo = 0, hi = 0;
                TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
                TRY(cudaStreamCreateWithPriority(&rss.side, cudaStreamNonBlocking, hi));
                TRY(cudaEventCreateWithFlags(&rss.fork, cudaEventDisableTiming));
                TRY(cudaEventCreateWithFlags(&rss.join, cudaEventDisableTiming));
            }
        }
        {
            void *q0 = nullptr;
            TRY(cudaMalloc(&q0, (size_t)B * n_img * 2 * slot * store_elem()));
            allocs.push_back(q0);
            store = q0;
        }
        if (sizeof(T) == sizeof(float)) {
            TRY(fwi::prepare_fp32_kernels());
            int rc = build_maps(maps, lvl, cp);
            if (rc == FWI_OK && cfg.store == FWI_STORE_BOUNDARY) rc = build_maps(rmaps, rlvl, cp);  // rebuild levels
            if (rc == FWI_OK && cfg.store == FWI_STORE_CHECKPOINT) {
                // the recompute's forward steps use its own first 4 CPML arrays
                T *const rcpv[8] = {rcp[0], rcp[1], rcp[2], rcp[3], cp[4], cp[5], cp[6], cp[7]};
                rc = build_maps(rmaps, rlvl, rcpv);
            }
            if (rc != FWI_OK) return rc;
            use_tma = true;
        }
        TRY(alloc(&scale, (size_t)B * nt_max));
        TRY(alloc(&amax, (size_t)B * (nt_max + 1)));
        TRY(alloc(&rec, (size_t)B * nt_max * nrec_max));
        TRY(alloc(&obs, (size_t)B * nt_max * nrec_max));
        TRY(alloc(&mask, (size_t)B * nrec_max));
        TRY(alloc(&mask_off, B));
        TRY(alloc(&shots, B));
        TRY(alloc(&status, 1));
        TRY(alloc(&partial, (size_t)B * red_blocks));
        TRY(alloc(&misfit, 1));
        for (auto &p : grad) TRY(alloc(&p, mslot));
        for (T **p : {&mb[0], &mb[1], &mb[2], &gb[0], &gb[1], &gb[2], &q[0], &q[1], &q[2], &r[0], &r[1], &r[2]})
            TRY(alloc(p, mslot));
        TRY(alloc(&lbs, 1));
        TRY(alloc(&ds.partial, (size_t)red_blocks * 12));
        TRY(alloc(&ds.counter, 1));
        TRY(cudaMemsetAsync(ds.counter, 0, sizeof(unsigned), st));
        TRY(cudaMemsetAsync(lbs, 0, sizeof(LbScalars), st));
        for (T *p : {vh, vp, vn, mh, mp, mn}) TRY(cudaMemsetAsync(p, 0, mslot * sizeof(T), st));
        int rcc = cpml_table();
        if (rcc) return rcc;
        TRY_LAUNCH();
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    int build_maps(fwi::HostTmaMaps &m, T *const (&lv)[6], T *const (&cpv)[8])
    {
        using namespace fwi;
        for (int k = 0; k < 4; k++) {
            int rc = make_tensor_map_3d(&m.lvl[k], lv[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pitch, nz, B, 40, 40, 1);
            if (rc) return rc;
        }
        for (int k = 0; k < 2; k++) {  // P levels with the x-halo only, F levels with the z-halo only
            int rc = make_tensor_map_3d(&m.px[k], lv[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pitch, nz, B, 40, 32, 1);
            if (rc) return rc;
            rc = make_tensor_map_3d(&m.fz[k], lv[2 + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pitch, nz, B, 32, 40, 1);
            if (rc) return rc;
        }
        for (int k = 0; k < 2; k++) {  // P, F increments without a halo (forward interior tiles)
            int rc = make_tensor_map_3d(&m.inc[k], lv[4 + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pitch, nz, B, 32, 32, 1);
            if (rc) return rc;
        }
        for (int k = 0; k < 8; k++) {  // CPML memory variables, both halo shapes (layer tiles)
            int rc = make_tensor_map_3d(&m.mx[k], cpv[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pitch, nz, B, 40, 32, 1);
            if (rc) return rc;
            rc = make_tensor_map_3d(&m.mz[k], cpv[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pitch, nz, B, 32, 40, 1);
            if (rc) return rc;
        }
        return FWI_OK;
    }

    // Shots per group of the interior tile passes (a group of several windows
    // runs their MIXED kernels; the layer passes then take one shot per
    // block).  The tile passes are latency-bound, so many short blocks beat
    // few long ones: the
    // group count gives about three waves of adjoint tile blocks (3 resident
    // per SM).  Measured on 601 x 301, 32 shots: 5 shots
    // per group (7 groups) 56.8 shots/s, 8: 53.8, 3: 52.3, 16: 40.6.
    static bool uniform_windows(const std::vector<DevShot> &bs)
    {
        for (const DevShot &d : bs)
            if (d.x0 != bs[0].x0 || d.nx != bs[0].nx) return false;
        return true;
    }

    int shots_per_group(const std::vector<DevShot> &bs, int nxm) const
    {
        if (!use_tma) return 1;
        if (const char *e = getenv("FWI_SHOTS_PER_GROUP")) {  // tuning override
            const int v = atoi(e);
            if (v >= 1) return std::min(v, 64);
        }
        const long tiles = (long)((nxm - 5) / 32 + 1) * ((nz - 5) / 32 + 1);  // tiles holding interior points
        const long slots = 3L * n_sm;
        const long nb = (long)bs.size();
        const long groups = std::max(1L, std::min(nb, (3 * slots + tiles / 2) / tiles));
        const long sg = (nb + groups - 1) / groups;
        return (int)std::max(1L, std::min(sg, 64L));
    }

    // Shots per group of the layer tiles (with identical windows).  They run
    // on the side stream beside the interior tiles; the group count gives
    // about half a wave of adjoint blocks (3 per SM): short enough a
    // pass, without a block prologue per shot.  Measured on 601 x 301, 32
    // shots (54 layer tiles): 8 shots per group 60.2 shots/s, 5: 59.1,
    // 16: 54.9, 2: 56.6, 1: 53.4.
    int layer_shots_per_group(int nb, int nxm, int xbase, int zbase) const
    {
        if (const char *e = getenv("FWI_LAYER_SHOTS_PER_GROUP")) {  // tuning override
            const int v = atoi(e);
            if (v >= 1) return std::min(v, 64);
        }
        long tiles = 0;
        for (int z0 = zbase; z0 < nz; z0 += fwi::kTileEdge)
            for (int x0 = xbase; x0 < nxm; x0 += fwi::kTileEdge)
                tiles += fwi::tile_role(x0, z0, nxm, nz, cfg.cpml + fwi::kRad) == 2;
        const long slots = 3L * n_sm / 2;
        const long groups = std::max(1L, std::min((long)nb, (slots + tiles / 2) / std::max(1L, tiles)));
        return (int)std::max(1L, std::min((nb + groups - 1) / groups, 64L));
    }

    // Launch choices of a batch's tile passes: shots per block of the interior
    // and of the layer tile passes, and whether the layer tiles advance the
    // CPML memory variables themselves (when the tile grid allows it) or
    // after the strip pass.  Built-in choices from the rules above, or the
    // ones fwi_autotune measured for the batch's shape.
    struct Choice {  // of one phase (forward or adjoint)
        int sg = 1, sg_layer = 1, inline_strip = 0;
        bool operator==(const Choice &o) const
        {
            return sg == o.sg && sg_layer == o.sg_layer && inline_strip == o.inline_strip;
        }
    };
    struct Choices {  // the two phases share no state that depends on it
        Choice fwd, adj;
    };
    struct Tuned {
        std::vector<long> key;
        Choices c;
    };
    std::vector<Tuned> tuned;

    // The order in which the shots of a call form batches: longest first (stable: shots of one
    // length keep the caller's order).  A batch runs as many steps as its longest shot, its
    // shorter shots idle until their own start, so batches of similar length keep the GPU busy;
    // the gradient and misfit are sums over the shots.
    static std::vector<int> batch_order(const std::vector<DevShot> &all)
    {
        std::vector<int> o(all.size());
        for (size_t k = 0; k < o.size(); k++) o[k] = (int)k;
        std::stable_sort(o.begin(), o.end(), [&](int a, int c) { return all[a].nt > all[c].nt; });
        return o;
    }

    // What the fastest choice depends on: shots in the batch, widest window,
    // one window for all, mode, image store type.
    std::vector<long> choice_key(const std::vector<DevShot> &bs, int nxm) const
    {
        return {(long)bs.size(), (long)nxm, uniform_windows(bs) ? 1L : 0L, (long)cfg.mode, (long)store_type()};
    }

    Choice default_choice(const std::vector<DevShot> &bs, int nxm) const
    {
        Choice c;
        c.sg = shots_per_group(bs, nxm);
        fwi::TileGrid tg;
        if (use_tma && uniform_windows(bs)) tg = fwi::tile_grid(nxm, nz, cfg.cpml);
        c.inline_strip = tg.inline_strip ? 1 : 0;
        c.sg_layer = c.sg == 1 || !uniform_windows(bs) ? 1
                                                       : layer_shots_per_group((int)bs.size(), nxm, tg.xbase, tg.zbase);
        return c;
    }

    Choices choice_for(const std::vector<DevShot> &bs, int nxm) const
    {
        const std::vector<long> key = choice_key(bs, nxm);
        for (const Tuned &t : tuned)
            if (t.key == key) return t.c;
        const Choice d = default_choice(bs, nxm);
        return {d, d};
    }

    void record_choice(const std::vector<long> &key, const Choices &c)
    {
        for (Tuned &t : tuned)
            if (t.key == key) {
                t.c = c;
                return;
            }
        tuned.push_back({key, c});
    }

    // A batch of several windows: the interior passes' groups run the MIXED
    // kernels, the layer passes take one shot per block, no in-tile memory
    // variables (no tile origin fits every window's bands).
    void apply_choice(Batch<T> &b, const std::vector<DevShot> &bs, int nxm, const Choice &c) const
    {
        const bool uniform = uniform_windows(bs);
        b.sg = c.sg;
        b.sg_layer = uniform ? c.sg_layer : 1;
        b.mixed = use_tma && !uniform && c.sg > 1 ? 1 : 0;
        if (use_tma && uniform) {  // one tile grid fits every shot
            const fwi::TileGrid tg = fwi::tile_grid(nxm, nz, cfg.cpml);
            b.xbase = tg.xbase;
            b.zbase = tg.zbase;
            b.inline_strip = tg.inline_strip && c.inline_strip;
            if (const char *e = getenv("FWI_INLINE_STRIP"))  // 0: the strip pass path (tests)
                if (atoi(e) == 0) b.inline_strip = 0;
            // one block per tile of each pass's role (the exact adjoint's layers reach 4 points further)
            const int aw_adj = cfg.mode == FWI_MODE_EXACT ? cfg.cpml + fwi::kRad : cfg.cpml;
            const int role_aw[4][2] = {{1, cfg.cpml}, {2, cfg.cpml}, {1, aw_adj}, {2, aw_adj}};
            for (int l = 0; l < 4; l++)
                b.tiles[l] = tile_list(nxm, b.xbase, b.zbase, role_aw[l][1], role_aw[l][0], b.ntiles[l]);
        }
    }

    // Whether a batch of windows nxm wide runs on the small-shot cluster path: FP32, exact
    // adjoint, every step's images kept (the path has no checkpoint or boundary variant), the
    // window fitting a cluster's shared memory, and FWI_CLUSTER not set to 0.  Cached per width.
    mutable std::vector<std::pair<int, bool>> cluster_fit;
    bool cluster_path(int nxm) const
    {
        if (!(sizeof(T) == 4 && use_tma && cfg.mode == FWI_MODE_EXACT && cfg.store == FWI_STORE_FULL)) return false;
        if (const char *e = getenv("FWI_CLUSTER"))
            if (atoi(e) == 0) return false;
        for (const auto &c : cluster_fit)
            if (c.first == nxm) return c.second;
        const bool ok = fwi::cluster_shot_fits(nxm, nz, cfg.cpml, store_type());
        cluster_fit.emplace_back(nxm, ok);
        return ok;
    }

    // Device copies of the compact tile lists (Batch::tiles), one per window width, grid
    // origin, layer width and role, made on first use and kept for the context's life (a
    // captured graph reads them).  Null (full grid) if the list cannot be made.
    struct TileListEntry {
        int nxm, xbase, zbase, aw, role, n;
        int *dev;
    };
    mutable std::vector<TileListEntry> tile_lists;
    const int *tile_list(int nxm, int xbase, int zbase, int aw, int role, int &n) const
    {
        for (const TileListEntry &e : tile_lists)
            if (e.nxm == nxm && e.xbase == xbase && e.zbase == zbase && e.aw == aw && e.role == role) {
                n = e.n;
                return e.dev;
            }
        std::vector<int> t;
        for (int tz = 0; zbase + tz * fwi::kTileEdge < nz; tz++)
            for (int tx = 0; xbase + tx * fwi::kTileEdge < nxm; tx++)
                if (fwi::tile_role(xbase + tx * fwi::kTileEdge, zbase + tz * fwi::kTileEdge, nxm, nz, aw) == role)
                    t.push_back(tx | (tz << 16));
        n = (int)t.size();
        int *d = nullptr;
        if (t.empty() || cudaMalloc(&d, t.size() * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
            return nullptr;
        }
        if (cudaMemcpy(d, t.data(), t.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(d);
            n = 0;
            return nullptr;
        }
        tile_lists.push_back({nxm, xbase, zbase, aw, role, n, d});
        return d;
    }

    // CPML table by distance (src/main.c:48-51: L = CPML dh, d0 = -3 ln R / (2 L), in T)
    int cpml_table()
    {
        const T L = cfg.cpml * (T)cfg.dh;
        const T d0 = (T)(-3 * log((double)cfg.r_coef) / (double)(2 * L));
        k_cpml_table<T><<<(cfg.cpml + 128) / 128, 128, 0, st>>>(cpa, cpb, cfg.cpml, (T)cfg.vmax, (T)cfg.dt,
                                                                 (T)cfg.dh, (T)cfg.f_cpml, d0, L);
        TRY_LAUNCH();
        return FWI_OK;
    }

    int set_frequency(float f, int nt) override
    {
        if (!(f > 0) || nt <= 0 || nt > nt_max) return FWI_ERR_ARG;
        cfg.f_cpml = f;
        int rc = cpml_table();
        if (rc) return rc;
        return set_ricker(f, nt);
    }

    int copy_model_in(T *dst, const void *src)
    {
        TRY(cudaMemcpy2DAsync(dst, mpitch * sizeof(T), src, nx * sizeof(T), nx * sizeof(T), nz,
                              cudaMemcpyDefault, st));
        return FWI_OK;
    }

    int set_model(const void *a, const void *b, const void *c) override
    {
        if (!a || !b || !c) return FWI_ERR_ARG;
        int rc;
        if ((rc = copy_model_in(vh, a)) || (rc = copy_model_in(vp, b)) || (rc = copy_model_in(vn, c))) return rc;
        have_model = true;
        models_dirty = true;
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    int set_model_vti(const void *vel, const void *eps, const void *del) override
    {
        if (!vel || !eps || !del) return FWI_ERR_ARG;
        // stage the three inputs in the gradient buffers (free here), then transform
        const size_t bytes = (size_t)nx * nz * sizeof(T);
        TRY(cudaMemcpyAsync(grad[0], vel, bytes, cudaMemcpyDefault, st));
        TRY(cudaMemcpyAsync(grad[1], eps, bytes, cudaMemcpyDefault, st));
        TRY(cudaMemcpyAsync(grad[2], del, bytes, cudaMemcpyDefault, st));
        k_pre_variables<T><<<eg((long)nx * nz), 256, 0, st>>>(grad[0], grad[1], grad[2], vh, vp, vn, nx,
                                                                     nz, mpitch);
        TRY_LAUNCH();
        launches++;
        have_model = true;
        have_grad = false;
        models_dirty = true;
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    int get_model(void *a, void *b, void *c) override
    {
        T *src[3] = {vh, vp, vn};
        void *dst[3] = {a, b, c};
        for (int k = 0; k < 3; k++)
            if (dst[k])
                TRY(cudaMemcpy2DAsync(dst[k], nx * sizeof(T), src[k], mpitch * sizeof(T), nx * sizeof(T), nz,
                                      cudaMemcpyDefault, st));
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    int set_wavelet(const void *w, int nt) override
    {
        if (!w || nt <= 0 || nt > nt_max) return FWI_ERR_ARG;
        TRY(cudaMemsetAsync(wavelet, 0, nt_max * sizeof(T), st));
        TRY(cudaMemcpyAsync(wavelet, w, nt * sizeof(T), cudaMemcpyDefault, st));
        TRY(cudaStreamSynchronize(st));
        have_wavelet = true;
        wavelet_nt = nt;
        return FWI_OK;
    }

    int set_ricker(float f, int nt) override
    {
        if (nt <= 0 || nt > nt_max || !(f > 0)) return FWI_ERR_ARG;
        // src/main.c:328-332 (host setup of the source, FP32 time accumulation)
        std::vector<T> w(nt);
        float t = 0;
        for (int it = 0; it < nt; it++) {
            t += cfg.dt;
            double a = 3.141592653589793 * f * (t - (1 / f));
            w[it] = (T)(1 * (1 - 2 * pow(a, 2)) * exp(-pow(a, 2)));
        }
        return set_wavelet(w.data(), nt);
    }

    int refresh_models()
    {
        if (!models_dirty) return FWI_OK;
        const T dt2 = (T)cfg.dt * (T)cfg.dt;
        k_scale_models<T><<<eg(mslot), 256, 0, st>>>(vh, vp, vn, mh, mp, mn, dt2, mslot);
        TRY_LAUNCH();
        launches++;
        models_dirty = false;
        return FWI_OK;
    }

    int check_shot(const fwi_shot &s, DevShot &d) const
    {
        const int x0 = s.nxw > 0 ? s.x0 : 0;
        const int w = s.nxw > 0 ? s.nxw : nx;
        if (x0 < 0 || x0 + w > nx || w > (cfg.max_window > 0 ? cfg.max_window : nx)) return FWI_ERR_ARG;
        if (w < 2 * cfg.cpml + 9 || nz < cfg.cpml + 9) return FWI_ERR_ARG;
        if (s.nt <= 0 || s.nt > nt_max || s.nt > wavelet_nt) return FWI_ERR_ARG;
        const int lsx = s.sx - x0, lr0 = s.rx0 - x0, lr1 = s.rx1 - x0;
        if (!fwi::interior(lsx, s.sz, w, nz)) return FWI_ERR_ARG;
        if (lr1 <= lr0 || lr1 - lr0 > nrec_max) return FWI_ERR_ARG;
        if (!fwi::interior(lr0, s.rz, w, nz) || !fwi::interior(lr1 - 1, s.rz, w, nz)) return FWI_ERR_ARG;
        d.x0 = x0; d.nx = w; d.sx = lsx; d.sz = s.sz; d.rz = s.rz; d.rx0 = lr0; d.rx1 = lr1; d.nt = s.nt;
        d.rec_off = 0;
        return FWI_OK;
    }

    Batch<T> batch_view(int nb) const
    {
        Batch<T> b;
        b.B = nb; b.nz = nz; b.pitch = pitch; b.mpitch = mpitch; b.cpml = cfg.cpml; b.nt_max = nt_max;
        b.slot = slot;
        for (int k = 0; k < 6; k++) b.lvl[k] = lvl[k];
        for (int k = 0; k < 8; k++) b.cp[k] = cp[k];
        for (int k = 0; k < 3; k++) b.g[k] = gs[k];
        b.store = store; b.store_type = store_type(); b.n_img = n_img;
        b.scale = scale; b.amax = amax; b.rec = rec; b.shots = shots;
        b.mh = mh; b.mp = mp; b.mn = mn; b.cpa = cpa; b.cpb = cpb; b.wavelet = wavelet;
        b.inv_dh = T(1) / (T)cfg.dh;
        b.inv_dh2 = T(1) / ((T)cfg.dh * (T)cfg.dh);
        b.img_scale = cfg.mode == FWI_MODE_EXACT ? (T)cfg.dt * (T)cfg.dt : (T)cfg.dt;
        b.status = status;
        b.sg = 1;
        b.sg_layer = 1;
        b.xbase = b.zbase = 0;
        b.inline_strip = 0;
        b.mixed = 0;
        b.tma = use_tma ? (const void *)&maps : nullptr;
        for (int l = 0; l < 4; l++) {
            b.tiles[l] = nullptr;
            b.ntiles[l] = 0;
        }
        return b;
    }

    int save_checkpoint(int k, int nb, int cur)
    {
        const size_t bytes = (size_t)nb * slot * sizeof(T);
        T *src[8] = {lvl[cur], lvl[2 + cur], lvl[4], lvl[5], cp[0], cp[1], cp[2], cp[3]};
        for (int a = 0; a < 8; a++)
            TRY(cudaMemcpyAsync(ck + ((size_t)k * 8 + a) * B * slot, src[a], bytes, cudaMemcpyDeviceToDevice, st));
        return FWI_OK;
    }

    int restore_checkpoint(int k, int nb, int cur, cudaStream_t s)
    {
        const size_t bytes = (size_t)nb * slot * sizeof(T);
        T *dst[8] = {rlvl[cur], rlvl[2 + cur], rlvl[4], rlvl[5], rcp[0], rcp[1], rcp[2], rcp[3]};
        for (int a = 0; a < 8; a++)
            TRY(cudaMemcpyAsync(dst[a], ck + ((size_t)k * 8 + a) * B * slot, bytes, cudaMemcpyDeviceToDevice, s));
        // a shot that starts later inside the segment reads the other level when it starts:
        // give both levels the checkpointed state (zero for such a shot)
        TRY(cudaMemcpyAsync(rlvl[1 - cur], ck + ((size_t)k * 8 + 0) * B * slot, bytes, cudaMemcpyDeviceToDevice, s));
        TRY(cudaMemcpyAsync(rlvl[3 - cur], ck + ((size_t)k * 8 + 1) * B * slot, bytes, cudaMemcpyDeviceToDevice, s));
        return FWI_OK;
    }

    // Forward (+ residual + adjoint) of all shots, batch by batch.
    int run(const fwi_shot *sh, int n, const void *obs_in, const unsigned char *mask_in, void *o_h, void *o_p,
            void *o_n, double *misfit_out, void *traces, bool want_grad) override
    {
        if (!have_model || !have_wavelet) return FWI_ERR_STATE;
        if (!sh || n <= 0) return FWI_ERR_ARG;
        // without observed data from the caller: the records kept on the device, for the same shots
        const bool from_store = (want_grad || misfit_out) && !obs_in;
        if (from_store) {
            if ((size_t)n != ostore_shots.size()) return FWI_ERR_ARG;
            for (int k = 0; k < n; k++)
                if (std::memcmp(&sh[k], &ostore_shots[k], sizeof(fwi_shot)) != 0) return FWI_ERR_ARG;
        }
        const bool have_obs = obs_in || from_store;
        std::vector<DevShot> all(n);
        std::vector<long> off(n + 1, 0), moff(n + 1, 0);
        for (int k = 0; k < n; k++) {
            int rc = check_shot(sh[k], all[k]);
            if (rc) return rc;
            off[k + 1] = off[k] + (long)all[k].nt * (all[k].rx1 - all[k].rx0);
            moff[k + 1] = moff[k] + (all[k].rx1 - all[k].rx0);
        }
        const bool exact = cfg.mode == FWI_MODE_EXACT;
        int rc = refresh_models();
        if (rc) return rc;
        TRY(cudaEventRecord(ev[0], st));
        long launches0 = launches;
        for (int p = 0; p < kPhases; p++) { tile_ms[p] = tile_pts[p] = 0; tile_n[p] = 0; }
        recompute_steps = 0;
        const long kps = sizeof(T) == 4 ? 3 : 2;  // kernels per time step (see the file comment)
        if (want_grad)
            for (auto &p : grad) TRY(cudaMemsetAsync(p, 0, mslot * sizeof(T), st));
        TRY(cudaMemsetAsync(misfit, 0, sizeof(double), st));
        TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
        float t_fwd = 0, t_adj = 0;
        const std::vector<int> order = batch_order(all);
        for (int b0 = 0; b0 < n; b0 += B) {
            const int nb = std::min(B, n - b0);
            int ntb = 0, nxm = 0;
            // the batch's shots (order[b0 ..]), their records and mask rows packed in that order;
            // runs of consecutive shots of the caller's arrays move in one copy
            std::vector<DevShot> bs(nb);
            std::vector<long> bmo(nb);
            long nrec_elems = 0, nmask = 0;
            for (int k = 0; k < nb; k++) {
                bs[k] = all[order[b0 + k]];
                bs[k].rec_off = nrec_elems;
                bmo[k] = nmask;
                nrec_elems += off[order[b0 + k] + 1] - off[order[b0 + k]];
                nmask += moff[order[b0 + k] + 1] - moff[order[b0 + k]];
                ntb = std::max(ntb, bs[k].nt);
                nxm = std::max(nxm, bs[k].nx);
            }
            // copy(dst, src, per-shot offsets (records or mask rows), element size): runs of consecutive shots
            auto gather = [&](void *dst, const void *src, const std::vector<long> &o, const std::vector<long> &dsto,
                              size_t elem, cudaMemcpyKind kind) -> int {
                for (int k = 0; k < nb;) {
                    int e = k + 1;
                    while (e < nb && order[b0 + e] == order[b0 + e - 1] + 1) e++;
                    const int s0 = order[b0 + k];
                    const long len = o[s0 + e - k] - o[s0];
                    TRY(cudaMemcpyAsync((char *)dst + dsto[k] * elem, (const char *)src + o[s0] * elem, len * elem,
                                        kind, st));
                    k = e;
                }
                return FWI_OK;
            };
            std::vector<long> rec_dst(nb), mask_dst(nb);
            for (int k = 0; k < nb; k++) {
                rec_dst[k] = bs[k].rec_off;
                mask_dst[k] = bmo[k];
            }
            TRY(cudaMemcpyAsync(shots, bs.data(), nb * sizeof(DevShot), cudaMemcpyHostToDevice, st));
            TRY(cudaMemcpyAsync(mask_off, bmo.data(), nb * sizeof(long), cudaMemcpyHostToDevice, st));
            if (obs_in) {
                if ((rc = gather(obs, obs_in, off, rec_dst, sizeof(T), cudaMemcpyDefault))) return rc;
            } else if (from_store && ostore) {
                if ((rc = gather(obs, ostore, off, rec_dst, sizeof(T), cudaMemcpyDeviceToDevice))) return rc;
            } else if (from_store)
                for (int k = 0; k < nb; k++) {
                    const int s0 = order[b0 + k];
                    const int nr = all[s0].rx1 - all[s0].rx0;
                    k_trace_decode<T><<<eg((long)all[s0].nt * nr), 256, 0, st>>>(
                        ostore_h, off[s0], all[s0].nt, nr, ostore_scale + moff[s0], obs, bs[k].rec_off);
                    TRY_LAUNCH();
                    launches++;
                }
            if (mask_in && (rc = gather(mask, mask_in, moff, mask_dst, 1, cudaMemcpyDefault))) return rc;
            const size_t lb = (size_t)nb * slot * sizeof(T);
            for (auto &p : lvl) TRY(cudaMemsetAsync(p, 0, lb, st));
            for (int k = 0; k < 4; k++) TRY(cudaMemsetAsync(cp[k], 0, lb, st));
            TRY(cudaMemsetAsync(amax, 0, (size_t)nb * (nt_max + 1) * sizeof(float), st));
            // the adjoint's view (its groups own the gradient slots) and the forward's
            const Choices ch = choice_for(bs, nxm);
            Batch<T> b = batch_view(nb);
            apply_choice(b, bs, nxm, ch.adj);
            Batch<T> bf = b;
            apply_choice(bf, bs, nxm, ch.fwd);
            const int ngroups = (nb + b.sg - 1) / b.sg;
            // gradient slots in use: the interior groups' and the layer tiles' (same window in all)
            const int nslots = std::max(ngroups, (nb + b.sg_layer - 1) / b.sg_layer);
            cudaEvent_t e0 = ev[1], e1 = ev[2], e2 = ev[3];
            TRY(cudaEventRecord(e0, st));
            const bool ckpt = want_grad && cfg.store == FWI_STORE_CHECKPOINT;
            const bool bnd = want_grad && cfg.store == FWI_STORE_BOUNDARY;
            // sampled steps of the interior tile timing: events and interior points updated
            const bool timed = tile_timing && sizeof(T) == 4;
            const int tstride = std::max(1, ntb / kTimeSamples);
            int nsamp[kPhases] = {0, 0, 0};
            double spts[kPhases][kTimeSamples] = {};
            auto sample = [&](int phase, int step, fwi::StepStreams &sst) {
                if (!timed || step % tstride != tstride / 2 || nsamp[phase] >= kTimeSamples) return;
                const bool fwd = phase != 1;  // forward steps: the forward and the recompute
                const int aw = fwd || !exact ? cfg.cpml : cfg.cpml + fwi::kRad;
                double pts = 0;
                for (const DevShot &d : bs)
                    if (fwd ? step - (ntb - d.nt) >= 0 : step < d.nt)
                        pts += (double)interior_tile_points(d.nx, aw, b.xbase, b.zbase);
                const int k = nsamp[phase]++;
                spts[phase][k] = pts;
                sst.t0 = tev[phase][k][0];
                sst.t1 = tev[phase][k][1];
            };
            // launch parameters the sections bake in besides the batch view: the
            // section, the step counts and storage, and each shot's steps and width
            // (which shots run at a step, the timing samples' points)
            auto section_key = [&](long tag) {
                std::vector<long> k = {tag, nb, ntb, nxm, exact, want_grad, ckpt, bnd, ck_every, timed, tstride,
                                       nslots};
                key_batch(k, bf);  // the adjoint section's segment recompute runs forward steps
                key_batch(k, b);
                for (const DevShot &d : bs) {
                    k.push_back(d.nt);
                    k.push_back(d.nx);
                }
                return k;
            };
            // checkpoint storage: the last two segments' images fit the two-segment image buffer, so
            // the forward writes them there itself; the adjoint starts on them at once and only the
            // segments before them are recomputed from their checkpoints
            const int last_seg = ckpt ? (ntb - 1) / ck_every : 0;
            const int first_direct = ckpt ? std::max(0, last_seg - 1) : 0;
            auto fwd_img_slot = [&](int g) {
                if (!want_grad || bnd) return -1;
                if (!ckpt) return g;
                const int seg = g / ck_every;
                return seg >= first_direct ? g - seg * ck_every + (seg & 1) * ck_every : -1;
            };
            // small shots on chip: one cluster per shot, every step in one launch (prop_cluster.cuh)
            const bool on_cluster = cluster_path(nxm);
            NvtxRange fwd_range("fwi forward steps");
            if constexpr (sizeof(T) == 4) {
                if (on_cluster) {
                    TRY(fwi::launch_cluster_forward(bf, nxm, ntb, want_grad, st));
                    launches++;
                }
            }
            rc = on_cluster ? FWI_OK : run_section(section_key(0), 1u, nsamp, spts, [&]() -> int {
                int cur = 0;
                for (int g = 0; g < ntb; g++) {
                    if (ckpt && g % ck_every == 0 && g / ck_every < first_direct) {
                        int rc2 = save_checkpoint(g / ck_every, nb, cur);
                        if (rc2) return rc2;
                    }
                    fwi::StepStreams sst = ss;
                    sample(0, g, sst);
                    if (bnd) fwi::launch_save_ring<T>(bf, nxm, g, ntb, cur, ring, ring_len, st);
                    fwi::launch_forward_step<T>(bf, nxm, g, ntb, cur, fwd_img_slot(g), exact, sst);
                    cur ^= 1;
                }
                TRY_LAUNCH();
                launches += (kps + (bnd ? 1 : 0)) * ntb;
                if (bnd) {
                    // the final state (P, F, increments) starts the backward rebuild
                    for (auto &p : rlvl) TRY(cudaMemsetAsync(p, 0, lb, st));
                    TRY(cudaMemcpyAsync(rlvl[0], lvl[cur], lb, cudaMemcpyDeviceToDevice, st));
                    TRY(cudaMemcpyAsync(rlvl[2], lvl[2 + cur], lb, cudaMemcpyDeviceToDevice, st));
                    TRY(cudaMemcpyAsync(rlvl[4], lvl[4], lb, cudaMemcpyDeviceToDevice, st));
                    TRY(cudaMemcpyAsync(rlvl[5], lvl[5], lb, cudaMemcpyDeviceToDevice, st));
                    // images of the layer points stay zero
                    TRY(cudaMemsetAsync(store, 0, (size_t)nb * n_img * 2 * slot * store_elem(), st));
                }
                return FWI_OK;
            });
            if (rc) return rc;
            TRY(cudaEventRecord(e1, st));
            if (have_obs) {
                k_residual<T><<<dim3(red_blocks, nb), kRedThreads, 0, st>>>(rec, obs, mask_in ? mask : nullptr, shots,
                                                                          mask_off, partial);
                k_misfit_finish<<<1, 256, 0, st>>>(partial, (long)nb * red_blocks, misfit);
                TRY_LAUNCH();
                launches += 2;
            }
            if (traces)  // back to the caller's order, runs of consecutive shots in one copy
                for (int k = 0; k < nb;) {
                    int e = k + 1;
                    while (e < nb && order[b0 + e] == order[b0 + e - 1] + 1) e++;
                    const int s0 = order[b0 + k];
                    TRY(cudaMemcpyAsync((T *)traces + off[s0], rec + bs[k].rec_off,
                                        (off[s0 + e - k] - off[s0]) * sizeof(T), cudaMemcpyDefault, st));
                    k = e;
                }
            if (want_grad && on_cluster) {
                NvtxRange adj_range("fwi adjoint steps + imaging");
                for (auto &p : gs) TRY(cudaMemsetAsync(p, 0, lb, st));
                if constexpr (sizeof(T) == 4) TRY(fwi::launch_cluster_adjoint(b, nxm, ntb, st));
                // one gradient slot per shot
                k_accumulate_gradient<T><<<eg((long)nx * nz), 256, 0, st>>>(grad[0], grad[1], grad[2], gs[0], gs[1],
                                                                            gs[2], shots, nb, 1, nx, nz, mpitch, pitch,
                                                                            slot);
                TRY_LAUNCH();
                launches += 2;
            } else if (want_grad) {
                NvtxRange adj_range("fwi adjoint steps + imaging");
                rc = run_section(section_key(1), 6u, nsamp, spts, [&]() -> int {
                    for (auto &p : lvl) TRY(cudaMemsetAsync(p, 0, lb, st));
                    for (auto &p : cp) TRY(cudaMemsetAsync(p, 0, lb, st));
                    for (auto &p : gs) TRY(cudaMemsetAsync(p, 0, lb, st));
                    int cur = 0;
                    int zsel = 0;
                    // image halves the adjoint consumed in this section (an event of an
                    // earlier batch is complete: that batch ended in a synchronize)
                    bool consumed[2] = {false, false};
                    if (bnd) {
                        // rebuild the CPML-free region backwards one step ahead of the adjoint
                        // iteration that images it (image slot 0 holds the step just rebuilt)
                        const int lag = exact ? 0 : 1;
                        Batch<T> rb = b;
                        for (int k = 0; k < 6; k++) rb.lvl[k] = rlvl[k];
                        rb.tma = use_tma ? (const void *)&rmaps : nullptr;
                        // the rebuild stream starts after everything issued so far (the final state copies)
                        TRY(cudaEventRecord(ev_rfork, st));
                        TRY(cudaStreamWaitEvent(rst, ev_rfork, 0));
                        fwi::launch_rebuild_begin<T>(rb, nxm, ntb - 1, ntb, 0, ring, ring_len, rst);
                        launches += 2;
                        int rcur = 1, next_g = ntb - 1;
                        for (int j = 0; j < ntb; j++) {
                            const int need = ntb - 1 - lag - j;
                            for (; next_g >= 0 && next_g >= need; next_g--) {
                                // slot next_g & 1 is free once the adjoint iteration imaging step next_g + 2 is done
                                if (consumed[next_g & 1]) TRY(cudaStreamWaitEvent(rst, ev_adj[next_g & 1], 0));
                                fwi::launch_rebuild_step<T>(rb, nxm, next_g, ntb, rcur, ring, ring_len, next_g & 1, rst);
                                TRY(cudaEventRecord(ev_reb[next_g & 1], rst));
                                rcur ^= 1;
                                launches += sizeof(T) == 4 ? 1 : 2;
                            }
                            if (need >= 0) TRY(cudaStreamWaitEvent(st, ev_reb[need & 1], 0));
                            fwi::StepStreams sst = ss;
                            sample(1, j, sst);
                            fwi::launch_adjoint_step<T>(b, nxm, j, ntb, cur, zsel, exact, need >= 0 ? need - (need & 1) : 0,
                                                        sst);
                            if (need >= 0) {
                                TRY(cudaEventRecord(ev_adj[need & 1], st));
                                consumed[need & 1] = true;
                            }
                            cur ^= 1;
                            zsel ^= 1;
                            launches += kps;
                        }
                        // the main stream is past every rebuild: the last adjoint iteration with an
                        // image waited for it; join the rebuild stream all the same
                        TRY(cudaEventRecord(ev_reb[0], rst));
                        TRY(cudaStreamWaitEvent(st, ev_reb[0], 0));
                        TRY_LAUNCH();
                    } else if (!ckpt) {
                        for (int j = 0; j < ntb; j++) {
                            fwi::StepStreams sst = ss;
                            sample(1, j, sst);
                            fwi::launch_adjoint_step<T>(b, nxm, j, ntb, cur, zsel, exact, 0, sst);
                            cur ^= 1;
                            zsel ^= 1;
                        }
                        TRY_LAUNCH();
                        launches += kps * ntb;
                    } else {
                        // segments from the last: recompute its images from the checkpoint, then
                        // run the adjoint iterations that image inside it
                        const int lag = exact ? 0 : 1;
                        Batch<T> rb = bf;  // forward steps: the forward's choice
                        // frames of the recompute levels stay zero: never written by the steps
                        for (auto &p : rlvl) TRY(cudaMemsetAsync(p, 0, lb, st));
                        for (int k = 0; k < 6; k++) rb.lvl[k] = rlvl[k];
                        for (int k = 0; k < 4; k++) rb.cp[k] = rcp[k];
                        rb.tma = use_tma ? (const void *)&rmaps : nullptr;
                        // `rec` holds the residuals now; the recomputed traces go to the spent obs copy
                        rb.rec = obs;
                        // segment seg's images go to half seg & 1 of the image buffer; the
                        // recompute of segment seg - 1 (on rss) overlaps the adjoint iterations
                        // imaging inside segment seg (on ss)
                        TRY(cudaEventRecord(ev_rfork, st));
                        TRY(cudaStreamWaitEvent(rst, ev_rfork, 0));
                        auto recompute = [&](int seg) -> int {
                            const int a = seg * ck_every, e = std::min(a + ck_every, ntb), h = seg & 1;
                            if (consumed[h]) TRY(cudaStreamWaitEvent(rst, ev_adj[h], 0));  // half h consumed (segment seg + 2)
                            int rcur = a & 1;
                            int rc2 = restore_checkpoint(seg, nb, rcur, rst);
                            if (rc2) return rc2;
                            for (int g = a; g < e; g++) {
                                fwi::StepStreams rsst = rss;
                                sample(2, g, rsst);
                                fwi::launch_forward_step<T>(rb, nxm, g, ntb, rcur, (g - a) + h * ck_every, exact, rsst);
                                rcur ^= 1;
                            }
                            TRY(cudaEventRecord(ev_reb[h], rst));
                            launches += kps * (e - a);
                            recompute_steps += e - a;
                            return FWI_OK;
                        };
                        // segments first_direct .. last_seg were imaged by the forward itself
                        int rc3 = FWI_OK;
                        int j = 0;
                        for (int seg = last_seg; seg >= 0; seg--) {
                            const int a = seg * ck_every, h = seg & 1;
                            if (seg > 0 && seg - 1 < first_direct && (rc3 = recompute(seg - 1))) return rc3;
                            if (seg < first_direct) TRY(cudaStreamWaitEvent(st, ev_reb[h], 0));
                            for (; j < ntb && ntb - 1 - lag - j >= a; j++) {
                                fwi::StepStreams sst = ss;
                                sample(1, j, sst);
                                fwi::launch_adjoint_step<T>(b, nxm, j, ntb, cur, zsel, exact, a - h * ck_every, sst);
                                cur ^= 1;
                                zsel ^= 1;
                                launches += kps;
                            }
                            TRY(cudaEventRecord(ev_adj[h], st));
                            consumed[h] = true;
                        }
                        TRY(cudaEventRecord(ev_reb[0], rst));  // join the recompute stream
                        TRY(cudaStreamWaitEvent(st, ev_reb[0], 0));
                        for (; j < ntb; j++) {  // iterations without an image (reference lag)
                            fwi::launch_adjoint_step<T>(b, nxm, j, ntb, cur, zsel, exact, 0, ss);
                            cur ^= 1;
                            zsel ^= 1;
                            launches += kps;
                        }
                        TRY_LAUNCH();
                    }
                    k_accumulate_gradient<T><<<eg((long)nx * nz), 256, 0, st>>>(
                        grad[0], grad[1], grad[2], gs[0], gs[1], gs[2], shots, nslots, 1, nx, nz, mpitch, pitch, slot);
                    TRY_LAUNCH();
                    launches++;
                    return FWI_OK;
                });
                if (rc) return rc;
            }
            TRY(cudaEventRecord(e2, st));
            TRY(cudaEventSynchronize(e2));
            float a = 0, c = 0;
            cudaEventElapsedTime(&a, e0, e1);
            cudaEventElapsedTime(&c, e1, e2);
            t_fwd += a;
            t_adj += c;
            for (int p = 0; p < kPhases; p++)
                for (int k = 0; k < nsamp[p]; k++) {
                    float ms = 0;
                    TRY(cudaEventElapsedTime(&ms, tev[p][k][0], tev[p][k][1]));
                    tile_ms[p] += ms;
                    tile_pts[p] += spts[p][k];
                    tile_n[p]++;
                }
        }
        unsigned stat = 0;
        TRY(cudaMemcpyAsync(&stat, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        if (misfit_out) TRY(cudaMemcpyAsync(misfit_out, misfit, sizeof(double), cudaMemcpyDeviceToHost, st));
        if (want_grad) {
            void *outs[3] = {o_h, o_p, o_n};
            for (int k = 0; k < 3; k++)
                if (outs[k])
                    TRY(cudaMemcpy2DAsync(outs[k], nx * sizeof(T), grad[k], mpitch * sizeof(T), nx * sizeof(T), nz,
                                          cudaMemcpyDefault, st));
            have_grad = true;
        }
        cudaEvent_t eend;
        TRY(cudaEventCreate(&eend));
        cudaEventRecord(eend, st);
        cudaError_t se = cudaEventSynchronize(eend);
        float tot = 0;
        cudaEventElapsedTime(&tot, ev[0], eend);
        cudaEventDestroy(eend);
        TRY(se);
        timing[0] = tot;
        timing[1] = t_fwd;
        timing[2] = t_adj;
        timing[3] = tot - t_fwd - t_adj;
        launches = launches - launches0;
        if (stat & fwi::kStatusTimeout) return FWI_ERR_CUDA;
        if (stat & fwi::kStatusSaturated) return FWI_ERR_NUMERIC;
        if (misfit_out && !std::isfinite(*misfit_out)) return FWI_ERR_NUMERIC;
        return FWI_OK;
    }

    // ---------------------------------------------------------------- observed data on the device

    int free_observed() override
    {
        for (void *p : {(void *)ostore, (void *)ostore_h, (void *)ostore_scale})
            if (p) cudaFree(p);
        ostore = nullptr;
        ostore_h = nullptr;
        ostore_scale = nullptr;
        ostore_shots.clear();
        ostore_off.clear();
        ostore_moff.clear();
        return FWI_OK;
    }

    // Room for the records of these shots (offsets as fwi_gradient lays them out).
    int observed_layout(const fwi_shot *sh, int n, int sprec)
    {
        if (!sh || n <= 0 || (sprec != FWI_SPREC_NATIVE && sprec != FWI_SPREC_FP16)) return FWI_ERR_ARG;
        std::vector<long> off(n + 1, 0), moff(n + 1, 0);
        for (int k = 0; k < n; k++) {
            DevShot d;
            int rc = check_shot(sh[k], d);
            if (rc) return rc;
            off[k + 1] = off[k] + (long)d.nt * (d.rx1 - d.rx0);
            moff[k + 1] = moff[k] + (d.rx1 - d.rx0);
        }
        free_observed();
        cudaError_t e = sprec == FWI_SPREC_NATIVE ? cudaMalloc(&ostore, off[n] * sizeof(T))
                                                  : cudaMalloc(&ostore_h, off[n] * sizeof(__half));
        if (e == cudaSuccess && sprec == FWI_SPREC_FP16) e = cudaMalloc(&ostore_scale, moff[n] * sizeof(float));
        if (e != cudaSuccess) {
            free_observed();
            return fail(e);
        }
        ostore_shots.assign(sh, sh + n);
        ostore_off = off;
        ostore_moff = moff;
        return FWI_OK;
    }

    // FP16 store: scales and codes of shots [k0, k0 + nk) from FP32 records at src (shot k at
    // src_off + ostore_off[k] - ostore_off[k0]).
    int encode_observed(const T *src, long src_base, int k0, int nk)
    {
        for (int k = k0; k < k0 + nk; k++) {
            DevShot d;
            check_shot(ostore_shots[k], d);
            const int nr = d.rx1 - d.rx0;
            const long so = src_base + ostore_off[k] - ostore_off[k0];
            k_trace_scale<T><<<(nr + 127) / 128, 128, 0, st>>>(src, so, d.nt, nr, ostore_scale + ostore_moff[k]);
            k_trace_encode<T><<<eg((long)d.nt * nr), 256, 0, st>>>(src, so, d.nt, nr, ostore_scale + ostore_moff[k],
                                                                   ostore_h, ostore_off[k]);
            TRY_LAUNCH();
        }
        return FWI_OK;
    }

    int store_observed(const fwi_shot *sh, int n, const void *obs_in, int sprec) override
    {
        if (!obs_in) return FWI_ERR_ARG;
        int rc = observed_layout(sh, n, sprec);
        if (rc) return rc;
        const long total = ostore_off[n];
        if (ostore) {
            TRY(cudaMemcpyAsync(ostore, obs_in, total * sizeof(T), cudaMemcpyDefault, st));
        } else {
            // stage through a device copy when the records are in host memory
            cudaPointerAttributes pa{};
            const bool dev = cudaPointerGetAttributes(&pa, obs_in) == cudaSuccess && pa.type == cudaMemoryTypeDevice;
            cudaGetLastError();
            const T *src = (const T *)obs_in;
            T *tmp = nullptr;
            if (!dev) {
                TRY(cudaMalloc(&tmp, total * sizeof(T)));
                TRY(cudaMemcpyAsync(tmp, obs_in, total * sizeof(T), cudaMemcpyHostToDevice, st));
                src = tmp;
            }
            rc = encode_observed(src, 0, 0, n);
            TRY(cudaStreamSynchronize(st));
            if (tmp) cudaFree(tmp);
            if (rc) return rc;
        }
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    // The records modelled on the device from the model (v_hor, v_po, v_nmo), straight into the
    // store; the context's own model is kept.
    int model_observed(const fwi_shot *sh, int n, const void *a, const void *b, const void *c, int sprec) override
    {
        if (!a || !b || !c) return FWI_ERR_ARG;
        if (!have_wavelet) return FWI_ERR_STATE;
        int rc = observed_layout(sh, n, sprec);
        if (rc) return rc;
        const bool had_model = have_model;
        T *m3[3] = {vh, vp, vn};
        for (int k = 0; k < 3; k++) {
            if (!model_keep[k]) TRY(alloc(&model_keep[k], mslot));
            TRY(cudaMemcpyAsync(model_keep[k], m3[k], mslot * sizeof(T), cudaMemcpyDeviceToDevice, st));
        }
        if ((rc = set_model(a, b, c))) return rc;
        if (ostore) {
            rc = run(sh, n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, ostore, false);
        } else {
            // FP16: model a batch at a time into FP32 scratch, then encode it
            if (!ostore_tmp) TRY(alloc(&ostore_tmp, (size_t)B * nt_max * nrec_max));
            for (int b0 = 0; b0 < n && rc == FWI_OK; b0 += B) {
                const int nb = std::min(B, n - b0);
                rc = run(sh + b0, nb, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, ostore_tmp, false);
                if (rc == FWI_OK) rc = encode_observed(ostore_tmp, 0, b0, nb);
            }
        }
        for (int k = 0; k < 3; k++)
            TRY(cudaMemcpyAsync(m3[k], model_keep[k], mslot * sizeof(T), cudaMemcpyDeviceToDevice, st));
        have_model = had_model;
        models_dirty = true;
        TRY(cudaStreamSynchronize(st));
        if (rc) free_observed();
        return rc;
    }

    // ---------------------------------------------------------------- autotuner

    // For each batch shape the shots form: time `steps` forward steps and
    // `steps` adjoint steps (the tile passes of the batch's shots, at steps
    // where they all run) of candidate choices, by coordinate descent from the
    // built-in choice over the interior shots per block, the layer shots per
    // block and the CPML path, and record the fastest for later calls.  A
    // candidate replaces the best so far only if at least 1 % faster.  The
    // candidates' steps run on the context's own buffers; every call clears
    // those before use, so results only depend on the choice recorded.
    int autotune(const fwi_shot *sh, int n, int steps, fwi_tuning *out) override
    {
        NvtxRange range("fwi autotune");
        if (!have_model || !have_wavelet) return FWI_ERR_STATE;
        if (!sh || n <= 0 || steps <= 0) return FWI_ERR_ARG;
        std::vector<DevShot> all(n);
        std::vector<long> off(n + 1, 0);
        for (int k = 0; k < n; k++) {
            int rc = check_shot(sh[k], all[k]);
            if (rc) return rc;
            off[k + 1] = off[k] + (long)all[k].nt * (all[k].rx1 - all[k].rx0);
        }
        int rc = refresh_models();
        if (rc) return rc;
        const bool exact = cfg.mode == FWI_MODE_EXACT;
        const bool tiles = sizeof(T) == 4 && use_tma;  // the choices only steer the FP32 tile passes
        const std::vector<int> order = batch_order(all);  // the batches gradient calls form
        for (int b0 = 0; b0 < n; b0 += B) {
            const int nb = std::min(B, n - b0);
            std::vector<DevShot> bs(nb);
            int ntb = 0, nxm = 0;
            long ro = 0;
            for (int k = 0; k < nb; k++) {
                bs[k] = all[order[b0 + k]];
                bs[k].rec_off = ro;
                ro += off[order[b0 + k] + 1] - off[order[b0 + k]];
                ntb = std::max(ntb, bs[k].nt);
                nxm = std::max(nxm, bs[k].nx);
            }
            const std::vector<long> key = choice_key(bs, nxm);
            bool done = false;
            for (const Tuned &t : tuned) done |= t.key == key;
            if (done && !(b0 == 0 && out)) continue;
            TRY(cudaMemcpyAsync(shots, bs.data(), nb * sizeof(DevShot), cudaMemcpyHostToDevice, st));
            const int K = std::min(steps, ntb);
            const size_t lb = (size_t)nb * slot * sizeof(T);
            const Choice dflt = default_choice(bs, nxm);
            Choices best{dflt, dflt};
            // device time per step of phase ph (0 forward, 1 adjoint) with choice c.  The adjoint
            // steps run beside what runs beside them in a gradient call: with checkpoint storage
            // the segment recompute (forward steps on the recompute streams, with the forward's
            // choice), with boundary storage the image rebuild, one step per adjoint step.
            auto trial = [&](const Choice &c, int ph, double &us) -> int {
                for (auto &p : lvl) TRY(cudaMemsetAsync(p, 0, lb, st));
                for (auto &p : cp) TRY(cudaMemsetAsync(p, 0, lb, st));
                TRY(cudaMemsetAsync(amax, 0, (size_t)nb * (nt_max + 1) * sizeof(float), st));
                Batch<T> b = batch_view(nb);
                apply_choice(b, bs, nxm, c);
                const bool partner = ph == 1 && cfg.store != FWI_STORE_FULL;
                const bool recompute = cfg.store == FWI_STORE_CHECKPOINT;
                Batch<T> rb = batch_view(nb);
                if (partner) {
                    apply_choice(rb, bs, nxm, recompute ? best.fwd : c);
                    for (int k = 0; k < 6; k++) rb.lvl[k] = rlvl[k];
                    if (recompute)
                        for (int k = 0; k < 4; k++) rb.cp[k] = rcp[k];
                    rb.tma = use_tma ? (const void *)&rmaps : nullptr;
                    rb.rec = obs;
                }
                TRY(cudaEventRecord(ev[1], st));
                if (partner) {
                    TRY(cudaEventRecord(ev_rfork, st));
                    TRY(cudaStreamWaitEvent(rst, ev_rfork, 0));
                }
                int cur = 0, zsel = 0, rcur = 0;
                const int lag = exact ? 0 : 1;
                for (int k = 0; k < K; k++) {
                    if (ph == 0) {  // every shot runs at the last steps
                        const int g = ntb - K + k;
                        const int img = cfg.store == FWI_STORE_FULL ? g
                                        : cfg.store == FWI_STORE_CHECKPOINT ? g % n_img : -1;
                        fwi::launch_forward_step<T>(b, nxm, g, ntb, cur, img, exact, ss);
                    } else {  // ... and at the first adjoint iterations
                        const int img_g = std::max(0, ntb - 1 - lag - k);
                        const int base = cfg.store == FWI_STORE_FULL ? 0 : img_g - img_g % n_img;
                        fwi::launch_adjoint_step<T>(b, nxm, k, ntb, cur, zsel, exact, base, ss);
                        zsel ^= 1;
                        if (partner) {
                            const int g = ntb - 1 - k;
                            if (recompute)
                                fwi::launch_forward_step<T>(rb, nxm, g, ntb, rcur, g % n_img, exact, rss);
                            else
                                fwi::launch_rebuild_step<T>(rb, nxm, g, ntb, rcur, ring, ring_len, g & 1, rst);
                            rcur ^= 1;
                        }
                    }
                    cur ^= 1;
                }
                TRY_LAUNCH();
                if (partner) {  // the partner stream joins the timed region's end
                    TRY(cudaEventRecord(ev_reb[0], rst));
                    TRY(cudaStreamWaitEvent(st, ev_reb[0], 0));
                }
                TRY(cudaEventRecord(ev[2], st));
                TRY(cudaEventSynchronize(ev[2]));
                float ms = 0;
                TRY(cudaEventElapsedTime(&ms, ev[1], ev[2]));
                us = 1e3 * ms / K;
                return FWI_OK;
            };
            // a candidate's time: the median of three timed runs (single runs vary by a few
            // per cent, about the differences between neighbouring choices)
            auto timed = [&](const Choice &c, int ph, double &us) -> int {
                double v[3];
                for (double &x : v) {
                    const int r = trial(c, ph, x);
                    if (r) return r;
                }
                std::sort(v, v + 3);
                us = v[1];
                return FWI_OK;
            };
            double t_best[2] = {0, 0}, t_dflt[2] = {0, 0}, t = 0;
            int trials = 0;
            for (int ph = 0; ph < 2; ph++) {
                if ((rc = trial(dflt, ph, t))) return rc;  // warm-up
                if ((rc = timed(dflt, ph, t_dflt[ph]))) return rc;
                t_best[ph] = t_dflt[ph];
                trials++;
                Choice &bp = ph == 0 ? best.fwd : best.adj;
                auto consider = [&](const Choice &c) -> int {
                    if (c == bp) return FWI_OK;
                    const int r = timed(c, ph, t);
                    if (r) return r;
                    trials++;
                    if (t < 0.99 * t_best[ph]) {
                        bp = c;
                        t_best[ph] = t;
                    }
                    return FWI_OK;
                };
                if (!tiles) continue;
                // several windows: only the interior groups vary (layer groups need one window)
                const bool uniform = uniform_windows(bs);
                const int cand[] = {1, 2, 3, 4, 5, 6, 8, 10, 12, 16, 24, 32, 48, 64};
                const fwi::TileGrid tg = uniform ? fwi::tile_grid(nxm, nz, cfg.cpml) : fwi::TileGrid{};
                for (int pass = 0; pass < 2; pass++) {
                    for (int v : cand)
                        if (v <= nb) {
                            Choice c = bp;
                            c.sg = v;
                            if ((rc = consider(c))) return rc;
                        }
                    if (!uniform) continue;
                    for (int v : cand)
                        if (v <= nb) {
                            Choice c = bp;
                            c.sg_layer = v;
                            if ((rc = consider(c))) return rc;
                        }
                    if (tg.inline_strip) {
                        Choice c = bp;
                        c.inline_strip = !c.inline_strip;
                        if ((rc = consider(c))) return rc;
                    }
                }
                // the two group sizes interact (both passes share the SMs): every pair within two
                // candidate steps of the best, which the one-at-a-time descent above can miss
                if (uniform) {
                    const int ncand = (int)(sizeof(cand) / sizeof(cand[0]));
                    auto index_of = [&](int v) {
                        for (int k = 0; k < ncand; k++)
                            if (cand[k] == v) return k;
                        return 0;
                    };
                    const Choice centre = bp;
                    const int i0 = index_of(centre.sg), j0 = index_of(centre.sg_layer);
                    for (int di = -2; di <= 2; di++)
                        for (int dj = -2; dj <= 2; dj++) {
                            const int i = i0 + di, jj = j0 + dj;
                            if (i < 0 || jj < 0 || i >= ncand || jj >= ncand || cand[i] > nb || cand[jj] > nb) continue;
                            Choice c = centre;
                            c.sg = cand[i];
                            c.sg_layer = cand[jj];
                            if ((rc = consider(c))) return rc;
                        }
                }
            }
            record_choice(key, best);
            if (b0 == 0 && out) {
                for (int ph = 0; ph < 2; ph++) {
                    const Choice &c = ph == 0 ? best.fwd : best.adj;
                    fwi_phase_choice &o = ph == 0 ? out->forward : out->adjoint;
                    o.shots_per_group = c.sg;
                    o.layer_shots_per_group = c.sg_layer;
                    o.inline_strip = c.inline_strip;
                }
                out->trials = trials;
                out->forward_us = t_best[0];
                out->adjoint_us = t_best[1];
                out->default_forward_us = t_dflt[0];
                out->default_adjoint_us = t_dflt[1];
            }
        }
        TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st));  // candidates ran on stale inputs
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    // fwi_check_bounded_wait: the wait gives up, the status word says so, the
    // context stays usable (the status word is cleared by every later call).
    int check_bounded_wait(long polls) override
    {
        if (polls < 1 || polls > fwi::kWaitLimit) return FWI_ERR_ARG;
        TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
        k_check_bounded_wait<<<1, 128, 0, st>>>(status, polls);
        TRY_LAUNCH();
        unsigned stat = 0;
        TRY(cudaMemcpyAsync(&stat, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        TRY(cudaStreamSynchronize(st));
        TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
        return (stat & fwi::kStatusTimeout) ? FWI_ERR_CUDA : FWI_OK;
    }

    // Records choice t for the batch shapes the shots form.
    int set_tuning(const fwi_shot *sh, int n, const fwi_tuning *t) override
    {
        if (!sh || n <= 0 || !t) return FWI_ERR_ARG;
        Choices c;
        for (int ph = 0; ph < 2; ph++) {
            const fwi_phase_choice &i = ph == 0 ? t->forward : t->adjoint;
            Choice &o = ph == 0 ? c.fwd : c.adj;
            o.sg = i.shots_per_group;
            o.sg_layer = i.layer_shots_per_group;
            o.inline_strip = i.inline_strip ? 1 : 0;
            if (o.sg < 1 || o.sg > 64 || o.sg_layer < 1 || o.sg_layer > 64) return FWI_ERR_ARG;
        }
        std::vector<DevShot> all(n);
        for (int k = 0; k < n; k++) {
            int rc = check_shot(sh[k], all[k]);
            if (rc) return rc;
        }
        std::vector<std::pair<std::vector<long>, Choices>> add;
        const std::vector<int> order = batch_order(all);  // the batches gradient calls form
        for (int b0 = 0; b0 < n; b0 += B) {
            const int nb = std::min(B, n - b0);
            std::vector<DevShot> bs(nb);
            for (int k = 0; k < nb; k++) bs[k] = all[order[b0 + k]];
            int nxm = 0;
            for (const DevShot &d : bs) nxm = std::max(nxm, d.nx);
            Choices cb = c;
            if (!(sizeof(T) == 4 && use_tma)) {  // no tile passes: one shot per block
                for (Choice *o : {&cb.fwd, &cb.adj})
                    if (o->sg != 1 || o->sg_layer != 1) return FWI_ERR_ARG;
            }
            if (!uniform_windows(bs)) {  // several windows: layer tiles take one shot per block
                for (Choice *o : {&cb.fwd, &cb.adj}) {
                    if (o->sg_layer != 1) return FWI_ERR_ARG;
                    o->inline_strip = 0;
                }
            }
            add.emplace_back(choice_key(bs, nxm), cb);
        }
        for (auto &a : add) record_choice(a.first, a.second);
        return FWI_OK;
    }

    // ---------------------------------------------------------------- L-BFGS

    Tri<T> tri(T *const (&a)[3]) const { Tri<T> t; for (int k = 0; k < 3; k++) t.p[k] = a[k]; return t; }
    CTri<T> ctri(T *const (&a)[3]) const { CTri<T> t; for (int k = 0; k < 3; k++) t.p[k] = a[k]; return t; }
    CTri<T> cnull() const { CTri<T> t; for (int k = 0; k < 3; k++) t.p[k] = nullptr; return t; }

    int copy3(T *const (&dst)[3], T *const (&src)[3])
    {
        for (int k = 0; k < 3; k++) TRY(cudaMemcpyAsync(dst[k], src[k], mslot * sizeof(T), cudaMemcpyDeviceToDevice, st));
        return FWI_OK;
    }

    int first_step(float a_hor, float a_po, float a_nmo) override
    {
        if (!have_grad || !have_model) return FWI_ERR_STATE;
        T *m3[3] = {vh, vp, vn};
        int rc;
        if ((rc = copy3(mb, m3)) || (rc = copy3(gb, grad))) return rc;
        have_back = true;
        // |g|^2 over the whole grid (src/main.c:551-559), in FP64
        k_lb_copy_dot<T><<<red_blocks, kRedThreads, 0, st>>>(tri(q), ctri(grad), ctri(grad), mslot, ds, lbs->dots);
        k_lb_inv_norm<<<1, 32, 0, st>>>(lbs);
        k_first_update<T><<<eg((long)nx * nz), 256, 0, st>>>(vh, vp, vn, grad[0], grad[1], grad[2], lbs, a_hor,
                                                                   a_po, a_nmo, nx, nz, mpitch);
        TRY_LAUNCH();
        launches += 3;
        models_dirty = true;
        hist_count = 0;
        hist_next = 0;
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    int ensure_history(int m)
    {
        if (m <= hist_m) return FWI_OK;
        for (int l = hist_m; l < m; l++)
            for (int p = 0; p < 3; p++) {
                TRY(alloc(&hs[l][p], mslot));
                TRY(alloc(&hy[l][p], mslot));
            }
        hist_m = m;
        return FWI_OK;
    }

    int lbfgs_direction(int m, double *stats) override
    {
        NvtxRange range("fwi L-BFGS direction");
        if (m < 1 || m > kMaxHist) return FWI_ERR_ARG;
        if (!have_grad || !have_back) return FWI_ERR_STATE;
        int rc = ensure_history(m);
        if (rc) return rc;
        if (hist_count > m) hist_count = m;
        // newest pair into the ring
        const int k = hist_next % m;
        T *sk[3] = {hs[k][0], hs[k][1], hs[k][2]}, *yk[3] = {hy[k][0], hy[k][1], hy[k][2]};
        T *m3[3] = {vh, vp, vn};
        k_lb_pair<T><<<red_blocks, kRedThreads, 0, st>>>(tri(sk), tri(yk), ctri(m3), ctri(mb), ctri(grad), ctri(gb),
                                                         mslot, ds, lbs->pair);
        hist_next = (hist_next + 1) % m;
        hist_count = std::min(hist_count + 1, m);
        // order newest .. oldest
        std::vector<int> order;
        for (int a = 0; a < hist_count; a++) order.push_back(((hist_next - 1 - a) % m + m) % m);
        // first loop; q = g and rho_k, alpha_k of the newest pair
        int rcq = copy3(q, grad);
        if (rcq) return rcq;
        k_lb_scalar<<<1, 32, 0, st>>>(lbs, 0, order[0], lb_guard);
        // rho of the older slots persists from when they were formed
        for (size_t a = 0; a < order.size(); a++) {
            const int l = order[a];
            T *yl[3] = {hy[l][0], hy[l][1], hy[l][2]};
            if (a > 0) k_lb_scalar<<<1, 32, 0, st>>>(lbs, 1, l, lb_guard);
            const bool has_next = a + 1 < order.size();
            const int ln = has_next ? order[a + 1] : l;
            T *sn[3] = {hs[ln][0], hs[ln][1], hs[ln][2]};
            k_lb_axpy_dot<T><<<red_blocks, kRedThreads, 0, st>>>(tri(q), ctri(yl), nullptr, lbs->coefB, ctri(sn),
                                                                 has_next ? 1 : 0, mslot, ds, lbs->dots);
        }
        // r = gamma q; then the second loop oldest .. newest
        LbOrder lo{};
        lo.n = (int)order.size();
        for (int a = 0; a < lo.n; a++) lo.slot[a] = order[a];
        k_lb_gamma<<<1, 32, 0, st>>>(lbs, lo, lb_guard);
        int first = order.back();
        T *y0[3] = {hy[first][0], hy[first][1], hy[first][2]};
        rcq = copy3(r, q);
        if (rcq) return rcq;
        k_lb_axpy_dot<T><<<red_blocks, kRedThreads, 0, st>>>(tri(r), cnull(), lbs->coefA, nullptr, ctri(y0), 1, mslot,
                                                             ds, lbs->dots);
        for (int a = (int)order.size() - 1; a >= 0; a--) {
            const int l = order[a];
            T *sl[3] = {hs[l][0], hs[l][1], hs[l][2]};
            k_lb_scalar<<<1, 32, 0, st>>>(lbs, 3, l, lb_guard);
            const bool has_next = a > 0;
            const int ln = has_next ? order[a - 1] : l;
            T *yn[3] = {hy[ln][0], hy[ln][1], hy[ln][2]};
            k_lb_axpy_dot<T><<<red_blocks, kRedThreads, 0, st>>>(tri(r), ctri(sl), nullptr, lbs->coefB, ctri(yn),
                                                                 has_next ? 1 : 0, mslot, ds, lbs->dots);
        }
        TRY_LAUNCH();
        // the model and gradient this direction starts from (src/main.c:683-688)
        if ((rc = copy3(mb, m3)) || (rc = copy3(gb, grad))) return rc;
        have_dir = true;
        if (stats) {
            LbScalars h;
            TRY(cudaMemcpyAsync(&h, lbs, sizeof(h), cudaMemcpyDeviceToHost, st));
            TRY(cudaStreamSynchronize(st));
            for (int p = 0; p < 3; p++) {
                stats[p] = h.gamma[p];
                stats[3 + p] = h.rho[p][order[0]];
                stats[6 + p] = h.pair[p];      // y.s of the newest pair
                stats[9 + p] = h.pair[3 + p];  // y.y of the newest pair
            }
        }
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    void set_lbfgs_guard(int on) override { lb_guard = on ? 1 : 0; }

    int direction_slope(double *out3) override
    {
        if (!have_dir) return FWI_ERR_STATE;
        k_lb_slope<T><<<red_blocks, kRedThreads, 0, st>>>(ctri(gb), ctri(r), nx, nz, mpitch, ds, lbs->dots);
        TRY_LAUNCH();
        launches++;
        double d[3];
        TRY(cudaMemcpyAsync(d, lbs->dots, sizeof(d), cudaMemcpyDeviceToHost, st));
        TRY(cudaStreamSynchronize(st));
        for (int p = 0; p < 3; p++) out3[p] = d[p];
        return FWI_OK;
    }

    int lbfgs_update(float av, float ad, float ae, int fmin, int fmax) override
    {
        if (!have_back) return FWI_ERR_STATE;
        // av, ad, ae pair with (v_po, v_nmo, v_hor) as update_LBFGS does (src/main.c:693)
        k_lb_update<T><<<eg((long)nx * nz), 256, 0, st>>>(vh, vp, vn, mb[0], mb[1], mb[2], r[0], r[1], r[2], av,
                                                                ad, ae, fmin, fmax, nx, nz, mpitch);
        TRY_LAUNCH();
        launches++;
        models_dirty = true;
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    int restore_model() override
    {
        if (!have_back) return FWI_ERR_STATE;
        T *m3[3] = {vh, vp, vn};
        int rc = copy3(m3, mb);
        if (rc) return rc;
        models_dirty = true;
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }

    int set_gradient(const void *a, const void *b, const void *c) override
    {
        if (!a || !b || !c) return FWI_ERR_ARG;
        int rc;
        if ((rc = copy_model_in(grad[0], a)) || (rc = copy_model_in(grad[1], b)) || (rc = copy_model_in(grad[2], c)))
            return rc;
        TRY(cudaStreamSynchronize(st));
        have_grad = true;
        return FWI_OK;
    }

    int gradient_vti(void *o0, void *o1, void *o2) override
    {
        if (!have_grad) return FWI_ERR_STATE;
        for (auto &p : vti_out)
            if (!p) TRY(alloc(&p, mslot));
        k_grad_vti<T><<<eg((long)nx * nz), 256, 0, st>>>(vh, vp, vn, grad[0], grad[1], grad[2], vti_out[0],
                                                               vti_out[1], vti_out[2], nx, nz, mpitch);
        TRY_LAUNCH();
        void *outs[3] = {o0, o1, o2};
        for (int k = 0; k < 3; k++)
            if (outs[k])
                TRY(cudaMemcpy2DAsync(outs[k], nx * sizeof(T), vti_out[k], mpitch * sizeof(T), nx * sizeof(T), nz,
                                      cudaMemcpyDefault, st));
        TRY(cudaStreamSynchronize(st));
        return FWI_OK;
    }
};

CtxBase *as_ctx(void *p) { return static_cast<CtxBase *>(p); }

}  // namespace

extern "C" {

void fwi_config_default(fwi_config *c)
{
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->nx = 201;
    c->nz = 201;
    c->dh = 10.f;
    c->dt = 1e-3f;
    c->cpml = 20;
    c->f_cpml = 10.f;
    c->vmax = 6000.f;
    c->r_coef = 1e-6f;
    c->nt_max = 2000;
    c->max_shots = 1;
    c->mode = FWI_MODE_EXACT;
    c->precision = FWI_PREC_FP32;
    c->store = FWI_STORE_FULL;
    c->store_prec = FWI_SPREC_NATIVE;
}

size_t fwi_config_bytes(const fwi_config *c)
{
    if (!c) return 0;
    const size_t e = c->precision == FWI_PREC_FP64 ? 8 : 4;
    const size_t se = c->store_prec == FWI_SPREC_NATIVE ? e : 2;
    const long win = c->max_window > 0 ? c->max_window : c->nx;
    const long slot = (long)c->nz * round_up(win, 32), mslot = (long)c->nz * round_up(c->nx, 32);
    const long nrec = c->max_receivers > 0 ? c->max_receivers : win;
    size_t b = 0;
    b += (size_t)(6 + 3 + 12) * mslot * e;                 // models, gradient, L-BFGS work arrays
    b += (size_t)c->max_shots * slot * e * (6 + 8 + 3);  // levels, CPML state, gradients
    if (c->store == FWI_STORE_CHECKPOINT) {
        const long k = checkpoint_interval(*c), n = (c->nt_max + k - 1) / k;
        b += (size_t)c->max_shots * slot * e * (8 * n + 10); // checkpoints, recompute state
        b += (size_t)c->max_shots * 2 * k * 2 * slot * se;   // images of two segments
    } else if (c->store == FWI_STORE_BOUNDARY) {
        b += (size_t)c->max_shots * c->nt_max * fwi::boundary_ring_len((int)win, c->nz, c->cpml) * e;  // rings
        b += (size_t)c->max_shots * slot * (6 * e + 4 * se);  // rebuild state, two images
    } else {
        b += (size_t)c->max_shots * c->nt_max * 2 * slot * se; // images
    }
    b += (size_t)c->max_shots * c->nt_max * nrec * e * 2;  // records and observed data
    return b;
}

int fwi_create(const fwi_config *cfg, void **out)
{
    if (!cfg || !out) return FWI_ERR_ARG;
    *out = nullptr;
    if (cfg->nx < 2 * cfg->cpml + 9 || cfg->nz < cfg->cpml + 9 || cfg->cpml < 0 || cfg->nt_max <= 0 ||
        cfg->max_shots <= 0 || !(cfg->dh > 0) || !(cfg->dt > 0) || cfg->max_window < 0 || cfg->max_window > cfg->nx ||
        cfg->ckpt_every < 0 || cfg->device < 0)
        return FWI_ERR_ARG;
    if (cfg->mode != FWI_MODE_EXACT && cfg->mode != FWI_MODE_REF_COMPAT) return FWI_ERR_ARG;
    if (cfg->store != FWI_STORE_FULL && cfg->store != FWI_STORE_CHECKPOINT && cfg->store != FWI_STORE_BOUNDARY)
        return FWI_ERR_ARG;
    if (cfg->store == FWI_STORE_BOUNDARY && cfg->cpml < 8) return FWI_ERR_UNSUPPORTED;  // ring inside the layers
    if (cfg->store_prec < FWI_SPREC_NATIVE || cfg->store_prec > FWI_SPREC_BF16) return FWI_ERR_ARG;
    if (cfg->precision == FWI_PREC_FP64 && cfg->store_prec != FWI_SPREC_NATIVE) return FWI_ERR_UNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device) {
        cudaGetLastError();
        return FWI_ERR_NODEVICE;
    }
    CtxBase *c = nullptr;
    if (cfg->precision == FWI_PREC_FP32) c = new Ctx<float>();
    else if (cfg->precision == FWI_PREC_FP64) c = new Ctx<double>();
    else return FWI_ERR_ARG;
    c->cfg = *cfg;
    int rc = c->init();
    if (rc) {
        delete c;
        return rc;
    }
    *out = c;
    return FWI_OK;
}

void fwi_destroy(void *ctx) { delete as_ctx(ctx); }

const char *fwi_strerror(int s)
{
    switch (s) {
    case FWI_OK: return "ok";
    case FWI_ERR_ARG: return "invalid argument";
    case FWI_ERR_CUDA: return "CUDA error";
    case FWI_ERR_NOMEM: return "out of device memory";
    case FWI_ERR_STATE: return "call out of order";
    case FWI_ERR_NUMERIC: return "non-finite value or saturated image storage";
    case FWI_ERR_UNSUPPORTED: return "unsupported configuration";
    case FWI_ERR_NODEVICE: return "no usable CUDA device";
    default: return "unknown status";
    }
}

int fwi_last_cuda_error(void *ctx) { return ctx ? as_ctx(ctx)->last_cuda : 0; }

int fwi_set_model(void *ctx, const void *a, const void *b, const void *c)
{
    return ctx ? as_ctx(ctx)->set_model(a, b, c) : FWI_ERR_ARG;
}
int fwi_set_model_vti(void *ctx, const void *a, const void *b, const void *c)
{
    return ctx ? as_ctx(ctx)->set_model_vti(a, b, c) : FWI_ERR_ARG;
}
int fwi_get_model(void *ctx, void *a, void *b, void *c) { return ctx ? as_ctx(ctx)->get_model(a, b, c) : FWI_ERR_ARG; }
int fwi_set_wavelet(void *ctx, const void *w, int nt) { return ctx ? as_ctx(ctx)->set_wavelet(w, nt) : FWI_ERR_ARG; }
int fwi_set_ricker(void *ctx, float f, int nt) { return ctx ? as_ctx(ctx)->set_ricker(f, nt) : FWI_ERR_ARG; }
int fwi_set_frequency(void *ctx, float f, int nt) { return ctx ? as_ctx(ctx)->set_frequency(f, nt) : FWI_ERR_ARG; }

int fwi_forward(void *ctx, const fwi_shot *shots, int n, void *traces)
{
    if (!ctx || !traces) return FWI_ERR_ARG;
    return as_ctx(ctx)->run(shots, n, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, traces, false);
}

int fwi_gradient(void *ctx, const fwi_shot *shots, int n, const void *obs, const unsigned char *mask, void *gh,
                 void *gp, void *gn, double *misfit)
{
    if (!ctx) return FWI_ERR_ARG;
    return as_ctx(ctx)->run(shots, n, obs, mask, gh, gp, gn, misfit, nullptr, true);
}

int fwi_misfit(void *ctx, const fwi_shot *shots, int n, const void *obs, const unsigned char *mask, double *misfit)
{
    if (!ctx || !misfit) return FWI_ERR_ARG;
    return as_ctx(ctx)->run(shots, n, obs, mask, nullptr, nullptr, nullptr, misfit, nullptr, false);
}

int fwi_set_gradient(void *ctx, const void *a, const void *b, const void *c)
{
    return ctx ? as_ctx(ctx)->set_gradient(a, b, c) : FWI_ERR_ARG;
}
int fwi_first_step(void *ctx, float a, float b, float c) { return ctx ? as_ctx(ctx)->first_step(a, b, c) : FWI_ERR_ARG; }
int fwi_lbfgs_direction(void *ctx, int m, double *stats)
{
    return ctx ? as_ctx(ctx)->lbfgs_direction(m, stats) : FWI_ERR_ARG;
}
int fwi_store_observed(void *ctx, const fwi_shot *shots, int n, const void *obs, int store_prec)
{
    return ctx ? as_ctx(ctx)->store_observed(shots, n, obs, store_prec) : FWI_ERR_ARG;
}
int fwi_model_observed(void *ctx, const fwi_shot *shots, int n, const void *v_hor, const void *v_po,
                       const void *v_nmo, int store_prec)
{
    return ctx ? as_ctx(ctx)->model_observed(shots, n, v_hor, v_po, v_nmo, store_prec) : FWI_ERR_ARG;
}
int fwi_free_observed(void *ctx) { return ctx ? as_ctx(ctx)->free_observed() : FWI_ERR_ARG; }

int fwi_set_lbfgs_guard(void *ctx, int on)
{
    if (!ctx) return FWI_ERR_ARG;
    as_ctx(ctx)->set_lbfgs_guard(on);
    return FWI_OK;
}

int fwi_get_config(void *ctx, fwi_config *out)
{
    if (!ctx || !out) return FWI_ERR_ARG;
    *out = as_ctx(ctx)->cfg;
    return FWI_OK;
}

int fwi_direction_slope(void *ctx, double *out3)
{
    if (!ctx || !out3) return FWI_ERR_ARG;
    return as_ctx(ctx)->direction_slope(out3);
}
int fwi_lbfgs_update(void *ctx, float av, float ad, float ae, int fmin, int fmax)
{
    return ctx ? as_ctx(ctx)->lbfgs_update(av, ad, ae, fmin, fmax) : FWI_ERR_ARG;
}
int fwi_restore_model(void *ctx) { return ctx ? as_ctx(ctx)->restore_model() : FWI_ERR_ARG; }
int fwi_gradient_vti(void *ctx, void *a, void *b, void *c) { return ctx ? as_ctx(ctx)->gradient_vti(a, b, c) : FWI_ERR_ARG; }

int fwi_set_tile_timing(void *ctx, int on)
{
    if (!ctx) return FWI_ERR_ARG;
    return as_ctx(ctx)->set_tile_timing(on != 0);
}

int fwi_last_tile_timing(void *ctx, double *out4)
{
    if (!ctx || !out4) return FWI_ERR_ARG;
    CtxBase *c = as_ctx(ctx);
    for (int p = 0; p < 2; p++) {
        const long n = c->tile_n[p];
        out4[2 * p] = n ? c->tile_ms[p] / n : 0.0;
        out4[2 * p + 1] = n ? c->tile_pts[p] / n : 0.0;
    }
    return FWI_OK;
}

int fwi_last_recompute_timing(void *ctx, double *out3)
{
    if (!ctx || !out3) return FWI_ERR_ARG;
    CtxBase *c = as_ctx(ctx);
    const long n = c->tile_n[2];
    out3[0] = n ? c->tile_ms[2] / n : 0.0;
    out3[1] = n ? c->tile_pts[2] / n : 0.0;
    out3[2] = (double)c->recompute_steps;
    return FWI_OK;
}

int fwi_last_timing(void *ctx, float *out4)
{
    if (!ctx || !out4) return FWI_ERR_ARG;
    memcpy(out4, as_ctx(ctx)->timing, sizeof(float) * 4);
    return FWI_OK;
}

long fwi_last_launches(void *ctx) { return ctx ? as_ctx(ctx)->launches : 0; }

int fwi_autotune(void *ctx, const fwi_shot *shots, int nshots, int steps, fwi_tuning *out)
{
    if (!ctx) return FWI_ERR_ARG;
    return as_ctx(ctx)->autotune(shots, nshots, steps, out);
}

int fwi_set_tuning(void *ctx, const fwi_shot *shots, int nshots, const fwi_tuning *t)
{
    if (!ctx) return FWI_ERR_ARG;
    return as_ctx(ctx)->set_tuning(shots, nshots, t);
}

int fwi_check_bounded_wait(void *ctx, long polls)
{
    if (!ctx) return FWI_ERR_ARG;
    return as_ctx(ctx)->check_bounded_wait(polls);
}

int fwi_set_graphs(void *ctx, int on)
{
    if (!ctx) return FWI_ERR_ARG;
    return as_ctx(ctx)->set_graphs(on != 0);
}

int fwi_graph_stats(void *ctx, long *out2)
{
    if (!ctx || !out2) return FWI_ERR_ARG;
    const CtxBase *c = as_ctx(ctx);
    out2[0] = c->graph_replays;
    out2[1] = c->graph_captures;
    return FWI_OK;
}

long fwi_strip_points(int nx, int nz, int cpml, int *ix, int *iz, long cap)
{
    fwi::StripMap sm = fwi::StripMap::make(nx, nz, cpml);
    long n = sm.count();
    for (long k = 0; k < n && k < cap; k++) {
        int a, b;
        sm.point(k, a, b);
        if (ix) ix[k] = a;
        if (iz) iz[k] = b;
    }
    return n;
}

}  // extern "C"
