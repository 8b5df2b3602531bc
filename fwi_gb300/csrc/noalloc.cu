// Residual and misfit of device-resident traces without any device allocation
// (fwi_residual_misfit_noalloc in include/fwi.h).
//
// Callers that own all device memory themselves -- a host driver shaped like
// the reference's main.c, which allocates every buffer once before its shot
// loop (src/main.c:140-228), or a process whose device memory belongs to
// another allocator with a fixed budget -- cannot have the library call
// cudaMalloc inside their loop.  This entry point gives them the fused
// residual + FP64 misfit reduction of the native path (the work of
// src/parallelcalls.cu:133-142 plus the host loop of src/main.c:437-454)
// with its scratch in a fixed-size array in this file instead of a context.
#include "../../include/fwi.h"

#include <cuda_runtime.h>

namespace {

constexpr int kChunk = 4096;     // elements each block reduces (fixed, so the sum order is too)
constexpr int kThreads = 256;

// Per-block FP64 partial sums, then the completion counter in the last slot.
// Every GPU that loads the library holds this array (128 KiB + 8 B) until exit.
static __device__ __align__(256) double g_scratch[FWI_NOALLOC_MAX_BLOCKS + 1];

__global__ void k_residual_noalloc(float *res, const float *__restrict__ syn, const float *__restrict__ obs,
                                   const unsigned char *__restrict__ mask, long n, int nrec, double *scratch,
                                   double *misfit_out)
{
    double acc = 0.0;
    const long base = (long)blockIdx.x * kChunk;
    for (int k = threadIdx.x; k < kChunk; k += blockDim.x) {
        const long e = base + k;
        if (e >= n) break;
        float d = syn[e] - obs[e];
        if (mask && !mask[e % nrec]) d = 0.f;
        res[e] = d;
        acc += (double)d * (double)d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double w[kThreads / 32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < kThreads / 32; q++) t += w[q];
        scratch[blockIdx.x] = t;
        __threadfence();
        unsigned *counter = (unsigned *)&scratch[FWI_NOALLOC_MAX_BLOCKS];
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double t = 0.0;
    for (unsigned b = 0; b < gridDim.x; b++) t += ((volatile double *)scratch)[b];  // block order
    *misfit_out = 0.5 * t;
    *(unsigned *)&scratch[FWI_NOALLOC_MAX_BLOCKS] = 0u;
}

// Device address of the scratch array on the current device.  The host-side
// name g_scratch is not a device address, so it is looked up with the device
// current, on every call: a host-side table lookup once the module is loaded
// there, and never stale (after cudaDeviceReset the module loads again,
// possibly at another address) nor shared between host threads.
int scratch_for_current_device(double **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return FWI_ERR_NODEVICE;
    }
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return e == cudaErrorNoKernelImageForDevice ? FWI_ERR_NODEVICE : FWI_ERR_CUDA;
    }
    *out = (double *)p;
    return FWI_OK;
}

}  // namespace

extern "C" int fwi_residual_misfit_noalloc(float *res, const float *syn, const float *obs,
                                           const unsigned char *mask, long nt, int nrec, double *misfit,
                                           void *stream)
{
    if (!res || !syn || !obs || !misfit || nt <= 0 || nrec <= 0) return FWI_ERR_ARG;
    if (nt > FWI_NOALLOC_MAX_ELEMENTS / nrec) return FWI_ERR_ARG;  // before nt * nrec can overflow
    const long n = nt * (long)nrec;
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != FWI_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // the counter must start at zero whatever an earlier call left behind
    cudaError_t e = cudaMemsetAsync(scratch + FWI_NOALLOC_MAX_BLOCKS, 0, sizeof(double), st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return FWI_ERR_CUDA;
    }
    const unsigned blocks = (unsigned)((n + kChunk - 1) / kChunk);
    k_residual_noalloc<<<blocks, kThreads, 0, st>>>(res, syn, obs, mask, n, nrec, scratch, misfit);
    e = cudaGetLastError();
    return e == cudaSuccess ? FWI_OK : FWI_ERR_CUDA;
}
