// Tensor Memory Accelerator (TMA) bulk tile loads and mbarriers, as inline PTX
// for sm_103a, plus the host-side tensor-map encoder.
//
// Every wait on an mbarrier is bounded: after kWaitLimit polls the waiting
// thread records kStatusTimeout in the batch status word and the caller
// returns (no trap, no endless spin).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace fwi {

constexpr unsigned kStatusSaturated = 1u;  // an FP16 image value was clamped
constexpr unsigned kStatusTimeout = 2u;    // an mbarrier wait gave up
constexpr long kWaitLimit = 1L << 22;      // polls (each a try_wait with its own time slice)

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Returns false if the phase did not complete within `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, long limit = kWaitLimit)
{
    const uint32_t a = smem_addr(bar);
    for (long k = 0; k < limit; k++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) writes to the same buffers.
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 3-D tiled bulk copy global -> shared, completion counted on `bar`.
// x * element size must be a multiple of 16 bytes (callers pass x = a
// multiple of 4 floats or 8 halves); y and z may be negative or beyond the
// extent (zero fill).
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace fwi

// ------------------------------------------------------------------ host side

namespace fwi {

// cuTensorMapEncodeTiled, fetched from the driver at run time (no libcuda link).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn tensor_map_encoder();

// A [depth][rows][pitch] array of `elem`-byte elements (pitch, rows in
// elements), box (bx, by, bz).  Out-of-range elements load as zero.
int make_tensor_map_3d(CUtensorMap *map, const void *base, CUtensorMapDataType type, int elem, long pitch,
                       long rows, long depth, int bx, int by, int bz);

}  // namespace fwi
