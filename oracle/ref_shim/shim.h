/*
 * Force-included when compiling the reference's src/parallelcalls.cu as host
 * C++ (oracle/Makefile target `ref`).  The reference kernels use no shared
 * memory, no barriers and no intrinsics, so a kernel body run once per
 * (blockIdx, threadIdx) pair on the CPU gives what the GPU computes (up to
 * multiply-add fusion, which -ffp-contract=off turns off).
 *
 * Test infrastructure only: the result lands in oracle/_ref/, is never
 * committed and never linked into the product.
 */
#ifndef FWI_REF_SHIM_H
#define FWI_REF_SHIM_H

#include <cmath>
#include <math.h>

struct shim_dim3 {
    unsigned int x, y, z;
};

extern shim_dim3 threadIdx, blockIdx, blockDim;

#define __global__

#endif
