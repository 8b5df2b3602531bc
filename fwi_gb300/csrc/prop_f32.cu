// FP32 propagation, per step: the strip pass of prop.cuh (memory variables),
// the TMA tile pass, then the layer-point pass (prop_tma.cuh).  The generic
// main passes of prop.cuh serve FP64.
#include "prop_tma.cuh"

namespace fwi {

namespace {

template <typename K> void allow_smem(K kernel, size_t bytes)
{
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

inline dim3 tma_grid(const Batch<float> &b, int nx_max)
{
    return dim3((nx_max + TT - 1) / TT, (b.nz + TT - 1) / TT, (b.B + b.sg - 1) / b.sg);
}

// Layer-point kernels: enough blocks for every point of the widest window, `ny` in y.
inline dim3 layer_grid(const Batch<float> &b, int nx_max, int width, int ny)
{
    const long n = StripMap::make(nx_max, b.nz, width).count();
    long blocks = (n + kStripBlock - 1) / kStripBlock;
    if (blocks < 1) blocks = 1;
    return dim3((unsigned)blocks, (unsigned)ny);
}

template <int ST, bool EXACT>
void fwd_tma(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, cudaStream_t st)
{
    static bool set = false;
    const size_t sm = fwd_tma_smem();
    if (!set) { allow_smem(k_fwd_tma<ST, EXACT>, sm); set = true; }
    k_fwd_tma<ST, EXACT><<<tma_grid(b, nx_max), kTmaThreads, sm, st>>>(
        b, *static_cast<const TmaMaps *>(b.tma), g, ntb, cur, slot, b.sg);
    k_fwd_cpml<ST, EXACT><<<layer_grid(b, nx_max, b.cpml, b.B), kStripBlock, 0, st>>>(b, g, ntb, cur, slot);
}

template <int ST, bool EXACT>
void adj_tma(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, int img_base, cudaStream_t st)
{
    static bool set = false;
    const size_t sm = adj_tma_smem<typename Codec<float, ST>::S>();
    if (!set) { allow_smem(k_adj_tma<ST, EXACT>, sm); set = true; }
    k_adj_tma<ST, EXACT><<<tma_grid(b, nx_max), kTmaThreads, sm, st>>>(
        b, *static_cast<const TmaMaps *>(b.tma), j, ntb, cur, img_base, b.sg);
    const int width = EXACT ? b.cpml + kRad : b.cpml;
    k_adj_cpml<ST, EXACT><<<layer_grid(b, nx_max, width, (b.B + b.sg - 1) / b.sg), kStripBlock, 0, st>>>(
        b, j, ntb, cur, zsel, img_base, b.sg);
}

template <int ST>
void fwd_tma_mode(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, bool exact, cudaStream_t st)
{
    if (exact) fwd_tma<ST, true>(b, nx_max, g, ntb, cur, slot, st);
    else fwd_tma<ST, false>(b, nx_max, g, ntb, cur, slot, st);
}

template <int ST>
void adj_tma_mode(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact, int base,
                  cudaStream_t st)
{
    if (exact) adj_tma<ST, true>(b, nx_max, j, ntb, cur, zsel, base, st);
    else adj_tma<ST, false>(b, nx_max, j, ntb, cur, zsel, base, st);
}

}  // namespace

template <>
void launch_forward_step<float>(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int img_slot,
                                bool exact, cudaStream_t st)
{
    k_fwd_strip<float><<<strip_grid(b, nx_max), kStripBlock, 0, st>>>(b, g, ntb, cur);
    switch (b.store_type) {
    case kStoreHalf: fwd_tma_mode<kStoreHalf>(b, nx_max, g, ntb, cur, img_slot, exact, st); break;
    case kStoreBf16: fwd_tma_mode<kStoreBf16>(b, nx_max, g, ntb, cur, img_slot, exact, st); break;
    default: fwd_tma_mode<kStoreNative>(b, nx_max, g, ntb, cur, img_slot, exact, st); break;
    }
}

template <>
void launch_adjoint_step<float>(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact,
                                int img_base, cudaStream_t st)
{
    if (exact) k_adj_strip_exact<float><<<strip_grid(b, nx_max), kStripBlock, 0, st>>>(b, j, cur, zsel);
    else k_adj_strip_ref<float><<<strip_grid(b, nx_max), kStripBlock, 0, st>>>(b, j, cur);
    switch (b.store_type) {
    case kStoreHalf: adj_tma_mode<kStoreHalf>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st); break;
    case kStoreBf16: adj_tma_mode<kStoreBf16>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st); break;
    default: adj_tma_mode<kStoreNative>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st); break;
    }
}

}  // namespace fwi
