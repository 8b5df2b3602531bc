// FP32 propagation, per step (streams of StepStreams):
//   strip stream: strip pass (prop.cuh: the CPML memory variables)
//   side stream:  layer tiles (prop_tma.cuh, LAYER = true: their points
//                 outside the layers, and the stencils of the layer points to
//                 scratch) -> [after the strip pass] layer points
//                 (k_fwd_cpml / k_adj_cpml)
//   main stream:  interior tiles (prop_tma.cuh, LAYER = false)
// joined before the next step.  All of them read only the current time level
// and write disjoint points.  The generic passes of prop.cuh serve FP64.
#include "prop_tma.cuh"

namespace fwi {

namespace {

template <typename K> void allow_smem(K kernel, size_t bytes)
{
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

inline dim3 tma_grid(const Batch<float> &b, int nx_max, int sg)
{
    return dim3((nx_max + TT - 1) / TT, (b.nz + TT - 1) / TT, (b.B + sg - 1) / sg);
}

// Layer-point kernels: enough blocks for every point of the widest window, `ny` in y.
inline dim3 layer_grid(const Batch<float> &b, int nx_max, int width, int ny)
{
    const long n = StripMap::make(nx_max, b.nz, width).count();
    long blocks = (n + kStripBlock - 1) / kStripBlock;
    if (blocks < 1) blocks = 1;
    return dim3((unsigned)blocks, (unsigned)ny);
}

template <int ST, bool EXACT, bool LAYER>
void fwd_tiles(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, cudaStream_t st)
{
    static bool set = false;
    const size_t sm = fwd_tma_smem();
    if (!set) { allow_smem(k_fwd_tma<ST, EXACT, LAYER>, sm); set = true; }
    const int sg = LAYER ? b.sg_layer : b.sg;
    k_fwd_tma<ST, EXACT, LAYER><<<tma_grid(b, nx_max, sg), kTmaThreads, sm, st>>>(
        b, *static_cast<const TmaMaps *>(b.tma), g, ntb, cur, slot, sg);
}

template <int ST, bool EXACT, bool LAYER>
void adj_tiles(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, int img_base, cudaStream_t st)
{
    static bool set = false;
    const size_t sm = adj_tma_smem();
    if (!set) { allow_smem(k_adj_tma<ST, EXACT, LAYER>, sm); set = true; }
    const int sg = LAYER ? b.sg_layer : b.sg;
    k_adj_tma<ST, EXACT, LAYER><<<tma_grid(b, nx_max, sg), kTmaThreads, sm, st>>>(
        b, *static_cast<const TmaMaps *>(b.tma), j, ntb, cur, zsel, img_base, sg);
}

// The forward tiles compute the same thing in both modes (the points they
// finish have no CPML term, so their images are the plain stencils in both):
// one instantiation serves both; the layer points' images are k_fwd_cpml's.
template <int ST>
void fwd_step(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, cudaStream_t st, bool layer)
{
    if (!layer) fwd_tiles<ST, false, false>(b, nx_max, g, ntb, cur, slot, st);
    else fwd_tiles<ST, false, true>(b, nx_max, g, ntb, cur, slot, st);
}

template <int ST>
void fwd_points(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, bool exact, cudaStream_t st)
{
    const dim3 grid = layer_grid(b, nx_max, b.cpml, b.B);
    if (exact) k_fwd_cpml<ST, true><<<grid, kStripBlock, 0, st>>>(b, g, ntb, cur, slot);
    else k_fwd_cpml<ST, false><<<grid, kStripBlock, 0, st>>>(b, g, ntb, cur, slot);
}

template <int ST>
void adj_points(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact, int base,
                cudaStream_t st)
{
    const int ng = (b.B + b.sg - 1) / b.sg;
    if (exact)
        k_adj_cpml<ST, true><<<layer_grid(b, nx_max, b.cpml + kRad, ng), kStripBlock, 0, st>>>(b, j, ntb, cur, zsel,
                                                                                              base, b.sg);
    else
        k_adj_cpml<ST, false><<<layer_grid(b, nx_max, b.cpml, ng), kStripBlock, 0, st>>>(b, j, ntb, cur, zsel, base,
                                                                                        b.sg);
}

template <int ST>
void adj_step(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact, int base,
              cudaStream_t st, bool layer)
{
    if (exact) {
        if (layer) adj_tiles<ST, true, true>(b, nx_max, j, ntb, cur, zsel, base, st);
        else adj_tiles<ST, true, false>(b, nx_max, j, ntb, cur, zsel, base, st);
    } else {
        if (layer) adj_tiles<ST, false, true>(b, nx_max, j, ntb, cur, zsel, base, st);
        else adj_tiles<ST, false, false>(b, nx_max, j, ntb, cur, zsel, base, st);
    }
}

// One step's work on three streams: `strip_work` (strip pass) on ss.strip,
// `layer_work` (layer tiles) on ss.side then, after the strip pass,
// `point_work` (layer points) there too, and `interior_work` on ss.main,
// which then waits for ss.side.  Without side streams: all in that order on
// ss.main.
template <typename Strip, typename Layer, typename Points, typename Interior>
void fork_join(const StepStreams &ss, Strip strip_work, Layer layer_work, Points point_work,
               Interior interior_work)
{
    if (!ss.side) {
        strip_work(ss.main);
        layer_work(ss.main);
        point_work(ss.main);
        interior_work(ss.main);
        return;
    }
    cudaEventRecord(ss.fork, ss.main);
    cudaStreamWaitEvent(ss.strip, ss.fork, 0);
    cudaStreamWaitEvent(ss.side, ss.fork, 0);
    strip_work(ss.strip);
    cudaEventRecord(ss.strip_done, ss.strip);
    layer_work(ss.side);
    cudaStreamWaitEvent(ss.side, ss.strip_done, 0);
    point_work(ss.side);
    cudaEventRecord(ss.join, ss.side);
    if (ss.t0) cudaEventRecord(ss.t0, ss.main);
    interior_work(ss.main);
    if (ss.t1) cudaEventRecord(ss.t1, ss.main);
    cudaStreamWaitEvent(ss.main, ss.join, 0);
}

}  // namespace

template <>
void launch_forward_step<float>(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int img_slot,
                                bool exact, const StepStreams &ss)
{
    auto tiles = [&](cudaStream_t st, bool layer) {
        switch (b.store_type) {
        case kStoreHalf: fwd_step<kStoreHalf>(b, nx_max, g, ntb, cur, img_slot, st, layer); break;
        case kStoreBf16: fwd_step<kStoreBf16>(b, nx_max, g, ntb, cur, img_slot, st, layer); break;
        default: fwd_step<kStoreNative>(b, nx_max, g, ntb, cur, img_slot, st, layer); break;
        }
    };
    fork_join(
        ss, [&](cudaStream_t s) { k_fwd_strip<float><<<strip_grid(b, nx_max), kStripBlock, 0, s>>>(b, g, ntb, cur); },
        [&](cudaStream_t s) { tiles(s, true); },
        [&](cudaStream_t s) {
            switch (b.store_type) {
            case kStoreHalf: fwd_points<kStoreHalf>(b, nx_max, g, ntb, cur, img_slot, exact, s); break;
            case kStoreBf16: fwd_points<kStoreBf16>(b, nx_max, g, ntb, cur, img_slot, exact, s); break;
            default: fwd_points<kStoreNative>(b, nx_max, g, ntb, cur, img_slot, exact, s); break;
            }
        },
        [&](cudaStream_t s) { tiles(s, false); });
}

template <>
void launch_adjoint_step<float>(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact,
                                int img_base, const StepStreams &ss)
{
    auto tiles = [&](cudaStream_t st, bool layer) {
        switch (b.store_type) {
        case kStoreHalf: adj_step<kStoreHalf>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st, layer); break;
        case kStoreBf16: adj_step<kStoreBf16>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st, layer); break;
        default: adj_step<kStoreNative>(b, nx_max, j, ntb, cur, zsel, exact, img_base, st, layer); break;
        }
    };
    fork_join(
        ss,
        [&](cudaStream_t s) {
            if (exact) k_adj_strip_exact<float><<<strip_grid(b, nx_max), kStripBlock, 0, s>>>(b, j, cur, zsel);
            else k_adj_strip_ref<float><<<strip_grid(b, nx_max), kStripBlock, 0, s>>>(b, j, cur);
        },
        [&](cudaStream_t s) { tiles(s, true); },
        [&](cudaStream_t s) {
            switch (b.store_type) {
            case kStoreHalf: adj_points<kStoreHalf>(b, nx_max, j, ntb, cur, zsel, exact, img_base, s); break;
            case kStoreBf16: adj_points<kStoreBf16>(b, nx_max, j, ntb, cur, zsel, exact, img_base, s); break;
            default: adj_points<kStoreNative>(b, nx_max, j, ntb, cur, zsel, exact, img_base, s); break;
            }
        },
        [&](cudaStream_t s) { tiles(s, false); });
}

}  // namespace fwi
