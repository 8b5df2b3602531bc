// FP32 propagation, per step, on two streams (StepStreams):
//   side stream (high priority): layer tiles (prop_layer.cuh), which advance
//                 the CPML memory variables themselves when the tile grid
//                 allows (TileGrid::inline_strip), else after the strip
//                 pass of prop.cuh
//   main stream:  interior tiles (prop_tma.cuh)
// joined before the next step.  Both tile passes read only the current time
// level and write disjoint points.  The generic passes of prop.cuh serve FP64.
// Small shots with full storage take the other route: one thread-block cluster
// per shot runs every step of a phase in one launch (prop_cluster.cuh;
// launch_cluster_forward / launch_cluster_adjoint below).
#include <mutex>

#include "prop_boundary.cuh"
#include "prop_cluster.cuh"
#include "prop_layer.cuh"
#include "prop_rebuild.cuh"

namespace fwi {

// native.cu fills a host copy of TmaMaps with the same members in the same order
static_assert(sizeof(TmaMaps) == 26 * sizeof(CUtensorMap), "TmaMaps layout");

namespace {

template <typename K> cudaError_t allow_smem(K kernel, size_t bytes)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Tiles from the grid origin (b.xbase, b.zbase) to the window's far edges.
inline dim3 tma_grid(const Batch<float> &b, int nx_max, int sg)
{
    return dim3((nx_max - b.xbase + TT - 1) / TT, (b.nz - b.zbase + TT - 1) / TT, (b.B + sg - 1) / sg);
}

// Blocks of one tile pass: one per tile of its compact list and shot group, or the full grid.
inline dim3 pass_grid(const Batch<float> &b, int nx_max, int sg, int list)
{
    if (b.tiles[list]) return dim3(b.ntiles[list], 1, (b.B + sg - 1) / sg);
    return tma_grid(b, nx_max, sg);
}

template <int ST> void fwd_interior(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, cudaStream_t st)
{
    const size_t sm = fwd_tma_smem(b.sg);
    const TmaMaps &m = *static_cast<const TmaMaps *>(b.tma);
    if (b.mixed)
        k_fwd_tma<ST, true><<<tma_grid(b, nx_max, b.sg), kTmaThreads, sm, st>>>(b, m, g, ntb, cur, slot, b.sg);
    else
        k_fwd_tma<ST, false><<<pass_grid(b, nx_max, b.sg, kTilesFwdInterior), kTmaThreads, sm, st>>>(b, m, g, ntb,
                                                                                                   cur, slot, b.sg);
}

template <int ST, bool EXACT, bool INLINE>
void fwd_layer(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, cudaStream_t st)
{
    const size_t sm = fwd_layer_smem();
    k_fwd_layer<ST, EXACT, INLINE><<<pass_grid(b, nx_max, b.sg_layer, kTilesFwdLayer), kTmaThreads, sm, st>>>(
        b, *static_cast<const TmaMaps *>(b.tma), g, ntb, cur, slot, b.sg_layer);
}

template <int ST, bool EXACT>
void adj_interior(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, int base, cudaStream_t st)
{
    const size_t sm = adj_tma_smem();
    const TmaMaps &m = *static_cast<const TmaMaps *>(b.tma);
    if (b.mixed)
        k_adj_tma<ST, EXACT, true><<<tma_grid(b, nx_max, b.sg), kTmaThreads, sm, st>>>(b, m, j, ntb, cur, zsel, base,
                                                                                       b.sg);
    else
        k_adj_tma<ST, EXACT, false><<<pass_grid(b, nx_max, b.sg, kTilesAdjInterior), kTmaThreads, sm, st>>>(
            b, m, j, ntb, cur, zsel, base, b.sg);
}

template <int ST, bool EXACT, bool INLINE>
void adj_layer(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, int base, cudaStream_t st)
{
    const size_t sm = adj_layer_smem();
    k_adj_layer<ST, EXACT, INLINE><<<pass_grid(b, nx_max, b.sg_layer, kTilesAdjLayer), kTmaThreads, sm, st>>>(
        b, *static_cast<const TmaMaps *>(b.tma), j, ntb, cur, zsel, base, b.sg_layer);
}

// `side_work` on ss.side (after everything issued to ss.main so far),
// `main_work` on ss.main, which then waits for the side.  Without a side
// stream: both in that order on ss.main.
template <typename Side, typename Main> void fork_join(const StepStreams &ss, Side side_work, Main main_work)
{
    if (!ss.side) {
        side_work(ss.main);
        main_work(ss.main);
        return;
    }
    cudaEventRecord(ss.fork, ss.main);
    cudaStreamWaitEvent(ss.side, ss.fork, 0);
    side_work(ss.side);
    cudaEventRecord(ss.join, ss.side);
    // timing events: external event nodes when the step is captured into a graph
    unsigned rec_flags = cudaEventRecordDefault;
    if (ss.t0) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(ss.main, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
            rec_flags = cudaEventRecordExternal;
        cudaEventRecordWithFlags(ss.t0, ss.main, rec_flags);
    }
    main_work(ss.main);
    if (ss.t1) cudaEventRecordWithFlags(ss.t1, ss.main, rec_flags);
    cudaStreamWaitEvent(ss.main, ss.join, 0);
}

template <int ST>
void forward_step(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int slot, bool exact,
                  const StepStreams &ss)
{
    fork_join(
        ss,
        [&](cudaStream_t s) {
            if (b.inline_strip) {
                if (exact) fwd_layer<ST, true, true>(b, nx_max, g, ntb, cur, slot, s);
                else fwd_layer<ST, false, true>(b, nx_max, g, ntb, cur, slot, s);
                return;
            }
            k_fwd_strip<float><<<strip_grid(b, nx_max), kStripBlock, 0, s>>>(b, g, ntb, cur);
            if (exact) fwd_layer<ST, true, false>(b, nx_max, g, ntb, cur, slot, s);
            else fwd_layer<ST, false, false>(b, nx_max, g, ntb, cur, slot, s);
        },
        [&](cudaStream_t s) { fwd_interior<ST>(b, nx_max, g, ntb, cur, slot, s); });
}

template <int ST>
void adjoint_step(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact, int base,
                  const StepStreams &ss)
{
    fork_join(
        ss,
        [&](cudaStream_t s) {
            if (b.inline_strip) {
                if (exact) adj_layer<ST, true, true>(b, nx_max, j, ntb, cur, zsel, base, s);
                else adj_layer<ST, false, true>(b, nx_max, j, ntb, cur, zsel, base, s);
                return;
            }
            if (exact) {
                k_adj_strip_exact<float><<<strip_grid(b, nx_max), kStripBlock, 0, s>>>(b, j, cur, zsel);
                adj_layer<ST, true, false>(b, nx_max, j, ntb, cur, zsel, base, s);
            } else {
                k_adj_strip_ref<float><<<strip_grid(b, nx_max), kStripBlock, 0, s>>>(b, j, cur);
                adj_layer<ST, false, false>(b, nx_max, j, ntb, cur, zsel, base, s);
            }
        },
        [&](cudaStream_t s) {
            if (exact) adj_interior<ST, true>(b, nx_max, j, ntb, cur, zsel, base, s);
            else adj_interior<ST, false>(b, nx_max, j, ntb, cur, zsel, base, s);
        });
}

template <int ST> cudaError_t allow_all()
{
    cudaError_t e = cudaSuccess;
    auto keep = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
    keep(allow_smem(k_fwd_tma<ST, false>, fwd_tma_smem(kMaxGroup)));
    keep(allow_smem(k_fwd_tma<ST, true>, fwd_tma_smem(kMaxGroup)));
    keep(allow_smem(k_fwd_layer<ST, true, true>, fwd_layer_smem()));
    keep(allow_smem(k_fwd_layer<ST, true, false>, fwd_layer_smem()));
    keep(allow_smem(k_fwd_layer<ST, false, true>, fwd_layer_smem()));
    keep(allow_smem(k_fwd_layer<ST, false, false>, fwd_layer_smem()));
    keep(allow_smem(k_adj_tma<ST, true, false>, adj_tma_smem()));
    keep(allow_smem(k_adj_tma<ST, false, false>, adj_tma_smem()));
    keep(allow_smem(k_adj_tma<ST, true, true>, adj_tma_smem()));
    keep(allow_smem(k_adj_tma<ST, false, true>, adj_tma_smem()));
    keep(allow_smem(k_adj_layer<ST, true, true>, adj_layer_smem()));
    keep(allow_smem(k_adj_layer<ST, true, false>, adj_layer_smem()));
    keep(allow_smem(k_adj_layer<ST, false, true>, adj_layer_smem()));
    keep(allow_smem(k_adj_layer<ST, false, false>, adj_layer_smem()));
    keep(allow_smem(k_rebuild_tma<ST>, rebuild_tma_smem()));
    return e;
}

}  // namespace

// Dynamic shared memory above 48 KB for every FP32 tile kernel: a function
// attribute of the current device's context, set once per device.
cudaError_t prepare_fp32_kernels()
{
    static std::mutex mu;
    static bool done[256] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 256 && done[dev]) return cudaSuccess;
    for (cudaError_t r : {allow_all<kStoreNative>(), allow_all<kStoreHalf>(), allow_all<kStoreBf16>()})
        if (r != cudaSuccess) return r;
    if (dev >= 0 && dev < 256) done[dev] = true;
    return cudaSuccess;
}

template <>
void launch_forward_step<float>(const Batch<float> &b, int nx_max, int g, int ntb, int cur, int img_slot,
                                bool exact, const StepStreams &ss)
{
    switch (b.store_type) {
    case kStoreHalf: forward_step<kStoreHalf>(b, nx_max, g, ntb, cur, img_slot, exact, ss); break;
    case kStoreBf16: forward_step<kStoreBf16>(b, nx_max, g, ntb, cur, img_slot, exact, ss); break;
    default: forward_step<kStoreNative>(b, nx_max, g, ntb, cur, img_slot, exact, ss); break;
    }
}

template <>
void launch_adjoint_step<float>(const Batch<float> &b, int nx_max, int j, int ntb, int cur, int zsel, bool exact,
                                int img_base, const StepStreams &ss)
{
    switch (b.store_type) {
    case kStoreHalf: adjoint_step<kStoreHalf>(b, nx_max, j, ntb, cur, zsel, exact, img_base, ss); break;
    case kStoreBf16: adjoint_step<kStoreBf16>(b, nx_max, j, ntb, cur, zsel, exact, img_base, ss); break;
    default: adjoint_step<kStoreNative>(b, nx_max, j, ntb, cur, zsel, exact, img_base, ss); break;
    }
}

long boundary_ring_len(int nx_max, int nz, int cpml) { return Ring::make(nx_max, nz, cpml).count(); }

// ------------------------------------------------------------------ small shots on one cluster

namespace {

template <typename K> cudaError_t cluster_attrs(K kernel, size_t smem)
{
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

// One cluster of ncta CTAs per shot; `args` are the kernel's own.
template <typename... Args>
cudaError_t cluster_launch(void (*kernel)(Args...), int ncta, int nshots, size_t smem, cudaStream_t st,
                           Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(ncta * nshots);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = ncta;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

size_t cluster_smem_limit()
{
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (size_t)v - 1024;  // the kernels' static shared memory
}

int store_elem_bytes(int store_type) { return store_type == kStoreNative ? (int)sizeof(float) : 2; }

// The cluster plan of a window width, grid height, layer width and image type, made once (the
// partition is a small dynamic programme) and kept for the process.
bool cached_cluster_plan(int nx, int nz, int cpml, int store_type, ClusterPlan &p)
{
    struct Entry {
        int nx, nz, cpml, st;
        bool ok;
        ClusterPlan p;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    std::lock_guard<std::mutex> lock(mu);
    for (const Entry &e : cache)
        if (e.nx == nx && e.nz == nz && e.cpml == cpml && e.st == store_type) {
            p = e.p;
            return e.ok;
        }
    Entry e{nx, nz, cpml, store_type, false, {}};
    e.ok = cluster_plan(nx, nz, cpml, store_elem_bytes(store_type), cluster_smem_limit(), e.p);
    cache.push_back(e);
    p = e.p;
    return e.ok;
}

}  // namespace

bool cluster_shot_fits(int nx_max, int nz, int cpml, int store_type)
{
    ClusterPlan p;
    if (!cached_cluster_plan(nx_max, nz, cpml, store_type, p)) return false;
    // every kernel may take the device's whole opt-in shared memory: one setting serves all widths
    const size_t lim = cluster_smem_limit();
    for (cudaError_t e : {cluster_attrs(k_cluster_fwd<kStoreNative>, lim),
                          cluster_attrs(k_cluster_fwd<kStoreHalf>, lim),
                          cluster_attrs(k_cluster_fwd<kStoreBf16>, lim),
                          cluster_attrs(k_cluster_adj<kStoreNative>, lim),
                          cluster_attrs(k_cluster_adj<kStoreHalf>, lim),
                          cluster_attrs(k_cluster_adj<kStoreBf16>, lim)})
        if (e != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
    // clusters of p.ncta CTAs with this much shared memory each must fit on the device
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(p.ncta);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = p.smem_adj;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = p.ncta;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_cluster_adj<kStoreHalf>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n > 0;
}

cudaError_t launch_cluster_forward(const Batch<float> &b, int nx_max, int ntb, bool images, cudaStream_t st)
{
    ClusterPlan p;
    if (!cached_cluster_plan(nx_max, b.nz, b.cpml, b.store_type, p)) return cudaErrorInvalidValue;
    const int img = images ? 1 : 0, n = p.ncta;
    const size_t sm = p.smem_fwd;
    const int h = p.h, pt = p.pitch;
    switch (b.store_type) {
    case kStoreHalf: return cluster_launch(k_cluster_fwd<kStoreHalf>, n, b.B, sm, st, b, p.rows, ntb, h, pt, img);
    case kStoreBf16: return cluster_launch(k_cluster_fwd<kStoreBf16>, n, b.B, sm, st, b, p.rows, ntb, h, pt, img);
    default: return cluster_launch(k_cluster_fwd<kStoreNative>, n, b.B, sm, st, b, p.rows, ntb, h, pt, img);
    }
}

cudaError_t launch_cluster_adjoint(const Batch<float> &b, int nx_max, int ntb, cudaStream_t st)
{
    ClusterPlan p;
    if (!cached_cluster_plan(nx_max, b.nz, b.cpml, b.store_type, p)) return cudaErrorInvalidValue;
    const int n = p.ncta, ab = p.abuf;
    const size_t sm = p.smem_adj;
    switch (b.store_type) {
    case kStoreHalf: return cluster_launch(k_cluster_adj<kStoreHalf>, n, b.B, sm, st, b, p.rows, ntb, p.h, p.pitch, ab);
    case kStoreBf16: return cluster_launch(k_cluster_adj<kStoreBf16>, n, b.B, sm, st, b, p.rows, ntb, p.h, p.pitch, ab);
    default: return cluster_launch(k_cluster_adj<kStoreNative>, n, b.B, sm, st, b, p.rows, ntb, p.h, p.pitch, ab);
    }
}

template void launch_save_ring<float>(const Batch<float> &, int, int, int, int, float *, long, cudaStream_t);
template void launch_rebuild_begin<float>(const Batch<float> &, int, int, int, int, const float *, long,
                                          cudaStream_t);
// The tiled rebuild (prop_rebuild.cuh): one launch per step, the next level's ring included.
template <>
void launch_rebuild_step<float>(const Batch<float> &rb, int nx_max, int g, int ntb, int cur, const float *ring,
                                long ring_len, int img_slot, cudaStream_t st)
{
    const int sg = rb.mixed ? 1 : rb.sg;  // a group of the rebuild shares one window
    const dim3 grid = tma_grid(rb, nx_max, sg);
    const size_t sm = rebuild_tma_smem();
    const TmaMaps &m = *static_cast<const TmaMaps *>(rb.tma);
    switch (rb.store_type) {
    case kStoreHalf: k_rebuild_tma<kStoreHalf><<<grid, kTmaThreads, sm, st>>>(rb, m, g, ntb, cur, ring, ring_len, sg, img_slot); break;
    case kStoreBf16: k_rebuild_tma<kStoreBf16><<<grid, kTmaThreads, sm, st>>>(rb, m, g, ntb, cur, ring, ring_len, sg, img_slot); break;
    default: k_rebuild_tma<kStoreNative><<<grid, kTmaThreads, sm, st>>>(rb, m, g, ntb, cur, ring, ring_len, sg, img_slot); break;
    }
}

}  // namespace fwi
