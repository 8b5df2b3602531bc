// Internal interface between the native context (native.cu) and the batched
// propagation kernels (prop.cuh, instantiated in prop_f32.cu / prop_f64.cu).
#pragma once

#include <cuda_runtime.h>

namespace fwi {

// One shot of a batch, in the shot's own window coordinates.
struct DevShot {
    int x0;        // first model column of the window
    int nx;        // window width (the shot's grid nx)
    int sx, sz;    // source point
    int rz, rx0, rx1;  // receiver row and columns [rx0, rx1)
    int nt;        // time steps
    long rec_off;  // offset of this shot's [nt][nrec] record / residual / observed block
};

enum StoreType { kStoreNative = 0, kStoreHalf = 1, kStoreBf16 = 2 };

// Device buffers of one batch of up to B shots.  Per-shot arrays are
// [B][nz][pitch] (slot = nz * pitch elements per shot).
template <typename T> struct Batch {
    int B, nz, pitch, mpitch, cpml, nt_max;
    long slot;
    T *lvl[6];      // P level 0, P level 1, F level 0, F level 1, P increment, F increment
    T *cp[8];       // CPML memory variables (forward uses 0..3)
    T *g[3];        // per-shot gradient accumulators: v_hor, v_po, v_nmo
    void *store;    // images: [B][n_img][2][slot] of the store type
    int store_type; // StoreType
    int n_img;      // image slots per shot
    float *scale;   // [B][nt_max] encode scale of each stored image step
    float *amax;    // [B][nt_max + 1] max |P|, |F| after each step
    T *rec;         // records / residuals, at DevShot::rec_off
    const DevShot *shots;
    const T *mh, *mp, *mn;  // dt^2 v_hor, dt^2 v_po, dt^2 v_nmo, [nz][mpitch]
    const T *cpa, *cpb;     // CPML a, b by distance into the layer [cpml + 1]
    const T *wavelet;
    T inv_dh, inv_dh2;
    T img_scale;            // dt (reference imaging) or dt^2 (exact)
    unsigned *status;       // bit 0: stored image saturated, bit 1: a pipeline wait gave up
    int sg;                 // shots per group: shots [q sg, (q+1) sg) share a window, and
                            // g[k] + q * slot accumulates the imaging of group q
    int sg_layer;           // the same for the FP32 layer tiles (their points are disjoint
                            // from the other passes', so the slots do not collide)
    int xbase, zbase;       // FP32 tile grid origin (TileGrid)
    int mixed;              // FP32: the interior passes' groups hold several windows (their
                            // MIXED kernels); the layer passes then take one shot per block
    int inline_strip;       // FP32: the layer tiles advance the CPML memory variables
    const void *tma;        // host copy of the batch's TMA tensor maps (FP32 path), or null
    // Compact tile lists of the FP32 tile passes when every shot has one window: for each
    // pass (TileList), the tiles of its role, packed tx | tz << 16 on the grid from (xbase,
    // zbase); one block per listed tile and shot group.  Null: the full tile grid, whose
    // blocks on tiles of another role return at once (groups of several windows).
    const int *tiles[4];
    int ntiles[4];
};

// The tile lists of Batch::tiles.
enum TileList { kTilesFwdInterior = 0, kTilesFwdLayer = 1, kTilesAdjInterior = 2, kTilesAdjLayer = 3 };

// Shots of a batch run end-aligned on one global clock of `ntb` steps (the
// batch's longest shot): shot s does its local step it = g - (ntb - nt_s),
// so every shot's adjoint starts at the same global iteration and the image
// a given adjoint iteration needs sits at the same global step for all shots.

// Time stepping is in increment form: u^{n+1} = u^n + v, v = v + dt^2 (...),
// with u ping-ponged between two levels (neighbours of other blocks read the
// old level) and the increment v updated in place.  Algebraically the
// reference's leapfrog; in FP32 it keeps the low bits of each small update
// that 2 u^n - u^{n-1} + dt^2 (...) rounds away.

// Tiles of the FP32 tile passes: kTileEdge x kTileEdge points.
constexpr int kTileEdge = 32;

// Points the CPML layers touch.  `aw` is the CPML width (forward, reference
// adjoint) or CPML width + 4 (exact adjoint, whose transpose terms reach 4
// points further).  Same shape as the reference's strip predicate
// (src/parallelcalls.cu:55).
__host__ __device__ inline bool layer_point(int ix, int iz, int nx, int nz, int aw)
{
    return ix < aw || ix > nx - aw - 1 || iz > nz - aw - 1;
}

// Tile grid origin of a window: tiles start at (xbase + 32 i, zbase + 32 j),
// xbase, zbase in (-32, 0], xbase a multiple of 4 (TMA: the x coordinate of
// every load, x0 - 4, stays a multiple of 16 bytes).  With `inline_strip`
// the origin puts each CPML band together with the 4 points beside it (the
// points whose updates read the band's memory variables) inside one tile
// column (side bands) or row (bottom band); the layer tiles then advance
// the memory variables themselves.  When no origin does that, both are 0.
struct TileGrid {
    int xbase = 0, zbase = 0;
    bool inline_strip = false;
};

__host__ __device__ inline int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

inline TileGrid tile_grid(int nx, int nz, int cpml)
{
    TileGrid t;
    const int w = cpml + 4;  // band plus the points beside it
    if (cpml < 5 || w > kTileEdge || nx < 2 * w + 8 || nz < w + 8) return t;
    auto same_tile = [](int a, int b, int base) {
        return floor_div(a - base, kTileEdge) == floor_div(b - base, kTileEdge);
    };
    for (int xb = 0; xb > -kTileEdge; xb -= 4) {
        if (!same_tile(4, w - 1, xb) || !same_tile(nx - w, nx - 5, xb)) continue;
        for (int zb = 0; zb > -kTileEdge; zb--) {
            if (!same_tile(nz - w, nz - 5, zb)) continue;
            t.xbase = xb;
            t.zbase = zb;
            t.inline_strip = true;
            return t;
        }
    }
    return t;
}

// Role of the tile at (x0, z0) of an nx x nz window: 0 no interior point,
// 1 interior tile (no layer point), 2 layer tile.
__host__ __device__ inline int tile_role(int x0, int z0, int nx, int nz, int aw)
{
    // the tile's interior points: columns [xa, xb], rows [za, zb]
    const int xa = x0 > 4 ? x0 : 4, za = z0 > 4 ? z0 : 4;
    const int xb = x0 + kTileEdge - 1 < nx - 5 ? x0 + kTileEdge - 1 : nx - 5;
    const int zb = z0 + kTileEdge - 1 < nz - 5 ? z0 + kTileEdge - 1 : nz - 5;
    if (xa > xb || za > zb) return 0;  // the frame only (or beyond the window)
    return (xa < aw || xb > nx - aw - 1 || zb > nz - aw - 1) ? 2 : 1;
}

// Boundary storage (FWI_STORE_BOUNDARY, prop_boundary.cuh): the ring the
// forward saves around the CPML-free region of each window.
// Ring of an nx x nz window: P at columns [cpml-4, cpml) and [nx-cpml,
// nx-cpml+4) of rows [4, nz-cpml); F at rows [nz-cpml, nz-cpml+4) of
// columns [cpml, nx-cpml).  Enumerated P-left, P-right, then F-bottom, x fastest.
struct Ring {
    int nx, nz, cpml, h, w;  // h rows of R, w columns of R
    __host__ __device__ static Ring make(int nx, int nz, int cpml)
    {
        Ring r;
        r.nx = nx; r.nz = nz; r.cpml = cpml;
        r.h = nz - cpml - 4;
        r.w = nx - 2 * cpml;
        if (r.h < 0) r.h = 0;
        if (r.w < 0) r.w = 0;
        return r;
    }
    __host__ __device__ long count() const { return 8L * h + 4L * w; }
    // The inverse of point(): the ring index of (ix, iz) and whether it is an
    // F point, or -1 for a point off the ring.
    __host__ __device__ long index(int ix, int iz, bool &isF) const
    {
        isF = false;
        if (iz >= 4 && iz < nz - cpml) {
            if (ix >= cpml - 4 && ix < cpml) return (long)(iz - 4) * 4 + (ix - (cpml - 4));
            if (ix >= nx - cpml && ix < nx - cpml + 4) return 4L * h + (long)(iz - 4) * 4 + (ix - (nx - cpml));
            return -1;
        }
        if (iz >= nz - cpml && iz < nz - cpml + 4 && ix >= cpml && ix < nx - cpml) {
            isF = true;
            return 8L * h + (long)(iz - (nz - cpml)) * w + (ix - cpml);
        }
        return -1;
    }
    // point k: (ix, iz) and whether it belongs to F (else P)
    __host__ __device__ void point(long k, int &ix, int &iz, bool &isF) const
    {
        if (k < 8L * h) {
            const int side = (int)(k / (4L * h)), kk = (int)(k - side * 4L * h);
            iz = 4 + kk / 4;
            ix = (side == 0 ? cpml - 4 : nx - cpml) + kk % 4;
            isF = false;
            return;
        }
        k -= 8L * h;
        iz = nz - cpml + (int)(k / w);
        ix = cpml + (int)(k % w);
        isF = true;
    }
};

// Streams of a step.  The FP32 path runs the interior tiles on `main` and
// the strip pass (CPML memory variables) followed by the layer tiles on
// `side`, both from the current time level, and `main` joins `side` before
// the next step.  side == nullptr: everything on `main` (as the FP64 path
// does).
struct StepStreams {
    cudaStream_t main = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;  // if set: recorded on `main` around the interior tiles
};

// Forward global step g.  `cur` is the level holding each shot's current
// state; the new state goes to level 1 - cur.  With img_slot >= 0 the
// step's images go to that slot (G, H for exact imaging, Dxx P and Dzz F for
// the reference's).  Receiver traces are always recorded.
template <typename T>
void launch_forward_step(const Batch<T> &b, int nx_max, int g, int ntb, int cur, int img_slot,
                         bool exact, const StepStreams &ss);

// Adjoint iteration j: lambda^m, m = nt_s - j, of every shot with nt_s > j.
// `cur` holds lambda^{m+1}; lambda^m goes to level 1 - cur (increment form).  `zsel`
// selects the ping-pong half of the exact adjoint's Z state.  The image of
// global step ntb - 1 - lag - j (lag 0 exact, 1 reference) is read from slot
// (that step - img_base); img_base <= that step is the caller's contract.
template <typename T>
void launch_adjoint_step(const Batch<T> &b, int nx_max, int j, int ntb, int cur, int zsel,
                         bool exact, int img_base, const StepStreams &ss);

// Sets the FP32 tile kernels' dynamic shared-memory limit on the current
// device (once per device); call before their first launch there.
cudaError_t prepare_fp32_kernels();

// Small shots resident on chip (prop_cluster.cuh): one thread-block cluster per
// shot takes it through every step in one launch.  cluster_shot_fits: the
// window nx wide on an nz-row grid fits the cluster's shared memory and
// clusters of that size can run on the current device (FP32, exact adjoint,
// full image storage).  The launches cover every shot of the batch view.
bool cluster_shot_fits(int nx_max, int nz, int cpml, int store_type);
cudaError_t launch_cluster_forward(const Batch<float> &b, int nx_max, int ntb, bool images, cudaStream_t st);
cudaError_t launch_cluster_adjoint(const Batch<float> &b, int nx_max, int ntb, cudaStream_t st);

// Boundary storage (prop_boundary.cuh): ring length per shot, saving the
// ring of step g, and the backward rebuild of the CPML-free region.
long boundary_ring_len(int nx_max, int nz, int cpml);
template <typename T>
void launch_save_ring(const Batch<T> &b, int nx_max, int g, int ntb, int cur, T *ring, long ring_len,
                      cudaStream_t st);
template <typename T>
void launch_rebuild_begin(const Batch<T> &rb, int nx_max, int g, int ntb, int src, const T *ring, long ring_len,
                          cudaStream_t st);
template <typename T>
void launch_rebuild_step(const Batch<T> &rb, int nx_max, int g, int ntb, int cur, const T *ring, long ring_len,
                         int img_slot, cudaStream_t st);

}  // namespace fwi
