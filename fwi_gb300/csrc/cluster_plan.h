// The small-shot cluster path's plan (prop_cluster.cuh): how many CTAs, which interior rows
// each holds, and the shared memory each needs.  Host code (with the CUDA headers' qualifiers),
// so that the partition can be checked on the CPU.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <vector>

#include "common.cuh"

namespace fwi {

constexpr int kClusterMaxCtas = 16;
constexpr int kClusterThreads = 704;  // 4 columns a thread: one pass over 13 rows of a 209-wide window
constexpr int kClHalo = 2 * kRad;  // halo rows of the copied fields

// Interior rows of each CTA: CTA k owns interior rows [start[k], start[k + 1]) (global rows
// 4 + start[k] ...), at least kClHalo of them when the cluster has more than one CTA.
struct ClRows {
    int start[kClusterMaxCtas + 1];
};

// CTAs, their rows, the largest CTA's row count h and the shared-memory row pitch of a window nx
// wide on an nz-row grid with a cpml-wide layer, for images of elem bytes.  Shared arrays:
// "haloed" ones carry kClHalo rows above and below the own rows, "banded" ones kRad rows (the
// recomputed CPML fields), the rest only the own rows; the CPML coefficients sit in shared
// tables by column and by banded row.  Each step's images pass through a staging area of the
// own rows (rows of whole 16-byte chunks): the forward writes one and copies it out at the start
// of the next step, the adjoint prefetches into one or two (abuf; two when they fit).
struct ClusterPlan {
    int ncta = 0, h = 0, pitch = 0, abuf = 0;
    int hcap = 0;  // the most rows a CTA could take (shared memory; two image buffers where possible)
    size_t smem_fwd = 0, smem_adj = 0;
    ClRows rows{};
};

// forward: F0 F1 haloed; PSZ banded; P0 P1 PSX VP VF ZX ZZ MH MP MN own; the receiver row
// adjoint: UZ0 UZ1 haloed; YZ banded; LP LF WP WF UX0 UX1 ZX ZZ YX MH MP MN own
constexpr int kClFwdHaloed = 2, kClFwdOwn = 10;
constexpr int kClAdjHaloed = 2, kClAdjOwn = 12;

// floats of the arrays and tables (rounded to 16 bytes), then the image staging
__host__ __device__ inline size_t cluster_floats(int h, int pitch, int haloed, int own, int extra_rows)
{
    const size_t rows = (size_t)haloed * (h + 2 * kClHalo) + (h + 2 * kRad) + (size_t)own * h + extra_rows;
    return (rows * pitch + 2 * (size_t)pitch + 2 * (size_t)(h + 2 * kRad) + 3) / 4 * 4;
}
// elements of a staged image row: whole 16-byte chunks covering nx
__host__ __device__ inline int cluster_img_pitch(int nx, int elem) { return (nx * elem + 15) / 16 * 16 / elem; }

// Relative cost of one step of the CTA holding interior rows [a, a + n): passes of the main
// phase over groups of 4 columns (a row within 4 of the bottom layer costs half as much again:
// the CPML terms), plus the passes of the recomputed z-band rows and of the side-band columns.  A
// model of the measured phase times, used only to balance the partition.
inline double cluster_row_cost(int a, int n, int nx, int nz, int cpml)
{
    const double T = kClusterThreads;
    const int nxi = nx - 8, nq = (nxi + 3) / 4, zb = nz - cpml, g0 = 4 + a, g1 = 4 + a + n;
    const int heavy = std::max(0, g1 - std::max(g0, zb - 4));
    // passes (the slowest warp) and work (issue slots) weigh half each
    const double w = n * (double)nq / T, f = 1.0 + 0.5 * heavy / n;
    double c = 0.5 * std::ceil(w) * f + 0.5 * w * f;
    const int lo = std::max(std::max(4, zb), g0 - kRad), hi = std::min(nz - 4, g1 + kRad);
    if (hi > lo) c += 0.5 * std::ceil((hi - lo) * (double)nq / T);
    const int nbx = cpml > 4 ? std::min(2 * (cpml - 4), nxi) : 0;
    if (nbx > 0) c += 0.3 * std::ceil(n * (double)nbx / T);
    return c;
}

// Partition of nzi interior rows into ncta chunks of [lo, hcap] rows minimising the largest
// chunk cost (dynamic programme over chunk ends).  Returns that cost, or a negative value if
// no partition exists.
inline double cluster_partition(int nzi, int ncta, int lo, int hcap, int nx, int nz, int cpml, ClRows &out)
{
    const double inf = 1e300;
    std::vector<double> best((size_t)(ncta + 1) * (nzi + 1), inf);
    std::vector<int> from((size_t)(ncta + 1) * (nzi + 1), -1);
    best[0] = 0.0;
    for (int k = 1; k <= ncta; k++)
        for (int r = 1; r <= nzi; r++)
            for (int n = lo; n <= std::min(hcap, r); n++) {
                const double prev = best[(size_t)(k - 1) * (nzi + 1) + r - n];
                if (prev >= inf) continue;
                const double c = std::max(prev, cluster_row_cost(r - n, n, nx, nz, cpml));
                double &cur = best[(size_t)k * (nzi + 1) + r];
                if (c < cur - 1e-9) {
                    cur = c;
                    from[(size_t)k * (nzi + 1) + r] = r - n;
                }
            }
    const double c = best[(size_t)ncta * (nzi + 1) + nzi];
    if (c >= inf) return -1.0;
    int r = nzi;
    for (int k = ncta; k >= 1; k--) {
        out.start[k] = r;
        r = from[(size_t)k * (nzi + 1) + r];
    }
    out.start[0] = 0;
    for (int k = ncta + 1; k <= kClusterMaxCtas; k++) out.start[k] = nzi;
    return c;
}

inline bool cluster_plan(int nx, int nz, int cpml, int elem, size_t smem_limit, ClusterPlan &p)
{
    const int nzi = nz - 8;
    if (nzi < kClHalo || nx < 9) return false;
    // a halo comes from one neighbour only: every CTA holds at least 8 rows
    p.ncta = std::min(kClusterMaxCtas, nzi / kClHalo);
    p.pitch = (nx + 3) / 4 * 4;
    const int ip = cluster_img_pitch(nx, elem);
    auto fwd_bytes = [&](int h) {
        return sizeof(float) * cluster_floats(h, p.pitch, kClFwdHaloed, kClFwdOwn, 1) + (size_t)2 * h * ip * elem;
    };
    auto adj_bytes = [&](int h, int abuf) {
        return sizeof(float) * cluster_floats(h, p.pitch, kClAdjHaloed, kClAdjOwn, 0) +
               (size_t)abuf * 2 * h * ip * elem;
    };
    int hmax = 0;
    for (int h = kClHalo; h <= nzi && fwd_bytes(h) <= smem_limit && adj_bytes(h, 1) <= smem_limit; h++) hmax = h;
    if (hmax == 0 || (long)hmax * p.ncta < nzi) return false;
    // rows per CTA that leave room for two adjoint image buffers (the prefetch one step ahead),
    // if such a partition exists
    int hmax2 = 0;
    for (int h = kClHalo; h <= hmax && adj_bytes(h, 2) <= smem_limit; h++) hmax2 = h;
    if ((long)hmax2 * p.ncta >= nzi) hmax = hmax2;
    p.hcap = hmax;
    const int lo = p.ncta > 1 ? kClHalo : nzi;
    // the least cost, then the fewest rows per CTA (shared memory) that still reach it
    const double cbest = cluster_partition(nzi, p.ncta, lo, hmax, nx, nz, cpml, p.rows);
    if (cbest < 0) return false;
    // (the least cost cannot rise as the cap grows: a bisection over the cap)
    int lo_h = (nzi + p.ncta - 1) / p.ncta, hi_h = hmax;
    while (lo_h < hi_h) {
        const int mid = (lo_h + hi_h) / 2;
        ClRows r{};
        const double c = cluster_partition(nzi, p.ncta, lo, mid, nx, nz, cpml, r);
        if (c >= 0 && c <= cbest + 1e-9) hi_h = mid;
        else lo_h = mid + 1;
    }
    if (lo_h < hmax) cluster_partition(nzi, p.ncta, lo, lo_h, nx, nz, cpml, p.rows);
    p.h = 0;
    for (int k = 0; k < p.ncta; k++) p.h = std::max(p.h, p.rows.start[k + 1] - p.rows.start[k]);
    p.smem_fwd = fwd_bytes(p.h);
    p.abuf = adj_bytes(p.h, 2) <= smem_limit ? 2 : 1;
    p.smem_adj = adj_bytes(p.h, p.abuf);
    return p.smem_adj <= smem_limit && p.smem_fwd <= smem_limit;
}

}  // namespace fwi
