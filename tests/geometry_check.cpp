// Brute-force check of the tile geometry the FP32 tile passes rely on
// (fwi_gb300/csrc/prop.h, common.cuh), on the host: built and run by
// tests/test_geometry_cpu.py.  Prints "OK <cases>" or the first failure.
//
//  1. tile_grid: origin in (-32, 0], x origin a multiple of 4 (TMA: every x
//     coordinate x0 - 4 a multiple of 16 bytes); with inline_strip, each CPML
//     band with the 4 points beside it in one tile column (sides) or row
//     (bottom).
//  2. tile_role against the points of the tile: 0 no interior point, 2 some
//     interior point the layers of width aw touch, else 1.
//  3. What the interior passes assume of an interior tile (role 1), also for
//     groups of several windows: every column of the tile is an interior
//     column (its mask depends on the row only), and the tile with its 4-point
//     halo lies inside the window (columns) and above the last row.
//  4. The boundary ring's index of a point inverts its enumeration.
#include "common.cuh"
#include "prop.h"

#include <cstdio>

using namespace fwi;

static bool same_col(int a, int b, int base) { return floor_div(a - base, kTileEdge) == floor_div(b - base, kTileEdge); }

static int check(int nx, int nz, int cpml)
{
    const TileGrid tg = tile_grid(nx, nz, cpml);
    if (tg.xbase % 4 != 0 || tg.xbase > 0 || tg.xbase <= -kTileEdge || tg.zbase > 0 || tg.zbase <= -kTileEdge) {
        printf("FAIL origin nx=%d nz=%d cpml=%d: %d %d\n", nx, nz, cpml, tg.xbase, tg.zbase);
        return 1;
    }
    if (tg.inline_strip) {
        const int w = cpml + 4;
        if (!same_col(4, w - 1, tg.xbase) || !same_col(nx - w, nx - 5, tg.xbase) ||
            !same_col(nz - w, nz - 5, tg.zbase)) {
            printf("FAIL bands nx=%d nz=%d cpml=%d\n", nx, nz, cpml);
            return 1;
        }
    }
    const int bases[2][2] = {{tg.xbase, tg.zbase}, {0, 0}};
    for (const auto &bz : bases)
        for (int aw : {cpml, cpml + kRad})
            for (int z0 = bz[1]; z0 < nz; z0 += kTileEdge)
                for (int x0 = bz[0]; x0 < nx; x0 += kTileEdge) {
                    bool has_int = false, has_layer = false, rows_only = true;
                    for (int iz = z0; iz < z0 + kTileEdge; iz++)
                        for (int ix = x0; ix < x0 + kTileEdge; ix++) {
                            if (ix < 0 || iz < 0 || ix >= nx || iz >= nz) continue;
                            const bool in = interior(ix, iz, nx, nz);
                            has_int |= in;
                            has_layer |= in && layer_point(ix, iz, nx, nz, aw);
                            rows_only &= in == (iz > 3 && iz < nz - 4);
                        }
                    const int want = !has_int ? 0 : has_layer ? 2 : 1;
                    const int role = tile_role(x0, z0, nx, nz, aw);
                    if (role != want) {
                        printf("FAIL role nx=%d nz=%d aw=%d tile (%d, %d): %d, points say %d\n", nx, nz, aw, x0, z0,
                               role, want);
                        return 1;
                    }
                    if (role == 1 && (!rows_only || x0 - kRad < 0 || x0 + kTileEdge + kRad > nx ||
                                      z0 + kTileEdge + kRad > nz)) {
                        printf("FAIL interior tile nx=%d nz=%d aw=%d tile (%d, %d)\n", nx, nz, aw, x0, z0);
                        return 1;
                    }
                }
    return 0;
}

// The boundary ring (FWI_STORE_BOUNDARY): index() inverts point() over the
// whole ring and gives -1 for every other point of the window.
static int check_ring(int nx, int nz, int cpml)
{
    const Ring R = Ring::make(nx, nz, cpml);
    for (long k = 0; k < R.count(); k++) {
        int ix, iz;
        bool f, f2;
        R.point(k, ix, iz, f);
        if (R.index(ix, iz, f2) != k || f2 != f) {
            printf("FAIL ring nx=%d nz=%d cpml=%d k=%ld\n", nx, nz, cpml, k);
            return 1;
        }
    }
    long n = 0;
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            bool f;
            const bool onP = iz >= 4 && iz < nz - cpml &&
                             ((ix >= cpml - 4 && ix < cpml) || (ix >= nx - cpml && ix < nx - cpml + 4));
            const bool onF = iz >= nz - cpml && iz < nz - cpml + 4 && ix >= cpml && ix < nx - cpml;
            const long k = R.index(ix, iz, f);
            if ((k >= 0) != (onP || onF) || (k >= 0 && f != onF)) {
                printf("FAIL ring point nx=%d nz=%d cpml=%d (%d, %d)\n", nx, nz, cpml, ix, iz);
                return 1;
            }
            n += k >= 0;
        }
    if (n != R.count()) {
        printf("FAIL ring count nx=%d nz=%d cpml=%d\n", nx, nz, cpml);
        return 1;
    }
    return 0;
}

int main()
{
    long cases = 0;
    const int nzs[] = {41, 57, 88, 129, 309, 809};
    for (int cpml : {5, 8, 12, 20, 28})
        for (int nz : nzs) {
            if (nz < cpml + 9) continue;
            for (int nx = 2 * cpml + 9; nx < 420; nx += 7) {
                if (check(nx, nz, cpml)) return 1;
                cases++;
            }
            for (int nx : {609, 1049, 1649, 2009}) {
                if (check(nx, nz, cpml)) return 1;
                cases++;
            }
        }
    for (int nx : {4009, 1611, 437}) {  // C4-sized grid and windows
        if (check(nx, 1209, 20)) return 1;
        cases++;
    }
    for (int cpml : {8, 12, 20})
        for (int nx : {2 * cpml + 9, 72, 137, 609})
            for (int nz : {cpml + 9, 56, 309}) {
                if (check_ring(nx, nz, cpml)) return 1;
                cases++;
            }
    printf("OK %ld\n", cases);
    return 0;
}
