// CPU check of the small-shot cluster path's plan (fwi_gb300/csrc/cluster_plan.h): over a sweep
// of window widths, grid heights, layer widths and image types, every plan the path accepts
// covers the interior rows exactly with CTAs of at least 8 rows (a halo comes from one
// neighbour), fits the shared-memory limit, keeps the 16-byte alignments the kernels rely on,
// and has the least largest-CTA cost (against brute force on small grids); every plan it
// refuses is one that cannot fit.  Prints "OK <plans checked>" or the first failure.
#include <cstdio>
#include <functional>

#include "cluster_plan.h"

using namespace fwi;

static const size_t kLimit = 232448 - 1024;  // the opt-in shared memory of an sm_103 CTA, less the static part

static int fail(const char *what, int nx, int nz, int cpml, int elem)
{
    std::printf("FAIL %s: nx %d nz %d cpml %d elem %d\n", what, nx, nz, cpml, elem);
    return 1;
}

// least largest-CTA cost over every split of nzi rows into ncta chunks of [lo, hcap] rows
static double brute(int nzi, int ncta, int lo, int hcap, int nx, int nz, int cpml)
{
    double best = 1e300;
    std::vector<int> len(ncta);
    std::function<void(int, int, double)> rec = [&](int k, int used, double worst) {
        if (worst >= best) return;
        if (k == ncta) {
            if (used == nzi) best = worst;
            return;
        }
        for (int n = lo; n <= hcap && used + n <= nzi; n++)
            rec(k + 1, used + n, std::max(worst, cluster_row_cost(used, n, nx, nz, cpml)));
    };
    rec(0, 0, 0.0);
    return best;
}

int main()
{
    long checked = 0;
    for (int elem : {2, 4})
        for (int cpml : {0, 4, 8, 12, 20, 30})
            for (int nx = 9; nx <= 420; nx += 29)
                for (int nz = 12; nz <= 620; nz += 19) {
                    ClusterPlan p;
                    const bool ok = cluster_plan(nx, nz, cpml, elem, kLimit, p);
                    const int nzi = nz - 8;
                    const int ip = cluster_img_pitch(nx, elem);
                    if (!ok) {
                        // refused: too few rows, or no split fits the shared memory
                        if (nzi < kClHalo) continue;
                        const int ncta = std::min(kClusterMaxCtas, nzi / kClHalo);
                        const int hmin = (nzi + ncta - 1) / ncta;
                        const int pitch = (nx + 3) / 4 * 4;
                        const size_t fwd = sizeof(float) * cluster_floats(hmin, pitch, kClFwdHaloed, kClFwdOwn, 1) +
                                           (size_t)2 * hmin * ip * elem;
                        const size_t adj = sizeof(float) * cluster_floats(hmin, pitch, kClAdjHaloed, kClAdjOwn, 0) +
                                           (size_t)2 * hmin * ip * elem;
                        if (fwd <= kLimit && adj <= kLimit) return fail("refused a plan that fits", nx, nz, cpml, elem);
                        continue;
                    }
                    checked++;
                    if (p.ncta != std::min(kClusterMaxCtas, nzi / kClHalo)) return fail("CTA count", nx, nz, cpml, elem);
                    if (p.rows.start[0] != 0 || p.rows.start[p.ncta] != nzi) return fail("rows not covered", nx, nz, cpml, elem);
                    int h = 0;
                    for (int k = 0; k < p.ncta; k++) {
                        const int n = p.rows.start[k + 1] - p.rows.start[k];
                        if (n < (p.ncta > 1 ? kClHalo : 1)) return fail("CTA below 8 rows", nx, nz, cpml, elem);
                        h = std::max(h, n);
                    }
                    if (h != p.h || h > p.hcap) return fail("largest CTA", nx, nz, cpml, elem);
                    if (p.smem_fwd > kLimit || p.smem_adj > kLimit) return fail("shared memory", nx, nz, cpml, elem);
                    if (p.abuf != 1 && p.abuf != 2) return fail("image buffers", nx, nz, cpml, elem);
                    const size_t adj1 = sizeof(float) * cluster_floats(p.h, p.pitch, kClAdjHaloed, kClAdjOwn, 0);
                    if (p.smem_adj != adj1 + (size_t)p.abuf * 2 * p.h * ip * elem) return fail("adjoint bytes", nx, nz, cpml, elem);
                    if (p.abuf == 1 && adj1 + (size_t)4 * p.h * ip * elem <= kLimit)
                        return fail("one image buffer where two fit", nx, nz, cpml, elem);
                    // the 4-column groups read x windows [ix - 4, ix + 8) up to the last group's end
                    const int nq = (nx - 8 + 3) / 4;
                    if (p.pitch % 4 || p.pitch < 4 * nq + 8 || p.pitch < nx) return fail("row pitch", nx, nz, cpml, elem);
                    if ((ip * elem) % 16 || ip < nx) return fail("image row pitch", nx, nz, cpml, elem);
                    if (cluster_floats(p.h, p.pitch, kClFwdHaloed, kClFwdOwn, 1) % 4) return fail("staging alignment", nx, nz, cpml, elem);
                    // least cost, against brute force where that is cheap
                    if (nzi <= 48 && p.ncta <= 5) {
                        const double want = brute(nzi, p.ncta, p.ncta > 1 ? kClHalo : nzi, p.hcap, nx, nz, cpml);
                        double got = 0;
                        for (int k = 0; k < p.ncta; k++)
                            got = std::max(got, cluster_row_cost(p.rows.start[k], p.rows.start[k + 1] - p.rows.start[k],
                                                                 nx, nz, cpml));
                        if (got > want + 1e-9) return fail("partition not the least cost", nx, nz, cpml, elem);
                    }
                }
    std::printf("OK %ld\n", checked);
    return 0;
}
