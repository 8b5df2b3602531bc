/*
 * Native-semantics oracle: forward step, EXACT discrete adjoint and imaging.
 * Included twice by vti_oracle.c with R = float / double.
 *
 * Forward step n (the reference's step, src/parallelcalls.cu:48-130, with a
 * free source/receiver geometry):
 *   on strip points s (interior and within the CPML layers):
 *     psx' = bx psx + ax Dx P,   psz' = bz psz + az Dz F
 *     zx'  = bx zx + ax (Dxx P + Dx psx'),  zz' = bz zz + az (Dzz F + Dz psz')
 *     Ap = Dx psx' + zx',  Af = Dz psz' + zz'      (zero off the strips)
 *   G = Dxx P + Ap,  H = Dzz F + Af
 *   P+ = 2P - P- + dt^2 (v_hor G + v_po H),  F+ = 2F - F- + dt^2 (v_nmo G + v_po H)
 *   P+[src] += w[n], F+[src] += w[n];  rec[n][r] = P+ + F+ at (rx0 + r, rz)
 *
 * EXACT adjoint (transpose of the step above, D^T = -D for the first
 * derivative, Dxx^T = Dxx), iteration j = 0..nt-1 computing lam^m, m = nt-j,
 * from lam^{m+1} (cur) and lam^{m+2} (old):
 *   g = dt^2 (v_hor lP + v_nmo lF),  h = dt^2 v_po (lP + lF)      (of lam^{m+1})
 *   Zx' = S (g + bx Zx),   Zz' = S (h + bz Zz)
 *   Yx' = S (-Dx[S (g + ax Zx')] + bx Yx),   Yz' likewise in z
 *   lP^m = 2 lP - lP_old + Dxx(g + S ax Zx') - Dx(S ax Yx')
 *   lF^m = 2 lF - lF_old + Dzz(h + S az Zz') - Dz(S az Yz')
 *   lam^m[rec] += mask * (rec[m-1] - obs[m-1])
 *   dJ/dv_hor += dt^2 G^{m-1} lP^m, dJ/dv_nmo += dt^2 G^{m-1} lF^m,
 *   dJ/dv_po  += dt^2 H^{m-1} (lP^m + lF^m)
 * with J = 1/2 sum mask (rec - obs)^2 accumulated in FP64.
 */

#define IDX(ix, iz) ((long)(ix) + (long)nx * (long)(iz))
#define INTERIOR(ix, iz) ((ix) > 3 && (ix) < nx - 4 && (iz) > 3 && (iz) < nz - 4)
#define STRIP(ix, iz) (INTERIOR(ix, iz) && ((ix) < cpml || (ix) > (nx - cpml - 1) || (iz) > (nz - cpml - 1)))

static inline R FN(x_d1)(const R *f, long i, long s, R inv_dh)
{
    return ((R)(4.0 / 5.0) * (f[i + s] - f[i - s]) - (R)(1.0 / 5.0) * (f[i + 2 * s] - f[i - 2 * s]) +
            (R)(4.0 / 105.0) * (f[i + 3 * s] - f[i - 3 * s]) -
            (R)(1.0 / 280.0) * (f[i + 4 * s] - f[i - 4 * s])) *
           inv_dh;
}

static inline R FN(x_d2)(const R *f, long i, long s, R inv_dh2)
{
    return ((R)(-205.0 / 72.0) * f[i] + (R)(8.0 / 5.0) * (f[i + s] + f[i - s]) -
            (R)(1.0 / 5.0) * (f[i + 2 * s] + f[i - 2 * s]) +
            (R)(8.0 / 315.0) * (f[i + 3 * s] + f[i - 3 * s]) -
            (R)(1.0 / 560.0) * (f[i + 4 * s] + f[i - 4 * s])) *
           inv_dh2;
}

/* Forward modelling of one shot; rec is [nt][rx1-rx0]; img_g/img_h (optional)
 * are [nt][nx*nz] and receive G^n and H^n (exact != 0) or Dxx P^n and Dzz F^n. */
void FN(orx_forward)(int nx, int nz, int nt, int cpml, R dh, R dt, const R *a_x, const R *b_x,
                     const R *a_z, const R *b_z, const R *v_hor, const R *v_po, const R *v_nmo,
                     int sx, int sz, const R *wavelet, int rz, int rx0, int rx1, R *rec, R *img_g,
                     R *img_h, int exact)
{
    long n = (long)nx * nz;
    int nrec = rx1 - rx0;
    R inv_dh = (R)1 / dh, inv_dh2 = (R)1 / (dh * dh), dt2 = dt * dt;
    R *P = (R *)calloc(n, sizeof(R)), *Pm = (R *)calloc(n, sizeof(R));
    R *F = (R *)calloc(n, sizeof(R)), *Fm = (R *)calloc(n, sizeof(R));
    R *psx = (R *)calloc(n, sizeof(R)), *psz = (R *)calloc(n, sizeof(R));
    R *zx = (R *)calloc(n, sizeof(R)), *zz = (R *)calloc(n, sizeof(R));
    R *G = (R *)calloc(n, sizeof(R)), *H = (R *)calloc(n, sizeof(R));
    R *G0 = (R *)calloc(n, sizeof(R)), *H0 = (R *)calloc(n, sizeof(R));
    for (int it = 0; it < nt; it++) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                if (!STRIP(ix, iz)) continue;
                long i = IDX(ix, iz);
                psx[i] = b_x[ix] * psx[i] + a_x[ix] * FN(x_d1)(P, i, 1, inv_dh);
                psz[i] = b_z[iz] * psz[i] + a_z[iz] * FN(x_d1)(F, i, nx, inv_dh);
            }
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                long i = IDX(ix, iz);
                if (!INTERIOR(ix, iz)) { G[i] = H[i] = 0; continue; }
                R p2 = FN(x_d2)(P, i, 1, inv_dh2), r2 = FN(x_d2)(F, i, nx, inv_dh2);
                R ap = 0, af = 0;
                if (STRIP(ix, iz)) {
                    R tx = FN(x_d1)(psx, i, 1, inv_dh), tz = FN(x_d1)(psz, i, nx, inv_dh);
                    zx[i] = b_x[ix] * zx[i] + a_x[ix] * (p2 + tx);
                    zz[i] = b_z[iz] * zz[i] + a_z[iz] * (r2 + tz);
                    ap = tx + zx[i];
                    af = tz + zz[i];
                }
                G0[i] = p2;
                H0[i] = r2;
                G[i] = p2 + ap;
                H[i] = r2 + af;
            }
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                if (!INTERIOR(ix, iz)) continue;
                long i = IDX(ix, iz);
                R pn = 2 * P[i] - Pm[i] + dt2 * (v_hor[i] * G[i] + v_po[i] * H[i]);
                R fn = 2 * F[i] - Fm[i] + dt2 * (v_nmo[i] * G[i] + v_po[i] * H[i]);
                Pm[i] = pn;
                Fm[i] = fn;
            }
        { long s = IDX(sx, sz); Pm[s] += wavelet[it]; Fm[s] += wavelet[it]; }
        for (int r = 0; r < nrec; r++) {
            long i = IDX(rx0 + r, rz);
            rec[(long)it * nrec + r] = Pm[i] + Fm[i];
        }
        if (img_g) memcpy(img_g + (long)it * n, exact ? G : G0, n * sizeof(R));
        if (img_h) memcpy(img_h + (long)it * n, exact ? H : H0, n * sizeof(R));
        R *t = P; P = Pm; Pm = t;
        t = F; F = Fm; Fm = t;
    }
    free(P); free(Pm); free(F); free(Fm); free(psx); free(psz); free(zx); free(zz);
    free(G); free(H); free(G0); free(H0);
}

/* Misfit and EXACT gradient of one shot.  obs is [nt][nrec] (ignored when
 * res_override, a [nt][nrec] adjoint source, is given: then the return value
 * is 0 and the adjoint of that source is computed).  mask (optional) is
 * [nrec].  adj_src_trace (optional, [nt]) receives lP^{n+1} + lF^{n+1} at the
 * source, i.e. the transpose of the wavelet-to-data map applied to the
 * adjoint source.  Gradients accumulate into g_vh/g_vp/g_vn. */
double FN(orx_gradient_shot)(int nx, int nz, int nt, int cpml, R dh, R dt, const R *a_x,
                             const R *b_x, const R *a_z, const R *b_z, const R *v_hor,
                             const R *v_po, const R *v_nmo, int sx, int sz, const R *wavelet,
                             int rz, int rx0, int rx1, const R *obs, const unsigned char *mask,
                             int mode, R *g_vh, R *g_vp, R *g_vn, R *adj_src_trace,
                             const R *res_override)
{
    if (mode != ORX_MODE_EXACT) return NAN;
    long n = (long)nx * nz;
    int nrec = rx1 - rx0;
    R inv_dh = (R)1 / dh, inv_dh2 = (R)1 / (dh * dh), dt2 = dt * dt;
    R *rec = (R *)calloc((long)nt * nrec, sizeof(R));
    R *img_g = (R *)malloc(sizeof(R) * n * (long)nt);
    R *img_h = (R *)malloc(sizeof(R) * n * (long)nt);
    FN(orx_forward)(nx, nz, nt, cpml, dh, dt, a_x, b_x, a_z, b_z, v_hor, v_po, v_nmo, sx, sz, wavelet,
                    rz, rx0, rx1, rec, img_g, img_h, 1);
    R *res = (R *)calloc((long)nt * nrec, sizeof(R));
    double J = 0;
    for (int it = 0; it < nt; it++)
        for (int r = 0; r < nrec; r++) {
            long k = (long)it * nrec + r;
            if (res_override) { res[k] = res_override[k]; continue; }
            R m = mask ? (R)(mask[r] != 0) : (R)1;
            R d = m * (rec[k] - obs[k]);
            res[k] = d;
            J += 0.5 * (double)d * (double)d;
        }

    R *lP = (R *)calloc(n, sizeof(R)), *lPo = (R *)calloc(n, sizeof(R));
    R *lF = (R *)calloc(n, sizeof(R)), *lFo = (R *)calloc(n, sizeof(R));
    R *Zx = (R *)calloc(n, sizeof(R)), *Zz = (R *)calloc(n, sizeof(R));
    R *Yx = (R *)calloc(n, sizeof(R)), *Yz = (R *)calloc(n, sizeof(R));
    R *g = (R *)calloc(n, sizeof(R)), *h = (R *)calloc(n, sizeof(R));
    R *wx = (R *)calloc(n, sizeof(R)), *wz = (R *)calloc(n, sizeof(R));
    R *ux = (R *)calloc(n, sizeof(R)), *uz = (R *)calloc(n, sizeof(R));
    R *vx = (R *)calloc(n, sizeof(R)), *vz = (R *)calloc(n, sizeof(R));
    for (int j = 0; j < nt; j++) {
        int m = nt - j;
        /* pointwise: g, h and the new Z; w = S(g + a Z'), u = g + S a Z' */
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                long i = IDX(ix, iz);
                if (!INTERIOR(ix, iz)) { g[i] = h[i] = wx[i] = wz[i] = ux[i] = uz[i] = 0; continue; }
                g[i] = dt2 * (v_hor[i] * lP[i] + v_nmo[i] * lF[i]);
                h[i] = dt2 * v_po[i] * (lP[i] + lF[i]);
                ux[i] = g[i];
                uz[i] = h[i];
                wx[i] = wz[i] = 0;
                if (STRIP(ix, iz)) {
                    Zx[i] = g[i] + b_x[ix] * Zx[i];
                    Zz[i] = h[i] + b_z[iz] * Zz[i];
                    wx[i] = g[i] + a_x[ix] * Zx[i];
                    wz[i] = h[i] + a_z[iz] * Zz[i];
                    ux[i] += a_x[ix] * Zx[i];
                    uz[i] += a_z[iz] * Zz[i];
                }
            }
        /* Y' = S(-D w + b Y), then v = S a Y' */
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                long i = IDX(ix, iz);
                vx[i] = vz[i] = 0;
                if (!STRIP(ix, iz)) continue;
                Yx[i] = -FN(x_d1)(wx, i, 1, inv_dh) + b_x[ix] * Yx[i];
                Yz[i] = -FN(x_d1)(wz, i, nx, inv_dh) + b_z[iz] * Yz[i];
                vx[i] = a_x[ix] * Yx[i];
                vz[i] = a_z[iz] * Yz[i];
            }
        /* leapfrog into the old level */
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                if (!INTERIOR(ix, iz)) continue;
                long i = IDX(ix, iz);
                R np = 2 * lP[i] - lPo[i] + FN(x_d2)(ux, i, 1, inv_dh2) - FN(x_d1)(vx, i, 1, inv_dh);
                R nf = 2 * lF[i] - lFo[i] + FN(x_d2)(uz, i, nx, inv_dh2) - FN(x_d1)(vz, i, nx, inv_dh);
                lPo[i] = np;
                lFo[i] = nf;
            }
        for (int r = 0; r < nrec; r++) {
            long i = IDX(rx0 + r, rz);
            R d = res[(long)(m - 1) * nrec + r];
            lPo[i] += d;
            lFo[i] += d;
        }
        if (adj_src_trace) { long s = IDX(sx, sz); adj_src_trace[m - 1] = lPo[s] + lFo[s]; }
        const R *Gm = img_g + (long)(m - 1) * n, *Hm = img_h + (long)(m - 1) * n;
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int iz = 0; iz < nz; iz++)
            for (int ix = 0; ix < nx; ix++) {
                if (!INTERIOR(ix, iz)) continue;
                long i = IDX(ix, iz);
                g_vh[i] += dt2 * Gm[i] * lPo[i];
                g_vn[i] += dt2 * Gm[i] * lFo[i];
                g_vp[i] += dt2 * Hm[i] * (lPo[i] + lFo[i]);
            }
        R *t = lP; lP = lPo; lPo = t;
        t = lF; lF = lFo; lFo = t;
    }
    free(lP); free(lPo); free(lF); free(lFo); free(Zx); free(Zz); free(Yx); free(Yz);
    free(g); free(h); free(wx); free(wz); free(ux); free(uz); free(vx); free(vz);
    free(rec); free(img_g); free(img_h); free(res);
    return J;
}

#undef IDX
#undef INTERIOR
#undef STRIP
