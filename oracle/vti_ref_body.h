/*
 * Reference-arithmetic restatement of danielvn/Fwi's kernels and host loops.
 * Included twice by vti_oracle.c: R = float / S = _f32 and R = double / S = _f64.
 *
 * Arithmetic rules kept from the reference (they decide the last bits):
 *  - stencil differences/sums of two neighbours are formed in R, then scaled
 *    by double-literal coefficients (4/5., 205/72., ...) in FP64, divided by
 *    dh or dh2 (R promoted), and the result is rounded to R on assignment
 *    (src/parallelcalls.cu:57, 127, 188, 207, 225, 252);
 *  - everything else (CPML recursions, leapfrog update, imaging, L-BFGS
 *    axpys) is plain R arithmetic in the reference's operand order;
 *  - host accumulations follow src/main.c (float sums, "/2.0" in double).
 * Build with -ffp-contract=off so that no multiply-add is fused.
 *
 * Every loop visits points in any order: each reference kernel writes only
 * its own point and never reads what the same kernel writes, so the serial
 * (or row-parallel) loops give the GPU kernels' results.
 */

#define IDX(ix, iz) ((long)(ix) + (long)nx * (long)(iz))
#define INTERIOR(ix, iz) ((ix) > 3 && (ix) < nx - 4 && (iz) > 3 && (iz) < nz - 4)
#define IN_STRIP(ix, iz) ((ix) < cpml || (ix) > (nx - cpml - 1) || (iz) > (nz - cpml - 1))

/* 8th-order first derivative along a stride (1 = x, nx = z); reference form. */
static inline double FN(ref_d1)(const R *f, long i, long s, R dh)
{
    return ((4 / 5.) * (f[i + s] - f[i - s]) - (1 / 5.) * (f[i + 2 * s] - f[i - 2 * s]) +
            (4 / 105.) * (f[i + 3 * s] - f[i - 3 * s]) -
            (1 / 280.) * (f[i + 4 * s] - f[i - 4 * s])) /
           dh;
}

/* 8th-order second derivative along a stride; reference form. */
static inline double FN(ref_d2)(const R *f, long i, long s, R dh2)
{
    return (-(205 / 72.) * f[i] + (8 / 5.) * (f[i + s] + f[i - s]) -
            (1 / 5.) * (f[i + 2 * s] + f[i - 2 * s]) +
            (8 / 315.) * (f[i + 3 * s] + f[i - 3 * s]) -
            (1 / 560.) * (f[i + 4 * s] + f[i - 4 * s])) /
           dh2;
}

/* src/parallelcalls.cu:3-16 */
void FN(orc_pre_variables)(const R *vel, const R *eps, const R *del, R *v_hor, R *v_po, R *v_nmo,
                           int nx, int nz)
{
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            long i = IDX(ix, iz);
            v_po[i] = vel[i] * vel[i];
            v_hor[i] = v_po[i] * (1 + 2 * eps[i]);
            v_nmo[i] = v_po[i] * (1 + 2 * del[i]);
        }
}

/* CPML damping profile at distance `dist` (in points) into the layer.
 * src/parallelcalls.cu:25-26 (left), 31-32 (right), 43-44 (bottom). */
static void FN(cpml_point)(R *a, R *b, int dist, R vmax, R dt, R dh, R f, R d0, R L)
{
    R frac = dist * dh / L;                                /* float in the reference */
    double d = d0 * vmax * pow(frac, 2);                   /* (d0*Vmax) in R, then FP64 */
    double alpha = PI_D * f * (L - dist * dh) / L;         /* FP64 */
    *b = (R)exp(-(d + alpha) * dt);
    *a = (R)(d0 * vmax * pow(frac, 2) * (*b - 1) / (d0 * vmax * pow(frac, 2) + alpha));
}

/* src/parallelcalls.cu:18-34 */
void FN(orc_cpml_x)(R *a_x, R *b_x, int cpml, R vmax, int nx, R dt, R dh, R f, R d0, R L)
{
    for (int ix = 0; ix < nx; ix++) {
        if (ix < cpml) FN(cpml_point)(&a_x[ix], &b_x[ix], cpml - ix, vmax, dt, dh, f, d0, L);
        if (ix > (nx - cpml - 1))
            FN(cpml_point)(&a_x[ix], &b_x[ix], ix - nx + cpml + 1, vmax, dt, dh, f, d0, L);
    }
}

/* src/parallelcalls.cu:36-46 (bottom layer only; the top is a free surface of zeros) */
void FN(orc_cpml_z)(R *a_z, R *b_z, int cpml, R vmax, int nz, R dt, R dh, R f, R d0, R L)
{
    for (int iz = 0; iz < nz; iz++)
        if (iz > (nz - cpml - 1))
            FN(cpml_point)(&a_z[iz], &b_z[iz], iz - nz + cpml + 1, vmax, dt, dh, f, d0, L);
}

/* src/parallelcalls.cu:48-63 */
void FN(orc_psi_f)(const R *P, const R *F, const R *a_x, const R *b_x, const R *a_z, const R *b_z,
                   R *psi_px, R *psi_fz, int nx, int nz, R dh, int cpml)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            if (!(INTERIOR(ix, iz) && IN_STRIP(ix, iz))) continue;
            long i = IDX(ix, iz);
            R tpx = (R)FN(ref_d1)(P, i, 1, dh);
            R tfz = (R)FN(ref_d1)(F, i, nx, dh);
            psi_px[i] = b_x[ix] * psi_px[i] + a_x[ix] * tpx;
            psi_fz[i] = b_z[iz] * psi_fz[i] + a_z[iz] * tfz;
        }
}

/* src/parallelcalls.cu:65-86 */
void FN(orc_zeta_f)(const R *p2, const R *r2, const R *a_x, const R *b_x, const R *a_z,
                    const R *b_z, const R *psi_px, const R *psi_fz, R *z_px, R *z_fz, R *aten_p,
                    R *aten_f, int nx, int nz, R dh, int cpml)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            if (!(INTERIOR(ix, iz) && IN_STRIP(ix, iz))) continue;
            long i = IDX(ix, iz);
            R tx = (R)FN(ref_d1)(psi_px, i, 1, dh);
            R tz = (R)FN(ref_d1)(psi_fz, i, nx, dh);
            R tpx = p2[i] + tx;
            R tfz = r2[i] + tz;
            z_px[i] = b_x[ix] * z_px[i] + a_x[ix] * tpx;
            z_fz[i] = b_z[iz] * z_fz[i] + a_z[iz] * tfz;
            aten_p[i] = tx + z_px[i];
            aten_f[i] = tz + z_fz[i];
        }
}

/* src/parallelcalls.cu:120-130 */
void FN(orc_second_derivate_p)(const R *P_pre, const R *F_pre, R *p2, R *r2, R dh2, int nx, int nz)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            if (!INTERIOR(ix, iz)) continue;
            long i = IDX(ix, iz);
            p2[i] = (R)FN(ref_d2)(P_pre, i, 1, dh2);
            r2[i] = (R)FN(ref_d2)(F_pre, i, nx, dh2);
        }
}

/* src/parallelcalls.cu:88-117.  The source and receiver branches belong to the
 * same thread as the update of that point, so they follow it. */
void FN(orc_propagator_f)(const R *p2, const R *r2, R *PF, const R *P_pre, const R *F_pre,
                          R *P_past, R *F_past, const R *v_hor, const R *v_po, const R *v_nmo,
                          const R *aten_p, const R *aten_f, const R *source, R *shot, R C, R dh2,
                          int nx, int nz, int sx, int sz, int it, int cpml)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            long i = IDX(ix, iz);
            if (INTERIOR(ix, iz)) {
                R tp = dh2 * (p2[i] + aten_p[i]);
                R tf = dh2 * (r2[i] + aten_f[i]);
                P_past[i] = 2 * P_pre[i] - P_past[i] + v_hor[i] * C * tp + v_po[i] * C * tf;
                F_past[i] = 2 * F_pre[i] - F_past[i] + v_nmo[i] * C * tp + v_po[i] * C * tf;
                PF[i] = P_past[i] + F_past[i];
            }
            if (ix == (sx - 1) && iz == (sz - 1)) {
                P_past[i] += source[it];
                F_past[i] += source[it];
            }
            if (ix > (cpml - 1) && ix < (nx - cpml) && iz == (sz - 1))
                shot[ix + (long)nx * it] = P_past[i] + F_past[i];
        }
}

/* src/parallelcalls.cu:133-142 (called with nt rows, src/main.c:437) */
void FN(orc_res)(R *Res, const R *shot1, const R *shot2, int nx, int nt)
{
    long n = (long)nx * nt;
    for (long i = 0; i < n; i++) Res[i] = shot2[i] - shot1[i];
}

/* src/parallelcalls.cu:166-177 */
void FN(orc_entry_point)(const R *P_pre, const R *F_pre, R *aux1, R *aux2, R *aux3, R *aux4,
                         const R *v_hor, const R *v_po, const R *v_nmo, int nx, int nz)
{
    long n = (long)nx * nz;
    for (long i = 0; i < n; i++) {
        aux1[i] = v_hor[i] * P_pre[i];
        aux2[i] = v_po[i] * P_pre[i];
        aux3[i] = v_nmo[i] * F_pre[i];
        aux4[i] = v_po[i] * F_pre[i];
    }
}

/* src/parallelcalls.cu:179-198 */
void FN(orc_psi_r)(const R *aux1, const R *aux2, const R *aux3, const R *aux4, const R *a_x,
                   const R *b_x, const R *a_z, const R *b_z, R *psixcx, R *psixcz, R *psizdx,
                   R *psizcz, int nx, int nz, R dh, int cpml)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            if (!(INTERIOR(ix, iz) && IN_STRIP(ix, iz))) continue;
            long i = IDX(ix, iz);
            R p1cx = (R)FN(ref_d1)(aux1, i, 1, dh);
            R p1cz = (R)FN(ref_d1)(aux2, i, nx, dh);
            R r1dx = (R)FN(ref_d1)(aux3, i, 1, dh);
            R r1cz = (R)FN(ref_d1)(aux4, i, nx, dh);
            psixcx[i] = b_x[ix] * psixcx[i] + a_x[ix] * p1cx;
            psixcz[i] = b_z[iz] * psixcz[i] + a_z[iz] * p1cz;
            psizdx[i] = b_x[ix] * psizdx[i] + a_x[ix] * r1dx;
            psizcz[i] = b_z[iz] * psizcz[i] + a_z[iz] * r1cz;
        }
}

/* src/parallelcalls.cu:200-214 */
void FN(orc_second_derivate)(const R *aux1, const R *aux2, const R *aux3, const R *aux4, R *p2cx,
                             R *p2cz, R *r2dx, R *r2cz, R dh2, int nx, int nz)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            if (!INTERIOR(ix, iz)) continue;
            long i = IDX(ix, iz);
            p2cx[i] = (R)FN(ref_d2)(aux1, i, 1, dh2);
            p2cz[i] = (R)FN(ref_d2)(aux2, i, nx, dh2);
            r2dx[i] = (R)FN(ref_d2)(aux3, i, 1, dh2);
            r2cz[i] = (R)FN(ref_d2)(aux4, i, nx, dh2);
        }
}

/* src/parallelcalls.cu:216-243 */
void FN(orc_zeta_r)(const R *p2cx, const R *p2cz, const R *r2dx, const R *r2cz, const R *a_x,
                    const R *b_x, const R *a_z, const R *b_z, const R *psixcx, const R *psixcz,
                    const R *psizdx, const R *psizcz, R *zitaxcx, R *zitaxcz, R *zitazdx,
                    R *zitazcz, R *atenxcx, R *atenxcz, R *atenzdx, R *atenzcz, int nx, int nz,
                    R dh, int cpml)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            if (!(INTERIOR(ix, iz) && IN_STRIP(ix, iz))) continue;
            long i = IDX(ix, iz);
            R dxcx = (R)FN(ref_d1)(psixcx, i, 1, dh);
            R dxcz = (R)FN(ref_d1)(psixcz, i, nx, dh);
            R dzdx = (R)FN(ref_d1)(psizdx, i, 1, dh);
            R dzcz = (R)FN(ref_d1)(psizcz, i, nx, dh);
            zitaxcx[i] = b_x[ix] * zitaxcx[i] + a_x[ix] * (dxcx + p2cx[i]);
            zitaxcz[i] = b_z[iz] * zitaxcz[i] + a_z[iz] * (dxcz + p2cz[i]);
            zitazdx[i] = b_x[ix] * zitazdx[i] + a_x[ix] * (dzdx + r2dx[i]);
            zitazcz[i] = b_z[iz] * zitazcz[i] + a_z[iz] * (dzcz + r2cz[i]);
            atenxcx[i] = zitaxcx[i] + dxcx;
            atenxcz[i] = zitaxcz[i] + dxcz;
            atenzdx[i] = zitazdx[i] + dzdx;
            atenzcz[i] = zitazcz[i] + dzcz;
        }
}

/* src/parallelcalls.cu:144-164 */
void FN(orc_retro_propagation)(R *PF, const R *P_pre, const R *F_pre, R *P_past, R *F_past,
                               const R *res, R C, R dh2, int nx, int nz, int nt, int sz, int it,
                               int cpml, const R *p2cx, const R *p2cz, const R *r2dx,
                               const R *r2cz, const R *atenxcx, const R *atenxcz,
                               const R *atenzdx, const R *atenzcz)
{
    (void)PF; /* the reference passes PF but never touches it here */
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            long i = IDX(ix, iz);
            if (INTERIOR(ix, iz)) {
                P_past[i] = 2 * P_pre[i] - P_past[i] +
                            dh2 * C * (p2cx[i] + atenxcx[i] + r2dx[i] + atenzdx[i]);
                F_past[i] = 2 * F_pre[i] - F_past[i] +
                            dh2 * C * (p2cz[i] + r2cz[i] + atenxcz[i] + atenzcz[i]);
            }
            if (ix > (cpml - 1) && ix < (nx - cpml) && iz == (sz - 1)) {
                P_past[i] += res[ix + (long)nx * (nt - it - 1)];
                F_past[i] += res[ix + (long)nx * (nt - it - 1)];
            }
        }
}

/* src/parallelcalls.cu:245-259 */
void FN(orc_gradient)(const R *P_pre, const R *F_pre, const R *P_past, const R *F_past, R *gcx,
                      R *gcz, R *gdx, R dh2, R dt, int nx, int nz)
{
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            if (!INTERIOR(ix, iz)) continue;
            long i = IDX(ix, iz);
            R p2 = (R)FN(ref_d2)(P_pre, i, 1, dh2);
            R r2 = (R)FN(ref_d2)(F_pre, i, nx, dh2);
            gcx[i] += dt * p2 * P_past[i];
            gcz[i] += dt * r2 * (P_past[i] + F_past[i]);
            gdx[i] += dt * p2 * F_past[i];
        }
}

/* src/parallelcalls.cu:261-271 */
void FN(orc_normal)(R *gcx, R *gcz, R *gdx, int nx, int nz, R ngcx, R ngcz, R ngdx)
{
    for (int iz = ORC_LAYER + 1; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            long i = IDX(ix, iz);
            gcx[i] = gcx[i] / ngcx;
            gcz[i] = gcz[i] / ngcz;
            gdx[i] = gdx[i] / ngdx;
        }
}

/* src/parallelcalls.cu:273-286 */
void FN(orc_update_model)(const R *gcx, const R *gcz, const R *gdx, R *v_hor, R *v_po, R *v_nmo,
                          R alpha1, R alpha2, R alpha3, int nx, int nz)
{
    for (int iz = ORC_LAYER + 1; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            long i = IDX(ix, iz);
            v_po[i] = v_po[i] - (alpha2 * gcz[i]);
            v_nmo[i] = v_nmo[i] - (alpha3 * gdx[i]);
            v_hor[i] = v_hor[i] - (alpha1 * gcx[i]);
            if (v_hor[i] < v_nmo[i]) v_hor[i] = v_nmo[i];
        }
}

/* src/parallelcalls.cu:288-302 */
void FN(orc_compute_sy)(R *s_vp, R *s_vn, R *s_vh, R *y_b1, R *y_b2, R *y_b3, const R *vp,
                        const R *vn, const R *vh, const R *back_vp, const R *back_vn,
                        const R *back_vh, const R *b1, const R *b2, const R *b3, const R *back_b1,
                        const R *back_b2, const R *back_b3, int nx, int nz, int k)
{
    long n = (long)nx * nz, o = (long)k * n;
    for (long i = 0; i < n; i++) {
        s_vp[i + o] = vp[i] - back_vp[i];
        s_vn[i + o] = vn[i] - back_vn[i];
        s_vh[i + o] = vh[i] - back_vh[i];
        y_b1[i + o] = b1[i] - back_b1[i];
        y_b2[i + o] = b2[i] - back_b2[i];
        y_b3[i + o] = b3[i] - back_b3[i];
    }
}

/* src/parallelcalls.cu:304-315 */
void FN(orc_compute_qi)(R *q_b1, R *q_b2, R *q_b3, const R *y_b1, const R *y_b2, const R *y_b3,
                        R eps_v, R eps_d, R eps_e, int nx, int nz, int k)
{
    long n = (long)nx * nz, o = (long)k * n;
    for (long i = 0; i < n; i++) {
        q_b1[i] -= eps_v * y_b1[i + o];
        q_b2[i] -= eps_d * y_b2[i + o];
        q_b3[i] -= eps_e * y_b3[i + o];
    }
}

/* src/parallelcalls.cu:317-328 */
void FN(orc_compute_ri)(R *r_b1, R *r_b2, R *r_b3, const R *q_b1, const R *q_b2, const R *q_b3,
                        R gamma_v, R gamma_d, R gamma_e, int nx, int nz)
{
    long n = (long)nx * nz;
    for (long i = 0; i < n; i++) {
        r_b1[i] = gamma_v * q_b1[i];
        r_b2[i] = gamma_d * q_b2[i];
        r_b3[i] = gamma_e * q_b3[i];
    }
}

/* src/parallelcalls.cu:330-341 */
void FN(orc_update_r)(R *r_b1, R *r_b2, R *r_b3, const R *s_vp, const R *s_vn, const R *s_vh,
                      R eps_v, R eps_d, R eps_e, R beta_v, R beta_d, R beta_e, int nx, int nz,
                      int k)
{
    long n = (long)nx * nz, o = (long)k * n;
    for (long i = 0; i < n; i++) {
        r_b1[i] += (eps_v - beta_v) * s_vp[i + o];
        r_b2[i] += (eps_d - beta_d) * s_vn[i + o];
        r_b3[i] += (eps_e - beta_e) * s_vh[i + o];
    }
}

/* src/parallelcalls.cu:343-404; bounds from include/parallelcalls.h:7-12 */
void FN(orc_update_lbfgs)(const R *r_b1, const R *r_b2, const R *r_b3, R *vp, R *vn, R *vh,
                          const R *back_vp, const R *back_vn, const R *back_vh, int nx, int nz,
                          R alpha_v, R alpha_d, R alpha_e, int flag_v, int flag_d, int flag_e,
                          int flag_min, int flag_max)
{
    for (int iz = ORC_LAYER + 1; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            long i = IDX(ix, iz);
            if (flag_v == 1) {
                vp[i] = back_vp[i] - alpha_v * r_b1[i];
                if (flag_max == 1 && vp[i] > ORC_MAX_V) vp[i] = ORC_MAX_V;
                if (flag_min == 1 && vp[i] < ORC_MIN_V) vp[i] = ORC_MIN_V;
            }
            if (flag_d == 1) {
                vn[i] = back_vn[i] - alpha_d * r_b2[i];
                if (flag_max == 1 && vn[i] > ORC_MAX_D) vn[i] = ORC_MAX_D;
                if (flag_min == 1 && vn[i] < ORC_MIN_D) vn[i] = ORC_MIN_D;
            }
            if (flag_e == 1) {
                vh[i] = back_vh[i] - alpha_e * r_b3[i];
                if (flag_max == 1 && vh[i] > ORC_MAX_E) vh[i] = ORC_MAX_E;
                if (flag_min == 1 && vh[i] < ORC_MIN_E) vh[i] = ORC_MIN_E;
                if (vh[i] < vn[i]) vh[i] = vn[i];
            }
        }
}

/* ---------------- host loops of src/main.c ---------------- */

/* src/main.c:448-453: fi += powf(res,2) in R, then fi/2 */
R FN(orc_host_misfit)(const R *res, long n)
{
    R fi = 0;
    for (long j = 0; j < n; j++) fi += POW2(res[j]);
    fi = fi / 2;
    return fi;
}

/* src/main.c:551-559: float sum of squares, then sqrtf */
R FN(orc_host_norm)(const R *g, long n)
{
    R s = 0;
    for (long i = 0; i < n; i++) s += POW2(g[i]);
    return (R)sqrt(s);
}

/* src/main.c:578-580 (and the other dots of the two-loop): t += (a*b)/2.0 */
R FN(orc_host_halfdot)(const R *a, const R *b, long n)
{
    R t = 0;
    for (long i = 0; i < n; i++) t += (a[i] * b[i]) / 2.0;
    return t;
}

/* src/main.c:626-631: s.y/2 and y.y/2 in one pass */
void FN(orc_host_sy_yy)(const R *s, const R *y, long n, R *sy, R *yy)
{
    R a = 0, b = 0;
    for (long i = 0; i < n; i++) {
        a += (s[i] * y[i]) / 2.0;
        b += POW2(y[i]) / 2.0;
    }
    *sy = a;
    *yy = b;
}

/* src/main.c:328-332: Ricker wavelet, t accumulated in R, delay 1/f */
void FN(orc_ricker)(R *source, int nt, R dt, R f)
{
    R t = 0;
    for (int it = 0; it < nt; it++) {
        t += dt;
        source[it] = 1 * (1 - 2 * pow(PI_D * f * (t - (1 / f)), 2)) *
                     exp(-pow(PI_D * f * (t - (1 / f)), 2));
    }
}

/* src/main.c:48-51, 276-279, 318-319: zeroed a/b, then the CPML profiles */
void FN(orc_setup_cpml)(R *a_x, R *b_x, R *a_z, R *b_z, int nx, int nz, int cpml, R dh, R dt, R f,
                        R vmax, R R_coef)
{
    R L = cpml * dh;
    R d0 = -3 * log(R_coef) / (2 * L);
    memset(a_x, 0, sizeof(R) * nx);
    memset(b_x, 0, sizeof(R) * nx);
    memset(a_z, 0, sizeof(R) * nz);
    memset(b_z, 0, sizeof(R) * nz);
    FN(orc_cpml_x)(a_x, b_x, cpml, vmax, nx, dt, dh, f, d0, L);
    FN(orc_cpml_z)(a_z, b_z, cpml, vmax, nz, dt, dh, f, d0, L);
}

typedef struct {
    R *P_pre, *P_past, *F_pre, *F_past, *PF, *p2, *r2;
    R *psi_px, *psi_fz, *z_px, *z_fz, *aten_p, *aten_f;
    R *buf0, *buf1; /* P and F of one time level are contiguous (src/main.c:162-165) */
} FN(fwd_state);

static void FN(fwd_alloc)(FN(fwd_state) *s, long n)
{
    s->buf0 = (R *)calloc(2 * n, sizeof(R));
    s->buf1 = (R *)calloc(2 * n, sizeof(R));
    s->P_pre = s->buf0; s->F_pre = s->buf0 + n;
    s->P_past = s->buf1; s->F_past = s->buf1 + n;
    s->PF = (R *)calloc(n, sizeof(R));
    s->p2 = (R *)calloc(n, sizeof(R));
    s->r2 = (R *)calloc(n, sizeof(R));
    s->psi_px = (R *)calloc(n, sizeof(R));
    s->psi_fz = (R *)calloc(n, sizeof(R));
    s->z_px = (R *)calloc(n, sizeof(R));
    s->z_fz = (R *)calloc(n, sizeof(R));
    s->aten_p = (R *)calloc(n, sizeof(R));
    s->aten_f = (R *)calloc(n, sizeof(R));
}

static void FN(fwd_free)(FN(fwd_state) *s)
{
    free(s->buf0); free(s->buf1); free(s->PF); free(s->p2); free(s->r2);
    free(s->psi_px); free(s->psi_fz); free(s->z_px); free(s->z_fz);
    free(s->aten_p); free(s->aten_f);
}

static void FN(swap_levels)(R **Pa, R **Pb, R **Fa, R **Fb)
{
    R *t = *Pa; *Pa = *Pb; *Pb = t;
    t = *Fa; *Fa = *Fb; *Fb = t;
}

/* One shot forward (src/main.c:336-365 and, with `snap`, 410-434 where
 * launchPropagation, src/serialcalls.cu:55-66, copies P_past|F_past before the
 * update: snap[it] holds the previous-previous state).  `shot` is nx*nt and is
 * only written on the receiver row. */
void FN(orc_forward_shot)(int nx, int nz, int nt, int cpml, int sx, int sz, R dh, R dt,
                          const R *a_x, const R *b_x, const R *a_z, const R *b_z, const R *v_hor,
                          const R *v_po, const R *v_nmo, const R *source, R *shot, R *snap)
{
    long n = (long)nx * nz;
    R dh2 = dh * dh;
    R C = (dt * dt) / dh2;
    FN(fwd_state) s;
    FN(fwd_alloc)(&s, n);
    for (int it = 0; it < nt; it++) {
        if (snap) memcpy(snap + 2 * (long)it * n, s.P_past, 2 * n * sizeof(R));
        FN(orc_psi_f)(s.P_pre, s.F_pre, a_x, b_x, a_z, b_z, s.psi_px, s.psi_fz, nx, nz, dh, cpml);
        FN(orc_second_derivate_p)(s.P_pre, s.F_pre, s.p2, s.r2, dh2, nx, nz);
        FN(orc_zeta_f)(s.p2, s.r2, a_x, b_x, a_z, b_z, s.psi_px, s.psi_fz, s.z_px, s.z_fz,
                       s.aten_p, s.aten_f, nx, nz, dh, cpml);
        FN(orc_propagator_f)(s.p2, s.r2, s.PF, s.P_pre, s.F_pre, s.P_past, s.F_past, v_hor, v_po,
                             v_nmo, s.aten_p, s.aten_f, source, shot, C, dh2, nx, nz, sx, sz, it,
                             cpml);
        FN(swap_levels)(&s.P_past, &s.P_pre, &s.F_past, &s.F_pre);
    }
    FN(fwd_free)(&s);
}

/* Misfit and gradient of one shot as src/main.c:408-495 computes them: forward
 * with snapshots, residual (syn - obs), float misfit, then `nt_adj` (normally
 * nt) steps of launchBackPropagation (src/serialcalls.cu:68-90) accumulating
 * into gcx/gcz/gdx.  Returns fi of src/main.c:448-453. */
R FN(orc_gradient_shot)(int nx, int nz, int nt, int cpml, int sx, int sz, R dh, R dt,
                        const R *a_x, const R *b_x, const R *a_z, const R *b_z, const R *v_hor,
                        const R *v_po, const R *v_nmo, const R *source, const R *shot_obs, R *gcx,
                        R *gcz, R *gdx, R *res_out, int nt_adj)
{
    long n = (long)nx * nz;
    R dh2 = dh * dh;
    R C = (dt * dt) / dh2;
    R *snap = (R *)malloc(sizeof(R) * 2 * n * (long)nt);
    R *shot2 = (R *)calloc((long)nx * nt, sizeof(R));
    R *Res = (R *)calloc((long)nx * nt, sizeof(R));
    FN(orc_forward_shot)(nx, nz, nt, cpml, sx, sz, dh, dt, a_x, b_x, a_z, b_z, v_hor, v_po, v_nmo,
                         source, shot2, snap);
    FN(orc_res)(Res, shot_obs, shot2, nx, nt);
    R fi = FN(orc_host_misfit)(Res, (long)nx * nt);
    if (res_out) memcpy(res_out, Res, sizeof(R) * nx * (long)nt);

    /* adjoint state: fresh zeroed buffers stand for the memsets of src/main.c:457-475 */
    R *b0 = (R *)calloc(2 * n, sizeof(R)), *b1 = (R *)calloc(2 * n, sizeof(R));
    R *P_pre = b0, *F_pre = b0 + n, *P_past = b1, *F_past = b1 + n;
    R *a1 = (R *)calloc(n, sizeof(R)), *a2 = (R *)calloc(n, sizeof(R));
    R *a3 = (R *)calloc(n, sizeof(R)), *a4 = (R *)calloc(n, sizeof(R));
    R *p2cx = (R *)calloc(n, sizeof(R)), *p2cz = (R *)calloc(n, sizeof(R));
    R *r2dx = (R *)calloc(n, sizeof(R)), *r2cz = (R *)calloc(n, sizeof(R));
    R *psixcx = (R *)calloc(n, sizeof(R)), *psixcz = (R *)calloc(n, sizeof(R));
    R *psizdx = (R *)calloc(n, sizeof(R)), *psizcz = (R *)calloc(n, sizeof(R));
    R *zxcx = (R *)calloc(n, sizeof(R)), *zxcz = (R *)calloc(n, sizeof(R));
    R *zzdx = (R *)calloc(n, sizeof(R)), *zzcz = (R *)calloc(n, sizeof(R));
    R *axcx = (R *)calloc(n, sizeof(R)), *axcz = (R *)calloc(n, sizeof(R));
    R *azdx = (R *)calloc(n, sizeof(R)), *azcz = (R *)calloc(n, sizeof(R));
    R *PF = (R *)calloc(n, sizeof(R));
    for (int it = 0; it < nt_adj; it++) {
        const R *snapP = snap + 2 * n * (long)(nt - it - 1);
        const R *snapF = snapP + n;
        FN(orc_entry_point)(P_pre, F_pre, a1, a2, a3, a4, v_hor, v_po, v_nmo, nx, nz);
        FN(orc_second_derivate)(a1, a2, a3, a4, p2cx, p2cz, r2dx, r2cz, dh2, nx, nz);
        FN(orc_psi_r)(a1, a2, a3, a4, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx, psizcz, nx, nz,
                      dh, cpml);
        FN(orc_zeta_r)(p2cx, p2cz, r2dx, r2cz, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx, psizcz,
                       zxcx, zxcz, zzdx, zzcz, axcx, axcz, azdx, azcz, nx, nz, dh, cpml);
        FN(orc_retro_propagation)(PF, P_pre, F_pre, P_past, F_past, Res, C, dh2, nx, nz, nt, sz,
                                  it, cpml, p2cx, p2cz, r2dx, r2cz, axcx, axcz, azdx, azcz);
        FN(orc_gradient)(snapP, snapF, P_past, F_past, gcx, gcz, gdx, dh2, dt, nx, nz);
        FN(swap_levels)(&P_past, &P_pre, &F_past, &F_pre);
    }
    free(b0); free(b1); free(a1); free(a2); free(a3); free(a4);
    free(p2cx); free(p2cz); free(r2dx); free(r2cz);
    free(psixcx); free(psixcz); free(psizdx); free(psizcz);
    free(zxcx); free(zxcz); free(zzdx); free(zzcz);
    free(axcx); free(axcz); free(azdx); free(azcz); free(PF);
    free(snap); free(shot2); free(Res);
    return fi;
}

/* One L-BFGS direction as src/main.c:570-682 computes it (iteration n >=
 * it_LBFGS, history slot k): s/y into slot k, first loop l = k..0, gamma from
 * slot k, second loop l = 0..k.  sigma/epsilon are [3][m] (v, d, e) and
 * gamma3 gets (gamma_v, gamma_d, gamma_e).  Pairings as src/main.c:573. */
void FN(orc_lbfgs_direction)(int nx, int nz, int k, R *s_vp, R *s_vn, R *s_vh, R *y_gcz,
                             R *y_gdx, R *y_gcx, const R *v_po, const R *v_nmo, const R *v_hor,
                             const R *back_vpo, const R *back_vnmo, const R *back_vhor,
                             const R *gcz, const R *gdx, const R *gcx, const R *back_gcz,
                             const R *back_gdx, const R *back_gcx, R *q_gcz, R *q_gdx, R *q_gcx,
                             R *r_b1, R *r_b2, R *r_b3, R *sigma, R *epsilon, R *gamma3)
{
    long n = (long)nx * nz;
    R *sv = sigma, *sd = sigma + 5, *se = sigma + 10; /* m = 5 (src/main.c:59) */
    R *ev = epsilon, *ed = epsilon + 5, *ee = epsilon + 10;
    memcpy(q_gcz, gcz, sizeof(R) * n);
    memcpy(q_gcx, gcx, sizeof(R) * n);
    memcpy(q_gdx, gdx, sizeof(R) * n);
    FN(orc_compute_sy)(s_vp, s_vn, s_vh, y_gcz, y_gdx, y_gcx, v_po, v_nmo, v_hor, back_vpo,
                       back_vnmo, back_vhor, gcz, gdx, gcx, back_gcz, back_gdx, back_gcx, nx, nz, k);
    for (int l = k; l >= 0; l--) {
        long o = (long)l * n;
        R t;
        t = FN(orc_host_halfdot)(y_gcz + o, s_vp + o, n);
        sv[l] = 1.0 / t;
        ev[l] = sv[l] * FN(orc_host_halfdot)(q_gcz, s_vp + o, n);
        t = FN(orc_host_halfdot)(y_gdx + o, s_vn + o, n);
        sd[l] = 1.0 / t;
        ed[l] = sd[l] * FN(orc_host_halfdot)(q_gdx, s_vn + o, n);
        t = FN(orc_host_halfdot)(y_gcx + o, s_vh + o, n);
        se[l] = 1.0 / t;
        ee[l] = se[l] * FN(orc_host_halfdot)(q_gcx, s_vh + o, n);
        FN(orc_compute_qi)(q_gcz, q_gdx, q_gcx, y_gcz, y_gdx, y_gcx, ev[l], ed[l], ee[l], nx, nz, l);
    }
    long ok = (long)k * n;
    R sy, yy;
    FN(orc_host_sy_yy)(s_vp + ok, y_gcz + ok, n, &sy, &yy);
    gamma3[0] = sy / yy;
    FN(orc_host_sy_yy)(s_vn + ok, y_gdx + ok, n, &sy, &yy);
    gamma3[1] = sy / yy;
    FN(orc_host_sy_yy)(s_vh + ok, y_gcx + ok, n, &sy, &yy);
    gamma3[2] = sy / yy;
    FN(orc_compute_ri)(r_b1, r_b2, r_b3, q_gcz, q_gdx, q_gcx, gamma3[0], gamma3[1], gamma3[2], nx,
                       nz);
    for (int l = 0; l <= k; l++) {
        long o = (long)l * n;
        R bv = sv[l] * FN(orc_host_halfdot)(y_gcz + o, r_b1, n);
        R bd = sd[l] * FN(orc_host_halfdot)(y_gdx + o, r_b2, n);
        R be = se[l] * FN(orc_host_halfdot)(y_gcx + o, r_b3, n);
        FN(orc_update_r)(r_b1, r_b2, r_b3, s_vp, s_vn, s_vh, ev[l], ed[l], ee[l], bv, bd, be, nx, nz,
                         l);
    }
}

#undef IDX
#undef INTERIOR
#undef IN_STRIP
