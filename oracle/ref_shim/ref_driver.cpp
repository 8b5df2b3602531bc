/*
 * Driver for the reference's own kernels compiled for the CPU (test
 * infrastructure only; built into oracle/_ref/libref.so by `make -C oracle ref`).
 *
 * Each ref_* entry point runs one reference kernel over the launch grid that
 * src/serialcalls.cu gives it (32x32 blocks; 512-thread 1-D blocks for the
 * CPML profiles), or sequences one shot / one L-BFGS direction the way
 * src/main.c does.  Signatures equal the oracle's orc_*_f32 functions so that
 * tests can feed both the same inputs and compare bit for bit.
 */
#include "shim.h"
#include "parallelcalls.h"

#include <cmath>
#include <cstdlib>
#include <cstring>

shim_dim3 threadIdx, blockIdx, blockDim;

template <class Body>
static void run_grid(unsigned gx, unsigned gy, unsigned bx, unsigned by, Body &&body)
{
    blockDim = {bx, by, 1};
    for (unsigned kby = 0; kby < gy; kby++)
        for (unsigned kbx = 0; kbx < gx; kbx++) {
            blockIdx = {kbx, kby, 0};
            for (unsigned ty = 0; ty < by; ty++)
                for (unsigned tx = 0; tx < bx; tx++) {
                    threadIdx = {tx, ty, 0};
                    body();
                }
        }
}

/* grid extent as src/serialcalls.cu:18 computes it */
static unsigned blocks(int n, int b) { return (unsigned)ceil(n / (float)b); }

#define GRID2(nx, nz) blocks(nx, 32), blocks(nz, 32), 32, 32

extern "C" {

void ref_pre_variables(float *vel, float *eps, float *del, float *v_hor, float *v_po, float *v_nmo,
                       int nx, int nz)
{
    run_grid(GRID2(nx, nz), [&] { pre_variables(vel, eps, del, v_hor, v_po, v_nmo, nx, nz); });
}

void ref_cpml_x(float *a_x, float *b_x, int cpml, float vmax, int nx, float dt, float dh, float f,
                float d0, float L)
{
    run_grid(blocks(nx, 512), 1, 512, 1,
             [&] { CPML_x(a_x, b_x, cpml, vmax, nx, dt, dh, f, d0, L); });
}

void ref_cpml_z(float *a_z, float *b_z, int cpml, float vmax, int nz, float dt, float dh, float f,
                float d0, float L)
{
    run_grid(blocks(nz, 512), 1, 512, 1,
             [&] { CPML_z(a_z, b_z, cpml, vmax, nz, dt, dh, f, d0, L); });
}

void ref_psi_f(float *P, float *F, float *a_x, float *b_x, float *a_z, float *b_z, float *psi_px,
               float *psi_fz, int nx, int nz, float dh, int cpml)
{
    run_grid(GRID2(nx, nz),
             [&] { PSI_F(P, F, a_x, b_x, a_z, b_z, psi_px, psi_fz, nx, nz, dh, cpml); });
}

void ref_zeta_f(float *p2, float *r2, float *a_x, float *b_x, float *a_z, float *b_z,
                float *psi_px, float *psi_fz, float *z_px, float *z_fz, float *aten_p,
                float *aten_f, int nx, int nz, float dh, int cpml)
{
    /* ZETA_F takes P and F but does not read them (src/parallelcalls.cu:65-86) */
    float dh2 = dh * dh;
    run_grid(GRID2(nx, nz), [&] {
        ZETA_F(p2, r2, nullptr, nullptr, a_x, b_x, a_z, b_z, psi_px, psi_fz, z_px, z_fz, aten_p,
               aten_f, nx, nz, dh, dh2, cpml);
    });
}

void ref_second_derivate_p(float *P_pre, float *F_pre, float *p2, float *r2, float dh2, int nx,
                           int nz)
{
    run_grid(GRID2(nx, nz), [&] { SecondDerivate_P(P_pre, F_pre, p2, r2, dh2, nx, nz); });
}

void ref_propagator_f(float *p2, float *r2, float *PF, float *P_pre, float *F_pre, float *P_past,
                      float *F_past, float *v_hor, float *v_po, float *v_nmo, float *aten_p,
                      float *aten_f, float *source, float *shot, float C, float dh2, int nx,
                      int nz, int sx, int sz, int it, int cpml)
{
    run_grid(GRID2(nx, nz), [&] {
        propagator_F(p2, r2, PF, P_pre, F_pre, P_past, F_past, v_hor, v_po, v_nmo, aten_p, aten_f,
                     source, shot, C, dh2, nx, nz, sx, sz, it, cpml);
    });
}

void ref_res(float *Res, float *shot1, float *shot2, int nx, int nt)
{
    run_grid(GRID2(nx, nt), [&] { res(Res, shot1, shot2, nx, nt); });
}

void ref_entry_point(float *P_pre, float *F_pre, float *aux1, float *aux2, float *aux3,
                     float *aux4, float *v_hor, float *v_po, float *v_nmo, int nx, int nz)
{
    run_grid(GRID2(nx, nz),
             [&] { entryPoint(P_pre, F_pre, aux1, aux2, aux3, aux4, v_hor, v_po, v_nmo, nx, nz); });
}

void ref_psi_r(float *aux1, float *aux2, float *aux3, float *aux4, float *a_x, float *b_x,
               float *a_z, float *b_z, float *psixcx, float *psixcz, float *psizdx, float *psizcz,
               int nx, int nz, float dh, int cpml)
{
    run_grid(GRID2(nx, nz), [&] {
        PSI_R(aux1, aux2, aux3, aux4, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx, psizcz, nx, nz,
              dh, cpml);
    });
}

void ref_second_derivate(float *aux1, float *aux2, float *aux3, float *aux4, float *p2cx,
                         float *p2cz, float *r2dx, float *r2cz, float dh2, int nx, int nz)
{
    run_grid(GRID2(nx, nz), [&] {
        secondDerivate(aux1, aux2, aux3, aux4, p2cx, p2cz, r2dx, r2cz, dh2, nx, nz);
    });
}

void ref_zeta_r(float *p2cx, float *p2cz, float *r2dx, float *r2cz, float *a_x, float *b_x,
                float *a_z, float *b_z, float *psixcx, float *psixcz, float *psizdx,
                float *psizcz, float *zitaxcx, float *zitaxcz, float *zitazdx, float *zitazcz,
                float *atenxcx, float *atenxcz, float *atenzdx, float *atenzcz, int nx, int nz,
                float dh, int cpml)
{
    float dh2 = dh * dh;
    run_grid(GRID2(nx, nz), [&] {
        ZETA_R(p2cx, p2cz, r2dx, r2cz, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx, psizcz, zitaxcx,
               zitaxcz, zitazdx, zitazcz, atenxcx, atenxcz, atenzdx, atenzcz, nx, nz, dh, dh2,
               cpml);
    });
}

void ref_retro_propagation(float *PF, float *P_pre, float *F_pre, float *P_past, float *F_past,
                           float *resid, float C, float dh2, int nx, int nz, int nt, int sz,
                           int it, int cpml, float *p2cx, float *p2cz, float *r2dx, float *r2cz,
                           float *atenxcx, float *atenxcz, float *atenzdx, float *atenzcz)
{
    run_grid(GRID2(nx, nz), [&] {
        retroPropagation(PF, P_pre, F_pre, P_past, F_past, resid, C, dh2, nx, nz, nt, sz, it, cpml,
                         p2cx, p2cz, r2dx, r2cz, atenxcx, atenxcz, atenzdx, atenzcz);
    });
}

void ref_gradient(float *P_pre, float *F_pre, float *P_past, float *F_past, float *gcx,
                  float *gcz, float *gdx, float dh2, float dt, int nx, int nz)
{
    run_grid(GRID2(nx, nz),
             [&] { GRADIENT(P_pre, F_pre, P_past, F_past, gcx, gcz, gdx, dh2, dt, nx, nz); });
}

void ref_normal(float *gcx, float *gcz, float *gdx, int nx, int nz, float ngcx, float ngcz,
                float ngdx)
{
    run_grid(GRID2(nx, nz), [&] { NORMAL(gcx, gcz, gdx, nx, nz, ngcx, ngcz, ngdx); });
}

void ref_update_model(float *gcx, float *gcz, float *gdx, float *v_hor, float *v_po, float *v_nmo,
                      float alpha1, float alpha2, float alpha3, int nx, int nz)
{
    run_grid(GRID2(nx, nz), [&] {
        UpdateModel(gcx, gcz, gdx, v_hor, v_po, v_nmo, alpha1, alpha2, alpha3, nx, nz);
    });
}

void ref_compute_sy(float *s_vp, float *s_vn, float *s_vh, float *y_b1, float *y_b2, float *y_b3,
                    float *vp, float *vn, float *vh, float *back_vp, float *back_vn,
                    float *back_vh, float *b1, float *b2, float *b3, float *back_b1,
                    float *back_b2, float *back_b3, int nx, int nz, int k)
{
    run_grid(GRID2(nx, nz), [&] {
        compute_sy(s_vp, s_vn, s_vh, y_b1, y_b2, y_b3, vp, vn, vh, back_vp, back_vn, back_vh, b1,
                   b2, b3, back_b1, back_b2, back_b3, nx, nz, k);
    });
}

void ref_compute_qi(float *q_b1, float *q_b2, float *q_b3, float *y_b1, float *y_b2, float *y_b3,
                    float ev, float ed, float ee, int nx, int nz, int k)
{
    run_grid(GRID2(nx, nz),
             [&] { compute_qi(q_b1, q_b2, q_b3, y_b1, y_b2, y_b3, ev, ed, ee, nx, nz, k); });
}

void ref_compute_ri(float *r_b1, float *r_b2, float *r_b3, float *q_b1, float *q_b2, float *q_b3,
                    float gv, float gd, float ge, int nx, int nz)
{
    run_grid(GRID2(nx, nz),
             [&] { compute_ri(r_b1, r_b2, r_b3, q_b1, q_b2, q_b3, gv, gd, ge, nx, nz); });
}

void ref_update_r(float *r_b1, float *r_b2, float *r_b3, float *s_vp, float *s_vn, float *s_vh,
                  float ev, float ed, float ee, float bv, float bd, float be, int nx, int nz,
                  int k)
{
    run_grid(GRID2(nx, nz), [&] {
        update_r(r_b1, r_b2, r_b3, s_vp, s_vn, s_vh, ev, ed, ee, bv, bd, be, nx, nz, k);
    });
}

void ref_update_lbfgs(float *r_b1, float *r_b2, float *r_b3, float *vp, float *vn, float *vh,
                      float *back_vp, float *back_vn, float *back_vh, int nx, int nz,
                      float alpha_v, float alpha_d, float alpha_e, int flag_v, int flag_d,
                      int flag_e, int flag_min, int flag_max)
{
    run_grid(GRID2(nx, nz), [&] {
        update_LBFGS(r_b1, r_b2, r_b3, vp, vn, vh, back_vp, back_vn, back_vh, nx, nz, alpha_v,
                     alpha_d, alpha_e, flag_v, flag_d, flag_e, flag_min, flag_max);
    });
}

/* ---------------- one shot, sequenced as src/main.c ---------------- */

/* src/main.c:336-365 (observed data) and 410-434 (launchPropagation with the
 * pinned-host snapshot copy taken before the update, src/serialcalls.cu:60) */
void ref_forward_shot(int nx, int nz, int nt, int cpml, int sx, int sz, float dh, float dt,
                      float *a_x, float *b_x, float *a_z, float *b_z, float *v_hor, float *v_po,
                      float *v_nmo, float *source, float *shot, float *snap)
{
    long n = (long)nx * nz;
    float dh2 = dh * dh;
    float C = (dt * dt) / dh2;
    float *lvl0 = (float *)calloc(2 * n, sizeof(float)), *lvl1 = (float *)calloc(2 * n, sizeof(float));
    float *P_pre = lvl0, *F_pre = lvl0 + n, *P_past = lvl1, *F_past = lvl1 + n;
    float *PF = (float *)calloc(n, sizeof(float)), *p2 = (float *)calloc(n, sizeof(float));
    float *r2 = (float *)calloc(n, sizeof(float));
    float *psi_px = (float *)calloc(n, sizeof(float)), *psi_fz = (float *)calloc(n, sizeof(float));
    float *z_px = (float *)calloc(n, sizeof(float)), *z_fz = (float *)calloc(n, sizeof(float));
    float *aten_p = (float *)calloc(n, sizeof(float)), *aten_f = (float *)calloc(n, sizeof(float));
    for (int it = 0; it < nt; it++) {
        if (snap) memcpy(snap + 2 * n * it, P_past, 2 * n * sizeof(float));
        ref_second_derivate_p(P_pre, F_pre, p2, r2, dh2, nx, nz);
        ref_psi_f(P_pre, F_pre, a_x, b_x, a_z, b_z, psi_px, psi_fz, nx, nz, dh, cpml);
        ref_zeta_f(p2, r2, a_x, b_x, a_z, b_z, psi_px, psi_fz, z_px, z_fz, aten_p, aten_f, nx, nz,
                   dh, cpml);
        ref_propagator_f(p2, r2, PF, P_pre, F_pre, P_past, F_past, v_hor, v_po, v_nmo, aten_p,
                         aten_f, source, shot, C, dh2, nx, nz, sx, sz, it, cpml);
        float *t = P_past; P_past = P_pre; P_pre = t;
        t = F_past; F_past = F_pre; F_pre = t;
    }
    free(lvl0); free(lvl1); free(PF); free(p2); free(r2); free(psi_px); free(psi_fz);
    free(z_px); free(z_fz); free(aten_p); free(aten_f);
}

/* src/main.c:408-495 for one shot; returns fi (src/main.c:448-453) */
float ref_gradient_shot(int nx, int nz, int nt, int cpml, int sx, int sz, float dh, float dt,
                        float *a_x, float *b_x, float *a_z, float *b_z, float *v_hor, float *v_po,
                        float *v_nmo, float *source, float *shot_obs, float *gcx, float *gcz,
                        float *gdx, float *res_out, int nt_adj)
{
    long n = (long)nx * nz;
    float dh2 = dh * dh;
    float C = (dt * dt) / dh2;
    float *PF_h = (float *)malloc(sizeof(float) * 2 * n * nt);
    float *shot2 = (float *)calloc((long)nx * nt, sizeof(float));
    float *Res = (float *)calloc((long)nx * nt, sizeof(float));
    ref_forward_shot(nx, nz, nt, cpml, sx, sz, dh, dt, a_x, b_x, a_z, b_z, v_hor, v_po, v_nmo,
                     source, shot2, PF_h);
    ref_res(Res, shot_obs, shot2, nx, nt);
    float fi = 0;
    for (long j = 0; j < (long)nx * nt; j++) fi += powf(Res[j], 2);
    fi = fi / 2;
    if (res_out) memcpy(res_out, Res, sizeof(float) * nx * nt);

    float *lvl0 = (float *)calloc(2 * n, sizeof(float)), *lvl1 = (float *)calloc(2 * n, sizeof(float));
    float *P_pre = lvl0, *F_pre = lvl0 + n, *P_past = lvl1, *F_past = lvl1 + n;
    float *P_pre2 = (float *)calloc(2 * n, sizeof(float));
    float *F_pre2 = P_pre2 + n;
    float *buf[21];
    for (int q = 0; q < 21; q++) buf[q] = (float *)calloc(n, sizeof(float));
    float *aux1 = buf[0], *aux2 = buf[1], *aux3 = buf[2], *aux4 = buf[3];
    float *p2cx = buf[4], *p2cz = buf[5], *r2dx = buf[6], *r2cz = buf[7];
    float *psixcx = buf[8], *psixcz = buf[9], *psizdx = buf[10], *psizcz = buf[11];
    float *zitaxcx = buf[12], *zitaxcz = buf[13], *zitazdx = buf[14], *zitazcz = buf[15];
    float *atenxcx = buf[16], *atenxcz = buf[17], *atenzdx = buf[18], *atenzcz = buf[19];
    float *PF = buf[20];
    for (int it = 0; it < nt_adj; it++) {
        /* launchBackPropagation, src/serialcalls.cu:76-88 */
        memcpy(P_pre2, PF_h + (long)(nt - it - 1) * n * 2, 2 * n * sizeof(float));
        ref_entry_point(P_pre, F_pre, aux1, aux2, aux3, aux4, v_hor, v_po, v_nmo, nx, nz);
        ref_second_derivate(aux1, aux2, aux3, aux4, p2cx, p2cz, r2dx, r2cz, dh2, nx, nz);
        ref_psi_r(aux1, aux2, aux3, aux4, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx, psizcz, nx,
                  nz, dh, cpml);
        ref_zeta_r(p2cx, p2cz, r2dx, r2cz, a_x, b_x, a_z, b_z, psixcx, psixcz, psizdx, psizcz,
                   zitaxcx, zitaxcz, zitazdx, zitazcz, atenxcx, atenxcz, atenzdx, atenzcz, nx, nz,
                   dh, cpml);
        ref_retro_propagation(PF, P_pre, F_pre, P_past, F_past, Res, C, dh2, nx, nz, nt, sz, it,
                              cpml, p2cx, p2cz, r2dx, r2cz, atenxcx, atenxcz, atenzdx, atenzcz);
        ref_gradient(P_pre2, F_pre2, P_past, F_past, gcx, gcz, gdx, dh2, dt, nx, nz);
        float *t = P_past; P_past = P_pre; P_pre = t;
        t = F_past; F_past = F_pre; F_pre = t;
    }
    for (int q = 0; q < 21; q++) free(buf[q]);
    free(lvl0); free(lvl1); free(P_pre2); free(PF_h); free(shot2); free(Res);
    return fi;
}

/* src/main.c:570-682 for history slot k (m = 5); sigma and epsilon are
 * [3][5] (v, d, e), gamma3 = (gamma_v, gamma_d, gamma_e) */
void ref_lbfgs_direction(int nx, int nz, int k, float *s_vp, float *s_vn, float *s_vh,
                         float *y_gcz, float *y_gdx, float *y_gcx, float *v_po, float *v_nmo,
                         float *v_hor, float *back_vpo, float *back_vnmo, float *back_vhor,
                         float *gcz, float *gdx, float *gcx, float *back_gcz, float *back_gdx,
                         float *back_gcx, float *q_gcz, float *q_gdx, float *q_gcx, float *r_b1,
                         float *r_b2, float *r_b3, float *sigma, float *epsilon, float *gamma3)
{
    long n = (long)nx * nz;
    float *sigma_v = sigma, *sigma_d = sigma + 5, *sigma_e = sigma + 10;
    float *epsilon_v = epsilon, *epsilon_d = epsilon + 5, *epsilon_e = epsilon + 10;
    memcpy(q_gcz, gcz, n * sizeof(float));
    memcpy(q_gcx, gcx, n * sizeof(float));
    memcpy(q_gdx, gdx, n * sizeof(float));
    ref_compute_sy(s_vp, s_vn, s_vh, y_gcz, y_gdx, y_gcx, v_po, v_nmo, v_hor, back_vpo, back_vnmo,
                   back_vhor, gcz, gdx, gcx, back_gcz, back_gdx, back_gcx, nx, nz, k);
    for (int l = k; l >= 0; l--) {
        float *y1 = y_gcz + l * n, *s1 = s_vp + l * n;
        float ts = 0, tq = 0;
        for (long i = 0; i < n; i++) ts += (y1[i] * s1[i]) / 2.0;
        for (long i = 0; i < n; i++) tq += (q_gcz[i] * s1[i]) / 2.0;
        sigma_v[l] = 1.0 / ts;
        epsilon_v[l] = sigma_v[l] * tq;

        float *y2 = y_gdx + l * n, *s2 = s_vn + l * n;
        ts = 0; tq = 0;
        for (long i = 0; i < n; i++) ts += (y2[i] * s2[i]) / 2.0;
        for (long i = 0; i < n; i++) tq += (q_gdx[i] * s2[i]) / 2.0;
        sigma_d[l] = 1.0 / ts;
        epsilon_d[l] = sigma_d[l] * tq;

        float *y3 = y_gcx + l * n, *s3 = s_vh + l * n;
        ts = 0; tq = 0;
        for (long i = 0; i < n; i++) ts += (y3[i] * s3[i]) / 2.0;
        for (long i = 0; i < n; i++) tq += (q_gcx[i] * s3[i]) / 2.0;
        sigma_e[l] = 1.0 / ts;
        epsilon_e[l] = sigma_e[l] * tq;

        ref_compute_qi(q_gcz, q_gdx, q_gcx, y_gcz, y_gdx, y_gcx, epsilon_v[l], epsilon_d[l],
                       epsilon_e[l], nx, nz, l);
    }
    float *pairs_s[3] = {s_vp + k * n, s_vn + k * n, s_vh + k * n};
    float *pairs_y[3] = {y_gcz + k * n, y_gdx + k * n, y_gcx + k * n};
    for (int c = 0; c < 3; c++) {
        float sy = 0, yy = 0;
        for (long i = 0; i < n; i++) {
            sy += (pairs_s[c][i] * pairs_y[c][i]) / 2.0;
            yy += powf(pairs_y[c][i], 2) / 2.0;
        }
        gamma3[c] = sy / yy;
    }
    ref_compute_ri(r_b1, r_b2, r_b3, q_gcz, q_gdx, q_gcx, gamma3[0], gamma3[1], gamma3[2], nx, nz);
    for (int l = 0; l <= k; l++) {
        float tv = 0, td = 0, te = 0;
        for (long i = 0; i < n; i++) tv += (y_gcz[l * n + i] * r_b1[i]) / 2.0;
        for (long i = 0; i < n; i++) td += (y_gdx[l * n + i] * r_b2[i]) / 2.0;
        for (long i = 0; i < n; i++) te += (y_gcx[l * n + i] * r_b3[i]) / 2.0;
        float beta_v = sigma_v[l] * tv, beta_d = sigma_d[l] * td, beta_e = sigma_e[l] * te;
        ref_update_r(r_b1, r_b2, r_b3, s_vp, s_vn, s_vh, epsilon_v[l], epsilon_d[l], epsilon_e[l],
                     beta_v, beta_d, beta_e, nx, nz, l);
    }
}

} /* extern "C" */
