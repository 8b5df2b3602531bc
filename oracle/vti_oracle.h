/*
 * CPU oracle for the 2-D pseudo-acoustic VTI FWI gradient path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library under
 * fwi_gb300/) links, loads or calls this code; only tests/, the smoke check
 * in __graft_entry__.py and the cpu_baseline / reference arm of bench.py use
 * it, and only to check results against it or to time it as the CPU baseline.
 *
 * Two families of functions:
 *
 *  orc_*  Restatement of danielvn/Fwi in the reference's own arithmetic.
 *         One function per reference kernel (src/parallelcalls.cu) with the
 *         same argument meaning, plus the host loops of src/main.c (misfit,
 *         norms, L-BFGS dot products) and drivers that sequence one shot the
 *         way src/main.c does.  The _f32 variant stores FP32 and evaluates the
 *         finite-difference stencils in FP64 exactly as the reference does
 *         (its coefficients are double literals); built with
 *         -ffp-contract=off it is bit-identical to the reference kernels run
 *         on the CPU (pinned by tests/golden).  The _f64 variant stores FP64.
 *
 *  orx_*  The native library's semantics (fwi.h): arbitrary source and
 *         receiver geometry, trace masks, FP64 misfit, and the EXACT discrete
 *         adjoint of the forward step including the CPML memory variables,
 *         whose imaging condition gives dJ/d(v_hor, v_po, v_nmo).  Pinned by
 *         its forward equalling orc_* and by dot-product and finite-difference
 *         tests in FP64.
 *
 * Layout everywhere: x fastest, index = ix + nx*iz (include/parallelcalls.h:5).
 */
#ifndef VTI_ORACLE_H
#define VTI_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* include/parallelcalls.h:6-12 */
#define ORC_LAYER 15
#define ORC_MIN_V 1.8e6
#define ORC_MAX_V 3.5e6
#define ORC_MIN_D 1.8e6
#define ORC_MAX_D 4e6
#define ORC_MIN_E 1.8e6
#define ORC_MAX_E 4.5e6

void orc_set_threads(int n);
int orc_get_threads(void);

/* ---------------- reference kernels, one for one ---------------- */
#define ORC_DECLARE(R, S)                                                                       \
void orc_pre_variables##S(const R *vel, const R *eps, const R *del, R *v_hor, R *v_po, R *v_nmo, \
                          int nx, int nz);                                                      \
void orc_cpml_x##S(R *a_x, R *b_x, int cpml, R vmax, int nx, R dt, R dh, R f, R d0, R L);       \
void orc_cpml_z##S(R *a_z, R *b_z, int cpml, R vmax, int nz, R dt, R dh, R f, R d0, R L);       \
void orc_psi_f##S(const R *P, const R *F, const R *a_x, const R *b_x, const R *a_z,             \
                  const R *b_z, R *psi_px, R *psi_fz, int nx, int nz, R dh, int cpml);          \
void orc_zeta_f##S(const R *p2, const R *r2, const R *a_x, const R *b_x, const R *a_z,          \
                   const R *b_z, const R *psi_px, const R *psi_fz, R *z_px, R *z_fz, R *aten_p, \
                   R *aten_f, int nx, int nz, R dh, int cpml);                                  \
void orc_second_derivate_p##S(const R *P_pre, const R *F_pre, R *p2, R *r2, R dh2, int nx,      \
                              int nz);                                                          \
void orc_propagator_f##S(const R *p2, const R *r2, R *PF, const R *P_pre, const R *F_pre,       \
                         R *P_past, R *F_past, const R *v_hor, const R *v_po, const R *v_nmo,   \
                         const R *aten_p, const R *aten_f, const R *source, R *shot, R C,       \
                         R dh2, int nx, int nz, int sx, int sz, int it, int cpml);              \
void orc_res##S(R *Res, const R *shot1, const R *shot2, int nx, int nt);                        \
void orc_entry_point##S(const R *P_pre, const R *F_pre, R *aux1, R *aux2, R *aux3, R *aux4,     \
                        const R *v_hor, const R *v_po, const R *v_nmo, int nx, int nz);         \
void orc_psi_r##S(const R *aux1, const R *aux2, const R *aux3, const R *aux4, const R *a_x,     \
                  const R *b_x, const R *a_z, const R *b_z, R *psixcx, R *psixcz, R *psizdx,    \
                  R *psizcz, int nx, int nz, R dh, int cpml);                                   \
void orc_second_derivate##S(const R *aux1, const R *aux2, const R *aux3, const R *aux4,         \
                            R *p2cx, R *p2cz, R *r2dx, R *r2cz, R dh2, int nx, int nz);         \
void orc_zeta_r##S(const R *p2cx, const R *p2cz, const R *r2dx, const R *r2cz, const R *a_x,    \
                   const R *b_x, const R *a_z, const R *b_z, const R *psixcx,                   \
                   const R *psixcz, const R *psizdx, const R *psizcz, R *zitaxcx, R *zitaxcz,   \
                   R *zitazdx, R *zitazcz, R *atenxcx, R *atenxcz, R *atenzdx, R *atenzcz,      \
                   int nx, int nz, R dh, int cpml);                                             \
void orc_retro_propagation##S(R *PF, const R *P_pre, const R *F_pre, R *P_past, R *F_past,      \
                              const R *res, R C, R dh2, int nx, int nz, int nt, int sz, int it, \
                              int cpml, const R *p2cx, const R *p2cz, const R *r2dx,            \
                              const R *r2cz, const R *atenxcx, const R *atenxcz,                \
                              const R *atenzdx, const R *atenzcz);                              \
void orc_gradient##S(const R *P_pre, const R *F_pre, const R *P_past, const R *F_past, R *gcx,  \
                     R *gcz, R *gdx, R dh2, R dt, int nx, int nz);                              \
void orc_normal##S(R *gcx, R *gcz, R *gdx, int nx, int nz, R ngcx, R ngcz, R ngdx);             \
void orc_update_model##S(const R *gcx, const R *gcz, const R *gdx, R *v_hor, R *v_po, R *v_nmo, \
                         R alpha1, R alpha2, R alpha3, int nx, int nz);                         \
void orc_compute_sy##S(R *s_vp, R *s_vn, R *s_vh, R *y_b1, R *y_b2, R *y_b3, const R *vp,       \
                       const R *vn, const R *vh, const R *back_vp, const R *back_vn,            \
                       const R *back_vh, const R *b1, const R *b2, const R *b3,                 \
                       const R *back_b1, const R *back_b2, const R *back_b3, int nx, int nz,    \
                       int k);                                                                  \
void orc_compute_qi##S(R *q_b1, R *q_b2, R *q_b3, const R *y_b1, const R *y_b2, const R *y_b3,  \
                       R eps_v, R eps_d, R eps_e, int nx, int nz, int k);                       \
void orc_compute_ri##S(R *r_b1, R *r_b2, R *r_b3, const R *q_b1, const R *q_b2, const R *q_b3,  \
                       R gamma_v, R gamma_d, R gamma_e, int nx, int nz);                        \
void orc_update_r##S(R *r_b1, R *r_b2, R *r_b3, const R *s_vp, const R *s_vn, const R *s_vh,    \
                     R eps_v, R eps_d, R eps_e, R beta_v, R beta_d, R beta_e, int nx, int nz,   \
                     int k);                                                                    \
void orc_update_lbfgs##S(const R *r_b1, const R *r_b2, const R *r_b3, R *vp, R *vn, R *vh,      \
                         const R *back_vp, const R *back_vn, const R *back_vh, int nx, int nz,  \
                         R alpha_v, R alpha_d, R alpha_e, int flag_v, int flag_d, int flag_e,   \
                         int flag_min, int flag_max);                                           \
/* ---- host loops of src/main.c, accumulation precision as there ---- */                       \
R orc_host_misfit##S(const R *res, long n);                                                     \
R orc_host_norm##S(const R *g, long n);                                                         \
R orc_host_halfdot##S(const R *a, const R *b, long n);                                          \
void orc_host_sy_yy##S(const R *s, const R *y, long n, R *sy, R *yy);                           \
/* ---- drivers that sequence one shot as src/main.c does ---- */                               \
void orc_ricker##S(R *source, int nt, R dt, R f);                                               \
void orc_setup_cpml##S(R *a_x, R *b_x, R *a_z, R *b_z, int nx, int nz, int cpml, R dh, R dt,    \
                       R f, R vmax, R R_coef);                                                  \
void orc_forward_shot##S(int nx, int nz, int nt, int cpml, int sx, int sz, R dh, R dt,          \
                         const R *a_x, const R *b_x, const R *a_z, const R *b_z,                \
                         const R *v_hor, const R *v_po, const R *v_nmo, const R *source,        \
                         R *shot, R *snap);                                                     \
R orc_gradient_shot##S(int nx, int nz, int nt, int cpml, int sx, int sz, R dh, R dt,            \
                       const R *a_x, const R *b_x, const R *a_z, const R *b_z,                  \
                       const R *v_hor, const R *v_po, const R *v_nmo, const R *source,          \
                       const R *shot_obs, R *gcx, R *gcz, R *gdx, R *res_out, int nt_adj);      \
void orc_lbfgs_direction##S(int nx, int nz, int k, R *s_vp, R *s_vn, R *s_vh, R *y_gcz,         \
                            R *y_gdx, R *y_gcx, const R *v_po, const R *v_nmo,                  \
                            const R *v_hor, const R *back_vpo, const R *back_vnmo,              \
                            const R *back_vhor, const R *gcz, const R *gdx, const R *gcx,       \
                            const R *back_gcz, const R *back_gdx, const R *back_gcx, R *q_gcz,  \
                            R *q_gdx, R *q_gcx, R *r_b1, R *r_b2, R *r_b3, R *sigma,            \
                            R *epsilon, R *gamma3);

ORC_DECLARE(float, _f32)
ORC_DECLARE(double, _f64)
#undef ORC_DECLARE

/* ---------------- native semantics (fwi.h), exact adjoint ---------------- */
#define ORX_MODE_REF_COMPAT 0
#define ORX_MODE_EXACT 1

#define ORX_DECLARE(R, S)                                                                        \
void orx_forward##S(int nx, int nz, int nt, int cpml, R dh, R dt, const R *a_x, const R *b_x,    \
                    const R *a_z, const R *b_z, const R *v_hor, const R *v_po, const R *v_nmo,  \
                    int sx, int sz, const R *wavelet, int rz, int rx0, int rx1, R *rec,         \
                    R *img_g, R *img_h, int exact);                                             \
double orx_gradient_shot##S(int nx, int nz, int nt, int cpml, R dh, R dt, const R *a_x,          \
                            const R *b_x, const R *a_z, const R *b_z, const R *v_hor,            \
                            const R *v_po, const R *v_nmo, int sx, int sz, const R *wavelet,     \
                            int rz, int rx0, int rx1, const R *obs, const unsigned char *mask,   \
                            int mode, R *g_vh, R *g_vp, R *g_vn, R *adj_src_trace,               \
                            const R *res_override);

ORX_DECLARE(float, _f32)
ORX_DECLARE(double, _f64)
#undef ORX_DECLARE

#ifdef __cplusplus
}
#endif
#endif
