/*
 * fwi_compat.h -- drop-in replacement for danielvn/Fwi's include/serialcalls.h.
 *
 * The same 17 host entry points with the same signatures and argument
 * meaning, so that the reference's src/main.c links against
 * libfwi_gb300.so instead of src/serialcalls.cu + src/parallelcalls.cu.
 * Each one runs the library's own sm_103a kernels and leaves every buffer
 * the reference kernels write in the state they leave it (up to FP32
 * rounding: the reference evaluates its stencils in FP64 because of double
 * literals, this library in FP32).
 *
 * Conventions kept from the reference:
 *  - every pointer is a DEVICE pointer (cudaMalloc), except PF_h, a pinned
 *    host buffer (cudaMallocHost);
 *  - arrays are nx*nz floats, x fastest, I(ix,iz) = ix + nx*iz;
 *  - launches go to the legacy default stream, except where the reference
 *    uses stream1 / stream2 (launchPropagation, launchBackPropagation);
 *    with blocking streams (cudaStreamCreate) this gives the reference's
 *    ordering, including the snapshot copy before the update;
 *  - no status is returned (the reference returns void); the first CUDA
 *    error seen is kept and can be read with fwi_compat_last_error().
 */
#ifndef FWI_COMPAT_H
#define FWI_COMPAT_H

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* replaces src/serialcalls.cu:17-21 (kernel src/parallelcalls.cu:3-16):
 * v_po = vel^2, v_hor = v_po (1 + 2 epsilon), v_nmo = v_po (1 + 2 delta) */
void pre_variables_h(float *vel, float *epsilon, float *delta, float *v_hor, float *v_po,
                     float *v_nmo, int nx, int nz);

/* replaces src/serialcalls.cu:4-8 (kernel src/parallelcalls.cu:18-34): CPML a_x, b_x on the
 * left and right layers; other entries are left untouched */
void CPML_x_h(float *a_x, float *b_x, int CPML, float Vmax, int nx, float dt, float dh, float f,
              float d0, float L);

/* replaces src/serialcalls.cu:11-15 (kernel src/parallelcalls.cu:36-46): bottom layer only */
void CPML_z_h(float *a_z, float *b_z, int CPML, float Vmax, int nz, float dt, float dh, float f,
              float d0, float L);

/* replaces src/serialcalls.cu:23-28 (kernel src/parallelcalls.cu:48-63) */
void PSI_F_h(float *P, float *F, float *a_x, float *b_x, float *a_z, float *b_z, float *psi_px,
             float *psi_fz, int nx, int nz, float dh, int CPML);

/* replaces src/serialcalls.cu:37-41 (kernel src/parallelcalls.cu:65-86) */
void ZETA_F_h(float *p2, float *r2, float *P, float *F, float *a_x, float *b_x, float *a_z,
              float *b_z, float *psi_px, float *psi_fz, float *z_px, float *z_fz, float *aten_p,
              float *aten_f, int nx, int nz, float dh, float dh2, int CPML);

/* replaces src/serialcalls.cu:43-47 (kernel src/parallelcalls.cu:88-117) */
void propagator_F_h(float *p2, float *r2, float *PF, float *P_pre, float *F_pre, float *P_past,
                    float *F_past, float *v_hor, float *v_po, float *v_nmo, float *aten_p,
                    float *aten_f, float *source, float *shot, float C, float dh2, int nx, int nz,
                    int sx, int sz, int it, int CPML);

/* replaces src/serialcalls.cu:49-53 (kernel src/parallelcalls.cu:133-142); the reference's
 * caller passes nt as the last argument (src/main.c:437) */
void res_h(float *Res, float *shot1, float *shot2, int nx, int nz);

/* replaces src/serialcalls.cu:30-35 (kernel src/parallelcalls.cu:120-130) */
void SecondDerivate_P_h(float *P_pre, float *F_pre, float *p2, float *r2, float dh2, int nx,
                        int nz);

/* replaces src/serialcalls.cu:55-66: D2H copy of P_past|F_past (2*nx*nz floats, F = P +
 * nx*nz) into PF_h on stream1, then one forward time step (PSI_F, SecondDerivate_P, ZETA_F,
 * propagator_F of src/parallelcalls.cu) in two fused kernels */
void launchPropagation(cudaStream_t stream1, cudaStream_t stream2, float *PF_h, float *PF,
                       float *P_past, float *P_pre, float *F_past, float *F_pre, float *p2,
                       float *r2, float dh2, int nx, int nz, float *a_x, float *b_x, float *a_z,
                       float *b_z, float *psi_px, float *psi_fz, float dh, int CPML, float *z_px,
                       float *z_fz, float *aten_p, float *aten_f, float *v_hor, float *v_po,
                       float *v_nmo, float *source, float *shot2, float C, int sx, int sz, int it);

/* replaces src/serialcalls.cu:68-90: H2D copy of the snapshot into P_pre2|F_pre2 on
 * stream1, then one adjoint + imaging step (entryPoint, secondDerivate, PSI_R, ZETA_R,
 * retroPropagation, GRADIENT of src/parallelcalls.cu) in three fused kernels */
void launchBackPropagation(cudaStream_t stream1, cudaStream_t stream2, int nx, int nz, int nt,
                           float *PF_h, float *P_pre, float *P_past, float *F_pre, float *F_past,
                           float *aux1, float *aux2, float *aux3, float *aux4, float *v_hor,
                           float *v_po, float *v_nmo, float *p2cx, float *p2cz, float *r2dx,
                           float *r2cz, float dh2, float *P_pre2, float *F_pre2, float *a_x,
                           float *b_x, float *a_z, float *b_z, float *psixcx, float *psixcz,
                           float *psizdx, float *psizcz, float dh, int CPML, float *zitaxcx,
                           float *zitaxcz, float *zitazdx, float *zitazcz, float *atenxcx,
                           float *atenxcz, float *atenzdx, float *atenzcz, float *Res, float C,
                           float *PF, int it, int sx, int sz, float dt, float *gcx, float *gcz,
                           float *gdx);

/* replaces src/serialcalls.cu:92-96 (kernel src/parallelcalls.cu:261-271) */
void NORMAL_h(float *gcx, float *gcz, float *gdx, int nx, int nz, float ngcx, float ngcz,
              float ngdx);

/* replaces src/serialcalls.cu:98-103 (kernel src/parallelcalls.cu:273-286) */
void UpdateModel_h(float *gcx, float *gcz, float *gdx, float *v_hor, float *v_po, float *v_nmo,
                   float alpha1, float alpha2, float alpha3, int nx, int nz);

/* replaces src/serialcalls.cu:105-109 (kernel src/parallelcalls.cu:288-302) */
void compute_sy_h(float *s_vp, float *s_vn, float *s_vh, float *y_b1, float *y_b2, float *y_b3,
                  float *vp, float *vn, float *vh, float *back_vp, float *back_vn, float *back_vh,
                  float *b1, float *b2, float *b3, float *back_b1, float *back_b2, float *back_b3,
                  int nx, int nz, int k);

/* replaces src/serialcalls.cu:111-115 (kernel src/parallelcalls.cu:304-315) */
void compute_qi_h(float *q_b1, float *q_b2, float *q_b3, float *y_b1, float *y_b2, float *y_b3,
                  float epsilon_v, float epsilon_d, float epsilon_e, int nx, int nz, int k);

/* replaces src/serialcalls.cu:117-121 (kernel src/parallelcalls.cu:317-328) */
void compute_ri_h(float *r_b1, float *r_b2, float *r_b3, float *q_b1, float *q_b2, float *q_b3,
                  float gamma_v, float gamma_d, float gamma_e, int nx, int nz);

/* replaces src/serialcalls.cu:123-127 (kernel src/parallelcalls.cu:330-341) */
void update_r_h(float *r_b1, float *r_b2, float *r_b3, float *s_vp, float *s_vn, float *s_vh,
                float epsilon_v, float epsilon_d, float epsilon_e, float beta_v, float beta_d,
                float beta_e, int nx, int nz, int k);

/* replaces src/serialcalls.cu:129-133 (kernel src/parallelcalls.cu:343-404) */
void update_LBFGS_h(float *r_b1, float *r_b2, float *r_b3, float *vp, float *vn, float *vh,
                    float *back_vp, float *back_vn, float *back_vh, int nx, int nz,
                    float alpha_v, float alpha_d, float alpha_e, int flag_v, int flag_d,
                    int flag_e, int flag_min, int flag_max);

/* No reference counterpart (the reference checks no errors): the first CUDA error any
 * compat entry point met since the last call (cudaSuccess = 0), cleared on read. */
int fwi_compat_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
