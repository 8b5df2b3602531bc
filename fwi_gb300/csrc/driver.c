/*
 * Host driver in C over the native C-ABI: the reference's inversion loop
 * (src/main.c:274-806) without MPI.
 *
 *   fwi_invert (one frequency band, src/main.c:396-801):
 *     iteration 0: gradient, then the steepest-descent step with fixed
 *                  lengths (src/main.c:539-568);
 *     iteration n: gradient, L-BFGS direction, then backtracking: trial
 *                  model m_back - alpha r, misfit of all shots; a NaN misfit
 *                  or one above the iteration's misfit halves alpha (with
 *                  armijo_c1 > 0, also one above J - c1 alpha g.r); more
 *                  than max_halvings halvings restore m_back and end the
 *                  band (src/main.c:690-786).
 *   fwi_invert_bands: the band loop around it (src/main.c:274-333, 802).
 *   fwi_load_model_files / fwi_save_model_files: the raw float32 model
 *     files (src/main.c:101-123, 823-835).
 *
 * reset_alpha = 0 keeps the reference's behaviour: alpha and the halving
 * count persist across the iterations of a band (src/main.c:308-311 resets
 * them only per band).
 */
#include "../../include/fwi.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void fwi_invert_defaults(fwi_invert_opts *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->iterations = 100;        /* src/main.c:12 */
    o->lbfgs_m = 5;             /* src/main.c:59 */
    o->first_alpha[0] = 3e5f;   /* v_hor, src/main.c:567 */
    o->first_alpha[1] = 2e5f;   /* v_po */
    o->first_alpha[2] = 2.5e5f; /* v_nmo */
    o->alpha0 = 1.0f;           /* src/main.c:62 */
    o->max_halvings = 5;        /* src/main.c:777 */
    o->reset_alpha = 0;
    o->flag_min = 0;            /* src/main.c:693 passes 0, 0 */
    o->flag_max = 0;
    o->armijo_c1 = 0.0;
    o->curvature_guard = 0;     /* the reference's two-loop: every pair */
}

int fwi_invert(void *ctx, const fwi_shot *shots, int nshots, const void *obs, const unsigned char *mask,
               const fwi_invert_opts *opts, double *misfit_history, int *iterations_done)
{
    fwi_invert_opts o;
    if (opts) o = *opts;
    else fwi_invert_defaults(&o);
    /* obs == NULL: the records kept in the context (fwi_store_observed / fwi_model_observed) */
    if (!ctx || !shots || nshots <= 0 || o.iterations <= 0 || o.armijo_c1 < 0.0) return FWI_ERR_ARG;
    float alpha = o.alpha0;
    int count = 0;
    int done = 0;
    int rc = fwi_set_lbfgs_guard(ctx, o.curvature_guard);
    if (rc != FWI_OK) return rc;
    for (int n = 0; n < o.iterations; n++) {
        double phi = 0.0;
        rc = fwi_gradient(ctx, shots, nshots, obs, mask, NULL, NULL, NULL, &phi);
        if (rc != FWI_OK) break;
        if (misfit_history) misfit_history[n] = phi;
        done = n + 1;
        if (n == 0) {
            rc = fwi_first_step(ctx, o.first_alpha[0], o.first_alpha[1], o.first_alpha[2]);
            if (rc != FWI_OK) break;
            continue;
        }
        rc = fwi_lbfgs_direction(ctx, o.lbfgs_m, NULL);
        if (rc != FWI_OK) break;
        double slope = 0.0; /* sum of g.r: the misfit falls by about alpha * slope */
        if (o.armijo_c1 > 0.0) {
            double s3[3];
            rc = fwi_direction_slope(ctx, s3);
            if (rc != FWI_OK) break;
            slope = s3[0] + s3[1] + s3[2];
        }
        if (o.reset_alpha) {
            alpha = o.alpha0;
            count = 0;
        }
        double trial = 1e10;
        int stop = 0;
        for (;;) {
            rc = fwi_lbfgs_update(ctx, alpha, alpha, alpha, o.flag_min, o.flag_max);
            if (rc != FWI_OK) break;
            rc = fwi_misfit(ctx, shots, nshots, obs, mask, &trial);
            int accept;
            if (rc == FWI_ERR_NUMERIC || isnan(trial)) {
                rc = FWI_OK;
                accept = 0;
            } else if (rc != FWI_OK) {
                break;
            } else {
                accept = trial <= phi;  /* the reference loops while trial > phi */
                if (accept && o.armijo_c1 > 0.0 && slope > 0.0)
                    accept = trial <= phi - o.armijo_c1 * (double)alpha * slope;
            }
            if (accept) break;
            count++;
            alpha *= 0.5f;
            if (count > o.max_halvings) {
                rc = fwi_restore_model(ctx);
                stop = 1;
                break;
            }
        }
        if (rc != FWI_OK || stop) break;
    }
    if (iterations_done) *iterations_done = done;
    return rc;
}

int fwi_invert_bands(void *ctx, const fwi_shot *shots, int nshots, const unsigned char *mask, float f0, float df,
                     int nbands, int nt, fwi_band_obs_fn band_obs, void *user, const fwi_invert_opts *opts,
                     int restart_model, double *misfit_history, int *iterations_done)
{
    fwi_invert_opts o;
    if (opts) o = *opts;
    else fwi_invert_defaults(&o);
    if (!ctx || !shots || nshots <= 0 || nbands <= 0 || nt <= 0 || !band_obs || !(f0 > 0.0f)) return FWI_ERR_ARG;
    fwi_config cfg;
    int rc = fwi_get_config(ctx, &cfg);
    if (rc != FWI_OK) return rc;
    void *m0 = NULL;
    size_t plane = 0;
    if (restart_model) {
        const size_t elem = cfg.precision == FWI_PREC_FP64 ? 8 : 4;
        plane = (size_t)cfg.nx * (size_t)cfg.nz * elem;
        m0 = malloc(3 * plane);
        if (!m0) return FWI_ERR_NOMEM;
        rc = fwi_get_model(ctx, m0, (char *)m0 + plane, (char *)m0 + 2 * plane);
        if (rc != FWI_OK) {
            free(m0);
            return rc;
        }
    }
    for (int b = 0; b < nbands && rc == FWI_OK; b++) {
        const float f = f0 + (float)b * df;
        if (restart_model && b > 0) {
            rc = fwi_set_model(ctx, m0, (char *)m0 + plane, (char *)m0 + 2 * plane);
            if (rc != FWI_OK) break;
        }
        rc = fwi_set_frequency(ctx, f, nt);
        if (rc != FWI_OK) break;
        /* the band's records: the callback's, or (NULL) those it left in the context's store */
        const void *obs = NULL;
        if (band_obs(user, b, f, &obs) != 0) {
            rc = FWI_ERR_ARG;
            break;
        }
        int done = 0;
        rc = fwi_invert(ctx, shots, nshots, obs, mask, &o, misfit_history ? misfit_history + (size_t)b * o.iterations : NULL,
                        &done);
        if (iterations_done) iterations_done[b] = done;
    }
    free(m0);
    return rc;
}

/* Reads n float32 values; FWI_ERR_ARG if the file is missing or shorter. */
static int read_f32(const char *path, float *out, size_t n)
{
    FILE *fp = path ? fopen(path, "rb") : NULL;
    if (!fp) return FWI_ERR_ARG;
    const size_t got = fread(out, sizeof(float), n, fp);
    fclose(fp);
    return got == n ? FWI_OK : FWI_ERR_ARG;
}

static int write_f32(const char *path, const float *in, size_t n)
{
    FILE *fp = path ? fopen(path, "wb") : NULL;
    if (!fp) return FWI_ERR_ARG;
    const size_t put = fwrite(in, sizeof(float), n, fp);
    const int closed = fclose(fp);
    return (put == n && closed == 0) ? FWI_OK : FWI_ERR_ARG;
}

int fwi_load_model_files(void *ctx, const char *vp_path, const char *eps_path, const char *delta_path)
{
    fwi_config cfg;
    int rc = fwi_get_config(ctx, &cfg);
    if (rc != FWI_OK) return rc;
    const size_t n = (size_t)cfg.nx * (size_t)cfg.nz;
    const size_t elem = cfg.precision == FWI_PREC_FP64 ? 8 : 4;
    float *f = (float *)malloc(3 * n * sizeof(float));
    void *m = elem == 8 ? malloc(3 * n * elem) : (void *)f;
    if (!f || !m) {
        free(f);
        if (elem == 8) free(m);
        return FWI_ERR_NOMEM;
    }
    rc = read_f32(vp_path, f, n);
    if (rc == FWI_OK) rc = read_f32(eps_path, f + n, n);
    if (rc == FWI_OK) rc = read_f32(delta_path, f + 2 * n, n);
    if (rc == FWI_OK) {
        if (elem == 8)
            for (size_t i = 0; i < 3 * n; i++) ((double *)m)[i] = (double)f[i];
        rc = fwi_set_model_vti(ctx, m, (char *)m + n * elem, (char *)m + 2 * n * elem);
    }
    if (elem == 8) free(m);
    free(f);
    return rc;
}

int fwi_save_model_files(void *ctx, const char *vh_path, const char *vp_path, const char *vn_path)
{
    fwi_config cfg;
    int rc = fwi_get_config(ctx, &cfg);
    if (rc != FWI_OK) return rc;
    const size_t n = (size_t)cfg.nx * (size_t)cfg.nz;
    const size_t elem = cfg.precision == FWI_PREC_FP64 ? 8 : 4;
    void *m = malloc(3 * n * elem);
    float *f = (float *)malloc(3 * n * sizeof(float));
    if (!m || !f) {
        free(m);
        free(f);
        return FWI_ERR_NOMEM;
    }
    rc = fwi_get_model(ctx, m, (char *)m + n * elem, (char *)m + 2 * n * elem);
    if (rc == FWI_OK) {
        for (size_t i = 0; i < 3 * n; i++) f[i] = elem == 8 ? (float)((double *)m)[i] : ((float *)m)[i];
        rc = write_f32(vh_path, f, n);
        if (rc == FWI_OK) rc = write_f32(vp_path, f + n, n);
        if (rc == FWI_OK) rc = write_f32(vn_path, f + 2 * n, n);
    }
    free(m);
    free(f);
    return rc;
}
