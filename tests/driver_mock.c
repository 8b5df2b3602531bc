/* A stand-in for the library's entry points that the C driver
 * (fwi_gb300/csrc/driver.c) calls, so that its inversion policy runs on the
 * CPU: tests/test_driver_cpu.py builds driver.c with this file into one
 * shared object and drives fwi_invert / fwi_invert_bands through ctypes.
 *
 * The "model" is three arrays of nx*nz floats and the misfit the quadratic
 * J(m) = 1/2 |m - t|^2 towards a target t; the gradient is m - t, the first
 * step m -= a g / max|g| per parameter, the L-BFGS direction r = rscale g
 * with m_back = m, the update m = m_back - alpha r.  Controls: trial misfits
 * are NaN for step lengths above nan_above; every trial alpha, band
 * frequency and call is recorded for the test to read. */
#include "fwi.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXREC 256

typedef struct {
    fwi_config cfg;
    int n;
    float *m[3], *back[3], *g[3], *gback[3], *r[3], *t[3];
    float rscale, nan_above;
    float trials[MAXREC];
    int ntrials;
    float freqs[MAXREC];
    int nfreqs;
    int gradients, misfits, restores, first_steps, set_models;
} mock_ctx;

static double quad(const mock_ctx *c)
{
    double j = 0.0;
    for (int p = 0; p < 3; p++)
        for (int i = 0; i < c->n; i++) {
            const double d = (double)c->m[p][i] - (double)c->t[p][i];
            j += 0.5 * d * d;
        }
    return j;
}

void *mock_create(int nx, int nz, float start, float target)
{
    mock_ctx *c = (mock_ctx *)calloc(1, sizeof(mock_ctx));
    if (!c) return NULL;
    c->cfg.nx = nx;
    c->cfg.nz = nz;
    c->cfg.precision = FWI_PREC_FP32;
    c->n = nx * nz;
    c->rscale = 1.0f;
    c->nan_above = INFINITY;
    for (int p = 0; p < 3; p++) {
        float **arr[6] = {&c->m[p], &c->back[p], &c->g[p], &c->gback[p], &c->r[p], &c->t[p]};
        for (int k = 0; k < 6; k++) *arr[k] = (float *)calloc((size_t)c->n, sizeof(float));
        for (int i = 0; i < c->n; i++) {
            c->m[p][i] = start;
            c->t[p][i] = target;
        }
    }
    return c;
}

void mock_free(void *ctx)
{
    mock_ctx *c = (mock_ctx *)ctx;
    if (!c) return;
    for (int p = 0; p < 3; p++) {
        free(c->m[p]); free(c->back[p]); free(c->g[p]); free(c->gback[p]); free(c->r[p]); free(c->t[p]);
    }
    free(c);
}

void mock_set(void *ctx, float rscale, float nan_above)
{
    mock_ctx *c = (mock_ctx *)ctx;
    c->rscale = rscale;
    c->nan_above = nan_above;
}

/* out: trials (up to cap), returns how many */
int mock_trials(void *ctx, float *out, int cap)
{
    const mock_ctx *c = (const mock_ctx *)ctx;
    for (int i = 0; i < c->ntrials && i < cap; i++) out[i] = c->trials[i];
    return c->ntrials;
}

int mock_freqs(void *ctx, float *out, int cap)
{
    const mock_ctx *c = (const mock_ctx *)ctx;
    for (int i = 0; i < c->nfreqs && i < cap; i++) out[i] = c->freqs[i];
    return c->nfreqs;
}

/* gradients, misfits, restores, first steps, set_model calls */
void mock_counts(void *ctx, int *out5)
{
    const mock_ctx *c = (const mock_ctx *)ctx;
    out5[0] = c->gradients;
    out5[1] = c->misfits;
    out5[2] = c->restores;
    out5[3] = c->first_steps;
    out5[4] = c->set_models;
}

float mock_model(void *ctx, int p, int i) { return ((mock_ctx *)ctx)->m[p][i]; }

/* ---- the entry points driver.c calls ---- */

int fwi_get_config(void *ctx, fwi_config *out)
{
    if (!ctx || !out) return FWI_ERR_ARG;
    *out = ((mock_ctx *)ctx)->cfg;
    return FWI_OK;
}

int fwi_get_model(void *ctx, void *a, void *b, void *d)
{
    mock_ctx *c = (mock_ctx *)ctx;
    void *dst[3] = {a, b, d};
    for (int p = 0; p < 3; p++) memcpy(dst[p], c->m[p], (size_t)c->n * sizeof(float));
    return FWI_OK;
}

int fwi_set_model(void *ctx, const void *a, const void *b, const void *d)
{
    mock_ctx *c = (mock_ctx *)ctx;
    const void *src[3] = {a, b, d};
    for (int p = 0; p < 3; p++) memcpy(c->m[p], src[p], (size_t)c->n * sizeof(float));
    c->set_models++;
    return FWI_OK;
}

int fwi_set_model_vti(void *ctx, const void *a, const void *b, const void *d)
{
    return fwi_set_model(ctx, a, b, d);
}

int fwi_set_frequency(void *ctx, float f, int nt)
{
    mock_ctx *c = (mock_ctx *)ctx;
    (void)nt;
    if (c->nfreqs < MAXREC) c->freqs[c->nfreqs++] = f;
    return FWI_OK;
}

int fwi_gradient(void *ctx, const fwi_shot *shots, int nshots, const void *obs, const unsigned char *mask,
                 void *g_vh, void *g_vp, void *g_vn, double *misfit)
{
    mock_ctx *c = (mock_ctx *)ctx;
    (void)shots; (void)nshots; (void)obs; (void)mask; (void)g_vh; (void)g_vp; (void)g_vn;
    for (int p = 0; p < 3; p++)
        for (int i = 0; i < c->n; i++) c->g[p][i] = c->m[p][i] - c->t[p][i];
    c->gradients++;
    if (misfit) *misfit = quad(c);
    return FWI_OK;
}

int fwi_misfit(void *ctx, const fwi_shot *shots, int nshots, const void *obs, const unsigned char *mask,
               double *misfit)
{
    mock_ctx *c = (mock_ctx *)ctx;
    (void)shots; (void)nshots; (void)obs; (void)mask;
    c->misfits++;
    const float last = c->ntrials ? c->trials[c->ntrials - 1] : 0.0f;
    *misfit = last > c->nan_above ? NAN : quad(c);
    return FWI_OK;
}

int fwi_first_step(void *ctx, float a_hor, float a_po, float a_nmo)
{
    mock_ctx *c = (mock_ctx *)ctx;
    const float a[3] = {a_hor, a_po, a_nmo};
    for (int p = 0; p < 3; p++) {
        float mx = 0.0f;
        for (int i = 0; i < c->n; i++) mx = fmaxf(mx, fabsf(c->g[p][i]));
        for (int i = 0; i < c->n; i++) {
            c->back[p][i] = c->m[p][i];
            if (mx > 0.0f) c->m[p][i] -= a[p] * c->g[p][i] / mx;
        }
    }
    c->first_steps++;
    return FWI_OK;
}

int fwi_lbfgs_direction(void *ctx, int m, double *stats)
{
    mock_ctx *c = (mock_ctx *)ctx;
    (void)m; (void)stats;
    for (int p = 0; p < 3; p++)
        for (int i = 0; i < c->n; i++) {
            c->back[p][i] = c->m[p][i];
            c->gback[p][i] = c->g[p][i];
            c->r[p][i] = c->rscale * c->g[p][i];
        }
    return FWI_OK;
}

int fwi_set_lbfgs_guard(void *ctx, int on)
{
    (void)ctx; (void)on;  /* the stand-in's direction is a scaled gradient: no pairs to guard */
    return FWI_OK;
}

int fwi_direction_slope(void *ctx, double *out3)
{
    mock_ctx *c = (mock_ctx *)ctx;
    for (int p = 0; p < 3; p++) {
        out3[p] = 0.0;
        for (int i = 0; i < c->n; i++) out3[p] += (double)c->gback[p][i] * (double)c->r[p][i];
    }
    return FWI_OK;
}

int fwi_lbfgs_update(void *ctx, float av, float ad, float ae, int flag_min, int flag_max)
{
    mock_ctx *c = (mock_ctx *)ctx;
    const float a[3] = {av, ad, ae};
    (void)flag_min; (void)flag_max;
    for (int p = 0; p < 3; p++)
        for (int i = 0; i < c->n; i++) c->m[p][i] = c->back[p][i] - a[p] * c->r[p][i];
    if (c->ntrials < MAXREC) c->trials[c->ntrials++] = av;
    return FWI_OK;
}

int fwi_restore_model(void *ctx)
{
    mock_ctx *c = (mock_ctx *)ctx;
    for (int p = 0; p < 3; p++) memcpy(c->m[p], c->back[p], (size_t)c->n * sizeof(float));
    c->restores++;
    return FWI_OK;
}
