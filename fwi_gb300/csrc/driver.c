/*
 * Host driver in C over the native C-ABI: one frequency band of the
 * reference's inversion loop (src/main.c:396-801) without MPI.
 *
 *   iteration 0: gradient, then the steepest-descent step with fixed
 *                lengths (src/main.c:539-568);
 *   iteration n: gradient, L-BFGS direction, then backtracking: trial
 *                model m_back - alpha r, misfit of all shots; a NaN misfit
 *                or one above the iteration's misfit halves alpha; more
 *                than max_halvings halvings restore m_back and end the
 *                band (src/main.c:690-786).
 *
 * reset_alpha = 0 keeps the reference's behaviour: alpha and the halving
 * count persist across the iterations of a band (src/main.c:308-311 resets
 * them only per band).
 */
#include "../../include/fwi.h"

#include <math.h>
#include <string.h>

void fwi_invert_defaults(fwi_invert_opts *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->iterations = 100;      /* src/main.c:12 */
    o->lbfgs_m = 5;           /* src/main.c:59 */
    o->first_alpha[0] = 3e5f; /* v_hor, src/main.c:567 */
    o->first_alpha[1] = 2e5f; /* v_po */
    o->first_alpha[2] = 2.5e5f; /* v_nmo */
    o->alpha0 = 1.0f;         /* src/main.c:62 */
    o->max_halvings = 5;      /* src/main.c:777 */
    o->reset_alpha = 0;
    o->flag_min = 0;          /* src/main.c:693 passes 0, 0 */
    o->flag_max = 0;
}

int fwi_invert(void *ctx, const fwi_shot *shots, int nshots, const void *obs, const unsigned char *mask,
               const fwi_invert_opts *opts, double *misfit_history, int *iterations_done)
{
    fwi_invert_opts o;
    if (opts) o = *opts;
    else fwi_invert_defaults(&o);
    if (!ctx || !shots || nshots <= 0 || !obs || o.iterations <= 0) return FWI_ERR_ARG;
    float alpha = o.alpha0;
    int count = 0;
    int done = 0;
    int rc = FWI_OK;
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
        if (o.reset_alpha) {
            alpha = o.alpha0;
            count = 0;
        }
        double trial = 1e10;
        int stop = 0;
        while (trial > phi) {
            rc = fwi_lbfgs_update(ctx, alpha, alpha, alpha, o.flag_min, o.flag_max);
            if (rc != FWI_OK) break;
            rc = fwi_misfit(ctx, shots, nshots, obs, mask, &trial);
            if (rc == FWI_ERR_NUMERIC || isnan(trial)) {
                rc = FWI_OK;
                trial = 1e30;
                count++;
                alpha *= 0.5f;
            } else if (rc != FWI_OK) {
                break;
            } else if (trial > phi) {
                count++;
                alpha *= 0.5f;
            }
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
