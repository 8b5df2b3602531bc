/* A C99 client of both C-ABIs of the library, as the reference's src/main.c
 * (C99) is one: tests/test_c_client_cpu.py compiles it with gcc -std=c99
 * -Wall -Wextra -Werror (not -pedantic, which CUDA's own headers do not
 * meet), links it against
 * libfwi_gb300.so and runs it.  It calls host-side entry points only (no
 * GPU needed) and takes the address of every compatibility entry point, so
 * that each one must resolve at link time. */
#include "fwi.h"
#include "fwi_compat.h"

#include <stdio.h>

int main(void)
{
    fwi_config cfg;
    size_t bytes;
    typedef void (*entry)(void);
    entry compat[17];
    int i, n = 0;

    fwi_config_default(&cfg);
    cfg.nx = 609;
    cfg.nz = 309;
    cfg.nt_max = 3000;
    cfg.max_shots = 32;
    cfg.store_prec = FWI_SPREC_FP16;
    bytes = fwi_config_bytes(&cfg);

    compat[0] = (entry)pre_variables_h;
    compat[1] = (entry)CPML_x_h;
    compat[2] = (entry)CPML_z_h;
    compat[3] = (entry)PSI_F_h;
    compat[4] = (entry)ZETA_F_h;
    compat[5] = (entry)propagator_F_h;
    compat[6] = (entry)res_h;
    compat[7] = (entry)SecondDerivate_P_h;
    compat[8] = (entry)launchPropagation;
    compat[9] = (entry)launchBackPropagation;
    compat[10] = (entry)NORMAL_h;
    compat[11] = (entry)UpdateModel_h;
    compat[12] = (entry)compute_sy_h;
    compat[13] = (entry)compute_qi_h;
    compat[14] = (entry)compute_ri_h;
    compat[15] = (entry)update_r_h;
    compat[16] = (entry)update_LBFGS_h;
    for (i = 0; i < 17; i++) n += compat[i] != 0;

    printf("bytes %lu compat %d arg \"%s\"\n", (unsigned long)bytes, n, fwi_strerror(FWI_ERR_ARG));
    return bytes > 0 && n == 17 ? 0 : 1;
}
