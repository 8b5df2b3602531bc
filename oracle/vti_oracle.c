/*
 * CPU oracle (test infrastructure only; see vti_oracle.h).
 * Instantiates the reference-arithmetic restatement (vti_ref_body.h) and the
 * native-semantics exact-adjoint oracle (vti_exact_body.h) for float and double.
 * Must be compiled with -ffp-contract=off (oracle/Makefile does).
 */
#include "vti_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_D 3.141592653589793 /* include/parallelcalls.h:3 */

static int g_threads = 1;

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)

#define R float
#define SFX _f32
#define FN(name) CAT(name, SFX)
#define POW2(x) powf((x), 2)
#include "vti_ref_body.h"
#include "vti_exact_body.h"
#undef R
#undef SFX
#undef FN
#undef POW2

#define R double
#define SFX _f64
#define FN(name) CAT(name, SFX)
#define POW2(x) pow((x), 2)
#include "vti_ref_body.h"
#include "vti_exact_body.h"
#undef R
#undef SFX
#undef FN
#undef POW2
