/*
 * fwi.h -- native C-ABI of the GB300 (sm_103a) VTI FWI gradient library.
 *
 * One context owns every device buffer of the path.  Shots are a batch
 * dimension: fwi_gradient() runs all shots of a call through one sequence of
 * batched launches (forward, residual + misfit, adjoint + imaging, reduction)
 * instead of the reference's one-shot-per-MPI-rank loop (src/main.c:408-496).
 *
 * Physics and grid are the reference's (src/parallelcalls.cu): 8th-order
 * pseudo-acoustic VTI leapfrog on the coupled fields P, F; CPML on the left,
 * right and bottom edges (none at the top); a 4-point zero frame on every
 * edge; arrays [nz][nx], x fastest.  Models are the squared velocities
 * v_hor = Vp^2 (1 + 2 eps), v_po = Vp^2, v_nmo = Vp^2 (1 + 2 delta).
 *
 * Element type of every array argument: float for FWI_PREC_FP32 contexts,
 * double for FWI_PREC_FP64 contexts.  Pointers may be host or device memory
 * (detected per call); host buffers are staged through the context.
 *
 * Every function returns FWI_OK (0) or a negative FWI_ERR_* status.
 */
#ifndef FWI_H
#define FWI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FWI_OK 0
#define FWI_ERR_ARG (-1)       /* invalid argument or geometry */
#define FWI_ERR_CUDA (-2)      /* a CUDA call failed (details: fwi_last_cuda_error) */
#define FWI_ERR_NOMEM (-3)     /* device memory for the requested batch does not fit (or a host buffer) */
#define FWI_ERR_STATE (-4)     /* call out of order (e.g. no model set) */
#define FWI_ERR_NUMERIC (-5)   /* NaN/Inf met, or reduced-precision storage saturated */
#define FWI_ERR_UNSUPPORTED (-6)
#define FWI_ERR_NODEVICE (-7)  /* no CUDA device, or not an sm_103 device */

/* Adjoint / imaging semantics of fwi_gradient(). */
#define FWI_MODE_REF_COMPAT 0 /* the reference's gradient, src/main.c:408-496: its CPML adjoint
                                 (src/parallelcalls.cu:179-243), forward image of the step
                                 before the one the adjoint pairs with (the snapshot taken
                                 before the update, src/serialcalls.cu:60), scale dt */
#define FWI_MODE_EXACT 1      /* the exact discrete adjoint of the forward step including the
                                 CPML memory variables: dJ/dv_hor, dJ/dv_po, dJ/dv_nmo of
                                 J = 1/2 sum mask (d - d_obs)^2 */

#define FWI_PREC_FP32 0
#define FWI_PREC_FP64 1

/* How the forward images that the imaging condition needs are kept. */
#define FWI_STORE_FULL 0       /* every step, in HBM */
#define FWI_STORE_CHECKPOINT 1 /* full states every ckpt_every steps; segments recomputed */
#define FWI_STORE_BOUNDARY 2   /* the ring of the state around the region the CPML layers do not
                                  touch, every step; that region rebuilt backwards in time during
                                  the adjoint (FP rounding: approximate), gradient zero in the layers */

/* Element type of stored images (per-snapshot scaled for FP16). */
#define FWI_SPREC_NATIVE 0 /* same as the compute precision */
#define FWI_SPREC_FP16 1
#define FWI_SPREC_BF16 2

typedef struct {
    int nx, nz;       /* grid points including the 4-point frame (src/main.c:39-40) */
    float dh, dt;     /* grid step (m) and time step (s) */
    int cpml;         /* absorbing layer width in points (src/main.c:38) */
    float f_cpml;     /* frequency (Hz) in the CPML alpha term (src/parallelcalls.cu:25) */
    float vmax;       /* CPML velocity, 6000 in the reference (src/main.c:51) */
    float r_coef;     /* CPML reflection coefficient, 1e-6 (src/main.c:48) */
    int nt_max;       /* longest shot (time steps) */
    int max_shots;    /* shots resident on the device at once */
    int max_window;   /* widest shot aperture in columns (0 = nx) */
    int max_receivers;/* most receivers of one shot (0 = max_window) */
    int mode;         /* FWI_MODE_* */
    int precision;    /* FWI_PREC_* */
    int store;        /* FWI_STORE_* */
    int store_prec;   /* FWI_SPREC_* */
    int ckpt_every;   /* checkpoint interval for FWI_STORE_CHECKPOINT (0 = automatic: the least
                         memory; a longer one recomputes fewer steps); >= 0 */
    int device;       /* CUDA device ordinal, >= 0 */
} fwi_config;

/* One shot.  Coordinates are 0-based model grid points.  The simulation grid
 * of the shot is the model's columns [x0, x0 + nxw) (all rows) with its own
 * frame and CPML layers at the window edges; nxw = 0 means the whole model.
 * The source (sx, sz) and the receivers (row rz, columns [rx0, rx1)) must lie
 * inside the window's updated interior.  The reference's geometry is
 * sx = posShots[i] - 1, sz = rz = 4 (sz - 1 with sz = 5), rx = [CPML, nx - CPML)
 * (src/main.c:45-46, 260-262; src/parallelcalls.cu:107-116). */
typedef struct {
    int sx, sz;
    int rz, rx0, rx1;
    int nt;
    int x0, nxw;
} fwi_shot;

/* Defaults: the reference's constants (src/main.c:38-52) on a 201 x 201 grid. */
void fwi_config_default(fwi_config *cfg);

/* Device bytes a context with this configuration allocates. */
size_t fwi_config_bytes(const fwi_config *cfg);

int fwi_create(const fwi_config *cfg, void **ctx_out);
void fwi_destroy(void *ctx);

/* The configuration a context was created with. */
int fwi_get_config(void *ctx, fwi_config *out);
const char *fwi_strerror(int status);
/* The cudaError_t behind the last FWI_ERR_CUDA of this context (0 if none). */
int fwi_last_cuda_error(void *ctx);

/* Models as squared velocities [nz][nx].  Replaces src/serialcalls.cu:17-21 when given
 * (Vp, epsilon, delta) through fwi_set_model_vti. */
int fwi_set_model(void *ctx, const void *v_hor, const void *v_po, const void *v_nmo);
int fwi_set_model_vti(void *ctx, const void *vp, const void *eps, const void *delta);
int fwi_get_model(void *ctx, void *v_hor, void *v_po, void *v_nmo);

/* Source wavelet shared by all shots, nt samples (src/main.c:328-333 makes a Ricker). */
int fwi_set_wavelet(void *ctx, const void *wavelet, int nt);
/* Ricker wavelet of src/main.c:328-332 with peak frequency f. */
int fwi_set_ricker(void *ctx, float f, int nt);

/* Forward modelling (src/main.c:334-366).  traces: per shot, [nt][rx1 - rx0], shots
 * concatenated in order. */
int fwi_forward(void *ctx, const fwi_shot *shots, int nshots, void *traces);

/* Misfit J = 1/2 sum mask (d - obs)^2 (FP64) and, with gradients requested,
 * dJ/dv_hor, dJ/dv_po, dJ/dv_nmo summed over the shots, [nz][nx] each
 * (src/main.c:408-534 with the MPI reduction replaced by an on-device sum).
 * obs: per shot [nt][nrec], concatenated; NULL: the records kept on the device (below).  mask: per shot [nrec] bytes
 * (0 = dropped trace), concatenated, or NULL.  g_* may be NULL (the gradient
 * then stays in the context for the L-BFGS calls below). */
int fwi_gradient(void *ctx, const fwi_shot *shots, int nshots, const void *obs,
                 const unsigned char *mask, void *g_vh, void *g_vp, void *g_vn, double *misfit);

/* ---- observed data kept on the device ----
 * The reference re-models its observed data from the true model for every frequency band
 * (src/main.c:321-366) and keeps the records of all shots in device memory (shot1,
 * src/main.c:168).  fwi_store_observed copies given records (host or device, laid out as
 * fwi_gradient takes them) into a store inside the context; fwi_model_observed models them
 * there from the given model (squared velocities [nz][nx]) with fwi_forward's arithmetic, without
 * a host copy, and keeps the context's own model.  store_prec FWI_SPREC_NATIVE keeps the records
 * as they are (4 B per sample in FP32 contexts: 65.5 GB for 512 shots of 8000 x 4001); FWI_SPREC_FP16
 * keeps 2 B per sample with one scale per trace (max |d| / 32768), a relative error of about 2^-12
 * of each trace's largest value.  Later fwi_gradient / fwi_misfit calls (and fwi_invert,
 * fwi_invert_bands) with obs == NULL on the same shots, in the same order, read the store
 * (FWI_ERR_ARG for other shots).  fwi_free_observed releases it.  No counterpart in the reference's
 * call surface. */
int fwi_store_observed(void *ctx, const fwi_shot *shots, int nshots, const void *obs, int store_prec);
int fwi_model_observed(void *ctx, const fwi_shot *shots, int nshots, const void *v_hor, const void *v_po,
                       const void *v_nmo, int store_prec);
int fwi_free_observed(void *ctx);

/* Misfit only (forward + residual), e.g. for line-search trials (src/main.c:695-737). */
int fwi_misfit(void *ctx, const fwi_shot *shots, int nshots, const void *obs,
               const unsigned char *mask, double *misfit);

/* Replaces the context's gradient, e.g. with one summed over several processes
 * (the role of src/main.c:510-538's MPI reduction), before the update calls below. */
int fwi_set_gradient(void *ctx, const void *g_vh, const void *g_vp, const void *g_vn);

/* ---- model update: steepest descent and L-BFGS, on the device ----
 * Pairings as src/main.c:573: (v_po, dJ/dv_po), (v_nmo, dJ/dv_nmo), (v_hor, dJ/dv_hor),
 * each with its own scalars.  Dot products accumulate in FP64. */

/* First iteration (src/main.c:539-568): normalise each gradient by its L2 norm below
 * the near-surface layer and step the model by (a_hor, a_po, a_nmo).  Keeps the model
 * and gradient as the pair the next direction differences against. */
int fwi_first_step(void *ctx, float a_hor, float a_po, float a_nmo);

/* L-BFGS two-loop direction (src/main.c:569-682, memory m <= 16) from the last gradient.
 * stats (optional, 12 doubles, order v_hor, v_po, v_nmo): gamma[3], 1/(y.s)[3], y.s[3], y.y[3]
 * of the newest pair. */
int fwi_lbfgs_direction(void *ctx, int m, double *stats);

/* Curvature safeguard of the two-loop recursion (no counterpart in the reference, whose
 * two-loop uses every pair: src/main.c:574-681).  With on != 0, later directions skip, per
 * parameter, every history pair whose y.s <= 0 (the gradient did not grow along the step, so
 * the pair carries no positive curvature and 1/(y.s) would turn the direction uphill), and
 * scale the initial matrix by the newest pair with y.s > 0, or by |s| / |y| of the newest pair
 * when there is none.  0 (the default) reproduces the reference. */
int fwi_set_lbfgs_guard(void *ctx, int on);

/* Trial model m = m_back - alpha r below the layer, optional clamps, v_hor >= v_nmo
 * (src/parallelcalls.cu:343-404). */
int fwi_lbfgs_update(void *ctx, float alpha_v, float alpha_d, float alpha_e, int flag_min,
                     int flag_max);

/* Model back to m_back (src/main.c:777-784). */
int fwi_restore_model(void *ctx);

/* Directional derivative along the last L-BFGS direction r from (m_back, g_back):
 * out[p] = sum over the rows fwi_lbfgs_update changes of g_back . r, FP64, order v_hor,
 * v_po, v_nmo.  The trial m_back - alpha r changes the misfit by about -alpha sum(out).
 * No counterpart in the reference (its line search compares misfits only). */
int fwi_direction_slope(void *ctx, double *out3);

/* ---- host driver (C) ----
 * One frequency band of the reference's inversion loop (src/main.c:396-801) over the calls
 * above: steepest first step, then L-BFGS directions with the backtracking line search
 * (halve alpha on a NaN misfit or one above the iteration's; more than max_halvings
 * halvings restore the model and end the band).  misfit_history (optional) receives the
 * misfit of each iteration's gradient. */
typedef struct {
    int iterations;       /* src/main.c:12: 100 */
    int lbfgs_m;          /* src/main.c:59: 5 */
    float first_alpha[3]; /* steepest-descent lengths for v_hor, v_po, v_nmo (src/main.c:567) */
    float alpha0;         /* first L-BFGS step length (src/main.c:62: 1) */
    int max_halvings;     /* src/main.c:777: 5 */
    int reset_alpha;      /* 0: alpha and the halving count persist over the band, as the reference */
    int flag_min, flag_max; /* clamps of update_LBFGS (src/parallelcalls.cu:343-404) */
    double armijo_c1;     /* 0: the reference's acceptance (trial misfit below the iteration's);
                             > 0: also J_trial <= J - c1 alpha sum(fwi_direction_slope), FP64 */
    int curvature_guard;  /* fwi_set_lbfgs_guard for the band's directions (0: the reference's
                             two-loop, every pair) */
} fwi_invert_opts;

void fwi_invert_defaults(fwi_invert_opts *opts);
int fwi_invert(void *ctx, const fwi_shot *shots, int nshots, const void *obs,
               const unsigned char *mask, const fwi_invert_opts *opts, double *misfit_history,
               int *iterations_done);

/* Next frequency band (src/main.c:318-319, 328-333, 802): CPML profiles for peak
 * frequency f and a Ricker wavelet of nt samples at f. */
int fwi_set_frequency(void *ctx, float f, int nt);

/* Multiscale inversion (src/main.c:274-806): band b at peak frequency f0 + b df
 * (the reference: f += 3).  Per band: fwi_set_frequency(f, nt); the band's observed data
 * from band_obs (the caller's records, or its own forward modelling with
 * fwi_forward), host or device, laid out as fwi_gradient takes them, or NULL when the
 * callback left them in the context's store (fwi_model_observed: re-modelled on the device at
 * the band's frequency); then fwi_invert with
 * alpha and the halving count starting afresh (src/main.c:308-311).  restart_model != 0
 * starts every band from the model the call began with, as the reference does (it
 * rebuilds the model from the initial Vp, eps, delta at src/main.c:318); 0 continues from
 * the previous band.  misfit_history: nbands x opts->iterations (optional);
 * iterations_done: nbands (optional). */
typedef int (*fwi_band_obs_fn)(void *user, int band, float f, const void **obs);
int fwi_invert_bands(void *ctx, const fwi_shot *shots, int nshots, const unsigned char *mask, float f0,
                     float df, int nbands, int nt, fwi_band_obs_fn band_obs, void *user,
                     const fwi_invert_opts *opts, int restart_model, double *misfit_history,
                     int *iterations_done);

/* ---- model files (src/main.c:101-123, 823-835) ----
 * Raw float32 [nz][nx], x fastest, no header.  fwi_load_model_files reads Vp (m/s),
 * epsilon and delta (the reference's vp_ori.bin, vh_ori.bin, vn_ori.bin) into the model
 * (fwi_set_model_vti); fwi_save_model_files writes the squared velocities v_hor, v_po,
 * v_nmo (the reference's vh_ini.bin, vp_ini.bin, vn_ini.bin).  FWI_ERR_ARG on a missing
 * or short file. */
int fwi_load_model_files(void *ctx, const char *vp_path, const char *eps_path, const char *delta_path);
int fwi_save_model_files(void *ctx, const char *vh_path, const char *vp_path, const char *vn_path);

/* Chain rule to the Vp / epsilon / delta parameterisation of the current model:
 * dJ/dVp = 2 Vp (g_po + (1 + 2 eps) g_hor + (1 + 2 delta) g_nmo),
 * dJ/deps = 2 Vp^2 g_hor, dJ/ddelta = 2 Vp^2 g_nmo (outputs [nz][nx]). */
int fwi_gradient_vti(void *ctx, void *g_vp, void *g_eps, void *g_delta);

/* Timing of the last fwi_gradient / fwi_misfit / fwi_forward call (device time, ms):
 * out[0] total, out[1] forward, out[2] adjoint, out[3] other. */
int fwi_last_timing(void *ctx, float *out4);

/* Per-launch timing of the interior tile kernels (no counterpart in the
 * reference).  With on != 0, later fwi_gradient / fwi_misfit / fwi_forward
 * calls record CUDA events on the launching stream around the interior tile
 * launch of up to 16 sampled time steps per phase (FP32 contexts only).
 * fwi_last_tile_timing: out[0] mean forward launch duration (ms), out[1]
 * interior points it updated (summed over the batch's shots), out[2], out[3]
 * the same for the adjoint; zeros when nothing was sampled. */
int fwi_set_tile_timing(void *ctx, int on);
int fwi_last_tile_timing(void *ctx, double *out4);
/* With checkpoint storage the adjoint section also runs the forward steps of
 * each segment's recompute (beside the adjoint steps, on their own streams):
 * out[0] mean duration (ms) of their sampled interior tile launches, out[1]
 * interior points such a launch updated, out[2] forward steps the last call
 * recomputed (zeros without checkpoint storage or samples). */
int fwi_last_recompute_timing(void *ctx, double *out3);

/* How many of this library's kernels the last call launched. */
long fwi_last_launches(void *ctx);

/* Autotuner (no counterpart in the reference).  The FP32 tile passes have a
 * fixed 32 x 32 point tile (the TMA box and four points per thread); what
 * shapes their work is how many shots one block takes through the tile (the
 * interior and the layer tile passes separately; a layer block takes more
 * than one only when every shot of the batch has one window, an interior
 * block also from several windows) and whether the layer tiles advance the
 * CPML memory variables themselves or after a strip pass; the forward and
 * the adjoint are chosen separately.  fwi_autotune times `steps` steps of
 * candidate choices of each phase for each batch the shots form (coordinate
 * descent from the built-in choice, then every pair of group sizes near the
 * best; each candidate timed three times, the median kept; a candidate must
 * be 1 % faster to replace it) and records the fastest per batch shape (shots in the batch,
 * widest window, one window or several, mode, image type); later
 * fwi_gradient / fwi_misfit / fwi_forward calls on batches of that shape use
 * it.  Results stay within FP32 rounding of the built-in choice's; for a
 * given choice they are deterministic.  `out` (may be NULL): the first
 * batch's choice and its device time per step, beside the built-in one's.
 * Time blocking (several steps per pass) is not implemented: one step per
 * pass. */
typedef struct {
    int shots_per_group;        /* shots per block, interior tile passes */
    int layer_shots_per_group;  /* shots per block, layer tile passes */
    int inline_strip;           /* 1: layer tiles advance the CPML memory variables; 0: strip pass first */
} fwi_phase_choice;
typedef struct {
    fwi_phase_choice forward, adjoint;
    int trials;                                   /* candidate runs timed */
    double forward_us, adjoint_us;                /* device time per step with the choice (us) */
    double default_forward_us, default_adjoint_us;/* the same with the built-in choice */
} fwi_tuning;
int fwi_autotune(void *ctx, const fwi_shot *shots, int nshots, int steps, fwi_tuning *out);
/* Records t's choice (forward, adjoint) for the batch shapes the shots form,
 * as fwi_autotune does: a choice tuned once, kept and given again gives the
 * same results bit for bit.  FWI_ERR_ARG when it does not fit: a group size
 * outside 1..64, or a layer group above 1 for a batch of several windows. */
int fwi_set_tuning(void *ctx, const fwi_shot *shots, int nshots, const fwi_tuning *t);

/* Check of the device-side failure path (no counterpart in the reference):
 * one block waits, as the tile passes wait for their staged tiles, on a
 * barrier phase that nothing completes, gives up after `polls` polls
 * (1 .. 4194304, the tile passes' own limit) and records the timeout in the
 * context's status word.  Returns FWI_ERR_CUDA when the timeout was seen,
 * as a gradient call would after a wait that gave up; the context stays
 * usable.  No fault, trap or unbounded wait is involved. */
int fwi_check_bounded_wait(void *ctx, long polls);

/* CUDA graphs (no counterpart in the reference, which launches every kernel
 * from the host).  A batch of fwi_gradient / fwi_misfit / fwi_forward runs as
 * two sections: the forward steps, and the adjoint with its image rebuild and
 * the gradient sum.  A section whose launch parameters (batch size, steps,
 * storage, each shot's steps and window width) repeat is captured into a
 * CUDA graph the second time and replayed after that: one launch from the
 * host instead of several per time step, same kernels, same results.  On by
 * default (environment FWI_GRAPHS=0 at fwi_create: off).  fwi_set_graphs(ctx,
 * 0) turns graphs off and frees them.  fwi_graph_stats: out[0] sections
 * replayed, out[1] sections captured, both since fwi_create. */
int fwi_set_graphs(void *ctx, int on);
int fwi_graph_stats(void *ctx, long *out2);

/* ---- residual and misfit without device allocation ----
 * No counterpart in the reference (it copies the residual to the host and sums it there,
 * src/main.c:437-454).  For callers that cannot let the library allocate device memory:
 * drivers shaped like src/main.c that allocate every buffer once before the shot loop, or
 * processes whose device memory is owned by another allocator with a fixed budget.
 * res = mask (syn - obs) over an [nt][nrec] block of FP32 traces (mask: [nrec] bytes,
 * 0 = dropped trace, or NULL) and *misfit = 1/2 sum res^2 accumulated in FP64, in a fixed
 * order.  All pointers are device pointers (misfit: one double); the work is ordered on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and nothing is waited for.
 * Scratch is a fixed array inside the library (FWI_NOALLOC_MAX_BLOCKS + 1 doubles per
 * device, held until the process exits); it limits nt * nrec to FWI_NOALLOC_MAX_ELEMENTS
 * (larger requests return FWI_ERR_ARG).  Every call shares that array, so calls that
 * overlap on the GPU (other streams, other threads) race; serialise them.  Each call looks
 * up the array's device address on the current device (cudaGetSymbolAddress); the first
 * call on a device also loads the library's module there, so make it before any stream
 * capture.  The mask is ONE row of nrec bytes applied to every one of the nt trace rows
 * (fwi_misfit takes one row per shot, concatenated): pass a block of shots that share it. */
#define FWI_NOALLOC_MAX_BLOCKS 16384
#define FWI_NOALLOC_MAX_ELEMENTS (16384L * 4096L)
int fwi_residual_misfit_noalloc(float *res, const float *syn, const float *obs,
                                const unsigned char *mask, long nt, int nrec, double *misfit,
                                void *stream);

/* Host-side helper, no GPU needed: the CPML strip points of an nx x nz grid
 * (the points src/parallelcalls.cu:55 updates), in the order the strip kernels
 * visit them.  Returns the count; writes at most cap pairs. */
long fwi_strip_points(int nx, int nz, int cpml, int *ix, int *iz, long cap);

#ifdef __cplusplus
}
#endif
#endif
