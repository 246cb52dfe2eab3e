/*
 * merc_diag.h - diagnostic entry points of libmerc.so (no reference
 * counterpart: the reference exposes no library).  They let a caller check the
 * device math library against a host evaluation, measure the FP64 FMA peak
 * of the GPU for roofline fractions, and time the kick kernels inside the
 * captured step graph.
 */
#ifndef MERC_DIAG_H
#define MERC_DIAG_H

#include <stdint.h>

#include "merc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Evaluate a merc_math function on the GPU for n inputs: fn 0 sin, 1 cos,
 * 2 atan2(x, y), 3 acos, 4 log, 5 sinh, 6 cosh, 7 cbrt, 8 exp; and the
 * quotients of the Richardson combination: 9 x / 3, 11 x / 15, 12 x / 63 by
 * the known-reciprocal correction, 10 x / y by the division. */
int merc_diag_math(int device, int fn, int64_t n, const double* x, const double* y, double* out);

/* FP64 FMA throughput of the device in TFLOP/s (2 flops per FMA), best of
 * three runs of a register-resident FMA loop over 4 blocks per SM. */
int merc_diag_fp64_peak(int device, double* tflops);

/* Loss and gradient of the warm-start network on n samples (5 floats each,
 * as logged) with parameter blob `blob` (MERC_MLP_BLOB floats): loss = mean of
 * 0.5 (net - target)^2 in normalised units; grad: the 1249 network parameters. */
int merc_diag_mlp_grad(int device, int64_t n, const float* samples, const float* blob, float* loss, float* grad);

/* Warm-start guess and FP64 solve for n drift inputs (pos/vel 3 x n,
 * component-major): blob NULL gives the plain guess dt / r0. */
int merc_diag_warm_start(int device, int64_t n, const double* pos, const double* vel, double dt, const float* blob,
                         double tol, int32_t max_iter, double* guess, double* solved, int32_t* iters);

/* Write `bytes` of a scratch buffer on the context's stream (evicts L2 between
 * timed steps) and wait for it. */
int merc_diag_flush_l2(merc_ctx* ctx, int64_t bytes);

/* on != 0: record CUDA events around each kick kernel when the step graph is
 * next captured.  merc_diag_kick_ms returns the mean kick duration of the
 * most recent graph replay and the number of kick launches it averaged. */
int merc_diag_time_kicks(merc_ctx* ctx, int on);
int merc_diag_kick_ms(merc_ctx* ctx, double* avg_ms, int32_t* n_launches);

/* on != 0: record CUDA events around the big systems' encounter sub-step
 * kernel when the step graph is next captured.  merc_diag_encounter_ms
 * returns its mean duration over the most recent graph replays and the number
 * of launches it averaged. */
int merc_diag_time_encounter(merc_ctx* ctx, int on);
int merc_diag_encounter_ms(merc_ctx* ctx, double* avg_ms, int32_t* n_launches);

/* Kicks of big systems sum the far field once for the two kicks around a step
 * boundary inside a step graph; when a source's far-field radius moved between
 * them (orbits with e > 1/3) the second far-field pass runs.  *count: how many
 * such passes ran since the load. */
int merc_diag_far_recomputes(merc_ctx* ctx, int64_t* count);

/* on != 0 (the default): the kernels of the step graphs are launched as
 * programmatic dependent launches (scheduled while the previous kernel
 * finishes; each waits for it before touching memory).  Results do not
 * depend on it.  Takes effect when the step graphs are next captured. */
int merc_diag_pdl(merc_ctx* ctx, int on);

/* Check of the bounded waits of the encounter sub-step (big systems): runs the
 * encounter task kernel once for the first body of the first big system with
 * the tasks of its first evaluation of row 2 skipped, so the later
 * evaluations of that row wait for a state that is never published, with a
 * short wait limit.  *gave_up = 1 when the kernel reported that a wait gave up
 * (the expected outcome).  The body's state is not touched; the step state
 * of the encounter kernel is cleared afterwards.  MERC_ERR_STATE without a
 * loaded big system. */
int merc_diag_encounter_wait(merc_ctx* ctx, int32_t* gave_up);

#ifdef __cplusplus
}
#endif
#endif /* MERC_DIAG_H */
