/*
 * galax_gb300_bench.h -- measurement entry points of libgalaxcu.so.
 *
 * These serve the benchmark and the profiles, not a caller of the force backend:
 * they have no counterpart in the reference (galax-gpu/src/lib.rs) and are kept
 * out of the product header galax_gb300.h.  Same conventions: plain pointers,
 * a gx_status return, gx_last_error() for the message.
 */
#ifndef GALAX_GB300_BENCH_H
#define GALAX_GB300_BENCH_H
#include "galax_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Runs `reps` force evaluations on the resident bodies and returns the CUDA-event
 * time of each on the context stream (ms) and the time of one kernel of it
 * (`which`: 0 = the P2P kernel, timed on its own stream beside the far-field chain;
 * 1 = the M2L pass; 2 = the P2P kernel started after the far-field chain, so that it
 * runs alone).  With flush_l2 != 0 a 256 MB buffer (twice the L2) is written before
 * each evaluation, outside its timed interval. */
int gx_bench_forces(gx_ctx *ctx, int32_t reps, int32_t flush_l2, double *ms_each, int32_t which,
                    double *kernel_ms_each);
/* FP32 FMA throughput of this GPU in TFLOP/s (best of 5 timed launches of a
 * kernel of independent FMA chains): the ceiling used for the FP32 P2P pass. */
int gx_probe_fp32_tflops(gx_ctx *ctx, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
