/*
 * sw4g_dev -- developer and measurement hooks of libsw4g.so.
 *
 * Not part of the drop-in boundary (include/sw4g.h): these calls serve the
 * benchmark, launch-shape sweeps and tests.  A caller replacing sw4lite's time
 * loop needs none of them.
 */
#ifndef SW4G_DEV_H
#define SW4G_DEV_H

#include "sw4g.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-kernel device time of a fused step (CUDA events on the EW stream), each
 * piece launched nrep times on the current levels without advancing time; the
 * counterpart of the reference's phase timers (src/EW.C:2863-2873, reporttiming):
 * ms[0] predictor stage kernel, ms[1] corrector stage kernel, ms[2] one-sided
 * rows, ms[3] boundary conditions and forcing.  Synchronises the stream. */
int sw4g_ew_profile_kernels(sw4g_ew* ew, int nrep, double* ms);

/* Tuning (no reference counterpart): the number of k chunks every stage kernel
 * splits its planes into, for all objects of the process; 0 restores the automatic
 * choice (the count that fills the GPU's SMs in whole waves). */
int sw4g_dev_set_stage_chunks(int chunks);
/* Comparison switch (no reference counterpart): 1 (the default) runs the FP32-mixed
 * predictor and corrector stages on the tensor-copy kernels wherever the array
 * strides allow, 0 on the synchronous kernels; for all objects of the process. */
int sw4g_dev_set_mixed_tma(int on);
/* Comparison switch (no reference counterpart): 1 (the default) runs the one-sided
 * rows next to a free surface on a second stream beside each fused stage kernel, 0
 * after it on the object's stream; for all objects of the process. */
int sw4g_dev_set_rows_overlap(int on);
/* Comparison switch (no reference counterpart): 1 (the default) lets sw4g_ew_gradient
 * recompute the next segment beside the current segment's adjoint steps (without CUDA
 * graphs, with two or more segments kept), 0 runs them one after the other; for all
 * objects of the process.  Results are the same bits either way. */
int sw4g_dev_set_adjoint_pipeline(int on);
/* Tuning (no reference counterpart): the planes per k chunk that the automatic
 * choice gives a stage kernel of `cols` CTA columns over nk planes with `resident`
 * CTAs per SM on the current device's SMs (152 when no device answers), at least
 * min_planes planes per chunk where nk allows.  Host arithmetic only. */
int sw4g_dev_stage_kchunk(long long cols, int nk, int resident, int min_planes, int* planes);

#ifdef __cplusplus
}
#endif
#endif
