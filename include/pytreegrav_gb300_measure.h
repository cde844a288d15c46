/*
 * pytreegrav_gb300 measurement utilities (not part of the pytreegrav boundary; used by bench.py).
 */
#ifndef PYTREEGRAV_GB300_MEASURE_H
#define PYTREEGRAV_GB300_MEASURE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Traversal steps (warp-wide stack pops) of the last walk on a tree (opaque tg_tree handle). */
int64_t tg_tree_last_walk_steps(void *tree);

/* Quadrupole node interactions (target-node pairs) of the last walk on a tree. */
int64_t tg_tree_last_walk_quad_interactions(void *tree);

/* Device time of the last walk's kernel launch on a tree (CUDA events on the launching stream). */
double tg_tree_last_walk_kernel_ms(void *tree);

/* Kernels this library has launched since it was loaded (all entry points, all streams). */
int64_t tg_launch_count(void);

/* FP32 CUDA-core throughput of this GPU, measured: a grid of FFMA chains (8 independent chains per
 * thread, every SM saturated) timed with CUDA events on `stream`. Writes TFLOP/s (2 flops per FMA)
 * and the kernel's duration. */
int tg_measure_fp32_fma(double *tflops, double *ms, void *stream);

/* Self-check of the library's integer binary64 -> binary32 conversions (used where kernels repack
 * FP64 tree data as FP32) against the GPU's own conversion: for each of the n doubles at x (device
 * memory, finite or not) float(x), and the split hi = float(x), lo = float(x - hi), are compared bit
 * for bit (NaN results: NaN on both sides). *mismatches receives the count of differing values. */
int tg_check_f32_conversion(const double *x, int64_t n, int64_t *mismatches, void *stream);

/* Bounds of the library's bounded device loops, for tests that make each one run out (0 or less:
 * the built-in bound): polls of one look-back word in a radix pass (built in: 2^22; running out
 * gives TG_ERR_QUEUE_TIMEOUT), traversal steps of one group of a tree walk (the node count, which
 * always suffices; TG_ERR_ITER_LIMIT), element visits of one column-density walk (the element count;
 * TG_ERR_ITER_LIMIT), and list entries after which a group of a plain walk is split across warps
 * (2^15; results stay within rounding). Every loop stays in bounds when its limit runs out, and the
 * library stays usable. Process-wide, read when a call launches its kernels; not for concurrent
 * use with other calls. Returns 0. */
int tg_set_loop_limits(int64_t sort_spin, int64_t walk_steps, int64_t column_visits, int64_t heavy_entries);

#ifdef __cplusplus
}
#endif
#endif
