/* Learned opening angle for the grouped walk: per-group features, a 16-64-64-1 MLP trained with
 * the library's own forward, backward and Adam kernels, BF16 tensor-core inference, and a walk
 * that takes one opening angle per group from the network.
 *
 * None of these entries has a counterpart in pytreegrav, which uses one global theta. They work on
 * the tree grouping (TG_GROUP_TREE, TG_ORDER_TREE) of single-system trees; all arrays are device
 * arrays unless a `mem` argument says otherwise, and all calls are stream-ordered on `stream`. */
#ifndef PYTREEGRAV_GB300_THETA_H
#define PYTREEGRAV_GB300_THETA_H

#include "pytreegrav_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TG_THETA_NFEAT 16 /* features per group */
#define TG_MLP_H 64       /* hidden width */
/* FP32 parameters, one flat array: W1 (64 x 16, row-major), b1 (64), W2 (64 x 64), b2 (64),
 * W3 (64), b3 (1). */
#define TG_MLP_NPARAM (TG_MLP_H * TG_THETA_NFEAT + TG_MLP_H + TG_MLP_H * TG_MLP_H + TG_MLP_H + TG_MLP_H + 1)
/* Index of the feature that carries log10(lambda), the weight of force error against cost. */
#define TG_THETA_FEAT_LAMBDA 13

/* Number of groups of the tree grouping at group_size (made and kept on the tree if needed). */
tg_status tg_tree_groups(tg_tree tree, int group_size, int64_t *ngroups, void *stream);

/* The groups: first target (walk order), target count, and the node whose subtree holds the group;
 * int32 arrays of ngroups (any may be NULL), host or device per mem. */
tg_status tg_tree_groups_copy(tg_tree tree, int group_size, int32_t *first, int32_t *count,
                              int32_t *node, int mem, void *stream);

/* While enabled, every tg_tree_fields / tg_tree_fields_learned call records per-group counters:
 * list entries evaluated as point masses, entries evaluated as quadrupole nodes, nodes tested. */
tg_status tg_tree_record_group_stats(tg_tree tree, int enable);

/* Counters of the last walk, ngroups x 3 uint32 (host or device per mem). */
tg_status tg_tree_last_group_stats(tg_tree tree, uint32_t *out, int mem, void *stream);

/* Each group's estimated relative truncation error in the last walk with per-group tolerances
 * (recorded while tg_tree_record_group_stats is on), ngroups float32: the sum, over the nodes the
 * group accepted, of M s^p / (r - delta)^(p+2) (p = 3 with quadrupoles, 2 without; r the node's
 * distance from the group box), divided by the RMS acceleration of the group's targets. */
tg_status tg_tree_last_group_error(tg_tree tree, float *out, int mem, void *stream);

/* Per-group features, ngroups x TG_THETA_NFEAT float32 (device): group size and extent, the
 * mass, size and density of the node holding the group, its distance from the system centre, the
 * field of the tree's top three levels at the group (sum of m/r^2, |sum of m r/r^3|, sum of m/r,
 * and their ratio), the largest softening, box shape and spacing, log10(lambda) (set to 0 here;
 * tg_theta_infer fills it), the quadrupole flag and log10 N. */
tg_status tg_theta_features(tg_tree tree, int group_size, int quadrupole, float *features, void *stream);

/* ---- training kernels (FP32) ---- */

/* Forward pass of n samples: x (n x 16) -> y (n), the pre-sigmoid output. acts (n x 128) keeps
 * both hidden layers' pre-activations for tg_mlp_backward (may be NULL when not training). */
tg_status tg_mlp_forward(const float *params, const float *x, int64_t n, float *acts, float *y, void *stream);

/* Gradient of sum_i dy_i * y_i with respect to params, written to grad (TG_MLP_NPARAM floats).
 * work: n x 128 floats of scratch. */
tg_status tg_mlp_backward(const float *params, const float *x, const float *acts, const float *dy, int64_t n,
                          float *work, float *grad, void *stream);

/* One Adam step (bias-corrected, step counted from 1) on nparam parameters. */
tg_status tg_adam_step(float *params, const float *grad, float *m, float *v, int64_t nparam, float lr, float beta1,
                       float beta2, float eps, int step, void *stream);

/* Opening-angle loss of n samples. Each sample carries cost and log-error tables over a theta grid
 * (ngrid values theta_lo + k * theta_step, rows of ngrid floats: log cost, log error), and a
 * weight lambda. theta = theta_min + (theta_max - theta_min) * sigmoid(y); the loss is
 * mean_i [cost_i(theta_i) + lambda_i * err_i(theta_i)], both interpolated linearly in log space.
 * Writes d loss / d y_i to dy and adds the loss to *loss_sum (one float, device). */
tg_status tg_theta_loss(const float *y, const float *log_cost, const float *log_err, const float *lambda, int64_t n,
                        int ngrid, float theta_lo, float theta_step, float theta_min, float theta_max, float *dy,
                        float *loss_sum, void *stream);

/* Per-group tolerances for the mass-aware test of tg_tree_fields_grouped: tol_g = 10^u_g * A * M / S^2,
 * where M and S are the system's mass and root size and A the mass-weighted RMS of the features'
 * top-level field |sum of m r/r^3| in those units, an estimate of the system's RMS acceleration
 * known before the walk. u: ngroups floats (log10 of the tolerance relative to that estimate). */
tg_status tg_theta_tolerances(tg_tree tree, int group_size, int quadrupole, const float *u, float *tol,
                              void *stream);

/* ---- inference ---- */

/* A model ready for inference: BF16 copies of W1 and W2, FP32 biases and output layer, the feature
 * normalisation (x - mean) / std applied before the first layer, and the output range: the network
 * gives out_min + (out_max - out_min) * sigmoid(y). kind says what the output is: an opening angle
 * per group (TG_THETA_KIND_ANGLE) or u, the log10 relative tolerance of tg_theta_tolerances
 * (TG_THETA_KIND_TOLERANCE), walked with the angle cap theta_max. */
enum { TG_THETA_KIND_ANGLE = 0, TG_THETA_KIND_TOLERANCE = 1 };
typedef struct tg_theta_model_s *tg_theta_model;
tg_status tg_theta_model_create(const float *params, const float *feat_mean, const float *feat_std, int kind,
                                float out_min, float out_max, float theta_max, int mem, tg_theta_model *out);
tg_status tg_theta_model_free(tg_theta_model model);

/* Error budget of a tolerance model (default 0, no check): in tg_tree_fields_learned, a group whose
 * estimated relative truncation error (tg_tree_last_group_error's quantity) exceeds it is walked
 * again at theta_fallback, the global opening angle, and its rows rewritten. */
tg_status tg_theta_model_set_error_budget(tg_theta_model model, float budget);

/* Network output per sample from features (n x 16; feature TG_THETA_FEAT_LAMBDA replaced by
 * log10_lambda): a fused BF16 tensor-core forward pass with FP32 accumulation. */
tg_status tg_theta_infer(tg_theta_model model, const float *features, int64_t n, float log10_lambda, float *out,
                         void *stream);

/* tg_tree_fields (TG_ORDER_TREE, TG_GROUP_TREE, FP32) with per-group control of the acceptance test,
 * in the tree grouping's group order: theta_per_group (NULL: theta for every group) and
 * tol_per_group (NULL: off). A group with tolerance tau > 0 accepts a node of mass M and size s
 * when its distance to the group box, less the node's delta, exceeds both s / theta and
 * (M s^p / tau)^(1/(p+2)), p = 3 with quadrupoles and 2 without (the size of the first neglected
 * multipole term), besides pytreegrav's softening condition. */
tg_status tg_tree_fields_grouped(tg_tree tree, int fields, int quadrupole, double G, int group_size, double theta,
                                 const float *theta_per_group, const float *tol_per_group, int mem, double *out,
                                 void *stream);

/* tg_tree_fields (TG_ORDER_TREE, TG_GROUP_TREE, FP32) with the acceptance test of every group set
 * by the model at weight log10_lambda: its opening angle, or its mass-aware tolerance under the
 * model's angle cap. With model NULL this is the plain walk at theta_fallback, and a group whose
 * output is not finite falls back to it. With a tolerance model whose error budget is set
 * (tg_theta_model_set_error_budget), groups over the budget are walked again at theta_fallback. */
tg_status tg_tree_fields_learned(tg_tree tree, int fields, int quadrupole, double G, int group_size,
                                 tg_theta_model model, float log10_lambda, double theta_fallback, int mem,
                                 double *out, void *stream);

/* The learned acceptance test for external targets (tg_targets_create's groups of the source tree's
 * walk): tg_tree_fields_learned's walk, with each group's features taken from its targets and from
 * the deepest source node holding its box, and the tolerance unit from the RMS of the coarse field
 * at the targets. Groups over the model's error budget are walked again at theta_fallback. */
tg_status tg_targets_fields_learned(tg_targets targets, int fields, int quadrupole, double G, tg_theta_model model,
                                    float log10_lambda, double theta_fallback, int mem, double *out, void *stream);

/* Features of a target set's groups (ngroups x TG_THETA_NFEAT float32, device), as tg_theta_features. */
tg_status tg_targets_features(tg_targets targets, int quadrupole, float *features, void *stream);

/* Per-group tolerances of a target set's groups from u (log10 relative tolerance per group), as
 * tg_theta_tolerances. */
tg_status tg_targets_tolerances(tg_targets targets, int quadrupole, const float *u, float *tol, void *stream);

#ifdef __cplusplus
}
#endif

#endif
