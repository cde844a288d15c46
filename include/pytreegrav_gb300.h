/*
 * pytreegrav_gb300 -- C ABI of the GB300 (sm_103a) Barnes-Hut gravity engine.
 *
 * Drop-in boundary for pytreegrav's tree and brute-force paths. Every entry point takes plain
 * pointers and sizes, returns a tg_status, and runs on the CUDA stream passed as `stream`
 * (a cudaStream_t; NULL = the legacy default stream). Arrays are C-contiguous float64:
 * positions (n, 3), masses/softenings (n,), outputs (n, W) packed potential | accel(3) |
 * tidal(9), only the requested fields, in the caller's order.
 *
 * `mem` says where the caller's arrays live: TG_MEM_HOST (pageable or pinned host memory; the
 * library copies in and out on `stream` and synchronises before returning) or TG_MEM_DEVICE
 * (device pointers; the call is asynchronous on `stream` except where noted).
 *
 * Citations name the pytreegrav interface each entry replaces (paths relative to the pytreegrav
 * project).
 */
#ifndef PYTREEGRAV_GB300_H
#define PYTREEGRAV_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TG_OK = 0,
    TG_ERR_BAD_ARG = 1,        /* ValueError/TypeError in the Python layer */
    TG_ERR_NONFINITE = 2,      /* non-finite input (frontend.py:123-125) */
    TG_ERR_OOM = 3,            /* device allocation failed */
    TG_ERR_STACK_OVERFLOW = 4, /* a walk's node stack overflowed (result not written) */
    TG_ERR_ITER_LIMIT = 5,     /* a bounded device loop ran out of iterations */
    TG_ERR_QUEUE_TIMEOUT = 6,  /* a work queue did not drain within its bound */
    TG_ERR_CUDA = 7,           /* a CUDA runtime call failed; see tg_last_error() */
    TG_ERR_NO_QUADRUPOLES = 8  /* quadrupole walk on a monopole tree (frontend.py:28-37) */
} tg_status;

enum { TG_MEM_HOST = 0, TG_MEM_DEVICE = 1 };

/* Field bits for tg_tree_fields / tg_bruteforce. */
enum { TG_FIELD_POTENTIAL = 1, TG_FIELD_ACCEL = 2, TG_FIELD_TIDAL = 4 };

/* Arithmetic of a walk or brute-force sum. */
enum { TG_FP32 = 0, TG_FP64 = 1 };

typedef struct tg_tree_s *tg_tree;

/* Description of a built tree. Device pointers index the pytreegrav Octree arrays
 * (octree.py:8-28): particles at [0, npart) in Morton order, nodes at [npart, node_hi). */
typedef struct {
    int64_t npart;          /* NumParticles */
    int64_t num_nodes;      /* NumNodes: capacity, grown as octree.py:1188-1206, 1280-1298 */
    int64_t node_hi;        /* one past the last allocated node */
    int32_t has_quads;      /* HasQuads */
    int32_t has_coincident; /* HasCoincidentPoints */
    int32_t n_systems;      /* independent systems in the arena (1 unless batched) */
    int32_t reserved;
    const double *coord;    /* (node_hi, 3) Coordinates */
    const double *mass;     /* (node_hi,) Masses */
    const double *size;     /* (node_hi,) Sizes */
    const double *delta;    /* (node_hi,) Deltas */
    const double *soft;     /* (node_hi,) Softenings */
    const double *quad;     /* (node_hi, 3, 3) Quadrupoles once computed (tg_tree_quadrupoles), else NULL */
    const int64_t *first;   /* (node_hi,) FirstSubnode */
    const int64_t *next;    /* (node_hi,) NextBranch */
    const int64_t *walk_idx;/* (npart,) TreewalkIndices */
} tg_tree_info;

/* Last CUDA error string recorded by this thread's most recent failing call. */
const char *tg_last_error(void);

/* ConstructTree(pos, m, softening, quadrupole, compute_moments) on the radix path
 * (frontend.py:73-142 -> octree.py:664-723, 817-1091, 199-292).
 * m == NULL: zero masses and compute_moments forced off (frontend.py:115-117).
 * h == NULL: zero softenings. Synchronises `stream` once (the node count is data dependent), before
 * the moment pass, and returns with that pass (node masses, centres of mass, Deltas, softenings,
 * quadrupoles) still running on `stream`. Every entry point taking the tree orders its own stream
 * after it; a caller reading the device arrays of tg_tree_info directly does so on `stream`, or after
 * synchronising it. */
tg_status tg_tree_build(const double *pos, const double *m, const double *h, int64_t n,
                        int quadrupole, int compute_moments, int mem, void *stream, tg_tree *out);

/* Batched build: n_systems independent systems stored back to back; system s owns particles
 * [offsets[s], offsets[s+1]). One segmented sort, one tree arena. Each system's tree equals the
 * tree tg_tree_build would give for that system alone (node indices offset into the arena). */
tg_status tg_tree_build_batched(const double *pos, const double *m, const double *h,
                                const int64_t *offsets, int32_t n_systems, int quadrupole,
                                int mem, void *stream, tg_tree *out);

/* Sizes and flags of a tree, and its device arrays (complete once the build's stream has passed the
 * build; see tg_tree_build). */
tg_status tg_tree_info_get(tg_tree tree, tg_tree_info *info);

/* The FP64 quadrupoles of a quadrupole tree (the Octree's Quadrupoles, octree.py:234-292, bit for bit):
 * the build sums FP32 quadrupoles for FP32 walks and computes these on `stream` the first time they
 * are needed (this call, tg_tree_copy_out, an FP64 walk). *quad receives the device array (mtot x 9,
 * node rows only; tg_tree_info.quad points there from then on), complete on `stream`; NULL for a
 * monopole tree. */
tg_status tg_tree_quadrupoles(tg_tree tree, const double **quad, void *stream);

/* Copy the Octree arrays to host buffers sized for info.num_nodes rows (rows past node_hi are
 * written as the reference leaves them: zeros, and -1 links). Any pointer may be NULL. */
tg_status tg_tree_copy_out(tg_tree tree, double *coord, double *mass, double *size, double *delta,
                           double *soft, double *quad, int64_t *first, int64_t *next,
                           int64_t *walk_idx, void *stream);

tg_status tg_tree_free(tg_tree tree);

/* FieldsTarget_grouped (grouped_treewalk.py:350-397) at n targets.
 * order: TG_ORDER_TREE -- targets are the tree's own particles (pos/h ignored, may be NULL),
 *   results scattered back through TreewalkIndices (frontend.py:244-288);
 *   TG_ORDER_MORTON -- targets are Morton-sorted by their own bounding cube first
 *   (grouped_treewalk.py:269-275) and results scattered back (frontend.py:392-416);
 *   TG_ORDER_GIVEN -- targets are grouped in the order given.
 * theta > 0; group_size in {1,2,4,8,16,32}; precision TG_FP32 (default engine) or TG_FP64.
 * grouping: TG_GROUP_BLOCKS -- groups of group_size consecutive targets in walk order, exactly
 *   pytreegrav's grouping (grouped_treewalk.py:180-182), so the accepted node set is pytreegrav's;
 *   TG_GROUP_TREE -- groups taken from the tree (subtrees and runs of siblings holding at most
 *   group_size particles), never straddling a jump of the Morton curve; TG_ORDER_TREE only.
 * theta_per_group: optional device array of one opening angle per group (NULL = theta). */
enum { TG_ORDER_TREE = 0, TG_ORDER_MORTON = 1, TG_ORDER_GIVEN = 2 };
enum { TG_GROUP_BLOCKS = 0, TG_GROUP_TREE = 1 };
tg_status tg_tree_fields(tg_tree tree, const double *pos, const double *h, int64_t n, int fields,
                         int quadrupole, double theta, double G, int group_size, int grouping,
                         int order, int precision, const float *theta_per_group, int mem,
                         double *out, void *stream);

/* Launch shape of this tree's walks (no counterpart in pytreegrav): warps_per_block in {2, 4, 8}
 * and the node stack a walk starts with: 1024 entries per warp (groups that overflow it are
 * rewalked, on the device, with 4096) or 4096 (fewer resident warps, no second pass). Results do
 * not depend on it; pytreegrav_gb300.autotune picks it by timing. Default: 4, 1024. */
tg_status tg_tree_set_walk_config(tg_tree tree, int warps_per_block, int first_stack);

/* A tree's walk (tg_tree_fields with TG_ORDER_TREE, FP32) captured in a CUDA graph, for calling
 * many times on one tree -- typically a batched tree of many systems (no counterpart in
 * pytreegrav). Creation makes the groups, the walk arena and the scratch, and synchronises; a
 * launch replays the graph on `stream` (zeroing the counters, the walk, and the large-stack pass
 * over the groups that overflowed the first stack) with no host synchronisation and writes `out`
 * (device, ntot x W, the caller's order); status waits for `stream` and returns the last replay's
 * status. The tree and `out` must outlive the graph; replays on one graph must not overlap. */
typedef struct tg_walk_graph_s *tg_walk_graph;
tg_status tg_walk_graph_create(tg_tree tree, int fields, int quadrupole, double theta, double G,
                               int group_size, int grouping, double *out, tg_walk_graph *graph);
tg_status tg_walk_graph_launch(tg_walk_graph graph, void *stream);
tg_status tg_walk_graph_status(tg_walk_graph graph, void *stream);
tg_status tg_walk_graph_free(tg_walk_graph graph);

/* External target points prepared once for walks of one single-system source tree: the target forms
 * PotentialTarget / AccelTarget / TidalTensorTarget (frontend.py:296-418, 563-685, 792-901), which
 * pytreegrav walks in blocks of group_size consecutive targets after sorting them by their own
 * Morton keys (_morton_order, grouped_treewalk.py:269-275; that grouping is tg_tree_fields with
 * TG_ORDER_MORTON). Here the targets get an octree of their own (the radix build, no masses) and
 * are grouped by it -- subtrees and runs of siblings of at most group_size targets, the rule of
 * TG_GROUP_TREE -- so no group straddles a jump of the Morton curve; a group whose box holds many
 * more sources than targets (the deepest source cell around it, taken as evenly filled) is cut
 * into runs of consecutive targets, so that, as in the source tree's own grouping, a group's box
 * holds about as many sources as targets. pos (n, 3) and h (n,; NULL: zeros) are read from host or
 * device memory (mem); the source tree must outlive the set. Synchronises `stream`. */
typedef struct tg_targets_s *tg_targets;
tg_status tg_targets_create(tg_tree source, const double *pos, const double *h, int64_t n, int group_size, int mem,
                            void *stream, tg_targets *out);
tg_status tg_targets_free(tg_targets targets);

/* Target count and group count of a target set. */
tg_status tg_targets_info(tg_targets targets, int64_t *n, int64_t *ngroups);

/* The groups of a target set: first target and count (walk order, int32, ngroups each), the deepest
 * node of the source tree whose cell holds each group's bounding box (int32), and each walk-order
 * target's index in the caller's arrays (int64, n). Any pointer may be NULL; host or device per mem. */
tg_status tg_targets_groups_copy(tg_targets targets, int32_t *first, int32_t *count, int32_t *src_node,
                                 int64_t *walk_idx, int mem, void *stream);

/* FieldsTarget_grouped (grouped_treewalk.py:350-397) of the source tree at the target set's groups:
 * fields as tg_tree_fields, rows in the caller's order. tol_per_group: optional device array of one
 * tolerance per group for the mass-aware acceptance test of tg_tree_fields_grouped (FP32 only;
 * NULL: pytreegrav's criterion at theta). */
tg_status tg_targets_fields(tg_targets targets, int fields, int quadrupole, double theta, double G, int precision,
                            const float *tol_per_group, int mem, double *out, void *stream);

/* Interaction statistics of the last tg_tree_fields call on this tree: total interactions and
 * node tests, the deepest node stack seen, and the number of groups. */
tg_status tg_tree_last_walk_stats(tg_tree tree, int64_t *interactions, int64_t *node_tests,
                                  int64_t *max_stack, int64_t *groups);

/* _morton_order (grouped_treewalk.py:269-275): the stable permutation sorting points by their
 * Morton keys in their own bounding cube. perm: int64 (n,). */
tg_status tg_morton_order(const double *pos, int64_t n, int mem, int64_t *perm, void *stream);

/* No counterpart in the reference: tg_morton_order for callers that cannot allocate device memory
 * (a host that owns every device allocation through its own pool, or a latency-critical path that
 * must not enter an allocator). pos (n x 3 doubles) and perm (n int64) are device pointers on the
 * current device; every temporary lives in one fixed scratch array of TG_NOALLOC_SCRATCH_BYTES that
 * the library holds on each GPU that loads it, until exit. n above TG_NOALLOC_MAX_POINTS returns
 * TG_ERR_BAD_ARG. All calls on a device share that array: calls whose GPU work overlaps race, so
 * order them (e.g. one stream). The first call on a device looks the array up (again after the
 * device's context is reset); make it before any stream capture on that device. Returns when perm
 * is written (the stream is synchronised).
 * The result equals tg_morton_order's. */
#define TG_NOALLOC_MAX_POINTS 262144
#define TG_NOALLOC_SCRATCH_BYTES 6358528
tg_status tg_morton_order_noalloc(const double *pos, int64_t n, int64_t *perm, void *stream);

/* Brute force (bruteforce.py). mutual = 1: targets are the sources, self excluded by index
 * (Potential/Accel/TidalTensor_bruteforce_parallel, bruteforce.py:86-116, 164-206, 319-350);
 * mutual = 0: target form, r == 0 pairs skipped (bruteforce.py:7-50, 209-256, 353-386; pos_t/h_t
 * used). precision TG_FP64 reproduces the CPU sums; TG_FP32 is the fast path (the numba-cuda
 * CudaPotentialBruteforce/CudaAccelBruteforce, cuda.py:627-796). */
tg_status tg_bruteforce(const double *pos_t, const double *h_t, int64_t nt, const double *pos_s,
                        const double *m_s, const double *h_s, int64_t ns, int fields, int mutual,
                        double G, int precision, int mem, double *out, void *stream);

/* Column density of uniform spheres (mass, radius = softening) integrated from each target to
 * infinity (frontend.py:1321-1458). binned = 0: pytreegrav's ray-traced walk (treewalk.py:904-973) for
 * every (target, ray); rays are unit vectors, (nrays, 3) shared by all targets (ray_stride 0) or
 * target i's own set at rays + i * ray_stride (ray_stride 3 * nrays); out is (n, nrays).
 * binned = 1: the six-bin angular estimator with opening angle theta; rays ignored; out is (n, 6):
 * group_size 0 gives the per-target walk (treewalk.py:976-1030), group_size 1..32 the grouped walk
 * of that many consecutive targets (treewalk.py:1197-1294), pytreegrav's choice from 1000 targets.
 * FP64 in the reference's order of operations. Trees of one system only. TG_ERR_ITER_LIMIT if a walk
 * does not end within one visit per element. pos NULL: the targets are the tree's own particles in
 * walk (Morton) order, n must be its particle count, per-target rays are given in that order, and
 * row i of out belongs to the caller's particle i (the results scattered through TreewalkIndices on
 * the device, frontend.py:1450-1452). */
tg_status tg_tree_column_density(tg_tree tree, const double *pos, int64_t n, const double *rays, int64_t nrays,
                                 int64_t ray_stride, int binned, double theta, int group_size, int mem, double *out,
                                 void *stream);

/* Velocities of a tree's particles, and of its nodes as pytreegrav's DynamicOctree carries them
 * (ConstructTree(..., vel=v), frontend.py:73-142 -> dynamic_tree.py:89-246, ComputeMomentsDynamic
 * dynamic_tree.py:246-310): each node's mass-weighted mean velocity and its mass-weighted velocity
 * dispersion (children's dispersions plus their spread about the mean), children in octant order.
 * On inputs without coincident points the DynamicOctree has this tree's topology and traversal order,
 * so the velocities are attached to the tree. vel (n, 3) in the caller's order, host or device per
 * mem; synchronises `stream`. TG_ERR_ITER_LIMIT if the tree's parent links do not end. */
tg_status tg_tree_set_velocities(tg_tree tree, const double *vel, int mem, void *stream);

/* Host copies of the velocities (rows as tg_tree_copy_out: NumNodes x 3, padding zeros) and
 * dispersions (NumNodes; particles 0) -- DynamicOctree.Velocities and .VelocityDisp. Either may be NULL. */
tg_status tg_tree_copy_velocities(tg_tree tree, double *vel, double *vdisp, void *stream);

/* The two-point functions (frontend.py:1047-1320, treewalk.py:344-818): per target, pytreegrav's walk
 * bins the tree's elements by log10 distance into nbins bins with edges rbins (nbins + 1, logarithmic),
 * whole nodes when they pass the opening test at theta and are smaller than max_bin_size_ratio times
 * their bin's width -- spread over the bins they overlap (weighted_binning) or at a distance jittered
 * by their size, drawn from a counter-based generator keyed by (seed, target index, draw); periodic
 * when boxsize > 0. kind TG_CORR_DENSITY: binsums = sum over targets of the mass per bin (weight
 * ignored; DensityCorrFunc divides by n; wtsums, if not NULL, gets the same sums); TG_CORR_VELOCITY /
 * TG_CORR_STRUCTURE (trees with velocities): binsums = sum of weight * mass * v.V (resp. |v - V|^2, plus a
 * node's dispersion) per bin and wtsums = sum of weight * mass (VelocityCorrFunc / VelocityStructFunc
 * divide one by the other). Each contribution is multiplied by its target's weight (pytreegrav weights
 * a target's per-bin sums: the same up to rounding). pos == NULL: the targets are the tree's own
 * particles in tree (walk) order, with their velocities and masses as vel and weight (n, vel and weight
 * ignored) -- what pytreegrav's frontends pass for a tree they build. Otherwise targets pos,
 * vel (n, 3) and weight (n) in any order (the jitter stream follows it), host or device per mem, as are
 * rbins, binsums and wtsums (nbins each). A bin index outside [0, nbins) from jitter or spreading is
 * clamped into it (pytreegrav writes past its array there). FP64. Synchronises `stream`. */
enum { TG_CORR_DENSITY = 0, TG_CORR_VELOCITY = 1, TG_CORR_STRUCTURE = 2 };
#define TG_CORR_MAX_BINS 4096
tg_status tg_tree_correlation(tg_tree tree, int kind, const double *pos, const double *vel, const double *weight,
                              int64_t n, const double *rbins, int nbins, double max_bin_size_ratio, double theta,
                              double boxsize, int weighted_binning, uint64_t seed, int mem, double *binsums,
                              double *wtsums, void *stream);

/* Number of visible CUDA devices (0, not an error, when there is no driver or device); the check
 * behind pytreegrav.cuda.is_available (cuda.py:70-80). */
tg_status tg_device_count(int *count);

/* A source set uploaded once and summed against new targets on every call: the device side of the
 * numba-cuda CudaPotentialBruteforce / CudaAccelBruteforce contexts (cuda.py:737-796).
 * tg_sources_create copies pos (n, 3), m (n,) and h (n,) (h NULL: zeros) from host or device memory
 * (mem). tg_sources_bruteforce writes fields (W columns) for nt targets; pos_t NULL takes the sources
 * themselves as the targets, with their softenings (nt ignored). Pairs at r == 0 are skipped in
 * either case (the target form, bruteforce.py:7-50), so a target coinciding with a source drops
 * that source, as in the reference contexts. */
typedef struct tg_sources_s *tg_sources;
tg_status tg_sources_create(const double *pos, const double *m, const double *h, int64_t n, int mem, void *stream,
                            tg_sources *out);
tg_status tg_sources_bruteforce(tg_sources s, const double *pos_t, const double *h_t, int64_t nt, int fields,
                                double G, int precision, int mem, double *out, void *stream);
tg_status tg_sources_free(tg_sources s);

#ifdef __cplusplus
}
#endif
#endif
