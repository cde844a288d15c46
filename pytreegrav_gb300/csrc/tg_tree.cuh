// Device-resident octree and the walk arena derived from it.
#pragma once

#include <type_traits>
#include <vector>

#include "tg_common.cuh"

namespace tg {

// 32-byte FP64 quadruple (the CUDA double4 vector type is deprecated in CUDA 13).
struct alignas(32) D4 {
    double x, y, z, w;
};
template <typename T>
using vec4 = typename std::conditional<sizeof(T) == 4, float4, D4>::type;

// Walk arena: the octree repacked for the grouped walk. Nodes keep their final numbering
// (node j = arena element npart_total + j) because pytreegrav's numbering already makes every
// node's node-children contiguous; each node's particle children are copied into a contiguous
// leaf range. Positions are split into a float "hi" part and the float rounding residual "lo",
// so the walk can form source-target offsets relative to its group to ~2^-48 relative accuracy.
template <typename T>
struct Arena {
    int64_t n_nodes = 0, n_leaves = 0;
    // per node
    // traversal record, two per node: (hi.x, hi.y, hi.z, size), (delta, hmax, first node child << 4 |
    // node children, leaf start << 4 | leaves) -- the integers stored as the bit pattern of T
    vec4<T> *n_trav = nullptr;
    vec4<T> *n_pos = nullptr;   // interaction record: hi.xyz, M
    vec4<T> *n_lo = nullptr;    // lo.xyz, hmax
    vec4<T> *n_quad = nullptr;  // two per node: (xx, xy, xz, yy), (yz, zz, 0, 0)
    // FP32 arenas: per node (M s^3)^(1/5) and (M s^2)^(1/4), the mass-aware acceptance test's
    // node factor for quadrupole and monopole walks (a group's tolerance scales it)
    float2 *n_tol = nullptr;
    int4 *n_link = nullptr;     // first node child, node children, leaf start, leaves (build scratch)
    // per leaf
    vec4<T> *l_pos = nullptr;  // hi.xyz, m
    vec4<T> *l_lo = nullptr;   // lo.xyz, h
    int *bad = nullptr;        // device: nonzero if the tree's links did not make a valid arena
    bool built = false;
    bool has_quad = false;
};

struct WalkStats {
    int64_t interactions = 0, node_tests = 0, max_stack = 0, groups = 0, steps = 0, quad_interactions = 0;
    float kernel_ms = 0.f;  // device time of the walk kernel launch(es)
};

}  // namespace tg

struct tg_tree_s {
    int64_t ntot = 0;       // particles in the arena (all systems)
    int64_t mtot = 0;       // nodes in the arena (all systems)
    int32_t nsys = 1;
    int dev = 0;  // the CUDA device it lives on
    int has_quads = 0;
    int has_coincident = 0;
    int compute_moments = 1;
    std::vector<int64_t> sys_off;       // host: particle offsets per system (nsys + 1)
    std::vector<int64_t> sys_node_off;  // host: node offsets per system (nsys + 1), roots first
    std::vector<int64_t> sys_capacity;  // host: NumNodes per system (reference capacity rule)
    cudaStream_t stream = nullptr;

    // Octree arrays over the arena: particles [0, ntot), nodes [ntot, ntot + mtot).
    double *coord = nullptr;   // 3 per element
    double *mass = nullptr;
    double *size = nullptr;
    double *delta = nullptr;
    double *soft = nullptr;
    double *quad = nullptr;    // 9 per NODE (mtot rows): FP64 quadrupoles, null until ensure_quad64
    float4 *quad32 = nullptr;  // 2 per NODE: FP32 quadrupoles (xx xy xz yy)(yz zz 0 0) for FP32 walks
    // The depth lists of the moment pass, kept for ensure_quad64 (quadrupole trees until it has run).
    int32_t *lvl_list = nullptr;
    int8_t *fdepth = nullptr;
    std::vector<int> lvl_off;  // host: section offsets per depth (DEPTH_CAP + 2)
    int64_t *first = nullptr;
    int64_t *next = nullptr;
    int64_t *walk_idx = nullptr;  // per particle: index into the caller's input arrays
    int64_t *parent = nullptr;    // per element: owning node (arena index), -1 for roots
    int2 *node_range = nullptr;   // per node: particle range [lo, hi) of its subtree
    double *cell_center = nullptr;  // per node: geometric centre of its cell (3)

    // The look-back error word of every radix sort made for this tree (build, grouping, queue
    // order), read back by the build and by each walk (nonzero: a sort failed).
    int *sort_err = nullptr;

    // Velocities (tg_tree_set_velocities): per element, particles' own and nodes' mass-weighted mean
    // (3 each), and per element the velocity dispersion (particles 0); null until set.
    double *vel = nullptr, *vdisp = nullptr;

    tg::Arena<float> arena32;
    tg::Arena<double> arena64;
    // FP32 walk targets of the tree's own particles in walk order (ntot hi rows, then ntot lo rows),
    // made on the side stream beside the first grouping; null until then.
    float4 *own32 = nullptr;
    tg::WalkStats last_stats;
    int64_t *stats_dev = nullptr;  // 8 counters

    // Tree grouping (TG_GROUP_TREE, TG_ORDER_TREE) at group size groups_G, made on first use and
    // kept: groups as (first target, count) in start order, each group's system root and the node
    // whose subtree holds it.
    int groups_G = 0;
    int64_t ngroups = 0;
    int2 *groups = nullptr;
    int *group_root = nullptr;
    int *group_node = nullptr;
    // Per-group walk counters, three per group (list entries evaluated as point masses, entries
    // evaluated as quadrupole nodes, nodes tested), written by walks while record_group_stats is set.
    int record_group_stats = 0;
    unsigned *gstats = nullptr;
    int64_t gstats_n = 0;
    // Walks with per-group tolerances: each group's estimated relative truncation error (recorded
    // with the counters above), and the budget above which a group is walked again at the global
    // theta (0: no check); set by the learned entry from its model for the duration of its walk.
    float *gerr = nullptr;
    float err_budget = 0.f;
    double rewalk_theta = 0.7;
    // Walk launch shape (tg_tree_set_walk_config): warps per block, and the node stack a walk starts
    // with (1024: groups that overflow it are rewalked with 4096; 4096: every group starts there).
    int walk_warps = 4;
    int walk_stack = 1024;
    // Side stream (non-blocking, made on first use) on which the walk arena is packed while the
    // grouping runs on the caller's stream, and the two events that order it.
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // Recorded on the build's stream: ev_topo once the topology and geometry (links, ranges, cells,
    // particle data) are final, before the moment pass; ev_built after it. A build returns once the
    // host-visible results are known, with the moment pass still running on its stream: every entry
    // point orders its own stream after ev_built, and tree grouping, which needs no moments, starts
    // from ev_topo on the side stream.
    cudaEvent_t ev_topo = nullptr, ev_built = nullptr;
};

namespace tg {
// Orders work on s after the tree's build (a no-op when s is the build's stream).
inline void tree_wait_built(const tg_tree_s *t, cudaStream_t s) {
    if (t && t->ev_built) cudaStreamWaitEvent(s, t->ev_built, 0);
}
// The FP64 quadrupoles (t->quad) of a quadrupole tree, computed on s the first time they are needed.
tg_status ensure_quad64(tg_tree_s *t, cudaStream_t s);
}  // namespace tg
