// A set of external target points prepared for walks of one source tree (tg_targets_*; declared in
// include/pytreegrav_gb300.h and include/pytreegrav_gb300_theta.h).
#pragma once

#include "tg_tree.cuh"

struct tg_targets_s {
    tg_tree_s *src = nullptr;  // the source tree (not owned; must outlive the target set)
    tg_tree_s *tt = nullptr;   // octree of the targets themselves (owned; no masses, no moments)
    int group_size = 32;       // at most this many targets per group
    int64_t n = 0;
    // Per group: the deepest node of the source tree whose cell holds the group's bounding box
    // (made on first need, for the learned opening test's features).
    int *src_node = nullptr;
    cudaStream_t stream = nullptr;
};

namespace tg {
// Source-tree node of every target group (kept on the target set).
tg_status targets_src_nodes(tg_targets_s *ts, cudaStream_t st);
}  // namespace tg
