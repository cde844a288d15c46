// External target points prepared once for walks of one source tree: the target forms
// (PotentialTarget / AccelTarget / TidalTensorTarget, frontend.py:296-418, 563-685, 792-901) with the
// targets grouped by their own octree instead of in consecutive Morton blocks.
//
// pytreegrav sorts the targets by their Morton keys in their own bounding cube (_morton_order,
// grouped_treewalk.py:269-275) and walks consecutive blocks of group_size of them. A block that
// straddles a jump of the Morton curve gets a bounding box spanning both sides and opens far more of
// the source tree than either half would. Here the targets get an octree of their own (the same
// radix build as the sources, without masses or moments) and its tree grouping: subtrees and runs
// of siblings of at most group_size targets, which never straddle such a jump. Where the sources are
// much denser than the targets (external targets in the core of a source distribution) such a group
// still spans a region holding far more sources than targets and opens a large part of the tree, so
// it is cut into shorter runs (targets_refine_groups): the groups then hold about as many sources as
// targets, as the source tree's own groups do. Walks of the source tree take those groups; results
// are scattered back to the caller's order through the target tree's TreewalkIndices.
#include <new>

#include "tg_targets.cuh"

namespace tg {

tg_status tree_groups(tg_tree_s *t, int G, cudaStream_t st);
template <typename T>
tg_status build_arena(tg_tree_s *t, Arena<T> &ar, cudaStream_t st);
tg_status run_walk(tg_tree_s *t, const double *tpos, const double *th, int64_t ntargets, const int2 *groups,
                   const int *group_root, const int *group_order, int64_t ngroups, const int64_t *scatter, int fields,
                   int quadrupole, double theta, double G, int group_size, int precision, const float *theta_group,
                   const float *tol_group, double *out, cudaStream_t st);

namespace {

bool valid_gs(int gs) { return gs == 1 || gs == 2 || gs == 4 || gs == 8 || gs == 16 || gs == 32; }

int width_of(int fields) { return ((fields & 1) ? 1 : 0) + ((fields & 2) ? 3 : 0) + ((fields & 4) ? 9 : 0); }

// One thread per group: the group's FP64 bounding box, then a descent from the source root (node 0)
// through the node child whose cell (cell centre +- size / 2) holds the whole box, as long as one
// does. Children come from the walk arena's traversal records (first node child << 4 | count). The
// descent goes one level deeper per step; it is bounded by the node count in any case.
// With nsub non-null, also the number of pieces the group is cut into (see k_split_groups). The
// local source density comes from the smallest source cell that holds the box's centre and is at
// least as large as the box (found by continuing the descent through the children holding the
// centre): taking its n sources as spread evenly over its cell of size s, the box holds about
// n_in = n (e / s)^3 sources (e the box's largest extent). A group whose box holds more than 2G
// sources would open far more of the tree per target than a group of the sources' own tree does,
// so it is cut into runs of k consecutive targets, k the largest power of two with
// k n_in / count <= 2G.
__global__ void k_target_src_nodes(int64_t ntot, int64_t mtot, const double *cell, const double *size, Arena<float> ar,
                                   const int2 *node_range, const double *tpos, const int2 *groups, int64_t ng, int G,
                                   int *node, int *nsub, int *sublen) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int2 gr = groups[g];
    double lo[3], hi[3];
    for (int k = 0; k < 3; k++) lo[k] = hi[k] = tpos[3 * (int64_t)gr.x + k];
    for (int i = 1; i < gr.y; i++)
        for (int k = 0; k < 3; k++) {
            const double v = tpos[3 * ((int64_t)gr.x + i) + k];
            lo[k] = fmin(lo[k], v);
            hi[k] = fmax(hi[k], v);
        }
    int j = 0;
    if (!(ar.bad && *ar.bad)) {
        for (int64_t steps = 0; steps < mtot; steps++) {
            const int cb = __float_as_int(ar.n_trav[2 * j + 1].z);
            const int fc = cb >> 4, nc = cb & 15;
            int nxt = -1;
            for (int c = fc; c < fc + nc; c++) {
                if (c < 0 || c >= mtot) break;
                const double hs = 0.5 * size[ntot + c];
                bool inside = true;
                for (int k = 0; k < 3; k++)
                    inside = inside && lo[k] >= cell[3 * (int64_t)c + k] - hs && hi[k] <= cell[3 * (int64_t)c + k] + hs;
                if (inside) {
                    nxt = c;
                    break;
                }
            }
            if (nxt < 0) break;
            j = nxt;
        }
    }
    node[g] = j;
    if (nsub) {
        int k = gr.y;
        const double e = fmax(fmax(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
        const double ctr[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
        int d = j;  // the density cell: from j down through the children holding the centre
        if (!(ar.bad && *ar.bad)) {
            for (int64_t steps = 0; steps < mtot; steps++) {
                const int cb = __float_as_int(ar.n_trav[2 * d + 1].z);
                const int fc = cb >> 4, nc = cb & 15;
                int nxt = -1;
                for (int c = fc; c < fc + nc; c++) {
                    if (c < 0 || c >= mtot) break;
                    const double sc = size[ntot + c], hs = 0.5 * sc;
                    if (sc < e) continue;
                    bool inside = true;
                    for (int q = 0; q < 3; q++)
                        inside = inside && ctr[q] >= cell[3 * (int64_t)c + q] - hs && ctr[q] <= cell[3 * (int64_t)c + q] + hs;
                    if (inside) {
                        nxt = c;
                        break;
                    }
                }
                if (nxt < 0) break;
                d = nxt;
            }
        }
        const double sd = size[ntot + d];
        if (!(ar.bad && *ar.bad) && sd > 0.0 && gr.y > 1) {
            const double q = e / sd;
            const double n_in = (double)(node_range[d].y - node_range[d].x) * q * q * q;
            k = 1;  // the largest power of two (at most the count) with k n_in <= 2 G count
            while (2 * k <= gr.y && (double)(2 * k) * n_in <= 2.0 * G * gr.y) k *= 2;
            if (n_in <= 2.0 * G) k = gr.y;
        }
        nsub[g] = (gr.y + k - 1) / k;
        sublen[g] = k;
    }
}

// The refined groups: group g's targets cut into nsub[g] runs of sublen[g] (the last shorter), at
// offset off[g], in start order.
__global__ void k_split_groups(const int2 *groups, const int *gnode, int64_t ng, const int *nsub, const int *sublen,
                               const int *off, int2 *out, int *out_root, int *out_node) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int2 gr = groups[g];
    const int k = sublen[g], o = off[g];
    for (int i = 0; i < nsub[g]; i++) {
        const int first = gr.x + i * k;
        out[o + i] = make_int2(first, min(k, gr.x + gr.y - first));
        out_root[o + i] = 0;
        out_node[o + i] = gnode[g];
    }
}

}  // namespace

tg_status targets_src_nodes(tg_targets_s *ts, cudaStream_t st) {
    if (ts->src_node) return TG_OK;
    tg_tree_s *src = ts->src, *tt = ts->tt;
    TG_TRY(build_arena(src, src->arena32, st));
    const int64_t ng = tt->ngroups;
    TG_CUDA(dev_malloc((void **)&ts->src_node, sizeof(int) * std::max<int64_t>(ng, 1), st));
    if (ng > 0) {
        k_target_src_nodes<<<div_up(ng, 128), 128, 0, st>>>(src->ntot, src->mtot, src->cell_center, src->size,
                                                            src->arena32, src->node_range, tt->coord, tt->groups, ng,
                                                            ts->group_size, ts->src_node, nullptr, nullptr);
        note_launch();
        TG_CUDA(cudaGetLastError());
    }
    return TG_OK;
}

// Cuts the target tree's groups where the sources are denser than the targets (see
// k_target_src_nodes); the groups stay in start order, so the result does not depend on timing.
tg_status targets_refine_groups(tg_targets_s *ts, cudaStream_t st) {
    tg_tree_s *src = ts->src, *tt = ts->tt;
    const int64_t ng = tt->ngroups;
    if (ng <= 0) return TG_OK;
    tree_wait_built(src, st);
    TG_TRY(build_arena(src, src->arena32, st));
    DevArray<int> node(st), nsub(st), sublen(st), off(st);
    TG_CUDA(node.alloc(ng));
    TG_CUDA(nsub.alloc(ng + 1));
    TG_CUDA(sublen.alloc(ng));
    TG_CUDA(off.alloc(ng + 1));
    TG_CUDA(cudaMemsetAsync(nsub.p + ng, 0, sizeof(int), st));
    { k_target_src_nodes<<<div_up(ng, 128), 128, 0, st>>>(src->ntot, src->mtot, src->cell_center, src->size,
                                                         src->arena32, src->node_range, tt->coord, tt->groups, ng,
                                                         ts->group_size, node.p, nsub.p, sublen.p); note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_TRY(exclusive_scan_i32(nsub.p, off.p, ng + 1, st));
    int total = 0;
    TG_CUDA(cudaMemcpyAsync(&total, off.p + ng, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    if (total == ng) return TG_OK;  // nothing to cut
    int2 *groups = nullptr;
    int *root = nullptr, *gnode = nullptr;
    TG_CUDA(dev_malloc((void **)&groups, sizeof(int2) * total, st));
    TG_CUDA(dev_malloc((void **)&root, sizeof(int) * total, st));
    TG_CUDA(dev_malloc((void **)&gnode, sizeof(int) * total, st));
    { k_split_groups<<<div_up(ng, 128), 128, 0, st>>>(tt->groups, tt->group_node, ng, nsub.p, sublen.p, off.p, groups,
                                                     root, gnode); note_launch(); }
    TG_CUDA(cudaGetLastError());
    cudaFreeAsync(tt->groups, st);
    cudaFreeAsync(tt->group_root, st);
    cudaFreeAsync(tt->group_node, st);
    tt->groups = groups;
    tt->group_root = root;
    tt->group_node = gnode;
    tt->ngroups = total;
    return TG_OK;
}

}  // namespace tg

using namespace tg;

extern "C" {

tg_status tg_targets_create(tg_tree src, const double *pos, const double *h, int64_t n, int group_size, int mem,
                            void *stream, tg_targets *out) {
    if (!out) return TG_ERR_BAD_ARG;
    *out = nullptr;
    if (!src || !pos || n < 1 || !valid_gs(group_size) || (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE))
        return TG_ERR_BAD_ARG;
    if (src->nsys != 1 || src->sys_node_off.empty() || src->sys_node_off[0] != 0) {
        set_last_error_msg("target sets need a single-system source tree");
        return TG_ERR_BAD_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    tg_targets_s *ts = new (std::nothrow) tg_targets_s();
    if (!ts) return TG_ERR_OOM;
    ts->src = src;
    ts->group_size = group_size;
    ts->n = n;
    ts->stream = st;
    // the targets' own octree: positions and softenings, no masses, no moments
    tg_status rc = tg_tree_build(pos, nullptr, h, n, 0, 0, mem, stream, &ts->tt);
    if (rc == TG_OK) {
        tree_wait_built(ts->tt, st);
        rc = tree_groups(ts->tt, group_size, st);
    }
    if (rc == TG_OK) rc = targets_refine_groups(ts, st);
    if (rc != TG_OK) {
        tg_targets_free(ts);
        return rc;
    }
    *out = ts;
    return TG_OK;
}

tg_status tg_targets_free(tg_targets ts) {
    if (!ts) return TG_OK;
    if (ts->src_node) cudaFreeAsync(ts->src_node, ts->stream);
    if (ts->tt) tg_tree_free(ts->tt);
    delete ts;
    return TG_OK;
}

tg_status tg_targets_info(tg_targets ts, int64_t *n, int64_t *ngroups) {
    if (!ts) return TG_ERR_BAD_ARG;
    if (n) *n = ts->n;
    if (ngroups) *ngroups = ts->tt->ngroups;
    return TG_OK;
}

tg_status tg_targets_groups_copy(tg_targets ts, int32_t *first, int32_t *count, int32_t *src_node, int64_t *walk_idx,
                                 int mem, void *stream) {
    if (!ts || (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE)) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tg_tree_s *tt = ts->tt;
    const int64_t ng = tt->ngroups;
    tree_wait_built(ts->src, st);
    if (src_node) TG_TRY(targets_src_nodes(ts, st));
    const cudaMemcpyKind kind = mem == TG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (first || count) {
        std::vector<int2> g(ng);
        TG_CUDA(cudaMemcpyAsync(g.data(), tt->groups, sizeof(int2) * ng, cudaMemcpyDeviceToHost, st));
        TG_CUDA(cudaStreamSynchronize(st));
        std::vector<int32_t> a(ng), b(ng);
        for (int64_t i = 0; i < ng; i++) {
            a[i] = g[i].x;
            b[i] = g[i].y;
        }
        if (first) TG_CUDA(cudaMemcpyAsync(first, a.data(), sizeof(int32_t) * ng, mem == TG_MEM_HOST ?
                                           cudaMemcpyHostToHost : cudaMemcpyHostToDevice, st));
        if (count) TG_CUDA(cudaMemcpyAsync(count, b.data(), sizeof(int32_t) * ng, mem == TG_MEM_HOST ?
                                           cudaMemcpyHostToHost : cudaMemcpyHostToDevice, st));
        TG_CUDA(cudaStreamSynchronize(st));
    }
    if (src_node) TG_CUDA(cudaMemcpyAsync(src_node, ts->src_node, sizeof(int32_t) * ng, kind, st));
    if (walk_idx) TG_CUDA(cudaMemcpyAsync(walk_idx, tt->walk_idx, sizeof(int64_t) * ts->n, kind, st));
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

tg_status tg_targets_fields(tg_targets ts, int fields, int quadrupole, double theta, double G, int precision,
                            const float *tol_per_group, int mem, double *out, void *stream) {
    if (!ts || !out || (fields & 7) == 0 || (fields & ~7) || !(theta > 0) ||
        (precision != TG_FP32 && precision != TG_FP64) || (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE))
        return TG_ERR_BAD_ARG;
    if (tol_per_group && precision != TG_FP32) return TG_ERR_BAD_ARG;
    tg_tree_s *src = ts->src, *tt = ts->tt;
    if (quadrupole && !src->has_quads) return TG_ERR_NO_QUADRUPOLES;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(src, st);
    tree_wait_built(tt, st);
    const int64_t n = ts->n;
    const int W = width_of(fields);
    double *dout = out;
    if (mem == TG_MEM_HOST) TG_CUDA(dev_malloc((void **)&dout, sizeof(double) * n * W, st));
    tg_status rc = run_walk(src, tt->coord, tt->soft, n, tt->groups, tt->group_root, nullptr, tt->ngroups,
                            tt->walk_idx, fields, quadrupole, theta, G, ts->group_size, precision, nullptr,
                            tol_per_group, dout, st);
    if (rc == TG_OK && mem == TG_MEM_HOST)
        TG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * n * W, cudaMemcpyDeviceToHost, st));
    if (mem == TG_MEM_HOST) cudaFreeAsync(dout, st);
    TG_CUDA(cudaStreamSynchronize(st));
    return rc;
}

}  // extern "C"
