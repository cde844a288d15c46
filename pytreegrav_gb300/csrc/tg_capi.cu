// extern "C" entry points of libpytreegrav_gb300 (declared in include/pytreegrav_gb300.h).
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "tg_tree.cuh"

namespace tg {
tg_status build_tree(tg_tree_s *T, const double *pos, const double *m, const double *h,
                     const std::vector<int64_t> &sys_off_host, int quadrupole, int compute_moments,
                     const int *nonfinite, cudaStream_t st, cudaEvent_t m_h_ready);
tg_status tree_side_stream(tg_tree_s *t);
tg_status morton_order_device(const double *pos, int64_t n, uint32_t *perm, cudaStream_t st);
template <typename T>
tg_status build_arena(tg_tree_s *t, Arena<T> &ar, cudaStream_t st);
template <typename T>
void free_arena(Arena<T> &ar, cudaStream_t st);
tg_status run_walk(tg_tree_s *t, const double *tpos, const double *th, int64_t ntargets, const int2 *groups,
                   const int *group_root, const int *group_order, int64_t ngroups, const int64_t *scatter, int fields,
                   int quadrupole, double theta, double G, int group_size, int precision, const float *theta_group,
                   const float *tol_group, double *out, cudaStream_t st);
tg_status make_groups(tg_tree_s *t, const std::vector<int64_t> &sys_off_host, int gs, int2 **groups,
                      int **group_root, int64_t *ngroups, cudaStream_t st);
tg_status tree_groups(tg_tree_s *t, int G, cudaStream_t st);
tg_status tree_groups_with_arena(tg_tree_s *t, int G, bool fp64, cudaStream_t st);
tg_status make_cost_order(const double *tpos, const int2 *groups, int64_t ngroups, int **order, cudaStream_t st,
                          int *sort_err);
tg_status run_bruteforce(const double *pt, const double *ht, int64_t nt, const double *ps, const double *ms,
                         const double *hs, int64_t ns, int fields, int mutual, double G, int precision, double *out,
                         cudaStream_t st);

namespace {

// Infinity or NaN: the all-ones exponent, tested on the bits (integer units, not the FP64 pipe).
__device__ __forceinline__ bool nonfinite_bits(const double *p) {
    return (~(unsigned long long)__ldg((const long long *)p) & 0x7ff0000000000000ull) == 0;
}

__global__ void k_nonfinite(const double *a, int64_t n, int *flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && nonfinite_bits(a + i)) atomicOr(flag, 1);
}

// Any non-finite value among positions (3n), masses (n, may be NULL) and softenings (n, may be NULL).
__global__ void k_nonfinite3(const double *pos, const double *m, const double *h, int64_t n, int *flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 5 * n) return;
    const double *p = i < 3 * n ? pos + i : (i < 4 * n ? (m ? m + (i - 3 * n) : nullptr) : (h ? h + (i - 4 * n) : nullptr));
    if (p && nonfinite_bits(p)) atomicOr(flag, 1);
}

__global__ void k_u32_to_i64(const uint32_t *a, int64_t n, int64_t *b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

__global__ void k_gather_targets(const uint32_t *perm, int64_t n, const double *pos, const double *h, double *pos_s,
                                 double *h_s) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t o = perm[i];
    pos_s[3 * i] = pos[3 * o];
    pos_s[3 * i + 1] = pos[3 * o + 1];
    pos_s[3 * i + 2] = pos[3 * o + 2];
    h_s[i] = h ? h[o] : 0.0;
}

// Device copies of caller arrays (or the caller's own device pointers), freed on scope exit.
struct DevBuf {
    const double *ptr = nullptr;
    double *owned = nullptr;
    cudaStream_t st = nullptr;
    ~DevBuf() {
        if (owned) cudaFreeAsync(owned, st);
    }
};

tg_status stage_in(const double *src, int64_t count, int mem, cudaStream_t st, DevBuf &b) {
    b.st = st;
    if (!src) {
        b.ptr = nullptr;
        return TG_OK;
    }
    if (mem == TG_MEM_DEVICE) {
        b.ptr = src;
        return TG_OK;
    }
    TG_CUDA(tg::dev_malloc((void **)&b.owned, sizeof(double) * std::max<int64_t>(count, 1), st));
    TG_CUDA(cudaMemcpyAsync(b.owned, src, sizeof(double) * count, cudaMemcpyHostToDevice, st));
    b.ptr = b.owned;
    return TG_OK;
}

tg_status check_finite(const double *const *arrs, const int64_t *counts, int k, cudaStream_t st) {
    int *flag = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&flag, sizeof(int), st));
    TG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    for (int q = 0; q < k; q++)
        if (arrs[q] && counts[q] > 0) { k_nonfinite<<<div_up(counts[q], 256), 256, 0, st>>>(arrs[q], counts[q], flag); tg::note_launch(); }
    int hflag = 0;
    TG_CUDA(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaFreeAsync(flag, st));
    TG_CUDA(cudaStreamSynchronize(st));
    return hflag ? TG_ERR_NONFINITE : TG_OK;
}

void destroy(tg_tree_s *t) {
    if (!t) return;
    cudaStream_t st = t->stream;
    auto f = [&](void *p) {
        if (p) cudaFreeAsync(p, st);
    };
    f(t->coord); f(t->mass); f(t->size); f(t->delta); f(t->soft); f(t->quad);
    f(t->first); f(t->next); f(t->walk_idx); f(t->parent); f(t->node_range); f(t->cell_center);
    free_arena(t->arena32, st);
    free_arena(t->arena64, st);
    if (t->stats_dev) cudaFreeAsync(t->stats_dev, st);
    f(t->groups); f(t->group_root); f(t->group_node); f(t->gstats); f(t->gerr); f(t->sort_err); f(t->vel); f(t->vdisp); f(t->quad32); f(t->lvl_list); f(t->fdepth); f(t->own32);
    release_stream(t->side);  // back to the library's pool, its queued work still to run
    release_event(t->ev_fork, false, t->dev);
    release_event(t->ev_join, false, t->dev);
    release_event(t->ev_topo, false, t->dev);
    release_event(t->ev_built, false, t->dev);
    delete t;
}

int field_width(int fields) {
    return ((fields & 1) ? 1 : 0) + ((fields & 2) ? 3 : 0) + ((fields & 4) ? 9 : 0);
}

bool valid_group_size(int gs) { return gs == 1 || gs == 2 || gs == 4 || gs == 8 || gs == 16 || gs == 32; }

}  // namespace
}  // namespace tg

using namespace tg;

// A source set kept on the device between direct-sum calls.
struct tg_sources_s {
    double *pos = nullptr, *m = nullptr, *h = nullptr;
    int64_t n = 0;
};

extern "C" {

const char *tg_last_error(void) { return tg::last_error(); }

static tg_status build_common(const double *pos, const double *m, const double *h, std::vector<int64_t> off,
                              int quadrupole, int compute_moments, int mem, void *stream, tg_tree *out) {
    if (!out || !pos) return TG_ERR_BAD_ARG;
    *out = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = off.back();
    if (n < 1) return TG_ERR_BAD_ARG;
    if (!m) compute_moments = 0;
    tg_tree_s *t = new (std::nothrow) tg_tree_s();
    if (t) t->dev = current_device_or(0);
    if (!t) return TG_ERR_OOM;
    tg_status rc = TG_OK;
    {
        DevBuf dp, dm, dh;
        int *flag = nullptr;
        cudaEvent_t m_h_ready = nullptr;
        auto stage = [&]() -> tg_status {
            TG_TRY(stage_in(pos, 3 * n, mem, st, dp));
            // the input check runs ahead of the build on the stream; the build reads its flag back
            // with its first summary and reports non-finite input with its closing read-back
            TG_CUDA(tg::dev_malloc((void **)&flag, sizeof(int), st));
            TG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
            if (mem == TG_MEM_HOST && (m || h)) {
                { k_nonfinite<<<div_up(3 * n, 256), 256, 0, st>>>(dp.ptr, 3 * n, flag); tg::note_launch(); }
                // masses and softenings are uploaded (and checked) on the tree's side stream while
                // the build sorts the positions; the build waits for them where it first reads them
                TG_TRY(tree_side_stream(t));
                TG_CUDA(cudaEventRecord(t->ev_fork, st));
                TG_CUDA(cudaStreamWaitEvent(t->side, t->ev_fork, 0));
                TG_TRY(stage_in(m, n, mem, t->side, dm));
                TG_TRY(stage_in(h, n, mem, t->side, dh));
                dm.st = dh.st = st;  // freed on st, after the build's last read
                if (dm.ptr) { k_nonfinite<<<div_up(n, 256), 256, 0, t->side>>>(dm.ptr, n, flag); tg::note_launch(); }
                if (dh.ptr) { k_nonfinite<<<div_up(n, 256), 256, 0, t->side>>>(dh.ptr, n, flag); tg::note_launch(); }
                TG_CUDA(cudaEventRecord(t->ev_join, t->side));
                m_h_ready = t->ev_join;
            } else {
                TG_TRY(stage_in(m, n, mem, st, dm));
                TG_TRY(stage_in(h, n, mem, st, dh));
                { k_nonfinite3<<<div_up(5 * n, 256), 256, 0, st>>>(dp.ptr, dm.ptr, dh.ptr, n, flag); tg::note_launch(); }
            }
            TG_CUDA(cudaGetLastError());
            return TG_OK;
        };
        rc = stage();
        if (rc == TG_OK) rc = build_tree(t, dp.ptr, dm.ptr, dh.ptr, off, quadrupole, compute_moments, flag, st, m_h_ready);
        // st is ordered after the side stream's uploads before anything staged is freed
        if (m_h_ready) cudaStreamWaitEvent(st, m_h_ready, 0);
        if (flag) cudaFreeAsync(flag, st);
    }
    if (rc != TG_OK) {
        destroy(t);
        return rc;
    }
    *out = t;
    return TG_OK;
}

tg_status tg_tree_build(const double *pos, const double *m, const double *h, int64_t n, int quadrupole,
                        int compute_moments, int mem, void *stream, tg_tree *out) {
    if (n < 1) return TG_ERR_BAD_ARG;
    return build_common(pos, m, h, {0, n}, quadrupole, compute_moments, mem, stream, out);
}

tg_status tg_tree_build_batched(const double *pos, const double *m, const double *h, const int64_t *offsets,
                                int32_t n_systems, int quadrupole, int mem, void *stream, tg_tree *out) {
    if (!offsets || n_systems < 1) return TG_ERR_BAD_ARG;
    std::vector<int64_t> off(offsets, offsets + n_systems + 1);
    if (off[0] != 0) return TG_ERR_BAD_ARG;
    for (int s = 0; s < n_systems; s++)
        if (off[s + 1] <= off[s]) return TG_ERR_BAD_ARG;
    return build_common(pos, m, h, off, quadrupole, 1, mem, stream, out);
}

tg_status tg_tree_info_get(tg_tree t, tg_tree_info *info) {
    if (!t || !info) return TG_ERR_BAD_ARG;
    memset(info, 0, sizeof(*info));
    info->npart = t->ntot;
    info->node_hi = t->ntot + t->mtot;
    info->num_nodes = t->nsys == 1 ? t->sys_capacity[0] : t->ntot + t->mtot;
    info->has_quads = t->has_quads;
    info->has_coincident = t->has_coincident;
    info->n_systems = t->nsys;
    info->coord = t->coord;
    info->mass = t->mass;
    info->size = t->size;
    info->delta = t->delta;
    info->soft = t->soft;
    info->quad = t->quad;
    info->first = t->first;
    info->next = t->next;
    info->walk_idx = t->walk_idx;
    return TG_OK;
}

tg_status tg_tree_quadrupoles(tg_tree t, const double **quad, void *stream) {
    if (!t || !quad) return TG_ERR_BAD_ARG;
    *quad = nullptr;
    if (!t->has_quads) return TG_OK;
    TG_TRY(ensure_quad64(t, (cudaStream_t)stream));
    *quad = t->quad;
    return TG_OK;
}

tg_status tg_tree_copy_out(tg_tree t, double *coord, double *mass, double *size, double *delta, double *soft,
                           double *quad, int64_t *first, int64_t *next, int64_t *walk_idx, void *stream) {
    if (!t) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    const int64_t NE = t->ntot + t->mtot;
    const int64_t cap = t->nsys == 1 ? t->sys_capacity[0] : NE;
    const int64_t pad = cap - NE;
    auto cp = [&](void *dst, const void *src, size_t bytes) -> tg_status {
        TG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
        return TG_OK;
    };
    if (coord) TG_TRY(cp(coord, t->coord, sizeof(double) * 3 * NE));
    if (mass) TG_TRY(cp(mass, t->mass, sizeof(double) * NE));
    if (size) TG_TRY(cp(size, t->size, sizeof(double) * NE));
    if (delta) TG_TRY(cp(delta, t->delta, sizeof(double) * NE));
    if (soft) TG_TRY(cp(soft, t->soft, sizeof(double) * NE));
    if (quad && t->has_quads) {
        TG_TRY(ensure_quad64(t, st));
        TG_TRY(cp(quad + 9 * t->ntot, t->quad, sizeof(double) * 9 * t->mtot));
    }
    if (first) TG_TRY(cp(first, t->first, sizeof(int64_t) * NE));
    if (next) TG_TRY(cp(next, t->next, sizeof(int64_t) * NE));
    if (walk_idx) TG_TRY(cp(walk_idx, t->walk_idx, sizeof(int64_t) * t->ntot));
    TG_CUDA(cudaStreamSynchronize(st));
    if (pad > 0) {
        if (coord) memset(coord + 3 * NE, 0, sizeof(double) * 3 * pad);
        if (mass) memset(mass + NE, 0, sizeof(double) * pad);
        if (size) memset(size + NE, 0, sizeof(double) * pad);
        if (delta) memset(delta + NE, 0, sizeof(double) * pad);
        if (soft) memset(soft + NE, 0, sizeof(double) * pad);
        if (quad) memset(quad + 9 * NE, 0, sizeof(double) * 9 * pad);
        if (first)
            for (int64_t i = NE; i < cap; i++) first[i] = -1;
        if (next)
            for (int64_t i = NE; i < cap; i++) next[i] = -1;
    }
    if (quad) memset(quad, 0, sizeof(double) * 9 * t->ntot);
    return TG_OK;
}

tg_status tg_tree_set_walk_config(tg_tree t, int warps_per_block, int first_stack) {
    if (!t || (warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8) ||
        (first_stack != 1024 && first_stack != 4096))
        return TG_ERR_BAD_ARG;
    t->walk_warps = warps_per_block;
    t->walk_stack = first_stack;
    return TG_OK;
}

tg_status tg_tree_free(tg_tree t) {
    destroy(t);
    return TG_OK;
}

tg_status tg_tree_fields(tg_tree t, const double *pos, const double *h, int64_t n, int fields, int quadrupole,
                         double theta, double G, int group_size, int grouping, int order, int precision,
                         const float *theta_per_group, int mem, double *out, void *stream) {
    if (!t || !out) return TG_ERR_BAD_ARG;
    if (grouping != TG_GROUP_BLOCKS && grouping != TG_GROUP_TREE) return TG_ERR_BAD_ARG;
    if (grouping == TG_GROUP_TREE && order != TG_ORDER_TREE) return TG_ERR_BAD_ARG;
    if ((fields & 7) == 0 || (fields & ~7)) return TG_ERR_BAD_ARG;
    if (!(theta > 0) || !valid_group_size(group_size)) return TG_ERR_BAD_ARG;
    if (precision != TG_FP32 && precision != TG_FP64) return TG_ERR_BAD_ARG;
    if (quadrupole && !t->has_quads) return TG_ERR_NO_QUADRUPOLES;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    const int W = field_width(fields);
    int2 *groups = nullptr;
    int *groot = nullptr, *gorder = nullptr;
    int64_t ngroups = 0;
    double *dout = nullptr;
    int64_t nt = 0;
    tg_status rc = TG_OK;
    if (order == TG_ORDER_TREE) {
        nt = t->ntot;
        const int2 *wg = nullptr;
        const int *wr = nullptr;
        if (grouping == TG_GROUP_TREE) {  // kept on the tree, not freed here
            TG_TRY(tree_groups_with_arena(t, group_size, precision == TG_FP64, st));
            wg = t->groups;
            wr = t->group_root;
            ngroups = t->ngroups;
        } else {
            TG_TRY(make_groups(t, t->sys_off, group_size, &groups, &groot, &ngroups, st));
            TG_TRY(make_cost_order(t->coord, groups, ngroups, &gorder, st, t->sort_err));
            wg = groups;
            wr = groot;
        }
        if (mem == TG_MEM_HOST) TG_CUDA(tg::dev_malloc((void **)&dout, sizeof(double) * nt * W, st));
        else dout = out;
        rc = run_walk(t, t->coord, t->soft, nt, wg, wr, gorder, ngroups, t->walk_idx, fields, quadrupole, theta,
                      G, group_size, precision, theta_per_group, nullptr, dout, st);
    } else if (order == TG_ORDER_MORTON || order == TG_ORDER_GIVEN) {
        if (t->nsys != 1 || !pos || n < 1) return TG_ERR_BAD_ARG;
        nt = n;
        DevBuf dp, dh;
        TG_TRY(stage_in(pos, 3 * n, mem, st, dp));
        TG_TRY(stage_in(h, n, mem, st, dh));
        const double *arrs[2] = {dp.ptr, dh.ptr};
        int64_t counts[2] = {3 * n, n};
        TG_TRY(check_finite(arrs, counts, 2, st));
        double *sp = nullptr, *sh = nullptr;
        int64_t *scatter = nullptr;
        if (order == TG_ORDER_MORTON) {
            uint32_t *perm = nullptr;
            TG_CUDA(tg::dev_malloc((void **)&perm, sizeof(uint32_t) * n, st));
            TG_TRY(morton_order_device(dp.ptr, n, perm, st));
            TG_CUDA(tg::dev_malloc((void **)&sp, sizeof(double) * 3 * n, st));
            TG_CUDA(tg::dev_malloc((void **)&sh, sizeof(double) * n, st));
            TG_CUDA(tg::dev_malloc((void **)&scatter, sizeof(int64_t) * n, st));
            { k_gather_targets<<<div_up(n, 256), 256, 0, st>>>(perm, n, dp.ptr, dh.ptr, sp, sh); tg::note_launch(); }
            { k_u32_to_i64<<<div_up(n, 256), 256, 0, st>>>(perm, n, scatter); tg::note_launch(); }
            TG_CUDA(cudaGetLastError());
            TG_CUDA(cudaFreeAsync(perm, st));
        } else {
            TG_CUDA(tg::dev_malloc((void **)&sh, sizeof(double) * n, st));
            if (dh.ptr) TG_CUDA(cudaMemcpyAsync(sh, dh.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            else TG_CUDA(cudaMemsetAsync(sh, 0, sizeof(double) * n, st));
        }
        std::vector<int64_t> toff = {0, n};
        TG_TRY(make_groups(t, toff, group_size, &groups, &groot, &ngroups, st));
        TG_TRY(make_cost_order(sp ? sp : dp.ptr, groups, ngroups, &gorder, st, t->sort_err));
        if (mem == TG_MEM_HOST) TG_CUDA(tg::dev_malloc((void **)&dout, sizeof(double) * nt * W, st));
        else dout = out;
        rc = run_walk(t, sp ? sp : dp.ptr, sh, nt, groups, groot, gorder, ngroups, scatter, fields, quadrupole, theta, G,
                      group_size, precision, theta_per_group, nullptr, dout, st);
        if (sp) cudaFreeAsync(sp, st);
        if (sh) cudaFreeAsync(sh, st);
        if (scatter) cudaFreeAsync(scatter, st);
    } else {
        return TG_ERR_BAD_ARG;
    }
    if (groups) cudaFreeAsync(groups, st);
    if (groot) cudaFreeAsync(groot, st);
    if (gorder) cudaFreeAsync(gorder, st);
    if (rc == TG_OK && mem == TG_MEM_HOST)
        TG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * nt * W, cudaMemcpyDeviceToHost, st));
    if (mem == TG_MEM_HOST && dout) cudaFreeAsync(dout, st);
    TG_CUDA(cudaStreamSynchronize(st));
    return rc;
}

tg_status tg_tree_last_walk_stats(tg_tree t, int64_t *interactions, int64_t *node_tests, int64_t *max_stack,
                                  int64_t *groups) {
    if (!t) return TG_ERR_BAD_ARG;
    if (interactions) *interactions = t->last_stats.interactions;
    if (node_tests) *node_tests = t->last_stats.node_tests;
    if (max_stack) *max_stack = t->last_stats.max_stack;
    if (groups) *groups = t->last_stats.groups;
    return TG_OK;
}

int64_t tg_tree_last_walk_steps(tg_tree t) {
    return t ? t->last_stats.steps : 0;
}

int64_t tg_tree_last_walk_quad_interactions(tg_tree t) {
    return t ? t->last_stats.quad_interactions : 0;
}

double tg_tree_last_walk_kernel_ms(tg_tree t) {
    return t ? (double)t->last_stats.kernel_ms : 0.0;
}

tg_status tg_morton_order(const double *pos, int64_t n, int mem, int64_t *perm, void *stream) {
    if (!perm || (!pos && n > 0) || n < 0) return TG_ERR_BAD_ARG;
    if (n == 0) return TG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf dp;
    TG_TRY(stage_in(pos, 3 * n, mem, st, dp));
    const double *arrs[1] = {dp.ptr};
    int64_t counts[1] = {3 * n};
    TG_TRY(check_finite(arrs, counts, 1, st));
    DevArray<uint32_t> p32(st);
    DevArray<int64_t> p64buf(st);
    TG_CUDA(p32.alloc(n));
    TG_TRY(morton_order_device(dp.ptr, n, p32.p, st));
    int64_t *p64 = perm;
    if (mem == TG_MEM_HOST) {
        TG_CUDA(p64buf.alloc(n));
        p64 = p64buf.p;
    }
    { k_u32_to_i64<<<div_up(n, 256), 256, 0, st>>>(p32.p, n, p64); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    if (mem == TG_MEM_HOST) TG_CUDA(cudaMemcpyAsync(perm, p64, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

tg_status tg_bruteforce(const double *pos_t, const double *h_t, int64_t nt, const double *pos_s, const double *m_s,
                        const double *h_s, int64_t ns, int fields, int mutual, double G, int precision, int mem,
                        double *out, void *stream) {
    if ((fields & 7) == 0 || (fields & ~7) || !out || !pos_s || !m_s || ns < 0) return TG_ERR_BAD_ARG;
    if (precision != TG_FP32 && precision != TG_FP64) return TG_ERR_BAD_ARG;
    if (mutual) {
        pos_t = pos_s;
        h_t = h_s;
        nt = ns;
    }
    if (!pos_t || nt < 0) return TG_ERR_BAD_ARG;
    if (nt == 0) return TG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int W = field_width(fields);
    DevBuf dpt, dht, dps, dms, dhs;
    TG_TRY(stage_in(pos_s, 3 * ns, mem, st, dps));
    TG_TRY(stage_in(m_s, ns, mem, st, dms));
    TG_TRY(stage_in(h_s, ns, mem, st, dhs));
    if (mutual) {
        dpt.ptr = dps.ptr;
        dht.ptr = dhs.ptr;
    } else {
        TG_TRY(stage_in(pos_t, 3 * nt, mem, st, dpt));
        TG_TRY(stage_in(h_t, nt, mem, st, dht));
    }
    double *zt = nullptr, *zs = nullptr;
    if (!dht.ptr) {
        TG_CUDA(tg::dev_malloc((void **)&zt, sizeof(double) * nt, st));
        TG_CUDA(cudaMemsetAsync(zt, 0, sizeof(double) * nt, st));
        dht.ptr = zt;
    }
    if (!dhs.ptr) {
        TG_CUDA(tg::dev_malloc((void **)&zs, sizeof(double) * std::max<int64_t>(ns, 1), st));
        TG_CUDA(cudaMemsetAsync(zs, 0, sizeof(double) * std::max<int64_t>(ns, 1), st));
        dhs.ptr = zs;
        if (mutual) dht.ptr = zs;
    }
    double *dout = out;
    if (mem == TG_MEM_HOST) TG_CUDA(tg::dev_malloc((void **)&dout, sizeof(double) * nt * W, st));
    tg_status rc = run_bruteforce(dpt.ptr, dht.ptr, nt, dps.ptr, dms.ptr, dhs.ptr, ns, fields, mutual, G, precision,
                                  dout, st);
    if (rc == TG_OK && mem == TG_MEM_HOST)
        TG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * nt * W, cudaMemcpyDeviceToHost, st));
    if (mem == TG_MEM_HOST) cudaFreeAsync(dout, st);
    if (zt) cudaFreeAsync(zt, st);
    if (zs) cudaFreeAsync(zs, st);
    TG_CUDA(cudaStreamSynchronize(st));
    return rc;
}

/* ------------------------------------------------------------------------------------------ */
/* Device-resident source sets (the numba-cuda brute-force contexts, cuda.py:737-796).           */

tg_status tg_device_count(int *count) {
    if (!count) return TG_ERR_BAD_ARG;
    *count = 0;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();  // no driver or no device: report zero devices, not an error
        return TG_OK;
    }
    *count = n;
    return TG_OK;
}

tg_status tg_sources_create(const double *pos, const double *m, const double *h, int64_t n, int mem, void *stream,
                            tg_sources *out) {
    if (!out) return TG_ERR_BAD_ARG;
    *out = nullptr;
    if (n < 0 || (n > 0 && (!pos || !m))) return TG_ERR_BAD_ARG;
    if (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tg_sources_s *S = new (std::nothrow) tg_sources_s();
    if (!S) return TG_ERR_OOM;
    S->n = n;
    const int64_t cnt = std::max<int64_t>(n, 1);
    const cudaMemcpyKind kind = mem == TG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    auto fail = [&](tg_status r) {
        tg_sources_free(S);
        return r;
    };
    if (cudaMalloc((void **)&S->pos, sizeof(double) * 3 * cnt) != cudaSuccess ||
        cudaMalloc((void **)&S->m, sizeof(double) * cnt) != cudaSuccess ||
        cudaMalloc((void **)&S->h, sizeof(double) * cnt) != cudaSuccess) {
        cudaGetLastError();
        set_last_error_msg("out of device memory for the source set");
        return fail(TG_ERR_OOM);
    }
    if (n > 0) {
        if (cudaMemcpyAsync(S->pos, pos, sizeof(double) * 3 * n, kind, st) != cudaSuccess ||
            cudaMemcpyAsync(S->m, m, sizeof(double) * n, kind, st) != cudaSuccess ||
            (h ? cudaMemcpyAsync(S->h, h, sizeof(double) * n, kind, st)
               : cudaMemsetAsync(S->h, 0, sizeof(double) * n, st)) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            tg::set_last_error("tg_sources_create", cudaGetLastError());
            return fail(TG_ERR_CUDA);
        }
    }
    *out = S;
    return TG_OK;
}

tg_status tg_sources_bruteforce(tg_sources S, const double *pos_t, const double *h_t, int64_t nt, int fields,
                                double G, int precision, int mem, double *out, void *stream) {
    if (!S || !out || (fields & 7) == 0 || (fields & ~7)) return TG_ERR_BAD_ARG;
    if (precision != TG_FP32 && precision != TG_FP64) return TG_ERR_BAD_ARG;
    if (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf dpt, dht;
    if (!pos_t) {  // the sources themselves, in the target form: r == 0 pairs are skipped
        nt = S->n;
        dpt.ptr = S->pos;
        dht.ptr = S->h;
    } else {
        if (nt < 0) return TG_ERR_BAD_ARG;
        TG_TRY(stage_in(pos_t, 3 * nt, mem, st, dpt));
        TG_TRY(stage_in(h_t, nt, mem, st, dht));
    }
    if (nt == 0) return TG_OK;
    double *zt = nullptr;
    if (!dht.ptr) {
        TG_CUDA(tg::dev_malloc((void **)&zt, sizeof(double) * nt, st));
        TG_CUDA(cudaMemsetAsync(zt, 0, sizeof(double) * nt, st));
        dht.ptr = zt;
    }
    const int W = field_width(fields);
    double *dout = out;
    if (mem == TG_MEM_HOST) TG_CUDA(tg::dev_malloc((void **)&dout, sizeof(double) * nt * W, st));
    tg_status rc = TG_OK;
    if (S->n > 0) {
        rc = run_bruteforce(dpt.ptr, dht.ptr, nt, S->pos, S->m, S->h, S->n, fields, 0, G, precision, dout, st);
    } else {
        TG_CUDA(cudaMemsetAsync(dout, 0, sizeof(double) * nt * W, st));
    }
    if (rc == TG_OK && mem == TG_MEM_HOST)
        TG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * nt * W, cudaMemcpyDeviceToHost, st));
    if (mem == TG_MEM_HOST) cudaFreeAsync(dout, st);
    if (zt) cudaFreeAsync(zt, st);
    TG_CUDA(cudaStreamSynchronize(st));
    return rc;
}

tg_status tg_sources_free(tg_sources S) {
    if (!S) return TG_OK;
    if (S->pos) cudaFree(S->pos);
    if (S->m) cudaFree(S->m);
    if (S->h) cudaFree(S->h);
    delete S;
    return TG_OK;
}

}  // extern "C"
