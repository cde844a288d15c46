// Grouped Barnes-Hut walk (pytreegrav grouped_treewalk.py:163-241 with the per-interaction kernel
// of :45-155), one warp per group of consecutive Morton-ordered targets.
//
// Traversal: the warp pops up to 32 pending nodes from a per-warp stack in shared memory, tests
// them in parallel against the group's bounding box (nearest-corner distance and the group's
// maximum softening, as pytreegrav does), and votes with __ballot_sync: accepted nodes go to the
// interaction list, opened nodes push their node children (contiguous indices) onto the stack and
// append their particle children (a contiguous leaf range) to the interaction list.
// The test runs in FP32 with an error bound; a node inside the bound is re-tested with the exact
// FP64 expression on the tree's FP64 arrays, so the accepted set is exactly pytreegrav's.
//
// Evaluation: every 32 list entries are staged in shared memory as offsets from a group reference
// point (hi/lo float pairs keep near-field offsets exact to FP32 rounding) and swept by all lanes:
// lane = (target, slice): a group of n targets takes P lanes per slice, P the smallest power of two
// >= n (at most group_size), and each of the 32/P slices sweeps its own share of every batch, so
// small groups keep the warp busy. Sources that cannot be
// within any target's softening length (checked once per source against the group box) take the
// point-mass path; the rest take the full softened path. Each lane sums a batch in registers and
// adds the batch total into a Kahan-compensated accumulator.
#include <algorithm>
#include <new>
#include <type_traits>
#include <vector>

#include "tg_tree.cuh"

namespace tg {

constexpr int MAX_WALK_WARPS = 8;  // block shapes of 2, 4 or 8 warps, chosen per tree
constexpr int STACK_SMALL = 1024;  // per-warp node stack; a walk that overflows it is rerun with
constexpr int STACK_LARGE = 4096;  // the large stack (fewer resident warps)
constexpr int ILIST_CAP = 320;
constexpr int NLIST_CAP = 64;

// Integers carried in a traversal record, as the bit pattern of the record's element type.
__device__ __forceinline__ float int_bits(int v, float) { return __int_as_float(v); }
__device__ __forceinline__ double int_bits(int v, double) { return __longlong_as_double((long long)v); }
__device__ __forceinline__ int bits_int(float x) { return __float_as_int(x); }
__device__ __forceinline__ int bits_int(double x) { return (int)__double_as_longlong(x); }

// ---------------------------------------------------------------------------------------------
// Softening kernels (kernel.py:5-75) in the walk's precision.
template <typename T>
__device__ __forceinline__ T force_kernel(T r, T h) {
    if (r > h) return T(1) / (r * r * r);
    T hinv = T(1) / h;
    T q = r * hinv;
    T h3 = hinv * hinv * hinv;
    if (q <= T(0.5)) return (T(10.666666666666666666) + q * q * (T(-38.4) + T(32.0) * q)) * h3;
    return (T(21.333333333333) - T(48.0) * q + T(38.4) * q * q - T(10.666666666667) * q * q * q -
            T(0.066666666667) / (q * q * q)) * h3;
}
template <typename T>
__device__ __forceinline__ T potential_kernel(T r, T h) {
    if (h == T(0)) return T(-1) / r;
    T hinv = T(1) / h;
    T q = r * hinv;
    if (q <= T(0.5)) return (T(-2.8) + q * q * (T(5.33333333333333333) + q * q * (T(6.4) * q - T(9.6)))) * hinv;
    if (q <= T(1))
        return (T(-3.2) + T(0.066666666666666666666) / q +
                q * q * (T(10.666666666666666666666) + q * (T(-16.0) + q * (T(9.6) - T(2.1333333333333333333333) * q)))) *
               hinv;
    return T(-1) / r;
}
template <typename T>
__device__ __forceinline__ T tidal_kernel(T r, T h) {
    if (r > h) {
        T r2 = r * r;
        return T(3) / (r2 * r2 * r);
    }
    T hinv = T(1) / h;
    T hinv2 = hinv * hinv;
    T hinv5 = hinv2 * hinv2 * hinv;
    T q = r * hinv;
    if (q <= T(0.5)) return (T(76.8) - T(96.0) * q) * hinv5;
    T qinv = T(1) / q;
    T qinv3 = qinv * qinv * qinv;
    return (T(48.0) * qinv - T(76.8) + T(32.0) * q - T(0.2) * qinv3 * qinv * qinv) * hinv5;
}

// One MUFU instruction (flush-to-zero; positions here are never denormal).
__device__ __forceinline__ float rsqrt_t(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }

// Two FP32 values in one 64-bit register and the paired (f32x2) arithmetic of this GPU: one issued
// instruction computes both halves, leaving issue slots to other warps' traversal work.
typedef unsigned long long f2;
__device__ __forceinline__ f2 f2_pack(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_rsqrt(f2 x) {
    float a, b;
    f2_unpack(x, a, b);
    return f2_pack(rsqrt_t(a), rsqrt_t(b));
}

// ---------------------------------------------------------------------------------------------
// Arena packing.
__device__ __forceinline__ void split_hi_lo(double x, float &hi, float &lo) { d2f_split(x, hi, lo); }
__device__ __forceinline__ void split_hi_lo(double x, double &hi, double &lo) {
    hi = x;
    lo = 0.0;
}
// FP64 value in the walk precision (integer conversion for FP32).
__device__ __forceinline__ float narrow(double x, float) { return d2f(x); }
__device__ __forceinline__ double narrow(double x, double) { return x; }

__global__ void k_arena_links(int64_t ntot, int64_t mtot, const int64_t *first, const int64_t *next, int4 *link,
                              int64_t *nleaf, int *bad) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mtot) return;
    int64_t f = ntot + j, stop = next[f];
    int fc = -1, nc = 0, nl = 0, steps = 0;
    for (int64_t c = first[f]; c != stop && c >= 0; c = next[c]) {
        if (++steps > 8) {  // an octree node has at most 8 children
            atomicOr(bad, 1);
            break;
        }
        if (c < ntot) nl++;
        else {
            if (nc == 0) fc = (int)(c - ntot);
            else if (c - ntot != fc + nc) atomicOr(bad, 2);  // node children must be consecutive
            nc++;
        }
    }
    if (nc > 0 && (fc < 0 || fc + nc > mtot)) atomicOr(bad, 4);
    link[j] = make_int4(fc, nc, 0, nl);
    nleaf[j] = nl;
}

// Leaf ranges: each node's particle children, in chain order, copied to its range of the leaf
// arrays; the range start also goes into the node's link. Reads particle data only, which is final
// before the moment pass.
template <typename T>
__global__ void k_arena_leaves(int64_t ntot, int64_t mtot, const int64_t *first, const int64_t *next,
                               const double *coord, const double *mass, const double *soft,
                               const int64_t *leaf_start, Arena<T> ar) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mtot) return;
    int64_t f = ntot + j, stop = next[f];
    int64_t ls = leaf_start[j];
    int4 lk = ar.n_link[j];
    lk.z = (int)ls;
    ar.n_link[j] = lk;
    if (ls < 0 || ls + lk.w > ar.n_leaves) {  // leaf ranges from invalid links: nothing written
        atomicOr(ar.bad, 16);
        return;
    }
    int64_t k = ls;
    const int64_t kend = ls + lk.w;
    T hx, hy, hz, lx, ly, lz;
    for (int64_t c = first[f]; c != stop && c >= 0 && k < kend; c = next[c]) {
        if (c < ntot) {
            split_hi_lo(coord[3 * c], hx, lx);
            split_hi_lo(coord[3 * c + 1], hy, ly);
            split_hi_lo(coord[3 * c + 2], hz, lz);
            ar.l_pos[k] = vec4<T>{hx, hy, hz, narrow(mass[c], T(0))};
            ar.l_lo[k] = vec4<T>{lx, ly, lz, narrow(soft[c], T(0))};
            k++;
        }
    }
}

// Node records (centre of mass, mass, h_max, size, Delta, links, quadrupole): after the moment pass.
template <typename T>
__global__ void k_arena_nodes(int64_t ntot, int64_t mtot, const double *coord, const double *mass,
                              const double *soft, const double *size, const double *delta, const double *quad,
                              const float4 *quad32, Arena<T> ar) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mtot) return;
    const int64_t f = ntot + j;
    const int4 lk = ar.n_link[j];
    T hx, hy, hz, lx, ly, lz;
    split_hi_lo(coord[3 * f], hx, lx);
    split_hi_lo(coord[3 * f + 1], hy, ly);
    split_hi_lo(coord[3 * f + 2], hz, lz);
    T hm = narrow(soft[f], T(0));
    ar.n_pos[j] = vec4<T>{hx, hy, hz, narrow(mass[f], T(0))};
    ar.n_lo[j] = vec4<T>{lx, ly, lz, hm};
    const int fc = lk.y > 0 ? lk.x : 0;
    ar.n_trav[2 * j] = vec4<T>{hx, hy, hz, narrow(size[f], T(0))};
    ar.n_trav[2 * j + 1] = vec4<T>{narrow(delta[f], T(0)), hm, int_bits((fc << 4) | lk.y, T(0)),
                                   int_bits((lk.z << 4) | lk.w, T(0))};
    if (ar.n_tol) {  // log form: no underflow for tiny nodes; zero for massless or empty ones
        const float mf = d2f(mass[f]), sf = d2f(size[f]);
        float a3 = 0.f, a2 = 0.f;
        if (mf > 0.f && sf > 0.f) {
            const float lm = log2f(mf), ls = log2f(sf);
            a3 = exp2f(0.2f * (lm + 3.f * ls));
            a2 = exp2f(0.25f * (lm + 2.f * ls));
        }
        ar.n_tol[j] = make_float2(a3, a2);
    }
    if (ar.n_quad) {
        if constexpr (sizeof(T) == 4) {  // FP32 walks: the moment pass's FP32 quadrupoles
            ar.n_quad[2 * j] = quad32[2 * j];
            ar.n_quad[2 * j + 1] = quad32[2 * j + 1];
        } else {
            const double *Q = quad + 9 * j;
            ar.n_quad[2 * j] = vec4<T>{narrow(Q[0], T(0)), narrow(Q[1], T(0)), narrow(Q[2], T(0)), narrow(Q[4], T(0))};
            ar.n_quad[2 * j + 1] = vec4<T>{narrow(Q[5], T(0)), narrow(Q[8], T(0)), T(0), T(0)};
        }
    }
}

// Every particle must be exactly one node's leaf.
__global__ void k_arena_total(const int64_t *ltot, int64_t ntot, int *bad) {
    if (threadIdx.x == 0 && *ltot != ntot) atomicOr(bad, 8);
}

// The arena's topology part: allocation, node links, leaf ranges (validated on the device, see
// k_arena_total) and the leaf records. Needs no moments.
template <typename T>
tg_status build_arena_topology(tg_tree_s *t, Arena<T> &ar, cudaStream_t st) {
    const int64_t M = t->mtot, N = t->ntot;
    ar.n_nodes = M;
    ar.n_leaves = N;
    ar.has_quad = t->has_quads;
    if (M >= (1 << 27) || N >= (1 << 27)) {  // node and leaf indices are packed with 4 count bits
        set_last_error_msg("tree too large for the walk arena (2^27 nodes or particles)");
        return TG_ERR_BAD_ARG;
    }
    TG_CUDA(tg::dev_malloc((void **)&ar.n_pos, sizeof(vec4<T>) * M, st));
    TG_CUDA(tg::dev_malloc((void **)&ar.n_lo, sizeof(vec4<T>) * M, st));
    TG_CUDA(tg::dev_malloc((void **)&ar.n_trav, sizeof(vec4<T>) * 2 * M, st));
    TG_CUDA(tg::dev_malloc((void **)&ar.n_link, sizeof(int4) * M, st));
    if (ar.has_quad) TG_CUDA(tg::dev_malloc((void **)&ar.n_quad, sizeof(vec4<T>) * 2 * M, st));
    if (sizeof(T) == 4) TG_CUDA(tg::dev_malloc((void **)&ar.n_tol, sizeof(float2) * M, st));
    TG_CUDA(tg::dev_malloc((void **)&ar.l_pos, sizeof(vec4<T>) * N, st));
    TG_CUDA(tg::dev_malloc((void **)&ar.l_lo, sizeof(vec4<T>) * N, st));
    int64_t *nleaf = nullptr, *lstart = nullptr, *ltot = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&nleaf, sizeof(int64_t) * M, st));
    TG_CUDA(tg::dev_malloc((void **)&lstart, sizeof(int64_t) * M, st));
    TG_CUDA(tg::dev_malloc((void **)&ltot, sizeof(int64_t), st));
    TG_CUDA(tg::dev_malloc((void **)&ar.bad, sizeof(int), st));
    TG_CUDA(cudaMemsetAsync(ar.bad, 0, sizeof(int), st));
    // validated on the device: the fill writes only in-range leaf ranges, and every walk checks the
    // flag before it reads the arena (no host synchronisation here)
    { k_arena_links<<<div_up(M, 256), 256, 0, st>>>(N, M, t->first, t->next, ar.n_link, nleaf, ar.bad); tg::note_launch(); }
    TG_TRY(exclusive_scan_i64(nleaf, lstart, M, ltot, st));
    { k_arena_total<<<1, 32, 0, st>>>(ltot, N, ar.bad); tg::note_launch(); }
    TG_CUDA(cudaFreeAsync(ltot, st));
    { k_arena_leaves<T><<<div_up(M, 256), 256, 0, st>>>(N, M, t->first, t->next, t->coord, t->mass, t->soft, lstart,
                                                       ar); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaFreeAsync(nleaf, st));
    TG_CUDA(cudaFreeAsync(lstart, st));
    return TG_OK;
}

// The node records, after the moment pass; completes the arena.
template <typename T>
tg_status build_arena_nodes(tg_tree_s *t, Arena<T> &ar, cudaStream_t st) {
    const int64_t M = t->mtot, N = t->ntot;
    if (sizeof(T) == 8 && ar.n_quad) TG_TRY(ensure_quad64(t, st));
    { k_arena_nodes<T><<<div_up(M, 256), 256, 0, st>>>(N, M, t->coord, t->mass, t->soft, t->size, t->delta, t->quad,
                                                      t->quad32, ar); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    ar.built = true;
    return TG_OK;
}

template <typename T>
tg_status build_arena(tg_tree_s *t, Arena<T> &ar, cudaStream_t st) {
    if (ar.built) return TG_OK;
    TG_TRY(build_arena_topology(t, ar, st));
    return build_arena_nodes(t, ar, st);
}

template <typename T>
void free_arena(Arena<T> &ar, cudaStream_t st) {
    if (ar.n_pos) cudaFreeAsync(ar.n_pos, st);
    if (ar.n_lo) cudaFreeAsync(ar.n_lo, st);
    if (ar.n_trav) cudaFreeAsync(ar.n_trav, st);
    if (ar.n_link) cudaFreeAsync(ar.n_link, st);
    if (ar.n_quad) cudaFreeAsync(ar.n_quad, st);
    if (ar.n_tol) cudaFreeAsync(ar.n_tol, st);
    if (ar.l_pos) cudaFreeAsync(ar.l_pos, st);
    if (ar.l_lo) cudaFreeAsync(ar.l_lo, st);
    if (ar.bad) cudaFreeAsync(ar.bad, st);
    ar = Arena<T>();
}
template tg_status build_arena<float>(tg_tree_s *, Arena<float> &, cudaStream_t);
template tg_status build_arena<double>(tg_tree_s *, Arena<double> &, cudaStream_t);
template void free_arena<float>(Arena<float> &, cudaStream_t);
template void free_arena<double>(Arena<double> &, cudaStream_t);

// ---------------------------------------------------------------------------------------------
// Walk kernel.
enum { F_POT = 1, F_ACC = 2, F_TID = 4 };

template <typename T>
struct WalkArgs {
    Arena<T> ar;
    int64_t ntot;
    const double *tc, *ts, *tsize, *tdelta;  // tree FP64 arrays for exact acceptance
    const double *tpos, *th;                   // targets in walk order (FP64)
    const vec4<T> *thi, *tlo;                  // the same split into hi (x, y, z, h) and lo (x, y, z, 0)
    const int64_t *scatter;                    // output row of walk-order target (null: identity)
    const int2 *groups;                        // (first target, count)
    const int *group_root;                     // arena node index of each group's tree root
    const int *group_order;                    // queue position -> group (null: identity)
    int64_t ngroups;
    double theta;
    const float *theta_group;
    // per group error tolerance (null or <= 0: pytreegrav's geometric criterion). A group with a
    // tolerance tau accepts a node once r exceeds both s/theta and (M s^p / tau)^(1/(p+2)) (plus
    // delta), p = 3 with quadrupoles and 2 without: the size of the first neglected multipole term.
    const float *tol_group;
    double G;
    int out_fields;  // requested fields (bits) -> output packing
    int out_w;
    double *out;
    int gs;  // group size (targets per group, divides 32)
    int *queue;
    int *status;
    unsigned long long *stats;  // interactions, node tests, max stack, steps, quadrupole-node interactions
    unsigned *gstats;           // per group (3): point-mass entries, quadrupole entries, nodes tested; or null
    // Small-stack pass: a group that overflows the stack is appended to retry (count in *retry_count)
    // for the large-stack pass instead of failing. Null: overflow is an error.
    int *retry, *retry_count;
    const int *ngroups_dev;  // non-null: the number of groups is read here (the retry pass)
    // Groups walked with a tolerance: each sums, over the nodes it accepts, the first neglected
    // multipole term M s^p / (r - delta)^(p+2) (r the node's distance from the group box), and divides
    // by its targets' RMS acceleration. gerr (or null) receives that estimate per group; a group whose
    // estimate exceeds err_budget (> 0) is appended to rewalk, for a pass at the global theta.
    float err_budget = 0.f;
    float *gerr = nullptr;
    int *rewalk = nullptr, *rewalk_count = nullptr;
    double rewalk_theta = 0.0;  // the global theta of the rewalk pass
    // Heavy groups: with heavy set, a group whose evaluated list entries exceed heavy_budget stops
    // (its partial work taken back) and is appended to heavy, for the split walk (walk_heavy).
    int *heavy = nullptr, *heavy_count = nullptr;
    unsigned heavy_budget = 0;
    // Item mode (the split walk): unit k walks, for group item_group[k], the subtree of item_node[k]
    // (a node; or a particle, ~leaf, taken as one interaction) and writes its unscaled partial sums,
    // 10 components for each of gs target slots, to partial + 10 * gs * k.
    const int *item_group = nullptr, *item_node = nullptr;
    double *partial = nullptr;
    int64_t step_limit = 0;  // traversal steps per group (0: the node count, which always suffices)
    // the arena does not fit in L2: records of pushed nodes, listed leaves and accepted nodes are
    // prefetched into L2 when they are queued, ahead of the step or batch that reads them
    int prefetch = 0;
};

__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

template <typename T, bool QUAD, int STACK>
struct WarpSmem {
    int stack[STACK];
    int ilist[ILIST_CAP];
    int nlist[QUAD ? NLIST_CAP : 1];
    vec4<T> spos[32];   // offsets + mass for the point-mass sweep (near sources: mass 0, far away)
    vec4<T> snear[32];  // offsets + mass of the near sources, swept with softening
    T sh[32];
    vec4<T> sq[QUAD ? 64 : 1];   // quadrupole records of the staged nodes
    double xbox[8];  // the exact test's FP64 group box: min (3), max (3), max softening, theta
};

template <typename T>
struct Acc {
    T v[10];  // pot | ax ay az | txx txy txz tyy tyz tzz
};

template <typename T, int FIELDS>
__device__ __forceinline__ void point_mass(T m, T dx, T dy, T dz, T rinv, Acc<T> &p) {
    T rinv2 = rinv * rinv;
    T mr = m * rinv;
    if (FIELDS & F_POT) p.v[0] -= mr;
    if (FIELDS & (F_ACC | F_TID)) {
        T mr3 = mr * rinv2;
        if (FIELDS & F_ACC) {
            p.v[1] += mr3 * dx;
            p.v[2] += mr3 * dy;
            p.v[3] += mr3 * dz;
        }
        if (FIELDS & F_TID) {
            T q3 = T(3) * mr3 * rinv2;
            T qx = q3 * dx, qy = q3 * dy;
            p.v[4] += qx * dx - mr3;
            p.v[5] += qx * dy;
            p.v[6] += qx * dz;
            p.v[7] += qy * dy - mr3;
            p.v[8] += qy * dz;
            p.v[9] += q3 * dz * dz - mr3;
        }
    }
}

// General interaction (grouped_treewalk.py:74-107): skips r == 0, softened when r < max(h_s, h_t).
template <typename T, int FIELDS>
__device__ __forceinline__ void softened(T m, T hs, T ht_target, T dx, T dy, T dz, T r2, Acc<T> &p) {
    if (!(r2 > T(0))) return;
    T rinv = rsqrt_t(r2);
    T r = r2 * rinv;
    T ht = hs > ht_target ? hs : ht_target;
    if (!(r < ht)) {
        point_mass<T, FIELDS>(m, dx, dy, dz, rinv, p);
        return;
    }
    if (FIELDS & F_POT) p.v[0] += m * potential_kernel(r, ht);
    if (FIELDS & (F_ACC | F_TID)) {
        T K = m * force_kernel(r, ht);
        if (FIELDS & F_ACC) {
            p.v[1] += K * dx;
            p.v[2] += K * dy;
            p.v[3] += K * dz;
        }
        if (FIELDS & F_TID) {
            T Q = m * tidal_kernel(r, ht);
            p.v[4] += Q * dx * dx - K;
            p.v[5] += Q * dx * dy;
            p.v[6] += Q * dx * dz;
            p.v[7] += Q * dy * dy - K;
            p.v[8] += Q * dy * dz;
            p.v[9] += Q * dz * dz - K;
        }
    }
}

// Quadrupole terms of an accepted node (grouped_treewalk.py:109-133).
template <typename T, int FIELDS>
__device__ __forceinline__ void quad_terms(const T *q, T dx, T dy, T dz, T rinv, Acc<T> &p) {
    T rinv2 = rinv * rinv;
    T r5inv = rinv2 * rinv2 * rinv;
    T r7inv = r5inv * rinv2;
    T qxx = q[0], qxy = q[1], qxz = q[2], qyy = q[3], qyz = q[4], qzz = q[5];
    T qdx = qxx * dx + qxy * dy + qxz * dz;
    T qdy = qxy * dx + qyy * dy + qyz * dz;
    T qdz = qxz * dx + qyz * dy + qzz * dz;
    T A = dx * qdx + dy * qdy + dz * qdz;
    if (FIELDS & F_POT) p.v[0] += T(-0.5) * A * r5inv;
    if (FIELDS & F_ACC) {
        T qf = T(2.5) * A * r7inv;
        p.v[1] += qf * dx - qdx * r5inv;
        p.v[2] += qf * dy - qdy * r5inv;
        p.v[3] += qf * dz - qdz * r5inv;
    }
    if (FIELDS & F_TID) {
        T diag = T(-2.5) * A * r7inv;
        T fac = T(17.5) * A * r7inv * rinv2;
        p.v[4] += qxx * r5inv - T(10) * dx * qdx * r7inv + diag + fac * dx * dx;
        p.v[7] += qyy * r5inv - T(10) * dy * qdy * r7inv + diag + fac * dy * dy;
        p.v[9] += qzz * r5inv - T(10) * dz * qdz * r7inv + diag + fac * dz * dz;
        p.v[5] += qxy * r5inv - T(5) * (dx * qdy + dy * qdx) * r7inv + fac * dx * dy;
        p.v[6] += qxz * r5inv - T(5) * (dx * qdz + dz * qdx) * r7inv + fac * dx * dz;
        p.v[8] += qyz * r5inv - T(5) * (dy * qdz + dz * qdy) * r7inv + fac * dy * dz;
    }
}

// Acceleration of an accepted node, monopole and quadrupole together (the sum of point_mass and
// quad_terms for F_ACC): a += dx (m r^-3 + 2.5 A r^-7) - (Q dx) r^-5, with A = dx.Q.dx.
template <typename T>
__device__ __forceinline__ void acc_mono_quad(T m, const T *q, T dx, T dy, T dz, T rinv, Acc<T> &p) {
    T rinv2 = rinv * rinv;
    T r3inv = rinv * rinv2;
    T r5inv = r3inv * rinv2;
    T r7inv = r5inv * rinv2;
    T qdx = q[0] * dx + q[1] * dy + q[2] * dz;
    T qdy = q[1] * dx + q[3] * dy + q[4] * dz;
    T qdz = q[2] * dx + q[4] * dy + q[5] * dz;
    T A = dx * qdx + dy * qdy + dz * qdz;
    T sc = fma(T(2.5) * A, r7inv, m * r3inv);
    p.v[1] = fma(-qdx, r5inv, fma(sc, dx, p.v[1]));
    p.v[2] = fma(-qdy, r5inv, fma(sc, dy, p.v[2]));
    p.v[3] = fma(-qdz, r5inv, fma(sc, dz, p.v[3]));
}

template <int FIELDS>
__device__ __forceinline__ constexpr bool comp(int c) {
    return c == 0 ? (FIELDS & F_POT) : (c <= 3 ? (FIELDS & F_ACC) : (FIELDS & F_TID));
}

// Kahan-compensated add of a batch sum (float); plain add for double.
template <typename T, int FIELDS>
__device__ __forceinline__ void kahan_add(Acc<T> &S, Acc<T> &C, const Acc<T> &b) {
#pragma unroll
    for (int c = 0; c < 10; c++) {
        if (!comp<FIELDS>(c)) continue;
        if (sizeof(T) == 4) {
            T y = b.v[c] - C.v[c];
            T t = S.v[c] + y;
            C.v[c] = (t - S.v[c]) - y;
            S.v[c] = t;
        } else {
            S.v[c] += b.v[c];
        }
    }
}

__device__ __forceinline__ float pow_fifth(float q) { return q > 0.f ? __powf(q, 0.2f) : 0.f; }
__device__ __forceinline__ double pow_fifth(double q) { return q > 0.0 ? pow(q, 0.2) : 0.0; }

// Exact FP64 acceptance, the expression of treewalk.py:22-25 on the group box r_min
// (grouped_treewalk.py:209-231), each operation rounded once.
__device__ __forceinline__ bool accept_exact(int64_t f, const double *tc, const double *ts, const double *tsize,
                                             const double *tdelta, const double bmin[3], const double bmax[3],
                                             double hmax, double theta) {
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double c = tc[3 * f + k];
        d[k] = 0.0;
        if (c < bmin[k]) d[k] = dsub(bmin[k], c);
        else if (c > bmax[k]) d[k] = dsub(c, bmax[k]);
    }
    double r_min = __dsqrt_rn(dadd(dadd(dmul(d[0], d[0]), dmul(d[1], d[1])), dmul(d[2], d[2])));
    double h = pymax(ts[f], hmax);
    double size = tsize[f], delta = tdelta[f];
    double crit = pymax(dadd(ddiv(size, theta), delta), dadd(dadd(h, dmul(size, 0.6)), delta));
    return r_min > crit;
}

// One target's row of the output: G times the requested fields of v (pot | accel(3) | tidal(6 unique
// components, written as the full symmetric 3x3)).
__device__ __forceinline__ void write_fields(double *o, int out_fields, const double *v, double G) {
    int k = 0;
    if (out_fields & F_POT) o[k++] = G * v[0];
    if (out_fields & F_ACC) {
        o[k] = G * v[1];
        o[k + 1] = G * v[2];
        o[k + 2] = G * v[3];
        k += 3;
    }
    if (out_fields & F_TID) {
        const double txx = G * v[4], txy = G * v[5], txz = G * v[6], tyy = G * v[7], tyz = G * v[8], tzz = G * v[9];
        o[k] = txx; o[k + 1] = txy; o[k + 2] = txz;
        o[k + 3] = txy; o[k + 4] = tyy; o[k + 5] = tyz;
        o[k + 6] = txz; o[k + 7] = tyz; o[k + 8] = tzz;
    }
}

// Register caps (registers are granted 8 per thread at a time): the FP32 quadrupole acceleration
// walk with the small stack runs at 72, which with its shared memory lets 7 blocks of 4 warps share
// an SM (6 at 80); the other small-stack walks at 80 (6 blocks of 4 warps, 3 of 8; 81 would round
// to 88 and leave 5 or 2); large-stack walks uncapped.
template <typename T, int FIELDS, bool QUAD, int STACK>
constexpr int walk_reg_cap() {
    if (STACK != STACK_SMALL) return 255;
    return (sizeof(T) == 4 && FIELDS == F_ACC && QUAD) ? 72 : 80;
}
template <typename T, int FIELDS, bool QUAD, int STACK>
__global__ void __launch_bounds__(MAX_WALK_WARPS * 32) __maxnreg__((walk_reg_cap<T, FIELDS, QUAD, STACK>()))
    k_walk(WalkArgs<T> a) {
    extern __shared__ unsigned char smem_raw[];
    WarpSmem<T, QUAD, STACK> &sm = reinterpret_cast<WarpSmem<T, QUAD, STACK> *>(smem_raw)[threadIdx.x >> 5];
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    unsigned long long n_int = 0, n_tests = 0, n_steps = 0, n_qint = 0;
    int max_sp = 0;
    const int64_t ngroups = a.ngroups_dev ? (int64_t)*a.ngroups_dev : a.ngroups;
    if (a.ar.bad && *a.ar.bad) {  // the tree's links did not make a valid arena: read nothing
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(a.status, 1 << TG_ERR_CUDA);
        return;
    }

    for (;;) {
        int g = 0;
        if (lane == 0) g = atomicAdd(a.queue, 1);
        g = __shfl_sync(FULL, g, 0);
        if (g >= ngroups) break;
        const int unit = g;
        int start;  // the node the traversal starts from (an item may be a particle: ~leaf)
        if (a.item_group) {
            start = a.item_node[unit];
            g = a.item_group[unit];
        } else {
            if (a.group_order) g = a.group_order[g];
            start = a.group_root[g];
        }
        const int2 gr = a.groups[g];
        // lanes per target slot: the smallest power of two holding the group (at most a.gs); the
        // other lanes of the warp take interleaved shares of every source batch
        int GS = a.gs;
        while (GS > 1 && (GS >> 1) >= gr.y) GS >>= 1;
        const int tl = lane & (GS - 1);  // target of this lane within the group
        const int slice = lane / GS;     // which share of each batch this lane sums
        const bool valid = tl < gr.y;
        const int64_t t = gr.x + (valid ? tl : 0);
        const vec4<T> thv = a.thi[t], tlv = a.tlo[t];
        const double theta = a.theta_group ? (double)a.theta_group[g] : a.theta;
        // group reference point: the first target's hi part; target offsets from it
        const T gcx = __shfl_sync(FULL, thv.x, 0), gcy = __shfl_sync(FULL, thv.y, 0), gcz = __shfl_sync(FULL, thv.z, 0);
        const T tx = (thv.x - gcx) + tlv.x, ty = (thv.y - gcy) + tlv.y, tz = (thv.z - gcz) + tlv.z;
        const T th = thv.w;
        // group box, relative (for the near-source test) and absolute (for the node tests)
        T rbmin[3] = {tx, ty, tz}, rbmax[3] = {tx, ty, tz};
        T abmin[3] = {thv.x, thv.y, thv.z}, abmax[3] = {thv.x, thv.y, thv.z};
        T hmax_g = th;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                rbmin[k] = fmin(rbmin[k], __shfl_xor_sync(FULL, rbmin[k], o));
                rbmax[k] = fmax(rbmax[k], __shfl_xor_sync(FULL, rbmax[k], o));
                abmin[k] = fmin(abmin[k], __shfl_xor_sync(FULL, abmin[k], o));
                abmax[k] = fmax(abmax[k], __shfl_xor_sync(FULL, abmax[k], o));
            }
            hmax_g = fmax(hmax_g, __shfl_xor_sync(FULL, hmax_g, o));
        }
        // FP64 box for the exact acceptance test, computed on first need and kept in the warp's
        // shared memory (with theta), not in registers through the whole traversal
        bool have_box_d = false;
        if (lane == 0) sm.xbox[7] = theta;
        auto box_d = [&]() {
            double bmin[3], bmax[3], hmax_d;
            double px = a.tpos[3 * t], py = a.tpos[3 * t + 1], pz = a.tpos[3 * t + 2];
            bmin[0] = bmax[0] = px;
            bmin[1] = bmax[1] = py;
            bmin[2] = bmax[2] = pz;
            hmax_d = a.th[t];
#pragma unroll
            for (int o = 16; o; o >>= 1) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    bmin[k] = fmin(bmin[k], __shfl_xor_sync(FULL, bmin[k], o));
                    bmax[k] = fmax(bmax[k], __shfl_xor_sync(FULL, bmax[k], o));
                }
                hmax_d = fmax(hmax_d, __shfl_xor_sync(FULL, hmax_d, o));
            }
            if (lane == 0) {
                for (int k = 0; k < 3; k++) {
                    sm.xbox[k] = bmin[k];
                    sm.xbox[3 + k] = bmax[k];
                }
                sm.xbox[6] = hmax_d;
            }
            __syncwarp();
            have_box_d = true;
        };
        const T gscale = fabs(abmin[0]) + fabs(abmin[1]) + fabs(abmin[2]) + fabs(abmax[0]) + fabs(abmax[1]) +
                         fabs(abmax[2]);
        const T inv_theta = (T)(1.0 / theta);
        const float tolg = a.tol_group ? a.tol_group[g] : 0.f;
        const bool mass_aware = tolg > 0.f;  // warp-uniform
        const bool track_err = mass_aware && (FIELDS & F_ACC) && (a.gerr || a.rewalk);
        float err_est = 0.f;  // this lane's share of the group's truncation estimate
        const T inv_tol = mass_aware ? (T)(1.0 / (double)tolg) : T(0);
        // FP32: a node's mass-aware radius is its stored factor times tol^(-1/(p+2))
        const float tol_k = (sizeof(T) == 4 && mass_aware) ? exp2f(-log2f(tolg) * (QUAD ? 0.2f : 0.25f)) : 0.f;
        const T rel_eps = sizeof(T) == 4 ? T(1e-5) : T(0);
        const T abs_eps = sizeof(T) == 4 ? T(1e-6) : T(0);
        // softening-path threshold: a source whose squared distance to the box exceeds this cannot
        // be within any target's softening length, nor coincide with a target
        const T near_eps = (sizeof(T) == 4 ? T(4e-7) : T(1e-15)) * (gscale + T(1e-30));

        Acc<T> S, C;
#pragma unroll
        for (int c = 0; c < 10; c++) S.v[c] = C.v[c] = T(0);

        // evaluate list entries [0, cnt) of `list` (monopole: nodes >= 0, leaves as ~index)
        // Each slice of lanes sweeps one contiguous chunk of GS staged sources. Sources that may lie
        // within a softening length of the group (or coincide with a target) are staged as
        // zero-mass points far away for the branch-free point-mass sweep and swept separately
        // with the full softened kernel; empty slots of a short batch are staged the same way.
        const T FAR = sizeof(T) == 4 ? T(1e18) : T(1e150);
        auto eval_batch = [&](const int *list, int cnt) {
            bool slow = false;
            vec4<T> st = vec4<T>{FAR, FAR, FAR, T(0)};
            if (lane < cnt) {
                int e = list[lane];
                vec4<T> p, q;
                if (e >= 0) {
                    p = a.ar.n_pos[e];
                    q = a.ar.n_lo[e];
                } else {
                    p = a.ar.l_pos[~e];
                    q = a.ar.l_lo[~e];
                }
                T sx = (p.x - gcx) + q.x, sy = (p.y - gcy) + q.y, sz = (p.z - gcz) + q.z;
                T dx = fmax(fmax(rbmin[0] - sx, sx - rbmax[0]), T(0));
                T dy = fmax(fmax(rbmin[1] - sy, sy - rbmax[1]), T(0));
                T dz = fmax(fmax(rbmin[2] - sz, sz - rbmax[2]), T(0));
                T d2 = dx * dx + dy * dy + dz * dz;
                T hh = q.w > hmax_g ? q.w : hmax_g;
                T lim = hh * T(1.001) + near_eps;
                slow = !(d2 > lim * lim);
                if (slow) {
                    sm.snear[lane] = vec4<T>{sx, sy, sz, p.w};
                    sm.sh[lane] = q.w;
                } else {
                    st = vec4<T>{sx, sy, sz, p.w};
                }
            }
            // potential and/or acceleration with groups of 2 or more targets: sources staged as pairs
            // [x x y y] [z z m m] for the paired sweep; otherwise one 16-byte word per source. (The
            // monopole walk of both fields together measured 2% slower paired: it stays unpaired.) The
            // tidal tensor alone is paired as well.
            bool paired = false;
            if constexpr (sizeof(T) == 4 && (FIELDS == F_TID || ((FIELDS & F_TID) == 0 &&
                                                                  (QUAD || FIELDS != (F_POT | F_ACC)))))
                paired = GS >= 2;
            if (paired) {
                float *o = reinterpret_cast<float *>(sm.spos) + 8 * (lane >> 1) + (lane & 1);
                o[0] = (float)st.x;
                o[2] = (float)st.y;
                o[4] = (float)st.z;
                o[6] = (float)st.w;
            } else {
                sm.spos[lane] = st;
            }
            const unsigned slowmask = __ballot_sync(FULL, slow);
            __syncwarp();
            Acc<T> b;
#pragma unroll
            for (int c = 0; c < 10; c++) b.v[c] = T(0);
            const vec4<T> *chunk = sm.spos + slice * GS;
            if (paired) {
                const f2 TX = f2_pack((float)tx, (float)tx), TY = f2_pack((float)ty, (float)ty);
                const f2 TZ = f2_pack((float)tz, (float)tz);
                // even and odd sources summed apart (bit pattern 0 is +0.0f); ph sums m/r; t0..t5 the
                // tidal tensor's xx xy xz yy yz zz
                f2 ax = 0, ay = 0, az = 0, ph = 0, t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0;
                const f2 C3 = f2_pack(3.f, 3.f);
                const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(sm.spos) + 2 * ((slice * GS) >> 1);
#pragma unroll 4
                for (int i = 0; i < (GS >> 1); i++) {
                    const ulonglong2 w0 = src[2 * i], w1 = src[2 * i + 1];
                    const f2 dx = f2_sub(w0.x, TX), dy = f2_sub(w0.y, TY), dz = f2_sub(w1.x, TZ);
                    const f2 rinv = f2_rsqrt(f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx))));
                    const f2 mr = f2_mul(w1.y, rinv);
                    if constexpr ((FIELDS & F_POT) != 0) ph = f2_add(ph, mr);
                    if constexpr ((FIELDS & F_ACC) != 0) {
                        const f2 mr3 = f2_mul(mr, f2_mul(rinv, rinv));
                        ax = f2_fma(mr3, dx, ax);
                        ay = f2_fma(mr3, dy, ay);
                        az = f2_fma(mr3, dz, az);
                    }
                    if constexpr ((FIELDS & F_TID) != 0) {  // T_ab += 3 m r^-5 d_a d_b - delta_ab m r^-3
                        const f2 u = f2_mul(rinv, rinv);
                        const f2 mr3 = f2_mul(mr, u);
                        const f2 q3 = f2_mul(f2_mul(mr3, C3), u);
                        const f2 qx = f2_mul(q3, dx), qy = f2_mul(q3, dy);
                        t0 = f2_sub(f2_fma(qx, dx, t0), mr3);
                        t1 = f2_fma(qx, dy, t1);
                        t2 = f2_fma(qx, dz, t2);
                        t3 = f2_sub(f2_fma(qy, dy, t3), mr3);
                        t4 = f2_fma(qy, dz, t4);
                        t5 = f2_sub(f2_fma(f2_mul(q3, dz), dz, t5), mr3);
                    }
                }
                float h0, h1;
                if constexpr ((FIELDS & F_POT) != 0) {
                    f2_unpack(ph, h0, h1);
                    b.v[0] = -(T)(h0 + h1);
                }
                if constexpr ((FIELDS & F_TID) != 0) {
                    const f2 tt[6] = {t0, t1, t2, t3, t4, t5};
#pragma unroll
                    for (int c = 0; c < 6; c++) {
                        f2_unpack(tt[c], h0, h1);
                        b.v[4 + c] = (T)(h0 + h1);
                    }
                }
                if constexpr ((FIELDS & F_ACC) != 0) {
                    f2_unpack(ax, h0, h1);
                    b.v[1] = (T)(h0 + h1);
                    f2_unpack(ay, h0, h1);
                    b.v[2] = (T)(h0 + h1);
                    f2_unpack(az, h0, h1);
                    b.v[3] = (T)(h0 + h1);
                }
            } else if (GS == 32) {
#pragma unroll 16
                for (int i = 0; i < 32; i++) {
                    vec4<T> s = chunk[i];
                    T dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
                    point_mass<T, FIELDS>(s.w, dx, dy, dz, rsqrt_t(dx * dx + dy * dy + dz * dz), b);
                }
            } else {
#pragma unroll 4
                for (int i = 0; i < GS; i++) {
                    vec4<T> s = chunk[i];
                    T dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
                    point_mass<T, FIELDS>(s.w, dx, dy, dz, rsqrt_t(dx * dx + dy * dy + dz * dz), b);
                }
            }
            const unsigned chunk_bits = GS == 32 ? FULL : ((1u << GS) - 1u) << (slice * GS);
            for (unsigned mk = slowmask & chunk_bits; mk; mk &= mk - 1) {
                int k = __ffs(mk) - 1;
                vec4<T> s = sm.snear[k];
                T dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
                softened<T, FIELDS>(s.w, sm.sh[k], th, dx, dy, dz, dx * dx + dy * dy + dz * dz, b);
            }
            __syncwarp();
            kahan_add<T, FIELDS>(S, C, b);
            n_int += (unsigned long long)cnt * (unsigned long long)gr.y;
        };
        // Quadrupole acceleration sweep with paired arithmetic (FP32, groups of 2 or more targets).
        // Sources are staged as pairs (2p, 2p + 1), each 16-byte word holding one quantity of both:
        // [x x y y] [z z m m] [q0 q0 q1 q1] [q2 q2 q3 q3] [q4 q4 q5 q5], the quadrupole negated. Per pair:
        // a += r^-5 (t dx - Q dx) with t = m r^2 + 2.5 A r^-2 and A = dx.Q.dx, the same expansion as
        // acc_mono_quad rearranged. The two halves sum the even and the odd sources separately.
        auto eval_nodes_paired = [&](const int *list, int cnt) {
            float *buf = reinterpret_cast<float *>(sm.spos);
            {
                float v[10] = {(float)FAR, (float)FAR, (float)FAR, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (lane < cnt) {
                    const int e = list[lane];
                    const vec4<T> p = a.ar.n_pos[e], q = a.ar.n_lo[e];
                    const vec4<T> qa = a.ar.n_quad[2 * e], qb = a.ar.n_quad[2 * e + 1];
                    v[0] = (p.x - gcx) + q.x;
                    v[1] = (p.y - gcy) + q.y;
                    v[2] = (p.z - gcz) + q.z;
                    v[3] = p.w;
                    v[4] = -qa.x; v[5] = -qa.y; v[6] = -qa.z; v[7] = -qa.w; v[8] = -qb.x; v[9] = -qb.y;
                }
                float *o = buf + 20 * (lane >> 1) + (lane & 1);
#pragma unroll
                for (int k = 0; k < 10; k++) o[2 * k] = v[k];
            }
            __syncwarp();
            const f2 TX = f2_pack(tx, tx), TY = f2_pack(ty, ty), TZ = f2_pack(tz, tz);
            const f2 C25 = f2_pack(-2.5f, -2.5f), CH = f2_pack(-0.5f, -0.5f);
            // two partial sums each (bit pattern 0 is +0.0f, +0.0f); ph sums m/r + A/(2 r^5) = -phi;
            // t0..t5 the tidal tensor's xx xy xz yy yz zz
            f2 ax = 0, ay = 0, az = 0, ph = 0, t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0;
            const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(buf) + 5 * ((slice * GS) >> 1);
#pragma unroll 4
            for (int i = 0; i < (GS >> 1); i++) {
                const ulonglong2 w0 = src[5 * i], w1 = src[5 * i + 1], w2 = src[5 * i + 2], w3 = src[5 * i + 3],
                                 w4 = src[5 * i + 4];
                const f2 dx = f2_sub(w0.x, TX), dy = f2_sub(w0.y, TY), dz = f2_sub(w1.x, TZ);
                const f2 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
                const f2 rinv = f2_rsqrt(r2);
                const f2 u = f2_mul(rinv, rinv);
                const f2 r5 = f2_mul(f2_mul(rinv, u), u);
                // n = -Q dx from the negated quadrupole; A' = dx.n = -A
                const f2 nx = f2_fma(w3.x, dz, f2_fma(w2.y, dy, f2_mul(w2.x, dx)));
                const f2 ny = f2_fma(w4.x, dz, f2_fma(w3.y, dy, f2_mul(w2.y, dx)));
                const f2 nz = f2_fma(w4.y, dz, f2_fma(w4.x, dy, f2_mul(w3.x, dx)));
                const f2 A = f2_fma(dz, nz, f2_fma(dy, ny, f2_mul(dx, nx)));
                // potential: m/r - (-A)/(2 r^5) summed, negated at the end (-m/r - A/(2 r^5))
                if constexpr ((FIELDS & F_POT) != 0) ph = f2_fma(f2_mul(A, CH), r5, f2_fma(w1.y, rinv, ph));
                if constexpr ((FIELDS & F_ACC) != 0) {
                    const f2 t = f2_fma(f2_mul(A, C25), u, f2_mul(w1.y, r2));
                    ax = f2_fma(r5, f2_fma(t, dx, nx), ax);
                    ay = f2_fma(r5, f2_fma(t, dy, ny), ay);
                    az = f2_fma(r5, f2_fma(t, dz, nz), az);
                }
                if constexpr ((FIELDS & F_TID) != 0) {
                    // monopole + quadrupole, with n = -Q dx, A = dx.n and the staged w = -Q:
                    // T_ab += g d_a d_b - w_ab r^-5 + 5 r^-7 (d_a n_b + d_b n_a) + delta_ab hd,
                    // g = r^-2 (3 m r^-3 - 17.5 A r^-7), hd = 2.5 A r^-7 - m r^-3
                    const f2 r7 = f2_mul(r5, u);
                    const f2 mr3 = f2_mul(w1.y, f2_mul(rinv, u));
                    const f2 Ar7 = f2_mul(A, r7);
                    const f2 g = f2_mul(f2_fma(Ar7, f2_pack(-17.5f, -17.5f), f2_mul(mr3, f2_pack(3.f, 3.f))), u);
                    const f2 hd = f2_sub(f2_mul(Ar7, f2_pack(2.5f, 2.5f)), mr3);
                    const f2 s5 = f2_mul(r7, f2_pack(5.f, 5.f)), s10 = f2_mul(r7, f2_pack(10.f, 10.f));
                    const f2 nr5 = f2_mul(r5, f2_pack(-1.f, -1.f));
                    t0 = f2_add(f2_fma(w2.x, nr5, f2_fma(s10, f2_mul(dx, nx), f2_fma(g, f2_mul(dx, dx), t0))), hd);
                    t1 = f2_fma(w2.y, nr5, f2_fma(s5, f2_fma(dx, ny, f2_mul(dy, nx)), f2_fma(g, f2_mul(dx, dy), t1)));
                    t2 = f2_fma(w3.x, nr5, f2_fma(s5, f2_fma(dx, nz, f2_mul(dz, nx)), f2_fma(g, f2_mul(dx, dz), t2)));
                    t3 = f2_add(f2_fma(w3.y, nr5, f2_fma(s10, f2_mul(dy, ny), f2_fma(g, f2_mul(dy, dy), t3))), hd);
                    t4 = f2_fma(w4.x, nr5, f2_fma(s5, f2_fma(dy, nz, f2_mul(dz, ny)), f2_fma(g, f2_mul(dy, dz), t4)));
                    t5 = f2_add(f2_fma(w4.y, nr5, f2_fma(s10, f2_mul(dz, nz), f2_fma(g, f2_mul(dz, dz), t5))), hd);
                }
            }
            __syncwarp();
            Acc<T> b;
#pragma unroll
            for (int c = 0; c < 10; c++) b.v[c] = T(0);
            float h0, h1;
            if constexpr ((FIELDS & F_POT) != 0) {
                f2_unpack(ph, h0, h1);
                b.v[0] = -(h0 + h1);
            }
            if constexpr ((FIELDS & F_TID) != 0) {
                const f2 tt[6] = {t0, t1, t2, t3, t4, t5};
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    f2_unpack(tt[c], h0, h1);
                    b.v[4 + c] = h0 + h1;
                }
            }
            if constexpr ((FIELDS & F_ACC) != 0) {
                f2_unpack(ax, h0, h1);
                b.v[1] = h0 + h1;
                f2_unpack(ay, h0, h1);
                b.v[2] = h0 + h1;
                f2_unpack(az, h0, h1);
                b.v[3] = h0 + h1;
            }
            kahan_add<T, FIELDS>(S, C, b);
            n_int += (unsigned long long)cnt * (unsigned long long)gr.y;
            n_qint += (unsigned long long)cnt * (unsigned long long)gr.y;
        };
        auto eval_nodes = [&](const int *list, int cnt) {
            if constexpr (sizeof(T) == 4 && ((FIELDS & F_TID) == 0 || FIELDS == F_TID)) {
                if (GS >= 2) {
                    eval_nodes_paired(list, cnt);
                    return;
                }
            }
            vec4<T> st = vec4<T>{FAR, FAR, FAR, T(0)}, q0 = vec4<T>{T(0), T(0), T(0), T(0)}, q1 = q0;
            if (lane < cnt) {
                int e = list[lane];
                vec4<T> p = a.ar.n_pos[e], q = a.ar.n_lo[e];
                q0 = a.ar.n_quad[2 * e];
                q1 = a.ar.n_quad[2 * e + 1];
                st = vec4<T>{(p.x - gcx) + q.x, (p.y - gcy) + q.y, (p.z - gcz) + q.z, p.w};
            }
            sm.spos[lane] = st;
            sm.sq[2 * lane] = q0;
            sm.sq[2 * lane + 1] = q1;
            __syncwarp();
            Acc<T> b;
#pragma unroll
            for (int c = 0; c < 10; c++) b.v[c] = T(0);
            const int k0 = slice * GS;
#pragma unroll 4
            for (int i = 0; i < GS; i++) {
                vec4<T> s = sm.spos[k0 + i];
                vec4<T> qa = sm.sq[2 * (k0 + i)], qb = sm.sq[2 * (k0 + i) + 1];
                T qv[6] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y};
                T dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
                T rinv = rsqrt_t(dx * dx + dy * dy + dz * dz);
                if (FIELDS == F_ACC) {
                    acc_mono_quad(s.w, qv, dx, dy, dz, rinv, b);
                } else {
                    point_mass<T, FIELDS>(s.w, dx, dy, dz, rinv, b);
                    quad_terms<T, FIELDS>(qv, dx, dy, dz, rinv, b);
                }
            }
            __syncwarp();
            kahan_add<T, FIELDS>(S, C, b);
            n_int += (unsigned long long)cnt * (unsigned long long)gr.y;
            n_qint += (unsigned long long)cnt * (unsigned long long)gr.y;
        };

        unsigned g_mono = 0, g_quad = 0, g_tests = 0, g_steps = 0;  // this group's counters (warp-uniform)
        int sp = 1, ni = 0, nn = 0;
        if (start >= 0) {
            if (lane == 0) sm.stack[0] = start;
        } else {  // an item that is one particle
            if (lane == 0) sm.ilist[0] = start;
            sp = 0;
            ni = 1;
        }
        __syncwarp();
        bool overflow = false, runaway = false, heavy = false;
        // a traversal tests every node at most once, and each step tests at least one
        int64_t steps_left = a.step_limit > 0 && a.step_limit < a.ar.n_nodes + 2 ? a.step_limit : a.ar.n_nodes + 2;
        for (;;) {
            if (--steps_left < 0) {
                runaway = true;
                break;
            }
            if (sp > 0) {
                n_steps++;
                g_steps++;
                const int cnt = min(sp, 32);
                g_tests += cnt;
                const int node = lane < cnt ? sm.stack[sp - 1 - lane] : -1;
                sp -= cnt;
                bool acc = false, unsure = false;
                vec4<T> r1 = vec4<T>{T(0), T(0), T(0), T(0)};
                if (node >= 0) {
                    n_tests++;
                    const vec4<T> p = a.ar.n_trav[2 * node];
                    r1 = a.ar.n_trav[2 * node + 1];
                    float2 tq = make_float2(0.f, 0.f);
                    if constexpr (sizeof(T) == 4) {
                        if (mass_aware) tq = a.ar.n_tol[node];  // issued with the traversal record
                    }
                    T dx = fmax(fmax(abmin[0] - p.x, p.x - abmax[0]), T(0));
                    T dy = fmax(fmax(abmin[1] - p.y, p.y - abmax[1]), T(0));
                    T dz = fmax(fmax(abmin[2] - p.z, p.z - abmax[2]), T(0));
                    T r2 = dx * dx + dy * dy + dz * dz;
                    T h = r1.y > hmax_g ? r1.y : hmax_g;
                    T c1 = p.w * inv_theta + r1.x, c2 = h + T(0.6) * p.w + r1.x;
                    T msp = T(0);  // M s^p of the node (tolerance test only)
                    if (mass_aware) {
                        if constexpr (sizeof(T) == 4) {
                            const float av = QUAD ? tq.x : tq.y;
                            const float av2 = av * av;
                            msp = QUAD ? av2 * av2 * av : av2 * av2;
                            c1 = fmax(p.w * inv_theta, av * tol_k) + r1.x;
                        } else {
                            msp = a.ar.n_pos[node].w * (QUAD ? p.w * p.w * p.w : p.w * p.w);
                            const T q = msp * inv_tol;
                            const T rc = QUAD ? pow_fifth(q) : sqrt(sqrt(q));
                            c1 = fmax(p.w * inv_theta, rc) + r1.x;
                        }
                    }
                    T crit = c1 > c2 ? c1 : c2;
                    // FP32 error bound: node positions near the boundary are within gscale + 2 crit of
                    // the origin, so the relative term covers their rounding
                    T tol = rel_eps * crit + abs_eps * gscale;
                    T hiq = crit + tol, loq = crit - tol;
                    if (mass_aware) {  // no pytreegrav decision to reproduce
                        acc = r2 > crit * crit;
                        if (acc && track_err) {  // r - delta > rc >= 0 here; an estimate: approximate ops
                            const float d = (float)r2 * rsqrt_t((float)r2) - (float)r1.x, d2 = d * d;
                            err_est += __fdividef((float)msp, QUAD ? d2 * d2 * d : d2 * d2);
                        }
                    }
                    else if (sizeof(T) == 8) unsure = true;
                    else if (r2 > hiq * hiq) acc = true;
                    else if (loq > T(0) && r2 < loq * loq) acc = false;
                    else unsure = true;
                }
                if (__any_sync(FULL, unsure)) {
                    if (!have_box_d) box_d();
                    if (unsure)
                        acc = accept_exact(a.ntot + node, a.tc, a.ts, a.tsize, a.tdelta, sm.xbox, sm.xbox + 3,
                                           sm.xbox[6], sm.xbox[7]);
                }
                const bool opn = node >= 0 && !acc;
                const int cbits = opn ? bits_int(r1.z) : 0, lbits = opn ? bits_int(r1.w) : 0;
                const unsigned am = __ballot_sync(FULL, acc);
                if (QUAD) {
                    if (acc) sm.nlist[nn + __popc(am & lt)] = node;
                    nn += __popc(am);
                } else {
                    if (acc) sm.ilist[ni + __popc(am & lt)] = node;
                    ni += __popc(am);
                }
                const int nc = cbits & 15, nl = lbits & 15;
                const int both = warp_inclusive_scan(nc | (nl << 16));  // both counts in one scan
                const int sc = both & 0xffff, sl = both >> 16;
                const int tot = __shfl_sync(FULL, both, 31);
                const int totc = tot & 0xffff, totl = tot >> 16;
                if (sp + totc > STACK) {
                    overflow = true;
                    break;
                }
                const int fc = cbits >> 4, ls = lbits >> 4;
                for (int j = 0, o = sp + sc - nc; j < nc; j++) sm.stack[o + j] = fc + j;
                for (int j = 0, o = ni + sl - nl; j < nl; j++) sm.ilist[o + j] = ~(ls + j);
                if (a.prefetch) {  // warp-uniform; records are 16 or 32 bytes, lines 128
                    if (nc > 0) {
                        prefetch_l2(a.ar.n_trav + 2 * fc);
                        if (nc > 2) prefetch_l2(a.ar.n_trav + 2 * (fc + nc - 1));
                        if constexpr (sizeof(T) == 4) {
                            if (mass_aware) prefetch_l2(a.ar.n_tol + fc);
                        }
                    }
                    if (nl > 0) {
                        prefetch_l2(a.ar.l_pos + ls);
                        prefetch_l2(a.ar.l_lo + ls);
                    }
                    if (acc) {
                        prefetch_l2(a.ar.n_pos + node);
                        prefetch_l2(a.ar.n_lo + node);
                        if (QUAD) prefetch_l2(a.ar.n_quad + 2 * node);
                    }
                }
                sp += totc;
                ni += totl;
                max_sp = max(max_sp, sp);
                __syncwarp();
            }
            while (ni >= 32) {
                eval_batch(sm.ilist + ni - 32, 32);
                ni -= 32;
                g_mono += 32;
            }
            if (QUAD) {
                while (nn >= 32) {
                    eval_nodes(sm.nlist + nn - 32, 32);
                    nn -= 32;
                    g_quad += 32;
                }
            }
            if (sp == 0) break;
            if (a.heavy && g_mono + g_quad > a.heavy_budget) {  // warp-uniform
                heavy = true;
                break;
            }
        }
        if ((overflow && a.retry) || heavy) {
            // handed to the large-stack pass or to the split walk; its counts so far are taken back
            // so the statistics count the group once
            if (lane == 0) {
                if (heavy) a.heavy[atomicAdd(a.heavy_count, 1)] = g;
                else a.retry[atomicAdd(a.retry_count, 1)] = g;
                n_tests -= g_tests;
            }
            n_int -= (unsigned long long)(g_mono + g_quad) * (unsigned long long)gr.y;
            n_qint -= (unsigned long long)g_quad * (unsigned long long)gr.y;
            n_steps -= g_steps;
            __syncwarp();
            continue;
        }
        if (overflow || runaway) {
            if (lane == 0) atomicOr(a.status, 1 << (overflow ? TG_ERR_STACK_OVERFLOW : TG_ERR_ITER_LIMIT));
            __syncwarp();
            continue;
        }
        if (ni > 0) eval_batch(sm.ilist, ni);
        if (QUAD && nn > 0) eval_nodes(sm.nlist, nn);
        g_mono += ni;
        g_quad += QUAD ? nn : 0;
        if (a.gstats && lane == 0) {
            a.gstats[3 * g] = g_mono;
            a.gstats[3 * g + 1] = g_quad;
            a.gstats[3 * g + 2] = g_tests;
        }

        // combine the slices of each target and write G * field in the caller's order
#pragma unroll
        for (int c = 0; c < 10; c++) {
            if (!comp<FIELDS>(c)) continue;
            for (int o = GS; o < 32; o <<= 1) {
                S.v[c] += __shfl_xor_sync(FULL, S.v[c], o);
                C.v[c] += __shfl_xor_sync(FULL, C.v[c], o);
            }
        }
        if (track_err) {  // warp-uniform
            float e = err_est, a2 = 0.f;
            if (slice == 0 && valid) {
                const float ax = (float)(S.v[1] - C.v[1]), ay = (float)(S.v[2] - C.v[2]), az = (float)(S.v[3] - C.v[3]);
                a2 = ax * ax + ay * ay + az * az;
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                e += __shfl_xor_sync(FULL, e, o);
                a2 += __shfl_xor_sync(FULL, a2, o);
            }
            const float rms = sqrtf(a2 / (float)gr.y);
            const float eta = rms > 0.f ? e / rms : (e > 0.f ? INFINITY : 0.f);
            if (lane == 0) {
                if (a.gerr) a.gerr[g] = eta;
                if (a.rewalk && a.err_budget > 0.f && !(eta <= a.err_budget)) a.rewalk[atomicAdd(a.rewalk_count, 1)] = g;
            }
        }
        if (slice == 0 && valid) {
            double v[10];
#pragma unroll
            for (int c = 0; c < 10; c++) v[c] = comp<FIELDS>(c) ? (double)S.v[c] - (double)C.v[c] : 0.0;
            if (a.partial) {  // an item of a split walk: unscaled partial sums of this target slot
                double *o = a.partial + ((int64_t)unit * a.gs + tl) * 10;
#pragma unroll
                for (int c = 0; c < 10; c++) o[c] = v[c];
            } else {
                const int64_t row = a.scatter ? a.scatter[t] : t;
                write_fields(a.out + row * a.out_w, a.out_fields, v, a.G);
            }
        }
        __syncwarp();
    }
    // statistics (interactions are counted per batch entry; each covers the group's targets)
    if (lane == 0 && a.stats) {
        atomicAdd(a.stats + 0, n_int);
        atomicMax(a.stats + 2, (unsigned long long)max_sp);
        atomicAdd(a.stats + 3, n_steps);
        atomicAdd(a.stats + 4, n_qint);
    }
    unsigned long long tests = n_tests;
    for (int o = 16; o; o >>= 1) tests += __shfl_xor_sync(FULL, tests, o);
    if (lane == 0 && a.stats) atomicAdd(a.stats + 1, tests);
}

__global__ void k_make_groups(const int64_t *sys_off, int nsys, int gs, const int64_t *group_off, const int *sys_root,
                              int2 *groups, int *group_root) {
    int s = blockIdx.x;
    if (s >= nsys) return;
    int64_t a = sys_off[s], b = sys_off[s + 1];
    int64_t g0 = group_off[s];
    for (int64_t t = a + (int64_t)threadIdx.x * gs; t < b; t += (int64_t)blockDim.x * gs) {
        int64_t g = g0 + (t - a) / gs;
        groups[g] = make_int2((int)t, (int)((b - t) < gs ? (b - t) : gs));
        group_root[g] = sys_root[s];
    }
}

// Engine grouping: groups are taken from the tree, so a group never straddles a jump of the Morton
// curve. A system root with at most G particles is one group. Every node with more than G
// particles emits its children, in order, packed greedily into runs of at most G particles; a child
// with more than G particles breaks the run (it emits its own children), and a child joins the run
// only if the run's bounding box stays clear of every such large sibling's cell -- a group whose
// box reached into a dense sibling would open that sibling down to its particles.
// A node with more than G particles, queued by k_tree_groups_mark with its children in chain order.
struct LargeNode {
    int64_t child[8];
    int64_t node;  // node index j (arena element ntot + j)
    int root;      // its system's root node
    int nch;
};

// One thread per node: a system root with at most G particles is one group; a node with more than
// G particles is queued, children gathered here (their chain is walked once, by every such node's
// thread at the same time), for k_tree_groups_large.
__global__ void k_tree_groups_mark(int64_t ntot, int64_t mtot, const int2 *node_range, const int64_t *first,
                                   const int64_t *next, const int64_t *parent, int G, const int64_t *sys_off,
                                   const int64_t *sys_node_off, int nsys, int2 *groups, int *group_root,
                                   int *group_node, unsigned long long *count, LargeNode *large, int *nlarge) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = j < mtot;
    int2 r = make_int2(0, 0);
    int root = 0;
    if (valid) {
        r = node_range[j];
        int s = 0;
        if (nsys > 1) {
            int lo = 0, hi = nsys;
            while (hi - lo > 1) {
                int mid = (lo + hi) >> 1;
                if (sys_off[mid] <= r.x) lo = mid;
                else hi = mid;
            }
            s = lo;
        }
        root = (int)sys_node_off[s];
        if (r.y - r.x <= G && parent[ntot + j] < 0) {
            unsigned long long q = atomicAdd(count, 1ull);
            groups[q] = make_int2(r.x, r.y - r.x);
            group_root[q] = root;
            group_node[q] = (int)j;
        }
    }
    const bool big = valid && r.y - r.x > G;
    const unsigned bm = __ballot_sync(FULL, big);
    if (!big) return;
    const int leader = __ffs(bm) - 1;
    int base = 0;
    if (lane_id() == leader) base = atomicAdd(nlarge, __popc(bm));
    base = __shfl_sync(bm, base, leader);
    LargeNode &e = large[base + __popc(bm & lanemask_lt())];
    const int64_t f = ntot + j, stop = next[f];
    int nch = 0;
    for (int64_t c = first[f]; c != stop && c >= 0 && nch < 8; c = next[c]) e.child[nch++] = c;
    e.node = j;
    e.root = root;
    e.nch = nch;
}

// Order-preserving integer image of a double (not NaN): u(a) <= u(b) exactly when a <= b, with -0.0
// taken as +0.0 (the two compare equal). Boxes are reduced and compared in this form, on the
// integer units: FP64 min/max/compare run on GB300's narrow FP64 pipe.
__device__ __forceinline__ unsigned long long order_key(double x) {
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ull) b = 0;
    b ^= (b >> 63) & 0x7fffffffffffffffll;
    return (unsigned long long)b ^ 0x8000000000000000ull;
}
__device__ __forceinline__ unsigned long long warp_min_key(unsigned long long u) {
    const unsigned hi = __reduce_min_sync(FULL, (unsigned)(u >> 32));
    const unsigned lo = __reduce_min_sync(FULL, (unsigned)(u >> 32) == hi ? (unsigned)u : 0xffffffffu);
    return ((unsigned long long)hi << 32) | lo;
}
__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long u) {
    const unsigned hi = __reduce_max_sync(FULL, (unsigned)(u >> 32));
    const unsigned lo = __reduce_max_sync(FULL, (unsigned)(u >> 32) == hi ? (unsigned)u : 0u);
    return ((unsigned long long)hi << 32) | lo;
}

// The groups inside one queued node, one warp per node (a persistent grid over the queue): every
// lane holds the same decisions; lane q keeps child q, and each small child's particle box is a
// warp reduction (lane p loads the child's particle p, all children's loads issued together).
// Boxes and cells are compared as order keys, which decides exactly as the FP64 comparisons do.
__global__ void k_tree_groups_large(int64_t ntot, const int2 *node_range, const double *cell, const double *size,
                                    const double *coord, int G, const LargeNode *large, const int *nlarge,
                                    int2 *groups, int *group_root, int *group_node, unsigned long long *count) {
    typedef unsigned long long u64;
    const int lane = lane_id();
    const int n = *nlarge;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += nwarps) {
        const LargeNode &e = large[w];
        const int64_t j = e.node;
        const int root = e.root;
        const int nch = e.nch;
        // this node's groups, collected on lanes 0.. and written with one atomic
        int nemit = 0, my_glo = 0, my_gcnt = 0;
        auto emit = [&](int lo, int cnt) {
            if (lane == nemit) {
                my_glo = lo;
                my_gcnt = cnt;
            }
            nemit++;
        };
        int my_lo = 0, my_hi = 0;
        int64_t my_c = -1;
        if (lane < nch) {
            my_c = e.child[lane];
            if (my_c < ntot) {
                my_lo = (int)my_c;
                my_hi = (int)my_c + 1;
            } else {
                const int2 cr = node_range[my_c - ntot];
                my_lo = cr.x;
                my_hi = cr.y;
            }
        }
        const bool my_big = lane < nch && my_hi - my_lo > G;
        u64 cbmin[3] = {0, 0, 0}, cbmax[3] = {0, 0, 0};  // large child's cell (lane q)
        if (my_big) {  // a large child is a node
            const double hs = 0.5 * size[my_c];
            for (int k = 0; k < 3; k++) {
                cbmin[k] = order_key(cell[3 * (my_c - ntot) + k] - hs);
                cbmax[k] = order_key(cell[3 * (my_c - ntot) + k] + hs);
            }
        }
        const unsigned bigmask = __ballot_sync(FULL, my_big);
        // this lane's particle of every small child (a large or missing child repeats a valid load)
        double v[8][3];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int lo = __shfl_sync(FULL, my_lo, q), hi = __shfl_sync(FULL, my_hi, q);
            const int64_t p = (int64_t)lo + lane;
            const int64_t src = (q < nch && hi - lo <= G && p < hi) ? p : (q < nch ? (int64_t)lo : 0);
#pragma unroll
            for (int k = 0; k < 3; k++) v[q][k] = coord[3 * src + k];
        }
        u64 pbmin[3] = {0, 0, 0}, pbmax[3] = {0, 0, 0};  // small child's particle box (lane q)
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if (q >= nch) break;
            if ((bigmask >> q) & 1u) continue;  // warp-uniform
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const u64 key = order_key(v[q][k]);
                const u64 mn = warp_min_key(key), mx = warp_max_key(key);
                if (lane == q) {
                    pbmin[k] = mn;
                    pbmax[k] = mx;
                }
            }
        }
        // greedy runs in chain order
        int run_lo = -1, run_cnt = 0;
        u64 rlo[3] = {0, 0, 0}, rhi[3] = {0, 0, 0};
        for (int q = 0; q < nch; q++) {
            const int lo = __shfl_sync(FULL, my_lo, q), hi = __shfl_sync(FULL, my_hi, q);
            const int sz = hi - lo;
            if (sz > G) {
                if (run_cnt) emit(run_lo, run_cnt);
                run_cnt = 0;
                continue;
            }
            u64 lo3[3], hi3[3];
            for (int k = 0; k < 3; k++) {
                lo3[k] = __shfl_sync(FULL, pbmin[k], q);
                hi3[k] = __shfl_sync(FULL, pbmax[k], q);
            }
            if (run_cnt) {
                u64 nlo[3], nhi[3];
                for (int k = 0; k < 3; k++) {
                    nlo[k] = rlo[k] < lo3[k] ? rlo[k] : lo3[k];
                    nhi[k] = rhi[k] > hi3[k] ? rhi[k] : hi3[k];
                }
                // does the grown box reach into a large sibling's cell? (lane b tests sibling b)
                bool overlap = my_big;
                for (int k = 0; k < 3; k++) overlap = overlap && nlo[k] <= cbmax[k] && nhi[k] >= cbmin[k];
                const bool hits = __any_sync(FULL, overlap);
                if (run_cnt + sz <= G && !hits) {
                    run_cnt += sz;
                    for (int k = 0; k < 3; k++) {
                        rlo[k] = nlo[k];
                        rhi[k] = nhi[k];
                    }
                    continue;
                }
                emit(run_lo, run_cnt);
            }
            run_lo = lo;
            run_cnt = sz;
            for (int k = 0; k < 3; k++) {
                rlo[k] = lo3[k];
                rhi[k] = hi3[k];
            }
        }
        if (run_cnt) emit(run_lo, run_cnt);
        if (nemit > 0) {  // at most one group per child, so nemit <= 8 lanes hold them
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(count, (unsigned long long)nemit);
            base = __shfl_sync(FULL, base, 0);
            if (lane < nemit) {
                groups[base + lane] = make_int2(my_glo, my_gcnt);
                group_root[base + lane] = root;
                group_node[base + lane] = (int)j;
            }
        }
    }
}

// Queue key for reference grouping: the group's bounding-box diagonal, largest first (as float
// bits, which order like the floats for non-negative values), so the few groups that straddle a
// Morton-curve jump -- and open most of the tree -- start first instead of forming the tail.
__global__ void k_group_cost_keys(const double *tpos, const int2 *groups, int64_t ngroups, uint64_t *keys,
                                  uint32_t *vals) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    int2 gr = groups[g];
    double lo[3], hi[3];
    for (int k = 0; k < 3; k++) lo[k] = hi[k] = tpos[3 * (int64_t)gr.x + k];
    for (int t = 1; t < gr.y; t++)
        for (int k = 0; k < 3; k++) {
            double v = tpos[3 * ((int64_t)gr.x + t) + k];
            lo[k] = fmin(lo[k], v);
            hi[k] = fmax(hi[k], v);
        }
    float d = (float)sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                          (hi[2] - lo[2]) * (hi[2] - lo[2]));
    keys[g] = (uint64_t)(0xffffffffu - __float_as_uint(d));
    vals[g] = (uint32_t)g;
}
__global__ void k_group_start_keys(const int2 *groups, int64_t ngroups, uint64_t *keys, uint32_t *vals) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    keys[g] = (uint32_t)groups[g].x;
    vals[g] = (uint32_t)g;
}
__global__ void k_permute_groups(const uint32_t *perm, int64_t ngroups, const int2 *gin, const int *rin, const int *nin,
                                 int2 *gout, int *rout, int *nout) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    gout[g] = gin[perm[g]];
    rout[g] = rin[perm[g]];
    if (nin) nout[g] = nin[perm[g]];
}

// Targets in walk order split once per walk into hi/lo parts in the walk precision.
template <typename T>
__global__ void k_prep_targets(const double *tpos, const double *th, int64_t n, vec4<T> *thi, vec4<T> *tlo) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T hx, hy, hz, lx, ly, lz;
    split_hi_lo(tpos[3 * i], hx, lx);
    split_hi_lo(tpos[3 * i + 1], hy, ly);
    split_hi_lo(tpos[3 * i + 2], hz, lz);
    thi[i] = vec4<T>{hx, hy, hz, narrow(th[i], T(0))};
    tlo[i] = vec4<T>{lx, ly, lz, T(0)};
}

// Persistent grid: as many blocks of `warps` warps as fit on the GPU (fewer when every group has a
// warp anyway; all of them for the retry pass, whose group count is known only on the device).
// ---------------------------------------------------------------------------------------------
// Split walk of heavy groups. A group of consecutive Morton targets that straddles a jump of the
// Morton curve gets a bounding box spanning both sides and can open most of the tree: at 1e6
// Plummer particles and pytreegrav's groups of 8, one group evaluates ~9e5 list entries, ~450x the
// median, and one warp would work through it alone. Such a group stops once it passes an entry
// budget; k_walk_top then walks it down to subtrees of at most split_npart particles without
// evaluating anything and lists the pieces -- every node it accepts, every particle of a node it
// opens, and every node child small enough -- as items; all warps walk the items (k_walk in item
// mode) and k_reduce_items adds each group's item sums in item order. The items together cover the
// group's accepted set exactly: each decision here is the exact FP64 criterion, which the walk's
// own test reproduces, and an item node is tested again when its walk starts. Only the summation
// order differs from an unsplit walk, and it is fixed, so results do not vary between runs.
constexpr int TOP_WARPS = 4;
constexpr int TOP_STACK = 2048;

template <typename T>
struct TopArgs {
    Arena<T> ar;
    int64_t ntot;
    const double *tc, *ts, *tsize, *tdelta;
    const double *tpos, *th;
    const int2 *groups;
    const int *group_root;
    const int *heavy;  // unit -> group
    int nheavy;
    double theta;
    const float *theta_group;
    const int2 *node_range;
    int split_npart;
    int *items;       // item_cap per unit
    int *item_count;  // per unit
    int item_cap;
    int *status;
};

template <typename T>
__global__ void __launch_bounds__(TOP_WARPS * 32) k_walk_top(TopArgs<T> a) {
    __shared__ int stack_all[TOP_WARPS][TOP_STACK];
    int *stack = stack_all[threadIdx.x >> 5];
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    const int u = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (u >= a.nheavy) return;
    if (a.ar.bad && *a.ar.bad) {
        if (lane == 0) atomicOr(a.status, 1 << TG_ERR_CUDA);
        return;
    }
    const int g = a.heavy[u];
    const int2 gr = a.groups[g];
    const int64_t t = gr.x + (lane < gr.y ? lane : 0);
    double bmin[3], bmax[3], hmax = a.th[t];
    for (int k = 0; k < 3; k++) bmin[k] = bmax[k] = a.tpos[3 * t + k];
#pragma unroll
    for (int o = 16; o; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            bmin[k] = fmin(bmin[k], __shfl_xor_sync(FULL, bmin[k], o));
            bmax[k] = fmax(bmax[k], __shfl_xor_sync(FULL, bmax[k], o));
        }
        hmax = fmax(hmax, __shfl_xor_sync(FULL, hmax, o));
    }
    const double theta = a.theta_group ? (double)a.theta_group[g] : a.theta;
    int *items = a.items + (int64_t)u * a.item_cap;
    int nitems = 0, sp = 1;
    if (lane == 0) stack[0] = a.group_root[g];
    __syncwarp();
    bool failed = false;
    for (int64_t steps_left = a.ar.n_nodes + 2; sp > 0; ) {
        if (--steps_left < 0) {
            if (lane == 0) atomicOr(a.status, 1 << TG_ERR_ITER_LIMIT);
            failed = true;
            break;
        }
        const int cnt = min(sp, 32);
        const int node = lane < cnt ? stack[sp - 1 - lane] : -1;
        sp -= cnt;
        __syncwarp();
        bool acc = false;
        int fc = 0, nc = 0, ls = 0, nl = 0;
        if (node >= 0) {
            acc = accept_exact(a.ntot + node, a.tc, a.ts, a.tsize, a.tdelta, bmin, bmax, hmax, theta);
            if (!acc) {
                const int cb = bits_int(a.ar.n_trav[2 * node + 1].z), lb = bits_int(a.ar.n_trav[2 * node + 1].w);
                fc = cb >> 4;
                nc = cb & 15;
                ls = lb >> 4;
                nl = lb & 15;
            }
        }
        // this lane's items (the node itself, or its particles and small node children) and pushes
        int nit = 0, npush = 0;
        unsigned small = 0;
        if (node >= 0) {
            if (acc) {
                nit = 1;
            } else {
                for (int j = 0; j < nc; j++) {
                    const int2 r = a.node_range[fc + j];
                    if (r.y - r.x <= a.split_npart) small |= 1u << j;
                }
                nit = nl + __popc(small);
                npush = nc - __popc(small);
            }
        }
        const int both = warp_inclusive_scan(nit | (npush << 16));
        const int tot = __shfl_sync(FULL, both, 31);
        const int toti = tot & 0xffff, totp = tot >> 16;
        if (nitems + toti > a.item_cap || sp + totp > TOP_STACK) {  // this group is walked whole instead
            nitems = -1;
            break;
        }
        int oi = nitems + (both & 0xffff) - nit, op = sp + (both >> 16) - npush;
        if (node >= 0) {
            if (acc) {
                items[oi] = node;
            } else {
                for (int j = 0; j < nl; j++) items[oi++] = ~(ls + j);
                for (int j = 0; j < nc; j++) {
                    if ((small >> j) & 1u) items[oi++] = fc + j;
                    else stack[op++] = fc + j;
                }
            }
        }
        nitems += toti;
        sp += totp;
        __syncwarp();
        (void)lt;
    }
    if (lane == 0) a.item_count[u] = failed ? 0 : nitems;  // -1: too many items, walk the group whole
}

// Items of every unit, flattened in unit order: item k -> (group, start node).
__global__ void k_flatten_items(const int *heavy, int nheavy, const int *items, int item_cap, const int64_t *off,
                                int *item_group, int *item_node) {
    const int u = blockIdx.x;
    if (u >= nheavy) return;
    const int64_t o = off[u], n = off[u + 1] - off[u];
    const int g = heavy[u];
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
        item_group[o + k] = g;
        item_node[o + k] = items[(int64_t)u * item_cap + k];
    }
}

// One block per (unit, target slot): thread t sums the unit's items t, t + RED_THREADS, ... in order,
// then a fixed-shape tree in shared memory adds the threads' sums (the same order on every run); G
// times the total is written to the target's row.
constexpr int RED_THREADS = 256;
__global__ void __launch_bounds__(RED_THREADS) k_reduce_items(const int *heavy, int nheavy, const int64_t *off,
                                                              const int *count, const int2 *groups, int gs,
                                                              const double *partial, const int64_t *scatter,
                                                              int out_fields, int out_w, double G, double *out) {
    __shared__ double sh[10][RED_THREADS];
    const int u = blockIdx.x / gs, slot = blockIdx.x % gs;
    if (u >= nheavy || count[u] < 0) return;  // block-uniform: walked whole
    const int2 gr = groups[heavy[u]];
    if (slot >= gr.y) return;  // block-uniform
    const int t = threadIdx.x;
    double v[10];
#pragma unroll
    for (int c = 0; c < 10; c++) v[c] = 0.0;
    for (int64_t k = off[u] + t; k < off[u + 1]; k += RED_THREADS) {
        const double *p = partial + (k * gs + slot) * 10;
#pragma unroll
        for (int c = 0; c < 10; c++) v[c] += p[c];
    }
#pragma unroll
    for (int c = 0; c < 10; c++) sh[c][t] = v[c];
    __syncthreads();
    for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
        if (t < w) {
#pragma unroll
            for (int c = 0; c < 10; c++) sh[c][t] += sh[c][t + w];
        }
        __syncthreads();
    }
    if (t == 0) {
        double tot[10];
#pragma unroll
        for (int c = 0; c < 10; c++) tot[c] = sh[c][0];
        const int64_t tg_ = gr.x + slot;
        const int64_t row = scatter ? scatter[tg_] : tg_;
        write_fields(out + row * out_w, out_fields, tot, G);
    }
}

template <typename T, int FIELDS, bool QUAD, int STACK>
static tg_status launch_walk(WalkArgs<T> &a, int warps, cudaStream_t st) {
    size_t smem = sizeof(WarpSmem<T, QUAD, STACK>) * warps;
    auto kern = k_walk<T, FIELDS, QUAD, STACK>;
    TG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the 72-register walk reaches 7 blocks per SM only with the largest shared-memory carveout; the
    // others keep the driver's choice, which leaves them more L1
    if (sizeof(T) == 4 && FIELDS == F_ACC && QUAD && STACK == STACK_SMALL)
        TG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared));
    int per_sm = 0;
    TG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = (int64_t)per_sm * num_sms();
    if (!a.ngroups_dev) {
        int64_t need = (a.ngroups + warps - 1) / warps;
        if (blocks > need) blocks = need;
    } else {  // a pass over a list counted on the device (groups that overflowed the small stack or
              // went over their error budget): usually empty or short, one block per SM
        blocks = num_sms();
    }
    if (blocks < 1) blocks = 1;
    { kern<<<(unsigned)blocks, warps * 32, smem, st>>>(a); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

template <typename T, int STACK>
static tg_status dispatch_walk(WalkArgs<T> &a, int fields, bool quad, int warps, cudaStream_t st) {
    // Fields computed: potential and/or acceleration alone; the tidal tensor alone in FP32 (its own
    // paired sweeps); else everything when the tidal tensor is wanted (its setup already contains
    // the other two).
    int fc = (fields & F_TID) ? (F_POT | F_ACC | F_TID) : fields;
    if constexpr (sizeof(T) == 4) {
        if (fields == F_TID) {
            if (quad) return launch_walk<T, F_TID, true, STACK>(a, warps, st);
            return launch_walk<T, F_TID, false, STACK>(a, warps, st);
        }
    }
    if (quad) {
        switch (fc) {
            case F_POT: return launch_walk<T, F_POT, true, STACK>(a, warps, st);
            case F_ACC: return launch_walk<T, F_ACC, true, STACK>(a, warps, st);
            case F_POT | F_ACC: return launch_walk<T, F_POT | F_ACC, true, STACK>(a, warps, st);
            default: return launch_walk<T, F_POT | F_ACC | F_TID, true, STACK>(a, warps, st);
        }
    }
    switch (fc) {
        case F_POT: return launch_walk<T, F_POT, false, STACK>(a, warps, st);
        case F_ACC: return launch_walk<T, F_ACC, false, STACK>(a, warps, st);
        case F_POT | F_ACC: return launch_walk<T, F_POT | F_ACC, false, STACK>(a, warps, st);
        default: return launch_walk<T, F_POT | F_ACC | F_TID, false, STACK>(a, warps, st);
    }
}

// Scratch of one walk, in ints: queue, status, retry count, retry queue, then the retry list.
constexpr int WS_QUEUE = 0, WS_STATUS = 1, WS_RETRY_COUNT = 2, WS_RETRY_QUEUE = 3, WS_REWALK_COUNT = 4,
              WS_REWALK_QUEUE = 5, WS_HEAVY_COUNT = 6, WS_HEAVY_QUEUE = 7,
              WS_RETRY_LIST = 8;  // then the retry list, the rewalk list and the heavy list
inline int64_t walk_scratch_ints(int64_t ngroups) { return WS_RETRY_LIST + 3 * std::max<int64_t>(ngroups, 1); }
// List entries after which a group counts as heavy (split_heavy walks): the median group of 8 at 1e6
// Plummer particles evaluates ~1.9e3, the 99.9th percentile ~7e3.
constexpr unsigned HEAVY_ENTRIES = 1u << 15;
constexpr int ITEM_CAP = 1 << 16;  // items per heavy group

// Enqueue a whole walk on st (no host synchronisation, so it can be captured): with the small
// first stack, the small-stack pass, then a large-stack pass over the groups that overflowed it
// (an empty pass when none did); with the large first stack, one large-stack pass. scratch:
// walk_scratch_ints(a.ngroups) ints, zeroed here.
template <typename T>
static tg_status enqueue_walk(WalkArgs<T> a, int fields, bool quad, int warps, int first_stack, int *scratch,
                              cudaStream_t st, bool split_heavy = false) {
    TG_CUDA(cudaMemsetAsync(scratch, 0, sizeof(int) * WS_RETRY_LIST, st));
    const int64_t ng1 = std::max<int64_t>(a.ngroups, 1);
    a.queue = scratch + WS_QUEUE;
    a.status = scratch + WS_STATUS;
    a.ngroups_dev = nullptr;
    // heavy groups stop and are listed for walk_heavy (which needs host synchronisation)
    a.heavy = split_heavy ? scratch + WS_RETRY_LIST + 2 * ng1 : nullptr;
    a.heavy_count = split_heavy ? scratch + WS_HEAVY_COUNT : nullptr;
    a.heavy_budget = loop_limits().heavy_entries > 0 ? (unsigned)std::min<long long>(loop_limits().heavy_entries, 1ll << 30)
                                                     : HEAVY_ENTRIES;
    a.step_limit = loop_limits().walk_steps;
    const bool budget = a.tol_group && a.err_budget > 0.f;
    a.rewalk = budget ? scratch + WS_RETRY_LIST + ng1 : nullptr;
    a.rewalk_count = budget ? scratch + WS_REWALK_COUNT : nullptr;
    if (first_stack == STACK_LARGE) {
        a.retry = a.retry_count = nullptr;
        TG_TRY((dispatch_walk<T, STACK_LARGE>(a, fields, quad, warps, st)));
    } else {
        a.retry = scratch + WS_RETRY_LIST;
        a.retry_count = scratch + WS_RETRY_COUNT;
        TG_TRY((dispatch_walk<T, STACK_SMALL>(a, fields, quad, warps, st)));
        WalkArgs<T> b = a;
        b.queue = scratch + WS_RETRY_QUEUE;
        b.group_order = scratch + WS_RETRY_LIST;  // retry list entries are group indices
        b.ngroups_dev = scratch + WS_RETRY_COUNT;
        b.retry = b.retry_count = nullptr;
        TG_TRY((dispatch_walk<T, STACK_LARGE>(b, fields, quad, warps, st)));
    }
    if (!budget) return TG_OK;
    // groups over their error budget, walked again with the global theta (their rows rewritten)
    WalkArgs<T> r = a;
    r.queue = scratch + WS_REWALK_QUEUE;
    r.group_order = scratch + WS_RETRY_LIST + ng1;
    r.ngroups_dev = scratch + WS_REWALK_COUNT;
    r.retry = r.retry_count = nullptr;
    r.rewalk = r.rewalk_count = nullptr;
    r.heavy = r.heavy_count = nullptr;
    r.tol_group = nullptr;
    r.theta_group = nullptr;
    r.gerr = nullptr;
    r.theta = a.rewalk_theta > 0.0 ? a.rewalk_theta : a.theta;
    return dispatch_walk<T, STACK_LARGE>(r, fields, quad, warps, st);
}

// The heavy groups listed by a walk (see k_walk_top): split into items, the items walked by all warps,
// each group's item sums reduced in item order into its rows. nheavy groups are listed at the heavy
// list of scratch. Synchronises st twice (item counts, then the flattened list's size).
template <typename T>
static tg_status walk_heavy(tg_tree_s *t, const WalkArgs<T> &a, Arena<T> &ar, int fields, bool quad, int warps,
                            int *scratch, int nheavy, cudaStream_t st) {
    const int64_t ng1 = std::max<int64_t>(a.ngroups, 1);
    const int *heavy = scratch + WS_RETRY_LIST + 2 * ng1;
    WalkArgs<T> b = a;
    b.retry = b.retry_count = nullptr;
    b.heavy = b.heavy_count = nullptr;
    b.rewalk = b.rewalk_count = nullptr;
    b.ngroups_dev = nullptr;
    b.queue = scratch + WS_HEAVY_QUEUE;
    // subtrees of at most split_npart particles become items; a top walk opens only larger nodes, of
    // which a tree holds about 2 N / split_npart, each giving at most 16 items (8 particles, 8 nodes)
    const int split_npart = (int)std::max<int64_t>(1024, t->ntot / 2048);
    const int cap = (int)std::min<int64_t>(1 << 16, std::max<int64_t>(1024, 16 * (2 * t->ntot / split_npart + 8)));
    if ((int64_t)nheavy * cap > ((int64_t)1 << 28)) {  // too many to list: walk them whole
        TG_CUDA(cudaMemsetAsync(b.queue, 0, sizeof(int), st));
        b.group_order = heavy;
        b.ngroups = nheavy;
        return dispatch_walk<T, STACK_LARGE>(b, fields, quad, warps, st);
    }
    DevArray<int> items(st), counts(st);
    TG_CUDA(items.alloc((int64_t)nheavy * cap));
    TG_CUDA(counts.alloc(nheavy));
    TopArgs<T> ta;
    ta.ar = ar;
    ta.ntot = a.ntot;
    ta.tc = a.tc; ta.ts = a.ts; ta.tsize = a.tsize; ta.tdelta = a.tdelta;
    ta.tpos = a.tpos; ta.th = a.th;
    ta.groups = a.groups;
    ta.group_root = a.group_root;
    ta.heavy = heavy;
    ta.nheavy = nheavy;
    ta.theta = a.theta;
    ta.theta_group = a.theta_group;
    ta.node_range = t->node_range;
    ta.split_npart = split_npart;
    ta.items = items.p;
    ta.item_count = counts.p;
    ta.item_cap = cap;
    ta.status = a.status;
    { k_walk_top<T><<<div_up(nheavy, TOP_WARPS), TOP_WARPS * 32, 0, st>>>(ta); note_launch(); }
    TG_CUDA(cudaGetLastError());
    std::vector<int> hc(nheavy), hg(nheavy);
    TG_CUDA(cudaMemcpyAsync(hc.data(), counts.p, sizeof(int) * nheavy, cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaMemcpyAsync(hg.data(), heavy, sizeof(int) * nheavy, cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    std::vector<int64_t> off(nheavy + 1, 0);
    std::vector<int> whole;  // groups with more items than the list holds
    for (int u = 0; u < nheavy; u++) {
        off[u + 1] = off[u] + std::max(hc[u], 0);
        if (hc[u] < 0) whole.push_back(hg[u]);
    }
    std::sort(whole.begin(), whole.end());
    const int64_t total = off[nheavy];
    DevArray<int> item_group(st), item_node(st), dwhole(st);
    DevArray<int64_t> doff(st);
    DevArray<double> partial(st);
    if (!whole.empty()) {
        TG_CUDA(dwhole.alloc((int64_t)whole.size()));
        TG_CUDA(cudaMemcpyAsync(dwhole.p, whole.data(), sizeof(int) * whole.size(), cudaMemcpyHostToDevice, st));
        TG_CUDA(cudaMemsetAsync(b.queue, 0, sizeof(int), st));
        WalkArgs<T> w = b;
        w.group_order = dwhole.p;
        w.ngroups = (int64_t)whole.size();
        TG_TRY((dispatch_walk<T, STACK_LARGE>(w, fields, quad, warps, st)));
    }
    if (total > 0) {
        TG_CUDA(item_group.alloc(total));
        TG_CUDA(item_node.alloc(total));
        TG_CUDA(doff.alloc(nheavy + 1));
        TG_CUDA(partial.alloc(10 * (int64_t)a.gs * total));
        TG_CUDA(cudaMemcpyAsync(doff.p, off.data(), sizeof(int64_t) * (nheavy + 1), cudaMemcpyHostToDevice, st));
        { k_flatten_items<<<nheavy, 256, 0, st>>>(heavy, nheavy, items.p, cap, doff.p, item_group.p, item_node.p); note_launch(); }
        TG_CUDA(cudaMemsetAsync(b.queue, 0, sizeof(int), st));
        b.group_order = nullptr;
        b.item_group = item_group.p;
        b.item_node = item_node.p;
        b.partial = partial.p;
        b.ngroups = total;
        TG_TRY((dispatch_walk<T, STACK_LARGE>(b, fields, quad, warps, st)));
        { k_reduce_items<<<(unsigned)((int64_t)nheavy * a.gs), RED_THREADS, 0, st>>>(heavy, nheavy, doff.p, counts.p,
                                                                                     a.groups, a.gs, partial.p, a.scatter,
                                                                                     a.out_fields, a.out_w, a.G, a.out); note_launch(); }
        TG_CUDA(cudaGetLastError());
    }
    // the host vectors above must outlive their copies
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

// Run a walk and time it on the stream; *status_out receives the device status word. With
// split_heavy, groups past the entry budget are walked by walk_heavy.
template <typename T>
static tg_status walk_with_fallback(tg_tree_s *t, WalkArgs<T> &a, Arena<T> &ar, int fields, bool quad, int warps,
                                    int first_stack, int *scratch, bool split_heavy, cudaStream_t st, int *status_out,
                                    float *kernel_ms) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    struct Events {  // back to the pool on every exit
        cudaEvent_t *a, *b;
        ~Events() {
            release_event(*a, true);
            release_event(*b, true);
        }
    } evs{&e0, &e1};
    TG_CUDA(pool_event(&e0, true));
    TG_CUDA(pool_event(&e1, true));
    TG_CUDA(cudaEventRecord(e0, st));
    tg_status rc = enqueue_walk<T>(a, fields, quad, warps, first_stack, scratch, st, split_heavy);
    int hdr[WS_RETRY_LIST] = {0};
    if (rc == TG_OK && split_heavy) {
        TG_CUDA(cudaMemcpyAsync(hdr, scratch, sizeof(hdr), cudaMemcpyDeviceToHost, st));
        TG_CUDA(cudaStreamSynchronize(st));
        if (hdr[WS_HEAVY_COUNT] > 0)
            rc = walk_heavy<T>(t, a, ar, fields, quad, warps, scratch, hdr[WS_HEAVY_COUNT], st);
    }
    TG_CUDA(cudaEventRecord(e1, st));
    int status = 0;
    TG_CUDA(cudaMemcpyAsync(&status, scratch + WS_STATUS, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    TG_CUDA(cudaEventElapsedTime(kernel_ms, e0, e1));
    *status_out = status;
    return rc;
}

// Whether a walk arena is larger than the GPU's L2 (the walk then prefetches the records it queues).
template <typename T>
static int arena_exceeds_l2(const Arena<T> &ar) {
    static int l2 = -1;
    if (l2 < 0) {
        int dev = 0;
        l2 = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
        if (l2 <= 0) l2 = 128 << 20;
    }
    const int64_t bytes = ar.n_nodes * (int64_t)sizeof(vec4<T>) * (ar.n_quad ? 6 : 4) +
                          ar.n_leaves * (int64_t)sizeof(vec4<T>) * 2 + (ar.n_tol ? ar.n_nodes * 8 : 0);
    return bytes > (int64_t)l2;
}

// Walk targets already in walk order (tpos/th on the device). groups/group_root describe the
// grouping; scatter maps walk order to output rows.
tg_status run_walk(tg_tree_s *t, const double *tpos, const double *th, int64_t ntargets, const int2 *groups,
                   const int *group_root, const int *group_order, int64_t ngroups, const int64_t *scatter, int fields,
                   int quadrupole, double theta, double G, int group_size, int precision, const float *theta_group,
                   const float *tol_group, double *out, cudaStream_t st) {
    int w = ((fields & F_POT) ? 1 : 0) + ((fields & F_ACC) ? 3 : 0) + ((fields & F_TID) ? 9 : 0);
    if (!t->stats_dev) TG_CUDA(tg::dev_malloc((void **)&t->stats_dev, sizeof(unsigned long long) * 8, st));
    int *scratch = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&scratch, sizeof(int) * walk_scratch_ints(ngroups), st));
    TG_CUDA(cudaMemsetAsync(t->stats_dev, 0, sizeof(unsigned long long) * 8, st));
    tg_status rc = TG_OK;
    int status = 0;
    float kms = 0.f;
    unsigned *gstats = nullptr;
    if (t->record_group_stats) {
        if (t->gstats_n < ngroups) {
            if (t->gstats) cudaFreeAsync(t->gstats, st);
            t->gstats = nullptr;
            t->gstats_n = 0;
            TG_CUDA(tg::dev_malloc((void **)&t->gstats, sizeof(unsigned) * 3 * std::max<int64_t>(ngroups, 1), st));
            t->gstats_n = ngroups;
        }
        TG_CUDA(cudaMemsetAsync(t->gstats, 0, sizeof(unsigned) * 3 * std::max<int64_t>(ngroups, 1), st));
        gstats = t->gstats;
    }
    // plain walks split their heavy groups (walks with per-group counters or tolerances keep every
    // group whole: their per-group results are read back)
    const bool split_heavy = !t->record_group_stats && !tol_group;
    float *gerr = nullptr;
    if (t->record_group_stats && tol_group) {
        if (t->gerr) cudaFreeAsync(t->gerr, st);
        t->gerr = nullptr;
        TG_CUDA(tg::dev_malloc((void **)&t->gerr, sizeof(float) * std::max<int64_t>(ngroups, 1), st));
        TG_CUDA(cudaMemsetAsync(t->gerr, 0, sizeof(float) * std::max<int64_t>(ngroups, 1), st));
        gerr = t->gerr;
    }
    if (precision == TG_FP64) {
        TG_TRY(build_arena(t, t->arena64, st));
        WalkArgs<double> a;
        a.ar = t->arena64;
        a.ntot = t->ntot;
        a.tc = t->coord; a.ts = t->soft; a.tsize = t->size; a.tdelta = t->delta;
        a.tpos = tpos; a.th = th; a.scatter = scatter; a.groups = groups; a.group_root = group_root;
        a.group_order = group_order;
        a.ngroups = ngroups; a.theta = theta; a.theta_group = theta_group; a.tol_group = tol_group; a.G = G;
        a.err_budget = tol_group ? t->err_budget : 0.f;
        a.gerr = gerr;
        a.rewalk_theta = t->rewalk_theta;
        a.out_fields = fields; a.out_w = w; a.out = out; a.gs = group_size;
        a.stats = (unsigned long long *)t->stats_dev;
        a.gstats = gstats;
        a.prefetch = arena_exceeds_l2(t->arena64);
        vec4<double> *thi = nullptr, *tlo = nullptr;
        TG_CUDA(tg::dev_malloc((void **)&thi, sizeof(vec4<double>) * std::max<int64_t>(ntargets, 1), st));
        TG_CUDA(tg::dev_malloc((void **)&tlo, sizeof(vec4<double>) * std::max<int64_t>(ntargets, 1), st));
        { k_prep_targets<double><<<div_up(ntargets, 256), 256, 0, st>>>(tpos, th, ntargets, thi, tlo); tg::note_launch(); }
        a.thi = thi;
        a.tlo = tlo;
        rc = walk_with_fallback<double>(t, a, t->arena64, fields, quadrupole != 0, t->walk_warps, t->walk_stack,
                                        scratch, split_heavy, st, &status,
                                        &kms);
        cudaFreeAsync(thi, st);
        cudaFreeAsync(tlo, st);
    } else {
        TG_TRY(build_arena(t, t->arena32, st));
        WalkArgs<float> a;
        a.ar = t->arena32;
        a.ntot = t->ntot;
        a.tc = t->coord; a.ts = t->soft; a.tsize = t->size; a.tdelta = t->delta;
        a.tpos = tpos; a.th = th; a.scatter = scatter; a.groups = groups; a.group_root = group_root;
        a.group_order = group_order;
        a.ngroups = ngroups; a.theta = theta; a.theta_group = theta_group; a.tol_group = tol_group; a.G = G;
        a.err_budget = tol_group ? t->err_budget : 0.f;
        a.gerr = gerr;
        a.rewalk_theta = t->rewalk_theta;
        a.out_fields = fields; a.out_w = w; a.out = out; a.gs = group_size;
        a.stats = (unsigned long long *)t->stats_dev;
        a.gstats = gstats;
        a.prefetch = arena_exceeds_l2(t->arena32);
        vec4<float> *thi = nullptr, *tlo = nullptr;
        const bool own = t->own32 && tpos == t->coord && th == t->soft && ntargets == t->ntot;
        if (own) {  // the tree's own particles, prepared beside the first grouping
            a.thi = t->own32;
            a.tlo = t->own32 + t->ntot;
        } else {
            TG_CUDA(tg::dev_malloc((void **)&thi, sizeof(vec4<float>) * std::max<int64_t>(ntargets, 1), st));
            TG_CUDA(tg::dev_malloc((void **)&tlo, sizeof(vec4<float>) * std::max<int64_t>(ntargets, 1), st));
            { k_prep_targets<float><<<div_up(ntargets, 256), 256, 0, st>>>(tpos, th, ntargets, thi, tlo); tg::note_launch(); }
            a.thi = thi;
            a.tlo = tlo;
        }
        rc = walk_with_fallback<float>(t, a, t->arena32, fields, quadrupole != 0, t->walk_warps, t->walk_stack,
                                       scratch, split_heavy, st, &status,
                                       &kms);
        if (thi) cudaFreeAsync(thi, st);
        if (tlo) cudaFreeAsync(tlo, st);
    }
    if (rc != TG_OK) return rc;
    unsigned long long stats[8];
    int sort_bad = 0;
    TG_CUDA(cudaMemcpyAsync(stats, t->stats_dev, sizeof(stats), cudaMemcpyDeviceToHost, st));
    if (t->sort_err) TG_CUDA(cudaMemcpyAsync(&sort_bad, t->sort_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaFreeAsync(scratch, st));
    TG_CUDA(cudaStreamSynchronize(st));
    t->last_stats.interactions = (int64_t)stats[0];
    t->last_stats.node_tests = (int64_t)stats[1];
    t->last_stats.max_stack = (int64_t)stats[2];
    t->last_stats.groups = ngroups;
    t->last_stats.steps = (int64_t)stats[3];
    t->last_stats.quad_interactions = (int64_t)stats[4];
    t->last_stats.kernel_ms = kms;
    if (sort_bad) {  // the grouping's or the queue order's sort (reported once; the groups are valid)
        cudaMemsetAsync(t->sort_err, 0, sizeof(int), st);
        set_last_error_msg("radix sort: a tile's look-back did not complete within its bound");
        return TG_ERR_QUEUE_TIMEOUT;
    }
    if (status & (1 << TG_ERR_CUDA)) {
        set_last_error_msg("internal error: tree links do not form a valid octree for the walk arena");
        return TG_ERR_CUDA;
    }
    if (status & (1 << TG_ERR_STACK_OVERFLOW)) return TG_ERR_STACK_OVERFLOW;
    if (status & (1 << TG_ERR_ITER_LIMIT)) return TG_ERR_ITER_LIMIT;
    return TG_OK;
}

// The tree grouping at group size G, made once per tree and size and kept on the tree.
tg_status tree_groups(tg_tree_s *t, int G, cudaStream_t st) {
    if (t->groups && t->groups_G == G) return TG_OK;
    if (t->groups) cudaFreeAsync(t->groups, st);
    if (t->group_root) cudaFreeAsync(t->group_root, st);
    if (t->group_node) cudaFreeAsync(t->group_node, st);
    t->groups = nullptr; t->group_root = nullptr; t->group_node = nullptr; t->ngroups = 0; t->groups_G = 0;
    const int64_t N = t->ntot, M = t->mtot;
    int64_t *d_sys = nullptr, *d_node = nullptr;
    unsigned long long *cnt = nullptr;
    int2 *g0 = nullptr;
    int *r0 = nullptr, *n0 = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&g0, sizeof(int2) * N, st));
    TG_CUDA(tg::dev_malloc((void **)&r0, sizeof(int) * N, st));
    TG_CUDA(tg::dev_malloc((void **)&n0, sizeof(int) * N, st));
    TG_CUDA(tg::dev_malloc((void **)&cnt, sizeof(unsigned long long), st));
    TG_CUDA(tg::dev_malloc((void **)&d_sys, sizeof(int64_t) * (t->nsys + 1), st));
    TG_CUDA(tg::dev_malloc((void **)&d_node, sizeof(int64_t) * (t->nsys + 1), st));
    TG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), st));
    TG_CUDA(cudaMemcpyAsync(d_sys, t->sys_off.data(), sizeof(int64_t) * (t->nsys + 1), cudaMemcpyHostToDevice, st));
    TG_CUDA(cudaMemcpyAsync(d_node, t->sys_node_off.data(), sizeof(int64_t) * (t->nsys + 1), cudaMemcpyHostToDevice,
                            st));
    LargeNode *large = nullptr;
    int *nlarge = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&large, sizeof(LargeNode) * std::max<int64_t>(M, 1), st));
    TG_CUDA(tg::dev_malloc((void **)&nlarge, sizeof(int), st));
    TG_CUDA(cudaMemsetAsync(nlarge, 0, sizeof(int), st));
    { k_tree_groups_mark<<<div_up(M, 256), 256, 0, st>>>(N, M, t->node_range, t->first, t->next, t->parent, G, d_sys,
                                                       d_node, t->nsys, g0, r0, n0, cnt, large, nlarge); tg::note_launch(); }
    { k_tree_groups_large<<<num_sms() * 8, 256, 0, st>>>(N, t->node_range, t->cell_center, t->size, t->coord, G, large,
                                                       nlarge, g0, r0, n0, cnt); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    unsigned long long ng = 0;
    TG_CUDA(cudaMemcpyAsync(&ng, cnt, sizeof(ng), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    // deterministic Morton order of the groups (their emission order depends on thread timing)
    uint64_t *keys = nullptr;
    uint32_t *vals = nullptr;
    const unsigned long long ng1 = std::max<unsigned long long>(ng, 1);
    TG_CUDA(tg::dev_malloc((void **)&keys, sizeof(uint64_t) * ng1, st));
    TG_CUDA(tg::dev_malloc((void **)&vals, sizeof(uint32_t) * ng1, st));
    TG_CUDA(tg::dev_malloc((void **)&t->groups, sizeof(int2) * ng1, st));
    TG_CUDA(tg::dev_malloc((void **)&t->group_root, sizeof(int) * ng1, st));
    TG_CUDA(tg::dev_malloc((void **)&t->group_node, sizeof(int) * ng1, st));
    { k_group_start_keys<<<div_up(ng, 256), 256, 0, st>>>(g0, ng, keys, vals); tg::note_launch(); }
    TG_TRY(radix_sort_pairs(keys, vals, ng, 32, st, t->sort_err));
    { k_permute_groups<<<div_up(ng, 256), 256, 0, st>>>(vals, ng, g0, r0, n0, t->groups, t->group_root, t->group_node); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaFreeAsync(keys, st));
    TG_CUDA(cudaFreeAsync(vals, st));
    TG_CUDA(cudaFreeAsync(g0, st));
    TG_CUDA(cudaFreeAsync(r0, st));
    TG_CUDA(cudaFreeAsync(n0, st));
    TG_CUDA(cudaFreeAsync(cnt, st));
    TG_CUDA(cudaFreeAsync(large, st));
    TG_CUDA(cudaFreeAsync(nlarge, st));
    TG_CUDA(cudaFreeAsync(d_sys, st));
    TG_CUDA(cudaFreeAsync(d_node, st));
    t->ngroups = (int64_t)ng;
    t->groups_G = G;
    return TG_OK;
}

// The tree's side stream and its two events, made on first use.
tg_status tree_side_stream(tg_tree_s *t) {
    if (!t->side) {
        TG_CUDA(pool_stream(&t->side));
        TG_CUDA(pool_event(&t->ev_fork, false));
        TG_CUDA(pool_event(&t->ev_join, false));
    }
    return TG_OK;
}

// Tree groups at size G and the walk arena of the given precision. Grouping and the arena's topology
// part (links, leaf ranges, leaf records) read only the tree's topology and particle data, so for a
// first grouping they run on the tree's side stream from the build's ev_topo, in parallel with the
// moment pass still running on the build's stream (and the grouping's one host read-back of its
// group count waits for the side stream alone). The arena's node records need the moments: st.
// st waits for the side stream before this returns, also on error.
tg_status tree_groups_with_arena(tg_tree_s *t, int G, bool fp64, cudaStream_t st) {
    const bool need_arena = fp64 ? !t->arena64.built : !t->arena32.built;
    const bool need_groups = !(t->groups && t->groups_G == G);
    if (need_groups && !t->groups && t->ev_topo) {  // a first grouping: off the build's critical path
        TG_TRY(tree_side_stream(t));
        TG_CUDA(cudaStreamWaitEvent(t->side, t->ev_topo, 0));
        tg_status r = tree_groups(t, G, t->side);
        const bool topo = r == TG_OK && need_arena;
        if (topo) r = fp64 ? build_arena_topology(t, t->arena64, t->side) : build_arena_topology(t, t->arena32, t->side);
        if (r == TG_OK && !fp64 && !t->own32 && t->ntot > 0) {  // the FP32 walk's own targets, here too
            const cudaError_t ea = tg::dev_malloc((void **)&t->own32, sizeof(float4) * 2 * t->ntot, t->side);
            if (ea != cudaSuccess) {
                t->own32 = nullptr;
                r = TG_ERR_CUDA;
            } else {
                k_prep_targets<float><<<div_up(t->ntot, 256), 256, 0, t->side>>>(t->coord, t->soft, t->ntot, t->own32,
                                                                                 t->own32 + t->ntot);
                tg::note_launch();
            }
        }
        const cudaError_t ej = cudaEventRecord(t->ev_join, t->side);
        if (ej != cudaSuccess) {  // the join could not be recorded: wait for the side stream from the host
            cudaStreamSynchronize(t->side);
            set_last_error_msg("could not record the tree grouping's completion event");
            return TG_ERR_CUDA;
        }
        TG_CUDA(cudaStreamWaitEvent(st, t->ev_join, 0));
        TG_TRY(r);
        if (topo) TG_TRY(fp64 ? build_arena_nodes(t, t->arena64, st) : build_arena_nodes(t, t->arena32, st));
        return TG_OK;
    }
    if (need_groups) TG_TRY(tree_groups(t, G, st));
    if (need_arena) TG_TRY(fp64 ? build_arena(t, t->arena64, st) : build_arena(t, t->arena32, st));
    return TG_OK;
}

// Largest-first queue order of consecutive-block groups (see k_group_cost_keys).
tg_status make_cost_order(const double *tpos, const int2 *groups, int64_t ngroups, int **order, cudaStream_t st,
                          int *sort_err) {
    uint64_t *keys = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&keys, sizeof(uint64_t) * std::max<int64_t>(ngroups, 1), st));
    TG_CUDA(tg::dev_malloc((void **)order, sizeof(int) * std::max<int64_t>(ngroups, 1), st));
    { k_group_cost_keys<<<div_up(ngroups, 256), 256, 0, st>>>(tpos, groups, ngroups, keys, (uint32_t *)*order); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_TRY(radix_sort_pairs(keys, (uint32_t *)*order, ngroups, 32, st, sort_err));
    TG_CUDA(cudaFreeAsync(keys, st));
    return TG_OK;
}

tg_status make_groups(tg_tree_s *t, const std::vector<int64_t> &sys_off_host, int gs, int2 **groups,
                      int **group_root, int64_t *ngroups, cudaStream_t st) {
    int nsys = (int)sys_off_host.size() - 1;
    std::vector<int64_t> goff(nsys + 1, 0);
    std::vector<int> roots(nsys);
    for (int s = 0; s < nsys; s++) {
        goff[s + 1] = goff[s] + (sys_off_host[s + 1] - sys_off_host[s] + gs - 1) / gs;
        roots[s] = (int)t->sys_node_off[s];
    }
    *ngroups = goff[nsys];
    int64_t *d_sys = nullptr, *d_goff = nullptr;
    int *d_roots = nullptr;
    TG_CUDA(tg::dev_malloc((void **)groups, sizeof(int2) * std::max<int64_t>(*ngroups, 1), st));
    TG_CUDA(tg::dev_malloc((void **)group_root, sizeof(int) * std::max<int64_t>(*ngroups, 1), st));
    TG_CUDA(tg::dev_malloc((void **)&d_sys, sizeof(int64_t) * (nsys + 1), st));
    TG_CUDA(tg::dev_malloc((void **)&d_goff, sizeof(int64_t) * (nsys + 1), st));
    TG_CUDA(tg::dev_malloc((void **)&d_roots, sizeof(int) * nsys, st));
    TG_CUDA(cudaMemcpyAsync(d_sys, sys_off_host.data(), sizeof(int64_t) * (nsys + 1), cudaMemcpyHostToDevice, st));
    TG_CUDA(cudaMemcpyAsync(d_goff, goff.data(), sizeof(int64_t) * (nsys + 1), cudaMemcpyHostToDevice, st));
    TG_CUDA(cudaMemcpyAsync(d_roots, roots.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice, st));
    { k_make_groups<<<nsys, 256, 0, st>>>(d_sys, nsys, gs, d_goff, d_roots, *groups, *group_root); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaFreeAsync(d_sys, st));
    TG_CUDA(cudaFreeAsync(d_goff, st));
    TG_CUDA(cudaFreeAsync(d_roots, st));
    // the host vectors above must outlive the async copies
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

}  // namespace tg

// ---------------------------------------------------------------------------------------------
// A tree's walk captured in a CUDA graph (tg_walk_graph_*; declared in include/pytreegrav_gb300.h).
// Everything that needs the host (groups, the arena, the targets' hi/lo split, scratch) is made
// once at creation; the graph holds only stream work: zeroing the counters, the small-stack pass
// and the large-stack pass over the groups that overflowed it. Replays run with no host
// synchronisation; tg_walk_graph_status reads the last replay's status word.

struct tg_walk_graph_s {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int *scratch = nullptr;
    float4 *thi = nullptr, *tlo = nullptr;
    int2 *groups = nullptr;  // owned when the grouping is not the tree's cached one
    int *groot = nullptr, *gorder = nullptr;
    int64_t kernels = 0;     // kernel nodes per replay
};

namespace {

void graph_release(tg_walk_graph_s *g) {
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    void *bufs[] = {g->scratch, g->thi, g->tlo, g->groups, g->groot, g->gorder};
    for (void *b : bufs)
        if (b) cudaFreeAsync(b, 0);
    delete g;
}

}  // namespace

extern "C" {

tg_status tg_walk_graph_create(tg_tree t, int fields, int quadrupole, double theta, double G, int group_size,
                               int grouping, double *out, tg_walk_graph *out_graph) {
    using namespace tg;
    if (!t || !out || !out_graph || (fields & 7) == 0 || (fields & ~7) || !(theta > 0)) return TG_ERR_BAD_ARG;
    if (group_size != 1 && group_size != 2 && group_size != 4 && group_size != 8 && group_size != 16 &&
        group_size != 32)
        return TG_ERR_BAD_ARG;
    if (grouping != TG_GROUP_BLOCKS && grouping != TG_GROUP_TREE) return TG_ERR_BAD_ARG;
    if (quadrupole && !t->has_quads) return TG_ERR_NO_QUADRUPOLES;
    *out_graph = nullptr;
    tg_walk_graph_s *g = new (std::nothrow) tg_walk_graph_s();
    if (!g) return TG_ERR_OOM;
    cudaStream_t cs = nullptr;
    tg_status rc = TG_OK;
    auto fail = [&](tg_status r) {
        if (cs) cudaStreamDestroy(cs);
        graph_release(g);
        return r;
    };
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return fail(TG_ERR_CUDA);
    tree_wait_built(t, cs);
    const int2 *wg;
    const int *wr;
    int64_t ng;
    if (grouping == TG_GROUP_TREE) {
        if ((rc = tree_groups(t, group_size, cs)) != TG_OK) return fail(rc);
        wg = t->groups;
        wr = t->group_root;
        ng = t->ngroups;
    } else {
        if ((rc = make_groups(t, t->sys_off, group_size, &g->groups, &g->groot, &ng, cs)) != TG_OK) return fail(rc);
        if ((rc = make_cost_order(t->coord, g->groups, ng, &g->gorder, cs, t->sort_err)) != TG_OK) return fail(rc);
        wg = g->groups;
        wr = g->groot;
    }
    if ((rc = build_arena(t, t->arena32, cs)) != TG_OK) return fail(rc);
    const int64_t n = t->ntot;
    if (!t->stats_dev && dev_malloc((void **)&t->stats_dev, sizeof(unsigned long long) * 8, cs) != cudaSuccess)
        return fail(TG_ERR_OOM);
    if (dev_malloc((void **)&g->thi, sizeof(float4) * std::max<int64_t>(n, 1), cs) != cudaSuccess ||
        dev_malloc((void **)&g->tlo, sizeof(float4) * std::max<int64_t>(n, 1), cs) != cudaSuccess ||
        dev_malloc((void **)&g->scratch, sizeof(int) * walk_scratch_ints(ng), cs) != cudaSuccess)
        return fail(TG_ERR_OOM);
    { k_prep_targets<float><<<div_up(n, 256), 256, 0, cs>>>(t->coord, t->soft, n, g->thi, g->tlo); note_launch(); }
    int sort_bad = 0;
    if (t->sort_err && cudaMemcpyAsync(&sort_bad, t->sort_err, sizeof(int), cudaMemcpyDeviceToHost, cs) != cudaSuccess)
        return fail(TG_ERR_CUDA);
    if (cudaStreamSynchronize(cs) != cudaSuccess) return fail(TG_ERR_CUDA);
    if (sort_bad) {  // the grouping's or the queue order's sort
        set_last_error_msg("radix sort: a tile's look-back did not complete within its bound");
        return fail(TG_ERR_QUEUE_TIMEOUT);
    }

    WalkArgs<float> a;
    a.ar = t->arena32;
    a.ntot = t->ntot;
    a.tc = t->coord; a.ts = t->soft; a.tsize = t->size; a.tdelta = t->delta;
    a.tpos = t->coord; a.th = t->soft; a.scatter = t->walk_idx; a.groups = wg; a.group_root = wr;
    a.group_order = g->gorder;
    a.ngroups = ng; a.theta = theta; a.theta_group = nullptr; a.tol_group = nullptr; a.G = G;
    a.out_fields = fields;
    a.out_w = ((fields & F_POT) ? 1 : 0) + ((fields & F_ACC) ? 3 : 0) + ((fields & F_TID) ? 9 : 0);
    a.out = out; a.gs = group_size;
    a.stats = (unsigned long long *)t->stats_dev;
    a.gstats = nullptr;
    a.thi = g->thi;
    a.tlo = g->tlo;
    const int64_t launches0 = launches_so_far();
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed) != cudaSuccess) return fail(TG_ERR_CUDA);
    rc = TG_OK;
    if (cudaMemsetAsync(t->stats_dev, 0, sizeof(unsigned long long) * 8, cs) != cudaSuccess) rc = TG_ERR_CUDA;
    if (rc == TG_OK) rc = enqueue_walk<float>(a, fields, quadrupole != 0, t->walk_warps, t->walk_stack, g->scratch, cs);
    cudaError_t ce = cudaStreamEndCapture(cs, &g->graph);
    note_launches(launches0 - launches_so_far());  // recorded, not run
    if (rc != TG_OK) return fail(rc);
    if (ce != cudaSuccess) {
        set_last_error("cudaStreamEndCapture", ce);
        return fail(TG_ERR_CUDA);
    }
    if ((ce = cudaGraphInstantiate(&g->exec, g->graph, 0)) != cudaSuccess) {
        set_last_error("cudaGraphInstantiate", ce);
        return fail(TG_ERR_CUDA);
    }
    size_t nn = 0;
    cudaGraphGetNodes(g->graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(g->graph, nodes.data(), &nn);
    for (auto nd : nodes) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) g->kernels++;
    }
    cudaStreamDestroy(cs);
    *out_graph = g;
    return TG_OK;
}

tg_status tg_walk_graph_launch(tg_walk_graph g, void *stream) {
    if (!g) return TG_ERR_BAD_ARG;
    TG_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    tg::note_launches(g->kernels);
    return TG_OK;
}

tg_status tg_walk_graph_status(tg_walk_graph g, void *stream) {
    if (!g) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    int status = 0;
    TG_CUDA(cudaMemcpyAsync(&status, g->scratch + tg::WS_STATUS, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    if (status & (1 << TG_ERR_CUDA)) {
        tg::set_last_error_msg("internal error: tree links do not form a valid octree for the walk arena");
        return TG_ERR_CUDA;
    }
    if (status & (1 << TG_ERR_STACK_OVERFLOW)) return TG_ERR_STACK_OVERFLOW;
    if (status & (1 << TG_ERR_ITER_LIMIT)) return TG_ERR_ITER_LIMIT;
    return TG_OK;
}

tg_status tg_walk_graph_free(tg_walk_graph g) {
    graph_release(g);
    return TG_OK;
}

}  // extern "C"
