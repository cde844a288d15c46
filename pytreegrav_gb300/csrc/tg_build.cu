// Octree build on the GPU, reproducing pytreegrav's radix build (octree.py:817-1175) bit for bit.
//
// pytreegrav splits Morton-sorted particles top-down with an explicit stack. Here the same tree is
// derived in parallel from the sorted keys alone:
//
//   * L[i], the number of complete 3-bit digits keys i and i+1 share (capped at 21), fixes every
//     node: a node at level k is a maximal run of >= 2 keys sharing their top 3k bits, so the nodes
//     starting at particle i are exactly the levels L[i-1]+1 .. L[i]. A prefix sum of those counts
//     enumerates all nodes; binary searches over the keys give each node's end and parent.
//   * FirstSubnode/NextBranch follow from L in O(1): the element after a subtree ending at e is
//     the outermost run starting at e (octree.py:1003-1009's sibling threading).
//   * Runs whose 63-bit keys are identical are re-keyed relative to their cell and re-split, up to
//     three rounds (octree.py:928-943, RekeySlice 1093-1126), then bucketed (BuildBucket 1128-1175).
//   * Node indices: the serial split allocates a node's children when it pops the node, and pops
//     in reverse preorder -- which sorts nodes by (end descending, depth ascending). Sorting every
//     node by (its allocating parent's position in that order, its own start) therefore yields the
//     reference's node numbering exactly.
//   * Moments are rolled up bottom-up in FP64 with pytreegrav's summation order (particles in
//     Morton order, then child nodes by descending index; octree.py:199-292), every operation
//     rounded once (no FMA), so masses, centres of mass, Deltas and quadrupoles match bit for bit.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "tg_tree.cuh"

namespace tg {

__constant__ double c_octant[8][3] = {
    {-0.25, -0.25, -0.25}, {0.25, -0.25, -0.25}, {-0.25, 0.25, -0.25}, {0.25, 0.25, -0.25},
    {-0.25, -0.25, 0.25},  {0.25, -0.25, 0.25},  {-0.25, 0.25, 0.25},  {0.25, 0.25, 0.25},
};

// Link references before final numbering: >= 0 particle (arena index), -1 none, <= -2 node slot.
__device__ __forceinline__ int64_t node_ref(int64_t slot) { return -(slot + 2); }

__device__ __forceinline__ int64_t find_seg(const int64_t *off, int nseg, int64_t i) {
    // last s with off[s] <= i
    int lo = 0, hi = nseg;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------------------------
// Bounding cube (octree.py:539-574): exact min/max through order-preserving integer atomics.
__global__ void k_bbox_init(unsigned long long *mn, unsigned long long *mx, int nsys) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3 * nsys) {
        mn[i] = ~0ull;
        mx[i] = 0ull;
    }
}

__global__ void __launch_bounds__(BB_THREADS) k_bbox(const double *pos, int64_t n, const int64_t *sys_off, int nsys,
                                                     unsigned long long *mn, unsigned long long *mx) {
    int64_t tile0 = (int64_t)blockIdx.x * BB_THREADS * BB_ITEMS;
    if (tile0 >= n) return;
    int64_t tile1 = min(tile0 + (int64_t)BB_THREADS * BB_ITEMS, n) - 1;
    int s0 = (int)find_seg(sys_off, nsys, tile0), s1 = (int)find_seg(sys_off, nsys, tile1);
    if (s0 == s1) {
        unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
        for (int it = 0; it < BB_ITEMS; it++) {
            int64_t i = tile0 + (int64_t)it * BB_THREADS + threadIdx.x;
            if (i <= tile1) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    unsigned long long u = dbl_to_ordered(pos[3 * i + k]);
                    lo[k] = min(lo[k], u);
                    hi[k] = max(hi[k], u);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            for (int o = 16; o; o >>= 1) {
                lo[k] = min(lo[k], __shfl_xor_sync(FULL, lo[k], o));
                hi[k] = max(hi[k], __shfl_xor_sync(FULL, hi[k], o));
            }
        }
        __shared__ unsigned long long slo[3][BB_THREADS / 32], shi[3][BB_THREADS / 32];
        int w = threadIdx.x >> 5;
        if (lane_id() == 0)
            for (int k = 0; k < 3; k++) {
                slo[k][w] = lo[k];
                shi[k][w] = hi[k];
            }
        __syncthreads();
        if (threadIdx.x < 3) {
            int k = threadIdx.x;
            unsigned long long a = ~0ull, b = 0;
            for (int ww = 0; ww < BB_THREADS / 32; ww++) {
                a = min(a, slo[k][ww]);
                b = max(b, shi[k][ww]);
            }
            atomicMin(&mn[3 * s0 + k], a);
            atomicMax(&mx[3 * s0 + k], b);
        }
    } else {
        for (int it = 0; it < BB_ITEMS; it++) {
            int64_t i = tile0 + (int64_t)it * BB_THREADS + threadIdx.x;
            if (i <= tile1) {
                int s = (int)find_seg(sys_off, nsys, i);
                for (int k = 0; k < 3; k++) {
                    unsigned long long u = dbl_to_ordered(pos[3 * i + k]);
                    atomicMin(&mn[3 * s + k], u);
                    atomicMax(&mx[3 * s + k], u);
                }
            }
        }
    }
}

__global__ void k_bbox_finish(const unsigned long long *mn, const unsigned long long *mx, int nsys, double *center,
                              double *size) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    double lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        lo[k] = ordered_to_dbl(mn[3 * s + k]);
        hi[k] = ordered_to_dbl(mx[3 * s + k]);
        center[3 * s + k] = dmul(0.5, dadd(hi[k], lo[k]));
    }
    double sz = dsub(hi[0], lo[0]);
    if (dsub(hi[1], lo[1]) > sz) sz = dsub(hi[1], lo[1]);
    if (dsub(hi[2], lo[2]) > sz) sz = dsub(hi[2], lo[2]);
    size[s] = sz;
}

// ---------------------------------------------------------------------------------------------
// Morton keys (octree.py:54-98), FP64 with every operation rounded once.
__device__ __forceinline__ uint64_t spread_bits(uint64_t x) {
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// A key cell as the key formula uses it: the corner (centre - size/2) and 1/size.
struct KeyCell {
    double o0, o1, o2, inv;
};
__device__ __forceinline__ KeyCell key_cell(const double *c, double size) {
    KeyCell k;
    k.inv = size > 0 ? ddiv(1.0, size) : 0.0;
    const double h = dmul(0.5, size);
    k.o0 = dsub(c[0], h);
    k.o1 = dsub(c[1], h);
    k.o2 = dsub(c[2], h);
    return k;
}

// int(t * 2^21) truncated toward zero, then clamped to [0, 2^21 - 1] (octree.py:85-96), read off the
// bits of t on the integer units. The product by 2^21 is exact unless it overflows (t >= 2^1003:
// clamped to the top either way) or underflows (t < 2^-1001: zero either way), so t decides alone:
// NaN, negative or below 2^-21 gives 0; 1 or more gives the top; else the top 21 + e bits of the
// significand, e = exponent(t) + 21.
__device__ __forceinline__ uint64_t quantize21(double t) {
    const long long b = __double_as_longlong(t);
    if (b <= 0) return 0;  // +0, and every value with the sign bit set
    const int E = (int)(b >> 52);
    if (E >= 1023) return (E == 2047 && (b & 0xfffffffffffffll)) ? 0 : (1u << MORTON_BITS) - 1;
    const int ev = E - 1023 + MORTON_BITS;
    if (ev < 0) return 0;
    return (uint64_t)(((b & 0xfffffffffffffll) | (1ll << 52)) >> (52 - ev));
}

// Per axis (x - corner) * (1/size), each FP64 operation rounded once, then quantize21.
__device__ __forceinline__ uint64_t morton_key(double x, double y, double z, const KeyCell &k) {
    const uint64_t qx = quantize21(dmul(dsub(x, k.o0), k.inv));
    const uint64_t qy = quantize21(dmul(dsub(y, k.o1), k.inv));
    const uint64_t qz = quantize21(dmul(dsub(z, k.o2), k.inv));
    return spread_bits(qx) | (spread_bits(qy) << 1) | (spread_bits(qz) << 2);
}
__device__ __forceinline__ uint64_t morton_key(double x, double y, double z, const double *c, double size) {
    return morton_key(x, y, z, key_cell(c, size));
}

__global__ void k_keys(const double *pos, int64_t n, const int64_t *sys_off, int nsys, const double *center,
                       const double *size, uint64_t *keys, uint64_t *keys_copy, uint32_t *vals) {
    __shared__ KeyCell one;  // one system: its cell (with the division) formed once per block
    if (nsys == 1) {
        if (threadIdx.x == 0) one = key_cell(center, size[0]);
        __syncthreads();
    }
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = nsys > 1 ? (int)find_seg(sys_off, nsys, i) : 0;
    const KeyCell kc = nsys == 1 ? one : key_cell(center + 3 * s, size[s]);
    uint64_t k = morton_key(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], kc);
    keys[i] = k;
    if (keys_copy) keys_copy[i] = k;
    vals[i] = (uint32_t)i;
}

__global__ void k_sys_of(const uint32_t *vals, int64_t n, const int64_t *sys_off, int nsys, uint64_t *out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint64_t)find_seg(sys_off, nsys, vals[i]);
}

// _permute_particles (octree.py:577-603)
// sort_err set (the sort gave up and left the identity permutation): the keys stay the sort's
// fallback keys i, so that every later kernel sees sorted keys (the build then reports the error).
__global__ void k_gather(const uint32_t *perm, int64_t n, const double *pos, const double *m, const double *h,
                         const uint64_t *keys_in, double *coord, double *mass, double *soft, uint64_t *keys_sorted,
                         int64_t *walk_idx, const int *sort_err) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t o = perm[i];
    coord[3 * i] = pos[3 * o];
    coord[3 * i + 1] = pos[3 * o + 1];
    coord[3 * i + 2] = pos[3 * o + 2];
    mass[i] = m ? m[o] : 0.0;
    soft[i] = h ? h[o] : 0.0;
    keys_sorted[i] = *sort_err ? (uint64_t)i : keys_in[o];
    walk_idx[i] = o;
}

// ---------------------------------------------------------------------------------------------
// Split rounds. A round works on segments: round 0 has one per system; a later round has one per
// key-exhausted node of the previous round. Elements e of a round enumerate the segments'
// particles in order.
struct Segs {
    int n = 0;
    int64_t *lo = nullptr, *hi = nullptr;      // particle range
    int64_t *root = nullptr;                   // existing root node slot, or -1 to create one
    double *center = nullptr, *size = nullptr; // cell the keys are relative to
    int32_t *depth0 = nullptr;                 // depth of the segment root
    int64_t *next_ref = nullptr;               // NextBranch of the segment root
    int32_t *sys = nullptr;                    // owning system
    int64_t *eoff = nullptr;                   // element offsets (n + 1)
};

struct Nodes {  // node slots in discovery order
    int64_t cap = 0, count = 0;
    int64_t *lo = nullptr, *hi = nullptr, *parent = nullptr, *first = nullptr, *next = nullptr;
    int64_t *aparent = nullptr, *rank = nullptr;  // allocating parent slot, sibling order key
    int8_t *digit = nullptr;  // octant digit at the slot's level: the sibling order among split nodes
    int32_t *depth = nullptr, *sys = nullptr;
    int32_t *seg = nullptr;  // segment of the round that made the slot (for k_node_centers)
    int8_t *level = nullptr;
    double *center = nullptr, *size = nullptr;
};

__device__ __forceinline__ int pair_level(uint64_t a, uint64_t b) {
    int c = __clzll((long long)(a ^ b));  // 64 when equal
    int l = (c - 1) / 3;
    return l > MAX_LEVEL ? MAX_LEVEL : l;
}

__device__ __forceinline__ uint64_t prefix(uint64_t key, int level) {
    return level <= 0 ? 0 : (key >> (63 - 3 * level));
}

struct RoundView {
    const int64_t *seg_lo, *seg_hi, *seg_root, *seg_next, *eoff;
    const double *seg_center, *seg_size;
    const int32_t *seg_depth0, *seg_sys;
    int nseg;
};

__device__ __forceinline__ void elem_loc(const RoundView &v, int64_t e, int &s, int64_t &i) {
    s = (int)find_seg(v.eoff, v.nseg, e);
    i = v.seg_lo[s] + (e - v.eoff[s]);
}

__global__ void k_levels(RoundView v, int64_t E, const uint64_t *keys, int8_t *L) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int s;
    int64_t i;
    elem_loc(v, e, s, i);
    L[e] = (i + 1 < v.seg_hi[s]) ? (int8_t)pair_level(keys[i], keys[i + 1]) : (int8_t)-1;
}

// lowest level of a node starting at element e (e's particle i); root level 0 only at a segment
// start whose root is created this round.
__device__ __forceinline__ int lvl0(const RoundView &v, const int8_t *L, int s, int64_t e, int64_t i) {
    if (i == v.seg_lo[s]) return v.seg_root[s] >= 0 ? 1 : 0;
    return L[e - 1] + 1;
}

__global__ void k_counts(RoundView v, int64_t E, const int8_t *L, int64_t *cnt) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int s;
    int64_t i;
    elem_loc(v, e, s, i);
    int lo = lvl0(v, L, s, e, i);
    int hi = L[e];
    if (lo == 0 && hi < 0) hi = 0;  // a one-particle system still has its root
    cnt[e] = hi >= lo ? (hi - lo + 1) : 0;
}

// last index in [a, b) with prefix(key, level) == p (keys sorted): upper bound - 1
__device__ __forceinline__ int64_t upper_prefix(const uint64_t *keys, int64_t a, int64_t b, uint64_t p, int level) {
    while (a < b) {
        int64_t mid = (a + b) >> 1;
        if (prefix(keys[mid], level) <= p) a = mid + 1;
        else b = mid;
    }
    return a;
}
// upper_prefix over [a, b) by galloping from a: cheap when the answer lies near a.
__device__ __forceinline__ int64_t gallop_upper_prefix(const uint64_t *keys, int64_t a, int64_t b, uint64_t p,
                                                       int level) {
    int64_t step = 1;
    while (a + step - 1 < b && prefix(keys[a + step - 1], level) <= p) {
        a += step;
        step <<= 1;
    }
    int64_t e = a + step - 1;
    return upper_prefix(keys, a, e < b ? e : b, p, level);
}
__device__ __forceinline__ int64_t lower_prefix(const uint64_t *keys, int64_t a, int64_t b, uint64_t p, int level) {
    while (a < b) {
        int64_t mid = (a + b) >> 1;
        if (prefix(keys[mid], level) < p) a = mid + 1;
        else b = mid;
    }
    return a;
}

// lower_prefix over [a, b] where keys[b] has prefix p, by galloping down from b: cheap when the
// run of prefix p starts near b (a node's particles end at or after i, and most runs are short).
__device__ __forceinline__ int64_t gallop_lower_prefix(const uint64_t *keys, int64_t a, int64_t b, uint64_t p,
                                                       int level) {
    int64_t step = 1;
    while (b - step >= a && prefix(keys[b - step], level) >= p) {
        b -= step;
        step <<= 1;
    }
    const int64_t lo = b - step + 1 > a ? b - step + 1 : a;  // keys[b - step] (if >= a) is below p
    return lower_prefix(keys, lo, b, p, level);
}

// slot of the node at `level` containing particle i (level >= lvl0 of the segment root)
__device__ __forceinline__ int64_t node_at(const RoundView &v, const int8_t *L, const int64_t *nstart,
                                           int64_t slot_base, const uint64_t *keys, int s, int64_t i, int level) {
    if (level == 0 && v.seg_root[s] >= 0) return v.seg_root[s];
    int64_t lo = v.seg_lo[s];
    int64_t p_lo = gallop_lower_prefix(keys, lo, i, prefix(keys[i], level), level);
    int64_t pe = v.eoff[s] + (p_lo - lo);
    return slot_base + nstart[pe] + (level - lvl0(v, L, s, pe, p_lo));
}

// NextBranch reference of an element whose particle range ends at e_end (exclusive)
__device__ __forceinline__ int64_t next_after(const RoundView &v, const int8_t *L, const int64_t *nstart,
                                              int64_t slot_base, int s, int64_t e_end_particle) {
    if (e_end_particle >= v.seg_hi[s]) return v.seg_next[s];
    int64_t pe = v.eoff[s] + (e_end_particle - v.seg_lo[s]);
    int outer = L[pe - 1] + 1;
    return (outer <= L[pe]) ? node_ref(slot_base + nstart[pe]) : e_end_particle;
}

// Node slots beyond nd.cap are not written (the host sees the round's node total, grows the slot
// arrays and runs the round's node kernels again); so are exhausted-run entries beyond exh_cap.
__global__ void k_nodes(RoundView v, int64_t E, const int8_t *L, const int64_t *nstart, const int64_t *cnt,
                        int64_t slot_base, const uint64_t *keys, Nodes nd, int64_t *exhausted,
                        unsigned long long *n_exhausted, int64_t exh_cap, int64_t *root_first) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    if (slot_base + nstart[e] + cnt[e] > nd.cap) return;
    int s;
    int64_t i;
    elem_loc(v, e, s, i);
    int l0 = lvl0(v, L, s, e, i);
    uint64_t key = keys[i];
    int64_t seg_lo = v.seg_lo[s], seg_hi = v.seg_hi[s];
    // existing segment root (a re-keyed node): its first child is the level-1 run at seg_lo
    if (i == seg_lo && v.seg_root[s] >= 0) {
        root_first[s] = (1 <= L[e]) ? node_ref(slot_base + nstart[e]) : i;
    }
    const int64_t nc = cnt[e];
    const int64_t slot0 = slot_base + nstart[e];
    for (int64_t j = 0; j < nc; j++) {
        int k = l0 + (int)j;
        int64_t slot = slot0 + j;
        nd.lo[slot] = i;
        nd.level[slot] = (int8_t)k;
        nd.depth[slot] = v.seg_depth0[s] + k;
        nd.sys[slot] = v.seg_sys[s];
        // the element's nodes are nested runs starting at i: all but the first have the
        // previous slot as parent
        int64_t par = (k == 0) ? -1 : (j > 0 ? slot - 1 : node_at(v, L, nstart, slot_base, keys, s, i, k - 1));
        nd.parent[slot] = par;
        nd.aparent[slot] = par;
        nd.rank[slot] = i;
        nd.digit[slot] = k > 0 ? (int8_t)((key >> (63 - 3 * k)) & 7) : (int8_t)0;
        nd.seg[slot] = s;
        if (k == MAX_LEVEL) {
            nd.first[slot] = -1;  // set by the re-key round or the bucket
            unsigned long long q = atomicAdd(n_exhausted, 1ull);
            if ((int64_t)q < exh_cap) exhausted[q] = slot;
        } else {
            nd.first[slot] = (k + 1 <= L[e]) ? node_ref(slot + 1) : i;
        }
    }
    // run ends, deepest first: a shallower run ends at or after the deeper one, so each search
    // gallops on from the previous end
    int64_t hi = i + 1;
    for (int64_t j = nc - 1; j >= 0; j--) {
        int k = l0 + (int)j;
        int64_t slot = slot0 + j;
        hi = (k == 0) ? seg_hi : gallop_upper_prefix(keys, hi, seg_hi, prefix(key, k), k);
        nd.hi[slot] = hi;
        nd.next[slot] = next_after(v, L, nstart, slot_base, s, hi);
    }
}

// x * 2^-q for q in {1, 2}, exactly: an exponent decrement when x and the result are normal
// numbers (the common case, on the integer units), else the FP64 multiply, which is then exact too.
__device__ __forceinline__ double scale_down(double x, int q) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex > q && ex < 0x7ff) return __longlong_as_double(b - ((long long)q << 52));
    return dmul(x, q == 1 ? 0.5 : 0.25);
}

// Geometric centre and size of every node slot of a round: the octant digits of the slot's key
// applied from its segment's cell down to the slot's level (octree.py:974-978), in the reference's
// order: centre += size * (+-1/4) per axis, then size *= 1/2. The products are powers-of-two
// scalings (exact), so only the additions round, each once, as there.
// FP64 instructions cost a warp the same with any number of active lanes, so the block's slots are
// first ordered by level (a counting sort in shared memory, deepest first): a warp's lanes then run
// equal numbers of steps. Which thread takes which slot does not change any result.
constexpr int CENTER_BLOCK = 256;
__global__ void __launch_bounds__(CENTER_BLOCK) k_node_centers(RoundView v, Nodes nd, int64_t slot_base,
                                                               int64_t count, const uint64_t *keys) {
    __shared__ int bin[MAX_LEVEL + 1];
    __shared__ int64_t order[CENTER_BLOCK];
    const int t = threadIdx.x;
    const int64_t mine = slot_base + (int64_t)blockIdx.x * CENTER_BLOCK + t;
    const bool valid = mine < slot_base + count && mine < nd.cap;
    int lv = valid ? (int)nd.level[mine] : 0;
    lv = lv < 0 ? 0 : (lv > MAX_LEVEL ? MAX_LEVEL : lv);
    if (t <= MAX_LEVEL) bin[t] = 0;
    __syncthreads();
    const int r = atomicAdd(&bin[lv], 1);
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int b = MAX_LEVEL; b >= 0; b--) {
            const int c = bin[b];
            bin[b] = run;
            run += c;
        }
    }
    __syncthreads();
    order[bin[lv] + r] = valid ? mine : -1;
    __syncthreads();
    const int64_t slot = order[t];
    if (slot < 0) return;
    const int s = nd.seg[slot];
    const int k = nd.level[slot];
    const uint64_t key = keys[nd.lo[slot]];
    double c0 = v.seg_center[3 * s], c1 = v.seg_center[3 * s + 1], c2 = v.seg_center[3 * s + 2];
    double sz = v.seg_size[s];
    for (int at = 0; at < k; at++) {
        const int d = (int)((key >> (63 - 3 * (at + 1))) & 7);
        const double q = scale_down(sz, 2);  // size / 4
        c0 = dadd(c0, (d & 1) ? q : -q);
        c1 = dadd(c1, (d & 2) ? q : -q);
        c2 = dadd(c2, (d & 4) ? q : -q);
        sz = scale_down(sz, 1);
    }
    nd.center[3 * slot] = c0;
    nd.center[3 * slot + 1] = c1;
    nd.center[3 * slot + 2] = c2;
    nd.size[slot] = sz;
}

__global__ void k_particles(RoundView v, int64_t E, const int8_t *L, const int64_t *nstart, int64_t slot_base,
                            const uint64_t *keys, int64_t *p_parent, int64_t *p_next) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int s;
    int64_t i;
    elem_loc(v, e, s, i);
    int lprev = (i == v.seg_lo[s]) ? -1 : L[e - 1];
    int K = max(lprev, (int)L[e]);
    if (K >= MAX_LEVEL) return;  // inside a key-exhausted run: the next round places it
    if (K < 0) K = 0;            // lone particle of its segment: child of the root
    p_parent[i] = node_at(v, L, nstart, slot_base, keys, s, i, K);
    p_next[i] = next_after(v, L, nstart, slot_base, s, i + 1);
}

__global__ void k_set_root_first(const int64_t *seg_root, const int64_t *root_first, int nseg, int64_t *nd_first) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nseg && seg_root[s] >= 0) nd_first[seg_root[s]] = root_first[s];
}

// Next round's segments from the exhausted node slots.
__global__ void k_make_segs(const int64_t *exh, int n, Nodes nd, Segs sg) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int64_t x = exh[q];
    sg.lo[q] = nd.lo[x];
    sg.hi[q] = nd.hi[x];
    sg.root[q] = x;
    sg.center[3 * q] = nd.center[3 * x];
    sg.center[3 * q + 1] = nd.center[3 * x + 1];
    sg.center[3 * q + 2] = nd.center[3 * x + 2];
    sg.size[q] = nd.size[x];
    sg.depth0[q] = nd.depth[x];
    sg.next_ref[q] = nd.next[x];
    sg.sys[q] = nd.sys[x];
}

__global__ void k_seg_sizes(const int64_t *lo, const int64_t *hi, int n, int64_t *sizes) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) sizes[q] = hi[q] - lo[q];
}

// RekeySlice (octree.py:1093-1126): keys relative to the node's cell, sorted stably per segment.
__global__ void k_rekey_keys(RoundView v, int64_t E, const double *coord, uint64_t *k_sort, uint32_t *vals) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    int s;
    int64_t i;
    elem_loc(v, e, s, i);
    k_sort[e] = morton_key(coord[3 * i], coord[3 * i + 1], coord[3 * i + 2], v.seg_center + 3 * s, v.seg_size[s]);
    vals[e] = (uint32_t)e;
}
__global__ void k_rekey_segkeys(RoundView v, const uint32_t *vals, int64_t E, uint64_t *out) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a < E) out[a] = (uint64_t)find_seg(v.eoff, v.nseg, (int64_t)vals[a]);
}
// gather the permuted slice into temporaries (by element), then write back
// sort_err set: the segments' keys become their element indices (sorted within every segment).
__global__ void k_rekey_gather(RoundView v, int64_t E, const uint32_t *vals, const double *coord, const double *mass,
                               const double *soft, const int64_t *widx, const uint64_t *newkeys_by_elem, double *tc,
                               double *tm, double *ts, int64_t *tw, uint64_t *tk, const int *sort_err) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= E) return;
    int64_t esrc = vals[a];
    int s;
    int64_t isrc;
    elem_loc(v, esrc, s, isrc);
    tc[3 * a] = coord[3 * isrc];
    tc[3 * a + 1] = coord[3 * isrc + 1];
    tc[3 * a + 2] = coord[3 * isrc + 2];
    tm[a] = mass[isrc];
    ts[a] = soft[isrc];
    tw[a] = widx[isrc];
    tk[a] = *sort_err ? (uint64_t)a : newkeys_by_elem[esrc];
}
__global__ void k_rekey_scatter(RoundView v, int64_t E, const double *tc, const double *tm, const double *ts,
                                const int64_t *tw, const uint64_t *tk, double *coord, double *mass, double *soft,
                                int64_t *widx, uint64_t *keys) {
    int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= E) return;
    int s;
    int64_t i;
    elem_loc(v, a, s, i);
    coord[3 * i] = tc[3 * a];
    coord[3 * i + 1] = tc[3 * a + 1];
    coord[3 * i + 2] = tc[3 * a + 2];
    mass[i] = tm[a];
    soft[i] = ts[a];
    widx[i] = tw[a];
    keys[i] = tk[a];
}

// BuildBucket (octree.py:1128-1175) for the nodes still exhausted after three re-keys.
__global__ void k_bucket_counts(const int64_t *exh, int n, const int64_t *nd_lo, const int64_t *nd_hi, int64_t *nchain) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int64_t c = nd_hi[exh[q]] - nd_lo[exh[q]];
    nchain[q] = c >= 2 ? (c - 2) / 7 : 0;
}

__global__ void k_bucket(const int64_t *exh, int n, const int64_t *chain_off, int64_t slot_base, Nodes nd,
                         int64_t *p_parent, int64_t *p_next) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int64_t x = exh[q];
    int64_t lo = nd.lo[x], hi = nd.hi[x], c = hi - lo;
    int64_t nch = c >= 2 ? (c - 2) / 7 : 0;
    int64_t base = slot_base + chain_off[q];
    int64_t xnext = nd.next[x];
    nd.first[x] = lo;
    double c0 = nd.center[3 * x], c1 = nd.center[3 * x + 1], c2 = nd.center[3 * x + 2], sz = nd.size[x];
    for (int64_t j = 1; j <= nch; j++) {
        int64_t sl = base + j - 1;
        c0 = dadd(c0, dmul(sz, c_octant[7][0]));
        c1 = dadd(c1, dmul(sz, c_octant[7][1]));
        c2 = dadd(c2, dmul(sz, c_octant[7][2]));
        sz = dmul(sz, 0.5);
        nd.lo[sl] = lo + 7 * j;
        nd.hi[sl] = hi;
        nd.level[sl] = MAX_LEVEL;
        nd.depth[sl] = nd.depth[x] + (int)j;
        nd.sys[sl] = nd.sys[x];
        nd.parent[sl] = (j == 1) ? x : sl - 1;
        nd.aparent[sl] = x;
        nd.rank[sl] = lo + 7 * j;
        nd.digit[sl] = 0;
        nd.center[3 * sl] = c0;
        nd.center[3 * sl + 1] = c1;
        nd.center[3 * sl + 2] = c2;
        nd.size[sl] = sz;
        nd.first[sl] = lo + 7 * j;
        nd.next[sl] = xnext;
    }
    for (int64_t jj = 0; jj < c; jj++) {
        int64_t owner = min(jj / 7, nch);
        int64_t i = lo + jj;
        p_parent[i] = owner == 0 ? x : base + owner - 1;
        if (jj == c - 1) p_next[i] = xnext;
        else if (owner < nch && jj == 7 * owner + 6) p_next[i] = node_ref(base + owner);
        else p_next[i] = i + 1;
    }
}

// ---------------------------------------------------------------------------------------------
// Index validation: every slot or particle reference the later kernels dereference is checked
// once; a bad one stops the build with an error instead of an out-of-bounds access.
__device__ __forceinline__ bool ref_ok(int64_t r, int64_t N, int64_t M) {
    if (r >= 0) return r < N;
    if (r == -1) return true;
    return (-r - 2) < M;
}
__global__ void k_validate_links(int64_t NE, const int64_t *first, const int64_t *next, const int64_t *parent,
                                 int *bad) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NE) return;
    bool ok = first[i] >= -1 && first[i] < NE && next[i] >= -1 && next[i] < NE && parent[i] >= -1 && parent[i] < NE;
    if (!ok) atomicOr(bad, 4);
}

// Values the host reads back after a split round, gathered so that one copy (one synchronisation)
// serves them all. depth_hist counts node slots per depth; depths >= DEPTH_CAP share the last bin.
constexpr int DEPTH_CAP = 48;
struct BuildSummary {
    unsigned long long nodes;  // node slots made by the round (its scan total)
    unsigned long long n_exh;  // key-exhausted runs found by the round
    int bad;                   // invalid references (bit flags)
    int nonfinite;             // the input check's flag, copied in before the read-back
    int depth_hist[DEPTH_CAP + 1];
};

// Slot validation (as above) plus the depth histogram, over the slots [0, M) with
// M = M_base + *M_round (clamped to the slot capacity).
__global__ void k_summarize_slots(Nodes nd, int64_t M_base, const unsigned long long *M_round, const int64_t *p_parent,
                                  const int64_t *p_next, int64_t N, BuildSummary *sum) {
    __shared__ int hist[DEPTH_CAP + 1];
    for (int b = threadIdx.x; b <= DEPTH_CAP; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    int64_t M = M_base + (M_round ? (int64_t)*M_round : 0);
    if (M > nd.cap) M = nd.cap;
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < M) {
        bool ok = nd.parent[c] >= -1 && nd.parent[c] < M && nd.aparent[c] >= -1 && nd.aparent[c] < M &&
                  ref_ok(nd.first[c], N, M) && ref_ok(nd.next[c], N, M) && nd.first[c] != -1 && nd.lo[c] >= 0 &&
                  nd.hi[c] <= N && nd.lo[c] < nd.hi[c];
        if (!ok) atomicOr(&sum->bad, 1);
        int d = nd.depth[c];
        atomicAdd(&hist[d < 0 ? 0 : (d > DEPTH_CAP ? DEPTH_CAP : d)], 1);
    }
    if (c < N) {
        bool ok = p_parent[c] >= 0 && p_parent[c] < M && ref_ok(p_next[c], N, M);
        if (!ok) atomicOr(&sum->bad, 2);
    }
    __syncthreads();
    for (int b = threadIdx.x; b <= DEPTH_CAP; b += blockDim.x)
        if (hist[b]) atomicAdd(&sum->depth_hist[b], hist[b]);
}

// Node slots per system -> node offsets (exclusive scan done by the caller).
__global__ void k_sys_node_counts(const int32_t *nd_sys, int64_t M, int64_t *cnt) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < M) atomicAdd((unsigned long long *)&cnt[nd_sys[c]], 1ull);
}
__global__ void k_single_sys_node_off(int64_t *sys_node_off, int64_t M) {
    sys_node_off[0] = 0;
    sys_node_off[1] = M;
}

// ---------------------------------------------------------------------------------------------
// Numbering.
struct NumberingBits {
    int lb;  // bits of a system-local particle index
    int db;  // bits of a depth
};

// root_key sorts after every other key (1 << the key width, or all ones when the width is 64).
// Nodes are numbered by allocating parent (its particle range's end, descending, then its depth) and
// among one parent's children by first particle. Without bucket chains a parent's children are split
// cells, whose first particles are in octant-digit order: compact keys then carry the 3-bit digit
// instead of the first particle, which saves sort passes. (A bucket chain hangs all its nodes on one
// allocating parent, so it needs the full first-particle rank.)
__global__ void k_number_keys(Nodes nd, int64_t count, const int64_t *sys_off, NumberingBits b, uint64_t root_key,
                              int compact, uint64_t *keys, uint32_t *vals, int64_t *root_slot_of_sys,
                              int *nonroot_count) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    int s = nd.sys[c];
    int64_t ap = nd.aparent[c];
    if (ap < 0) {  // a system root
        root_slot_of_sys[s] = c;
        keys[c] = root_key;
        vals[c] = (uint32_t)c;
        return;
    }
    int64_t off = sys_off[s];
    int64_t nsys_part = sys_off[s + 1] - off;
    const int low = compact ? 3 : b.lb;  // bits of the sibling order key
    const uint64_t sib = compact ? (uint64_t)(nd.digit[c] & 7) : (uint64_t)(nd.rank[c] - off);
    uint64_t k = ((uint64_t)s << (b.lb + b.db + low)) | ((uint64_t)(nsys_part - (nd.hi[ap] - off)) << (b.db + low)) |
                 ((uint64_t)nd.depth[ap] << low) | sib;
    keys[c] = k;
    vals[c] = (uint32_t)c;
    atomicAdd(nonroot_count, 1);
}

// sort_err set (the numbering sort left the identity, roots not last): every slot keeps its own
// index, a bijection onto the node range, so the arrays written from it stay in bounds.
__global__ void k_final_index(const uint32_t *vals, int64_t count, const int32_t *nd_sys, int64_t ntot,
                              const int64_t *sys_node_off, int64_t *final_of_slot, const int64_t *root_slot_of_sys,
                              int nsys, const int *sort_err) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (*sort_err) {
        if (q < count) final_of_slot[q] = ntot + q;
        return;
    }
    if (q < count) {
        int64_t c = vals[q];
        int s = nd_sys[c];
        if (q < count - nsys) final_of_slot[c] = ntot + q + s + 1;
    }
    if (q < nsys) final_of_slot[root_slot_of_sys[q]] = ntot + sys_node_off[q];
}

__device__ __forceinline__ int64_t resolve(int64_t ref, const int64_t *final_of_slot) {
    if (ref >= 0) return ref;
    if (ref == -1) return -1;
    return final_of_slot[-ref - 2];
}

// Besides the node arrays, files every node into the list of its depth (lvl_list, sections at
// lvl_off[d]; depths >= DEPTH_CAP share the last section) for the level-by-level moment pass.
__global__ void k_write_nodes(Nodes nd, int64_t count, const int64_t *final_of_slot, double *coord, double *size,
                              double *mass, double *soft, double *delta, int64_t *first, int64_t *next,
                              int64_t *parent, int2 *range, double *cell, int64_t ntot, const int *lvl_off,
                              int *lvl_cursor, int32_t *lvl_list, int8_t *fdepth) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    int64_t f = final_of_slot[c];
    mass[f] = 0.0;  // the moment pass fills these
    soft[f] = 0.0;
    delta[f] = 0.0;
    {
        int d = nd.depth[c];
        d = d < 0 ? 0 : (d > DEPTH_CAP ? DEPTH_CAP : d);
        unsigned peers = __match_any_sync(__activemask(), d);
        int leader = __ffs(peers) - 1;
        int base = 0;
        if (lane_id() == leader) base = atomicAdd(&lvl_cursor[d], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        lvl_list[lvl_off[d] + base + __popc(peers & lanemask_lt())] = (int32_t)(f - ntot);
        fdepth[f - ntot] = (int8_t)d;
    }
    range[f - ntot] = make_int2((int)nd.lo[c], (int)nd.hi[c]);
    cell[3 * (f - ntot)] = nd.center[3 * c];
    cell[3 * (f - ntot) + 1] = nd.center[3 * c + 1];
    cell[3 * (f - ntot) + 2] = nd.center[3 * c + 2];
    coord[3 * f] = nd.center[3 * c];
    coord[3 * f + 1] = nd.center[3 * c + 1];
    coord[3 * f + 2] = nd.center[3 * c + 2];
    size[f] = nd.size[c];
    first[f] = resolve(nd.first[c], final_of_slot);
    next[f] = resolve(nd.next[c], final_of_slot);
    parent[f] = nd.parent[c] < 0 ? -1 : final_of_slot[nd.parent[c]];
}

// Particle rows of the final arrays, the Morton-ordered coordinates, masses and softenings included.
__global__ void k_write_particles(int64_t ntot, const int64_t *p_parent, const int64_t *p_next,
                                  const int64_t *final_of_slot, const double *pc, const double *pm, const double *ps,
                                  double *coord, double *mass, double *soft, int64_t *first, int64_t *next,
                                  int64_t *parent, double *size, double *delta) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntot) return;
    coord[3 * i] = pc[3 * i];
    coord[3 * i + 1] = pc[3 * i + 1];
    coord[3 * i + 2] = pc[3 * i + 2];
    mass[i] = pm[i];
    soft[i] = ps[i];
    first[i] = -1;
    next[i] = resolve(p_next[i], final_of_slot);
    parent[i] = final_of_slot[p_parent[i]];
    size[i] = 0.0;
    delta[i] = 0.0;
}

// Children of every node in the order the moment sums take them (octree.py:199-292): particle
// children in chain order, then node children in reverse chain order. An entry >= 0 is a particle
// index, an entry < 0 the node ~entry; nk holds the count (at most 8, as the chain walks in the
// moment kernels allow). A second walk over the chain (whose lines the first one brought into L1)
// places the node children from the back, so no local array is needed.
__global__ void k_kids(int64_t ntot, int64_t mtot, const int64_t *first, const int64_t *next, int32_t *kids,
                       int8_t *nk) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mtot) return;
    const int64_t f = ntot + j, stop = next[f], ne = ntot + mtot;
    int32_t *out = kids + 8 * j;
    int np = 0, nn = 0;
    for (int64_t c = first[f]; c != stop && c >= 0 && c < ne && np + nn < 8; c = next[c]) {
        if (c < ntot) out[np++] = (int32_t)c;
        else nn++;
    }
    int w = np + nn;
    int s = 0;
    for (int64_t c = first[f]; c != stop && c >= 0 && c < ne && s < 8; c = next[c], s++)
        if (c >= ntot) out[--w] = ~(int32_t)(c - ntot);
    nk[j] = (int8_t)(np + nn);
}

// Capacity bookkeeping for a bucket (octree.py:930-933): new_node_idx when the bucket is reached
// plus the worst-case chain; new_node_idx there is 1 + the number of nodes the split allocated
// earlier, i.e. the sorted position of the bucket's first allocation.
__global__ void k_bucket_requirement(const int64_t *exh, int n, Nodes nd, const int64_t *sys_off, NumberingBits b,
                                     const uint64_t *sorted_keys, int64_t count, int64_t ntot,
                                     unsigned long long *req) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int64_t x = exh[q];
    int s = nd.sys[x];
    int64_t off = sys_off[s], np = sys_off[s + 1] - off;
    uint64_t key = ((uint64_t)s << (2 * b.lb + b.db)) | ((uint64_t)(np - (nd.hi[x] - off)) << (b.lb + b.db)) |
                   ((uint64_t)nd.depth[x] << b.lb) | (uint64_t)(nd.lo[x] - off);
    int64_t a = 0, z = count;
    while (a < z) {
        int64_t mid = (a + z) >> 1;
        if (sorted_keys[mid] < key) a = mid + 1;
        else z = mid;
    }
    // a = global sorted position; the system's earlier non-root nodes are those with smaller keys
    // from the same system: subtract the count of keys of earlier systems.
    uint64_t sys_key = (uint64_t)s << (2 * b.lb + b.db);
    int64_t a0 = 0, z0 = count;
    while (a0 < z0) {
        int64_t mid = (a0 + z0) >> 1;
        if (sorted_keys[mid] < sys_key) a0 = mid + 1;
        else z0 = mid;
    }
    int64_t new_node_idx = np + 1 + (a - a0);
    int64_t need = new_node_idx + (nd.hi[x] - nd.lo[x]) / 7 + 2;
    atomicMax(&req[s], (unsigned long long)need);
}

// ---------------------------------------------------------------------------------------------
// Moments. Children are reached through FirstSubnode/NextBranch: a node's chain lists its
// particle children and node children in digit order, and its node children carry consecutive
// indices, so "descending index" is the reverse of their order in the chain.
__global__ void k_count_node_children(int64_t ntot, int64_t mtot, const int64_t *parent, int *nchild) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mtot) return;
    int64_t p = parent[ntot + j];
    if (p >= 0) atomicAdd(&nchild[p - ntot], 1);
}

struct MomentArgs {
    int64_t ntot, mtot;
    double *coord, *mass, *soft, *delta;
    double *acc;                     // per node (3): mass-weighted coordinate sums
    float4 *quad32;                  // per node (2): FP32 quadrupole (xx xy xz yy)(yz zz 0 0), or null
    double *quad;                    // per node (9): FP64 quadrupole (the quadrupole pass only)
    const int64_t *first, *next, *parent;
    int *nchild, *arrived;
};

__device__ __forceinline__ void shift_quad(double *Q, double m, double r0, double r1, double r2) {
    double rsq = dadd(dadd(dmul(r0, r0), dmul(r1, r1)), dmul(r2, r2));
    double t;
    t = dmul(m, dsub(dmul(dmul(3.0, r0), r0), rsq)); Q[0] = dadd(Q[0], t);
    t = dmul(dmul(dmul(m, 3.0), r0), r1);           Q[1] = dadd(Q[1], t);
    t = dmul(dmul(dmul(m, 3.0), r0), r2);           Q[2] = dadd(Q[2], t);
    t = dmul(dmul(dmul(m, 3.0), r1), r0);           Q[3] = dadd(Q[3], t);
    t = dmul(m, dsub(dmul(dmul(3.0, r1), r1), rsq)); Q[4] = dadd(Q[4], t);
    t = dmul(dmul(dmul(m, 3.0), r1), r2);           Q[5] = dadd(Q[5], t);
    t = dmul(dmul(dmul(m, 3.0), r2), r0);           Q[6] = dadd(Q[6], t);
    t = dmul(dmul(dmul(m, 3.0), r2), r1);           Q[7] = dadd(Q[7], t);
    t = dmul(m, dsub(dmul(dmul(3.0, r2), r2), rsq)); Q[8] = dadd(Q[8], t);
}

// The FP32 quadrupole the FP32 walk uses, Q = (xx, xy, xz, yy, yz, zz): the same shift (a child of
// mass m at offset r from the node's centre of mass adds m (3 r_a r_b - delta_ab r^2), a node child
// its own quadrupole too) summed in FP32, the offsets formed from hi/lo FP32 splits (off32). GB300 issues
// FP64 at 1/73 of the FP32 rate and these sums were most of the moment pass's FP64 instructions;
// the FP64 quadrupoles (pytreegrav's, bit for bit) come from the quadrupole pass when first needed.
// Each child's term T = (its quadrupole, for a node) + shift is formed apart and then added to the
// node's sum in child order, every operation rounded once, so every kernel gives the same FP32 value.
__device__ __forceinline__ void quad32_term(float *T, float m, float rx, float ry, float rz) {
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)), __fmul_rn(rz, rz));
    const float m3 = __fmul_rn(3.f, m);
    T[0] = __fadd_rn(T[0], __fmul_rn(m, __fsub_rn(__fmul_rn(__fmul_rn(3.f, rx), rx), r2)));
    T[1] = __fadd_rn(T[1], __fmul_rn(__fmul_rn(m3, rx), ry));
    T[2] = __fadd_rn(T[2], __fmul_rn(__fmul_rn(m3, rx), rz));
    T[3] = __fadd_rn(T[3], __fmul_rn(m, __fsub_rn(__fmul_rn(__fmul_rn(3.f, ry), ry), r2)));
    T[4] = __fadd_rn(T[4], __fmul_rn(__fmul_rn(m3, ry), rz));
    T[5] = __fadd_rn(T[5], __fmul_rn(m, __fsub_rn(__fmul_rn(__fmul_rn(3.f, rz), rz), r2)));
}
__device__ __forceinline__ void load_quad32(float *T, float4 a, float4 b) {
    T[0] = a.x; T[1] = a.y; T[2] = a.z; T[3] = a.w; T[4] = b.x; T[5] = b.y;
}
// x - c in FP32 from the hi/lo FP32 splits of both (integer-unit conversions, no FP64 instruction):
// the hi parts of nearby values cancel exactly, so the offset keeps ~2^-24 of its own size.
__device__ __forceinline__ float off32(double x, float chi, float clo) {
    float xhi, xlo;
    d2f_split(x, xhi, xlo);
    return __fadd_rn(__fsub_rn(xhi, chi), __fsub_rn(xlo, clo));
}
__device__ __forceinline__ void store_quad32(float4 *q32, int64_t j, const float *Q) {
    q32[2 * j] = make_float4(Q[0], Q[1], Q[2], Q[3]);
    q32[2 * j + 1] = make_float4(Q[4], Q[5], 0.f, 0.f);
}

// Tests of FP64 values on the integer units (GB300 issues one FP64 warp instruction every ~76 cycles
// per SM sub-partition, comparisons included). nonzero64(x) is x != 0.0 for any x. fkey maps a
// non-NaN double to a signed integer of the same order, -0.0 and +0.0 to the same key, so
// fkey(b) > fkey(a) decides b > a exactly as the FP64 comparison does (pytreegrav's max keeps a on a
// tie); the inputs are checked finite before a build.
__device__ __forceinline__ bool nonzero64(double x) { return (__double_as_longlong(x) << 1) != 0; }
__device__ __forceinline__ long long fkey(double x) {
    const long long b = __double_as_longlong(x);
    return b < 0 ? -(b & 0x7fffffffffffffffll) : b;
}

// CG: read the children through L2 (ld.cg), for kernels in which another SM may have finished them.
template <bool CG>
__device__ __forceinline__ double ldm(const double *p) {
    if (CG) return __ldcg(p);
    return *p;
}
template <bool CG>
__device__ __forceinline__ float4 ldm4(const float4 *p) {
    if (CG) return __ldcg(p);
    return *p;
}

// One node's moments from its (finished) children, RollupMoments (octree.py:199-231) restricted to
// this node in FP64, plus the FP32 quadrupole. kids: the child list of k_kids (summation order as in
// the reference: particle children in chain (Morton) order, then node children in reverse chain order,
// zero-mass nodes skipped). Every child takes the same instructions: a particle adds (m, m x,
// softening) and a node (m, its mass-weighted coordinate sum, which 1.0 times the sum gives exactly,
// softening); a zero-mass node adds -0.0, the exact identity of a sum, and leaves the softening
// maximum alone, which is the reference's skipping it. A warp's lanes thus part only on the
// quadrupole's node-child term, and a warp of nodes with equal child counts (see k_moments_sorted)
// runs with every lane busy. The zero tests and the softening maximum run on the integer units.
template <bool CG>
__device__ __forceinline__ void node_moments_kids(const MomentArgs &a, int64_t j, const int32_t *kids, int n) {
    const int4 k0 = *reinterpret_cast<const int4 *>(kids + 8 * j);
    const int4 k1 = *reinterpret_cast<const int4 *>(kids + 8 * j + 4);
    const int32_t ch[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
    const int64_t N = a.ntot;
    double m = 0.0, ax = 0.0, ay = 0.0, az = 0.0, h = 0.0;
    long long hk = 0;  // fkey(h)
#pragma unroll
    for (int q = 0; q < 8; q++) {
        if (q < n) {
            const int32_t c = ch[q];
            const bool part = c >= 0;
            const int64_t g = part ? (int64_t)c : N + (int64_t)(~c);
            const double mc = ldm<CG>(a.mass + g);
            const double *src = part ? a.coord + 3 * g : a.acc + 3 * (int64_t)(~c);
            const bool use = part || nonzero64(mc);
            const double hc = ldm<CG>(a.soft + g);
            const double s0 = ldm<CG>(src), s1 = ldm<CG>(src + 1), s2 = ldm<CG>(src + 2);
            m = dadd(m, use ? mc : -0.0);
            // a particle adds m x; a node child its coordinate sums (1.0 times them, exactly)
            ax = dadd(ax, use ? (part ? dmul(mc, s0) : s0) : -0.0);
            ay = dadd(ay, use ? (part ? dmul(mc, s1) : s1) : -0.0);
            az = dadd(az, use ? (part ? dmul(mc, s2) : s2) : -0.0);
            const long long ck = fkey(hc);
            if (use && ck > hk) {  // pymax(h, hc)
                h = hc;
                hk = ck;
            }
        }
    }
    const int64_t f = N + j;
    a.mass[f] = m;
    a.soft[f] = h;
    a.acc[3 * j] = ax;
    a.acc[3 * j + 1] = ay;
    a.acc[3 * j + 2] = az;
    double com[3] = {ldm<CG>(a.coord + 3 * f), ldm<CG>(a.coord + 3 * f + 1), ldm<CG>(a.coord + 3 * f + 2)};
    if (nonzero64(m)) {
        double inv = __drcp_rn(m);  // 1 / m correctly rounded: the same value as 1.0 / m
        double accs[3] = {ax, ay, az};
        double d2 = 0.0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            double cm = dmul(accs[k], inv);
            double dx = dsub(cm, com[k]);
            d2 = dadd(d2, dmul(dx, dx));
            com[k] = cm;
            a.coord[3 * f + k] = cm;
        }
        a.delta[f] = __dsqrt_rn(d2);
    }
    if (a.quad32) {
        float Q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float ch_[3], cl_[3];
#pragma unroll
        for (int k = 0; k < 3; k++) d2f_split(com[k], ch_[k], cl_[k]);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if (q < n) {
                const int32_t c = ch[q];
                const bool part = c >= 0;
                const int64_t g = part ? (int64_t)c : N + (int64_t)(~c);
                const double mc = ldm<CG>(a.mass + g);
                if (part || nonzero64(mc)) {
                    float T[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                    if (!part) load_quad32(T, ldm4<CG>(a.quad32 + 2 * (int64_t)(~c)), ldm4<CG>(a.quad32 + 2 * (int64_t)(~c) + 1));
                    quad32_term(T, d2f(mc), off32(ldm<CG>(a.coord + 3 * g), ch_[0], cl_[0]),
                                off32(ldm<CG>(a.coord + 3 * g + 1), ch_[1], cl_[1]),
                                off32(ldm<CG>(a.coord + 3 * g + 2), ch_[2], cl_[2]));
#pragma unroll
                    for (int e = 0; e < 6; e++) Q[e] = __fadd_rn(Q[e], T[e]);
                }
            }
        }
        store_quad32(a.quad32, j, Q);
    }
}

// Large levels (FP64-throughput-bound): one thread per node, the block's nodes first ordered by
// child count (a counting sort in shared memory, most children first) so that a warp's lanes run
// the same number of child steps. Which thread takes which node does not change any result.
// MOM_BLOCK: 64, 128 or 256 threads.
template <int MOM_BLOCK>
__global__ void __launch_bounds__(MOM_BLOCK) k_moments_sorted(MomentArgs a, const int32_t *list, int count,
                                                              const int32_t *kids, const int8_t *nk) {
    __shared__ int bin[9];
    __shared__ int order[MOM_BLOCK];
    const int t = threadIdx.x;
    const int i = blockIdx.x * MOM_BLOCK + t;
    const int j0 = i < count ? list[i] : -1;
    int k0 = j0 >= 0 ? (int)nk[j0] : 0;
    k0 = k0 < 0 ? 0 : (k0 > 8 ? 8 : k0);
    if (t < 9) bin[t] = 0;
    __syncthreads();
    const int r = atomicAdd(&bin[k0], 1);
    __syncthreads();
    if (t == 0) {
        int run = 0;
        for (int b = 8; b >= 0; b--) {
            const int c = bin[b];
            bin[b] = run;
            run += c;
        }
    }
    __syncthreads();
    order[bin[k0] + r] = j0;
    __syncthreads();
    const int j = order[t];
    if (j < 0) return;
    node_moments_kids<false>(a, j, kids, nk[j]);
}

// Small levels. GB300 runs FP64 on one unit per SM sub-partition at about 76 cycles per warp
// instruction, with any number of lanes active, so a level whose nodes fill fewer warps than there
// are sub-partitions is bound by the length of one warp's FP64 instruction stream, not by lanes.
// Here 32 nodes share a block of eight warps (lane = node) and the stream is cut into stages that
// run side by side: the children's terms (one warp per child slot), the five mass-pass sums (one
// warp each), the centre of mass and Delta, and the children's FP32 quadrupole terms (one warp per
// child slot). Every FP64 sum takes its terms in node_moments_kids's order with the same
// operations, so the results are identical.
constexpr int WIDE_NODES = 32, WIDE_WARPS = 8, WIDE_THREADS = WIDE_NODES * WIDE_WARPS;
constexpr int WIDE_MAX_LEVEL = 12288;  // levels up to this many nodes use k_moments_wide

__global__ void __launch_bounds__(WIDE_THREADS) k_moments_wide(MomentArgs a, const int32_t *list, int count,
                                                              const int32_t *kids, const int8_t *nk) {
    __shared__ double s_m[8][WIDE_NODES], s_t[3][8][WIDE_NODES], s_h[8][WIDE_NODES];  // child terms
    __shared__ double s_sum[5][WIDE_NODES], s_com[3][WIDE_NODES];
    __shared__ float s_q[6][8][WIDE_NODES];  // the children's FP32 quadrupole terms
    __shared__ int8_t s_use[8][WIDE_NODES];  // child enters the sums (a particle, or a node of nonzero mass)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int idx = blockIdx.x * WIDE_NODES + lane;
    const int64_t N = a.ntot;
    // Global reads in three dependent rounds: the node; its child count, child w and (warp 0) its
    // cell centre; then everything of child w the later stages need (its mass, softening,
    // coordinates, and for a node child its coordinate sums and FP32 quadrupole), kept in registers,
    // since warp w handles child w in every stage.
    const int64_t j = idx < count ? (int64_t)list[idx] : -1;
    int n = 0;
    int32_t c = 0;
    double com[3] = {0.0, 0.0, 0.0};
    if (j >= 0) {
        n = (int)nk[j];
        c = kids[8 * j + w];  // slots past n are not used
        if (w == 0) {
#pragma unroll
            for (int k = 0; k < 3; k++) com[k] = a.coord[3 * (N + j) + k];
        }
    }
    const bool mine = w < n;  // this thread has a child
    const bool part = c >= 0;
    const int64_t g = part ? (int64_t)c : N + (int64_t)(~c);
    double mc = 0.0, hc = 0.0, cx[3] = {0.0, 0.0, 0.0}, sx[3];
    float4 qa = make_float4(0.f, 0.f, 0.f, 0.f), qb = qa;
    if (mine) {
        mc = a.mass[g];
        hc = a.soft[g];
#pragma unroll
        for (int k = 0; k < 3; k++) cx[k] = a.coord[3 * g + k];
        if (!part) {
#pragma unroll
            for (int k = 0; k < 3; k++) sx[k] = a.acc[3 * (int64_t)(~c) + k];
            if (a.quad32) {
                qa = a.quad32[2 * (int64_t)(~c)];
                qb = a.quad32[2 * (int64_t)(~c) + 1];
            }
        }
    }
    // stage 1: warp q, child q of every node: the mass-pass terms (use ? term : -0.0); a particle
    // adds m x, a node child its coordinate sums (times 1.0 in node_moments_kids, which is exact)
    const bool use = mine && (part || nonzero64(mc));
    if (mine) {
        s_m[w][lane] = use ? mc : -0.0;
#pragma unroll
        for (int k = 0; k < 3; k++) s_t[k][w][lane] = use ? (part ? dmul(mc, cx[k]) : sx[k]) : -0.0;
        s_h[w][lane] = hc;
        s_use[w][lane] = use ? 1 : 0;
    }
    __syncthreads();
    // stage 2: the five sums, child order (the softening maximum on the integer units)
    if (w < 5 && j >= 0) {
        double v = 0.0;
        long long vk = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if (q < n) {
                if (w == 0) v = dadd(v, s_m[q][lane]);
                else if (w < 4) v = dadd(v, s_t[w - 1][q][lane]);
                else if (s_use[q][lane]) {
                    const double hq = s_h[q][lane];
                    const long long kq = fkey(hq);
                    if (kq > vk) {  // pymax(v, hq)
                        v = hq;
                        vk = kq;
                    }
                }
            }
        }
        s_sum[w][lane] = v;
    }
    __syncthreads();
    // stage 3: mass, softening, centre of mass and Delta
    if (w == 0 && j >= 0) {
        const int64_t f = N + j;
        const double m = s_sum[0][lane];
        const double acc[3] = {s_sum[1][lane], s_sum[2][lane], s_sum[3][lane]};
        a.mass[f] = m;
        a.soft[f] = s_sum[4][lane];
        a.acc[3 * j] = acc[0];
        a.acc[3 * j + 1] = acc[1];
        a.acc[3 * j + 2] = acc[2];
        if (nonzero64(m)) {
            const double inv = __drcp_rn(m);  // 1 / m correctly rounded: the same value as 1.0 / m
            double d2 = 0.0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const double cm = dmul(acc[k], inv);
                const double dx = dsub(cm, com[k]);
                d2 = dadd(d2, dmul(dx, dx));
                com[k] = cm;
                a.coord[3 * f + k] = cm;
            }
            a.delta[f] = __dsqrt_rn(d2);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) s_com[k][lane] = com[k];
    }
    __syncthreads();
    if (!a.quad32) return;  // (uniform over the block)
    // stage 4: warp q, child q: its FP32 quadrupole term
    if (use) {
        float T[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (!part) load_quad32(T, qa, qb);
        float ch_[3], cl_[3];
#pragma unroll
        for (int k = 0; k < 3; k++) d2f_split(s_com[k][lane], ch_[k], cl_[k]);
        quad32_term(T, d2f(mc), off32(cx[0], ch_[0], cl_[0]), off32(cx[1], ch_[1], cl_[1]), off32(cx[2], ch_[2], cl_[2]));
#pragma unroll
        for (int e = 0; e < 6; e++) s_q[e][w][lane] = T[e];
    }
    __syncthreads();
    // stage 5: warp 0 adds the children's terms in child order
    if (w == 0 && j >= 0) {
        float Q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < 8; q++)
            if (q < n && s_use[q][lane])
#pragma unroll
                for (int e = 0; e < 6; e++) Q[e] = __fadd_rn(Q[e], s_q[e][q][lane]);
        store_quad32(a.quad32, j, Q);
    }
}

// Nodes at depth >= DEPTH_CAP (chains of re-keyed cells and coincident-point buckets, whose depth
// is unbounded): every such node without node children starts a thread; the last child to finish
// a parent carries on with the parent, up to the first ancestor above DEPTH_CAP, which the level
// pass then handles. Children are read through L2.
__global__ void k_moments_deep(MomentArgs a, const int32_t *list, int count, const int8_t *fdepth,
                               const int32_t *kids, const int8_t *nk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int64_t j = list[i];
    if (a.nchild[j] != 0) return;
    for (int64_t guard = 0; guard < a.mtot + 1; guard++) {
        node_moments_kids<true>(a, j, kids, nk[j]);
        __threadfence();
        int64_t p = a.parent[a.ntot + j];
        if (p < a.ntot || p >= a.ntot + a.mtot) return;
        int64_t pj = p - a.ntot;
        if (fdepth[pj] < DEPTH_CAP) return;
        int prev = atomicAdd(&a.arrived[pj], 1);
        if (prev != a.nchild[pj] - 1) return;
        __threadfence();
        j = pj;
    }
}

// The quadrupole pass: node j's FP64 quadrupole (RollupQuadrupoles, octree.py:234-292) from its
// children's final masses, centres of mass and FP64 quadrupoles, with the order and operations the
// moment pass used to take (shift_quad per child in k_kids's order, a node child's quadrupole added
// first), so the values are pytreegrav's bit for bit. The node's centre of mass is its final
// coordinate (its cell centre when massless, as in the moment pass).
template <bool CG>
__device__ __forceinline__ void node_quad64(const MomentArgs &a, int64_t j, const int32_t *kids, int n) {
    const int4 k0 = *reinterpret_cast<const int4 *>(kids + 8 * j);
    const int4 k1 = *reinterpret_cast<const int4 *>(kids + 8 * j + 4);
    const int32_t ch[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
    const int64_t N = a.ntot, f = N + j;
    const double com[3] = {ldm<CG>(a.coord + 3 * f), ldm<CG>(a.coord + 3 * f + 1), ldm<CG>(a.coord + 3 * f + 2)};
    double Q[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        if (q < n) {
            const int32_t c = ch[q];
            const bool part = c >= 0;
            const int64_t g = part ? (int64_t)c : N + (int64_t)(~c);
            const double mc = ldm<CG>(a.mass + g);
            if (part || mc != 0.0) {
                if (!part) {
#pragma unroll
                    for (int k = 0; k < 9; k++) Q[k] = dadd(Q[k], ldm<CG>(a.quad + 9 * (int64_t)(~c) + k));
                }
                shift_quad(Q, mc, dsub(ldm<CG>(a.coord + 3 * g), com[0]), dsub(ldm<CG>(a.coord + 3 * g + 1), com[1]),
                           dsub(ldm<CG>(a.coord + 3 * g + 2), com[2]));
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 9; k++) a.quad[9 * j + k] = Q[k];
}

__global__ void k_quad64_level(MomentArgs a, const int32_t *list, int count, const int32_t *kids, const int8_t *nk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int64_t j = list[i];
    node_quad64<false>(a, j, kids, nk[j]);
}

// The quadrupole pass below DEPTH_CAP, climbing as k_moments_deep does.
__global__ void k_quad64_deep(MomentArgs a, const int32_t *list, int count, const int8_t *fdepth, const int32_t *kids,
                              const int8_t *nk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int64_t j = list[i];
    if (a.nchild[j] != 0) return;
    for (int64_t guard = 0; guard < a.mtot + 1; guard++) {
        node_quad64<true>(a, j, kids, nk[j]);
        __threadfence();
        int64_t p = a.parent[a.ntot + j];
        if (p < a.ntot || p >= a.ntot + a.mtot) return;
        int64_t pj = p - a.ntot;
        if (fdepth[pj] < DEPTH_CAP) return;
        int prev = atomicAdd(&a.arrived[pj], 1);
        if (prev != a.nchild[pj] - 1) return;
        __threadfence();
        j = pj;
    }
}

// Section offsets of the level lists from the depth histogram; cursors reset.
__global__ void k_level_offsets(const BuildSummary *sum, int *lvl_off, int *lvl_cursor) {
    if (threadIdx.x != 0) return;
    int run = 0;
    for (int d = 0; d <= DEPTH_CAP; d++) {
        lvl_off[d] = run;
        lvl_cursor[d] = 0;
        run += sum->depth_hist[d];
    }
}

// compute_moments=False: node masses/softenings hold only the particles folded in by the split.
__global__ void k_fold_only(MomentArgs a) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.mtot) return;
    int64_t f = a.ntot + j;
    const int64_t stop = a.next[f];
    double m = 0.0, h = 0.0;
    int steps = 0;
    for (int64_t c = a.first[f]; c != stop && c >= 0 && steps < 9; c = a.next[c], steps++) {
        if (c < a.ntot) {
            m = dadd(m, a.mass[c]);
            h = pymax(h, a.soft[c]);
        }
    }
    a.mass[f] = m;
    a.soft[f] = h;
}

// ---------------------------------------------------------------------------------------------
// A non-blocking stream per host thread (and device) for build work that can run beside the
// build's own stream, with its fork and join events; created once.
struct BuildSide {
    int dev = -1;
    unsigned long long ctx = 0;  // id of the CUDA context the stream and events belong to
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
static tg_status build_side(BuildSide *&out) {
    static thread_local BuildSide side;
    int dev = 0;
    TG_CUDA(cudaGetDevice(&dev));
    // another device (this thread's old one is kept alive), or a new context after a device reset
    // (the old handles died with it)
    const unsigned long long ctx = tg::current_cuda_context_id();
    if (side.s && (side.dev != dev || (ctx && side.ctx && side.ctx != ctx))) side = BuildSide();
    if (!side.s) {
        TG_CUDA(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
        TG_CUDA(cudaEventCreateWithFlags(&side.fork, cudaEventDisableTiming));
        TG_CUDA(cudaEventCreateWithFlags(&side.join, cudaEventDisableTiming));
        side.dev = dev;
        side.ctx = tg::current_cuda_context_id();
    }
    if (!side.ctx) side.ctx = ctx;
    out = &side;
    return TG_OK;
}

template <typename T>
static tg_status dalloc(T **p, int64_t n, cudaStream_t s) {
    *p = nullptr;
    if (n <= 0) n = 1;
    TG_CUDA(tg::dev_malloc((void **)p, sizeof(T) * n, s));
    return TG_OK;
}
template <typename T>
static void dfree(T *&p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
}

static tg_status segs_alloc(Segs &g, int n, cudaStream_t s) {
    g.n = n;
    TG_TRY(dalloc(&g.lo, n, s));
    TG_TRY(dalloc(&g.hi, n, s));
    TG_TRY(dalloc(&g.root, n, s));
    TG_TRY(dalloc(&g.center, 3 * n, s));
    TG_TRY(dalloc(&g.size, n, s));
    TG_TRY(dalloc(&g.depth0, n, s));
    TG_TRY(dalloc(&g.next_ref, n, s));
    TG_TRY(dalloc(&g.sys, n, s));
    TG_TRY(dalloc(&g.eoff, n + 1, s));
    return TG_OK;
}
static void segs_free(Segs &g, cudaStream_t s) {
    dfree(g.lo, s); dfree(g.hi, s); dfree(g.root, s); dfree(g.center, s); dfree(g.size, s);
    dfree(g.depth0, s); dfree(g.next_ref, s); dfree(g.sys, s); dfree(g.eoff, s);
    g.n = 0;
}

template <typename T>
static tg_status grow_copy(T **p, int64_t old_n, int64_t new_n, int width, cudaStream_t s) {
    T *q = nullptr;
    TG_TRY(dalloc(&q, new_n * width, s));
    if (*p && old_n > 0) TG_CUDA(cudaMemcpyAsync(q, *p, sizeof(T) * old_n * width, cudaMemcpyDeviceToDevice, s));
    dfree(*p, s);
    *p = q;
    return TG_OK;
}

static tg_status nodes_reserve(Nodes &nd, int64_t need, cudaStream_t s) {
    if (need <= nd.cap) return TG_OK;
    int64_t nc = std::max<int64_t>(need, nd.cap + nd.cap / 2 + 64);
    TG_TRY(grow_copy(&nd.lo, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.hi, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.parent, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.first, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.next, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.aparent, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.rank, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.digit, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.depth, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.sys, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.seg, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.level, nd.count, nc, 1, s));
    TG_TRY(grow_copy(&nd.center, nd.count, nc, 3, s));
    TG_TRY(grow_copy(&nd.size, nd.count, nc, 1, s));
    nd.cap = nc;
    return TG_OK;
}
static void nodes_free(Nodes &nd, cudaStream_t s) {
    dfree(nd.lo, s); dfree(nd.hi, s); dfree(nd.parent, s); dfree(nd.first, s); dfree(nd.next, s);
    dfree(nd.aparent, s); dfree(nd.rank, s); dfree(nd.digit, s); dfree(nd.depth, s); dfree(nd.sys, s); dfree(nd.seg, s);
    dfree(nd.level, s);
    dfree(nd.center, s); dfree(nd.size, s);
}

static RoundView view_of(const Segs &g) {
    RoundView v;
    v.seg_lo = g.lo; v.seg_hi = g.hi; v.seg_root = g.root; v.seg_next = g.next_ref; v.eoff = g.eoff;
    v.seg_center = g.center; v.seg_size = g.size; v.seg_depth0 = g.depth0; v.seg_sys = g.sys; v.nseg = g.n;
    return v;
}

static int bits_for(int64_t v) {
    int b = 0;
    while (b < 63 && ((int64_t)1 << b) <= v) b++;
    return b;
}

static int64_t reference_capacity(int64_t npart, int64_t required) {
    int64_t cap = (int64_t)(1.5 * (double)npart + 1.0);
    while (cap < required) {
        int64_t inc = (int64_t)((double)cap * 1.2 + 1.0) - cap;
        cap += inc < 1 ? 1 : inc;
    }
    return cap;
}

__global__ void k_init_root_segs(Segs g, const int64_t *sys_off, const double *center, const double *size) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.n) return;
    g.lo[s] = sys_off[s];
    g.hi[s] = sys_off[s + 1];
    g.root[s] = -1;
    g.center[3 * s] = center[3 * s];
    g.center[3 * s + 1] = center[3 * s + 1];
    g.center[3 * s + 2] = center[3 * s + 2];
    g.size[s] = size[s];
    g.depth0[s] = 0;
    g.next_ref[s] = -1;
    g.sys[s] = s;
}

#define LAUNCH(n) div_up((n), 256), 256, 0, st

// Build the whole arena. pos/m/h are device pointers (m/h may be null). m_h_ready (may be null):
// an event after which m and h may be read; the build waits for it only where it first reads them
// (the gather into Morton order), so their upload overlaps the bounding cube, keys and sort.
tg_status build_tree(tg_tree_s *T, const double *pos, const double *m, const double *h,
                     const std::vector<int64_t> &sys_off_host, int quadrupole, int compute_moments,
                     const int *nonfinite, cudaStream_t st, cudaEvent_t m_h_ready) {
    const int nsys = (int)sys_off_host.size() - 1;
    const int64_t N = sys_off_host.back();
    if (N < 1 || nsys < 1) return TG_ERR_BAD_ARG;
    if (N > 0x7fffffffLL) return TG_ERR_BAD_ARG;
    int64_t max_sys_n = 0;
    for (int s = 0; s < nsys; s++) {
        int64_t ns = sys_off_host[s + 1] - sys_off_host[s];
        if (ns < 1) return TG_ERR_BAD_ARG;
        max_sys_n = std::max(max_sys_n, ns);
    }
    NumberingBits nb{bits_for(max_sys_n), 7};
    int sysbits = nsys > 1 ? bits_for(nsys - 1) : 0;
    if (sysbits + 2 * nb.lb + nb.db > 64) return TG_ERR_BAD_ARG;

    T->ntot = N;
    T->nsys = nsys;
    T->sys_off = sys_off_host;
    T->has_quads = quadrupole;
    T->compute_moments = compute_moments;
    T->stream = st;

    int64_t *sys_off = nullptr;
    TG_TRY(dalloc(&sys_off, nsys + 1, st));
    TG_CUDA(cudaMemcpyAsync(sys_off, sys_off_host.data(), sizeof(int64_t) * (nsys + 1), cudaMemcpyHostToDevice, st));
    TG_TRY(dalloc(&T->sort_err, 1, st));  // every sort of this tree reports here
    TG_CUDA(cudaMemsetAsync(T->sort_err, 0, sizeof(int), st));

    // 1. bounding cubes
    unsigned long long *mn = nullptr, *mx = nullptr;
    double *center = nullptr, *size = nullptr;
    TG_TRY(dalloc(&mn, 3 * nsys, st));
    TG_TRY(dalloc(&mx, 3 * nsys, st));
    TG_TRY(dalloc(&center, 3 * nsys, st));
    TG_TRY(dalloc(&size, nsys, st));
    { k_bbox_init<<<LAUNCH(3 * nsys)>>>(mn, mx, nsys); tg::note_launch(); }
    { k_bbox<<<div_up(N, BB_THREADS * BB_ITEMS), BB_THREADS, 0, st>>>(pos, N, sys_off, nsys, mn, mx); tg::note_launch(); }
    { k_bbox_finish<<<LAUNCH(nsys)>>>(mn, mx, nsys, center, size); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());

    // 2. keys and stable sort (system id as the most significant digit when batched)
    uint64_t *keys = nullptr, *keys_orig = nullptr;
    uint32_t *perm = nullptr;
    TG_TRY(dalloc(&keys, N, st));
    TG_TRY(dalloc(&keys_orig, N, st));
    TG_TRY(dalloc(&perm, N, st));
    { k_keys<<<LAUNCH(N)>>>(pos, N, sys_off, nsys, center, size, keys, keys_orig, perm); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_TRY(radix_sort_pairs(keys, perm, N, 63, st, T->sort_err));
    if (nsys > 1) {
        { k_sys_of<<<LAUNCH(N)>>>(perm, N, sys_off, nsys, keys); tg::note_launch(); }
        TG_TRY(radix_sort_pairs(keys, perm, N, sysbits, st, T->sort_err));
    }

    // 3. arena element arrays; particles gathered into Morton order
    const int64_t cap0 = N + N / 2 + 16;  // node slots, grown if needed
    TG_TRY(dalloc(&T->walk_idx, N, st));
    double *pc = nullptr, *pm = nullptr, *ps = nullptr;
    TG_TRY(dalloc(&pc, 3 * N, st));
    TG_TRY(dalloc(&pm, N, st));
    TG_TRY(dalloc(&ps, N, st));
    uint64_t *keys_sorted = keys;  // reuse
    if (m_h_ready) TG_CUDA(cudaStreamWaitEvent(st, m_h_ready, 0));
    { k_gather<<<LAUNCH(N)>>>(perm, N, pos, m, h, keys_orig, pc, pm, ps, keys_sorted, T->walk_idx, T->sort_err); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    dfree(keys_orig, st);

    // 4. split rounds
    Nodes nd;
    TG_TRY(nodes_reserve(nd, cap0, st));
    int64_t *p_parent = nullptr, *p_next = nullptr;
    TG_TRY(dalloc(&p_parent, N, st));
    TG_TRY(dalloc(&p_next, N, st));
    Segs sg;
    TG_TRY(segs_alloc(sg, nsys, st));
    { k_init_root_segs<<<LAUNCH(nsys)>>>(sg, sys_off, center, size); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    int64_t *exh = nullptr;
    int n_exh = 0;
    int64_t *root_first = nullptr;
    int has_coincident = 0;
    // What the host reads back after a round; final (covering every slot) once a round leaves no
    // key-exhausted run. The common case, one round and no buckets, synchronises here once.
    BuildSummary *sum = nullptr;
    TG_TRY(dalloc(&sum, 1, st));
    BuildSummary hs;
    memset(&hs, 0, sizeof(hs));
    bool summary_final = false;
    BuildSide *side = nullptr;  // k_node_centers of the last round runs there when set
    bool centers_forked = false;
    // Non-finite input is reported once the build has run to its end and freed its memory: every
    // kernel stays in bounds on such input (keys of NaN quantize to 0, every link is checked).
    bool nonfinite_seen = false;

    for (int round = 0; round <= MORTON_MAX_ROUNDS; round++) {
        // element offsets of the segments; round 0's segments are the systems
        int64_t E = N;
        if (round == 0) {
            TG_CUDA(cudaMemcpyAsync(sg.eoff, sys_off, sizeof(int64_t) * (nsys + 1), cudaMemcpyDeviceToDevice, st));
        } else {
            int64_t *sizes = nullptr;
            TG_TRY(dalloc(&sizes, sg.n, st));
            { k_seg_sizes<<<LAUNCH(sg.n)>>>(sg.lo, sg.hi, sg.n, sizes); tg::note_launch(); }
            TG_TRY(exclusive_scan_i64(sizes, sg.eoff, sg.n, sg.eoff + sg.n, st));
            dfree(sizes, st);
            TG_CUDA(cudaMemcpyAsync(&E, sg.eoff + sg.n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
            TG_CUDA(cudaStreamSynchronize(st));
        }
        RoundView v = view_of(sg);

        if (round > 0) {
            // re-key the exhausted runs relative to their cells and sort each run stably
            uint64_t *rk = nullptr, *rk_elem = nullptr;
            uint32_t *rv = nullptr;
            TG_TRY(dalloc(&rk, E, st));
            TG_TRY(dalloc(&rk_elem, E, st));
            TG_TRY(dalloc(&rv, E, st));
            { k_rekey_keys<<<LAUNCH(E)>>>(v, E, pc, rk, rv); tg::note_launch(); }
            TG_CUDA(cudaMemcpyAsync(rk_elem, rk, sizeof(uint64_t) * E, cudaMemcpyDeviceToDevice, st));
            TG_TRY(radix_sort_pairs(rk, rv, E, 63, st, T->sort_err));
            if (sg.n > 1) {
                { k_rekey_segkeys<<<LAUNCH(E)>>>(v, rv, E, rk); tg::note_launch(); }
                TG_TRY(radix_sort_pairs(rk, rv, E, bits_for(sg.n - 1), st, T->sort_err));
            }
            double *tc = nullptr, *tm = nullptr, *ts = nullptr;
            int64_t *tw = nullptr;
            uint64_t *tk = nullptr;
            TG_TRY(dalloc(&tc, 3 * E, st));
            TG_TRY(dalloc(&tm, E, st));
            TG_TRY(dalloc(&ts, E, st));
            TG_TRY(dalloc(&tw, E, st));
            TG_TRY(dalloc(&tk, E, st));
            { k_rekey_gather<<<LAUNCH(E)>>>(v, E, rv, pc, pm, ps, T->walk_idx, rk_elem, tc, tm, ts, tw, tk, T->sort_err); tg::note_launch(); }
            { k_rekey_scatter<<<LAUNCH(E)>>>(v, E, tc, tm, ts, tw, tk, pc, pm, ps, T->walk_idx, keys_sorted); tg::note_launch(); }
            TG_CUDA(cudaGetLastError());
            dfree(rk, st); dfree(rk_elem, st); dfree(rv, st);
            dfree(tc, st); dfree(tm, st); dfree(ts, st); dfree(tw, st); dfree(tk, st);
        }

        int8_t *L = nullptr;
        int64_t *cnt = nullptr, *nstart = nullptr;
        TG_TRY(dalloc(&L, E, st));
        TG_TRY(dalloc(&cnt, E, st));
        TG_TRY(dalloc(&nstart, E, st));
        TG_CUDA(cudaMemsetAsync(sum, 0, sizeof(BuildSummary), st));
        { k_levels<<<LAUNCH(E)>>>(v, E, keys_sorted, L); tg::note_launch(); }
        { k_counts<<<LAUNCH(E)>>>(v, E, L, cnt); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
        TG_TRY(exclusive_scan_i64(cnt, nstart, E, (int64_t *)&sum->nodes, st));
        const int64_t slot_base = nd.count;
        dfree(exh, st);
        dfree(root_first, st);
        int64_t exh_cap = std::max<int64_t>(nd.cap - slot_base, 1);
        TG_TRY(dalloc(&exh, exh_cap, st));
        TG_TRY(dalloc(&root_first, sg.n, st));
        // The round's nodes, particle links and the summary, read back with one copy. Slots that
        // do not fit are skipped by k_nodes; the host then grows the arrays and runs it again.
        auto run_round = [&]() -> tg_status {
            { k_nodes<<<LAUNCH(E)>>>(v, E, L, nstart, cnt, slot_base, keys_sorted, nd, exh, &sum->n_exh, exh_cap,
                                     root_first); tg::note_launch(); }
            { k_particles<<<LAUNCH(E)>>>(v, E, L, nstart, slot_base, keys_sorted, p_parent, p_next); tg::note_launch(); }
            if (round > 0) { k_set_root_first<<<LAUNCH(sg.n)>>>(sg.root, root_first, sg.n, nd.first); tg::note_launch(); }
            { k_summarize_slots<<<LAUNCH(std::max<int64_t>(nd.cap, N))>>>(nd, slot_base, &sum->nodes, p_parent, p_next,
                                                                       N, sum); tg::note_launch(); }
            TG_CUDA(cudaGetLastError());
            if (nonfinite) TG_CUDA(cudaMemcpyAsync(&sum->nonfinite, nonfinite, sizeof(int), cudaMemcpyDeviceToDevice, st));
            TG_CUDA(cudaMemcpyAsync(&hs, sum, sizeof(BuildSummary), cudaMemcpyDeviceToHost, st));
            TG_CUDA(cudaStreamSynchronize(st));
            if (hs.nonfinite) nonfinite_seen = true;
            return TG_OK;
        };
        TG_TRY(run_round());
        const int64_t Mr = (int64_t)hs.nodes;
        if (slot_base + Mr > nd.cap) {
            TG_TRY(nodes_reserve(nd, slot_base + Mr, st));
            dfree(exh, st);
            exh_cap = std::max<int64_t>(Mr, 1);
            TG_TRY(dalloc(&exh, exh_cap, st));
            TG_CUDA(cudaMemsetAsync(&sum->n_exh, 0, sizeof(unsigned long long), st));
            TG_CUDA(cudaMemsetAsync(&sum->bad, 0, sizeof(int) * (2 + DEPTH_CAP + 1), st));
            TG_TRY(run_round());
        }
        nd.count = slot_base + Mr;
        if (Mr > 0) {
            // the last round's centres (nothing re-keys or grows the slots after it) run beside the
            // node numbering, which does not read them; k_write_nodes joins them
            cudaStream_t cs = st;
            if (hs.n_exh == 0) {
                TG_TRY(build_side(side));
                TG_CUDA(cudaEventRecord(side->fork, st));
                TG_CUDA(cudaStreamWaitEvent(side->s, side->fork, 0));
                cs = side->s;
            }
            { k_node_centers<<<div_up(Mr, CENTER_BLOCK), CENTER_BLOCK, 0, cs>>>(v, nd, slot_base, Mr, keys_sorted); tg::note_launch(); }
            if (cs != st) {
                TG_CUDA(cudaEventRecord(side->join, cs));
                centers_forked = true;
            }
        }
        n_exh = (int)hs.n_exh;
        dfree(L, st); dfree(cnt, st); dfree(nstart, st);
        if (n_exh == 0) {
            summary_final = true;
            break;
        }
        if (round < MORTON_MAX_ROUNDS) {
            segs_free(sg, st);
            TG_TRY(segs_alloc(sg, n_exh, st));
            { k_make_segs<<<LAUNCH(n_exh)>>>(exh, n_exh, nd, sg); tg::note_launch(); }
            TG_CUDA(cudaGetLastError());
        }
    }
    if (!centers_forked) segs_free(sg, st);  // else k_node_centers still reads them: freed after the join
    dfree(root_first, st);

    // 5. buckets for runs still exhausted after three re-keys
    int n_bucket = (n_exh > 0) ? n_exh : 0;
    if (n_bucket > 0) {
        has_coincident = 1;
        int64_t *nchain = nullptr, *choff = nullptr, *chtot = nullptr;
        TG_TRY(dalloc(&nchain, n_bucket, st));
        TG_TRY(dalloc(&choff, n_bucket, st));
        TG_TRY(dalloc(&chtot, 1, st));
        { k_bucket_counts<<<LAUNCH(n_bucket)>>>(exh, n_bucket, nd.lo, nd.hi, nchain); tg::note_launch(); }
        TG_TRY(exclusive_scan_i64(nchain, choff, n_bucket, chtot, st));
        int64_t nch = 0;
        TG_CUDA(cudaMemcpyAsync(&nch, chtot, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        TG_CUDA(cudaStreamSynchronize(st));
        int64_t slot_base = nd.count;
        TG_TRY(nodes_reserve(nd, slot_base + nch, st));
        { k_bucket<<<LAUNCH(n_bucket)>>>(exh, n_bucket, choff, slot_base, nd, p_parent, p_next); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
        nd.count = slot_base + nch;
        dfree(nchain, st); dfree(choff, st); dfree(chtot, st);
    }
    T->has_coincident = has_coincident;

    // 6. reference numbering
    if (!summary_final) {  // buckets were made after the last summary: validate every slot again
        TG_CUDA(cudaMemsetAsync(sum, 0, sizeof(BuildSummary), st));
        { k_summarize_slots<<<LAUNCH(std::max<int64_t>(nd.count, N))>>>(nd, nd.count, nullptr, p_parent, p_next, N,
                                                                      sum); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
        TG_CUDA(cudaMemcpyAsync(&hs, sum, sizeof(BuildSummary), cudaMemcpyDeviceToHost, st));
        TG_CUDA(cudaStreamSynchronize(st));
    }
    if (hs.bad) {
        if (nonfinite_seen) return TG_ERR_NONFINITE;
        set_last_error_msg("internal error: octree build produced an invalid node reference");
        return TG_ERR_CUDA;
    }
    const int64_t M = nd.count;
    T->mtot = M;
    uint64_t *nkeys = nullptr;
    uint32_t *nvals = nullptr;
    int64_t *root_slot = nullptr, *final_of_slot = nullptr, *sys_node_off = nullptr;
    int *nonroot = nullptr;
    TG_TRY(dalloc(&nkeys, M, st));
    TG_TRY(dalloc(&nvals, M, st));
    TG_TRY(dalloc(&root_slot, nsys, st));
    TG_TRY(dalloc(&final_of_slot, M, st));
    TG_TRY(dalloc(&sys_node_off, nsys + 1, st));
    TG_TRY(dalloc(&nonroot, 1, st));
    TG_CUDA(cudaMemsetAsync(nonroot, 0, sizeof(int), st));
    const int compact = n_bucket == 0;
    const int key_bits = sysbits + nb.lb + nb.db + (compact ? 3 : nb.lb);
    const int sort_bits = key_bits < 64 ? key_bits + 1 : 64;
    const uint64_t root_key = key_bits < 64 ? (1ull << key_bits) : ~0ull;
    { k_number_keys<<<LAUNCH(M)>>>(nd, M, sys_off, nb, root_key, compact, nkeys, nvals, root_slot, nonroot); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_TRY(radix_sort_pairs(nkeys, nvals, M, sort_bits, st, T->sort_err));
    // per-system node offsets (roots first within each system's block), on the device; the host
    // copy is read with the final synchronisation
    if (nsys == 1) {
        { k_single_sys_node_off<<<1, 1, 0, st>>>(sys_node_off, M); tg::note_launch(); }
        T->sys_node_off = {0, M};
    } else {
        int64_t *ncnt = nullptr;
        TG_TRY(dalloc(&ncnt, nsys, st));
        TG_CUDA(cudaMemsetAsync(ncnt, 0, sizeof(int64_t) * nsys, st));
        { k_sys_node_counts<<<LAUNCH(M)>>>(nd.sys, M, ncnt); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
        TG_TRY(exclusive_scan_i64(ncnt, sys_node_off, nsys, sys_node_off + nsys, st));
        dfree(ncnt, st);
        T->sys_node_off.assign(nsys + 1, 0);
    }
    { k_final_index<<<LAUNCH(std::max<int64_t>(M, nsys))>>>(nvals, M, nd.sys, N, sys_node_off, final_of_slot, root_slot,
                                                         nsys, T->sort_err); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    // capacity (NumNodes) per system: bucket reservations, read with the final synchronisation
    unsigned long long *req = nullptr;
    if (n_bucket > 0) {
        TG_TRY(dalloc(&req, nsys, st));
        TG_CUDA(cudaMemsetAsync(req, 0, sizeof(unsigned long long) * nsys, st));
        { k_bucket_requirement<<<LAUNCH(n_bucket)>>>(exh, n_bucket, nd, sys_off, nb, nkeys, M, N, req); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
    }
    dfree(exh, st);

    // 7. final arrays; every node also goes into the list of its depth
    const int64_t NE = N + M;
    TG_TRY(dalloc(&T->coord, 3 * NE, st));
    TG_TRY(dalloc(&T->mass, NE, st));
    TG_TRY(dalloc(&T->size, NE, st));
    TG_TRY(dalloc(&T->delta, NE, st));
    TG_TRY(dalloc(&T->soft, NE, st));
    TG_TRY(dalloc(&T->first, NE, st));
    TG_TRY(dalloc(&T->next, NE, st));
    TG_TRY(dalloc(&T->parent, NE, st));
    TG_TRY(dalloc(&T->node_range, M, st));
    TG_TRY(dalloc(&T->cell_center, 3 * M, st));
    int *lvl = nullptr;  // section offsets, then cursors, of the depth lists
    int32_t *lvl_list = nullptr;
    int8_t *fdepth = nullptr;
    TG_TRY(dalloc(&lvl, 2 * (DEPTH_CAP + 1), st));
    TG_TRY(dalloc(&lvl_list, M, st));
    TG_TRY(dalloc(&fdepth, M, st));
    { k_level_offsets<<<1, 32, 0, st>>>(sum, lvl, lvl + DEPTH_CAP + 1); tg::note_launch(); }
    if (centers_forked) {
        TG_CUDA(cudaStreamWaitEvent(st, side->join, 0));
        segs_free(sg, st);
    }
    { k_write_nodes<<<LAUNCH(M)>>>(nd, M, final_of_slot, T->coord, T->size, T->mass, T->soft, T->delta, T->first,
                                 T->next, T->parent, T->node_range, T->cell_center, N, lvl, lvl + DEPTH_CAP + 1,
                                 lvl_list, fdepth); tg::note_launch(); }
    { k_write_particles<<<LAUNCH(N)>>>(N, p_parent, p_next, final_of_slot, pc, pm, ps, T->coord, T->mass, T->soft,
                                     T->first, T->next, T->parent, T->size, T->delta); tg::note_launch(); }
    dfree(pc, st); dfree(pm, st); dfree(ps, st);
    TG_CUDA(cudaMemsetAsync(&sum->bad, 0, sizeof(int), st));
    { k_validate_links<<<LAUNCH(NE)>>>(NE, T->first, T->next, T->parent, &sum->bad); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    nodes_free(nd, st);
    dfree(p_parent, st); dfree(p_next, st); dfree(nkeys, st); dfree(nvals, st); dfree(root_slot, st);
    dfree(final_of_slot, st); dfree(nonroot, st); dfree(keys, st); dfree(perm, st);

    // 8. the one closing synchronisation, ahead of the moment pass (nothing the host needs comes from
    // it): link check, per-system node offsets, bucket reservations. The moment pass is then enqueued
    // and the build returns while it runs; ev_topo marks the topology and geometry final, ev_built
    // the end of the moment pass.
    if (!T->ev_topo) {
        TG_CUDA(pool_event(&T->ev_topo, false));
        TG_CUDA(pool_event(&T->ev_built, false));
    }
    TG_CUDA(cudaEventRecord(T->ev_topo, st));
    int links_bad = 0, sort_bad = 0;
    std::vector<unsigned long long> rq(nsys, 0);
    TG_CUDA(cudaMemcpyAsync(&sort_bad, T->sort_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaMemcpyAsync(&links_bad, &sum->bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (nsys > 1)
        TG_CUDA(cudaMemcpyAsync(T->sys_node_off.data(), sys_node_off, sizeof(int64_t) * (nsys + 1),
                                cudaMemcpyDeviceToHost, st));
    if (req) TG_CUDA(cudaMemcpyAsync(rq.data(), req, sizeof(unsigned long long) * nsys, cudaMemcpyDeviceToHost, st));
    dfree(req, st); dfree(sum, st); dfree(sys_node_off, st);
    dfree(sys_off, st); dfree(mn, st); dfree(mx, st); dfree(center, st); dfree(size, st);
    TG_CUDA(cudaStreamSynchronize(st));
    if (nonfinite_seen || sort_bad || links_bad) {
        dfree(lvl, st); dfree(lvl_list, st); dfree(fdepth, st);
        if (nonfinite_seen) return TG_ERR_NONFINITE;
        if (sort_bad) {
            set_last_error_msg("radix sort: a tile's look-back did not complete within its bound");
            return TG_ERR_QUEUE_TIMEOUT;
        }
        set_last_error_msg("internal error: octree links out of range");
        return TG_ERR_CUDA;
    }
    T->sys_capacity.resize(nsys);
    for (int s = 0; s < nsys; s++) {
        int64_t np = sys_off_host[s + 1] - sys_off_host[s];
        int64_t node_hi = np + (T->sys_node_off[s + 1] - T->sys_node_off[s]);
        T->sys_capacity[s] = reference_capacity(np, std::max<int64_t>(node_hi, (int64_t)rq[s]));
    }
    // 9. moments: nodes deeper than DEPTH_CAP by climbing, then one launch per depth, deepest first
    // (the moment kernels bound every link they follow). With quadrupoles the pass sums them in FP32
    // for the FP32 walk; the FP64 quadrupoles come from ensure_quad64 when first needed, which the
    // depth lists are kept for.
    MomentArgs a;
    a.ntot = N;
    a.mtot = M;
    a.coord = T->coord; a.mass = T->mass; a.soft = T->soft; a.delta = T->delta;
    a.first = T->first; a.next = T->next; a.parent = T->parent;
    a.quad = nullptr;
    a.quad32 = nullptr;
    a.acc = nullptr;
    a.nchild = nullptr;
    a.arrived = nullptr;
    if (quadrupole) {
        TG_TRY(dalloc(&T->quad32, 2 * M, st));
        if (compute_moments) a.quad32 = T->quad32;  // every node's is written by the pass below
        else TG_CUDA(cudaMemsetAsync(T->quad32, 0, sizeof(float4) * 2 * M, st));
    }
    T->lvl_off.assign(DEPTH_CAP + 2, 0);
    for (int d = 0; d <= DEPTH_CAP; d++) T->lvl_off[d + 1] = T->lvl_off[d] + hs.depth_hist[d];
    if (compute_moments) {
        const int *off = T->lvl_off.data();
        // every node's children once, in summation order
        int32_t *kids = nullptr;
        int8_t *nk = nullptr;
        TG_TRY(dalloc(&kids, 8 * M, st));
        TG_TRY(dalloc(&nk, M, st));
        { k_kids<<<LAUNCH(M)>>>(N, M, T->first, T->next, kids, nk); tg::note_launch(); }
        TG_TRY(dalloc(&a.acc, 3 * M, st));
        const int ndeep = hs.depth_hist[DEPTH_CAP];
        if (ndeep > 0) {
            TG_TRY(dalloc(&a.nchild, M, st));
            TG_TRY(dalloc(&a.arrived, M, st));
            TG_CUDA(cudaMemsetAsync(a.nchild, 0, sizeof(int) * M, st));
            TG_CUDA(cudaMemsetAsync(a.arrived, 0, sizeof(int) * M, st));
            { k_count_node_children<<<LAUNCH(M)>>>(N, M, T->parent, a.nchild); tg::note_launch(); }
            { k_moments_deep<<<div_up(ndeep, 128), 128, 0, st>>>(a, lvl_list + off[DEPTH_CAP], ndeep, fdepth, kids, nk); tg::note_launch(); }
        }
        // one launch per depth, deepest first: k_moments_wide on the small levels (latency-bound),
        // k_moments_sorted on the large ones (FP64-throughput-bound), with the largest block that still
        // gives every SM about four blocks (the mid-size levels need the smaller ones to cover the SMs)
        const int64_t want = 4 * (int64_t)num_sms();
        for (int d = DEPTH_CAP - 1; d >= 0; d--) {
            const int c = hs.depth_hist[d];
            if (c <= 0) continue;
            const int32_t *lst = lvl_list + off[d];
            if (c <= WIDE_MAX_LEVEL)
                k_moments_wide<<<div_up(c, WIDE_NODES), WIDE_THREADS, 0, st>>>(a, lst, c, kids, nk);
            else if (div_up(c, 256) >= want)
                k_moments_sorted<256><<<div_up(c, 256), 256, 0, st>>>(a, lst, c, kids, nk);
            else if (div_up(c, 128) >= want)
                k_moments_sorted<128><<<div_up(c, 128), 128, 0, st>>>(a, lst, c, kids, nk);
            else
                k_moments_sorted<64><<<div_up(c, 64), 64, 0, st>>>(a, lst, c, kids, nk);
            tg::note_launch();
        }
        TG_CUDA(cudaGetLastError());
        dfree(kids, st); dfree(nk, st);
        dfree(a.acc, st); dfree(a.nchild, st); dfree(a.arrived, st);
    } else {
        { k_fold_only<<<LAUNCH(M)>>>(a); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
    }

    dfree(lvl, st);
    if (quadrupole && compute_moments) {  // kept for the FP64 quadrupole pass
        T->lvl_list = lvl_list;
        T->fdepth = fdepth;
    } else {
        dfree(lvl_list, st); dfree(fdepth, st);
    }
    TG_CUDA(cudaEventRecord(T->ev_built, st));
    return TG_OK;
}

// The FP64 quadrupoles of a quadrupole tree (pytreegrav's Octree.Quadrupoles, bit for bit), computed
// on `st` the first time something needs them: copy-out, the tree's info, an FP64 walk. One launch
// per depth over the depth lists the build kept, deepest first; nodes deeper than DEPTH_CAP climb.
tg_status ensure_quad64(tg_tree_s *T, cudaStream_t st) {
    if (!T->has_quads || T->quad) return TG_OK;
    tree_wait_built(T, st);
    const int64_t N = T->ntot, M = T->mtot;
    double *q = nullptr;
    TG_TRY(dalloc(&q, 9 * M, st));
    if (!T->compute_moments || !T->lvl_list) {
        TG_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * 9 * M, st));
        T->quad = q;
        return TG_OK;
    }
    MomentArgs a;
    a.ntot = N;
    a.mtot = M;
    a.coord = T->coord; a.mass = T->mass; a.soft = T->soft; a.delta = T->delta;
    a.first = T->first; a.next = T->next; a.parent = T->parent;
    a.quad = q;
    a.quad32 = nullptr;
    a.acc = nullptr;
    a.nchild = nullptr;
    a.arrived = nullptr;
    const int *off = T->lvl_off.data();
    int32_t *kids = nullptr;
    int8_t *nk = nullptr;
    TG_TRY(dalloc(&kids, 8 * M, st));
    TG_TRY(dalloc(&nk, M, st));
    { k_kids<<<LAUNCH(M)>>>(N, M, T->first, T->next, kids, nk); tg::note_launch(); }
    const int ndeep = off[DEPTH_CAP + 1] - off[DEPTH_CAP];
    if (ndeep > 0) {
        TG_TRY(dalloc(&a.nchild, M, st));
        TG_TRY(dalloc(&a.arrived, M, st));
        TG_CUDA(cudaMemsetAsync(a.nchild, 0, sizeof(int) * M, st));
        TG_CUDA(cudaMemsetAsync(a.arrived, 0, sizeof(int) * M, st));
        { k_count_node_children<<<LAUNCH(M)>>>(N, M, T->parent, a.nchild); tg::note_launch(); }
        { k_quad64_deep<<<div_up(ndeep, 128), 128, 0, st>>>(a, T->lvl_list + off[DEPTH_CAP], ndeep, T->fdepth, kids, nk); tg::note_launch(); }
    }
    for (int d = DEPTH_CAP - 1; d >= 0; d--) {
        const int c = off[d + 1] - off[d];
        if (c <= 0) continue;
        { k_quad64_level<<<div_up(c, 64), 64, 0, st>>>(a, T->lvl_list + off[d], c, kids, nk); tg::note_launch(); }
    }
    TG_CUDA(cudaGetLastError());
    dfree(kids, st); dfree(nk, st); dfree(a.nchild, st); dfree(a.arrived, st);
    dfree(T->lvl_list, st); dfree(T->fdepth, st);
    T->quad = q;
    return TG_OK;
}

// _morton_order (grouped_treewalk.py:269-275): stable order of points by their keys in their own
// bounding cube. perm receives uint32 indices.
tg_status morton_order_device(const double *pos, int64_t n, uint32_t *perm, cudaStream_t st) {
    if (n <= 0) return TG_OK;
    if (n > 0x7fffffffLL) return TG_ERR_BAD_ARG;
    const int64_t off[2] = {0, n};
    DevArray<int64_t> sys_off(st);
    DevArray<unsigned long long> mn(st), mx(st);
    DevArray<double> center(st), size(st);
    DevArray<uint64_t> keys(st);
    DevArray<int> err(st);
    TG_CUDA(sys_off.alloc(2));
    TG_CUDA(mn.alloc(3));
    TG_CUDA(mx.alloc(3));
    TG_CUDA(center.alloc(3));
    TG_CUDA(size.alloc(1));
    TG_CUDA(keys.alloc(n));
    TG_CUDA(err.alloc(1));
    TG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    TG_CUDA(cudaMemcpyAsync(sys_off.p, off, sizeof(int64_t) * 2, cudaMemcpyHostToDevice, st));
    { k_bbox_init<<<1, 32, 0, st>>>(mn.p, mx.p, 1); tg::note_launch(); }
    { k_bbox<<<div_up(n, BB_THREADS * BB_ITEMS), BB_THREADS, 0, st>>>(pos, n, sys_off.p, 1, mn.p, mx.p); tg::note_launch(); }
    { k_bbox_finish<<<1, 32, 0, st>>>(mn.p, mx.p, 1, center.p, size.p); tg::note_launch(); }
    { k_keys<<<LAUNCH(n)>>>(pos, n, sys_off.p, 1, center.p, size.p, keys.p, nullptr, perm); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    tg_status rc = radix_sort_pairs(keys.p, perm, n, 63, st, err.p);
    int bad = 0;
    if (rc == TG_OK) TG_CUDA(cudaMemcpyAsync(&bad, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    // the host array `off` must outlive its copy, also on error
    TG_CUDA(cudaStreamSynchronize(st));
    TG_TRY(rc);
    if (bad) {
        set_last_error_msg("radix sort: a tile's look-back did not complete within its bound");
        return TG_ERR_QUEUE_TIMEOUT;
    }
    return TG_OK;
}

}  // namespace tg
