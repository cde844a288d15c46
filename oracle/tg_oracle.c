/*
 * CPU oracle for the pytreegrav_gb300 hot path -- TEST INFRASTRUCTURE ONLY (see tg_oracle.h).
 *
 * Every function restates one piece of pytreegrav (paths relative to the pytreegrav project):
 *   kernels          src/pytreegrav/kernel.py:5-75
 *   bounding cube    src/pytreegrav/octree.py:539-574
 *   Morton keys      src/pytreegrav/octree.py:54-98
 *   radix argsort    src/pytreegrav/octree.py:101-132
 *   serial split     src/pytreegrav/octree.py:817-1091 (serial path; frontier disabled)
 *   RekeySlice       src/pytreegrav/octree.py:1093-1126
 *   BuildBucket      src/pytreegrav/octree.py:1128-1175
 *   RollupMoments    src/pytreegrav/octree.py:199-231
 *   RollupQuadrupoles src/pytreegrav/octree.py:234-292
 *   grouped walk     src/pytreegrav/grouped_treewalk.py:45-241
 *   acceptance       src/pytreegrav/treewalk.py:22-25
 *   brute force      src/pytreegrav/bruteforce.py:7-386
 *
 * Compiled with -O2 -fno-fast-math -ffp-contract=off so that every expression rounds exactly as the
 * Python source does when evaluated without FMA contraction.  Operand order inside every
 * expression follows the Python text (left-to-right evaluation of * and +).
 */
#include "tg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MORTON_BITS 21
#define MORTON_SCALE 2097152.0
#define MORTON_MAXQ ((int64_t)((1 << MORTON_BITS) - 1))
#define MORTON_MAX_ROUNDS 3
#define BSEARCH_MIN 512

/* Python's builtin max(a, b): returns a unless b > a. */
static inline double pymax(double a, double b) { return b > a ? b : a; }

static const double octant_offsets[8][3] = {
    {-0.25, -0.25, -0.25}, {0.25, -0.25, -0.25}, {-0.25, 0.25, -0.25}, {0.25, 0.25, -0.25},
    {-0.25, -0.25, 0.25},  {0.25, -0.25, 0.25},  {-0.25, 0.25, 0.25},  {0.25, 0.25, 0.25},
};

/* ------------------------------------------------------------------------------------------ */
/* kernel.py:5-27 */
double tgo_force_kernel(double r, double h) {
    if (r > h) return 1.0 / (r * r * r);
    double hinv = 1.0 / h;
    double q = r * hinv;
    if (q <= 0.5) return (10.666666666666666666 + q * q * (-38.4 + 32.0 * q)) * hinv * hinv * hinv;
    return (21.333333333333 - 48.0 * q + 38.4 * q * q - 10.666666666667 * q * q * q -
            0.066666666667 / (q * q * q)) *
           hinv * hinv * hinv;
}

/* kernel.py:29-52 */
double tgo_tidal_kernel(double r, double h) {
    if (r > h) {
        double r2 = r * r;
        return 3.0 / (r2 * r2 * r);
    }
    double hinv = 1.0 / h;
    double hinv2 = hinv * hinv;
    double hinv5 = hinv2 * hinv2 * hinv;
    double q = r * hinv;
    if (q <= 0.5) return (76.8 - 96.0 * q) * hinv5;
    double qinv = 1.0 / q;
    double qinv3 = qinv * qinv * qinv;
    return (48.0 * qinv - 76.8 + 32.0 * q - 0.2 * qinv3 * qinv * qinv) * hinv5;
}

/* kernel.py:54-75 */
double tgo_potential_kernel(double r, double h) {
    if (h == 0.0) return -1.0 / r;
    double hinv = 1.0 / h;
    double q = r * hinv;
    if (q <= 0.5) return (-2.8 + q * q * (5.33333333333333333 + q * q * (6.4 * q - 9.6))) * hinv;
    if (q <= 1)
        return (-3.2 + 0.066666666666666666666 / q +
                q * q * (10.666666666666666666666 + q * (-16.0 + q * (9.6 - 2.1333333333333333333333 * q)))) *
               hinv;
    return -1.0 / r;
}

/* ------------------------------------------------------------------------------------------ */
/* octree.py:539-574 */
void tgo_bounding_cube(const double *p, int64_t n, double center[3], double *size) {
    double lo0 = p[0], hi0 = p[0], lo1 = p[1], hi1 = p[1], lo2 = p[2], hi2 = p[2];
    for (int64_t i = 1; i < n; i++) {
        double x = p[3 * i], y = p[3 * i + 1], z = p[3 * i + 2];
        if (x < lo0) lo0 = x;
        else if (x > hi0) hi0 = x;
        if (y < lo1) lo1 = y;
        else if (y > hi1) hi1 = y;
        if (z < lo2) lo2 = z;
        else if (z > hi2) hi2 = z;
    }
    center[0] = 0.5 * (hi0 + lo0);
    center[1] = 0.5 * (hi1 + lo1);
    center[2] = 0.5 * (hi2 + lo2);
    double s = hi0 - lo0;
    if (hi1 - lo1 > s) s = hi1 - lo1;
    if (hi2 - lo2 > s) s = hi2 - lo2;
    *size = s;
}

/* octree.py:54-66 */
static inline int64_t spread_bits(int64_t x) {
    x &= 0x1FFFFF;
    x = (x | (x << 32)) & 0x1F00000000FFFFLL;
    x = (x | (x << 16)) & 0x1F0000FF0000FFLL;
    x = (x | (x << 8)) & 0x100F00F00F00F00FLL;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3LL;
    x = (x | (x << 2)) & 0x1249249249249249LL;
    return x;
}

/* Python int() of a float truncates toward zero; the clamp to [0, MAXQ] follows (octree.py:85-96).
 * Values >= 2^21 clamp high, values <= -1 clamp low; (-1, 0) truncates to 0. */
static inline int64_t quantize(double v) {
    if (v >= MORTON_SCALE) return MORTON_MAXQ;
    if (!(v > -1.0)) return 0;
    int64_t q = (int64_t)v;
    return q < 0 ? 0 : q;
}

/* octree.py:69-98 */
void tgo_morton_keys(const double *p, int64_t n, const double center[3], double size, int64_t *keys) {
    double inv = size > 0 ? 1.0 / size : 0.0;
    double cmin0 = center[0] - 0.5 * size;
    double cmin1 = center[1] - 0.5 * size;
    double cmin2 = center[2] - 0.5 * size;
    for (int64_t i = 0; i < n; i++) {
        int64_t qx = quantize((p[3 * i] - cmin0) * inv * MORTON_SCALE);
        int64_t qy = quantize((p[3 * i + 1] - cmin1) * inv * MORTON_SCALE);
        int64_t qz = quantize((p[3 * i + 2] - cmin2) * inv * MORTON_SCALE);
        keys[i] = spread_bits(qx) | (spread_bits(qy) << 1) | (spread_bits(qz) << 2);
    }
}

/* octree.py:101-132: stable LSD radix, 11-bit digits, keys carried alongside indices. */
void tgo_radix_argsort(const int64_t *keys, int64_t n, int64_t *perm) {
    size_t bytes = sizeof(int64_t) * (n > 0 ? n : 1);
    int64_t *ia = (int64_t *)malloc(bytes), *ib = (int64_t *)malloc(bytes);
    int64_t *ka = (int64_t *)malloc(bytes), *kb = (int64_t *)malloc(bytes);
    int64_t *count = (int64_t *)malloc(sizeof(int64_t) * 2049);
    int64_t *idx = ia, *idx_t = ib, *k_cur = ka, *k_t = kb;
    for (int64_t i = 0; i < n; i++) {
        idx[i] = i;
        k_cur[i] = keys[i];
    }
    const int bits = 11;
    const int64_t mask = (1 << bits) - 1;
    for (int shift = 0; shift < 63; shift += bits) {
        memset(count, 0, sizeof(int64_t) * 2049);
        for (int64_t i = 0; i < n; i++) count[((k_cur[i] >> shift) & mask) + 1]++;
        for (int b = 0; b < 2048; b++) count[b + 1] += count[b];
        for (int64_t i = 0; i < n; i++) {
            int64_t d = (k_cur[i] >> shift) & mask;
            int64_t pz = count[d]++;
            idx_t[pz] = idx[i];
            k_t[pz] = k_cur[i];
        }
        int64_t *s = idx; idx = idx_t; idx_t = s;
        s = k_cur; k_cur = k_t; k_t = s;
    }
    if (n > 0) memcpy(perm, idx, sizeof(int64_t) * n);
    free(ia); free(ib); free(ka); free(kb); free(count);
}

/* grouped_treewalk.py:269-275 (min/max per axis, then the same keys and sort) */
void tgo_morton_order(const double *pos, int64_t n, int64_t *perm) {
    if (n <= 0) return;
    double c[3], s;
    tgo_bounding_cube(pos, n, c, &s);
    int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * n);
    tgo_morton_keys(pos, n, c, s, keys);
    tgo_radix_argsort(keys, n, perm);
    free(keys);
}

/* ------------------------------------------------------------------------------------------ */
/* Tree storage and growth: Initialize (octree.py:1188-1206) and increase_tree_size (1280-1298). */
typedef struct {
    tgo_tree *t;
    double *acc;      /* (cap - npart, 3) */
    int64_t *parent;  /* (cap - npart,) */
    int64_t *pparent; /* (npart,) */
} build_ctx;

static void tree_alloc(tgo_tree *t, int64_t npart, int quads) {
    t->npart = npart;
    t->num_nodes = (int64_t)(1.5 * (double)npart + 1.0);
    t->has_quads = quads;
    t->has_coincident = 0;
    int64_t c = t->num_nodes;
    t->coord = (double *)calloc(3 * c, sizeof(double));
    t->mass = (double *)calloc(c, sizeof(double));
    t->size = (double *)calloc(c, sizeof(double));
    t->delta = (double *)calloc(c, sizeof(double));
    t->soft = (double *)calloc(c, sizeof(double));
    t->quad = quads ? (double *)calloc(9 * c, sizeof(double)) : NULL;
    t->first = (int64_t *)malloc(c * sizeof(int64_t));
    t->next = (int64_t *)malloc(c * sizeof(int64_t));
    for (int64_t i = 0; i < c; i++) t->first[i] = t->next[i] = -1;
    t->walk_idx = (int64_t *)malloc((npart > 0 ? npart : 1) * sizeof(int64_t));
}

static void *grow(void *p, int64_t old_n, int64_t new_n, size_t elem) {
    p = realloc(p, new_n * elem);
    memset((char *)p + old_n * elem, 0, (new_n - old_n) * elem);
    return p;
}

static void increase_tree_size(build_ctx *b) {
    tgo_tree *t = b->t;
    int64_t old = t->num_nodes;
    int64_t inc = (int64_t)((double)old * 1.2 + 1.0) - old;
    if (inc < 1) inc = 1;
    int64_t nw = old + inc;
    t->coord = (double *)grow(t->coord, 3 * old, 3 * nw, sizeof(double));
    t->mass = (double *)grow(t->mass, old, nw, sizeof(double));
    t->size = (double *)grow(t->size, old, nw, sizeof(double));
    t->delta = (double *)grow(t->delta, old, nw, sizeof(double));
    t->soft = (double *)grow(t->soft, old, nw, sizeof(double));
    if (t->quad) t->quad = (double *)grow(t->quad, 9 * old, 9 * nw, sizeof(double));
    t->first = (int64_t *)realloc(t->first, nw * sizeof(int64_t));
    t->next = (int64_t *)realloc(t->next, nw * sizeof(int64_t));
    for (int64_t i = old; i < nw; i++) t->first[i] = t->next[i] = -1;
    /* _grow_moment_arrays (octree.py:142-152) */
    b->acc = (double *)grow(b->acc, 3 * (old - t->npart), 3 * (nw - t->npart), sizeof(double));
    b->parent = (int64_t *)realloc(b->parent, (nw - t->npart) * sizeof(int64_t));
    for (int64_t i = old - t->npart; i < nw - t->npart; i++) b->parent[i] = -1;
    t->num_nodes = nw;
}

/* _octant_runs (octree.py:170-196); the binary-search and scanning branches give identical runs. */
static int octant_runs(const int64_t *keys, int64_t lo, int64_t hi, int shift, int64_t *bs, int64_t *be,
                       int *bd) {
    int nb = 0;
    int64_t start = lo;
    if (hi - lo > BSEARCH_MIN) {
        for (int d = 0; d < 8; d++) {
            if (start >= hi) break;
            int64_t a = start, z = hi; /* _digit_upper_bound (octree.py:155-167) */
            while (a < z) {
                int64_t mid = (a + z) >> 1;
                if (((keys[mid] >> shift) & 7) <= d) a = mid + 1;
                else z = mid;
            }
            if (a > start) {
                bs[nb] = start; be[nb] = a; bd[nb] = d;
                nb++;
                start = a;
            }
        }
    } else {
        while (start < hi) {
            int d = (int)((keys[start] >> shift) & 7);
            int64_t end = start + 1;
            while (end < hi && (int)((keys[end] >> shift) & 7) == d) end++;
            bs[nb] = start; be[nb] = end; bd[nb] = d;
            nb++;
            start = end;
        }
    }
    return nb;
}

/* RekeySlice (octree.py:1093-1126) */
static void rekey_slice(build_ctx *b, int64_t *keys_sorted, int64_t node, int64_t lo, int64_t hi) {
    tgo_tree *t = b->t;
    int64_t g = hi - lo;
    double center[3] = {t->coord[3 * node], t->coord[3 * node + 1], t->coord[3 * node + 2]};
    int64_t *subkeys = (int64_t *)malloc(g * sizeof(int64_t));
    int64_t *perm = (int64_t *)malloc(g * sizeof(int64_t));
    tgo_morton_keys(t->coord + 3 * lo, g, center, t->size[node], subkeys);
    tgo_radix_argsort(subkeys, g, perm);
    double *nc = (double *)malloc(3 * g * sizeof(double));
    double *nm = (double *)malloc(g * sizeof(double));
    double *ns = (double *)malloc(g * sizeof(double));
    int64_t *ni = (int64_t *)malloc(g * sizeof(int64_t));
    int64_t *nk = (int64_t *)malloc(g * sizeof(int64_t));
    for (int64_t a = 0; a < g; a++) {
        int64_t p = perm[a];
        for (int k = 0; k < 3; k++) nc[3 * a + k] = t->coord[3 * (lo + p) + k];
        nm[a] = t->mass[lo + p];
        ns[a] = t->soft[lo + p];
        ni[a] = t->walk_idx[lo + p];
        nk[a] = subkeys[p];
    }
    for (int64_t a = 0; a < g; a++) {
        for (int k = 0; k < 3; k++) t->coord[3 * (lo + a) + k] = nc[3 * a + k];
        t->mass[lo + a] = nm[a];
        t->soft[lo + a] = ns[a];
        t->walk_idx[lo + a] = ni[a];
        keys_sorted[lo + a] = nk[a];
    }
    free(subkeys); free(perm); free(nc); free(nm); free(ns); free(ni); free(nk);
}

/* Fold particle c into node `into` while standing on it (octree.py:956-966, 1162-1168). */
static inline void fold_particle(build_ctx *b, int64_t into, int64_t c) {
    tgo_tree *t = b->t;
    double mi = t->mass[c];
    t->mass[into] += mi;
    int64_t an = into - t->npart;
    for (int k = 0; k < 3; k++) b->acc[3 * an + k] += mi * t->coord[3 * c + k];
    t->soft[into] = pymax(t->soft[into], t->soft[c]);
    if (t->has_quads) b->pparent[c] = into;
}

/* BuildBucket (octree.py:1128-1175) */
static int64_t build_bucket(build_ctx *b, int64_t node, int64_t lo, int64_t hi, int64_t new_node_idx) {
    tgo_tree *t = b->t;
    t->has_coincident = 1;
    int64_t count = hi - lo, cur = node, last = -1;
    int slot = 0;
    for (int64_t jj = 0; jj < count; jj++) {
        int64_t remaining = count - 1 - jj;
        if (slot == 7 && remaining > 0) {
            int64_t nn = new_node_idx++;
            for (int k = 0; k < 3; k++)
                t->coord[3 * nn + k] = t->coord[3 * cur + k] + t->size[cur] * octant_offsets[7][k];
            t->size[nn] = t->size[cur] * 0.5;
            b->parent[nn - t->npart] = cur;
            if (last < 0) t->first[cur] = nn;
            else t->next[last] = nn;
            t->next[nn] = t->next[cur];
            cur = nn;
            slot = 0;
            last = -1;
        }
        int64_t c = lo + jj;
        fold_particle(b, cur, c);
        if (last < 0) t->first[cur] = c;
        else t->next[last] = c;
        last = c;
        slot++;
    }
    if (last >= 0) t->next[last] = t->next[cur];
    return new_node_idx;
}

typedef struct { int64_t node, lo, hi; int shift, rnd; } stack_ent;

/* BuildTreeRadix, serial path (octree.py:817-1091 with min_work = 0). Returns node_hi. */
static int64_t build_radix(build_ctx *b, const double *points, const double *masses, const double *soft,
                           int64_t N) {
    tgo_tree *t = b->t;
    double center[3], size;
    tgo_bounding_cube(points, N, center, &size);
    int64_t *keys = (int64_t *)malloc(N * sizeof(int64_t));
    int64_t *order = (int64_t *)malloc(N * sizeof(int64_t));
    int64_t *keys_sorted = (int64_t *)malloc(N * sizeof(int64_t));
    tgo_morton_keys(points, N, center, size, keys);
    tgo_radix_argsort(keys, N, order);
    memcpy(t->walk_idx, order, N * sizeof(int64_t));
    /* _permute_particles (octree.py:577-603) */
    for (int64_t i = 0; i < N; i++) {
        int64_t oi = order[i];
        for (int k = 0; k < 3; k++) t->coord[3 * i + k] = points[3 * oi + k];
        t->mass[i] = masses[oi];
        t->soft[i] = soft[oi];
        keys_sorted[i] = keys[oi];
    }
    int64_t root = N;
    t->size[root] = size;
    for (int k = 0; k < 3; k++) t->coord[3 * root + k] = center[k];
    int64_t new_node_idx = N + 1;

    int64_t cap = 64, top = 0;
    stack_ent *st = (stack_ent *)malloc(cap * sizeof(stack_ent));
    st[top++] = (stack_ent){root, 0, N, 3 * (MORTON_BITS - 1), 0};
    int64_t bs[8], be[8];
    int bd[8];
    while (top > 0) {
        stack_ent e = st[--top];
        int64_t node = e.node, lo = e.lo, hi = e.hi;
        int shift = e.shift, rnd = e.rnd;
        if (shift < 0) {
            if (rnd >= MORTON_MAX_ROUNDS) {
                while (new_node_idx + (hi - lo) / 7 + 2 > t->num_nodes) increase_tree_size(b);
                new_node_idx = build_bucket(b, node, lo, hi, new_node_idx);
                continue;
            }
            rekey_slice(b, keys_sorted, node, lo, hi);
            shift = 3 * (MORTON_BITS - 1);
            rnd += 1;
        }
        int64_t last_child = -1;
        int nb = octant_runs(keys_sorted, lo, hi, shift, bs, be, bd);
        for (int q = 0; q < nb; q++) {
            int64_t i = bs[q], j = be[q], c;
            int d = bd[q];
            if (j - i == 1) {
                c = i;
                fold_particle(b, node, i);
            } else {
                while (new_node_idx + 1 > t->num_nodes) increase_tree_size(b);
                int64_t cnode = new_node_idx++;
                for (int k = 0; k < 3; k++)
                    t->coord[3 * cnode + k] = t->coord[3 * node + k] + t->size[node] * octant_offsets[d][k];
                t->size[cnode] = t->size[node] * 0.5;
                b->parent[cnode - N] = node;
                c = cnode;
                if (top >= cap) {
                    cap *= 2;
                    st = (stack_ent *)realloc(st, cap * sizeof(stack_ent));
                }
                st[top++] = (stack_ent){cnode, i, j, shift - 3, rnd};
            }
            if (last_child < 0) t->first[node] = c;
            else t->next[last_child] = c;
            last_child = c;
        }
        if (last_child >= 0) t->next[last_child] = t->next[node];
    }
    free(st);
    free(keys);
    free(order);
    free(keys_sorted);
    return new_node_idx;
}

/* RollupMoments (octree.py:199-231) */
static void rollup_moments(build_ctx *b, int64_t node_hi) {
    tgo_tree *t = b->t;
    int64_t npart = t->npart;
    for (int64_t node = node_hi - 1; node > npart - 1; node--) {
        int64_t a = node - npart;
        double m = t->mass[node];
        if (m == 0.0) continue;
        double inv = 1.0 / m;
        double d2 = 0.0;
        int64_t p = b->parent[a];
        for (int k = 0; k < 3; k++) {
            double com = b->acc[3 * a + k] * inv;
            double dx = com - t->coord[3 * node + k];
            d2 += dx * dx;
            t->coord[3 * node + k] = com;
        }
        t->delta[node] = sqrt(d2);
        if (p >= npart) {
            int64_t pa = p - npart;
            for (int k = 0; k < 3; k++) b->acc[3 * pa + k] += b->acc[3 * a + k];
            t->mass[p] += m;
            t->soft[p] = pymax(t->soft[p], t->soft[node]);
        }
    }
}

/* _shift_quad_into (octree.py:234-250) */
static inline void shift_quad_into(double *Q, double m, double r0, double r1, double r2) {
    double rsq = r0 * r0 + r1 * r1 + r2 * r2;
    Q[0] += m * (3.0 * r0 * r0 - rsq);
    Q[1] += m * 3.0 * r0 * r1;
    Q[2] += m * 3.0 * r0 * r2;
    Q[3] += m * 3.0 * r1 * r0;
    Q[4] += m * (3.0 * r1 * r1 - rsq);
    Q[5] += m * 3.0 * r1 * r2;
    Q[6] += m * 3.0 * r2 * r0;
    Q[7] += m * 3.0 * r2 * r1;
    Q[8] += m * (3.0 * r2 * r2 - rsq);
}

/* RollupQuadrupoles (octree.py:253-292) */
static void rollup_quadrupoles(build_ctx *b, int64_t node_hi) {
    tgo_tree *t = b->t;
    int64_t npart = t->npart;
    double *Q = t->quad, *C = t->coord;
    for (int64_t i = 0; i < npart; i++) {
        int64_t p = b->pparent[i];
        if (p < npart) continue;
        shift_quad_into(Q + 9 * p, t->mass[i], C[3 * i] - C[3 * p], C[3 * i + 1] - C[3 * p + 1],
                        C[3 * i + 2] - C[3 * p + 2]);
    }
    for (int64_t node = node_hi - 1; node > npart - 1; node--) {
        int64_t p = b->parent[node - npart];
        if (p < npart) continue;
        double m = t->mass[node];
        if (m == 0.0) continue;
        double r0 = C[3 * node] - C[3 * p];
        double r1 = C[3 * node + 1] - C[3 * p + 1];
        double r2 = C[3 * node + 2] - C[3 * p + 2];
        for (int k = 0; k < 9; k++) Q[9 * p + k] += Q[9 * node + k];
        shift_quad_into(Q + 9 * p, m, r0, r1, r2);
    }
}

int tgo_build(const double *pos, const double *m, const double *h, int64_t n, int quadrupole,
              int compute_moments, tgo_tree *out) {
    if (n < 1) return 1;
    memset(out, 0, sizeof(*out));
    tree_alloc(out, n, quadrupole);
    double *mz = NULL, *hz = NULL;
    if (!m) {
        mz = (double *)calloc(n, sizeof(double));
        m = mz;
        compute_moments = 0;
    }
    if (!h) {
        hz = (double *)calloc(n, sizeof(double));
        h = hz;
    }
    build_ctx b;
    b.t = out;
    int64_t nn = out->num_nodes - n;
    b.acc = (double *)calloc(3 * nn, sizeof(double));
    b.parent = (int64_t *)malloc(nn * sizeof(int64_t));
    for (int64_t i = 0; i < nn; i++) b.parent[i] = -1;
    b.pparent = (int64_t *)malloc(n * sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) b.pparent[i] = -1;
    int64_t node_hi = build_radix(&b, pos, m, h, n);
    out->node_hi = node_hi;
    if (compute_moments) {
        rollup_moments(&b, node_hi);
        if (quadrupole) rollup_quadrupoles(&b, node_hi);
    }
    free(b.acc);
    free(b.parent);
    free(b.pparent);
    free(mz);
    free(hz);
    return 0;
}

void tgo_free(tgo_tree *t) {
    free(t->coord); free(t->mass); free(t->size); free(t->delta); free(t->soft); free(t->quad);
    free(t->first); free(t->next); free(t->walk_idx);
    memset(t, 0, sizeof(*t));
}

/* ------------------------------------------------------------------------------------------ */
/* acceptance_criterion (treewalk.py:22-25) */
static inline int accept(double r, double h, double size, double delta, double theta) {
    return r > pymax(size / theta + delta, h + size * 0.6 + delta);
}

typedef struct {
    int pot, acc, tid, quad;
} field_set;

/* One element's contribution to targets [a, b): the per-interaction kernel built by
 * _make_field_kernel (grouped_treewalk.py:45-155). */
static void field_kernel(const tgo_tree *t, int64_t no, int64_t a, int64_t b, const double *pos,
                         const double *soft, double *acc, int W, field_set f) {
    double cx = t->coord[3 * no], cy = t->coord[3 * no + 1], cz = t->coord[3 * no + 2];
    double M = t->mass[no];
    double hs = t->soft[no];
    int is_node = f.quad ? (no >= t->npart) : 0;
    double qxx = 0, qxy = 0, qxz = 0, qyx = 0, qyy = 0, qyz = 0, qzx = 0, qzy = 0, qzz = 0;
    if (f.quad && is_node) {
        const double *Q = t->quad + 9 * no;
        qxx = Q[0]; qxy = Q[1]; qxz = Q[2];
        qyx = Q[3]; qyy = Q[4]; qyz = Q[5];
        qzx = Q[6]; qzy = Q[7]; qzz = Q[8];
    }
    for (int64_t ti = a; ti < b; ti++) {
        double dx = cx - pos[3 * ti], dy = cy - pos[3 * ti + 1], dz = cz - pos[3 * ti + 2];
        double r2 = dx * dx + dy * dy + dz * dz;
        if (!(r2 > 0)) continue;
        double r = sqrt(r2);
        double ht = pymax(hs, soft[ti]);
        int softened = r < ht;
        double phi = 0.0, K = 0.0, Qk = 0.0;
        if (f.pot) phi = softened ? M * tgo_potential_kernel(r, ht) : -M / r;
        if (f.acc || f.tid) K = softened ? M * tgo_force_kernel(r, ht) : M / (r * r2);
        if (f.tid) Qk = softened ? M * tgo_tidal_kernel(r, ht) : 3.0 * K / r2;
        double gx = 0, gy = 0, gz = 0;
        if (f.acc) {
            gx = K * dx;
            gy = K * dy;
            gz = K * dz;
        }
        double txx = 0, tyy = 0, tzz = 0, txy = 0, txz = 0, tyz = 0;
        if (f.tid) {
            txx = Qk * dx * dx - K;
            tyy = Qk * dy * dy - K;
            tzz = Qk * dz * dz - K;
            txy = Qk * dx * dy;
            txz = Qk * dx * dz;
            tyz = Qk * dy * dz;
        }
        if (f.quad && is_node) {
            double r5inv = 1.0 / (r2 * r2 * r);
            double r7inv = r5inv / r2;
            double qdx = qxx * dx + qxy * dy + qxz * dz;
            double qdy = qyx * dx + qyy * dy + qyz * dz;
            double qdz = qzx * dx + qzy * dy + qzz * dz;
            double A = dx * qdx + dy * qdy + dz * qdz;
            if (f.pot) phi += -0.5 * A * r5inv;
            if (f.acc) {
                double quad_fac = A * r7inv;
                gx += 2.5 * quad_fac * dx - qdx * r5inv;
                gy += 2.5 * quad_fac * dy - qdy * r5inv;
                gz += 2.5 * quad_fac * dz - qdz * r5inv;
            }
            if (f.tid) {
                double diag = -2.5 * A * r7inv;
                double fac = 17.5 * A * r7inv / r2;
                txx += qxx * r5inv - 10.0 * dx * qdx * r7inv + diag + fac * dx * dx;
                tyy += qyy * r5inv - 10.0 * dy * qdy * r7inv + diag + fac * dy * dy;
                tzz += qzz * r5inv - 10.0 * dz * qdz * r7inv + diag + fac * dz * dz;
                txy += qxy * r5inv - 5.0 * (dx * qdy + dy * qdx) * r7inv + fac * dx * dy;
                txz += qxz * r5inv - 5.0 * (dx * qdz + dz * qdx) * r7inv + fac * dx * dz;
                tyz += qyz * r5inv - 5.0 * (dy * qdz + dz * qdy) * r7inv + fac * dy * dz;
            }
        }
        double *o = acc + (ti - a) * W;
        int k = 0;
        if (f.pot) o[k++] += phi;
        if (f.acc) {
            o[k] += gx; o[k + 1] += gy; o[k + 2] += gz;
            k += 3;
        }
        if (f.tid) {
            o[k] += txx; o[k + 1] += txy; o[k + 2] += txz;
            o[k + 3] += txy; o[k + 4] += tyy; o[k + 5] += tyz;
            o[k + 6] += txz; o[k + 7] += tyz; o[k + 8] += tzz;
        }
    }
}

/* One group's bounding box and maximum softening (grouped_treewalk.py:183-205). */
static void group_bbox(const double *pos, const double *soft, int64_t a, int64_t b, double bmin[3],
                       double bmax[3], double *hmax) {
    for (int k = 0; k < 3; k++) bmin[k] = bmax[k] = pos[3 * a + k];
    *hmax = soft[a];
    for (int64_t ti = a + 1; ti < b; ti++) {
        for (int k = 0; k < 3; k++) {
            double v = pos[3 * ti + k];
            if (v < bmin[k]) bmin[k] = v;
            else if (v > bmax[k]) bmax[k] = v;
        }
        if (soft[ti] > *hmax) *hmax = soft[ti];
    }
}

static inline double rmin_to_box(const double *c, const double *bmin, const double *bmax) {
    double d[3];
    for (int k = 0; k < 3; k++) {
        d[k] = 0.0;
        if (c[k] < bmin[k]) d[k] = bmin[k] - c[k];
        else if (c[k] > bmax[k]) d[k] = c[k] - bmax[k];
    }
    return sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

static void walk_group(const tgo_tree *t, const double *pos, const double *soft, int64_t a, int64_t b, field_set f,
                       int W, double theta, double G, double *out) {
    int64_t m = b - a;
    double bmin[3], bmax[3], hmax;
    group_bbox(pos, soft, a, b, bmin, bmax, &hmax);
    double *acc = (double *)calloc(m * W, sizeof(double));
    int64_t no = t->npart;
    while (no > -1) {
        double r_min = rmin_to_box(t->coord + 3 * no, bmin, bmax);
        double h = pymax(t->soft[no], hmax);
        if (no < t->npart || accept(r_min, h, t->size[no], t->delta[no], theta)) {
            field_kernel(t, no, a, b, pos, soft, acc, W, f);
            no = t->next[no];
        } else {
            no = t->first[no];
        }
    }
    for (int64_t ti = a; ti < b; ti++)
        for (int k = 0; k < W; k++) out[ti * W + k] = G * acc[(ti - a) * W + k];
    free(acc);
}

/* The same walk over explicitly given groups [start, start + count) of pos. */
int tgo_fields_groups(const tgo_tree *t, const double *pos, const double *soft, const int64_t *start,
                      const int64_t *count, int64_t ngroups, int want_pot, int want_acc, int want_tidal,
                      int quadrupole, double theta, double G, double *out, int nthreads) {
    if (!(want_pot || want_acc || want_tidal)) return 1;
    if (quadrupole && !t->has_quads) return 2;
    field_set f = {want_pot, want_acc, want_tidal, quadrupole};
    int W = want_pot + 3 * want_acc + 9 * want_tidal;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t gi = 0; gi < ngroups; gi++) walk_group(t, pos, soft, start[gi], start[gi] + count[gi], f, W, theta, G, out);
    return 0;
}

/* The traversal core built by _make_core (grouped_treewalk.py:163-241). */
int tgo_fields(const tgo_tree *t, const double *pos, const double *soft, int64_t n, int want_pot,
               int want_acc, int want_tidal, int quadrupole, int64_t group_size, double theta,
               double G, double *out, int nthreads) {
    if (!(want_pot || want_acc || want_tidal) || group_size < 1) return 1;
    if (quadrupole && !t->has_quads) return 2;
    field_set f = {want_pot, want_acc, want_tidal, quadrupole};
    int W = want_pot + 3 * want_acc + 9 * want_tidal;
    int64_t ngroups = (n + group_size - 1) / group_size;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t gi = 0; gi < ngroups; gi++) {
        int64_t a = gi * group_size;
        int64_t b = a + group_size < n ? a + group_size : n;
        int64_t m = b - a;
        double bmin[3], bmax[3], hmax;
        group_bbox(pos, soft, a, b, bmin, bmax, &hmax);
        double *acc = (double *)calloc(m * W, sizeof(double));
        int64_t no = t->npart;
        while (no > -1) {
            double r_min = rmin_to_box(t->coord + 3 * no, bmin, bmax);
            double h = pymax(t->soft[no], hmax);
            if (no < t->npart || accept(r_min, h, t->size[no], t->delta[no], theta)) {
                field_kernel(t, no, a, b, pos, soft, acc, W, f);
                no = t->next[no];
            } else {
                no = t->first[no];
            }
        }
        for (int64_t ti = a; ti < b; ti++)
            for (int k = 0; k < W; k++) out[ti * W + k] = G * acc[(ti - a) * W + k];
        free(acc);
    }
    return 0;
}

int tgo_walk_counts(const tgo_tree *t, const double *pos, const double *soft, int64_t n,
                    int64_t group_size, double theta, int64_t *n_interactions, int64_t *n_opened,
                    int nthreads) {
    int64_t ngroups = (n + group_size - 1) / group_size;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t gi = 0; gi < ngroups; gi++) {
        int64_t a = gi * group_size;
        int64_t b = a + group_size < n ? a + group_size : n;
        double bmin[3], bmax[3], hmax;
        group_bbox(pos, soft, a, b, bmin, bmax, &hmax);
        int64_t ni = 0, no_open = 0;
        int64_t no = t->npart;
        while (no > -1) {
            double r_min = rmin_to_box(t->coord + 3 * no, bmin, bmax);
            double h = pymax(t->soft[no], hmax);
            if (no < t->npart || accept(r_min, h, t->size[no], t->delta[no], theta)) {
                ni++;
                no = t->next[no];
            } else {
                no_open++;
                no = t->first[no];
            }
        }
        n_interactions[gi] = ni;
        n_opened[gi] = no_open;
    }
    return 0;
}

/* Interaction counts of the same walk for explicitly given groups [start, start + count). */
int tgo_walk_counts_groups(const tgo_tree *t, const double *pos, const double *soft, const int64_t *start,
                           const int64_t *count, int64_t ngroups, double theta, int64_t *n_interactions,
                           int64_t *n_opened, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t gi = 0; gi < ngroups; gi++) {
        int64_t a = start[gi], b = start[gi] + count[gi];
        double bmin[3], bmax[3], hmax;
        group_bbox(pos, soft, a, b, bmin, bmax, &hmax);
        int64_t ni = 0, no_open = 0;
        int64_t no = t->npart;
        while (no > -1) {
            double r_min = rmin_to_box(t->coord + 3 * no, bmin, bmax);
            double h = pymax(t->soft[no], hmax);
            if (no < t->npart || accept(r_min, h, t->size[no], t->delta[no], theta)) {
                ni++;
                no = t->next[no];
            } else {
                no_open++;
                no = t->first[no];
            }
        }
        n_interactions[gi] = ni;
        n_opened[gi] = no_open;
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Brute force (bruteforce.py).  Per target i, sources j in ascending order, FP64, as the
 * per-target parallel variants sum.  Target form skips r == 0 pairs; mutual form skips j == i
 * only, so a distinct coincident softened source still contributes to the potential
 * (bruteforce.py:86-116 vs 7-50). */
int tgo_bruteforce(const double *pt, const double *ht, int64_t nt, const double *ps, const double *ms,
                   const double *hs, int64_t ns, int want_pot, int want_acc, int want_tidal, int mode,
                   double G, double *out, int nthreads) {
    int W = want_pot + 3 * want_acc + 9 * want_tidal;
    if (W == 0) return 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t i = 0; i < nt; i++) {
        double phi = 0.0, a0 = 0.0, a1 = 0.0, a2 = 0.0;
        double T[9] = {0};
        for (int64_t j = 0; j < ns; j++) {
            if (mode == 1 && i == j) continue;
            /* argument order of max() as in each reference form (matters only for +-0) */
            double hij_pot = mode == 1 ? pymax(ht[i], hs[j]) : pymax(hs[j], ht[i]);
            double hij = pymax(ht[i], hs[j]);
            if (want_pot) {
                /* PotentialTarget_bruteforce: dx = x_t - x_s (bruteforce.py:25-27) */
                double d0 = pt[3 * i] - ps[3 * j], d1 = pt[3 * i + 1] - ps[3 * j + 1],
                       d2 = pt[3 * i + 2] - ps[3 * j + 2];
                double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                if (mode == 0) {
                    if (r == 0) goto skip_pot;
                    if (r < hij_pot) phi += ms[j] * tgo_potential_kernel(r, hij_pot);
                    else phi -= ms[j] / r;
                } else {
                    if (r < hij_pot) phi += ms[j] * tgo_potential_kernel(r, hij_pot);
                    else if (r > 0) phi -= ms[j] / r;
                }
            }
        skip_pot:
            if (want_acc || want_tidal) {
                /* AccelTarget_bruteforce: dx = x_s - x_t (bruteforce.py:236-238) */
                double d0 = ps[3 * j] - pt[3 * i], d1 = ps[3 * j + 1] - pt[3 * i + 1],
                       d2 = ps[3 * j + 2] - pt[3 * i + 2];
                double r2 = d0 * d0 + d1 * d1 + d2 * d2;
                if (r2 == 0) continue;
                double r = sqrt(r2);
                if (want_acc) {
                    if (r < hij) {
                        double kernel = tgo_force_kernel(r, hij);
                        a0 += kernel * ms[j] * d0;
                        a1 += kernel * ms[j] * d1;
                        a2 += kernel * ms[j] * d2;
                    } else {
                        double fac = 1 / (r2 * r);
                        a0 += ms[j] * fac * d0;
                        a1 += ms[j] * fac * d1;
                        a2 += ms[j] * fac * d2;
                    }
                }
                if (want_tidal) {
                    /* _add_tidal_pair (bruteforce.py:259-282) */
                    double K, Q;
                    if (r < hij) {
                        K = ms[j] * tgo_force_kernel(r, hij);
                        Q = ms[j] * tgo_tidal_kernel(r, hij);
                    } else {
                        K = ms[j] / (r * r2);
                        Q = 3.0 * K / r2;
                    }
                    T[0] += Q * d0 * d0 - K;
                    T[4] += Q * d1 * d1 - K;
                    T[8] += Q * d2 * d2 - K;
                    double txy = Q * d0 * d1, txz = Q * d0 * d2, tyz = Q * d1 * d2;
                    T[1] += txy; T[3] += txy;
                    T[2] += txz; T[6] += txz;
                    T[5] += tyz; T[7] += tyz;
                }
            }
        }
        double *o = out + i * W;
        int k = 0;
        if (want_pot) o[k++] = G * phi;
        if (want_acc) {
            o[k] = G * a0; o[k + 1] = G * a1; o[k + 2] = G * a2;
            k += 3;
        }
        if (want_tidal)
            for (int q = 0; q < 9; q++) o[k + q] = G * T[q];
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Column density.                                                                             */
#ifndef M_PI
#define M_PI 3.14159265358979323846 /* numpy.pi */
#endif

/* ColumnDensityWalk_singleray (treewalk.py:904-973), in its order of operations: the column from
 * pos to infinity along ray of the uniform spheres (mass, radius = softening) in the tree. */
static double column_singleray(const tgo_tree *t, const double *pos, const double *ray) {
    const int64_t N = t->npart;
    const double fac_density = 3.0 / (4.0 * M_PI);
    double column = 0.0;
    int64_t no = N;
    const int64_t stop = t->next[N];
    while (no > -1 && no != stop) {
        double dx[3], r2 = 0.0;
        for (int k = 0; k < 3; k++) {
            dx[k] = t->coord[3 * no + k] - pos[k];
            r2 += dx[k] * dx[k];
        }
        const double r = sqrt(r2);
        const double z = ray[0] * dx[0] + ray[1] * dx[1] + ray[2] * dx[2];
        if (r2 - z * z < 0) {
            no = t->next[no];
            continue;
        }
        const double h_no = t->soft[no];
        if (no < N) {
            if (h_no > 0) {
                const double h_inv = 1.0 / h_no;
                const double fac = fac_density * t->mass[no] * h_inv * h_inv;
                const double r_proj = sqrt(r2 - z * z);
                const double q = r_proj * h_inv;
                if (r_proj < h_no) {
                    if (r > h_no) {
                        if (z > 0) column += fac * 2 * sqrt(1 - q * q);
                    } else {
                        const double dz = z * h_inv;
                        column += fac * (dz + sqrt(1 - q * q));
                    }
                }
            }
            no = t->next[no];
        } else {
            const double R_eff = t->size[no] * 0.8660254037844386 + t->delta[no];
            int open = 0;
            if (r < h_no + R_eff) open = 1;
            else if (z > 0 && (r2 - z * z) < (t->soft[no] + R_eff) * (t->soft[no] + R_eff)) open = 1;
            no = open ? t->first[no] : t->next[no];
        }
    }
    return column;
}

void tgo_column_rays(const tgo_tree *t, const double *pos, int64_t n, const double *rays, int64_t nrays,
                     int64_t ray_stride, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < nrays; j++)
            out[i * nrays + j] = column_singleray(t, pos + 3 * i, rays + i * ray_stride + 3 * j);
}

/* angular_bin (treewalk.py:49-70): the axis of the largest |component|, sign first */
static int angular_bin(const double dx[3]) {
    if (fabs(dx[0]) > fabs(dx[1]) && fabs(dx[0]) > fabs(dx[2])) return dx[0] > 0 ? 0 : 1;
    if (fabs(dx[1]) > fabs(dx[2])) return dx[1] > 0 ? 2 : 3;
    return dx[2] > 0 ? 4 : 5;
}

/* ColumnDensityWalk_binned (treewalk.py:976-1030) */
static void column_binned(const tgo_tree *t, const double *pos, double theta, double *column) {
    const int64_t N = t->npart;
    const double angular_bin_size = (4 * M_PI) / 6;
    for (int k = 0; k < 6; k++) column[k] = 0.0;
    int64_t no = N;
    const int64_t stop = t->next[N];
    while (no > -1 && no != stop) {
        double dx[3], r2 = 0.0;
        for (int k = 0; k < 3; k++) {
            dx[k] = t->coord[3 * no + k] - pos[k];
            r2 += dx[k] * dx[k];
        }
        const double h = t->soft[no];
        if (no < N) {
            const int bin = angular_bin(dx);
            if (r2 > h * h) {
                column[bin] += t->mass[no] / r2 / angular_bin_size;
            } else if (h > 0) {
                const double col0 = t->mass[no] * (3 / (4 * M_PI * h * h));
                const double fac = sqrt(r2) / h;
                const double col_iso = (1 - fac) * col0;
                for (int k = 0; k < 6; k++) column[k] += col_iso;
                column[bin] += col0 * fac * 2;
            }
            no = t->next[no];
        } else {
            if (accept(sqrt(r2), h, t->size[no], t->delta[no], theta)) {
                column[angular_bin(dx)] += t->mass[no] / r2 / angular_bin_size;
                no = t->next[no];
            } else {
                no = t->first[no];
            }
        }
    }
}

void tgo_column_binned(const tgo_tree *t, const double *pos, int64_t n, double theta, double *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < n; i++) column_binned(t, pos + 3 * i, theta, out + 6 * i);
}

/* angular_bin_scalar (treewalk.py:38-45) is angular_bin on the three components */
void tgo_column_binned_grouped(const tgo_tree *t, const double *pos, int64_t n, double theta, int64_t group_size,
                               double *out, int nthreads) {
    const int64_t N = t->npart;
    const double angular_bin_size = (4 * M_PI) / 6;
    const int64_t ngroups = (n + group_size - 1) / group_size;
    for (int64_t i = 0; i < 6 * n; i++) out[i] = 0.0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t gi = 0; gi < ngroups; gi++) {
        const int64_t a = gi * group_size, b = a + group_size < n ? a + group_size : n;
        double bmin[3], bmax[3];
        for (int k = 0; k < 3; k++) bmin[k] = bmax[k] = pos[3 * a + k];
        for (int64_t tt = a + 1; tt < b; tt++)
            for (int k = 0; k < 3; k++) {
                const double v = pos[3 * tt + k];
                if (v < bmin[k]) bmin[k] = v;
                else if (v > bmax[k]) bmax[k] = v;
            }
        int64_t no = N;
        const int64_t stop = t->next[N];
        while (no > -1 && no != stop) {
            const double c[3] = {t->coord[3 * no], t->coord[3 * no + 1], t->coord[3 * no + 2]};
            const double h_no = t->soft[no], M = t->mass[no];
            if (no < N) {
                const double hh = h_no * h_no;
                for (int64_t tt = a; tt < b; tt++) {
                    const double d[3] = {c[0] - pos[3 * tt], c[1] - pos[3 * tt + 1], c[2] - pos[3 * tt + 2]};
                    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                    const int bin = angular_bin(d);
                    double *o = out + 6 * tt;
                    if (r2 > hh) {
                        o[bin] += M / r2 / angular_bin_size;
                    } else if (h_no > 0) {
                        const double col0 = M * (3 / (4 * M_PI * hh));
                        const double fac = sqrt(r2) / h_no;
                        const double col_iso = (1 - fac) * col0;
                        for (int k = 0; k < 6; k++) o[k] += col_iso;
                        o[bin] += col0 * fac * 2;
                    }
                }
                no = t->next[no];
            } else {
                double dm[3];
                for (int k = 0; k < 3; k++) {
                    dm[k] = 0.0;
                    if (c[k] < bmin[k]) dm[k] = bmin[k] - c[k];
                    else if (c[k] > bmax[k]) dm[k] = c[k] - bmax[k];
                }
                const double r_min = sqrt(dm[0] * dm[0] + dm[1] * dm[1] + dm[2] * dm[2]);
                if (accept(r_min, h_no, t->size[no], t->delta[no], theta)) {
                    for (int64_t tt = a; tt < b; tt++) {
                        const double d[3] = {c[0] - pos[3 * tt], c[1] - pos[3 * tt + 1], c[2] - pos[3 * tt + 2]};
                        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                        out[6 * tt + angular_bin(d)] += M / r2 / angular_bin_size;
                    }
                    no = t->next[no];
                } else {
                    no = t->first[no];
                }
            }
        }
    }
}
