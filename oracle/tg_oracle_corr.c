/*
 * CPU oracle for the two-point functions -- TEST INFRASTRUCTURE ONLY (see tg_oracle.h).
 *
 * Restates, on the oracle's radix tree (paths relative to the pytreegrav project):
 *   ComputeMomentsDynamic   src/pytreegrav/dynamic_tree.py:246-310 (velocities and dispersions only;
 *                           masses, centres and sizes are the radix tree's, which the DynamicOctree
 *                           shares on inputs without coincident points)
 *   NearestImage            src/pytreegrav/treewalk.py:70-75
 *   do_weighted_binning     src/pytreegrav/treewalk.py:344-375
 *   DensityCorrWalk         src/pytreegrav/treewalk.py:378-462
 *   VelocityCorrWalk        src/pytreegrav/treewalk.py:515-608
 *   VelocityStructWalk      src/pytreegrav/treewalk.py:668-761
 *   *CorrFunc_tree, VelocityStructFunc_tree (chunked accumulation) treewalk.py:465-510, 611-663, 764-818
 *
 * Departures, each shared with the CUDA path: the jitter of a node's distance (pytreegrav draws
 * np.random.rand()) comes from corr_uniform(seed, target, draw) below; a bin index outside
 * [0, nbins) from jitter is clamped into it (pytreegrav indexes past its array there), and the lowest
 * spread bin is clamped at 0 (below 0 pytreegrav's wrapped indices only meet bins with no overlap);
 * each contribution is multiplied by the target's weight (pytreegrav multiplies the target's per-bin
 * sums). With absval set, every contribution enters as its absolute value: the per-bin scale that a
 * test's rounding bound is taken relative to.
 */
#include "tg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CORR_CHUNKS 64

/* Uniform double in [0, 1) from (seed, target, draw): splitmix64 finalisation of a Weyl sequence. */
double tgo_corr_uniform(uint64_t seed, int64_t target, int64_t draw) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(target + 1) + 0xD1B54A32D192ED03ull * (uint64_t)(draw + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

/* ComputeMomentsDynamic: returns the node's dispersion; writes vel/disp for node f and below. */
static double moments(const tgo_tree *t, int64_t f, double *vel, double *disp) {
    if (f < t->npart) return 0.0;
    const int64_t stop = t->next[f];
    double m = 0.0, v[3] = {0.0, 0.0, 0.0}, vd = 0.0;
    for (int64_t c = t->first[f]; c != stop && c >= 0; c = t->next[c]) {
        const double vdc = moments(t, c, vel, disp);
        const double mc = t->mass[c];
        m += mc;
        for (int k = 0; k < 3; k++) v[k] += mc * vel[3 * c + k];
        vd += mc * vdc;
    }
    for (int k = 0; k < 3; k++) v[k] = v[k] / m;
    for (int64_t c = t->first[f]; c != stop && c >= 0; c = t->next[c]) {
        const double dv0 = vel[3 * c] - v[0], dv1 = vel[3 * c + 1] - v[1], dv2 = vel[3 * c + 2] - v[2];
        vd += t->mass[c] * (dv0 * dv0 + dv1 * dv1 + dv2 * dv2);
    }
    vd = vd / m;
    for (int k = 0; k < 3; k++) vel[3 * f + k] = v[k];
    disp[f] = vd;
    return vd;
}

void tgo_tree_velocities(const tgo_tree *t, const double *vel_in, double *vel, double *disp) {
    const int64_t N = t->npart;
    memset(vel, 0, sizeof(double) * 3 * t->num_nodes);
    memset(disp, 0, sizeof(double) * t->num_nodes);
    for (int64_t i = 0; i < N; i++)
        for (int k = 0; k < 3; k++) vel[3 * i + k] = vel_in[3 * t->walk_idx[i] + k];
    if (N > 0) moments(t, N, vel, disp);
}

static inline double nearest_image(double x, double box) {
    if (fabs(x) > box / 2) return -copysign(box - fabs(x), x);
    return x;
}

static inline int bin_of(double r, double logr_min, double dlogr, int nbins) {
    const double tt = nbins * (log10(r) - logr_min) / dlogr;
    if (!(tt >= 0.0)) return 0;
    if (tt >= (double)nbins) return nbins - 1;
    return (int)tt;
}

typedef struct {
    const tgo_tree *t;
    const double *vel, *disp;
    int kind, weighted, absval, nbins;
    const double *rbins;
    double mbr, theta, box;
    uint64_t seed;
} corr_ctx;

static inline double cabs_(const corr_ctx *c, double x) { return c->absval ? fabs(x) : x; }

static void spread(const corr_ctx *c, double *row, double r, int r_idx, double h, double M, double quantity,
                   double w) {
    const double *rb = c->rbins;
    if ((r + h < rb[r_idx + 1]) && (r - h > rb[r_idx])) {
        row[r_idx] += cabs_(c, w * (M * quantity));
        return;
    }
    const double lratio = log10(rb[1] / rb[0]);
    const double tmin = log10((r - h) / rb[0]) / lratio;
    const int min_bin = tmin >= (double)c->nbins ? c->nbins : (tmin > 0.0 ? (int)tmin : 0);
    const double tmax = log10((r + h) / rb[0]) / lratio + 1;
    const int max_bin = tmax >= (double)c->nbins ? c->nbins : (tmax > 0.0 ? (int)tmax : 0);
    double total = 0.0;
    for (int i = min_bin; i < max_bin; i++) {
        const double i1 = fmax(r - h, rb[i]), i2 = fmin(r + h, rb[i + 1]), ov = i2 - i1;
        if (ov > 0) {
            const double dr = fabs(r - 0.5 * (i1 + i2));
            total += fmax(0.0, 1 - dr * dr / (h * h)) * ov;
        }
    }
    for (int i = min_bin; i < max_bin; i++) {
        const double i1 = fmax(r - h, rb[i]), i2 = fmin(r + h, rb[i + 1]), ov = i2 - i1;
        if (ov > 0) {
            const double dr = fabs(r - 0.5 * (i1 + i2));
            const double wt = fmax(0.0, 1 - dr * dr / (h * h)) * ov / total;
            row[i] += cabs_(c, w * (wt * M * quantity));
        }
    }
}

/* One target's walk; bins at row[0, nbins), weight sums at row[nbins, 2 nbins) (kinds 1, 2). */
static void corr_walk(const corr_ctx *c, int64_t i, const double *pos, const double *tvel, double w, double *row) {
    const tgo_tree *t = c->t;
    const int64_t N = t->npart;
    const int nb = c->nbins;
    const double rmin = c->rbins[0], rmax = c->rbins[nb];
    const double logr_min = log10(rmin), dlogr = log10(rmax) - logr_min;
    double *bins = row, *wts = row + nb;
    int64_t draws = 0, no = N;
    const int64_t stop = t->next[N];
    while (no > -1 && no != stop) {
        double dx[3], r = 0.0;
        for (int k = 0; k < 3; k++) {
            dx[k] = t->coord[3 * no + k] - pos[k];
            if (c->box > 0) dx[k] = nearest_image(dx[k], c->box);
            r += dx[k] * dx[k];
        }
        r = sqrt(r);
        const int part = no < N;
        const double s = t->size[no], del = t->delta[no];
        const int far = !part && r > fmax(s / c->theta + del, s * 0.6 + del);
        if ((r > rmin) && (r < rmax)) {
            const int r_idx = bin_of(r, logr_min, dlogr, nb);
            const double M = t->mass[no];
            if (part) {
                double amount = M;
                if (c->kind == 1) {
                    amount = 0.0;
                    for (int k = 0; k < 3; k++) amount += tvel[k] * c->vel[3 * no + k] * M;
                } else if (c->kind == 2) {
                    amount = 0.0;
                    for (int k = 0; k < 3; k++)
                        amount += (tvel[k] - c->vel[3 * no + k]) * (tvel[k] - c->vel[3 * no + k]) * M;
                }
                bins[r_idx] += cabs_(c, w * amount);
                if (c->kind) wts[r_idx] += w * M;
                no = t->next[no];
            } else if (far && s < c->mbr * (c->rbins[r_idx + 1] - c->rbins[r_idx])) {
                double q = 1.0;
                if (c->kind == 1) {
                    q = 0.0;
                    for (int k = 0; k < 3; k++) q += tvel[k] * c->vel[3 * no + k];
                } else if (c->kind == 2) {
                    q = 0.0;
                    for (int k = 0; k < 3; k++) q += (tvel[k] - c->vel[3 * no + k]) * (tvel[k] - c->vel[3 * no + k]);
                    q += c->disp[no];
                }
                if (c->weighted) {
                    spread(c, bins, r, r_idx, 0.5 * s, M, q, w);
                    if (c->kind) {
                        corr_ctx c1 = *c;
                        c1.absval = 0;
                        spread(&c1, wts, r, r_idx, 0.5 * s, M, 1.0, w);
                    }
                } else {
                    const double rnew = r + (tgo_corr_uniform(c->seed, i, draws++) - 0.5) * s;
                    const int j = rnew > 0 ? bin_of(rnew, logr_min, dlogr, nb) : 0;
                    bins[j] += cabs_(c, w * (c->kind ? q * M : M));
                    if (c->kind) wts[j] += w * M;
                }
                no = t->next[no];
            } else {
                no = t->first[no];
            }
        } else {
            no = (part || far) ? t->next[no] : t->first[no];
        }
    }
}

/* Sums over targets in CORR_CHUNKS fixed chunks (chunk k: targets k, k + CORR_CHUNKS, ...), added in
 * chunk order, so the result does not depend on the thread count. */
int tgo_correlation(const tgo_tree *t, const double *vel, const double *disp, int kind, const double *pos,
                    const double *tvel, const double *weight, int64_t n, const double *rbins, int nbins,
                    double max_bin_size_ratio, double theta, double boxsize, int weighted_binning, uint64_t seed,
                    int absval, double *binsums, double *wtsums, int nthreads) {
    if (nbins < 1 || (kind && (!vel || !disp || !tvel || !weight))) return 1;
    corr_ctx c = {t, vel, disp, kind, weighted_binning ? 1 : 0, absval ? 1 : 0, nbins, rbins,
                  max_bin_size_ratio, theta, boxsize, seed};
    double *rows = (double *)calloc((size_t)CORR_CHUNKS * 2 * nbins, sizeof(double));
    if (!rows) return 2;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int k = 0; k < CORR_CHUNKS; k++)
        for (int64_t i = k; i < n; i += CORR_CHUNKS)
            corr_walk(&c, i, pos + 3 * i, kind ? tvel + 3 * i : NULL, kind ? weight[i] : 1.0,
                      rows + (size_t)k * 2 * nbins);
    for (int b = 0; b < nbins; b++) {
        double s = 0.0, sw = 0.0;
        for (int k = 0; k < CORR_CHUNKS; k++) {
            s += rows[(size_t)k * 2 * nbins + b];
            sw += rows[(size_t)k * 2 * nbins + nbins + b];
        }
        binsums[b] = s;
        if (wtsums) wtsums[b] = kind ? sw : s;
    }
    free(rows);
    return 0;
}
