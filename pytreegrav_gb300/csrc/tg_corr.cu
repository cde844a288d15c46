// Node velocities and the two-point functions of a tree (declared in include/pytreegrav_gb300.h):
// pytreegrav's DynamicOctree moments (dynamic_tree.py:246-310) and its density correlation,
// velocity correlation and velocity structure functions (treewalk.py:344-818, frontend.py:1047-1320).
//
// pytreegrav builds a separate insertion tree (DynamicOctree) for the velocity functions. On inputs
// without coincident points that tree has the radix tree's topology, traversal order, cell sizes and
// masses (both split the bounding cube at cell centres, octant by octant), so here the velocities are
// attached to the radix tree: every node gets the mass-weighted mean velocity of its children and
// their mass-weighted velocity dispersion about it, rolled up level by level, deepest first, with
// each node's children taken in chain (octant) order as pytreegrav's recursion takes them.
//
// The walks are pytreegrav's stackless per-target walk over FirstSubnode/NextBranch in FP64: an
// element inside the radial range (rbins[0], rbins[-1]) is binned by log10 of its distance; a node
// is binned whole when it passes the opening test and is smaller than max_bin_size_ratio times its
// bin's width, either spread over the bins its extent overlaps (weighted_binning) or at a distance
// jittered uniformly by its size. pytreegrav draws that jitter from numba's global generator; here it
// is a counter-based hash of (seed, target, draw), so a run is reproducible from its seed. A jittered
// or spread bin index outside [0, nbins) is clamped into it (pytreegrav indexes past the array there).
//
// One thread per target, each of a fixed set of threads accumulating its targets (a fixed stride) into
// a private row of bins in device memory; rows are added per bin by a fixed-shape reduction, so the
// result does not depend on timing.
#include <cmath>
#include <cstring>
#include <new>

#include "tg_tree.cuh"

namespace tg {

namespace {

constexpr int CORR_THREADS = 128;
constexpr int CORR_RED = 256;
constexpr int MAX_DEPTH_CLIMB = 4096;

__device__ __forceinline__ double nearest_image(double x, double box) {
    if (fabs(x) > 0.5 * box) return -copysign(box - fabs(x), x);
    return x;
}

// Uniform double in [0, 1) from (seed, target, draw): splitmix64 finalisation of a Weyl sequence.
__host__ __device__ __forceinline__ double corr_uniform(uint64_t seed, int64_t target, int64_t draw) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(target + 1) + 0xD1B54A32D192ED03ull * (uint64_t)(draw + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

// Depth of every node (root 0) by climbing parent links; a climb longer than the bound sets *bad.
__global__ void k_node_depth(int64_t ntot, int64_t mtot, const int64_t *parent, int *depth, int *maxdepth, int *bad) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mtot) return;
    int d = 0;
    int64_t p = parent[ntot + j];
    while (p >= 0 && d < MAX_DEPTH_CLIMB) {
        d++;
        p = (p >= ntot && p < ntot + mtot) ? parent[p] : -1;
    }
    if (d >= MAX_DEPTH_CLIMB) atomicOr(bad, 1);
    depth[j] = d;
    atomicMax(maxdepth, d);
}

// Particle velocities in tree (walk) order, and zero dispersion for particles.
__global__ void k_gather_vel(int64_t ntot, const int64_t *walk_idx, const double *vel_in, double *vel) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntot) return;
    const int64_t o = walk_idx[i];
    vel[3 * i] = vel_in[3 * o];
    vel[3 * i + 1] = vel_in[3 * o + 1];
    vel[3 * i + 2] = vel_in[3 * o + 2];
}

// ComputeMomentsDynamic (dynamic_tree.py:246-310) for the nodes at one depth: m = sum of the
// children's masses, vel = sum(m_c v_c) / m, and the dispersion sum(m_c disp_c) + sum(m_c |v_c - vel|^2)
// over m, children in chain order, each operation rounded once. disp is per element (particles 0).
__global__ void k_vel_level(int64_t ntot, int64_t mtot, int level, const int *depth, const int64_t *first,
                            const int64_t *next, const double *mass, double *vel, double *disp) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mtot || depth[j] != level) return;
    const int64_t f = ntot + j, stop = next[f], ne = ntot + mtot;
    int64_t ch[8];
    int n = 0;
    for (int64_t c = first[f]; c != stop && c >= 0 && c < ne && n < 8; c = next[c]) ch[n++] = c;
    double m = 0.0, vx = 0.0, vy = 0.0, vz = 0.0, vd = 0.0;
    for (int q = 0; q < n; q++) {
        const int64_t c = ch[q];
        const double mc = mass[c];
        m = dadd(m, mc);
        vx = dadd(vx, dmul(mc, vel[3 * c]));
        vy = dadd(vy, dmul(mc, vel[3 * c + 1]));
        vz = dadd(vz, dmul(mc, vel[3 * c + 2]));
        vd = dadd(vd, dmul(mc, disp[c]));
    }
    vx = ddiv(vx, m);
    vy = ddiv(vy, m);
    vz = ddiv(vz, m);
    for (int q = 0; q < n; q++) {
        const int64_t c = ch[q];
        const double dx = dsub(vel[3 * c], vx), dy = dsub(vel[3 * c + 1], vy), dz = dsub(vel[3 * c + 2], vz);
        vd = dadd(vd, dmul(mass[c], dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz))));
    }
    vel[3 * f] = vx;
    vel[3 * f + 1] = vy;
    vel[3 * f + 2] = vz;
    disp[f] = ddiv(vd, m);
}

struct CorrArgs {
    int64_t ntot, nelem;
    int *runaway;
    const double *coord, *mass, *size, *delta, *vel, *disp;
    const int64_t *first, *next;
    const double *pos, *tvel, *weight;  // targets (n), their velocities and weights (kinds 1, 2)
    int64_t n;
    const double *rbins;  // nbins + 1 edges, logarithmically spaced
    int nbins;
    double mbr, theta, box;
    int weighted, kind;
    uint64_t seed;
    int nrows;
    double *rows;  // nrows x 2 nbins: bin sums, then weight sums
    // the FP32 screen: per element hi parts of the position and, for nodes, the opening radius
    // max(s / theta + delta, 0.6 s + delta) rounded to FP32 (-1 for particles); lo parts and the size
    const float4 *ehi, *elo;
    float rmin32, rmax32, lmin32, dl32, box32;
};

// Bin of distance r: int(nbins (log10 r - log10 rbins[0]) / dlogr) as pytreegrav writes it, clamped to
// [0, nbins).
__device__ __forceinline__ int bin_of(double r, double logr_min, double dlogr, int nbins) {
    const double t = ddiv(dmul((double)nbins, dsub(log10(r), logr_min)), dlogr);
    if (!(t >= 0.0)) return 0;
    if (t >= (double)nbins) return nbins - 1;
    return (int)t;
}

__device__ __forceinline__ void bin_add(double *row, int b, double x) { row[b] = dadd(row[b], x); }

// do_weighted_binning (treewalk.py:344-378): a node of half-size h at distance r spread over the bins
// its extent overlaps with weights max(0, 1 - (r - r_eff)^2 / h^2) times the overlap, normalised; each
// bin gets w * ((weight * M) * quantity) (the whole M * quantity when the extent lies inside bin r_idx).
__device__ void spread_bins(const CorrArgs &a, double *row, double r, int r_idx, double h, double M, double quantity,
                            double w) {
    const double *rb = a.rbins;
    if (dadd(r, h) < rb[r_idx + 1] && dsub(r, h) > rb[r_idx]) {
        bin_add(row, r_idx, dmul(w, dmul(M, quantity)));
        return;
    }
    const double lratio = log10(ddiv(rb[1], rb[0]));
    const double tmin = ddiv(log10(ddiv(dsub(r, h), rb[0])), lratio);
    // below 0 only bins with no overlap (r - h > 0 here); above nbins nothing to spread
    const int min_bin = tmin >= (double)a.nbins ? a.nbins : (tmin > 0.0 ? (int)tmin : 0);
    const double tmax = dadd(ddiv(log10(ddiv(dadd(r, h), rb[0])), lratio), 1.0);
    const int max_bin = tmax >= (double)a.nbins ? a.nbins : (tmax > 0.0 ? (int)tmax : 0);
    double total = 0.0;
    for (int i = min_bin; i < max_bin; i++) {
        const double i1 = fmax(dsub(r, h), rb[i]), i2 = fmin(dadd(r, h), rb[i + 1]), ov = dsub(i2, i1);
        if (ov > 0.0) {
            const double dr = fabs(dsub(r, dmul(0.5, dadd(i1, i2))));
            total = dadd(total, dmul(fmax(0.0, dsub(1.0, ddiv(dmul(dr, dr), dmul(h, h)))), ov));
        }
    }
    for (int i = min_bin; i < max_bin; i++) {
        const double i1 = fmax(dsub(r, h), rb[i]), i2 = fmin(dadd(r, h), rb[i + 1]), ov = dsub(i2, i1);
        if (ov > 0.0) {
            const double dr = fabs(dsub(r, dmul(0.5, dadd(i1, i2))));
            const double wt = ddiv(dmul(fmax(0.0, dsub(1.0, ddiv(dmul(dr, dr), dmul(h, h)))), ov), total);
            bin_add(row, i, dmul(w, dmul(dmul(wt, M), quantity)));
        }
    }
}

// Per-target state of a walk: the target, its velocity and weight, the rows it adds into, the FP64
// bin constants, and the count of jitter draws so far.
struct CorrTarget {
    int64_t i;
    double px, py, pz, w;
    double tv[3];
    double logr_min, dlogr;
    double *bins, *wts;
    int64_t draws;
};

// A particle's contribution (in bin r_idx): its mass, v . V M, or |v - V|^2 M summed over the
// components, times the target's weight (w = 1 for the density).
__device__ __forceinline__ void add_particle(const CorrArgs &a, CorrTarget &t, int64_t no, int r_idx) {
    const double M = a.mass[no];
    double amount = M;
    if (a.kind == TG_CORR_VELOCITY) {
        amount = 0.0;
        for (int k = 0; k < 3; k++) amount = dadd(amount, dmul(dmul(t.tv[k], a.vel[3 * no + k]), M));
    } else if (a.kind == TG_CORR_STRUCTURE) {
        amount = 0.0;
        for (int k = 0; k < 3; k++) {
            const double u = dsub(t.tv[k], a.vel[3 * no + k]);
            amount = dadd(amount, dmul(dmul(u, u), M));
        }
    }
    bin_add(t.bins, r_idx, dmul(t.w, amount));
    if (a.kind) bin_add(t.wts, r_idx, dmul(t.w, M));
}

// A node's quantity per unit mass: 1, v . V, or |v - V|^2 plus its dispersion.
__device__ __forceinline__ double node_q(const CorrArgs &a, const CorrTarget &t, int64_t no) {
    double q = 1.0;
    if (a.kind == TG_CORR_VELOCITY) {
        q = 0.0;
        for (int k = 0; k < 3; k++) q = dadd(q, dmul(t.tv[k], a.vel[3 * no + k]));
    } else if (a.kind == TG_CORR_STRUCTURE) {
        q = 0.0;
        for (int k = 0; k < 3; k++) {
            const double u = dsub(t.tv[k], a.vel[3 * no + k]);
            q = dadd(q, dmul(u, u));
        }
        q = dadd(q, a.disp[no]);
    }
    return q;
}

// A binned node's contribution at jittered bin j.
__device__ __forceinline__ void add_node_at(const CorrArgs &a, CorrTarget &t, int64_t no, int j) {
    const double M = a.mass[no];
    bin_add(t.bins, j, dmul(t.w, a.kind ? dmul(node_q(a, t, no), M) : M));
    if (a.kind) bin_add(t.wts, j, dmul(t.w, M));
}

// The FP64 distance from the target to element no (nearest periodic image when box > 0).
__device__ __forceinline__ double dist64(const CorrArgs &a, const CorrTarget &t, int64_t no) {
    double dx = dsub(a.coord[3 * no], t.px), dy = dsub(a.coord[3 * no + 1], t.py), dz = dsub(a.coord[3 * no + 2], t.pz);
    if (a.box > 0.0) {
        dx = nearest_image(dx, a.box);
        dy = nearest_image(dy, a.box);
        dz = nearest_image(dz, a.box);
    }
    return sqrt(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)));
}

// One element of DensityCorrWalk / VelocityCorrWalk / VelocityStructWalk (treewalk.py:380-818) in FP64,
// pytreegrav's expressions with every operation rounded once: the contributions it makes, and the
// element the walk goes to next.
__device__ int64_t elem_exact(const CorrArgs &a, CorrTarget &t, int64_t no) {
    const int nb = a.nbins;
    const double r = dist64(a, t, no);
    const bool part = no < a.ntot;
    const double s = part ? 0.0 : a.size[no], del = part ? 0.0 : a.delta[no];
    const bool far = !part && r > fmax(dadd(ddiv(s, a.theta), del), dadd(dmul(s, 0.6), del));
    if (r > a.rbins[0] && r < a.rbins[nb]) {
        const int r_idx = bin_of(r, t.logr_min, t.dlogr, nb);
        if (part) {
            add_particle(a, t, no, r_idx);
            return a.next[no];
        }
        if (far && s < dmul(a.mbr, dsub(a.rbins[r_idx + 1], a.rbins[r_idx]))) {
            const double M = a.mass[no];
            if (a.weighted) {
                const double q = node_q(a, t, no);
                spread_bins(a, t.bins, r, r_idx, dmul(0.5, s), M, q, t.w);
                if (a.kind) spread_bins(a, t.wts, r, r_idx, dmul(0.5, s), M, 1.0, t.w);
            } else {
                const double rnew = dadd(r, dmul(dsub(corr_uniform(a.seed, t.i, t.draws++), 0.5), s));
                add_node_at(a, t, no, rnew > 0.0 ? bin_of(rnew, t.logr_min, t.dlogr, nb) : 0);
            }
            return a.next[no];
        }
        return a.first[no];
    }
    return (part || far) ? a.next[no] : a.first[no];
}

// x against threshold c known to within e: +1 above, -1 below, 0 undecided.
__device__ __forceinline__ int side(float x, float c, float e) { return x > c + e ? 1 : (x < c - e ? -1 : 0); }

// The bin of distance r (FP32, relative error below er / r) when the FP32 value of pytreegrav's bin
// formula is farther than its error bound from a bin edge (the clamps included); -1 otherwise.
__device__ __forceinline__ int bin_screen(const CorrArgs &a, float r, float er) {
    const float lr = log10f(r);
    const float tscale = (float)a.nbins / a.dl32;
    const float t = __fdiv_rn(__fmul_rn((float)a.nbins, __fsub_rn(lr, a.lmin32)), a.dl32);
    // log10f (a few ulp), the FP32 constants and r's own error, with a factor of 4 to spare
    const float dt = tscale * (4e-6f * (1.f + fabsf(lr) + fabsf(a.lmin32)) + 2.f * er / r);
    if (!(r > 0.f) || !(dt < 0.25f)) return -1;
    if (t < -dt) return 0;
    if (t - dt >= (float)a.nbins) return a.nbins - 1;
    const float fl = floorf(t);
    if (t - fl > dt && fl + 1.f - t > dt && fl >= 0.f && fl < (float)a.nbins) return (int)fl;
    return -1;
}

// The walk of target i (treewalk.py:380-818). Every decision -- inside the radial range, the opening
// test, the bin, a jittered node's bin -- is first taken in FP32 from hi/lo positions when the FP32
// value lies farther from its threshold than a bound on its error; otherwise (and for weighted
// binning) the element is evaluated by elem_exact. So the decisions are pytreegrav's FP64 ones, and
// GB300 (FP64 at 1/73 of the FP32 rate) spends FP64 only on the sums. Contributions add into row
// (bin sums at row[0..nbins), weight sums at row[nbins..2 nbins), kinds 1 and 2 only), each formed in
// pytreegrav's order of operations and multiplied by the target's weight (pytreegrav multiplies the
// target's per-bin sums instead, which differs in rounding only).
__device__ void corr_walk(const CorrArgs &a, int64_t i, double *row) {
    const int64_t N = a.ntot;
    const int nb = a.nbins;
    CorrTarget t;
    t.i = i;
    t.px = a.pos[3 * i];
    t.py = a.pos[3 * i + 1];
    t.pz = a.pos[3 * i + 2];
    t.tv[0] = t.tv[1] = t.tv[2] = 0.0;
    if (a.kind) {
        t.tv[0] = a.tvel[3 * i];
        t.tv[1] = a.tvel[3 * i + 1];
        t.tv[2] = a.tvel[3 * i + 2];
    }
    t.w = a.kind ? a.weight[i] : 1.0;
    t.logr_min = log10(a.rbins[0]);
    t.dlogr = dsub(log10(a.rbins[nb]), t.logr_min);
    t.bins = row;
    t.wts = row + nb;
    t.draws = 0;
    float phx, plx, phy, ply, phz, plz;
    d2f_split(t.px, phx, plx);
    d2f_split(t.py, phy, ply);
    d2f_split(t.pz, phz, plz);
    const float box = a.box32, half = 0.5f * a.box32;
    // the hi/lo splits keep positions to ~2^-48 of their size: an absolute error term for very close pairs
    const float eabs = 1e-12f * (fabsf(phx) + fabsf(phy) + fabsf(phz)) + 1e-30f;
    int64_t no = N;
    for (int64_t guard = 0; no > -1; guard++) {
        if (guard > a.nelem || no >= a.nelem) {  // one visit per element always suffices
            atomicOr(a.runaway, 1);
            return;
        }
        const float4 h = a.ehi[no], l = a.elo[no];
        float d[3] = {__fadd_rn(__fsub_rn(h.x, phx), __fsub_rn(l.x, plx)),
                      __fadd_rn(__fsub_rn(h.y, phy), __fsub_rn(l.y, ply)),
                      __fadd_rn(__fsub_rn(h.z, phz), __fsub_rn(l.z, plz))};
        bool sure = true;
        if (a.box > 0.0) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float ad = fabsf(d[k]);
                const int sd = side(ad, half, 1e-6f * box);
                if (sd == 0) sure = false;
                else if (sd > 0) d[k] = -copysignf(__fsub_rn(box, ad), d[k]);
            }
        }
        const float r = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
        // hi/lo offsets (~1e-7 relative), the nearest image, the squares and the root
        const float er = 2e-6f * (r + box) + 1e-12f * (fabsf(h.x) + fabsf(h.y) + fabsf(h.z)) + eabs;
        const bool part = no < N;
        const int inlo = side(r, a.rmin32, er + 2e-7f * a.rmin32), inhi = side(r, a.rmax32, er + 2e-7f * a.rmax32);
        const int fs = part ? -1 : side(r, h.w, er + 2e-7f * h.w);  // far: r > opening radius
        if (!sure || inlo == 0 || inhi == 0 || fs == 0 || a.weighted) {
            no = elem_exact(a, t, no);
            continue;
        }
        if (inlo > 0 && inhi < 0) {  // inside (rbins[0], rbins[-1])
            const int r_idx = bin_screen(a, r, er);
            if (r_idx < 0) {
                no = elem_exact(a, t, no);
                continue;
            }
            if (part) {
                add_particle(a, t, no, r_idx);
                no = a.next[no];
            } else if (fs > 0 && a.size[no] < dmul(a.mbr, dsub(a.rbins[r_idx + 1], a.rbins[r_idx]))) {
                // jittered distance r + (u - 0.5) s: its bin in FP32 when clear of the edges
                const double u = corr_uniform(a.seed, i, t.draws);
                const float rn = __fadd_rn(r, __fmul_rn((float)(u - 0.5), l.w));
                const int j = rn > 4.f * er ? bin_screen(a, rn, er + 1e-6f * l.w) : -1;
                if (j >= 0) {
                    t.draws++;
                    add_node_at(a, t, no, j);
                } else {  // the FP64 distance, then pytreegrav's expression
                    const double r64 = dist64(a, t, no);
                    const double rnew = dadd(r64, dmul(dsub(corr_uniform(a.seed, i, t.draws++), 0.5), a.size[no]));
                    add_node_at(a, t, no, rnew > 0.0 ? bin_of(rnew, t.logr_min, t.dlogr, nb) : 0);
                }
                no = a.next[no];
            } else {
                no = a.first[no];
            }
        } else {
            no = (part || fs > 0) ? a.next[no] : a.first[no];
        }
    }
}

// FP32 element records of the screen: hi/lo position, the node's opening radius (pytreegrav's
// max(s / theta + delta, 0.6 s + delta), formed in FP64 and rounded) or -1, the size.
__global__ void k_corr_prep(int64_t ntot, int64_t nelem, const double *coord, const double *size, const double *delta,
                            double theta, float4 *ehi, float4 *elo) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    float hx, lx, hy, ly, hz, lz;
    d2f_split(coord[3 * e], hx, lx);
    d2f_split(coord[3 * e + 1], hy, ly);
    d2f_split(coord[3 * e + 2], hz, lz);
    float crit = -1.f, s32 = 0.f;
    if (e >= ntot) {
        const double s = size[e], del = delta[e];
        crit = d2f(fmax(dadd(ddiv(s, theta), del), dadd(dmul(s, 0.6), del)));
        s32 = d2f(s);
    }
    ehi[e] = make_float4(hx, hy, hz, crit);
    elo[e] = make_float4(lx, ly, lz, s32);
}

__global__ void __launch_bounds__(CORR_THREADS) k_corr(CorrArgs a) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= a.nrows) return;
    double *row = a.rows + (int64_t)tid * 2 * a.nbins;
    for (int b = 0; b < 2 * a.nbins; b++) row[b] = 0.0;
    for (int64_t i = tid; i < a.n; i += a.nrows) corr_walk(a, i, row);
}

// One block per output value (bin sums, then weight sums): thread t adds rows t, t + CORR_RED, ...
// in order, then a fixed-shape tree adds the threads' sums.
__global__ void __launch_bounds__(CORR_RED) k_corr_reduce(const double *rows, int nrows, int nbins, double *out) {
    __shared__ double sh[CORR_RED];
    const int b = blockIdx.x, t = threadIdx.x;
    double s = 0.0;
    for (int r = t; r < nrows; r += CORR_RED) s += rows[(int64_t)r * 2 * nbins + b];
    sh[t] = s;
    __syncthreads();
    for (int w = CORR_RED / 2; w > 0; w >>= 1) {
        if (t < w) sh[t] += sh[t + w];
        __syncthreads();
    }
    if (t == 0) out[b] = sh[0];
}

}  // namespace
}  // namespace tg

using namespace tg;

extern "C" {

tg_status tg_tree_set_velocities(tg_tree t, const double *vel, int mem, void *stream) {
    if (!t || !vel || (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE)) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    const int64_t N = t->ntot, M = t->mtot, NE = N + M;
    DevArray<double> staged(st);
    const double *dv = vel;
    if (mem == TG_MEM_HOST) {
        TG_CUDA(staged.alloc(3 * N));
        TG_CUDA(cudaMemcpyAsync(staged.p, vel, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st));
        dv = staged.p;
    }
    if (!t->vel) TG_CUDA(dev_malloc((void **)&t->vel, sizeof(double) * 3 * NE, st));
    if (!t->vdisp) TG_CUDA(dev_malloc((void **)&t->vdisp, sizeof(double) * NE, st));
    TG_CUDA(cudaMemsetAsync(t->vdisp, 0, sizeof(double) * NE, st));
    { k_gather_vel<<<div_up(N, 256), 256, 0, st>>>(N, t->walk_idx, dv, t->vel); note_launch(); }
    DevArray<int> depth(st), flags(st);
    TG_CUDA(depth.alloc(M));
    TG_CUDA(flags.alloc(2));
    TG_CUDA(cudaMemsetAsync(flags.p, 0, 2 * sizeof(int), st));
    if (M > 0) { k_node_depth<<<div_up(M, 256), 256, 0, st>>>(N, M, t->parent, depth.p, flags.p, flags.p + 1); note_launch(); }
    TG_CUDA(cudaGetLastError());
    int hf[2] = {0, 0};
    TG_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    if (hf[1]) {
        set_last_error_msg("node velocities: a node's parent chain is longer than any octree's");
        return TG_ERR_ITER_LIMIT;
    }
    for (int d = hf[0]; d >= 0; d--) {
        k_vel_level<<<div_up(M, 256), 256, 0, st>>>(N, M, d, depth.p, t->first, t->next, t->mass, t->vel, t->vdisp);
        note_launch();
    }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

tg_status tg_tree_copy_velocities(tg_tree t, double *vel, double *vdisp, void *stream) {
    if (!t || !t->vel) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t NE = t->ntot + t->mtot;
    const int64_t cap = t->nsys == 1 ? t->sys_capacity[0] : NE;
    if (vel) {
        TG_CUDA(cudaMemcpyAsync(vel, t->vel, sizeof(double) * 3 * NE, cudaMemcpyDeviceToHost, st));
    }
    if (vdisp) TG_CUDA(cudaMemcpyAsync(vdisp, t->vdisp, sizeof(double) * NE, cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    for (int64_t i = NE; i < cap; i++) {
        if (vel) vel[3 * i] = vel[3 * i + 1] = vel[3 * i + 2] = 0.0;
        if (vdisp) vdisp[i] = 0.0;
    }
    return TG_OK;
}

tg_status tg_tree_correlation(tg_tree t, int kind, const double *pos, const double *vel, const double *weight,
                              int64_t n, const double *rbins, int nbins, double max_bin_size_ratio, double theta,
                              double boxsize, int weighted_binning, uint64_t seed, int mem, double *binsums,
                              double *wtsums, void *stream) {
    const bool own = pos == nullptr;  // the tree's own particles, in tree order, with their velocities and masses
    if (t && own) n = t->ntot;
    if (!t || n < 0 || !rbins || nbins < 1 || nbins > TG_CORR_MAX_BINS || !binsums ||
        (kind != TG_CORR_DENSITY && kind != TG_CORR_VELOCITY && kind != TG_CORR_STRUCTURE) || !(theta > 0) ||
        !(boxsize >= 0) || (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE))
        return TG_ERR_BAD_ARG;
    if (kind != TG_CORR_DENSITY && (!wtsums || (!own && (!vel || !weight)))) return TG_ERR_BAD_ARG;
    if (kind != TG_CORR_DENSITY && !t->vel) {
        set_last_error_msg("velocity functions need a tree with velocities (tg_tree_set_velocities)");
        return TG_ERR_BAD_ARG;
    }
    if (t->nsys != 1) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const bool host = mem == TG_MEM_HOST;
    if (n == 0) {  // no targets: empty sums
        for (double *o : {binsums, wtsums}) {
            if (!o) continue;
            if (host) memset(o, 0, sizeof(double) * nbins);
            else TG_CUDA(cudaMemsetAsync(o, 0, sizeof(double) * nbins, st));
        }
        TG_CUDA(cudaStreamSynchronize(st));
        return TG_OK;
    }
    tree_wait_built(t, st);
    DevArray<double> dpos(st), dvel(st), dw(st), drb(st), rows(st), dout(st);
    auto stage = [&](DevArray<double> &d, const double *src, int64_t count, const double *&p) -> tg_status {
        if (!src) {
            p = nullptr;
            return TG_OK;
        }
        if (!host) {
            p = src;
            return TG_OK;
        }
        TG_CUDA(d.alloc(count));
        TG_CUDA(cudaMemcpyAsync(d.p, src, sizeof(double) * count, cudaMemcpyHostToDevice, st));
        p = d.p;
        return TG_OK;
    };
    CorrArgs a;
    a.ntot = t->ntot;
    a.nelem = t->ntot + t->mtot;
    DevArray<int> runaway(st);
    TG_CUDA(runaway.alloc(1));
    TG_CUDA(cudaMemsetAsync(runaway.p, 0, sizeof(int), st));
    a.runaway = runaway.p;
    a.coord = t->coord; a.mass = t->mass; a.size = t->size; a.delta = t->delta; a.vel = t->vel; a.disp = t->vdisp;
    a.first = t->first; a.next = t->next;
    if (own) {
        a.pos = t->coord;
        a.tvel = kind ? t->vel : nullptr;
        a.weight = kind ? t->mass : nullptr;
    } else {
        TG_TRY(stage(dpos, pos, 3 * n, a.pos));
        TG_TRY(stage(dvel, kind ? vel : nullptr, 3 * n, a.tvel));
        TG_TRY(stage(dw, kind ? weight : nullptr, n, a.weight));
    }
    TG_TRY(stage(drb, rbins, nbins + 1, a.rbins));
    a.n = n;
    a.nbins = nbins;
    a.mbr = max_bin_size_ratio;
    a.theta = theta;
    a.box = boxsize;
    a.weighted = weighted_binning ? 1 : 0;
    a.kind = kind;
    a.seed = seed;
    // a fixed number of rows (threads), bounded so that the rows stay within 512 MB
    const int64_t per_row = 2 * (int64_t)nbins * (int64_t)sizeof(double);
    int64_t nrows = std::min<int64_t>((int64_t)num_sms() * 4 * CORR_THREADS, ((int64_t)1 << 29) / per_row);
    nrows = std::max<int64_t>(1, std::min<int64_t>(nrows, std::max<int64_t>(n, 1)));
    a.nrows = (int)nrows;
    TG_CUDA(rows.alloc(nrows * 2 * nbins));
    a.rows = rows.p;
    TG_CUDA(dout.alloc(2 * nbins));
    DevArray<float4> ehi(st), elo(st);
    TG_CUDA(ehi.alloc(a.nelem));
    TG_CUDA(elo.alloc(a.nelem));
    { k_corr_prep<<<div_up(a.nelem, 256), 256, 0, st>>>(t->ntot, a.nelem, t->coord, t->size, t->delta, theta, ehi.p,
                                                          elo.p); note_launch(); }
    a.ehi = ehi.p;
    a.elo = elo.p;
    {  // FP32 copies of the radial range for the screen (its error bounds cover their rounding)
        double rb0 = 0.0, rbn = 0.0;
        if (host) {
            rb0 = rbins[0];
            rbn = rbins[nbins];
        } else {
            TG_CUDA(cudaMemcpyAsync(&rb0, rbins, sizeof(double), cudaMemcpyDeviceToHost, st));
            TG_CUDA(cudaMemcpyAsync(&rbn, rbins + nbins, sizeof(double), cudaMemcpyDeviceToHost, st));
            TG_CUDA(cudaStreamSynchronize(st));
        }
        a.rmin32 = (float)rb0;
        a.rmax32 = (float)rbn;
        a.lmin32 = (float)std::log10(rb0);
        a.dl32 = (float)(std::log10(rbn) - std::log10(rb0));
        a.box32 = (float)boxsize;
    }
    { k_corr<<<div_up(nrows, CORR_THREADS), CORR_THREADS, 0, st>>>(a); note_launch(); }
    { k_corr_reduce<<<2 * nbins, CORR_RED, 0, st>>>(rows.p, a.nrows, nbins, dout.p); note_launch(); }
    TG_CUDA(cudaGetLastError());
    const cudaMemcpyKind kd = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    TG_CUDA(cudaMemcpyAsync(binsums, dout.p, sizeof(double) * nbins, kd, st));
    if (wtsums) TG_CUDA(cudaMemcpyAsync(wtsums, dout.p + (kind ? nbins : 0), sizeof(double) * nbins, kd, st));
    int hr = 0;
    TG_CUDA(cudaMemcpyAsync(&hr, runaway.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    if (hr) {
        set_last_error_msg("correlation walk did not end within one visit per element");
        return TG_ERR_ITER_LIMIT;
    }
    return TG_OK;
}

}  // extern "C"
