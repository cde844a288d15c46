/*
 * CPU oracle for the pytreegrav_gb300 hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of pytreegrav's radix octree build, moment roll-ups, grouped field walk and
 * brute-force sums, used by tests/ as the parity checker, by __graft_entry__.smoke() as the checker
 * and by bench.py as the timed CPU baseline.  The shipped library never links or calls this code.
 *
 * Parity of this restatement is pinned against fixtures generated by running pytreegrav's own
 * Python source (tests/golden/make_golden.py) -- bit-exact for keys, permutation, topology and
 * moments, and to the last ulp for the FP64 walk, which both evaluate without FMA contraction.
 */
#ifndef TG_ORACLE_H
#define TG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t npart;      /* NumParticles */
    int64_t num_nodes;  /* NumNodes: particles + node capacity, grown like octree.py:1280-1298 */
    int64_t node_hi;    /* one past the last allocated node */
    int has_quads;
    int has_coincident;
    double *coord;      /* (num_nodes, 3) */
    double *mass;       /* (num_nodes,) */
    double *size;       /* (num_nodes,) */
    double *delta;      /* (num_nodes,) */
    double *soft;       /* (num_nodes,) */
    double *quad;       /* (num_nodes, 3, 3) or NULL */
    int64_t *first;     /* FirstSubnode */
    int64_t *next;      /* NextBranch */
    int64_t *walk_idx;  /* TreewalkIndices (npart,) */
} tgo_tree;

void tgo_bounding_cube(const double *pos, int64_t n, double center[3], double *size);
void tgo_morton_keys(const double *pos, int64_t n, const double center[3], double size, int64_t *keys);
void tgo_radix_argsort(const int64_t *keys, int64_t n, int64_t *perm);
void tgo_morton_order(const double *pos, int64_t n, int64_t *perm);

/* ConstructTree(pos, m, softening, quadrupole, compute_moments) on the radix path, serial split.
 * m == NULL means zero masses and no moments (frontend.py:115-117). Returns 0 on success. */
int tgo_build(const double *pos, const double *m, const double *h, int64_t n, int quadrupole,
              int compute_moments, tgo_tree *out);
void tgo_free(tgo_tree *t);

/* FieldsTarget_grouped: pos/soft in the order the caller wants grouped (Morton order for the
 * frontend). out is (n, W) with W = pot + 3*acc + 9*tidal, packed in that order. */
int tgo_fields(const tgo_tree *t, const double *pos, const double *soft, int64_t n, int want_pot,
               int want_acc, int want_tidal, int quadrupole, int64_t group_size, double theta,
               double G, double *out, int nthreads);

/* The same walk over explicitly given groups [start[g], start[g] + count[g]) of pos. */
int tgo_fields_groups(const tgo_tree *t, const double *pos, const double *soft, const int64_t *start,
                      const int64_t *count, int64_t ngroups, int want_pot, int want_acc, int want_tidal,
                      int quadrupole, double theta, double G, double *out, int nthreads);

/* Per-group interaction and opened-node counts of the same walk, for the cost model. */
int tgo_walk_counts(const tgo_tree *t, const double *pos, const double *soft, int64_t n,
                    int64_t group_size, double theta, int64_t *n_interactions, int64_t *n_opened,
                    int nthreads);

int tgo_walk_counts_groups(const tgo_tree *t, const double *pos, const double *soft, const int64_t *start,
                           const int64_t *count, int64_t ngroups, double theta, int64_t *n_interactions,
                           int64_t *n_opened, int nthreads);

/* Column density (treewalk.py:904-1030). tgo_column_rays: the single-ray walk (904-973) of every
 * (target, ray) pair; rays (nrays, 3) unit vectors, shared by all targets when ray_stride == 0, else
 * target i's rays start at rays + i * ray_stride. out (n, nrays). tgo_column_binned: the
 * angle-binned walk (976-1030) with opening angle theta; out (n, 6). */
void tgo_column_rays(const tgo_tree *t, const double *pos, int64_t n, const double *rays, int64_t nrays,
                     int64_t ray_stride, double *out, int nthreads);
void tgo_column_binned(const tgo_tree *t, const double *pos, int64_t n, double theta, double *out, int nthreads);
/* ColumnDensityBinned_grouped (treewalk.py:1197-1294): groups of group_size consecutive targets share
 * one walk, accepting a node on its distance r_min from the group's bounding box; out (n, 6). */
void tgo_column_binned_grouped(const tgo_tree *t, const double *pos, int64_t n, double theta, int64_t group_size,
                               double *out, int nthreads);

/* Brute force.  mode 0: target form (r == 0 pairs skipped, bruteforce.py:7-50, 209-256, 353-386);
 * mode 1: mutual form (self excluded by index, bruteforce.py:86-116, 164-206, 319-350).
 * out is (nt, W) like tgo_fields. */
int tgo_bruteforce(const double *pos_t, const double *h_t, int64_t nt, const double *pos_s,
                   const double *m_s, const double *h_s, int64_t ns, int want_pot, int want_acc,
                   int want_tidal, int mode, double G, double *out, int nthreads);

/* Two-point functions (tg_oracle_corr.c): node velocities and dispersions of the DynamicOctree moment
 * pass (vel_in (n, 3) in the caller's order; vel (num_nodes, 3), disp (num_nodes)), and the density /
 * velocity-correlation / structure-function walks (kind 0 / 1 / 2) summed over targets. */
void tgo_tree_velocities(const tgo_tree *t, const double *vel_in, double *vel, double *disp);
double tgo_corr_uniform(uint64_t seed, int64_t target, int64_t draw);
int tgo_correlation(const tgo_tree *t, const double *vel, const double *disp, int kind, const double *pos,
                    const double *tvel, const double *weight, int64_t n, const double *rbins, int nbins,
                    double max_bin_size_ratio, double theta, double boxsize, int weighted_binning, uint64_t seed,
                    int absval, double *binsums, double *wtsums, int nthreads);

double tgo_force_kernel(double r, double h);
double tgo_potential_kernel(double r, double h);
double tgo_tidal_kernel(double r, double h);

#ifdef __cplusplus
}
#endif
#endif
