// Column density through the octree: pytreegrav's ray-traced and angle-binned walks
// (treewalk.py:904-1030, frontend.py:1321-1458) over the tree's FP64 arrays, in the reference's order
// of operations with every operation rounded once (explicit _rn intrinsics, no FMA contraction).
//
// The ray-traced walk has no truncation: a node opens whenever its bounding sphere, inflated by its
// largest particle radius, can meet the ray, and only particles contribute, each as a uniform sphere
// of its mass and radius (the softening). One thread walks one (target, ray) pair; lanes of a warp
// take consecutive targets (Morton order) for the same ray, so their walks stay together.
#include "tg_tree.cuh"

namespace tg {
namespace {

constexpr double FAC_DENSITY = 3.0 / (4.0 * 3.141592653589793);  // 3 / (4 pi), as numpy evaluates it
constexpr double FOUR_PI = 4.0 * 3.141592653589793;
constexpr double BIN_SOLID_ANGLE = (4.0 * 3.141592653589793) / 6.0;  // angular_bin_size

struct ColumnTree {
    const double *coord, *mass, *soft, *size, *delta;
    const int64_t *first, *next;
    int64_t npart, nelem;
    int64_t max_visits;  // visits one walk may make (one per element always suffices)
    // FP32 copy for the screen: coordinates split hi + lo, with the radius (hi.w) and, for nodes,
    // size * sqrt(3)/2 + delta (lo.w)
    const float4 *fhi, *flo;
    // output row of target i: rows[i] (the targets are the tree's own particles, results go back to
    // the caller's order), or i when null
    const int64_t *rows = nullptr;
    __device__ int64_t row(int64_t i) const { return rows ? rows[i] : i; }
};

__device__ __forceinline__ void split_f(double v, float &hi, float &lo) { d2f_split(v, hi, lo); }

__global__ void k_column_prep(ColumnTree t, float4 *fhi, float4 *flo) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= t.nelem) return;
    float4 a, b;
    split_f(t.coord[3 * e], a.x, b.x);
    split_f(t.coord[3 * e + 1], a.y, b.y);
    split_f(t.coord[3 * e + 2], a.z, b.z);
    a.w = d2f(t.soft[e]);
    b.w = e < t.npart ? 0.f : (float)(t.size[e] * 0.8660254037844386 + t.delta[e]);
    fhi[e] = a;
    flo[e] = b;
}

// ColumnDensityWalk_singleray (treewalk.py:904-973). Each visited element is first screened in FP32
// from its FP64 offset: distance r, along-ray coordinate z and impact parameter b (from |d x n|,
// which does not cancel). Their FP32 errors are a few 1e-7 of r, so with a margin of 4e-6 r the
// screen's "certainly" answers are the FP64 decisions. The element is evaluated in FP64, in the
// reference's order, only when its particle may contribute or a decision is within the margin,
// including the reference's skip of elements whose r^2 - z^2 rounds below zero. *runaway is set if
// the walk does not end within one visit per element (a malformed tree).
__device__ double column_singleray(const ColumnTree &t, double px, double py, double pz, double r0, double r1,
                                   double r2d, int *runaway) {
    const int64_t N = t.npart;
    const float n0 = (float)r0, n1 = (float)r1, n2 = (float)r2d;
    float phx, phy, phz, plx, ply, plz;
    split_f(px, phx, plx);
    split_f(py, phy, ply);
    split_f(pz, phz, plz);
    // absolute part of the margin: the lo parts' own rounding
    const float m_abs = 1e-13f * (fabsf(phx) + fabsf(phy) + fabsf(phz)) + 1e-30f;
    double column = 0.0;
    int64_t no = N;
    const int64_t stop = t.next[N];
    for (int64_t guard = 0; no > -1 && no != stop; guard++) {
        if (guard > t.max_visits || no >= t.nelem) {
            atomicOr(runaway, 1);
            return column;
        }
        // FP32 screen
        {
            const float4 ah = t.fhi[no], al = t.flo[no];
            const float fx = (ah.x - phx) + (al.x - plx), fy = (ah.y - phy) + (al.y - ply);
            const float fz = (ah.z - phz) + (al.z - plz), hf = ah.w;
            const float rf = sqrtf(fx * fx + fy * fy + fz * fz);
            const float zf = n0 * fx + n1 * fy + n2 * fz;
            const float cx = n1 * fz - n2 * fy, cy = n2 * fx - n0 * fz, cz = n0 * fy - n1 * fx;
            const float bf = sqrtf(cx * cx + cy * cy + cz * cz);
            const float m = 4e-6f * rf + m_abs;  // error margin of r, z and b
            bool decided = false;
            int64_t nxt = -1;
            if (no < N) {
                // no contribution: a point-like particle, or one the ray certainly misses (which also
                // makes r^2 - z^2 certainly positive)
                if (!(hf > 0.f) && !(t.soft[no] > 0.0)) {  // no cross-section
                    decided = true;
                    nxt = t.next[no];
                } else if (bf - m > hf * 1.000001f) {
                    decided = true;
                    nxt = t.next[no];
                }
            } else if (bf > m) {  // r^2 - z^2 certainly positive: the node test decides
                const float Rf = al.w;
                const float near = hf + Rf;
                if (rf + m < near * 0.999999f) {  // contains the target's neighbourhood: open
                    decided = true;
                    nxt = t.first[no];
                } else if (rf - m > near * 1.000001f) {
                    const float reach = near;  // Softenings[no] + R_eff
                    if (zf < -m || bf - m > reach * 1.000001f) {  // behind the target or missed: skip
                        decided = true;
                        nxt = t.next[no];
                    } else if (zf > m && bf + m < reach * 0.999999f) {  // ahead and hit: open
                        decided = true;
                        nxt = t.first[no];
                    }
                }
            }
            if (decided) {
                no = nxt;
                continue;
            }
        }
        // FP64, the reference's expression
        const double dx = dsub(t.coord[3 * no], px), dy = dsub(t.coord[3 * no + 1], py);
        const double dz = dsub(t.coord[3 * no + 2], pz);
        const double h_no = t.soft[no];
        const double r2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
        const double r = __dsqrt_rn(r2);
        const double z = dadd(dadd(dmul(r0, dx), dmul(r1, dy)), dmul(r2d, dz));
        const double b2 = dsub(r2, dmul(z, z));
        if (b2 < 0.0) {
            no = t.next[no];
            continue;
        }
        if (no < N) {
            if (h_no > 0.0) {
                const double h_inv = ddiv(1.0, h_no);
                const double fac = dmul(dmul(dmul(FAC_DENSITY, t.mass[no]), h_inv), h_inv);
                const double r_proj = __dsqrt_rn(b2);
                const double q = dmul(r_proj, h_inv);
                if (r_proj < h_no) {
                    if (r > h_no) {
                        if (z > 0.0) column = dadd(column, dmul(dmul(fac, 2.0), __dsqrt_rn(dsub(1.0, dmul(q, q)))));
                    } else {
                        const double dzh = dmul(z, h_inv);
                        column = dadd(column, dmul(fac, dadd(dzh, __dsqrt_rn(dsub(1.0, dmul(q, q))))));
                    }
                }
            }
            no = t.next[no];
        } else {
            const double R_eff = dadd(dmul(t.size[no], 0.8660254037844386), t.delta[no]);
            bool open = false;
            if (r < dadd(h_no, R_eff)) {
                open = true;
            } else if (z > 0.0) {
                const double reach = dadd(t.soft[no], R_eff);
                open = b2 < dmul(reach, reach);
            }
            no = open ? t.first[no] : t.next[no];
        }
    }
    return column;
}

// rays shared by all targets (ray_stride 0) or per target (ray_stride 3 * nrays): pair p is
// target p % n on ray p / n
__global__ void k_column_rays(ColumnTree t, const double *pos, int64_t n, const double *rays, int64_t nrays,
                              int64_t ray_stride, double *out, int *runaway) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n * nrays) return;
    const int64_t i = p % n, j = p / n;
    const double *ray = rays + i * ray_stride + 3 * j;
    out[t.row(i) * nrays + j] = column_singleray(t, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], ray[0], ray[1],
                                                 ray[2], runaway);
}

// angular_bin (treewalk.py:49-70)
__device__ __forceinline__ int angular_bin(double dx, double dy, double dz) {
    if (fabs(dx) > fabs(dy) && fabs(dx) > fabs(dz)) return dx > 0.0 ? 0 : 1;
    if (fabs(dy) > fabs(dz)) return dy > 0.0 ? 2 : 3;
    return dz > 0.0 ? 4 : 5;
}

// ColumnDensityWalk_binned (treewalk.py:976-1030): one thread per target, six sky bins.
__global__ void k_column_binned(ColumnTree t, const double *pos, int64_t n, double theta, double *out,
                                int *runaway) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
    double col[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int64_t N = t.npart;
    int64_t no = N;
    const int64_t stop = t.next[N];
    for (int64_t guard = 0; no > -1 && no != stop; guard++) {
        if (guard > t.max_visits || no >= t.nelem) {
            atomicOr(runaway, 1);
            break;
        }
        const double dx = dsub(t.coord[3 * no], px), dy = dsub(t.coord[3 * no + 1], py);
        const double dz = dsub(t.coord[3 * no + 2], pz);
        const double r2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
        const double h = t.soft[no];
        if (no < N) {
            const int bin = angular_bin(dx, dy, dz);
            if (r2 > dmul(h, h)) {
                const double c = ddiv(ddiv(t.mass[no], r2), BIN_SOLID_ANGLE);
#pragma unroll
                for (int k = 0; k < 6; k++)
                    if (k == bin) col[k] = dadd(col[k], c);
            } else if (h > 0.0) {
                const double col0 = dmul(t.mass[no], ddiv(3.0, dmul(dmul(FOUR_PI, h), h)));
                const double fac = ddiv(__dsqrt_rn(r2), h);
                const double iso = dmul(dsub(1.0, fac), col0);
                const double peak = dmul(dmul(col0, fac), 2.0);
#pragma unroll
                for (int k = 0; k < 6; k++) {
                    col[k] = dadd(col[k], iso);
                    if (k == bin) col[k] = dadd(col[k], peak);
                }
            }
            no = t.next[no];
        } else {
            const double size = t.size[no], delta = t.delta[no];
            const double crit = pymax(dadd(ddiv(size, theta), delta), dadd(dadd(h, dmul(size, 0.6)), delta));
            if (__dsqrt_rn(r2) > crit) {
                const double c = ddiv(ddiv(t.mass[no], r2), BIN_SOLID_ANGLE);
                const int bin = angular_bin(dx, dy, dz);
#pragma unroll
                for (int k = 0; k < 6; k++)
                    if (k == bin) col[k] = dadd(col[k], c);
                no = t.next[no];
            } else {
                no = t.first[no];
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) out[6 * t.row(i) + k] = col[k];
}

// ColumnDensityBinned_grouped (treewalk.py:1197-1294): one warp per group of gsz (<= 32)
// consecutive targets, lane k holding target k. The group's bounding box decides every node for all
// its targets, so the warp walks one path; each lane adds its own target's share of every accepted
// node and particle, in the walk's order.
__global__ void k_column_binned_grouped(ColumnTree t, const double *pos, int64_t n, double theta, int gsz,
                                        double *out, int *runaway) {
    const int64_t a = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * gsz;
    const int lane = threadIdx.x & 31;
    if (a >= n) return;  // whole warps leave together
    const int cnt = (int)(n - a < (int64_t)gsz ? n - a : (int64_t)gsz);
    const bool mine = lane < cnt;
    const int64_t ti = a + (mine ? lane : 0);
    const double px = pos[3 * ti], py = pos[3 * ti + 1], pz = pos[3 * ti + 2];
    double bmin[3] = {px, py, pz}, bmax[3] = {px, py, pz};
#pragma unroll
    for (int o = 16; o; o >>= 1)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            bmin[k] = fmin(bmin[k], __shfl_xor_sync(FULL, bmin[k], o));
            bmax[k] = fmax(bmax[k], __shfl_xor_sync(FULL, bmax[k], o));
        }
    double col[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int64_t N = t.npart;
    int64_t no = N;
    const int64_t stop = t.next[N];
    for (int64_t guard = 0; no > -1 && no != stop; guard++) {
        if (guard > t.max_visits || no >= t.nelem) {
            if (lane == 0) atomicOr(runaway, 1);
            break;
        }
        const double cx = t.coord[3 * no], cy = t.coord[3 * no + 1], cz = t.coord[3 * no + 2];
        const double h_no = t.soft[no], M = t.mass[no];
        if (no < N) {
            const double hh = dmul(h_no, h_no);
            const double d0 = dsub(cx, px), d1 = dsub(cy, py), d2 = dsub(cz, pz);
            const double r2 = dadd(dadd(dmul(d0, d0), dmul(d1, d1)), dmul(d2, d2));
            const int bin = angular_bin(d0, d1, d2);
            if (r2 > hh) {
                const double c = ddiv(ddiv(M, r2), BIN_SOLID_ANGLE);
#pragma unroll
                for (int k = 0; k < 6; k++)
                    if (k == bin) col[k] = dadd(col[k], c);
            } else if (h_no > 0.0) {
                const double col0 = dmul(M, ddiv(3.0, dmul(FOUR_PI, hh)));
                const double fac = ddiv(__dsqrt_rn(r2), h_no);
                const double iso = dmul(dsub(1.0, fac), col0);
                const double peak = dmul(dmul(col0, fac), 2.0);
#pragma unroll
                for (int k = 0; k < 6; k++) {
                    col[k] = dadd(col[k], iso);
                    if (k == bin) col[k] = dadd(col[k], peak);
                }
            }
            no = t.next[no];
        } else {
            const double c3[3] = {cx, cy, cz};
            double dm[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                dm[k] = 0.0;
                if (c3[k] < bmin[k]) dm[k] = dsub(bmin[k], c3[k]);
                else if (c3[k] > bmax[k]) dm[k] = dsub(c3[k], bmax[k]);
            }
            const double r_min = __dsqrt_rn(dadd(dadd(dmul(dm[0], dm[0]), dmul(dm[1], dm[1])), dmul(dm[2], dm[2])));
            const double size = t.size[no], delta = t.delta[no];
            const double crit = pymax(dadd(ddiv(size, theta), delta), dadd(dadd(h_no, dmul(size, 0.6)), delta));
            if (r_min > crit) {  // the same answer on every lane
                const double d0 = dsub(cx, px), d1 = dsub(cy, py), d2 = dsub(cz, pz);
                const double r2 = dadd(dadd(dmul(d0, d0), dmul(d1, d1)), dmul(d2, d2));
                const double c = ddiv(ddiv(M, r2), BIN_SOLID_ANGLE);
                const int bin = angular_bin(d0, d1, d2);
#pragma unroll
                for (int k = 0; k < 6; k++)
                    if (k == bin) col[k] = dadd(col[k], c);
                no = t.next[no];
            } else {
                no = t.first[no];
            }
        }
    }
    if (mine)
#pragma unroll
        for (int k = 0; k < 6; k++) out[6 * t.row(ti) + k] = col[k];
}

}  // namespace
}  // namespace tg

using namespace tg;

extern "C" {

tg_status tg_tree_column_density(tg_tree t, const double *pos, int64_t n, const double *rays, int64_t nrays,
                                 int64_t ray_stride, int binned, double theta, int group_size, int mem, double *out,
                                 void *stream) {
    if (!t || !out || n < 0) return TG_ERR_BAD_ARG;
    const bool own = !pos;  // the tree's own particles, results in the caller's order
    if (own && n != t->ntot) return TG_ERR_BAD_ARG;
    if (binned && (group_size < 0 || group_size > 32)) return TG_ERR_BAD_ARG;
    if (mem != TG_MEM_HOST && mem != TG_MEM_DEVICE) return TG_ERR_BAD_ARG;
    if (binned) {
        if (!(theta > 0)) return TG_ERR_BAD_ARG;
        nrays = 6;
        ray_stride = 0;
    } else if (!rays || nrays < 1 || (ray_stride != 0 && ray_stride != 3 * nrays)) {
        return TG_ERR_BAD_ARG;
    }
    if (t->nsys != 1) {
        set_last_error_msg("column density needs a tree of one particle system");
        return TG_ERR_BAD_ARG;
    }
    if (n == 0) return TG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    ColumnTree ct;
    ct.coord = t->coord; ct.mass = t->mass; ct.soft = t->soft; ct.size = t->size; ct.delta = t->delta;
    ct.first = t->first; ct.next = t->next;
    ct.npart = t->ntot;
    ct.nelem = t->ntot + t->mtot;
    ct.max_visits = loop_limits().column_visits > 0 ? std::min<int64_t>(loop_limits().column_visits, ct.nelem) : ct.nelem;
    ct.rows = own ? t->walk_idx : nullptr;
    const int64_t nray_vals = binned ? 0 : (ray_stride ? n * ray_stride : 3 * nrays);
    const double *dpos = pos, *drays = rays;
    double *dout = out, *owned = nullptr;
    int *flag = nullptr;
    // one allocation: flag, positions, rays and output when they come from or go to the host
    size_t bytes = 16;
    if (mem == TG_MEM_HOST) bytes += sizeof(double) * ((own ? 0 : 3 * n) + nray_vals + n * nrays);
    TG_CUDA(dev_malloc((void **)&owned, bytes, st));
    flag = (int *)owned;
    TG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    if (own) dpos = t->coord;  // rows [0, N) of the arena: the particles in walk order
    if (mem == TG_MEM_HOST) {
        double *p = owned + 2;
        if (!own) {
            TG_CUDA(cudaMemcpyAsync(p, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
            dpos = p;
            p += 3 * n;
        }
        if (nray_vals) {
            TG_CUDA(cudaMemcpyAsync(p, rays, sizeof(double) * nray_vals, cudaMemcpyHostToDevice, st));
            drays = p;
            p += nray_vals;
        }
        dout = p;
    }
    float4 *fcopy = nullptr;
    ct.fhi = ct.flo = nullptr;
    if (binned && group_size >= 1) {
        const int64_t ngroups = (n + group_size - 1) / group_size;
        k_column_binned_grouped<<<div_up(ngroups * 32, 128), 128, 0, st>>>(ct, dpos, n, theta, group_size, dout, flag);
        note_launch();
    } else if (binned) {
        k_column_binned<<<div_up(n, 128), 128, 0, st>>>(ct, dpos, n, theta, dout, flag);
        note_launch();
    } else {
        TG_CUDA(dev_malloc((void **)&fcopy, sizeof(float4) * 2 * ct.nelem, st));
        ct.fhi = fcopy;
        ct.flo = fcopy + ct.nelem;
        k_column_prep<<<div_up(ct.nelem, 256), 256, 0, st>>>(ct, fcopy, fcopy + ct.nelem);
        note_launch();
        k_column_rays<<<div_up(n * nrays, 128), 128, 0, st>>>(ct, dpos, n, drays, nrays, ray_stride, dout, flag);
        note_launch();
    }
    TG_CUDA(cudaGetLastError());
    int hflag = 0;
    if (mem == TG_MEM_HOST)
        TG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * n * nrays, cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaFreeAsync(owned, st));
    if (fcopy) TG_CUDA(cudaFreeAsync(fcopy, st));
    TG_CUDA(cudaStreamSynchronize(st));
    if (hflag) {
        set_last_error_msg("column density walk did not end within one visit per element");
        return TG_ERR_ITER_LIMIT;
    }
    return TG_OK;
}

}  // extern "C"
