// Learned opening angle (declared in include/pytreegrav_gb300_theta.h; no counterpart in pytreegrav,
// whose walk takes one global theta: grouped_treewalk.py:163-241, treewalk.py:22-25).
//
// Per group of the tree grouping: features from the tree (k_features), a 16-64-64-1 SiLU MLP that
// maps them to an opening angle, and the grouped walk run with that angle per group. The MLP is
// trained by the kernels here (FP32 forward, backward, Adam, and the interpolated cost/error loss)
// and evaluated by one fused BF16 tensor-core kernel (mma.sync m16n8k16, FP32 accumulation).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include <cuda_bf16.h>

#include "tg_targets.cuh"
#include "../../include/pytreegrav_gb300_theta.h"

namespace tg {

tg_status tree_groups(tg_tree_s *t, int G, cudaStream_t st);
tg_status tree_groups_with_arena(tg_tree_s *t, int G, bool fp64, cudaStream_t st);
template <typename T>
tg_status build_arena(tg_tree_s *t, Arena<T> &ar, cudaStream_t st);
tg_status run_walk(tg_tree_s *t, const double *tpos, const double *th, int64_t ntargets, const int2 *groups,
                   const int *group_root, const int *group_order, int64_t ngroups, const int64_t *scatter, int fields,
                   int quadrupole, double theta, double G, int group_size, int precision, const float *theta_group,
                   const float *tol_group, double *out, cudaStream_t st);
int field_width_of(int fields) { return ((fields & 1) ? 1 : 0) + ((fields & 2) ? 3 : 0) + ((fields & 4) ? 9 : 0); }

namespace {

constexpr int NF = TG_THETA_NFEAT;
constexpr int H = TG_MLP_H;
constexpr int NP = TG_MLP_NPARAM;
// parameter offsets in the flat array
constexpr int OW1 = 0, OB1 = OW1 + H * NF, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H;
static_assert(OB3 + 1 == NP, "parameter layout");

constexpr int TOP_DEPTH = 3;                      // levels of the tree whose nodes give the coarse field
constexpr int TOP_MAX = 8 + 64 + 512;             // nodes at depths 1..3

bool valid_gs(int gs) { return gs == 1 || gs == 2 || gs == 4 || gs == 8 || gs == 16 || gs == 32; }

__global__ void k_copy_groups(const int2 *groups, const int *node, int64_t ng, int32_t *first, int32_t *count,
                              int32_t *nodeo) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    if (first) first[g] = groups[g].x;
    if (count) count[g] = groups[g].y;
    if (nodeo) nodeo[g] = node[g];
}

// The frontier of the top TOP_DEPTH levels under the root (node 0): every node at depth TOP_DEPTH
// and every shallower node without node children, found level by level from the arena's child
// ranges and listed in ascending node order, and its FP32 records relative to the root's centre of
// mass: (x, y, z, m) and the square of half the node size (the field's softening), with the root's
// centre (float3 + pad). One block; *ntop receives the count.
__global__ void k_top_nodes(Arena<float> ar, int64_t ntot, const double *coord, const double *mass,
                            const double *size, int *top, int *ntop, float4 *rec, float *hs2, float4 *origin) {
    __shared__ int cur[TOP_MAX], nxt[TOP_MAX], fr[TOP_MAX];
    __shared__ int ncur, nnxt, nout;
    if (ar.bad && *ar.bad) {  // the arena is invalid (the walk reports it): no frontier
        if (threadIdx.x == 0) {
            *ntop = 0;
            *origin = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return;
    }
    if (threadIdx.x == 0) {
        cur[0] = 0;
        ncur = 1;
        nout = 0;
    }
    __syncthreads();
    for (int d = 0; d < TOP_DEPTH; d++) {
        if (threadIdx.x == 0) nnxt = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < ncur; i += blockDim.x) {
            const int j = cur[i];
            const int cb = __float_as_int(ar.n_trav[2 * j + 1].z);
            const int fc = cb >> 4, nc = cb & 15;
            if (nc == 0) {
                if (d > 0) {
                    int q = atomicAdd(&nout, 1);
                    if (q < TOP_MAX) fr[q] = j;
                }
            } else {
                int q = atomicAdd(&nnxt, nc);
                for (int k = 0; k < nc && q + k < TOP_MAX; k++) nxt[q + k] = fc + k;
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < min(nnxt, TOP_MAX); i += blockDim.x) cur[i] = nxt[i];
        if (threadIdx.x == 0) ncur = min(nnxt, TOP_MAX);
        __syncthreads();
    }
    for (int i = threadIdx.x; i < ncur; i += blockDim.x) {
        int q = atomicAdd(&nout, 1);
        if (q < TOP_MAX) fr[q] = cur[i];
    }
    __syncthreads();
    // ascending node order (the atomics' order varies from run to run; the features' sums do not)
    const int nt = min(nout, TOP_MAX);
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        const int j = fr[i];
        int r = 0;
        for (int k = 0; k < nt; k++) r += fr[k] < j ? 1 : 0;  // node indices are distinct
        nxt[r] = j;
    }
    __syncthreads();
    if (threadIdx.x == 0) *ntop = nt;
    const double ox = coord[3 * ntot], oy = coord[3 * ntot + 1], oz = coord[3 * ntot + 2];
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        const int j = nxt[i];
        top[i] = j;
        const int64_t f = ntot + j;
        rec[i] = make_float4((float)(coord[3 * f] - ox), (float)(coord[3 * f + 1] - oy), (float)(coord[3 * f + 2] - oz),
                             (float)mass[f]);
        const float hs = 0.5f * (float)size[f];
        hs2[i] = hs * hs;
    }
    if (threadIdx.x == 0) *origin = make_float4((float)ox, (float)oy, (float)oz, 0.f);
}

// One warp per group (see tg_theta_features for the list), in FP32 on coordinates relative to the
// root's centre of mass.
// Targets at tcoord/tsoft (the tree's own particles, or an external target set in its walk order);
// coord, mass and size are the source tree's, and group_node indexes its nodes.
__global__ void k_features(int64_t ntot, const double *coord, const double *mass, const double *size,
                           const double *tcoord, const double *tsoft, const int2 *groups, const int *group_node,
                           int64_t ngroups,
                           const float4 *rec, const float *hs2, const int *ntop_p, const float4 *origin, int quad,
                           float log10n, float *feat, unsigned long long *field_sums) {
    // the tolerance unit's sums, added per block and then once to field_sums
    __shared__ unsigned long long red[2];
    if (threadIdx.x == 0) red[0] = red[1] = 0ull;
    __syncthreads();
    const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (g < ngroups) {  // warp-uniform
        const int2 gr = groups[g];
        const float4 o4 = *origin;
        // targets: box and softening
        float lo[3], hi[3], hm;
        {
            const int64_t t = gr.x + (lane < gr.y ? lane : 0);
            const float o[3] = {o4.x, o4.y, o4.z};
            for (int k = 0; k < 3; k++) {  // (hi - o) + lo: the offset from the origin to ~1 float ulp
                float ch, cl;
                d2f_split(tcoord[3 * t + k], ch, cl);
                lo[k] = hi[k] = (ch - o[k]) + cl;
            }
            hm = d2f(tsoft[t]);
        }
    #pragma unroll
        for (int s = 16; s; s >>= 1) {
    #pragma unroll
            for (int k = 0; k < 3; k++) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(FULL, lo[k], s));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(FULL, hi[k], s));
            }
            hm = fmaxf(hm, __shfl_xor_sync(FULL, hm, s));
        }
        float gc[3], ext[3];
    #pragma unroll
        for (int k = 0; k < 3; k++) {
            gc[k] = 0.5f * (lo[k] + hi[k]);
            ext[k] = hi[k] - lo[k];
        }
        // coarse field of the top levels at the group centre, each node softened by half its size
        const int ntop = *ntop_p;
        float s1 = 0.f, s3 = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
#pragma unroll 4
        for (int i = lane; i < ntop; i += 32) {
            const float4 r = rec[i];
            const float dx = r.x - gc[0], dy = r.y - gc[1], dz = r.z - gc[2];
            const float r2 = dx * dx + dy * dy + dz * dz + hs2[i];
            const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
            const float mr = r.w * rinv;
            s1 += mr * rinv;
            s3 += mr;
            const float m3 = mr * rinv * rinv;
            vx += m3 * dx;
            vy += m3 * dy;
            vz += m3 * dz;
        }
    #pragma unroll
        for (int s = 16; s; s >>= 1) {
            s1 += __shfl_xor_sync(FULL, s1, s);
            s3 += __shfl_xor_sync(FULL, s3, s);
            vx += __shfl_xor_sync(FULL, vx, s);
            vy += __shfl_xor_sync(FULL, vy, s);
            vz += __shfl_xor_sync(FULL, vz, s);
        }
        // the features, one per lane (the sums above are on every lane after the butterfly)
        const int64_t R = ntot, P = ntot + group_node[g];  // system root (node 0) and the group's node
        // FP64 compares and conversions as integer work (finite inputs: x > 0 iff its bits are a
        // positive int64)
        auto pos = [](double x) { return __double_as_longlong(x) > 0; };
        const double sR = size[R], mR = mass[R], sPd = size[P], mPd = mass[P];
        const float S = pos(sR) ? d2f(sR) : 1.f, Mt = pos(mR) ? d2f(mR) : 1.f;
        const float tiny = 1e-9f * S;
        const float fa = s1 * S * S / Mt, fv = sqrtf(vx * vx + vy * vy + vz * vz) * S * S / Mt;
        // every lane takes one logarithm (lane k: feature k's argument; lane 13, the lambda slot,
        // log S for feature 12), then the differences come from the neighbours' values
        const float emax = fmaxf(ext[0], fmaxf(ext[1], ext[2])), emin = fminf(ext[0], fminf(ext[1], ext[2]));
        const float sP = pos(sPd) ? d2f(sPd) : tiny, mP = d2f(mPd);
        float arg = 1.f;
        switch (lane) {  // selects only
            case 1: arg = emax / S + 1e-9f; break;
            case 2: arg = sP / S; break;
            case 3: arg = mP / Mt + 1e-30f; break;
            case 5: arg = sqrtf(gc[0] * gc[0] + gc[1] * gc[1] + gc[2] * gc[2]) / S + 1e-6f; break;
            case 6: arg = fa + 1e-30f; break;
            case 7: arg = fv + 1e-30f; break;
            case 8: arg = s3 * S / Mt + 1e-30f; break;
            case 10: arg = hm / S + 1e-9f; break;
            case 12: arg = (ext[0] + tiny) * (ext[1] + tiny) * (ext[2] + tiny) / gr.y; break;
            case 13: arg = S; break;
            default: break;
        }
        const float lg = logf(arg);
        const float l2 = __shfl_sync(FULL, lg, 2), l3 = __shfl_sync(FULL, lg, 3), l6 = __shfl_sync(FULL, lg, 6),
                    l7 = __shfl_sync(FULL, lg, 7), l13 = __shfl_sync(FULL, lg, 13);
        const float lgn = log2f((float)gr.y);
        if (lane < NF) {
            float v = lg;
            if (lane == 0) v = lgn;
            else if (lane == 4) v = l3 - 3.f * l2;
            else if (lane == 9) v = l7 - l6;
            else if (lane == 11) v = emin / (emax + tiny);
            else if (lane == 12) v = lg / 3.f - l13;
            else if (lane == TG_THETA_FEAT_LAMBDA) v = 0.f;
            else if (lane == 14) v = quad ? 1.f : 0.f;
            else if (lane == 15) v = log10n;
            feat[g * NF + lane] = v;
        }
        if (lane == 0) {
            // group-size weighted sum of the field's square (units M / S^2, fixed point 2^-32: integer
            // sums do not depend on the order of the atomics) and of the weights, for the tolerance
            // unit of tg_theta_tolerances
            const uint32_t qb = __float_as_uint(fminf((float)gr.y * fv * fv, 1e8f) * 4294967296.f) & 0x7fffffffu;
            const int qe = (int)(qb >> 23) - 150;  // truncation to an integer, without a 64-bit conversion
            const unsigned long long qm = (qb & 0x7fffffu) | 0x800000u;
            atomicAdd(&red[0], qb < 0x3f800000u ? 0ull : (qe >= 0 ? qm << qe : qm >> -qe));
            atomicAdd(&red[1], (unsigned long long)gr.y);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && red[1] != 0ull) {
        atomicAdd(field_sums, red[0]);
        atomicAdd(field_sums + 1, red[1]);
    }
}

}  // namespace

namespace {

// ---------------------------------------------------------------------------------------------
// MLP, FP32 training path. h = silu(z) = z * sigmoid(z); silu'(z) = s (1 + z (1 - s)).
__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
    float s = sigm(z);
    return s * (1.f + z * (1.f - s));
}

constexpr int MLP_THREADS = 128;

// One thread per sample; parameters staged in shared memory (all threads read the same weight:
// broadcast). acts[i] = (z1[0..63], z2[0..63]).
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_forward(const float *P, const float *x, int64_t n, float *acts,
                                                             float *y) {
    __shared__ float w[NP];
    for (int i = threadIdx.x; i < NP; i += blockDim.x) w[i] = P[i];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float xin[NF];
#pragma unroll
    for (int k = 0; k < NF; k++) xin[k] = x[i * NF + k];
    float h1[H];
#pragma unroll
    for (int r = 0; r < H; r++) {
        float z = w[OB1 + r];
#pragma unroll
        for (int k = 0; k < NF; k++) z = fmaf(w[OW1 + r * NF + k], xin[k], z);
        if (acts) acts[i * 2 * H + r] = z;
        h1[r] = silu(z);
    }
    float out = w[OB3];
    for (int r = 0; r < H; r++) {
        float z = w[OB2 + r];
#pragma unroll
        for (int k = 0; k < H; k++) z = fmaf(w[OW2 + r * H + k], h1[k], z);
        if (acts) acts[i * 2 * H + H + r] = z;
        out = fmaf(w[OW3 + r], silu(z), out);
    }
    y[i] = out;
}

// Backward, per sample: work[i] = (dz1[0..63], dz2[0..63]) for the loss gradient dy[i].
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_backward_samples(const float *P, const float *acts,
                                                                      const float *dy, int64_t n, float *work) {
    __shared__ float w[NP];
    for (int i = threadIdx.x; i < NP; i += blockDim.x) w[i] = P[i];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = dy[i];
    float dh1[H];
#pragma unroll
    for (int k = 0; k < H; k++) dh1[k] = 0.f;
    for (int r = 0; r < H; r++) {
        const float dz2 = g * w[OW3 + r] * dsilu(acts[i * 2 * H + H + r]);
        work[i * 2 * H + H + r] = dz2;
#pragma unroll
        for (int k = 0; k < H; k++) dh1[k] = fmaf(w[OW2 + r * H + k], dz2, dh1[k]);
    }
#pragma unroll
    for (int k = 0; k < H; k++) work[i * 2 * H + k] = dh1[k] * dsilu(acts[i * 2 * H + k]);
}

// Weight gradients: one thread per parameter, samples split into chunks across blockIdx.y; each
// chunk's partial sum is added to grad (zeroed by the caller).
constexpr int GRAD_CHUNK = 256;
__global__ void k_mlp_backward_weights(const float *x, const float *acts, const float *dy, const float *work,
                                       int64_t n, float *grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NP) return;
    const int64_t i0 = (int64_t)blockIdx.y * GRAD_CHUNK, i1 = min(i0 + GRAD_CHUNK, n);
    float s = 0.f;
    if (p < OB1) {  // W1[r][k]: dz1[r] x[k]
        const int r = p / NF, k = p % NF;
        for (int64_t i = i0; i < i1; i++) s = fmaf(work[i * 2 * H + r], x[i * NF + k], s);
    } else if (p < OW2) {  // b1[r]
        const int r = p - OB1;
        for (int64_t i = i0; i < i1; i++) s += work[i * 2 * H + r];
    } else if (p < OB2) {  // W2[r][k]: dz2[r] h1[k]
        const int r = (p - OW2) / H, k = (p - OW2) % H;
        for (int64_t i = i0; i < i1; i++) s = fmaf(work[i * 2 * H + H + r], silu(acts[i * 2 * H + k]), s);
    } else if (p < OW3) {  // b2[r]
        const int r = p - OB2;
        for (int64_t i = i0; i < i1; i++) s += work[i * 2 * H + H + r];
    } else if (p < OB3) {  // W3[r]: dy h2[r]
        const int r = p - OW3;
        for (int64_t i = i0; i < i1; i++) s = fmaf(dy[i], silu(acts[i * 2 * H + H + r]), s);
    } else {  // b3
        for (int64_t i = i0; i < i1; i++) s += dy[i];
    }
    atomicAdd(grad + p, s);
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Loss per sample (see tg_theta_loss); block-reduced into *loss_sum.
__global__ void k_theta_loss(const float *y, const float *lc, const float *le, const float *lam, int64_t n, int K,
                             float t0, float dt, float tmin, float tmax, float *dy, float *loss_sum) {
    __shared__ float red[256];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const float s = sigm(y[i]);
        const float th = tmin + (tmax - tmin) * s;
        float u = (th - t0) / dt;
        int k = (int)floorf(u);
        k = k < 0 ? 0 : (k > K - 2 ? K - 2 : k);
        const float wgt = u - (float)k;
        const float *c = lc + i * K, *e = le + i * K;
        const float logc = c[k] + wgt * (c[k + 1] - c[k]);
        const float loge = e[k] + wgt * (e[k + 1] - e[k]);
        const float cost = __expf(logc), err = __expf(loge);
        const float la = lam[i];
        l = cost + la * err;
        const float dl_dth = (cost * (c[k + 1] - c[k]) + la * err * (e[k + 1] - e[k])) / dt;
        dy[i] = dl_dth * (tmax - tmin) * s * (1.f - s) / (float)n;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss_sum, red[0] / (float)n);
}

// ---------------------------------------------------------------------------------------------
// Inference: 16 samples per warp and mma.sync.m16n8k16 (BF16 in, FP32 accumulate). With g = lane/4
// and c = lane%4, a thread holds A elements (rows g, g+8; columns 2c, 2c+1, 2c+8, 2c+9), B elements
// (k = 2c, 2c+1, 2c+8, 2c+9; n = g) and accumulators (rows g, g+8; columns 2c, 2c+1) of each 8-wide
// output tile, so output tiles 2k and 2k+1 of one layer are exactly the A fragment of k-step k of
// the next: the hidden activations never leave registers.
struct ModelDev {
    const uint32_t *w1;  // W1 as BF16 pairs, [64][8]
    const uint32_t *w2;  // W2 as BF16 pairs, [64][32]
    const float *b1, *b2, *w3, *b3, *mean, *inv_std;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int INF_WARPS = 4;
// The tolerance unit A * M / S^2 (see tg_theta_tolerances) from the features kernel's field sums.
__device__ __forceinline__ float tol_scale(const unsigned long long *field_sums, const double *mass,
                                           const double *size, int64_t ntot) {
    const double S = size[ntot] > 0 ? size[ntot] : 1.0, M = mass[ntot] > 0 ? mass[ntot] : 1.0;
    const double w = field_sums[1] > 0 ? (double)field_sums[1] : 1.0;
    return (float)(sqrt((double)field_sums[0] / 4294967296.0 / w) * M / (S * S));
}

// Output per row: the model's value u in [tmin, tmax] into theta; or, with ts.tol set (a tolerance
// model), the tolerance 10^u times the unit into ts.tol, a non-finite u taking umin (the strictest).
struct TolOut {
    float *tol = nullptr;
    const unsigned long long *field_sums = nullptr;
    const double *mass = nullptr, *size = nullptr;
    int64_t ntot = 0;
    float umin = 0.f;
};

__global__ void __launch_bounds__(INF_WARPS * 32) k_theta_infer(ModelDev md, const float *feat, int64_t n,
                                                                float loglam, float tmin, float tmax, float *theta,
                                                                TolOut ts) {
    __shared__ uint32_t sw1[H * NF / 2], sw2[H * H / 2];
    __shared__ float sb1[H], sb2[H], sw3[H], smu[NF], sis[NF];
    __shared__ float sscale;
    if (ts.tol && threadIdx.x == 0) sscale = tol_scale(ts.field_sums, ts.mass, ts.size, ts.ntot);
    for (int i = threadIdx.x; i < H * NF / 2; i += blockDim.x) sw1[i] = md.w1[i];
    for (int i = threadIdx.x; i < H * H / 2; i += blockDim.x) sw2[i] = md.w2[i];
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        sb1[i] = md.b1[i];
        sb2[i] = md.b2[i];
        sw3[i] = md.w3[i];
    }
    for (int i = threadIdx.x; i < NF; i += blockDim.x) {
        smu[i] = md.mean[i];
        sis[i] = md.inv_std[i];
    }
    __syncthreads();
    const float b3 = md.b3[0];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, c = lane & 3;
    const int64_t ntiles = (n + 15) / 16;
    for (int64_t tile = (int64_t)blockIdx.x * INF_WARPS + warp; tile < ntiles; tile += (int64_t)gridDim.x * INF_WARPS) {
        const int64_t r0 = tile * 16 + g, r1 = r0 + 8;
        auto x = [&](int64_t r, int k) -> float {
            if (r >= n) return 0.f;
            float v = k == TG_THETA_FEAT_LAMBDA ? loglam : feat[r * NF + k];
            return (v - smu[k]) * sis[k];
        };
        uint32_t a[4];
        a[0] = pack_bf16(x(r0, 2 * c), x(r0, 2 * c + 1));
        a[1] = pack_bf16(x(r1, 2 * c), x(r1, 2 * c + 1));
        a[2] = pack_bf16(x(r0, 2 * c + 8), x(r0, 2 * c + 9));
        a[3] = pack_bf16(x(r1, 2 * c + 8), x(r1, 2 * c + 9));
        // layer 1: 16 x 64 = 8 tiles of 8 outputs, one k-step
        float acc[8][4];
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const float bl = sb1[8 * t + 2 * c], bh = sb1[8 * t + 2 * c + 1];
            acc[t][0] = bl; acc[t][1] = bh; acc[t][2] = bl; acc[t][3] = bh;
            mma_bf16(acc[t], a, sw1[(8 * t + g) * 8 + c], sw1[(8 * t + g) * 8 + c + 4]);
        }
        uint32_t a2[4][4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            a2[k][0] = pack_bf16(silu(acc[2 * k][0]), silu(acc[2 * k][1]));
            a2[k][1] = pack_bf16(silu(acc[2 * k][2]), silu(acc[2 * k][3]));
            a2[k][2] = pack_bf16(silu(acc[2 * k + 1][0]), silu(acc[2 * k + 1][1]));
            a2[k][3] = pack_bf16(silu(acc[2 * k + 1][2]), silu(acc[2 * k + 1][3]));
        }
        // layer 2: 8 tiles, four k-steps
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const float bl = sb2[8 * t + 2 * c], bh = sb2[8 * t + 2 * c + 1];
            acc[t][0] = bl; acc[t][1] = bh; acc[t][2] = bl; acc[t][3] = bh;
#pragma unroll
            for (int k = 0; k < 4; k++)
                mma_bf16(acc[t], a2[k], sw2[(8 * t + g) * 32 + 8 * k + c], sw2[(8 * t + g) * 32 + 8 * k + c + 4]);
        }
        // output layer in FP32: each thread's 16 columns, then the four threads of a row
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const float wl = sw3[8 * t + 2 * c], wh = sw3[8 * t + 2 * c + 1];
            s0 = fmaf(wl, silu(acc[t][0]), fmaf(wh, silu(acc[t][1]), s0));
            s1 = fmaf(wl, silu(acc[t][2]), fmaf(wh, silu(acc[t][3]), s1));
        }
        s0 += __shfl_xor_sync(FULL, s0, 1);
        s0 += __shfl_xor_sync(FULL, s0, 2);
        s1 += __shfl_xor_sync(FULL, s1, 1);
        s1 += __shfl_xor_sync(FULL, s1, 2);
        if (c == 0) {
            float u0 = tmin + (tmax - tmin) * sigm(s0 + b3), u1 = tmin + (tmax - tmin) * sigm(s1 + b3);
            if (ts.tol) {
                if (!isfinite(u0)) u0 = ts.umin;
                if (!isfinite(u1)) u1 = ts.umin;
                if (r0 < n) ts.tol[r0] = exp10f(u0) * sscale;
                if (r1 < n) ts.tol[r1] = exp10f(u1) * sscale;
            } else {
                if (r0 < n) theta[r0] = u0;
                if (r1 < n) theta[r1] = u1;
            }
        }
    }
}

__global__ void k_to_bf16_pairs(const float *w, int npairs, uint32_t *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npairs) out[i] = pack_bf16(w[2 * i], w[2 * i + 1]);
}

// Non-finite or out-of-range outputs (a damaged model) are replaced by `fallback`.
__global__ void k_theta_guard(float *theta, int64_t n, float fallback, float tmin, float tmax) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = theta[i];
    if (!(v >= tmin && v <= tmax)) theta[i] = fallback;
}

// Tolerance unit A * M / S^2 (see tg_theta_tolerances) from the features kernel's field sums.
__global__ void k_tol_scale(const unsigned long long *field_sums, const double *mass, const double *size,
                            int64_t ntot, float *scale) {
    *scale = tol_scale(field_sums, mass, size, ntot);
}

__global__ void k_u_to_tol(const float *u, int64_t ng, const float *scale, float umin, float *tol) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    float v = u[g];
    if (!isfinite(v)) v = umin;  // a damaged output takes the strictest tolerance
    tol[g] = exp10f(v) * *scale;
}

}  // namespace
}  // namespace tg

struct tg_theta_model_s {
    void *mem = nullptr;  // one device allocation holding everything below
    tg::ModelDev dev;
    int kind = TG_THETA_KIND_ANGLE;
    float tmin = 0.f, tmax = 0.f;  // output range
    float theta_max = 0.f;         // angle cap of a tolerance model
    float err_budget = 0.f;        // per-group relative error budget (0: no rewalk)
};

namespace {

using namespace tg;

// Features of ng groups of targets (tcoord/tsoft in walk order; group_node: the source tree's node
// holding each group) into feat (ng x NF); field_sums (2 x uint64, device, may be NULL) receives the
// sums behind the tolerance unit.
tg_status features_of_groups(tg_tree_s *t, const double *tcoord, const double *tsoft, const int2 *groups,
                             const int *group_node, int64_t ng, int quadrupole, float *feat, cudaStream_t st,
                             unsigned long long *field_sums) {
    if (t->nsys != 1) {
        set_last_error_msg("learned opening angles need a single-system tree");
        return TG_ERR_BAD_ARG;
    }
    TG_TRY(build_arena(t, t->arena32, st));
    // one scratch block: top count + indices, then the FP32 records and the origin
    const size_t rec_off = 16 * ((sizeof(int) * (TOP_MAX + 1) + 15) / 16);
    unsigned char *scr = nullptr;
    TG_CUDA(dev_malloc((void **)&scr, rec_off + (sizeof(float4) + sizeof(float)) * TOP_MAX + sizeof(float4) + 32, st));
    int *top = (int *)scr;
    float4 *rec = (float4 *)(scr + rec_off);
    float4 *origin = rec + TOP_MAX;
    float *hs2 = (float *)(origin + 1);
    unsigned long long *sums = field_sums ? field_sums : (unsigned long long *)(origin + 1 + TOP_MAX / 4);
    TG_CUDA(cudaMemsetAsync(sums, 0, 2 * sizeof(unsigned long long), st));
    { k_top_nodes<<<1, 256, 0, st>>>(t->arena32, t->ntot, t->coord, t->mass, t->size, top + 1, top, rec, hs2, origin); note_launch(); }
    if (ng > 0) {
        k_features<<<div_up(ng * 32, 256), 256, 0, st>>>(t->ntot, t->coord, t->mass, t->size, tcoord, tsoft, groups,
                                                         group_node, ng, rec, hs2, top, origin, quadrupole,
                                                         (float)log10((double)t->ntot), feat, sums);
        note_launch();
    }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaFreeAsync(scr, st));
    return TG_OK;
}

// Features of the tree grouping of the tree's own particles (see features_of_groups).
tg_status features_device(tg_tree_s *t, int group_size, int quadrupole, float *feat, cudaStream_t st,
                          unsigned long long *field_sums = nullptr) {
    if (t->nsys != 1) {
        set_last_error_msg("learned opening angles need a single-system tree");
        return TG_ERR_BAD_ARG;
    }
    TG_TRY(tree_groups(t, group_size, st));
    return features_of_groups(t, t->coord, t->soft, t->groups, t->group_node, t->ngroups, quadrupole, feat, st,
                              field_sums);
}

// Features of an external target set's groups (see features_of_groups).
tg_status features_targets(tg_targets_s *ts, int quadrupole, float *feat, cudaStream_t st,
                           unsigned long long *field_sums = nullptr) {
    TG_TRY(targets_src_nodes(ts, st));
    return features_of_groups(ts->src, ts->tt->coord, ts->tt->soft, ts->tt->groups, ts->src_node, ts->tt->ngroups,
                              quadrupole, feat, st, field_sums);
}

// field_sums: from features_of_groups over the ng groups; scale: one float of scratch (device).
tg_status tolerances_device(tg_tree_s *t, const unsigned long long *field_sums, const float *u, int64_t ng, float umin,
                            float *tol, float *scale, cudaStream_t st) {
    if (ng <= 0) return TG_OK;
    { k_tol_scale<<<1, 1, 0, st>>>(field_sums, t->mass, t->size, t->ntot, scale); note_launch(); }
    { k_u_to_tol<<<div_up(ng, 256), 256, 0, st>>>(u, ng, scale, umin, tol); note_launch(); }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

tg_status infer_device(const tg_theta_model_s *m, const float *feat, int64_t n, float loglam, float *theta,
                       cudaStream_t st, TolOut ts = TolOut()) {
    if (n <= 0) return TG_OK;
    const int64_t tiles = (n + 15) / 16;
    const int grid = (int)std::min<int64_t>((tiles + INF_WARPS - 1) / INF_WARPS, (int64_t)num_sms() * 8);
    { k_theta_infer<<<grid, INF_WARPS * 32, 0, st>>>(m->dev, feat, n, loglam, m->tmin, m->tmax, theta, ts); note_launch(); }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

// The walk of ng groups of targets (tpos/tsoft in walk order, results scattered through `scatter`)
// with each group's acceptance test from the model (see tg_tree_fields_learned); feats(feat, sums)
// writes the groups' features and the tolerance unit's sums. The source tree t must be built and
// its FP32 arena packed or packable on st.
template <typename FeatFn>
tg_status learned_walk(tg_tree_s *t, FeatFn feats, const double *tpos, const double *tsoft, int64_t nt,
                       const int2 *groups, const int *groot, int64_t ng, const int64_t *scatter, int fields,
                       int quadrupole, double G, int group_size, const tg_theta_model_s *m, float log10_lambda,
                       double theta_fallback, int mem, double *out, cudaStream_t st) {
    float *tg_theta = nullptr, *feat = nullptr, *tol = nullptr;
    double theta = theta_fallback;
    // every device buffer of this call, released on any exit
    struct Bufs {
        float **p[3];
        cudaStream_t st;
        ~Bufs() {
            for (float **q : p)
                if (*q) cudaFreeAsync(*q, st);
        }
    } bufs{{&tg_theta, &feat, &tol}, st};
    if (m) {
        const int64_t ng1 = std::max<int64_t>(ng, 1);
        TG_CUDA(dev_malloc((void **)&feat, sizeof(float) * (NF * ng1 + 8), st));
        unsigned long long *sums = (unsigned long long *)(feat + (NF * ng1 + 1) / 2 * 2);
        TG_TRY(feats(feat, sums));
        if (m->kind == TG_THETA_KIND_ANGLE) {
            TG_CUDA(dev_malloc((void **)&tg_theta, sizeof(float) * ng1, st));
            TG_TRY(infer_device(m, feat, ng, log10_lambda, tg_theta, st));
            { k_theta_guard<<<div_up(ng, 256), 256, 0, st>>>(tg_theta, ng, (float)theta_fallback, m->tmin, m->tmax); note_launch(); }
            TG_CUDA(cudaGetLastError());
        } else {  // the tolerances straight from the inference (tolerances_device's values)
            TG_CUDA(dev_malloc((void **)&tol, sizeof(float) * ng1, st));
            TolOut ts;
            ts.tol = tol;
            ts.field_sums = sums;
            ts.mass = t->mass;
            ts.size = t->size;
            ts.ntot = t->ntot;
            ts.umin = m->tmin;
            TG_TRY(infer_device(m, feat, ng, log10_lambda, nullptr, st, ts));
            theta = m->theta_max;
        }
    }
    const int W = field_width_of(fields);
    double *dout = out;
    if (mem == TG_MEM_HOST) TG_CUDA(dev_malloc((void **)&dout, sizeof(double) * nt * W, st));
    t->err_budget = (m && tol) ? m->err_budget : 0.f;
    t->rewalk_theta = theta_fallback;
    tg_status rc = run_walk(t, tpos, tsoft, nt, groups, groot, nullptr, ng, scatter, fields, quadrupole, theta, G,
                            group_size, TG_FP32, tg_theta, tol, dout, st);
    t->err_budget = 0.f;
    if (rc == TG_OK && mem == TG_MEM_HOST)
        TG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * nt * W, cudaMemcpyDeviceToHost, st));
    if (mem == TG_MEM_HOST) cudaFreeAsync(dout, st);
    TG_CUDA(cudaStreamSynchronize(st));
    return rc;
}

tg_status stage_to_host(const float *src, int64_t n, int mem, std::vector<float> &dst) {
    dst.resize(n);
    if (mem == TG_MEM_HOST) memcpy(dst.data(), src, sizeof(float) * n);
    else TG_CUDA(cudaMemcpy(dst.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return TG_OK;
}

}  // namespace

extern "C" {

tg_status tg_tree_groups(tg_tree t, int group_size, int64_t *ngroups, void *stream) {
    if (!t || !ngroups || !valid_gs(group_size)) return TG_ERR_BAD_ARG;
    tree_wait_built(t, (cudaStream_t)stream);
    TG_TRY(tree_groups(t, group_size, (cudaStream_t)stream));
    *ngroups = t->ngroups;
    return TG_OK;
}

tg_status tg_tree_groups_copy(tg_tree t, int group_size, int32_t *first, int32_t *count, int32_t *node, int mem,
                              void *stream) {
    if (!t || !valid_gs(group_size)) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    TG_TRY(tree_groups(t, group_size, st));
    const int64_t ng = t->ngroups;
    if (ng == 0) return TG_OK;
    int32_t *buf = nullptr;
    int32_t *d[3] = {first, count, node};
    if (mem == TG_MEM_HOST) {
        TG_CUDA(dev_malloc((void **)&buf, sizeof(int32_t) * 3 * ng, st));
        for (int k = 0; k < 3; k++) d[k] = buf + k * ng;
    }
    { k_copy_groups<<<div_up(ng, 256), 256, 0, st>>>(t->groups, t->group_node, ng, d[0], d[1], d[2]); note_launch(); }
    TG_CUDA(cudaGetLastError());
    if (mem == TG_MEM_HOST) {
        int32_t *h[3] = {first, count, node};
        for (int k = 0; k < 3; k++)
            if (h[k]) TG_CUDA(cudaMemcpyAsync(h[k], d[k], sizeof(int32_t) * ng, cudaMemcpyDeviceToHost, st));
        TG_CUDA(cudaFreeAsync(buf, st));
    }
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

tg_status tg_tree_record_group_stats(tg_tree t, int enable) {
    if (!t) return TG_ERR_BAD_ARG;
    t->record_group_stats = enable ? 1 : 0;
    return TG_OK;
}

tg_status tg_theta_model_set_error_budget(tg_theta_model m, float budget) {
    if (!m || !(budget >= 0.f)) return TG_ERR_BAD_ARG;
    m->err_budget = budget;
    return TG_OK;
}

tg_status tg_tree_last_group_error(tg_tree t, float *out, int mem, void *stream) {
    if (!t || !out || !t->gerr) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    TG_CUDA(cudaMemcpyAsync(out, t->gerr, sizeof(float) * t->last_stats.groups,
                            mem == TG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

tg_status tg_tree_last_group_stats(tg_tree t, uint32_t *out, int mem, void *stream) {
    if (!t || !out || !t->gstats) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t ng = t->last_stats.groups;  // the groups of the last walk (tree grouping or a target set)
    TG_CUDA(cudaMemcpyAsync(out, t->gstats, sizeof(uint32_t) * 3 * ng,
                            mem == TG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}

tg_status tg_theta_features(tg_tree t, int group_size, int quadrupole, float *features, void *stream) {
    if (!t || !features || !valid_gs(group_size)) return TG_ERR_BAD_ARG;
    tree_wait_built(t, (cudaStream_t)stream);
    return features_device(t, group_size, quadrupole, features, (cudaStream_t)stream);
}

tg_status tg_mlp_forward(const float *params, const float *x, int64_t n, float *acts, float *y, void *stream) {
    if (!params || !x || !y || n < 0) return TG_ERR_BAD_ARG;
    if (n == 0) return TG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    { k_mlp_forward<<<div_up(n, MLP_THREADS), MLP_THREADS, 0, st>>>(params, x, n, acts, y); note_launch(); }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

tg_status tg_mlp_backward(const float *params, const float *x, const float *acts, const float *dy, int64_t n,
                          float *work, float *grad, void *stream) {
    if (!params || !x || !acts || !dy || !work || !grad || n < 0) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    TG_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * NP, st));
    if (n == 0) return TG_OK;
    { k_mlp_backward_samples<<<div_up(n, MLP_THREADS), MLP_THREADS, 0, st>>>(params, acts, dy, n, work); note_launch(); }
    const int chunks = div_up(n, GRAD_CHUNK);
    if (chunks > 65535) return TG_ERR_BAD_ARG;
    { k_mlp_backward_weights<<<dim3(div_up(NP, 128), chunks), 128, 0, st>>>(x, acts, dy, work, n, grad); note_launch(); }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

tg_status tg_adam_step(float *params, const float *grad, float *m, float *v, int64_t nparam, float lr, float beta1,
                       float beta2, float eps, int step, void *stream) {
    if (!params || !grad || !m || !v || nparam < 0 || step < 1) return TG_ERR_BAD_ARG;
    if (nparam == 0) return TG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    { k_adam<<<div_up(nparam, 256), 256, 0, st>>>(params, grad, m, v, nparam, lr, beta1, beta2, eps, c1, c2); note_launch(); }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

tg_status tg_theta_loss(const float *y, const float *log_cost, const float *log_err, const float *lambda, int64_t n,
                        int ngrid, float theta_lo, float theta_step, float theta_min, float theta_max, float *dy,
                        float *loss_sum, void *stream) {
    if (!y || !log_cost || !log_err || !lambda || !dy || !loss_sum || n < 0 || ngrid < 2 || !(theta_step > 0) ||
        !(theta_max > theta_min))
        return TG_ERR_BAD_ARG;
    if (n == 0) return TG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    { k_theta_loss<<<div_up(n, 256), 256, 0, st>>>(y, log_cost, log_err, lambda, n, ngrid, theta_lo, theta_step,
                                                   theta_min, theta_max, dy, loss_sum); note_launch(); }
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

tg_status tg_theta_model_create(const float *params, const float *feat_mean, const float *feat_std, int kind,
                                float out_min, float out_max, float theta_max, int mem, tg_theta_model *out) {
    if (!params || !feat_mean || !feat_std || !out || !(out_max > out_min)) return TG_ERR_BAD_ARG;
    if (kind == TG_THETA_KIND_ANGLE ? !(out_min > 0) : (kind != TG_THETA_KIND_TOLERANCE || !(theta_max > 0)))
        return TG_ERR_BAD_ARG;
    std::vector<float> P, mu, sd;
    TG_TRY(stage_to_host(params, NP, mem, P));
    TG_TRY(stage_to_host(feat_mean, NF, mem, mu));
    TG_TRY(stage_to_host(feat_std, NF, mem, sd));
    // layout: w1 pairs, w2 pairs, b1, b2, w3, b3 (4), mean, inv_std, then FP32 W1 and W2 for the conversion
    const size_t n1 = H * NF / 2, n2 = H * H / 2;
    const size_t nf = 3 * H + 4 + 2 * NF;
    std::vector<float> tail(nf + H * NF + H * H);
    float *q = tail.data();
    memcpy(q, P.data() + OB1, sizeof(float) * H); q += H;
    memcpy(q, P.data() + OB2, sizeof(float) * H); q += H;
    memcpy(q, P.data() + OW3, sizeof(float) * H); q += H;
    q[0] = P[OB3]; q[1] = q[2] = q[3] = 0.f; q += 4;
    for (int k = 0; k < NF; k++) q[k] = mu[k];
    q += NF;
    for (int k = 0; k < NF; k++) {
        if (!(sd[k] > 0) || !std::isfinite(sd[k])) return TG_ERR_BAD_ARG;
        q[k] = 1.f / sd[k];
    }
    q += NF;
    memcpy(q, P.data() + OW1, sizeof(float) * H * NF); q += H * NF;
    memcpy(q, P.data() + OW2, sizeof(float) * H * H);
    tg_theta_model_s *m = new (std::nothrow) tg_theta_model_s();
    if (!m) return TG_ERR_OOM;
    const size_t bytes = sizeof(uint32_t) * (n1 + n2) + sizeof(float) * tail.size();
    cudaError_t e = cudaMalloc(&m->mem, bytes);
    if (e != cudaSuccess) {
        delete m;
        set_last_error("tg_theta_model_create", e);
        return TG_ERR_OOM;
    }
    uint32_t *w1 = (uint32_t *)m->mem, *w2 = w1 + n1;
    float *f = (float *)(w2 + n2);
    tg_status rc = TG_OK;
    if (cudaMemcpy(f, tail.data(), sizeof(float) * tail.size(), cudaMemcpyHostToDevice) != cudaSuccess) rc = TG_ERR_CUDA;
    if (rc == TG_OK) {
        const float *fw1 = f + nf, *fw2 = fw1 + H * NF;
        k_to_bf16_pairs<<<div_up(n1, 256), 256>>>(fw1, (int)n1, w1);
        note_launch();
        k_to_bf16_pairs<<<div_up(n2, 256), 256>>>(fw2, (int)n2, w2);
        note_launch();
        if (cudaDeviceSynchronize() != cudaSuccess) rc = TG_ERR_CUDA;
    }
    if (rc != TG_OK) {
        set_last_error_msg("tg_theta_model_create: device copy failed");
        cudaFree(m->mem);
        delete m;
        return rc;
    }
    m->dev.w1 = w1;
    m->dev.w2 = w2;
    m->dev.b1 = f;
    m->dev.b2 = f + H;
    m->dev.w3 = f + 2 * H;
    m->dev.b3 = f + 3 * H;
    m->dev.mean = f + 3 * H + 4;
    m->dev.inv_std = f + 3 * H + 4 + NF;
    m->kind = kind;
    m->tmin = out_min;
    m->tmax = out_max;
    m->theta_max = theta_max;
    *out = m;
    return TG_OK;
}

tg_status tg_theta_model_free(tg_theta_model m) {
    if (!m) return TG_OK;
    cudaFree(m->mem);
    delete m;
    return TG_OK;
}

tg_status tg_theta_infer(tg_theta_model m, const float *features, int64_t n, float log10_lambda, float *out,
                         void *stream) {
    if (!m || !features || !out || n < 0) return TG_ERR_BAD_ARG;
    return infer_device(m, features, n, log10_lambda, out, (cudaStream_t)stream);
}

tg_status tg_theta_tolerances(tg_tree t, int group_size, int quadrupole, const float *u, float *tol, void *stream) {
    if (!t || !u || !tol || !valid_gs(group_size)) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    TG_TRY(tree_groups(t, group_size, st));
    float *feat = nullptr;
    const int64_t nfeat = NF * std::max<int64_t>(t->ngroups, 1);
    TG_CUDA(dev_malloc((void **)&feat, sizeof(float) * (nfeat + 8), st));
    unsigned long long *sums = (unsigned long long *)(feat + (nfeat + 1) / 2 * 2);
    tg_status rc = features_device(t, group_size, quadrupole, feat, st, sums);
    if (rc == TG_OK) rc = tolerances_device(t, sums, u, t->ngroups, -30.f, tol, (float *)(sums + 2), st);
    cudaFreeAsync(feat, st);
    return rc;
}

tg_status tg_tree_fields_grouped(tg_tree t, int fields, int quadrupole, double G, int group_size, double theta,
                                 const float *theta_per_group, const float *tol_per_group, int mem, double *out,
                                 void *stream) {
    if (!t || !out || (fields & 7) == 0 || (fields & ~7) || !valid_gs(group_size) || !(theta > 0))
        return TG_ERR_BAD_ARG;
    if (quadrupole && !t->has_quads) return TG_ERR_NO_QUADRUPOLES;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    TG_TRY(tree_groups(t, group_size, st));
    const int64_t nt = t->ntot;
    const int W = field_width_of(fields);
    double *dout = out;
    if (mem == TG_MEM_HOST) TG_CUDA(dev_malloc((void **)&dout, sizeof(double) * nt * W, st));
    tg_status rc = run_walk(t, t->coord, t->soft, nt, t->groups, t->group_root, nullptr, t->ngroups, t->walk_idx,
                            fields, quadrupole, theta, G, group_size, TG_FP32, theta_per_group, tol_per_group, dout,
                            st);
    if (rc == TG_OK && mem == TG_MEM_HOST)
        TG_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * nt * W, cudaMemcpyDeviceToHost, st));
    if (mem == TG_MEM_HOST) cudaFreeAsync(dout, st);
    TG_CUDA(cudaStreamSynchronize(st));
    return rc;
}

tg_status tg_tree_fields_learned(tg_tree t, int fields, int quadrupole, double G, int group_size, tg_theta_model m,
                                 float log10_lambda, double theta_fallback, int mem, double *out, void *stream) {
    if (!t || !out || (fields & 7) == 0 || (fields & ~7) || !valid_gs(group_size) || !(theta_fallback > 0))
        return TG_ERR_BAD_ARG;
    if (quadrupole && !t->has_quads) return TG_ERR_NO_QUADRUPOLES;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    TG_TRY(tree_groups_with_arena(t, group_size, false, st));
    auto feats = [&](float *feat, unsigned long long *sums) {
        return features_device(t, group_size, quadrupole, feat, st, sums);
    };
    return learned_walk(t, feats, t->coord, t->soft, t->ntot, t->groups, t->group_root, t->ngroups, t->walk_idx,
                        fields, quadrupole, G, group_size, m, log10_lambda, theta_fallback, mem, out, st);
}

tg_status tg_targets_fields_learned(tg_targets ts, int fields, int quadrupole, double G, tg_theta_model m,
                                    float log10_lambda, double theta_fallback, int mem, double *out, void *stream) {
    if (!ts || !out || (fields & 7) == 0 || (fields & ~7) || !(theta_fallback > 0)) return TG_ERR_BAD_ARG;
    tg_tree_s *t = ts->src, *tt = ts->tt;
    if (quadrupole && !t->has_quads) return TG_ERR_NO_QUADRUPOLES;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(t, st);
    tree_wait_built(tt, st);
    auto feats = [&](float *feat, unsigned long long *sums) { return features_targets(ts, quadrupole, feat, st, sums); };
    return learned_walk(t, feats, tt->coord, tt->soft, ts->n, tt->groups, tt->group_root, tt->ngroups, tt->walk_idx,
                        fields, quadrupole, G, ts->group_size, m, log10_lambda, theta_fallback, mem, out, st);
}

tg_status tg_targets_features(tg_targets ts, int quadrupole, float *features, void *stream) {
    if (!ts || !features) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(ts->src, st);
    tree_wait_built(ts->tt, st);
    return features_targets(ts, quadrupole, features, st);
}

tg_status tg_targets_tolerances(tg_targets ts, int quadrupole, const float *u, float *tol, void *stream) {
    if (!ts || !u || !tol) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    tree_wait_built(ts->src, st);
    tree_wait_built(ts->tt, st);
    const int64_t ng = ts->tt->ngroups;
    float *feat = nullptr;
    const int64_t nfeat = NF * std::max<int64_t>(ng, 1);
    TG_CUDA(dev_malloc((void **)&feat, sizeof(float) * (nfeat + 8), st));
    unsigned long long *sums = (unsigned long long *)(feat + (nfeat + 1) / 2 * 2);
    tg_status rc = features_targets(ts, quadrupole, feat, st, sums);
    if (rc == TG_OK) rc = tolerances_device(ts->src, sums, u, ng, -30.f, tol, (float *)(sums + 2), st);
    cudaFreeAsync(feat, st);
    return rc;
}

}  // extern "C"
