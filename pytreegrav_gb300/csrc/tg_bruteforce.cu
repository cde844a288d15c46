// Exact direct summation (pytreegrav bruteforce.py).
//
// FP64: one target per thread, sources staged through shared memory tiles, every operation
// rounded once in pytreegrav's expression order and summed over sources in ascending order -- the
// same arithmetic as the per-target CPU kernels (bruteforce.py:7-50, 86-116, 164-256, 259-282,
// 319-386), so results agree bit for bit. This is the FP64 judge the FP32 walk is scored against.
//
// FP32: the fast path (the numba-cuda CudaPotentialBruteforce/CudaAccelBruteforce of cuda.py:627-796
// rebuilt): tiles of 256 sources in shared memory, two targets per thread so every broadcast source
// load feeds two interactions, rsqrt, and tile sums added into Kahan-compensated accumulators. For
// the potential and acceleration, four lanes share each pair of targets (k_bf32_split) and the two
// targets are computed with paired f32x2 arithmetic.
#include "tg_common.cuh"

namespace tg {

enum { BF_POT = 1, BF_ACC = 2, BF_TID = 4 };

// kernel.py:5-75 in FP64 with single rounding per operation.
__device__ __forceinline__ double force_kernel_x(double r, double h) {
    if (r > h) return ddiv(1.0, dmul(dmul(r, r), r));
    double hinv = ddiv(1.0, h);
    double q = dmul(r, hinv);
    if (q <= 0.5)
        return dmul(dmul(dmul(dadd(10.666666666666666666, dmul(dmul(q, q), dadd(-38.4, dmul(32.0, q)))), hinv), hinv),
                    hinv);
    double t = dsub(dadd(dsub(21.333333333333, dmul(48.0, q)), dmul(dmul(38.4, q), q)),
                    dmul(dmul(dmul(10.666666666667, q), q), q));
    t = dsub(t, ddiv(0.066666666667, dmul(dmul(q, q), q)));
    return dmul(dmul(dmul(t, hinv), hinv), hinv);
}

__device__ __forceinline__ double tidal_kernel_x(double r, double h) {
    if (r > h) {
        double r2 = dmul(r, r);
        return ddiv(3.0, dmul(dmul(r2, r2), r));
    }
    double hinv = ddiv(1.0, h);
    double hinv2 = dmul(hinv, hinv);
    double hinv5 = dmul(dmul(hinv2, hinv2), hinv);
    double q = dmul(r, hinv);
    if (q <= 0.5) return dmul(dsub(76.8, dmul(96.0, q)), hinv5);
    double qinv = ddiv(1.0, q);
    double qinv3 = dmul(dmul(qinv, qinv), qinv);
    double t = dadd(dsub(dmul(48.0, qinv), 76.8), dmul(32.0, q));
    t = dsub(t, dmul(dmul(dmul(0.2, qinv3), qinv), qinv));
    return dmul(t, hinv5);
}

__device__ __forceinline__ double potential_kernel_x(double r, double h) {
    if (h == 0.0) return ddiv(-1.0, r);
    double hinv = ddiv(1.0, h);
    double q = dmul(r, hinv);
    if (q <= 0.5) {
        double in = dsub(dmul(6.4, q), 9.6);
        in = dadd(5.33333333333333333, dmul(dmul(q, q), in));
        return dmul(dadd(-2.8, dmul(dmul(q, q), in)), hinv);
    }
    if (q <= 1) {
        double in = dsub(9.6, dmul(2.1333333333333333333333, q));
        in = dadd(-16.0, dmul(q, in));
        in = dadd(10.666666666666666666666, dmul(q, in));
        double t = dadd(dadd(-3.2, ddiv(0.066666666666666666666, q)), dmul(dmul(q, q), in));
        return dmul(t, hinv);
    }
    return ddiv(-1.0, r);
}

constexpr int BF64_THREADS = 128;

template <int FIELDS, bool MUTUAL>
__global__ void __launch_bounds__(BF64_THREADS) k_bf64(const double *pt, const double *ht, int64_t nt,
                                                       const double *ps, const double *ms, const double *hs,
                                                       int64_t ns, double G, double *out, int W) {
    __shared__ double sx[BF64_THREADS], sy[BF64_THREADS], sz[BF64_THREADS], sm[BF64_THREADS], sh[BF64_THREADS];
    int64_t i = (int64_t)blockIdx.x * BF64_THREADS + threadIdx.x;
    bool valid = i < nt;
    double x = valid ? pt[3 * i] : 0.0, y = valid ? pt[3 * i + 1] : 0.0, z = valid ? pt[3 * i + 2] : 0.0;
    double hti = valid ? ht[i] : 0.0;
    double phi = 0.0, a0 = 0.0, a1 = 0.0, a2 = 0.0;
    double T0 = 0, T1 = 0, T2 = 0, T4 = 0, T5 = 0, T8 = 0;
    for (int64_t base = 0; base < ns; base += BF64_THREADS) {
        int64_t j = base + threadIdx.x;
        if (j < ns) {
            sx[threadIdx.x] = ps[3 * j];
            sy[threadIdx.x] = ps[3 * j + 1];
            sz[threadIdx.x] = ps[3 * j + 2];
            sm[threadIdx.x] = ms[j];
            sh[threadIdx.x] = hs[j];
        }
        __syncthreads();
        int lim = (int)((ns - base) < BF64_THREADS ? (ns - base) : BF64_THREADS);
        if (valid) {
            for (int k = 0; k < lim; k++) {
                int64_t jj = base + k;
                if (MUTUAL && jj == i) continue;
                double m = sm[k];
                if (FIELDS & BF_POT) {
                    double d0 = dsub(x, sx[k]), d1 = dsub(y, sy[k]), d2 = dsub(z, sz[k]);
                    double r = __dsqrt_rn(dadd(dadd(dmul(d0, d0), dmul(d1, d1)), dmul(d2, d2)));
                    if (MUTUAL) {
                        double h = pymax(hti, sh[k]);
                        if (r < h) phi = dadd(phi, dmul(m, potential_kernel_x(r, h)));
                        else if (r > 0) phi = dsub(phi, ddiv(m, r));
                    } else if (r != 0) {
                        double h = pymax(sh[k], hti);
                        if (r < h) phi = dadd(phi, dmul(m, potential_kernel_x(r, h)));
                        else phi = dsub(phi, ddiv(m, r));
                    }
                }
                if (FIELDS & (BF_ACC | BF_TID)) {
                    double d0 = dsub(sx[k], x), d1 = dsub(sy[k], y), d2 = dsub(sz[k], z);
                    double r2 = dadd(dadd(dmul(d0, d0), dmul(d1, d1)), dmul(d2, d2));
                    if (r2 == 0) continue;
                    double r = __dsqrt_rn(r2);
                    double h = pymax(hti, sh[k]);
                    if (FIELDS & BF_ACC) {
                        if (r < h) {
                            double km = dmul(force_kernel_x(r, h), m);
                            a0 = dadd(a0, dmul(km, d0));
                            a1 = dadd(a1, dmul(km, d1));
                            a2 = dadd(a2, dmul(km, d2));
                        } else {
                            double mf = dmul(m, ddiv(1.0, dmul(r2, r)));
                            a0 = dadd(a0, dmul(mf, d0));
                            a1 = dadd(a1, dmul(mf, d1));
                            a2 = dadd(a2, dmul(mf, d2));
                        }
                    }
                    if (FIELDS & BF_TID) {
                        double K, Q;
                        if (r < h) {
                            K = dmul(m, force_kernel_x(r, h));
                            Q = dmul(m, tidal_kernel_x(r, h));
                        } else {
                            K = ddiv(m, dmul(r, r2));
                            Q = ddiv(dmul(3.0, K), r2);
                        }
                        T0 = dadd(T0, dsub(dmul(dmul(Q, d0), d0), K));
                        T4 = dadd(T4, dsub(dmul(dmul(Q, d1), d1), K));
                        T8 = dadd(T8, dsub(dmul(dmul(Q, d2), d2), K));
                        T1 = dadd(T1, dmul(dmul(Q, d0), d1));
                        T2 = dadd(T2, dmul(dmul(Q, d0), d2));
                        T5 = dadd(T5, dmul(dmul(Q, d1), d2));
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!valid) return;
    double *o = out + i * W;
    int k = 0;
    if (FIELDS & BF_POT) o[k++] = dmul(G, phi);
    if (FIELDS & BF_ACC) {
        o[k] = dmul(G, a0);
        o[k + 1] = dmul(G, a1);
        o[k + 2] = dmul(G, a2);
        k += 3;
    }
    if (FIELDS & BF_TID) {
        double v[9] = {T0, T1, T2, T1, T4, T5, T2, T5, T8};
        for (int q = 0; q < 9; q++) o[k + q] = dmul(G, v[q]);
    }
}

// ---------------------------------------------------------------------------------------------
constexpr int BF32_THREADS = 256;
constexpr int BF32_TPT = 2;

template <int FIELDS>
__device__ __forceinline__ void bf32_pair(float m, float hs, float ht, float dx, float dy, float dz, bool skip,
                                          float *p) {
    float r2 = dx * dx + dy * dy + dz * dz;
    if (skip || !(r2 > 0.f)) return;
    float rinv = rsqrtf(r2);
    float r = r2 * rinv;
    float h = hs > ht ? hs : ht;
    float K, Q = 0.f;
    if (r < h) {
        float hinv = 1.f / h, q = r * hinv, h3 = hinv * hinv * hinv;
        if (FIELDS & BF_POT) {
            float pk;
            if (q <= 0.5f) pk = (-2.8f + q * q * (5.333333333f + q * q * (6.4f * q - 9.6f))) * hinv;
            else pk = (-3.2f + 0.0666666667f / q + q * q * (10.66666667f + q * (-16.0f + q * (9.6f - 2.133333333f * q)))) * hinv;
            p[0] += m * pk;
        }
        if (q <= 0.5f) K = (10.66666667f + q * q * (-38.4f + 32.0f * q)) * h3;
        else K = (21.333333333f - 48.0f * q + 38.4f * q * q - 10.666666667f * q * q * q - 0.066666666667f / (q * q * q)) * h3;
        K *= m;
        if (FIELDS & BF_TID) {
            float h5 = h3 * hinv * hinv;
            float tk;
            if (q <= 0.5f) tk = (76.8f - 96.0f * q) * h5;
            else {
                float qi = 1.f / q, qi3 = qi * qi * qi;
                tk = (48.0f * qi - 76.8f + 32.0f * q - 0.2f * qi3 * qi * qi) * h5;
            }
            Q = m * tk;
        }
    } else {
        float rinv2 = rinv * rinv, mr = m * rinv;
        if (FIELDS & BF_POT) p[0] -= mr;
        K = mr * rinv2;
        if (FIELDS & BF_TID) Q = 3.f * K * rinv2;
    }
    if (FIELDS & BF_ACC) {
        p[1] += K * dx;
        p[2] += K * dy;
        p[3] += K * dz;
    }
    if (FIELDS & BF_TID) {
        float qx = Q * dx, qy = Q * dy;
        p[4] += qx * dx - K;
        p[5] += qx * dy;
        p[6] += qx * dz;
        p[7] += qy * dy - K;
        p[8] += qy * dz;
        p[9] += Q * dz * dz - K;
    }
}

template <int FIELDS, bool MUTUAL>
__global__ void __launch_bounds__(BF32_THREADS) k_bf32(const double *pt, const double *ht, int64_t nt,
                                                       const double *ps, const double *ms, const double *hs,
                                                       int64_t ns, double G, double *out, int W) {
    __shared__ float4 spos[BF32_THREADS];
    __shared__ float sh[BF32_THREADS];
    float tx[BF32_TPT], ty[BF32_TPT], tz[BF32_TPT], th[BF32_TPT];
    int64_t ti[BF32_TPT];
    float S[BF32_TPT][10], C[BF32_TPT][10];
#pragma unroll
    for (int u = 0; u < BF32_TPT; u++) {
        ti[u] = ((int64_t)blockIdx.x * BF32_TPT + u) * BF32_THREADS + threadIdx.x;
        int64_t i = ti[u] < nt ? ti[u] : 0;
        tx[u] = (float)pt[3 * i];
        ty[u] = (float)pt[3 * i + 1];
        tz[u] = (float)pt[3 * i + 2];
        th[u] = (float)ht[i];
#pragma unroll
        for (int c = 0; c < 10; c++) S[u][c] = C[u][c] = 0.f;
    }
    for (int64_t base = 0; base < ns; base += BF32_THREADS) {
        int64_t j = base + threadIdx.x;
        if (j < ns) {
            spos[threadIdx.x] = make_float4((float)ps[3 * j], (float)ps[3 * j + 1], (float)ps[3 * j + 2], (float)ms[j]);
            sh[threadIdx.x] = (float)hs[j];
        }
        __syncthreads();
        int lim = (int)((ns - base) < BF32_THREADS ? (ns - base) : BF32_THREADS);
        float P[BF32_TPT][10];
#pragma unroll
        for (int u = 0; u < BF32_TPT; u++)
#pragma unroll
            for (int c = 0; c < 10; c++) P[u][c] = 0.f;
        for (int k = 0; k < lim; k++) {
            float4 s = spos[k];
            float hsk = sh[k];
#pragma unroll
            for (int u = 0; u < BF32_TPT; u++) {
                bool skip = MUTUAL && (base + k == ti[u]);
                bf32_pair<FIELDS>(s.w, hsk, th[u], s.x - tx[u], s.y - ty[u], s.z - tz[u], skip, P[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < BF32_TPT; u++)
#pragma unroll
            for (int c = 0; c < 10; c++) {
                float yv = P[u][c] - C[u][c];
                float tv = S[u][c] + yv;
                C[u][c] = (tv - S[u][c]) - yv;
                S[u][c] = tv;
            }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < BF32_TPT; u++) {
        if (ti[u] >= nt) continue;
        double *o = out + ti[u] * W;
        double v[10];
        for (int c = 0; c < 10; c++) v[c] = G * ((double)S[u][c] - (double)C[u][c]);
        int k = 0;
        if (FIELDS & BF_POT) o[k++] = v[0];
        if (FIELDS & BF_ACC) {
            o[k] = v[1];
            o[k + 1] = v[2];
            o[k + 2] = v[3];
            k += 3;
        }
        if (FIELDS & BF_TID) {
            double tv[9] = {v[4], v[5], v[6], v[5], v[7], v[8], v[6], v[8], v[9]};
            for (int q = 0; q < 9; q++) o[k + q] = tv[q];
        }
    }
}

// Potential and/or acceleration, the main FP32 form: BF32S_LANES lanes share each pair of targets,
// lane q of the group taking the sources k = q (mod BF32S_LANES) of every shared-memory tile, so a
// target set of 1e5 still fills the GPU; the lanes' Kahan-compensated sums are combined at the end
// by a fixed pattern of shuffles (deterministic). The two targets of a lane are computed together
// with paired f32x2 arithmetic for every source outside both softening lengths (with a 1e-5 margin)
// and not coincident; any other source takes bf32_pair for each target.
constexpr int BF32S_THREADS = 256;
constexpr int BF32S_LANES = 4;
constexpr int BF32S_TARGETS = 2 * BF32S_THREADS / BF32S_LANES;  // per block

typedef unsigned long long bf2;
__device__ __forceinline__ bf2 bf2_pack(float a, float b) {
    bf2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void bf2_unpack(bf2 v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ bf2 bf2_fma(bf2 a, bf2 b, bf2 c) {
    bf2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ bf2 bf2_mul(bf2 a, bf2 b) {
    bf2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ bf2 bf2_sub(bf2 a, bf2 b) {
    bf2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

template <int FIELDS, bool MUTUAL>
__global__ void __launch_bounds__(BF32S_THREADS) k_bf32_split(const double *pt, const double *ht, int64_t nt,
                                                              const double *ps, const double *ms,
                                                              const double *hs, int64_t ns, double G,
                                                              double *out, int W) {
    __shared__ float4 spos[BF32S_THREADS];
    __shared__ float sh[BF32S_THREADS], sh2[BF32S_THREADS];
    const int q = threadIdx.x % BF32S_LANES;
    const int64_t pair = (int64_t)blockIdx.x * (BF32S_THREADS / BF32S_LANES) + threadIdx.x / BF32S_LANES;
    float tx[2], ty[2], tz[2], th[2], th2[2];
    int64_t ti[2];
    float S[2][4], C[2][4];
#pragma unroll
    for (int u = 0; u < 2; u++) {
        ti[u] = 2 * pair + u;
        const int64_t i = ti[u] < nt ? ti[u] : 0;
        tx[u] = (float)pt[3 * i];
        ty[u] = (float)pt[3 * i + 1];
        tz[u] = (float)pt[3 * i + 2];
        th[u] = (float)ht[i];
        th2[u] = th[u] * th[u];
#pragma unroll
        for (int c = 0; c < 4; c++) S[u][c] = C[u][c] = 0.f;
    }
    const bf2 TX = bf2_pack(tx[0], tx[1]), TY = bf2_pack(ty[0], ty[1]), TZ = bf2_pack(tz[0], tz[1]);
    for (int64_t base = 0; base < ns; base += BF32S_THREADS) {
        const int64_t j = base + threadIdx.x;
        if (j < ns) {
            const float hj = (float)hs[j];
            spos[threadIdx.x] = make_float4((float)ps[3 * j], (float)ps[3 * j + 1], (float)ps[3 * j + 2], (float)ms[j]);
            sh[threadIdx.x] = hj;
            sh2[threadIdx.x] = hj * hj;
        }
        __syncthreads();
        const int lim = (int)((ns - base) < BF32S_THREADS ? (ns - base) : BF32S_THREADS);
        bf2 ph = 0, ax = 0, ay = 0, az = 0;  // the two targets' tile sums (bit pattern 0 is +0.0f, +0.0f)
        float P[2][10];
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
            for (int c = 0; c < 10; c++) P[u][c] = 0.f;
        for (int k = q; k < lim; k += BF32S_LANES) {
            const float4 s = spos[k];
            const bf2 dx = bf2_sub(bf2_pack(s.x, s.x), TX), dy = bf2_sub(bf2_pack(s.y, s.y), TY);
            const bf2 dz = bf2_sub(bf2_pack(s.z, s.z), TZ);
            const bf2 r2 = bf2_fma(dz, dz, bf2_fma(dy, dy, bf2_mul(dx, dx)));
            float r20, r21;
            bf2_unpack(r2, r20, r21);
            const float hs2 = sh2[k];
            const float lim0 = fmaxf(hs2, th2[0]) * 1.00001f, lim1 = fmaxf(hs2, th2[1]) * 1.00001f;
            bool slow = !(r20 > lim0) || !(r21 > lim1) || !(r20 > 0.f) || !(r21 > 0.f);
            if (MUTUAL) slow = slow || base + k == ti[0] || base + k == ti[1];
            if (slow) {
                float d[3][2];
                bf2_unpack(dx, d[0][0], d[0][1]);
                bf2_unpack(dy, d[1][0], d[1][1]);
                bf2_unpack(dz, d[2][0], d[2][1]);
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const bool skip = MUTUAL && (base + k == ti[u]);
                    bf32_pair<FIELDS>(s.w, sh[k], th[u], d[0][u], d[1][u], d[2][u], skip, P[u]);
                }
            } else {
                const float r0 = rsqrtf(r20), r1 = rsqrtf(r21);
                const bf2 rinv = bf2_pack(r0, r1);
                const bf2 mr = bf2_mul(bf2_pack(s.w, s.w), rinv);
                if (FIELDS & BF_POT) ph = bf2_sub(ph, mr);
                if (FIELDS & BF_ACC) {
                    const bf2 K = bf2_mul(mr, bf2_mul(rinv, rinv));
                    ax = bf2_fma(K, dx, ax);
                    ay = bf2_fma(K, dy, ay);
                    az = bf2_fma(K, dz, az);
                }
            }
        }
        float a0, a1;
        if (FIELDS & BF_POT) {
            bf2_unpack(ph, a0, a1);
            P[0][0] += a0;
            P[1][0] += a1;
        }
        if (FIELDS & BF_ACC) {
            bf2_unpack(ax, a0, a1);
            P[0][1] += a0;
            P[1][1] += a1;
            bf2_unpack(ay, a0, a1);
            P[0][2] += a0;
            P[1][2] += a1;
            bf2_unpack(az, a0, a1);
            P[0][3] += a0;
            P[1][3] += a1;
        }
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float yv = P[u][c] - C[u][c];
                const float tv = S[u][c] + yv;
                C[u][c] = (tv - S[u][c]) - yv;
                S[u][c] = tv;
            }
        __syncthreads();
    }
    // the group's lanes combined in double, the same fixed pattern on every lane
#pragma unroll
    for (int u = 0; u < 2; u++) {
        double v[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            v[c] = (double)S[u][c] - (double)C[u][c];
#pragma unroll
            for (int o = 1; o < BF32S_LANES; o <<= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
        }
        if (q != 0 || ti[u] >= nt) continue;
        double *o = out + ti[u] * W;
        int k = 0;
        if (FIELDS & BF_POT) o[k++] = G * v[0];
        if (FIELDS & BF_ACC) {
            o[k] = G * v[1];
            o[k + 1] = G * v[2];
            o[k + 2] = G * v[3];
        }
    }
}

template <int FIELDS, bool MUTUAL>
static void launch_bf(int precision, const double *pt, const double *ht, int64_t nt, const double *ps,
                      const double *ms, const double *hs, int64_t ns, double G, double *out, int W, cudaStream_t st) {
    if (precision == TG_FP64) {
        { k_bf64<FIELDS, MUTUAL><<<div_up(nt, BF64_THREADS), BF64_THREADS, 0, st>>>(pt, ht, nt, ps, ms, hs, ns, G, out, W); tg::note_launch(); }
    } else if constexpr ((FIELDS & BF_TID) == 0) {
        { k_bf32_split<FIELDS, MUTUAL><<<div_up(nt, BF32S_TARGETS), BF32S_THREADS, 0, st>>>(pt, ht, nt, ps, ms, hs, ns,
                                                                                          G, out, W); tg::note_launch(); }
    } else {
        { k_bf32<FIELDS, MUTUAL><<<div_up(nt, BF32_THREADS * BF32_TPT), BF32_THREADS, 0, st>>>(pt, ht, nt, ps, ms, hs, ns,
                                                                                           G, out, W); tg::note_launch(); }
    }
}

template <bool MUTUAL>
static void dispatch_bf(int fields, int precision, const double *pt, const double *ht, int64_t nt, const double *ps,
                        const double *ms, const double *hs, int64_t ns, double G, double *out, int W, cudaStream_t st) {
    switch (fields) {
        case 1: launch_bf<1, MUTUAL>(precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st); break;
        case 2: launch_bf<2, MUTUAL>(precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st); break;
        case 3: launch_bf<3, MUTUAL>(precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st); break;
        case 4: launch_bf<4, MUTUAL>(precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st); break;
        case 5: launch_bf<5, MUTUAL>(precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st); break;
        case 6: launch_bf<6, MUTUAL>(precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st); break;
        default: launch_bf<7, MUTUAL>(precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st); break;
    }
}

tg_status run_bruteforce(const double *pt, const double *ht, int64_t nt, const double *ps, const double *ms,
                         const double *hs, int64_t ns, int fields, int mutual, double G, int precision, double *out,
                         cudaStream_t st) {
    int W = ((fields & BF_POT) ? 1 : 0) + ((fields & BF_ACC) ? 3 : 0) + ((fields & BF_TID) ? 9 : 0);
    if (nt <= 0) return TG_OK;
    if (mutual) dispatch_bf<true>(fields, precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st);
    else dispatch_bf<false>(fields, precision, pt, ht, nt, ps, ms, hs, ns, G, out, W, st);
    TG_CUDA(cudaGetLastError());
    return TG_OK;
}

}  // namespace tg
