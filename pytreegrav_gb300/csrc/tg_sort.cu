// Device-wide exclusive scans and a stable LSD radix sort of (uint64 key, uint32 value) pairs.
//
// The sort replaces pytreegrav's _radix_argsort (octree.py:101-132). Any stable sort of the keys
// yields the same permutation, which is what makes the GPU order bit-identical to the reference:
// 8-bit digits, one tile of 4096 keys per CTA, ranks made stable by processing each warp's slice
// in order with __match_any_sync, and per-(digit, tile) offsets from a digit-major scan.
#include <cstdio>
#include <mutex>

#include "tg_common.cuh"

namespace tg {

static thread_local char g_err[512] = "";

void set_last_error(const char *where, cudaError_t e) {
    snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(e));
}
void set_last_error_msg(const char *msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }
const char *last_error() { return g_err; }

int num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

cudaError_t dev_malloc(void **p, size_t bytes, cudaStream_t s) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mu;
    static cudaMemPool_t pools[MAX_DEVICES] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaMallocAsync(p, bytes, s);
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            e = cudaMemPoolCreate(&pools[dev], &props);
            if (e != cudaSuccess) {
                pools[dev] = nullptr;
                return e;
            }
            unsigned long long keep = TG_POOL_KEEP_BYTES;
            e = cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
            if (e != cudaSuccess) return e;
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// ---------------------------------------------------------------------------------------------
// Exclusive scan: block sums -> scan of block sums (one CTA) -> per-block scan plus carry.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ T block_exclusive_scan(T v, T *total) {
    __shared__ T warp_sums[SCAN_THREADS / 32];
    T inc = warp_inclusive_scan(v);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 31) warp_sums[w] = inc;
    __syncthreads();
    if (w == 0) {
        T s = (l < SCAN_THREADS / 32) ? warp_sums[l] : T(0);
        T si = warp_inclusive_scan(s);
        if (l < SCAN_THREADS / 32) warp_sums[l] = si - s;
        if (l == SCAN_THREADS / 32 - 1) *total = si;
    }
    __syncthreads();
    T r = warp_sums[w] + inc - v;
    __syncthreads();
    return r;
}

template <typename T>
__global__ void scan_block_sums(const T *in, int64_t n, T *sums) {
    __shared__ T tot;
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    T v = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++)
        if (base + i < n) v += in[base + i];
    block_exclusive_scan(v, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void scan_sums_single(T *sums, int64_t nb, T *total) {
    __shared__ T tot;
    T carry = 0;
    for (int64_t base = 0; base < nb; base += SCAN_TILE) {
        int64_t i0 = base + (int64_t)threadIdx.x * SCAN_ITEMS;
        T vals[SCAN_ITEMS];
        T v = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            vals[i] = (i0 + i < nb) ? sums[i0 + i] : T(0);
            v += vals[i];
        }
        T ex = block_exclusive_scan(v, &tot) + carry;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; i++) {
            if (i0 + i < nb) sums[i0 + i] = ex;
            ex += vals[i];
        }
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

template <typename T>
__global__ void scan_apply(const T *in, T *out, int64_t n, const T *sums) {
    __shared__ T tot;
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    T vals[SCAN_ITEMS];
    T v = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        vals[i] = (base + i < n) ? in[base + i] : T(0);
        v += vals[i];
    }
    T ex = block_exclusive_scan(v, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        if (base + i < n) out[base + i] = ex;
        ex += vals[i];
    }
}

template <typename T>
static tg_status exclusive_scan(const T *in, T *out, int64_t n, T *total_dev, cudaStream_t s) {
    if (n <= 0) {
        if (total_dev) TG_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(T), s));
        return TG_OK;
    }
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    T *sums = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&sums, sizeof(T) * nb, s));
    { scan_block_sums<T><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums); tg::note_launch(); }
    { scan_sums_single<T><<<1, SCAN_THREADS, 0, s>>>(sums, nb, total_dev); tg::note_launch(); }
    { scan_apply<T><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, sums); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaFreeAsync(sums, s));
    return TG_OK;
}

tg_status exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *total_dev, cudaStream_t s) {
    return exclusive_scan<long long>((const long long *)in, (long long *)out, n, (long long *)total_dev, s);
}
tg_status exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s) {
    return exclusive_scan<int>(in, out, n, nullptr, s);
}

// ---------------------------------------------------------------------------------------------
// Radix sort.
constexpr int RS_WARPS = 8;
constexpr int RS_THREADS = RS_WARPS * 32;
constexpr int RS_ROUNDS = 16;                      // keys per thread
constexpr int RS_WARP_KEYS = RS_ROUNDS * 32;       // 512 consecutive keys per warp
constexpr int RS_TILE = RS_WARPS * RS_WARP_KEYS;   // 4096 keys per CTA
constexpr int RS_BINS = 256;

// Per-warp stable ranking of the warp's 512 keys; leaves per-warp digit counts in wcount.
__device__ __forceinline__ void rank_warp_slice(const uint64_t *keys, int64_t n, int64_t wbase, int shift,
                                                int *wcount, int *digit, int *rank) {
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        int64_t i = wbase + r * 32 + lane;
        int d = RS_BINS;  // sentinel for keys past the end
        if (i < n) d = (int)((keys[i] >> shift) & (RS_BINS - 1));
        unsigned peers = __match_any_sync(FULL, d);
        int base = (d < RS_BINS) ? wcount[d] : 0;
        __syncwarp();
        if (d < RS_BINS && (31 - __clz(peers)) == lane) wcount[d] = base + __popc(peers);
        __syncwarp();
        digit[r] = d;
        rank[r] = base + __popc(peers & lt);
    }
}

__global__ void __launch_bounds__(RS_THREADS) radix_hist(const uint64_t *keys, int64_t n, int shift, int ntiles,
                                                         int *hist) {
    __shared__ int wcount[RS_WARPS][RS_BINS];
    for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) (&wcount[0][0])[i] = 0;
    __syncthreads();
    int w = threadIdx.x >> 5;
    int64_t wbase = (int64_t)blockIdx.x * RS_TILE + (int64_t)w * RS_WARP_KEYS;
    int digit[RS_ROUNDS], rank[RS_ROUNDS];
    rank_warp_slice(keys, n, wbase, shift, wcount[w], digit, rank);
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
        int s = 0;
#pragma unroll
        for (int ww = 0; ww < RS_WARPS; ww++) s += wcount[ww][d];
        hist[(int64_t)d * ntiles + blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(RS_THREADS) radix_scatter(const uint64_t *keys, const uint32_t *vals, int64_t n,
                                                            int shift, int ntiles, const int *offs,
                                                            uint64_t *keys_out, uint32_t *vals_out) {
    __shared__ int wcount[RS_WARPS][RS_BINS];
    for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) (&wcount[0][0])[i] = 0;
    __syncthreads();
    int w = threadIdx.x >> 5;
    int64_t wbase = (int64_t)blockIdx.x * RS_TILE + (int64_t)w * RS_WARP_KEYS;
    int digit[RS_ROUNDS], rank[RS_ROUNDS];
    rank_warp_slice(keys, n, wbase, shift, wcount[w], digit, rank);
    __syncthreads();
    // warp offsets within the tile, then the tile's global offset per digit
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
        int run = offs[(int64_t)d * ntiles + blockIdx.x];
#pragma unroll
        for (int ww = 0; ww < RS_WARPS; ww++) {
            int c = wcount[ww][d];
            wcount[ww][d] = run;
            run += c;
        }
    }
    __syncthreads();
    const int lane = lane_id();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        int64_t i = wbase + r * 32 + lane;
        if (i < n) {
            int pos = wcount[w][digit[r]] + rank[r];
            keys_out[pos] = keys[i];
            vals_out[pos] = vals[i];
        }
    }
}

tg_status radix_sort_pairs(uint64_t *keys, uint32_t *vals, int64_t n, int bits, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return TG_OK;
    if (n > (int64_t)0x7fffffff) return TG_ERR_BAD_ARG;
    int ntiles = div_up(n, RS_TILE);
    uint64_t *k2 = nullptr;
    uint32_t *v2 = nullptr;
    int *hist = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&k2, sizeof(uint64_t) * n, s));
    TG_CUDA(tg::dev_malloc((void **)&v2, sizeof(uint32_t) * n, s));
    TG_CUDA(tg::dev_malloc((void **)&hist, sizeof(int) * (int64_t)RS_BINS * ntiles, s));
    uint64_t *kin = keys, *kout = k2;
    uint32_t *vin = vals, *vout = v2;
    for (int shift = 0; shift < bits; shift += 8) {
        { radix_hist<<<ntiles, RS_THREADS, 0, s>>>(kin, n, shift, ntiles, hist); tg::note_launch(); }
        TG_TRY(exclusive_scan_i32(hist, hist, (int64_t)RS_BINS * ntiles, s));
        { radix_scatter<<<ntiles, RS_THREADS, 0, s>>>(kin, vin, n, shift, ntiles, hist, kout, vout); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
        uint64_t *tk = kin; kin = kout; kout = tk;
        uint32_t *tv = vin; vin = vout; vout = tv;
    }
    if (kin != keys) {
        TG_CUDA(cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, s));
        TG_CUDA(cudaMemcpyAsync(vals, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    }
    TG_CUDA(cudaFreeAsync(k2, s));
    TG_CUDA(cudaFreeAsync(v2, s));
    TG_CUDA(cudaFreeAsync(hist, s));
    return TG_OK;
}

}  // namespace tg
