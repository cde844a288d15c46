// Device-wide exclusive scans and a stable LSD radix sort of (uint64 key, uint32 value) pairs.
//
// The sort replaces pytreegrav's _radix_argsort (octree.py:101-132). Any stable sort of the keys
// yields the same permutation, which is what makes the GPU order bit-identical to the reference:
// 8-bit digits, one tile of 4096 keys per CTA, ranks made stable by processing each warp's slice
// in order with __match_any_sync, and per-(digit, tile) offsets from a digit-major scan.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

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

unsigned long long current_cuda_context_id() {
    using CtxGetCurrent = int (*)(void **);
    using CtxGetId = int (*)(void *, unsigned long long *);
    static CtxGetCurrent get = nullptr;
    static CtxGetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get = (CtxGetCurrent)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetId)p;
    });
    if (!get || !get_id) return 0;
    void *ctx = nullptr;
    if (get(&ctx) != 0) ctx = nullptr;
    if (!ctx) {  // none bound to this thread yet (or just reset): let the runtime bind its context
        cudaFree(nullptr);
        if (get(&ctx) != 0) ctx = nullptr;
    }
    unsigned long long id = 0;
    if (!ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

namespace {
constexpr int POOL_DEVICES = 64;
std::mutex g_res_mu;
// Per device: the context the pooled streams and events belong to, and the pools. After a device
// reset (a new context) the old handles are dropped, not reused.
struct ResPool {
    unsigned long long ctx = 0;  // context id
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events[2];  // [timing]
};
ResPool g_res[POOL_DEVICES];
int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= POOL_DEVICES) return -1;
    return dev;
}
// The pool of device dev for the current context (g_res_mu held).
ResPool &res_pool(int dev) {
    ResPool &r = g_res[dev];
    const unsigned long long ctx = current_cuda_context_id();
    if (ctx && !r.ctx) r.ctx = ctx;  // filled before the context could be identified
    if (ctx && r.ctx != ctx) {
        r.streams.clear();
        r.events[0].clear();
        r.events[1].clear();
        r.ctx = ctx;
    }
    return r;
}
}  // namespace

int current_device_or(int fallback) {
    int dev = 0;
    return cudaGetDevice(&dev) == cudaSuccess ? dev : fallback;
}

cudaError_t pool_stream(cudaStream_t *s) {
    const int dev = current_device();
    if (dev >= 0) {
        std::lock_guard<std::mutex> lock(g_res_mu);
        ResPool &r = res_pool(dev);
        if (!r.streams.empty()) {
            *s = r.streams.back();
            r.streams.pop_back();
            return cudaSuccess;
        }
    }
    return cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
}

void release_stream(cudaStream_t s) {
    if (!s) return;
    int dev = -1;
    // pooled only on the current device, whose context the pool's key is checked against
    if (cudaStreamGetDevice(s, &dev) != cudaSuccess || dev < 0 || dev >= POOL_DEVICES || dev != current_device()) {
        cudaStreamDestroy(s);
        return;
    }
    std::lock_guard<std::mutex> lock(g_res_mu);
    res_pool(dev).streams.push_back(s);
}

cudaError_t pool_event(cudaEvent_t *e, bool timing) {
    const int dev = current_device();
    if (dev >= 0) {
        std::lock_guard<std::mutex> lock(g_res_mu);
        auto &v = res_pool(dev).events[timing ? 1 : 0];
        if (!v.empty()) {
            *e = v.back();
            v.pop_back();
            return cudaSuccess;
        }
    }
    return cudaEventCreateWithFlags(e, timing ? cudaEventDefault : cudaEventDisableTiming);
}

void release_event(cudaEvent_t e, bool timing, int dev) {
    if (!e) return;
    const int cur = current_device();
    if (dev < 0) dev = cur;
    if (dev < 0 || dev >= POOL_DEVICES || dev != cur) {  // pooled only on the current device (as streams)
        cudaEventDestroy(e);
        return;
    }
    std::lock_guard<std::mutex> lock(g_res_mu);
    res_pool(dev).events[timing ? 1 : 0].push_back(e);
}

cudaError_t dev_malloc(void **p, size_t bytes, cudaStream_t s) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mu;
    static cudaMemPool_t pools[MAX_DEVICES] = {};
    static unsigned long long pool_ctx[MAX_DEVICES] = {};  // context ids: a device reset makes a new context
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaMallocAsync(p, bytes, s);
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lock(mu);
        const unsigned long long ctx = current_cuda_context_id();
        if (pools[dev] && ctx && !pool_ctx[dev]) pool_ctx[dev] = ctx;          // made before a context was bound
        if (pools[dev] && ctx && pool_ctx[dev] != ctx) pools[dev] = nullptr;  // the old pool died with its context
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
            pool_ctx[dev] = current_cuda_context_id();
            size_t free_b = 0, total_b = 0;
            unsigned long long keep = TG_POOL_KEEP_BYTES;
            if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && total_b / 4 > keep) keep = total_b / 4;
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
// RS_* (tile geometry of the two-kernel passes) are defined in tg_common.cuh.

// Per-warp stable ranking of the warp's ROUNDS * 32 keys; leaves per-warp digit counts in wcount.
// kv: the slice's keys, one per round, loaded here up front (one memory round trip per slice) and
// left to the caller.
template <int ROUNDS>
__device__ __forceinline__ void rank_loaded_slice(const uint64_t *kv, int64_t n, int64_t wbase, int shift,
                                                  int *wcount, int *digit, int *rank);

template <int ROUNDS = RS_ROUNDS>
__device__ __forceinline__ void rank_warp_slice(const uint64_t *keys, int64_t n, int64_t wbase, int shift,
                                                int *wcount, int *digit, int *rank, uint64_t *kv) {
    const int lane = lane_id();
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int64_t i = wbase + r * 32 + lane;
        kv[r] = i < n ? __ldg(keys + i) : 0ull;
    }
    rank_loaded_slice<ROUNDS>(kv, n, wbase, shift, wcount, digit, rank);
}

template <int ROUNDS>
__device__ __forceinline__ void rank_loaded_slice(const uint64_t *kv, int64_t n, int64_t wbase, int shift,
                                                  int *wcount, int *digit, int *rank) {
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    // every round's lanes with the same digit first, from nine ballots (the eight digit bits and
    // "in range"); independent of the counters, so the rounds overlap
    unsigned peers[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int64_t i = wbase + r * 32 + lane;
        const bool in = i < n;
        const int d = in ? (int)((kv[r] >> shift) & (RS_BINS - 1)) : RS_BINS;  // RS_BINS: past the end
        unsigned m = __ballot_sync(FULL, in);
        m = in ? m : ~m;
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const bool bit = (d >> b) & 1;
            const unsigned v = __ballot_sync(FULL, bit);
            m &= bit ? v : ~v;
        }
        peers[r] = m;
        digit[r] = d;
    }
    // then the per-warp digit counters, round by round
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int d = digit[r];
        const int base = (d < RS_BINS) ? wcount[d] : 0;
        __syncwarp();
        if (d < RS_BINS && (31 - __clz(peers[r])) == lane) wcount[d] = base + __popc(peers[r]);
        __syncwarp();
        rank[r] = base + __popc(peers[r] & lt);
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
    uint64_t kv[RS_ROUNDS];
    rank_warp_slice(keys, n, wbase, shift, wcount[w], digit, rank, kv);
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
    uint64_t kv[RS_ROUNDS];
    rank_warp_slice(keys, n, wbase, shift, wcount[w], digit, rank, kv);
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
            keys_out[pos] = kv[r];
            vals_out[pos] = vals[i];
        }
    }
}

// ---------------------------------------------------------------------------------------------
// One-sweep passes (decoupled look-back). All digit histograms come from one read of the keys;
// then each pass is one kernel: a CTA takes the next tile from an atomic counter (so every earlier
// tile belongs to a CTA that is already running), ranks its keys stably as above, publishes its
// per-digit count, looks back over earlier tiles' published words for its exclusive prefix, and
// scatters. A look-back spin is bounded; running out sets the sort's own error word instead of
// hanging, and the sort then leaves the identity permutation (k_sort_fallback).

constexpr int MAX_PASSES = 8;
#ifndef TG_OS_ROUNDS
#define TG_OS_ROUNDS 8
#endif
#ifndef TG_OS_LB
#define TG_OS_LB 4
#endif
constexpr int OS_ROUNDS = TG_OS_ROUNDS;             // keys per thread in a one-sweep pass
constexpr int OS_WARP_KEYS = OS_ROUNDS * 32;
constexpr int OS_TILE = RS_WARPS * OS_WARP_KEYS;   // 2048 keys per CTA (8 per thread; measured against 2, 4 and 16)
// A status word: flag (bits 62-63: aggregate or inclusive), the pass it belongs to (bits 56-61, pass + 1),
// value (bits 0-55). Words of an earlier pass read as not yet published, so the status array is
// cleared once per sort rather than once per pass.
constexpr unsigned long long ST_AGG = 1ull << 62, ST_INC = 2ull << 62, ST_FLAGS = 3ull << 62;
constexpr unsigned long long ST_TAGS = 63ull << 56, ST_VAL = (1ull << 56) - 1;
constexpr long long SPIN_LIMIT = 1ll << 22;
constexpr int LB = TG_OS_LB;  // predecessors read per look-back round trip

__global__ void __launch_bounds__(256) k_sort_hist_all(const uint64_t *keys, int64_t n, int npass, int *hist) {
    __shared__ int h[MAX_PASSES * RS_BINS];
    for (int i = threadIdx.x; i < npass * RS_BINS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        for (int p = 0; p < npass; p++) atomicAdd(&h[p * RS_BINS + (int)((k >> (8 * p)) & (RS_BINS - 1))], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npass * RS_BINS; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// Exclusive scan of each pass's 256 digit counts, in place. One block of 256 threads.
__global__ void k_sort_digit_offsets(int *hist, int npass) {
    __shared__ int tot;
    for (int p = 0; p < npass; p++) {
        int v = hist[p * RS_BINS + threadIdx.x];
        int ex = block_exclusive_scan(v, &tot);
        hist[p * RS_BINS + threadIdx.x] = ex;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(RS_THREADS, 4) k_onesweep(const uint64_t *keys, const uint32_t *vals, int64_t n,
                                                         int shift, int pass, const int *digit_off,
                                                         unsigned long long *status, int *tile_counter,
                                                         uint64_t *keys_out, uint32_t *vals_out, int *err,
                                                         long long spin_limit) {
    const unsigned long long tag = (unsigned long long)(pass + 1) << 56;
    __shared__ int wcount[RS_WARPS][RS_BINS];
    __shared__ int prefix[RS_BINS];
    __shared__ int lstart[RS_BINS];  // the digit's first position within the tile
    __shared__ uint64_t skey[OS_TILE];
    __shared__ uint32_t sval[OS_TILE];
    __shared__ int tile_s;
    if (threadIdx.x == 0) tile_s = atomicAdd(tile_counter, 1);
    for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) (&wcount[0][0])[i] = 0;
    __syncthreads();
    const int t = tile_s;
    const int w = threadIdx.x >> 5;
    const int64_t wbase = (int64_t)t * OS_TILE + (int64_t)w * OS_WARP_KEYS;
    int digit[OS_ROUNDS], rank[OS_ROUNDS];
    uint64_t kv[OS_ROUNDS];
    uint32_t vv[OS_ROUNDS];  // values loaded with the keys, so the scatter reads nothing from memory
    {
        const int lane = lane_id();
#pragma unroll
        for (int r = 0; r < OS_ROUNDS; r++) {
            const int64_t i = wbase + r * 32 + lane;
            kv[r] = i < n ? __ldg(keys + i) : 0ull;
            vv[r] = i < n ? __ldg(vals + i) : 0u;
        }
    }
    rank_loaded_slice<OS_ROUNDS>(kv, n, wbase, shift, wcount[w], digit, rank);
    __syncthreads();
    {  // one thread per digit: offsets of the warps within the tile, then the tile's prefix
        const int d = threadIdx.x;
        int run = 0;
#pragma unroll
        for (int ww = 0; ww < RS_WARPS; ww++) {
            int c = wcount[ww][d];
            wcount[ww][d] = run;
            run += c;
        }
        volatile unsigned long long *st = status + (int64_t)t * RS_BINS + d;
        long long acc = 0;
        if (t == 0) {
            *st = ST_INC | tag | (unsigned long long)run;
        } else {
            *st = ST_AGG | tag | (unsigned long long)run;
            // earlier tiles publish their aggregate without waiting on anyone, so each wait ends
            // once that tile's CTA (already running: it took its tile before this one) has ranked.
            // The words of LB predecessors are read together (independent loads, one round trip),
            // then summed in order up to the first inclusive one.
            bool done = false;
            for (int64_t j = t - 1; j >= 0 && !done; j -= LB) {
                unsigned long long w[LB];
#pragma unroll
                for (int k = 0; k < LB; k++)
                    w[k] = j - k >= 0 ? ((const volatile unsigned long long *)status)[(j - k) * RS_BINS + d] : 0ull;
#pragma unroll
                for (int k = 0; k < LB; k++) {
                    if (done || j - k < 0) break;
                    unsigned long long wd = w[k];
                    const volatile unsigned long long *src = status + (j - k) * RS_BINS + d;
                    auto ready = [tag](unsigned long long x) { return (x & ST_FLAGS) && (x & ST_TAGS) == tag; };
                    for (long long spins = 0; !ready(wd) && spins < spin_limit; spins++) wd = *src;
                    if (!ready(wd)) {
                        atomicExch(err, 1);
                        done = true;
                        break;
                    }
                    acc += (long long)(wd & ST_VAL);
                    if ((wd & ST_FLAGS) == ST_INC) done = true;
                }
            }
            *st = ST_INC | tag | (unsigned long long)(acc + run);
        }
        prefix[d] = digit_off[d] + (int)acc;
        __shared__ int tot_s;
        lstart[d] = block_exclusive_scan(run, &tot_s);
    }
    __syncthreads();
    // the tile in digit order in shared memory, then written out: keys of one digit go to consecutive
    // places, so consecutive threads write consecutive words instead of one scattered sector each
    const int lane = lane_id();
#pragma unroll
    for (int r = 0; r < OS_ROUNDS; r++) {
        const int64_t i = wbase + r * 32 + lane;
        if (i < n) {
            const int loc = lstart[digit[r]] + wcount[w][digit[r]] + rank[r];
            skey[loc] = kv[r];
            sval[loc] = vv[r];
        }
    }
    __syncthreads();
    const int64_t rest = n - (int64_t)t * OS_TILE;
    const int cnt = rest < OS_TILE ? (int)rest : OS_TILE;
    for (int i = threadIdx.x; i < cnt; i += RS_THREADS) {
        const uint64_t k = skey[i];
        const int d = (int)((k >> shift) & (RS_BINS - 1));
        const int pos = prefix[d] + (i - lstart[d]);
        keys_out[pos] = k;
        vals_out[pos] = sval[i];
    }
}

// After the passes: if a look-back gave up (some keys went to wrong places, some places were never
// written), every value becomes its own index and every key its own position -- sorted pairs and a
// valid permutation, so every later kernel sees well-formed input -- and the caller's flag is set.
__global__ void k_sort_fallback(uint64_t *keys, uint32_t *vals, int64_t n, const int *local_err, int *err) {
    if (!*local_err) return;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 == 0) atomicExch(err, 1);
    for (int64_t i = i0; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = (uint64_t)i;
        vals[i] = (uint32_t)i;
    }
}

tg_status radix_sort_pairs(uint64_t *keys, uint32_t *vals, int64_t n, int bits, cudaStream_t s, int *err) {
    if (n <= 1 || bits <= 0) return TG_OK;
    if (n > (int64_t)0x7fffffff || !err) return TG_ERR_BAD_ARG;
    const long long spin_limit = loop_limits().sort_spin > 0 ? loop_limits().sort_spin : SPIN_LIMIT;
    const int ntiles = div_up(n, OS_TILE);
    const int npass = std::min((bits + 7) / 8, MAX_PASSES);
    uint64_t *k2 = nullptr;
    uint32_t *v2 = nullptr;
    unsigned char *scr = nullptr;
    const size_t st_bytes = sizeof(unsigned long long) * (size_t)ntiles * RS_BINS;
    const size_t hist_bytes = sizeof(int) * MAX_PASSES * RS_BINS;
    TG_CUDA(tg::dev_malloc((void **)&k2, sizeof(uint64_t) * n, s));
    TG_CUDA(tg::dev_malloc((void **)&v2, sizeof(uint32_t) * n, s));
    TG_CUDA(tg::dev_malloc((void **)&scr, st_bytes + hist_bytes + sizeof(int) * (MAX_PASSES + 1), s));
    unsigned long long *status = (unsigned long long *)scr;
    int *hist = (int *)(scr + st_bytes);
    int *counters = hist + MAX_PASSES * RS_BINS;
    int *local_err = counters + MAX_PASSES;
    TG_CUDA(cudaMemsetAsync(scr, 0, st_bytes + hist_bytes + sizeof(int) * (MAX_PASSES + 1), s));
    const int hblocks = (int)std::min<int64_t>(div_up(n, 256 * 16), (int64_t)num_sms() * 4);
    { k_sort_hist_all<<<hblocks, 256, 0, s>>>(keys, n, npass, hist); tg::note_launch(); }
    { k_sort_digit_offsets<<<1, RS_BINS, 0, s>>>(hist, npass); tg::note_launch(); }
    uint64_t *kin = keys, *kout = k2;
    uint32_t *vin = vals, *vout = v2;
    for (int p = 0; p < npass; p++) {
        { k_onesweep<<<ntiles, RS_THREADS, 0, s>>>(kin, vin, n, 8 * p, p, hist + p * RS_BINS, status, counters + p, kout,
                                                   vout, local_err, spin_limit); tg::note_launch(); }
        TG_CUDA(cudaGetLastError());
        uint64_t *tk = kin; kin = kout; kout = tk;
        uint32_t *tv = vin; vin = vout; vout = tv;
    }
    if (kin != keys) {
        TG_CUDA(cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, s));
        TG_CUDA(cudaMemcpyAsync(vals, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    }
    { k_sort_fallback<<<std::min(div_up(n, 256), 4 * num_sms()), 256, 0, s>>>(keys, vals, n, local_err, err); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaFreeAsync(k2, s));
    TG_CUDA(cudaFreeAsync(v2, s));
    TG_CUDA(cudaFreeAsync(scr, s));
    return TG_OK;
}

}  // namespace tg
