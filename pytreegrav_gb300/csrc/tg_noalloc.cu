// tg_morton_order_noalloc: the Morton ordering of tg_morton_order without any device allocation.
//
// Who needs it: code that runs where cudaMalloc (or cudaMallocAsync, or torch's caching allocator)
// is not available or not allowed -- a host that hands this library pre-allocated device buffers
// from its own pool and forbids allocations behind its back, a process whose device memory is
// already fully reserved by another allocator, or a caller that must not take the allocator's
// locks or implicit synchronisations on a latency-critical path. Such a caller passes device
// buffers for the input and the output, and every temporary the ordering needs lives in one
// fixed array compiled into this library.
//
// The scratch array is a file-scope __device__ variable, so the CUDA runtime reserves it on every
// GPU that loads this library, for the life of the process: TG_NOALLOC_SCRATCH_BYTES (about 6 MB),
// which bounds n at TG_NOALLOC_MAX_POINTS (2^18 = 262,144 points). Larger n is rejected.
//
// Every call on a device shares that device's one array, and the array keeps what the previous
// call left in it: the call clears what must start at zero itself. Two calls whose GPU work
// overlaps (different streams, or different host threads, without ordering between them) race on
// the array and produce garbage; callers must order such calls, e.g. on one stream.
//
// The first call on each device looks up the array's device address (cudaGetSymbolAddress, which
// may load this library's device code on that device); do that first call before any stream
// capture is begun on the device.
//
// The work is the same as tg_morton_order's, reusing its kernels: bounding cube and keys from
// tg_build.cu, stable 8-bit LSD radix passes from tg_sort.cu; only the per-pass scan of the digit
// counts is done here, by one CTA, because the library's device-wide scan allocates its partial
// sums. The permutation is therefore identical to tg_morton_order's.
#include <cstdio>
#include <mutex>

#include "tg_common.cuh"

namespace tg {

// Kernels defined in tg_build.cu (bounding cube, Morton keys) and tg_sort.cu (radix passes).
__global__ void k_bbox(const double *pos, int64_t n, const int64_t *sys_off, int nsys, unsigned long long *mn,
                       unsigned long long *mx);
__global__ void k_bbox_finish(const unsigned long long *mn, const unsigned long long *mx, int nsys, double *center,
                              double *size);
__global__ void k_keys(const double *pos, int64_t n, const int64_t *sys_off, int nsys, const double *center,
                       const double *size, uint64_t *keys, uint64_t *keys_copy, uint32_t *vals);
__global__ void radix_hist(const uint64_t *keys, int64_t n, int shift, int ntiles, int *hist);
__global__ void radix_scatter(const uint64_t *keys, const uint32_t *vals, int64_t n, int shift, int ntiles,
                              const int *offs, uint64_t *keys_out, uint32_t *vals_out);

namespace {

// Launch geometry those kernels are written for, taken from their own definitions (tg_common.cuh):
// k_bbox covers BB_THREADS x BB_ITEMS points per block; the radix kernels run RS_THREADS-thread CTAs
// over tiles of RS_TILE keys with RS_BINS digit bins.
constexpr int BBOX_THREADS = BB_THREADS, BBOX_POINTS = BB_THREADS * BB_ITEMS;
constexpr int SORT_THREADS = RS_THREADS, SORT_TILE = RS_TILE, SORT_BINS = RS_BINS;
static_assert(SORT_BINS == 256, "the passes below take 8-bit digits (shift += 8)");
constexpr int KEY_BITS = 63;

constexpr int64_t MAX_POINTS = TG_NOALLOC_MAX_POINTS;
constexpr int MAX_TILES = (int)((MAX_POINTS + SORT_TILE - 1) / SORT_TILE);
constexpr int64_t HIST_INTS = (int64_t)SORT_BINS * MAX_TILES;

// Byte offsets of the pieces of the scratch array, each 256-byte aligned.
constexpr int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }
constexpr int64_t OFF_KEYS0 = 0;
constexpr int64_t OFF_KEYS1 = OFF_KEYS0 + align256(8 * MAX_POINTS);
constexpr int64_t OFF_VALS0 = OFF_KEYS1 + align256(8 * MAX_POINTS);
constexpr int64_t OFF_VALS1 = OFF_VALS0 + align256(4 * MAX_POINTS);
constexpr int64_t OFF_HIST = OFF_VALS1 + align256(4 * MAX_POINTS);
constexpr int64_t OFF_MIN = OFF_HIST + align256(4 * HIST_INTS);   // 3 x u64
constexpr int64_t OFF_MAX = OFF_MIN + 256;                         // 3 x u64
constexpr int64_t OFF_CENTER = OFF_MAX + 256;                      // 3 x f64
constexpr int64_t OFF_SIZE = OFF_CENTER + 256;                     // 1 x f64
constexpr int64_t OFF_SYSOFF = OFF_SIZE + 256;                     // 2 x i64: {0, n}
constexpr int64_t OFF_FLAG = OFF_SYSOFF + 256;                     // 1 x int: non-finite input seen
constexpr int64_t SCRATCH_BYTES = OFF_FLAG + 256;
static_assert(SCRATCH_BYTES == TG_NOALLOC_SCRATCH_BYTES, "scratch size stated in the header is stale");

// The scratch array. In host code `g_noalloc_scratch` names a host-side shadow, not device
// memory: the host obtains the device address with cudaGetSymbolAddress (scratch_on_current_device).
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_addr_mutex;
// The address looked up on each device, with the CUDA context it belongs to: after a device reset
// (cudaDeviceReset, or a reset of the primary context by the host application) the context is a
// new one and the address is looked up again.
struct ScratchAddr {
    unsigned long long ctx = 0;  // context id
    unsigned char *addr = nullptr;
};
ScratchAddr g_addr[MAX_DEVICES];

// Device address of the scratch array on the current device, looked up once per device and context.
tg_status scratch_on_current_device(unsigned char **out) {
    int dev = 0;
    TG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) {
        set_last_error_msg("tg_morton_order_noalloc: device ordinal beyond the 64 this library tracks");
        return TG_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    ScratchAddr &c = g_addr[dev];
    const unsigned long long ctx = current_cuda_context_id();
    if (!c.addr || !ctx || c.ctx != ctx) {
        void *p = nullptr;
        TG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));  // makes the device's context current if needed
        c.addr = (unsigned char *)p;
        c.ctx = current_cuda_context_id();
    }
    *out = c.addr;
    return TG_OK;
}

// Resets what each call must find at zero (or at its identity): the non-finite flag and the
// bounding-box min/max words; writes the single-system offsets {0, n}.
__global__ void k_noalloc_prep(int64_t n, int *flag, unsigned long long *mn, unsigned long long *mx,
                               int64_t *sys_off) {
    int t = threadIdx.x;
    if (t < 3) {
        mn[t] = ~0ull;
        mx[t] = 0ull;
    }
    if (t == 0) {
        *flag = 0;
        sys_off[0] = 0;
        sys_off[1] = n;
    }
}

__global__ void k_noalloc_nonfinite(const double *a, int64_t n, int *flag) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !isfinite(a[i])) atomicOr(flag, 1);
}

// In-place exclusive scan of the digit-major counts (at most HIST_INTS ints) by one CTA.
constexpr int HSCAN_THREADS = 1024;
constexpr int HSCAN_ITEMS = 16;

__global__ void __launch_bounds__(HSCAN_THREADS) k_noalloc_hist_scan(int *h, int count) {
    __shared__ int warp_tot[HSCAN_THREADS / 32];
    __shared__ int carry_s;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < count; base += HSCAN_THREADS * HSCAN_ITEMS) {
        int i0 = base + threadIdx.x * HSCAN_ITEMS;
        int v[HSCAN_ITEMS];
        int sum = 0;
#pragma unroll
        for (int k = 0; k < HSCAN_ITEMS; k++) {
            v[k] = (i0 + k < count) ? h[i0 + k] : 0;
            sum += v[k];
        }
        int inc = warp_inclusive_scan(sum);
        if (lane == 31) warp_tot[w] = inc;
        __syncthreads();
        if (w == 0) {
            int s = warp_tot[lane];
            int si = warp_inclusive_scan(s);
            warp_tot[lane] = si - s;
        }
        __syncthreads();
        int carry = carry_s;
        int run = carry + warp_tot[w] + inc - sum;
#pragma unroll
        for (int k = 0; k < HSCAN_ITEMS; k++) {
            if (i0 + k < count) h[i0 + k] = run;
            run += v[k];
        }
        __syncthreads();
        if (threadIdx.x == HSCAN_THREADS - 1) carry_s = run;  // the last thread's running sum ends the tile
        __syncthreads();
    }
}

__global__ void k_noalloc_widen(const uint32_t *a, int64_t n, int64_t *b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}


// Accepts only memory the kernels can read on the current device: device or managed allocations.
tg_status require_device_pointer(const void *p, int dev, const char *what) {
    cudaPointerAttributes a;
    TG_CUDA(cudaPointerGetAttributes(&a, p));
    bool ok = a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
    if (!ok) {
        char msg[160];
        snprintf(msg, sizeof(msg), "tg_morton_order_noalloc: %s is not device memory of the current device", what);
        set_last_error_msg(msg);
        return TG_ERR_BAD_ARG;
    }
    return TG_OK;
}

}  // namespace
}  // namespace tg

extern "C" tg_status tg_morton_order_noalloc(const double *pos, int64_t n, int64_t *perm, void *stream) {
    using namespace tg;
    if (n < 0 || (n > 0 && (!pos || !perm))) {
        set_last_error_msg("tg_morton_order_noalloc: n must be >= 0 and pos, perm non-null");
        return TG_ERR_BAD_ARG;
    }
    if (n > MAX_POINTS) {
        char msg[200];
        snprintf(msg, sizeof(msg),
                 "tg_morton_order_noalloc: n = %lld exceeds the fixed scratch capacity of %lld points "
                 "(TG_NOALLOC_MAX_POINTS); use tg_morton_order",
                 (long long)n, (long long)MAX_POINTS);
        set_last_error_msg(msg);
        return TG_ERR_BAD_ARG;
    }
    if (n == 0) return TG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    TG_CUDA(cudaGetDevice(&dev));
    TG_TRY(require_device_pointer(pos, dev, "pos"));
    TG_TRY(require_device_pointer(perm, dev, "perm"));
    unsigned char *s = nullptr;
    TG_TRY(scratch_on_current_device(&s));
    uint64_t *keys[2] = {(uint64_t *)(s + OFF_KEYS0), (uint64_t *)(s + OFF_KEYS1)};
    uint32_t *vals[2] = {(uint32_t *)(s + OFF_VALS0), (uint32_t *)(s + OFF_VALS1)};
    int *hist = (int *)(s + OFF_HIST);
    unsigned long long *mn = (unsigned long long *)(s + OFF_MIN), *mx = (unsigned long long *)(s + OFF_MAX);
    double *center = (double *)(s + OFF_CENTER), *size = (double *)(s + OFF_SIZE);
    int64_t *sys_off = (int64_t *)(s + OFF_SYSOFF);
    int *flag = (int *)(s + OFF_FLAG);

    // Reject non-finite coordinates before ordering, as tg_morton_order does.
    { k_noalloc_prep<<<1, 32, 0, st>>>(n, flag, mn, mx, sys_off); tg::note_launch(); }
    { k_noalloc_nonfinite<<<div_up(3 * n, 256), 256, 0, st>>>(pos, 3 * n, flag); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    int hflag = 0;
    TG_CUDA(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaStreamSynchronize(st));
    if (hflag) return TG_ERR_NONFINITE;

    // Bounding cube and keys, then stable radix passes over the 63 key bits.
    { k_bbox<<<div_up(n, BBOX_POINTS), BBOX_THREADS, 0, st>>>(pos, n, sys_off, 1, mn, mx); tg::note_launch(); }
    { k_bbox_finish<<<1, 32, 0, st>>>(mn, mx, 1, center, size); tg::note_launch(); }
    { k_keys<<<div_up(n, 256), 256, 0, st>>>(pos, n, sys_off, 1, center, size, keys[0], nullptr, vals[0]); tg::note_launch(); }
    const int ntiles = div_up(n, SORT_TILE);
    int cur = 0;
    for (int shift = 0; shift < KEY_BITS; shift += 8) {
        { radix_hist<<<ntiles, SORT_THREADS, 0, st>>>(keys[cur], n, shift, ntiles, hist); tg::note_launch(); }
        { k_noalloc_hist_scan<<<1, HSCAN_THREADS, 0, st>>>(hist, SORT_BINS * ntiles); tg::note_launch(); }
        { radix_scatter<<<ntiles, SORT_THREADS, 0, st>>>(keys[cur], vals[cur], n, shift, ntiles, hist, keys[cur ^ 1],
                                                         vals[cur ^ 1]); tg::note_launch(); }
        cur ^= 1;
    }
    { k_noalloc_widen<<<div_up(n, 256), 256, 0, st>>>(vals[cur], n, perm); tg::note_launch(); }
    TG_CUDA(cudaGetLastError());
    TG_CUDA(cudaStreamSynchronize(st));
    return TG_OK;
}
