// Shared definitions for the pytreegrav_gb300 CUDA sources (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pytreegrav_gb300.h"

namespace tg {

constexpr int MORTON_BITS = 21;
constexpr int TOP_SHIFT = 3 * (MORTON_BITS - 1);  // 60: shift of a fresh key's top digit
constexpr int MAX_LEVEL = MORTON_BITS;            // a run sharing all 63 key bits is level 21
constexpr int MORTON_MAX_ROUNDS = 3;
constexpr uint32_t FULL = 0xffffffffu;

// Launch geometry of the bounding-box kernel (k_bbox, tg_build.cu) and of the two-kernel radix
// passes (radix_hist / radix_scatter, tg_sort.cu), shared with every file that launches them
// (tg_noalloc.cu sizes its fixed scratch array from these).
constexpr int BB_THREADS = 256, BB_ITEMS = 8;   // k_bbox: 256 threads x 8 points per block
constexpr int RS_WARPS = 8;
constexpr int RS_THREADS = RS_WARPS * 32;
constexpr int RS_ROUNDS = 16;                   // keys per thread
constexpr int RS_WARP_KEYS = RS_ROUNDS * 32;    // 512 consecutive keys per warp
constexpr int RS_TILE = RS_WARPS * RS_WARP_KEYS;  // 4096 keys per CTA
constexpr int RS_BINS = 256;                    // 8-bit digits

void set_last_error(const char *where, cudaError_t e);
void set_last_error_msg(const char *msg);
const char *last_error();

#define TG_CUDA(call)                                     \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) {                          \
            tg::set_last_error(#call, e_);                \
            return e_ == cudaErrorMemoryAllocation ? TG_ERR_OOM : TG_ERR_CUDA; \
        }                                                 \
    } while (0)

#define TG_TRY(expr)                    \
    do {                                \
        tg_status s_ = (expr);          \
        if (s_ != TG_OK) return s_;     \
    } while (0)

// ---------------------------------------------------------------------------------------------
// Exact FP64 arithmetic. The build reproduces pytreegrav's float64 results bit for bit, so every
// operation there rounds once, in source order: explicit _rn intrinsics keep nvcc from fusing a
// multiply and an add into one FMA.
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
// Python's builtin max(a, b): a unless b > a.
__device__ __forceinline__ double pymax(double a, double b) { return b > a ? b : a; }
__device__ __forceinline__ float pymaxf(float a, float b) { return b > a ? b : a; }

// Order-preserving map from double to uint64 (for exact atomic min/max).
__device__ __forceinline__ unsigned long long dbl_to_ordered(double x) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double ordered_to_dbl(unsigned long long u) {
    u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)u);
}

// ---------------------------------------------------------------------------------------------
// Binary64 -> binary32 conversion in integer arithmetic, round to nearest, ties to even (IEEE 754
// convertFormat), with float subnormals and overflow to infinity. GB300 executes FP64
// instructions, conversions from double included, at a small fraction of its integer rate, so
// kernels that only repack FP64 data as FP32 convert with these. Each result is bit-identical to
// a hardware conversion without flush-to-zero.

// Bits of the binary32 nearest to mag * 2^e2 (mag < 2^62), with the given sign bit. *r and *shift
// receive the rounded significand before renormalisation and the count of low bits of mag it
// dropped (r * 2^(e2 + shift) is the result's magnitude; shift <= 0: exact).
__device__ __forceinline__ uint32_t f32_rne(uint64_t mag, int e2, uint32_t sign, uint64_t *r_out = nullptr,
                                            int *shift_out = nullptr) {
    if (mag == 0) {
        if (r_out) *r_out = 0, *shift_out = 0;
        return sign;
    }
    const int top = e2 + 63 - __clzll((long long)mag);  // mag * 2^e2 lies in [2^top, 2^(top+1))
    const int q = max(top - 23, -149);                    // exponent of the result's last bit
    const int shift = q - e2;
    uint64_t r;
    if (shift <= 0) r = mag << (-shift);  // exact: at most 24 significant bits
    else if (shift >= 63) r = 0;          // below half the smallest subnormal
    else {
        r = mag >> shift;
        const uint64_t rem = mag & ((1ull << shift) - 1), half = 1ull << (shift - 1);
        if (rem > half || (rem == half && (r & 1))) r++;
    }
    if (r_out) *r_out = r, *shift_out = shift;
    if (r == 0) return sign;
    int qq = q;
    if (r >> 24) r >>= 1, qq++;  // rounding carried into a new bit
    if (r >> 23) {               // normal
        const int ef = qq + 150;
        return ef >= 255 ? (sign | 0x7f800000u) : (sign | ((uint32_t)ef << 23) | (uint32_t)(r & 0x7fffffu));
    }
    return sign | (uint32_t)r;  // subnormal (q == -149)
}

// Infinity or quiet NaN (payload's top bits kept) for a double with the all-ones exponent.
__device__ __forceinline__ uint32_t f32_special(uint64_t u) {
    const uint32_t sign = (uint32_t)(u >> 32) & 0x80000000u;
    const uint64_t m = u & 0xfffffffffffffull;
    return m ? (sign | 0x7fc00000u | (uint32_t)(m >> 29)) : (sign | 0x7f800000u);
}

// Generic path: any double (zeros, subnormal and overflowing results, infinities, NaN).
static __device__ __noinline__ void d2f_split_slow(uint64_t u, float &hi, float &lo) {
    const int E = (int)((u >> 52) & 0x7ff);
    if (E == 0x7ff) {  // x - x is NaN for an infinity and a NaN alike
        hi = __uint_as_float(f32_special(u));
        lo = __uint_as_float(0x7fffffffu);
        return;
    }
    const uint32_t sign = (uint32_t)(u >> 32) & 0x80000000u;
    const uint64_t mag = E ? ((u & 0xfffffffffffffull) | (1ull << 52)) : (u & 0xfffffffffffffull);
    const int e2 = (E ? E : 1) - 1075;
    uint64_t r;
    int shift;
    const uint32_t hb = f32_rne(mag, e2, sign, &r, &shift);
    hi = __uint_as_float(hb);
    if ((hb & 0x7fffffffu) == 0x7f800000u) {  // overflow: x - inf
        lo = -hi;
        return;
    }
    const int64_t d = shift <= 0 ? 0 : (int64_t)mag - (int64_t)(r == 0 || shift >= 63 ? 0 : (r << shift));
    lo = d == 0 ? 0.f : __uint_as_float(f32_rne((uint64_t)(d < 0 ? -d : d), e2, sign ^ (d < 0 ? 0x80000000u : 0u)));
}

// hi = float(x), lo = float(x - (double)hi) (the FP64 difference is exact). Fast path for
// 2^-74 <= |x| < 2^127, where hi and a nonzero lo are both normal floats: hi keeps the top 23
// fraction bits, rounded on the 29 dropped ones; lo is those dropped bits less the rounding step,
// a signed integer below 2^28 in magnitude, converted exactly by two magic-number additions and
// one rounding FP32 add, then scaled by a power of two.
__device__ __forceinline__ void d2f_split(double x, float &hi, float &lo) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const uint32_t uh = (uint32_t)(u >> 32), ul = (uint32_t)u;
    const uint32_t E = (uh >> 20) & 0x7ffu;
    if (E - 949u > 1149u - 949u) {
        d2f_split_slow(u, hi, lo);
        return;
    }
    const uint32_t sign = uh & 0x80000000u;
    const uint32_t rest = ul & 0x1fffffffu;  // the 29 dropped fraction bits
    uint32_t b = (((uh & 0xfffffu) << 3) | (ul >> 29)) + ((E - 896u) << 23);
    const uint32_t up = (rest > 0x10000000u || (rest == 0x10000000u && (b & 1u))) ? 1u : 0u;
    b += up;  // a carry out of the fraction moves into the exponent
    hi = __uint_as_float(sign | b);
    const int32_t d = (int32_t)rest - (int32_t)(up << 29);  // (x - hi) / 2^(e - 52)
    const uint32_t ad = (uint32_t)(d < 0 ? -d : d);
    const float fa = (__uint_as_float(0x4b000000u | (ad >> 6)) - 8388608.f) * 64.f;  // exact
    const float fb = __uint_as_float(0x4b000000u | (ad & 63u)) - 8388608.f;          // exact
    const float f = __fadd_rn(fa, fb) * __uint_as_float((E - 948u) << 23);             // RNE(|d|) * 2^(e-52)
    lo = d == 0 ? 0.f : __uint_as_float(__float_as_uint(f) | (sign ^ (d < 0 ? 0x80000000u : 0u)));
}

// float(x) (the hi part of d2f_split).
__device__ __forceinline__ float d2f(double x) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const uint32_t uh = (uint32_t)(u >> 32), ul = (uint32_t)u;
    const uint32_t E = (uh >> 20) & 0x7ffu;
    if (E - 949u > 1149u - 949u) {
        float hi, lo;
        d2f_split_slow(u, hi, lo);
        return hi;
    }
    const uint32_t rest = ul & 0x1fffffffu;
    uint32_t b = (((uh & 0xfffffu) << 3) | (ul >> 29)) + ((E - 896u) << 23);
    b += (rest > 0x10000000u || (rest == 0x10000000u && (b & 1u))) ? 1u : 0u;
    return __uint_as_float((uh & 0x80000000u) | b);
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T u = __shfl_up_sync(FULL, v, o);
        if (lane_id() >= o) v += u;
    }
    return v;
}

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Device-wide helpers implemented in tg_scan.cu / tg_sort.cu.
tg_status exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *total_dev,
                             cudaStream_t s);
tg_status exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on the low `bits` bits of the keys. keys/vals are
// sorted in place (scratch buffers are allocated stream-ordered and freed before return). A tile
// look-back that does not complete within its bound sets *err (a device int the caller owns and
// reads back with its results; nonzero: the sort failed) and leaves keys[i] = i and vals[i] = i, a
// sorted, well-formed result, so every later kernel stays in bounds.
tg_status radix_sort_pairs(uint64_t *keys, uint32_t *vals, int64_t n, int bits, cudaStream_t s, int *err);

// Bounds of the library's bounded device loops, overridable (tg_set_loop_limits in the measurement
// header) so that tests can make each one run out; 0 selects the built-in bound. Process-wide.
struct LoopLimits {
    long long sort_spin = 0;      // polls of one look-back word in a radix pass
    long long walk_steps = 0;     // traversal steps of one group of a tree walk
    long long column_visits = 0;  // element visits of one column-density walk
    long long heavy_entries = 0;  // list entries after which a walk's group is split (see tg_walk.cu)
};
LoopLimits &loop_limits();

int num_sms();

// The unique id of the calling thread's current CUDA context (the driver's cuCtxGetCurrent and
// cuCtxGetId, reached through the runtime's entry-point query so that the library needs no link to
// the driver library), the runtime's context bound first if none is (as after a device reset), or
// 0 if that fails. A context made after a device reset has a new id, even where its handle is the
// old one's. Library state tied to a device (pooled streams, events and memory, cached addresses)
// is kept with the id of the context it belongs to and made again when the id changes.
unsigned long long current_cuda_context_id();

// Stream-ordered device allocation from the library's own memory pool on the current device.
// The pool keeps freed memory mapped for later calls, up to a quarter of the device's memory and at
// least TG_POOL_KEEP_BYTES: a build and a walk allocate and free their temporaries on every call, and
// memory above the threshold is unmapped at each synchronisation and mapped again by the next call
// (at 3.2e7 particles a build's temporaries exceed 4 GiB, and that cost ~10 ms per build).
// Free with cudaFreeAsync.
#ifndef TG_POOL_KEEP_BYTES
#define TG_POOL_KEEP_BYTES (4ull << 30)
#endif
cudaError_t dev_malloc(void **p, size_t bytes, cudaStream_t s);

// Streams (non-blocking) and events (timing or not) of the current device from a library-owned pool:
// a tree takes a side stream and up to four events and a walk two timing events on every call, and
// creating and destroying them cost host time between the GPU's launches. A released stream may
// still have work queued; work put on it later runs after that work. A released event may be
// recorded again; waits already enqueued on it are unaffected.
cudaError_t pool_stream(cudaStream_t *s);
void release_stream(cudaStream_t s);
// dev: the device the event was made on (-1: the current device). A stream or event of another
// device than the current one is destroyed instead of pooled.
cudaError_t pool_event(cudaEvent_t *e, bool timing);
void release_event(cudaEvent_t e, bool timing, int dev = -1);
int current_device_or(int fallback);

// A stream-ordered device array from dev_malloc, freed on `st` when it goes out of scope.
template <typename T>
struct DevArray {
    T *p = nullptr;
    cudaStream_t st = nullptr;
    explicit DevArray(cudaStream_t s) : st(s) {}
    ~DevArray() {
        if (p) cudaFreeAsync(p, st);
    }
    DevArray(const DevArray &) = delete;
    DevArray &operator=(const DevArray &) = delete;
    cudaError_t alloc(int64_t n) { return dev_malloc((void **)&p, sizeof(T) * (size_t)(n > 1 ? n : 1), st); }
};

// Counts kernel launches (every launch site calls it; read through tg_launch_count()).
void note_launch();
// Adjusts the count by delta: + the kernels of a replayed CUDA graph, - the launches recorded (not
// run) while capturing one.
void note_launches(int64_t delta);
int64_t launches_so_far();

}  // namespace tg
