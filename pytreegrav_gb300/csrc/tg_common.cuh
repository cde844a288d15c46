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
// sorted in place (scratch buffers are allocated stream-ordered and freed before return).
tg_status radix_sort_pairs(uint64_t *keys, uint32_t *vals, int64_t n, int bits, cudaStream_t s);
// After a synchronisation: TG_ERR_QUEUE_TIMEOUT (and the flag cleared) if a sort's look-back ran
// out of its bound since the last check.
tg_status sort_error_check();
// The same flag taken into *dst (device) on `st` and cleared, without a synchronisation.
tg_status sort_error_take(int *dst, cudaStream_t st);

int num_sms();

// Stream-ordered device allocation from the library's own memory pool on the current device.
// The pool keeps up to TG_POOL_KEEP_BYTES of freed memory mapped for later calls (a build and a
// walk allocate and free their temporaries on every call; with the driver's default threshold of
// zero, that memory would be unmapped at each synchronisation and mapped again by the next call).
// Free with cudaFreeAsync.
#ifndef TG_POOL_KEEP_BYTES
#define TG_POOL_KEEP_BYTES (4ull << 30)
#endif
cudaError_t dev_malloc(void **p, size_t bytes, cudaStream_t s);

// Counts kernel launches (every launch site calls it; read through tg_launch_count()).
void note_launch();
// Adjusts the count by delta: + the kernels of a replayed CUDA graph, - the launches recorded (not
// run) while capturing one.
void note_launches(int64_t delta);
int64_t launches_so_far();

}  // namespace tg
