// Measurement utilities: kernel-launch counter and an FP32 FMA-throughput probe (the roofline
// denominator for the FP32-bound walk; see include/pytreegrav_gb300_measure.h).
#include <atomic>

#include "../../include/pytreegrav_gb300_measure.h"
#include "tg_common.cuh"

namespace tg {
static std::atomic<int64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(int64_t delta) { g_launches.fetch_add(delta, std::memory_order_relaxed); }
int64_t launches_so_far() { return g_launches.load(); }
static LoopLimits g_limits;
LoopLimits &loop_limits() { return g_limits; }
}  // namespace tg

namespace {
constexpr int FMA_ITERS = 4096;
constexpr int FMA_CHAINS = 8;

__global__ void __launch_bounds__(256) k_fma_probe(float *sink, float a, float b) {
    float v[FMA_CHAINS];
#pragma unroll
    for (int c = 0; c < FMA_CHAINS; c++) v[c] = threadIdx.x * 1e-3f + c;
    for (int i = 0; i < FMA_ITERS; i++) {
#pragma unroll
        for (int c = 0; c < FMA_CHAINS; c++) v[c] = fmaf(v[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < FMA_CHAINS; c++) s += v[c];
    if (s == 1234.5f) sink[0] = s;  // never true in practice; keeps the chains live
}

__global__ void k_check_conversion(const double *x, int64_t n, unsigned long long *bad) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float hw = __double2float_rn(v), hwlo = __double2float_rn(v - (double)hw);
    float hi, lo;
    tg::d2f_split(v, hi, lo);
    const float one = tg::d2f(v);
    // equal bits, or NaN where the hardware gives NaN (its payload is not specified)
    auto same = [](float a, float b) { return __float_as_uint(a) == __float_as_uint(b) || (b != b && a != a); };
    if (!same(one, hw) || !same(hi, hw) || !same(lo, hwlo)) atomicAdd(bad, 1ull);
}
}  // namespace

extern "C" {

int64_t tg_launch_count(void) { return tg::g_launches.load(); }

int tg_measure_fp32_fma(double *tflops, double *ms, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    float *sink = nullptr;
    TG_CUDA(cudaMalloc((void **)&sink, sizeof(float)));
    int per_sm = 0;
    TG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fma_probe, 256, 0));
    const int blocks = per_sm * tg::num_sms() * 4;
    cudaEvent_t e0, e1;
    TG_CUDA(cudaEventCreate(&e0));
    TG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
        TG_CUDA(cudaEventRecord(e0, st));
        k_fma_probe<<<blocks, 256, 0, st>>>(sink, 0.999999f, 1e-7f);
        TG_CUDA(cudaEventRecord(e1, st));
        TG_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        TG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        if (rep > 0 && t < best) best = t;  // first launch is warm-up
    }
    double flops = 2.0 * FMA_ITERS * FMA_CHAINS * 256.0 * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    *ms = best;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return TG_OK;
}

int tg_check_f32_conversion(const double *x, int64_t n, int64_t *mismatches, void *stream) {
    if (!mismatches || n < 0 || (n > 0 && !x)) return TG_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long *bad = nullptr;
    TG_CUDA(tg::dev_malloc((void **)&bad, sizeof(unsigned long long), st));
    TG_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st));
    if (n > 0) {
        k_check_conversion<<<tg::div_up(n, 256), 256, 0, st>>>(x, n, bad);
        tg::note_launch();
    }
    unsigned long long h = 0;
    TG_CUDA(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, st));
    TG_CUDA(cudaFreeAsync(bad, st));
    TG_CUDA(cudaStreamSynchronize(st));
    *mismatches = (int64_t)h;
    return TG_OK;
}

}  // extern "C"

extern "C" int tg_set_loop_limits(int64_t sort_spin, int64_t walk_steps, int64_t column_visits,
                                  int64_t heavy_entries) {
    tg::LoopLimits &l = tg::loop_limits();
    l.sort_spin = sort_spin > 0 ? sort_spin : 0;
    l.walk_steps = walk_steps > 0 ? walk_steps : 0;
    l.column_visits = column_visits > 0 ? column_visits : 0;
    l.heavy_entries = heavy_entries > 0 ? heavy_entries : 0;
    return 0;
}
