// peaks.cu -- FMA-chain microbenchmarks of the CUDA-core pipes: the FP32,
// packed FP32-pair and FP64 rates that the compute-bound paths (the FP64
// parity path, the mixed-precision push in analytic fields, the
// Bulirsch-Stoer stepper) are read against.  MEASURED_PEAKS.json holds the
// HBM copy and tensor-core figures only.
//
// Every thread runs eight independent multiply-add chains (acc = acc * a + b,
// a < 1, so the values settle near b / (1 - a) and never overflow); one
// multiply-add counts as two floating-point operations.  The grid fills every
// SM with 32 warps; the result depends on the SM clock during the run.
#include "../../include/tp_gpu.h"
#include "tp_internal.h"
#include "tp_mixed.cuh"

using namespace tp;

namespace {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;
constexpr int kPeakBlocksPerSM = 4;

template <class T>
__global__ void __launch_bounds__(kPeakThreads) fma_chain_kernel(T a, T b, int iters, T* sink)
{
    T acc[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) acc[c] = (T)(threadIdx.x & 7) * (T)0.125 + (T)c;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = fma(acc[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += acc[c];
    if (s == (T)-1) sink[blockIdx.x] = s;  // never true: keeps the chains
}

// Packed FP32 pairs (fma.rn.f32x2): two multiply-adds per instruction.
__global__ void __launch_bounds__(kPeakThreads) fma2_chain_kernel(float a, float b, int iters, float* sink)
{
    uint64_t acc[kChains];
    const uint64_t a2 = mixed::pack_f2(a, a), b2 = mixed::pack_f2(b, b);
#pragma unroll
    for (int c = 0; c < kChains; c++) acc[c] = mixed::pack_f2((float)(threadIdx.x & 7) * 0.125f + c, (float)c);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = mixed::fma_f2(acc[c], a2, b2);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        float x, y;
        mixed::unpack_f2(acc[c], x, y);
        s += x + y;
    }
    if (s == -1.0f) sink[blockIdx.x] = s;
}

}  // namespace

// kind 0: FP32 fma; 1: FP64 fma; 2: packed FP32-pair fma.  *flops: the
// measured floating-point operations per second (multiply-add = 2), from
// CUDA events around one launch after a warm-up launch.  Returns 0, or -1
// with tp_last_error set.
extern "C" int tp_measure_fma_peak(int kind, double* flops)
{
    if (!ensure_init()) return -1;
    if (kind < 0 || kind > 2 || !flops) {
        set_error(6, "tp_measure_fma_peak: kind %d", kind);
        return -1;
    }
    const int blocks = g.num_sms * kPeakBlocksPerSM;
    // launches of several milliseconds at this part's rates (FP64 runs far slower)
    const int iters = kind == 1 ? (1 << 12) : (1 << 18);
    void* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = cuda_ok(cudaMalloc(&sink, sizeof(double) * blocks), "peak sink") &&
              cuda_ok(cudaEventCreate(&e0), "event") && cuda_ok(cudaEventCreate(&e1), "event");
    float ms = 0.0f;
    for (int rep = 0; rep < 2 && ok; rep++) {  // the first launch warms up
        ok = cuda_ok(cudaEventRecord(e0, g.stream), "event");
        if (kind == 0)
            fma_chain_kernel<float><<<blocks, kPeakThreads, 0, g.stream>>>(0.999f, 1e-3f, iters, (float*)sink);
        else if (kind == 1)
            fma_chain_kernel<double><<<blocks, kPeakThreads, 0, g.stream>>>(0.999, 1e-3, iters, (double*)sink);
        else
            fma2_chain_kernel<<<blocks, kPeakThreads, 0, g.stream>>>(0.999f, 1e-3f, iters, (float*)sink);
        ok = ok && cuda_ok(cudaGetLastError(), "peak kernel") && cuda_ok(cudaEventRecord(e1, g.stream), "event") &&
             cuda_ok(cudaEventSynchronize(e1), "peak sync") && cuda_ok(cudaEventElapsedTime(&ms, e0, e1), "time");
    }
    if (sink) cudaFree(sink);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (!ok) return -1;
    const double per_thread = 2.0 * kChains * iters * (kind == 2 ? 2 : 1);
    *flops = per_thread * blocks * kPeakThreads / (ms * 1e-3);
    return 0;
}
