// tc_gemm.cu -- one 128-row tile of D = A * B^T on the 5th-generation tensor
// cores (tcgen05.mma, BF16 operands in 128-byte-swizzled shared memory, FP32
// accumulator in tensor memory).  A self-check of the tensor-core building
// blocks that the learned field model's inference uses.
#include <cstring>

#include "../../include/tp_gpu.h"
#include "tc_sm100.cuh"
#include "tp_internal.h"

namespace tp {
namespace tc {

constexpr int kRows = 128;
constexpr uint32_t kWaitLimit = 1u << 22;

__global__ void __launch_bounds__(kRows, 1) tile_gemm_kernel(const __nv_bfloat16* __restrict__ A,
                                                             const __nv_bfloat16* __restrict__ B,
                                                             float* __restrict__ D, int n, int k,
                                                             int* __restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    // 1024-byte aligned operand tiles
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
    unsigned char* a_s = smem_raw + pad;
    unsigned char* b_s = a_s + (size_t)kRows * k * 2;
    for (int c = tid; c < kRows * (k / 8); c += kRows) {
        const int r = c / (k / 8), kk = (c % (k / 8)) * 8;
        *reinterpret_cast<uint4*>(a_s + sw128_offset(kRows, r, kk)) =
            *reinterpret_cast<const uint4*>(A + (size_t)r * k + kk);
    }
    for (int c = tid; c < n * (k / 8); c += kRows) {
        const int r = c / (k / 8), kk = (c % (k / 8)) * 8;
        *reinterpret_cast<uint4*>(b_s + sw128_offset(n, r, kk)) =
            *reinterpret_cast<const uint4*>(B + (size_t)r * k + kk);
    }
    fence_async_smem();
    if (tid == 0) {
        mbar_init(smem_addr(&bar), 1);
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(smem_addr(&tmem_slot), 256);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (tid == 0) {
        const uint32_t idesc = idesc_bf16_f32(kRows, n);
        const uint32_t a0 = smem_addr(a_s), b0 = smem_addr(b_s);
        for (int ka = 0; ka < k / 64; ka++)
            for (int kk = 0; kk < 4; kk++)
                mma_bf16(tmem, desc_sw128(a0 + ka * kRows * 128 + kk * 32),
                         desc_sw128(b0 + ka * n * 128 + kk * 32), idesc, (ka | kk) != 0);
        mma_commit(smem_addr(&bar));
    }
    const bool ok = mbar_wait(smem_addr(&bar), 0, kWaitLimit);
    if (!ok && (tid & 31) == 0) atomicOr(status, ST_TIMEOUT);
    tc_fence_after();
    if (ok) {
        const int row = tid;
        for (int c = 0; c < n; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int i = 0; i < 16; i++) D[(size_t)row * n + c + i] = v[i];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

}  // namespace tc
}  // namespace tp

using namespace tp;

// D[128][n] = A[128][k] * B[n][k]^T with BF16 inputs (raw 16-bit patterns) and
// FP32 output; n a multiple of 16 in [16, 256], k a multiple of 64 in [64, 256].
extern "C" int tp_tc_gemm_bf16(int n, int k, const unsigned short* a, const unsigned short* b, float* d)
{
    if (n < 16 || n > 256 || n % 16 || k < 64 || k > 256 || k % 64 || !a || !b || !d) {
        set_error(6, "tp_tc_gemm_bf16: n must be 16..256 in steps of 16, k 64..256 in steps of 64");
        return -1;
    }
    if (!ensure_init()) return -1;
    cudaStream_t s = g.stream;
    const size_t sa = sizeof(uint16_t) * 128 * k, sb = sizeof(uint16_t) * n * k, sd = sizeof(float) * 128 * n;
    void *dA = nullptr, *dB = nullptr, *dD = nullptr;
    bool ok = cuda_ok(cudaMalloc(&dA, sa), "A") && cuda_ok(cudaMalloc(&dB, sb), "B") &&
              cuda_ok(cudaMalloc(&dD, sd), "D");
    const size_t smem = 1024 + sa + sb;
    if (ok) ok = cuda_ok(cudaFuncSetAttribute(tc::tile_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem), "smem attr");
    if (ok) {
        cudaMemcpyAsync(dA, a, sa, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dB, b, sb, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(dD, 0, sd, s);
        tc::tile_gemm_kernel<<<1, tc::kRows, smem, s>>>(static_cast<const __nv_bfloat16*>(dA),
                                                        static_cast<const __nv_bfloat16*>(dB),
                                                        static_cast<float*>(dD), n, k, g.d_status);
        ok = cuda_ok(cudaGetLastError(), "tile gemm");
    }
    if (ok) {
        cudaMemcpyAsync(d, dD, sd, cudaMemcpyDeviceToHost, s);
        ok = cuda_ok(cudaStreamSynchronize(s), "tile gemm sync");
    }
    if (dA) cudaFree(dA);
    if (dB) cudaFree(dB);
    if (dD) cudaFree(dD);
    return ok ? 0 : -1;
}
