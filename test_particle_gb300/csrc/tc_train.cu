// tc_train.cu -- the GEMMs of the learned field model's training on the
// 5th-generation tensor cores: C[M][N] = sum_k A[m][k] B[n][k], both operands
// BF16 and K-major in global memory (row-major with K contiguous), FP32
// accumulation in tensor memory, and a fused epilogue per use (bias + SiLU of
// the forward pass, the SiLU derivative of the backward pass, split-K
// partial sums of the weight gradients).
//
// One CTA of 128 threads computes a 128 x N tile (N <= 256) over a range of
// K: the K range streams through a ring of RING shared-memory stages, one
// k-atom (64 values of K) per stage, A (128 rows) and B (N rows) in the
// 128-byte-swizzled K-major layout of tc_sm100.cuh.  Every thread copies its
// share of a stage with 16-byte cp.async; once a stage has landed one thread
// issues its four K = 16 MMAs (M = 128, N) and commits them to the stage's
// mbarrier, which frees the stage for the copy RING - 1 atoms ahead.  After
// the last atom the four warps read their 32 accumulator lanes (rows) with
// tcgen05.ld, 32 columns at a time, and hand them to the epilogue.  Every
// mbarrier wait is bounded; a wait that runs out raises ST_TIMEOUT, the CTA
// skips its stores, drains its MMAs (bounded) and frees its tensor memory.
// Long K ranges (the weight gradients) use 4 stages; short ones (K <= 256:
// four atoms) use 2, which halves the shared memory so that two CTAs share
// an SM and one's epilogue overlaps the other's copies and MMAs.
#include <algorithm>
#include <cstdint>

#include "../../include/tp_gpu.h"
#include "mlp_common.cuh"
#include "tc_sm100.cuh"
#include "tc_train.cuh"
#include "tp_internal.h"

namespace tp {
namespace tct {

constexpr int kThreads = 128;
constexpr uint32_t kWaitLimit = 1u << 22;

__host__ __device__ constexpr uint32_t a_stage_bytes() { return 128u * 128u; }
__host__ __device__ constexpr uint32_t b_stage_bytes(int n) { return (uint32_t)n * 128u; }
#ifndef TP_TCT_SHORT_RING
#define TP_TCT_SHORT_RING 2
#endif
__host__ __device__ constexpr int ring_for(int k_atoms) { return k_atoms <= 4 ? TP_TCT_SHORT_RING : 4; }
size_t smem_bytes(int n, int ring) { return 1024 + (size_t)ring * (a_stage_bytes() + b_stage_bytes(n)); }

// one k-atom of A (128 rows from m0) and B (n rows) into a stage
__device__ __forceinline__ void load_stage(const __nv_bfloat16* __restrict__ A, int lda, int m0,
                                           const __nv_bfloat16* __restrict__ B, int ldb, int n, int k0,
                                           uint32_t sa, uint32_t sb)
{
    const int tid = threadIdx.x;
    for (int c = tid; c < 128 * 8; c += kThreads) {
        const int r = c >> 3, kk = (c & 7) * 8;
        const __nv_bfloat16* src = A + (size_t)(m0 + r) * lda + k0 + kk;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa + tc::sw128_offset(128, r, kk)),
                     "l"(src)
                     : "memory");
    }
    for (int c = tid; c < n * 8; c += kThreads) {
        const int r = c >> 3, kk = (c & 7) * 8;
        const __nv_bfloat16* src = B + (size_t)r * ldb + k0 + kk;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sb + tc::sw128_offset(n, r, kk)),
                     "l"(src)
                     : "memory");
    }
}

template <int RING, class Epi>
__global__ void __launch_bounds__(kThreads, 1) tcgemm_kernel(const __nv_bfloat16* __restrict__ A, int lda,
                                                             const __nv_bfloat16* __restrict__ B, int ldb,
                                                             int N, int kchunk, int K, Epi epi,
                                                             int* __restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[RING + 1];
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * 128;
    const int kbeg = blockIdx.y * kchunk, kend = min(K, kbeg + kchunk);
    const int nk = (kend - kbeg) / 64;
    const uint32_t raw = tc::smem_addr(smem_raw);
    const uint32_t base = raw + ((1024u - (raw & 1023u)) & 1023u);
    const uint32_t sa0 = base, sb0 = base + RING * a_stage_bytes();
    const uint32_t bar0 = tc::smem_addr(&bars[0]), done = tc::smem_addr(&bars[RING]);
    const uint32_t ncols = N <= 32 ? 32u : N <= 64 ? 64u : N <= 128 ? 128u : 256u;
    if (tid == 0) {
        for (int s = 0; s <= RING; s++) tc::mbar_init(bar0 + 8 * s, 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_addr(&tmem_slot), ncols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16_f32(128, N);
    bool ok = true;
    // prologue: the first RING - 1 atoms
    for (int s = 0; s < RING - 1; s++) {
        if (s < nk)
            load_stage(A, lda, m0, B, ldb, N, kbeg + 64 * s, sa0 + s * a_stage_bytes(), sb0 + s * b_stage_bytes(N));
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    for (int kc = 0; kc < nk; kc++) {
        const int s = kc % RING;
        asm volatile("cp.async.wait_group %0;" ::"n"(RING - 2) : "memory");
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0 && ok) {
            tc::tc_fence_after();
            const uint64_t ad = tc::desc_sw128(sa0 + s * a_stage_bytes());
            const uint64_t bd = tc::desc_sw128(sb0 + s * b_stage_bytes(N));
#pragma unroll
            for (int kk = 0; kk < 4; kk++) tc::mma_bf16(tmem, ad + 2 * kk, bd + 2 * kk, idesc, (kc | kk) != 0);
            tc::mma_commit(bar0 + 8 * s);
        }
        const int nxt = kc + RING - 1;
        if (nxt < nk) {
            if (kc >= 1) {  // the stage's previous atom (kc - 1) must have been consumed
                const int sp = (kc - 1) % RING;
                if (!tc::mbar_wait(bar0 + 8 * sp, (uint32_t)((kc - 1) / RING) & 1u, kWaitLimit)) ok = false;
            }
            if (ok)
                load_stage(A, lda, m0, B, ldb, N, kbeg + 64 * nxt, sa0 + (nxt % RING) * a_stage_bytes(),
                           sb0 + (nxt % RING) * b_stage_bytes(N));
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    ok = __syncthreads_and(ok) != 0;
    if (tid == 0) tc::mma_commit(done);
    // operands of the epilogue that do not depend on the MMAs (the SiLU
    // derivative's pre-activations) are loaded while they finish
    Epi e = epi;
    if (ok && nk > 0) e.begin(m0 + tid);
    const bool fine = tc::mbar_wait(done, 0, kWaitLimit);
    if (!(ok && fine) && (tid & 31) == 0) atomicOr(status, ST_TIMEOUT);
    tc::tc_fence_after();
    if (ok && fine && nk > 0) {
        const int row = m0 + tid;
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        if (N >= 32) {
            // 32 columns at a time (unrolled, so that per-row values an
            // epilogue holds stay in registers); a last chunk of 16 (N an odd
            // multiple of 16) reads 16 columns past N inside the allocation
            // and hands on only the 16 that exist
#pragma unroll
            for (int c = 0; c < 256; c += 32) {
                if (c < N) {
                    float v[32];
                    tc::tmem_ld32(tmem + lane_base + (uint32_t)c, v);
                    e(row, c, v, min(32, N - c));
                }
            }
        } else {
            float v[32];
            tc::tmem_ld16(tmem + lane_base, v);
            e(row, 0, v, 16);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

template <int RING, class Epi>
static cudaError_t launch_ring(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int N,
                               int K, int kchunk, int splits, const Epi& epi, int* status, cudaStream_t s)
{
    const size_t smem = smem_bytes(N, RING);
    cudaError_t e = cudaFuncSetAttribute(tcgemm_kernel<RING, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(M / 128, splits);
    tcgemm_kernel<RING, Epi><<<grid, kThreads, smem, s>>>(A, lda, B, ldb, N, kchunk, K, epi, status);
    return cudaGetLastError();
}

template <class Epi>
static cudaError_t launch(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int N, int K,
                          int splits, const Epi& epi, int* status, cudaStream_t s)
{
    if (M % 128 || N % 16 || N < 16 || N > 256 || K % 64 || K < 64 || splits < 1) return cudaErrorInvalidValue;
    int kchunk = (K / 64 + splits - 1) / splits * 64;
    splits = (K + kchunk - 1) / kchunk;
    if (ring_for(kchunk / 64) == 2) return launch_ring<2>(A, lda, B, ldb, M, N, K, kchunk, splits, epi, status, s);
    return launch_ring<4>(A, lda, B, ldb, M, N, K, kchunk, splits, epi, status, s);
}

// ---------------------------------------------------------------- epilogues
// Each gets 32 (or 16) consecutive columns c0.. of row m.
struct EpiStoreF32 {  // D[m][n] = acc (self-check)
    float* D;
    int ld;
    template <int CW = 256>
    __device__ void begin(int, int = 0) {}
    __device__ void operator()(int m, int c0, const float* v, int cnt) const
    {
        for (int i = 0; i < cnt; i++) D[(size_t)m * ld + c0 + i] = v[i];
    }
};

// z = acc + b; Z, H = silu(z) row-major [M][256] and H transposed [256][M]
struct EpiHiddenT {
    const float* b;
    __nv_bfloat16 *Z, *H, *HT;
    int M;
    template <int CW = 256>
    __device__ void begin(int, int = 0) {}
    __device__ void operator()(int m, int c0, const float* v, int cnt) const
    {
#pragma unroll
        for (int i = 0; i < 32; i += 8) {
            uint32_t zp[4], hp[4];
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
                const float z0 = v[i + j] + b[c0 + i + j], z1 = v[i + j + 1] + b[c0 + i + j + 1];
                zp[j / 2] = mlp::pack_bf16(z0, z1);
                hp[j / 2] = mlp::pack_bf16(mlp::silu(z0), mlp::silu(z1));
            }
            *reinterpret_cast<uint4*>(Z + (size_t)m * mlp::kHid + c0 + i) = make_uint4(zp[0], zp[1], zp[2], zp[3]);
            *reinterpret_cast<uint4*>(H + (size_t)m * mlp::kHid + c0 + i) = make_uint4(hp[0], hp[1], hp[2], hp[3]);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const uint32_t w = hp[j / 2];
                reinterpret_cast<unsigned short*>(HT)[(size_t)(c0 + i + j) * M + m] =
                    (unsigned short)((j & 1) ? (w >> 16) : (w & 0xffffu));
            }
        }
    }
};

// y = acc + b for the first kOut columns (FP32 [M][kOut])
struct EpiOutT {
    const float* b;
    float* Y;
    template <int CW = 256>
    __device__ void begin(int, int = 0) {}
    __device__ void operator()(int m, int c0, const float* v, int cnt) const
    {
        for (int c = 0; c < mlp::kOut; c++) Y[(size_t)m * mlp::kOut + c] = v[c] + b[c];
    }
};

// g = acc * silu'(Z): G row-major [M][256] and transposed [256][M]; the row's
// 256 pre-activations are loaded in one burst (begin) while the MMAs finish
struct EpiBackSiluT {
    const __nv_bfloat16* Z;
    __nv_bfloat16 *G, *GT;
    int M;
    uint4 zrow[mlp::kHid / 8];
    int zc0 = 0;  // first column of the preloaded window
    // preloads columns [c0, c0 + CW) of row m
    template <int CW = mlp::kHid>
    __device__ void begin(int m, int c0 = 0)
    {
        zc0 = c0;
        const uint4* src = reinterpret_cast<const uint4*>(Z + (size_t)m * mlp::kHid + c0);
#pragma unroll
        for (int i = 0; i < CW / 8; i++) zrow[i] = __ldg(src + i);
    }
    __device__ void operator()(int m, int c0, const float* v, int cnt) const
    {
#pragma unroll
        for (int i = 0; i < 32; i += 8) {
            const uint4 zr = zrow[(c0 - zc0 + i) / 8];
            const uint32_t zw[4] = {zr.x, zr.y, zr.z, zr.w};
            uint32_t gp[4];
#pragma unroll
            for (int j = 0; j < 8; j += 2) {
                const __nv_bfloat162 z2 = *reinterpret_cast<const __nv_bfloat162*>(&zw[j / 2]);
                const float g0 = v[i + j] * mlp::silu_grad(__low2float(z2));
                const float g1 = v[i + j + 1] * mlp::silu_grad(__high2float(z2));
                gp[j / 2] = mlp::pack_bf16(g0, g1);
            }
            *reinterpret_cast<uint4*>(G + (size_t)m * mlp::kHid + c0 + i) = make_uint4(gp[0], gp[1], gp[2], gp[3]);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const uint32_t w = gp[j / 2];
                reinterpret_cast<unsigned short*>(GT)[(size_t)(c0 + i + j) * M + m] =
                    (unsigned short)((j & 1) ? (w >> 16) : (w & 0xffffu));
            }
        }
    }
};

// split-K partial of a weight gradient: P[split][m][n] (FP32)
struct EpiPartial {
    float* P;
    int M, N;
    template <int CW = 256>
    __device__ void begin(int, int = 0) {}
    __device__ void operator()(int m, int c0, const float* v, int cnt) const
    {
        float* dst = P + ((size_t)blockIdx.y * M + m) * N + c0;
        for (int i = 0; i < cnt; i += 4)
            *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
};

// gr[m][n] (row length N) += sum over the splits of P[split][m][n]
__global__ void reduce_partials_kernel(const float* __restrict__ P, int splits, int M, int N, float* __restrict__ gr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * N) return;
    float s = 0.f;
    for (int k = 0; k < splits; k++) s += P[(size_t)k * M * N + i];
    gr[i] += s;
}

// ---------------------------------------------------------------- persistent, warp-specialised
// The forward and data-gradient GEMMs (N = 256, K <= 256) as a persistent
// kernel with one role per warp, one CTA per SM walking 128-row tiles:
//   warp 0  producer: the whole B operand (the layer's weights, N x K) once
//           into shared memory, where it stays; then the A k-atoms of every
//           tile through a ring of kWsRing stages with 16-byte cp.async, up to
//           kWsAhead atoms in flight, each signalled on its stage's `full`;
//   warp 1  MMA: one thread issues the four K = 16 MMAs per atom into one of
//           two 256-column accumulators in tensor memory (alternating per
//           tile), frees the stage on `empty` and signals `accf` per tile;
//   warps 2.. epilogue (kWsEpiWarps of them, up to four per quadrant of
//           tensor-memory lanes, each taking a slice of the columns): each
//           reads its 32 accumulator lanes (rows) of a finished tile and
//           signals `acce` when its part of the buffer is drained.
// So a tile's epilogue overlaps the next tile's copies and MMAs.  Every wait
// is bounded; one that runs out sets the block's abort flag, every other wait
// then gives up, the block drains its MMAs (bounded), frees tensor memory and
// raises ST_TIMEOUT.
#ifndef TP_TCT_EPI_WARPS
#define TP_TCT_EPI_WARPS 8
#endif
constexpr int kWsEpiWarps = TP_TCT_EPI_WARPS;  // 4, 8 or 16: 1, 2 or 4 per tensor-memory lane quadrant
constexpr int kWsThreads = 64 + 32 * kWsEpiWarps;
constexpr int kWsCols = 256 * 4 / kWsEpiWarps;  // accumulator columns per epilogue warp
constexpr int kWsRing = 4;
constexpr int kWsAhead = 2;
constexpr uint32_t kWsLimit = 1u << 22;

__device__ __forceinline__ bool ws_wait(uint32_t bar, uint32_t parity, volatile int* abort)
{
    for (uint32_t it = 0; it < kWsLimit; it++) {
        if (tc::mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && *abort) return false;
    }
    *abort = 1;
    return false;
}

size_t ws_smem_bytes(int k) { return 1024 + (size_t)(k / 64) * 256 * 128 + (size_t)kWsRing * a_stage_bytes(); }

template <class Epi>
__global__ void __launch_bounds__(kWsThreads, 1) tcgemm_ws_kernel(const __nv_bfloat16* __restrict__ A, int lda,
                                                                  const __nv_bfloat16* __restrict__ B, int ldb,
                                                                  int M, int K, Epi epi, int* __restrict__ status)
{
    constexpr int N = 256;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2 * kWsRing + 6];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int katoms = K / 64, ntiles = M / 128;
    const uint32_t raw = tc::smem_addr(smem_raw);
    const uint32_t sB = raw + ((1024u - (raw & 1023u)) & 1023u);
    const uint32_t sA = sB + (uint32_t)katoms * N * 128u;
    const uint32_t bar0 = tc::smem_addr(&bars[0]);
    auto full = [&](int st) { return bar0 + 8u * st; };
    auto empty = [&](int st) { return bar0 + 8u * (kWsRing + st); };
    const uint32_t bfull = bar0 + 8u * (2 * kWsRing);
    auto accf = [&](int b) { return bar0 + 8u * (2 * kWsRing + 1 + b); };
    auto acce = [&](int b) { return bar0 + 8u * (2 * kWsRing + 3 + b); };
    const uint32_t fin = bar0 + 8u * (2 * kWsRing + 5);
    volatile int* abort = &abort_flag;
    if (tid == 0) {
        for (int st = 0; st < kWsRing; st++) {
            tc::mbar_init(full(st), 32);
            tc::mbar_init(empty(st), 1);
        }
        tc::mbar_init(bfull, 32);
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(accf(b), 1);
            tc::mbar_init(acce(b), 32 * kWsEpiWarps);
        }
        tc::mbar_init(fin, 1);
        tc::mbar_fence_init();
        abort_flag = 0;
    }
    if (warp == 1) {
        tc::tmem_alloc(tc::smem_addr(&tmem_slot), 512);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        // B, resident for every tile of this block
        for (int c = lane; c < katoms * N * 8; c += 32) {
            const int a = c / (N * 8), rem = c % (N * 8), r = rem >> 3, kk = (rem & 7) * 8;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                         ::"r"(sB + (uint32_t)a * N * 128u + tc::sw128_offset(N, r, kk)),
                         "l"(B + (size_t)r * ldb + a * 64 + kk)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
        tc::fence_async_smem();
        tc::mbar_arrive(bfull);
        // A atoms of every tile through the ring
        uint32_t u = 0;
        bool ok = true;
        for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
            const int m0 = t * 128;
            for (int a = 0; ok && a < katoms; a++, u++) {
                const int st = (int)(u % kWsRing);
                const uint32_t use = u / kWsRing;
                if (use > 0) ok = ws_wait(empty(st), (use - 1) & 1u, abort);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                const uint32_t dst = sA + (uint32_t)st * a_stage_bytes();
                for (int c = lane; c < 128 * 8; c += 32) {
                    const int r = c >> 3, kk = (c & 7) * 8;
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                                 ::"r"(dst + tc::sw128_offset(128, r, kk)),
                                 "l"(A + (size_t)(m0 + r) * lda + a * 64 + kk)
                                 : "memory");
                }
                asm volatile("cp.async.commit_group;" ::: "memory");
                if (u >= (uint32_t)kWsAhead) {  // the atom kWsAhead behind has landed
                    asm volatile("cp.async.wait_group %0;" ::"n"(kWsAhead) : "memory");
                    tc::fence_async_smem();
                    tc::mbar_arrive(full((int)((u - kWsAhead) % kWsRing)));
                }
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        if (ok) {
            tc::fence_async_smem();
            for (uint32_t w = u >= (uint32_t)kWsAhead ? u - kWsAhead : 0; w < u; w++)
                tc::mbar_arrive(full((int)(w % kWsRing)));
        }
    } else if (warp == 1) {
        if (lane == 0 && ws_wait(bfull, 0, abort)) {
            tc::tc_fence_after();
            const uint32_t idesc = tc::idesc_bf16_f32(128, N);
            uint32_t u = 0, j = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x, j++) {
                const int b = (int)(j & 1u);
                const uint32_t v = j >> 1;
                if (v > 0) ok = ws_wait(acce(b), (v - 1) & 1u, abort);
                if (!ok) break;
                tc::tc_fence_after();
                for (int a = 0; ok && a < katoms; a++, u++) {
                    const int st = (int)(u % kWsRing);
                    ok = ws_wait(full(st), (u / kWsRing) & 1u, abort);
                    if (!ok) break;
                    tc::tc_fence_after();
                    const uint64_t ad = tc::desc_sw128(sA + (uint32_t)st * a_stage_bytes());
                    const uint64_t bd = tc::desc_sw128(sB + (uint32_t)a * N * 128u);
#pragma unroll
                    for (int kk = 0; kk < 4; kk++)
                        tc::mma_bf16(tmem + (uint32_t)(b * N), ad + 2 * kk, bd + 2 * kk, idesc, (a | kk) != 0);
                    tc::mma_commit(empty(st));
                }
                if (ok) tc::mma_commit(accf(b));
            }
        }
        __syncwarp();
    } else {
        const int q = warp & 3;  // the tensor-memory lanes this warp may read
        const int cbase = ((warp - 2) >> 2) * kWsCols;  // its slice of the columns
        const uint32_t lane_base = (uint32_t)(32 * q) << 16;
        uint32_t j = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, j++) {
            const int b = (int)(j & 1u);
            const int row = t * 128 + 32 * q + lane;
            Epi e = epi;
            e.template begin<kWsCols>(row, cbase);
            if (!ws_wait(accf(b), (j >> 1) & 1u, abort)) break;
            tc::tc_fence_after();
#pragma unroll
            for (int c = 0; c < kWsCols; c += 32) {
                float vals[32];
                tc::tmem_ld32(tmem + lane_base + (uint32_t)(b * N + cbase + c), vals);
                e(row, cbase + c, vals, 32);
            }
            tc::tc_fence_before();
            tc::mbar_arrive(acce(b));
        }
    }
    __syncthreads();
    if (warp == 1) {
        if (lane == 0) {  // every MMA this block issued has completed (bounded)
            tc::mma_commit(fin);
            if (!tc::mbar_wait(fin, 0, kWsLimit)) abort_flag = 1;
        }
        __syncwarp();
    }
    __syncthreads();
    if (tid == 0 && abort_flag) atomicOr(status, ST_TIMEOUT);
    if (warp == 1) tc::tmem_dealloc(tmem, 512);
}

template <class Epi>
static cudaError_t launch_ws(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int K,
                             const Epi& epi, int* status, cudaStream_t s)
{
    if (M % 128 || K % 64 || K < 64 || K > 256) return cudaErrorInvalidValue;
    const size_t smem = ws_smem_bytes(K);
    cudaError_t e = cudaFuncSetAttribute(tcgemm_ws_kernel<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = std::min(M / 128, g.num_sms > 0 ? g.num_sms : 148);
    tcgemm_ws_kernel<Epi><<<grid, kWsThreads, smem, s>>>(A, lda, B, ldb, M, K, epi, status);
    return cudaGetLastError();
}

}  // namespace tct

namespace tctrain {

using namespace tct;

#ifndef TP_TCT_WS
#define TP_TCT_WS 1
#endif

cudaError_t forward_hidden(const __nv_bfloat16* X, int lda, const __nv_bfloat16* W, int kin, int M, const float* b,
                           __nv_bfloat16* Z, __nv_bfloat16* H, __nv_bfloat16* HT, int* status, cudaStream_t s)
{
    if (TP_TCT_WS) return launch_ws(X, lda, W, kin, M, kin, EpiHiddenT{b, Z, H, HT, M}, status, s);
    return launch(X, lda, W, kin, M, mlp::kHid, kin, 1, EpiHiddenT{b, Z, H, HT, M}, status, s);
}

cudaError_t forward_out(const __nv_bfloat16* H3, const __nv_bfloat16* W4, int M, const float* b, float* Y,
                        int* status, cudaStream_t s)
{
    return launch(H3, mlp::kHid, W4, mlp::kHid, M, mlp::kOutPad, mlp::kHid, 1, EpiOutT{b, Y}, status, s);
}

cudaError_t backward_data(const __nv_bfloat16* Gin, int ldg, const __nv_bfloat16* WT, int kout, int M,
                          const __nv_bfloat16* Zprev, __nv_bfloat16* G, __nv_bfloat16* GT, int* status,
                          cudaStream_t s)
{
    if (TP_TCT_WS) return launch_ws(Gin, ldg, WT, kout, M, kout, EpiBackSiluT{Zprev, G, GT, M}, status, s);
    return launch(Gin, ldg, WT, kout, M, mlp::kHid, kout, 1, EpiBackSiluT{Zprev, G, GT, M}, status, s);
}

cudaError_t backward_weights(const __nv_bfloat16* GT, const __nv_bfloat16* XT, int kin, int nsamp, float* partial,
                             int splits, float* gr, int* status, cudaStream_t s)
{
    // dW[256][kin] = G^T X: M = 256 output features, N = kin, K = samples
    cudaError_t e = launch(GT, nsamp, XT, nsamp, mlp::kHid, kin, nsamp, splits,
                           EpiPartial{partial, mlp::kHid, kin}, status, s);
    if (e != cudaSuccess) return e;
    const int kchunk = (nsamp / 64 + splits - 1) / splits * 64;
    const int used = (nsamp + kchunk - 1) / kchunk;
    const int tot = mlp::kHid * kin;
    reduce_partials_kernel<<<(tot + 255) / 256, 256, 0, s>>>(partial, used, mlp::kHid, kin, gr);
    return cudaGetLastError();
}

cudaError_t gemm_f32(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, float* D, int* status,
                     cudaStream_t s)
{
    // the shapes of the forward and data-gradient GEMMs go through the kernel those use
    if (TP_TCT_WS && N == 256 && K <= 256) return launch_ws(A, K, B, K, M, K, EpiStoreF32{D, N}, status, s);
    return launch(A, K, B, K, M, N, K, 1, EpiStoreF32{D, N}, status, s);
}

}  // namespace tctrain
}  // namespace tp

using namespace tp;

// D[m][n] = A[m][k] * B[n][k]^T with BF16 inputs (raw 16-bit patterns) and FP32
// output, through the training GEMM kernel: m a multiple of 128, n a multiple
// of 16 in [16, 256], k a multiple of 64.
extern "C" int tp_tc_gemm_train_bf16(int m, int n, int k, const unsigned short* a, const unsigned short* b,
                                     float* d)
{
    if (m < 128 || m % 128 || n < 16 || n > 256 || n % 16 || k < 64 || k % 64 || !a || !b || !d) {
        set_error(6, "tp_tc_gemm_train_bf16: m a multiple of 128, n 16..256 in steps of 16, k a multiple of 64");
        return -1;
    }
    if (!ensure_init()) return -1;
    cudaStream_t s = g.stream;
    const size_t sa = sizeof(uint16_t) * (size_t)m * k, sb = sizeof(uint16_t) * (size_t)n * k,
                 sd = sizeof(float) * (size_t)m * n;
    void *dA = nullptr, *dB = nullptr, *dD = nullptr;
    bool ok = cuda_ok(cudaMalloc(&dA, sa), "A") && cuda_ok(cudaMalloc(&dB, sb), "B") &&
              cuda_ok(cudaMalloc(&dD, sd), "D");
    if (ok) {
        cudaMemcpyAsync(dA, a, sa, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dB, b, sb, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(dD, 0, sd, s);
        ok = cuda_ok(tctrain::gemm_f32(static_cast<const __nv_bfloat16*>(dA), static_cast<const __nv_bfloat16*>(dB),
                                       m, n, k, static_cast<float*>(dD), g.d_status, s),
                     "train gemm");
    }
    if (ok) {
        cudaMemcpyAsync(d, dD, sd, cudaMemcpyDeviceToHost, s);
        ok = cuda_ok(cudaStreamSynchronize(s), "train gemm sync");
    }
    if (dA) cudaFree(dA);
    if (dB) cudaFree(dB);
    if (dD) cudaFree(dD);
    return ok ? 0 : -1;
}
