// track_surrogate.cu -- tracking with the learned field model: the FP32 Wirz
// push of the mixed path, with every field evaluation done for the 256
// particles of a block at once as a chain of BF16 GEMMs on the 5th-generation
// tensor cores (tcgen05.mma, FP32 accumulators in tensor memory).
//
// Block layout: 256 consumer threads = two 128-row tiles, one MMA warp and
// three loader warps (three warps per SM sub-partition).  Consumer thread t
// owns row t % 128 of tile t / 128 (its particle), which is also the
// tensor-memory lane its warp may read.  Activations live in shared memory as
// the MMA A operand (128-byte swizzled, K-major), one 64 KB buffer per tile,
// rewritten in place by each layer's epilogue.  Weights are pre-packed in the
// same layout as 32 chunks per evaluation (16 KB: 128 output rows x 64
// inputs; the output layer 2 KB) and stream from L2 through a 4-stage ring
// of shared buffers, copied by the loader warps with 16-byte cp.async (a
// 1-D bulk copy engine moves at most about 25 B per cycle per SM; cp.async
// from several warps several times that).  One thread of the MMA warp issues
// the MMAs of both tiles per chunk; ring, accumulators and A operands are
// handed over through mbarriers, and every wait on them is bounded.
#include <cstring>

#include "../../include/tp_gpu.h"
#include "mlp_common.cuh"
#include "tc_sm100.cuh"
#include "tp_internal.h"
#include "wirz_f32.cuh"

namespace tp {
namespace mlp {

constexpr int kTiles = 2;
constexpr int kB = 128 * kTiles;         // particles (consumer threads) per block
constexpr int kLoaderWarps = 3;
constexpr int kLoaders = 32 * kLoaderWarps;
constexpr int kThreads = kB + 32 + kLoaders;  // + the MMA warp and the loader warps
constexpr int kMmaWarp = kB / 32, kLoaderWarp0 = kB / 32 + 1;
constexpr int kStages = 4;
constexpr uint32_t kStageBytes = 16384;
constexpr uint32_t kABytes = 128 * kHid * 2;  // one tile's activations (65536)
constexpr int kChunks = 32;              // weight chunks per evaluation
constexpr size_t kSmemDyn = 1024 + kTiles * kABytes + kStages * kStageBytes;
constexpr int kSurrSmemBins = 1024;
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t kTmemCols = 256 * kTiles;

// chunk j of an evaluation: layer, output half, k-atom, bytes and offset in the pack
struct Chunk {
    int layer, half, katom;
    uint32_t bytes, offset;
};

// The two output halves of a k-atom are consecutive, so that they land in
// adjacent ring stages and one N = 256 MMA reads both.
__host__ __device__ __forceinline__ Chunk chunk_of(int j)
{
    Chunk c;
    if (j < 4) {
        c.layer = 0; c.half = j & 1; c.katom = j >> 1;
        c.bytes = kStageBytes; c.offset = (uint32_t)j * kStageBytes;
    } else if (j < 28) {
        const int jj = (j - 4) & 7;
        c.layer = 1 + (j - 4) / 8; c.half = jj & 1; c.katom = jj >> 1;
        c.bytes = kStageBytes; c.offset = 65536u + (uint32_t)(j - 4) * kStageBytes;
    } else {
        c.layer = 4; c.half = 0; c.katom = j - 28;
        c.bytes = 2048; c.offset = 458752u + (uint32_t)(j - 28) * 2048u;
    }
    return c;
}

// byte offset in the pack of weight (n, k) of layer l (n < padded outputs)
__host__ __device__ __forceinline__ uint32_t pack_offset(int l, int n, int k)
{
    if (l == kLayers - 1) return 458752u + (uint32_t)(k >> 6) * 2048u + tc::sw128_offset(16, n, k & 63);
    const int h = n >> 7, a = k >> 6;
    const uint32_t base = l == 0 ? 0u : 65536u + (uint32_t)(l - 1) * 131072u;
    return base + (uint32_t)(2 * a + h) * kStageBytes + tc::sw128_offset(128, n & 127, k & 63);
}

// SiLU of two values given as h = z / 2: h + h tanh(h), in BF16 pairs.
__device__ __forceinline__ uint32_t silu_half_bf16x2(float h0, float h1)
{
    const uint32_t h = pack_bf16(h0, h1);
    uint32_t t, r;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(h));
    asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(r) : "r"(h), "r"(t));
    return r;
}

// First chunk of each layer in the per-evaluation sequence (and the end).
__host__ __device__ constexpr int layer_first_chunk(int l) { return l == 0 ? 0 : l < 5 ? 4 + 8 * (l - 1) : 32; }

// Shared state of the block's tensor-core pipeline.
struct Pipe {
    unsigned char* a[kTiles];        // activation tiles (A operands)
    uint32_t stage0;                 // shared address of stage 0
    uint32_t full, empty;            // ring mbarriers (kStages each, 8 B apart)
    uint32_t accf, aready;           // a layer's accumulators complete / A operands written
    uint32_t done;                   // MMA thread: every MMA it issued has completed
    uint32_t tmem;
    uint32_t lim;                    // polls before a hand-over wait gives up
    int* abort;                      // a bounded wait ran out (or the MMA thread failed)
    int* stop;                       // consumers are finished
    const float* bias;               // shared copy: 4 x 256 hidden biases then 6 output biases
    const float* hbias;              // halves of the 4 x 256 hidden biases
    const int* freq;
};

// Bounded wait that also gives up once the block has aborted; a wait that
// runs out marks the block aborted.
__device__ __forceinline__ bool wait_or_abort(uint32_t bar, uint32_t parity, int* abort, uint32_t lim)
{
    for (uint32_t it = 0; it < lim; it++) {
        if (tc::mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && *(volatile int*)abort) return false;
    }
    *(volatile int*)abort = 1;
    return false;
}

// The loader warps: stream the weight chunks in use order into the ring
// with 16-byte cp.async (per SM several times the rate of 1-D bulk copies).
// Loader warp w takes every kLoaderWarps-th chunk starting at w, waits until
// the MMAs that read the stage's previous chunk have completed, copies the
// chunk (each lane every 32nd piece), waits for its copies, fences them for
// the tensor core and signals the stage (32 arrivals on `full`).  So up to
// kLoaderWarps chunks are in flight and each is signalled as soon as it has
// landed.  Ends on `stop` or an abort.
__device__ __noinline__ void loader(const Pipe& pp, const unsigned char* wpack)
{
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x / 32 - kLoaderWarp0;
    for (uint32_t u = w;; u += kLoaderWarps) {
        const uint32_t s = u % kStages, use = u / kStages;
        if (use > 0) {
            bool ok = false;
            for (uint32_t it = 0; it < pp.lim && !ok; it++) {
                ok = tc::mbar_try_wait(pp.empty + 8 * s, (use - 1) & 1);
                if (!ok && (it & 63u) == 63u && (*(volatile int*)pp.abort || *(volatile int*)pp.stop)) break;
            }
            if (!ok) {
                if (!*(volatile int*)pp.stop) *(volatile int*)pp.abort = 1;
                break;
            }
        }
        const Chunk ch = chunk_of((int)(u % kChunks));
        const unsigned char* src = wpack + ch.offset;
        const uint32_t dst = pp.stage0 + s * kStageBytes;
        for (uint32_t off = lane * 16; off < ch.bytes; off += 512)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + off), "l"(src + off) : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        tc::fence_async_smem();
        tc::mbar_arrive(pp.full + 8 * s);
    }
}

// The MMA thread (lane 0 of the MMA warp).  Per layer: wait until the
// consumers of both tiles have written their A operands (and read the
// previous accumulators), then read the layer's weights from the ring: hidden
// layers by k-atom, both output halves (adjacent stages) in one N = 256 MMA
// per tile; the output layer (N = 16) chunk by chunk; commit to `accf`.  Ends
// when the consumers raise `stop` (or on a failed wait), after the MMAs it
// issued have completed (bounded wait).
__device__ __noinline__ void mma_issuer(const Pipe& pp, int* status)
{
    uint32_t next_use = 0, nready = 0;
    bool ok = true, stopped = false;
    uint64_t adesc[kTiles];
#pragma unroll
    for (int t = 0; t < kTiles; t++) adesc[t] = tc::desc_sw128(tc::smem_addr(pp.a[t]));
    while (ok) {
        for (int l = 0; ok && l < kLayers; l++) {
            ok = wait_or_abort(pp.aready, nready & 1, pp.abort, pp.lim);
            nready++;
            if (ok && *(volatile int*)pp.stop) {
                stopped = true;
                ok = false;
            }
            if (!ok) break;
            tc::tc_fence_after();
            const bool last = l == kLayers - 1;
            const uint32_t idesc = tc::idesc_bf16_f32(128, last ? 16 : 256);
            const uint32_t width = last ? 1u : 2u;
            const uint32_t c_end = next_use + (uint32_t)(layer_first_chunk(l + 1) - layer_first_chunk(l));
            for (uint32_t c = next_use; ok && c < c_end; c += width) {
                for (uint32_t w = 0; w < width && ok; w++)
                    ok = wait_or_abort(pp.full + 8 * ((c + w) % kStages), ((c + w) / kStages) & 1, pp.abort,
                                       pp.lim);
                if (!ok) break;
                tc::tc_fence_after();
                const Chunk ch = chunk_of((int)(c % kChunks));
                const uint64_t bdesc = tc::desc_sw128(pp.stage0 + (c % kStages) * kStageBytes);
#pragma unroll
                for (int t = 0; t < kTiles; t++) {
                    const uint64_t a = adesc[t] + (uint64_t)(ch.katom * (128 * 128 / 16));
                    const uint32_t d = pp.tmem + (uint32_t)(t * 256);
#pragma unroll
                    for (int kk = 0; kk < 4; kk++)
                        tc::mma_bf16(d, a + 2 * kk, bdesc + 2 * kk, idesc, (ch.katom | kk) != 0);
                }
                for (uint32_t w = 0; w < width; w++) tc::mma_commit(pp.empty + 8 * ((c + w) % kStages));
                next_use = c + width;
            }
            tc::mma_commit(pp.accf);
        }
    }
    // drain: the MMAs issued so far
    tc::mma_commit(pp.done);
    const bool fine = tc::mbar_wait(pp.done, 0, kWaitLimit);
    if (!stopped || !fine) {
        *(volatile int*)pp.abort = 1;
        atomicOr(status, ST_TIMEOUT);
    }
}

// Barrier of the kB consumer threads (the MMA and loader warps never join it).
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kB) : "memory"); }

// Per-thread position in the accumulator barrier's phases.
struct Cons {
    uint32_t nacc = 0;
};

// Consumer side of one field evaluation: every consumer thread of the block
// calls this together with its own position and receives the model's E and
// B there.  Per layer it waits for the accumulators, turns its row into the
// next layer's A operand and signals `aready`.  After an abort every wait
// returns at once and the values are meaningless (the caller discards them).
__device__ __noinline__ void field_tile(const Model& md, const Pipe& pp, Cons& cs, const uint64_t X[3],
                                        float E[3], float B[3])
{
    const int tid = threadIdx.x, warp = tid >> 5;
    const int tile = tid >> 7, row = tid & 127;
    unsigned char* arow = pp.a[tile];
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t tcol = pp.tmem + lane_base + (uint32_t)(tile * 256);
    const uint32_t accf = pp.accf, aready = pp.aready;
    // Fourier features of this thread's particle: inputs 0..63 sin, 64..127 cos
    {
        const uint32_t U0 = (uint32_t)(X[0] >> 32), U1 = (uint32_t)(X[1] >> 32), U2 = (uint32_t)(X[2] >> 32);
#pragma unroll 1
        for (int j0 = 0; j0 < kFeat; j0 += 8) {
            uint32_t ps[4], pc[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                float sv[2], cv[2];
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int j = j0 + 2 * q + e;
                    const uint32_t ph = (uint32_t)pp.freq[3 * j] * U0 + (uint32_t)pp.freq[3 * j + 1] * U1 +
                                        (uint32_t)pp.freq[3 * j + 2] * U2;
                    __sincosf(mixed::rev_to_rad(ph), &sv[e], &cv[e]);
                }
                ps[q] = pack_bf16(sv[0], sv[1]);
                pc[q] = pack_bf16(cv[0], cv[1]);
            }
            *reinterpret_cast<uint4*>(arow + tc::sw128_offset(128, row, j0)) = make_uint4(ps[0], ps[1], ps[2], ps[3]);
            *reinterpret_cast<uint4*>(arow + tc::sw128_offset(128, row, kFeat + j0)) =
                make_uint4(pc[0], pc[1], pc[2], pc[3]);
        }
    }
    tc::fence_async_smem();
    tc::tc_fence_before();
    tc::mbar_arrive(aready);
    for (int l = 0; l < kLayers; l++) {
        wait_or_abort(accf, cs.nacc & 1, pp.abort, pp.lim);
        cs.nacc++;
        tc::tc_fence_after();
        if (l < kLayers - 1) {
            // SiLU(z) = h + h tanh(h), h = z / 2 = acc / 2 + bias / 2, in packed
            // BF16 pairs (one tanh per two values); the result is already the
            // next layer's BF16 input
            const float4* hb4 = reinterpret_cast<const float4*>(pp.hbias + l * kHid);
            const uint32_t rbase = (uint32_t)(row >> 3) * 1024u + (uint32_t)(row & 7) * 128u;
            const uint32_t rx = (uint32_t)(row & 7);
#pragma unroll 1
            for (int c0 = 0; c0 < kHid; c0 += 32) {
                float v[32];
                tc::tmem_ld32(tcol + (uint32_t)c0, v);
                uint32_t pk[16];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const float4 hb = hb4[(c0 >> 2) + q];
                    pk[2 * q] = silu_half_bf16x2(fmaf(0.5f, v[4 * q], hb.x), fmaf(0.5f, v[4 * q + 1], hb.y));
                    pk[2 * q + 1] = silu_half_bf16x2(fmaf(0.5f, v[4 * q + 2], hb.z), fmaf(0.5f, v[4 * q + 3], hb.w));
                }
                // 128-byte-swizzled row chunk positions of columns c0, c0 + 8, c0 + 16, c0 + 24
                const uint32_t atom = (uint32_t)(c0 >> 6) * 16384u, ch = (uint32_t)((c0 >> 3) & 7);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    *reinterpret_cast<uint4*>(arow + atom + rbase + (((ch + k) ^ rx) << 4)) =
                        make_uint4(pk[4 * k], pk[4 * k + 1], pk[4 * k + 2], pk[4 * k + 3]);
            }
            tc::fence_async_smem();
            tc::tc_fence_before();
            tc::mbar_arrive(aready);
        } else {
            float v[16];
            tc::tmem_ld16(tcol, v);
            const float* bo = pp.bias + (kLayers - 1) * kHid;
            B[0] = (v[0] + bo[0]) * md.out_scale[0] + md.out_shift[0];
            B[1] = (v[1] + bo[1]) * md.out_scale[1] + md.out_shift[1];
            B[2] = (v[2] + bo[2]) * md.out_scale[2] + md.out_shift[2];
            E[0] = (v[3] + bo[3]) * md.out_scale[3] + md.out_shift[3];
            E[1] = (v[4] + bo[4]) * md.out_scale[4] + md.out_shift[4];
            E[2] = (v[5] + bo[5]) * md.out_scale[5] + md.out_shift[5];
            tc::tc_fence_before();
        }
    }
}

// Block set-up shared by the kernels: shared layout, biases and frequencies,
// mbarriers and tensor memory.
struct SmemStatic {
    float bias[kLayers * kHid];
    __align__(16) float hbias[(kLayers - 1) * kHid];
    int freq[3 * kFeat];
    uint64_t bars[2 * kStages + 3];
    uint32_t tmem_slot;
    int abort;
    int stop;
};

__device__ void pipe_setup(Pipe& pp, SmemStatic& st, unsigned char* dyn, const Model& md, uint32_t wait_limit)
{
    const int tid = threadIdx.x;
    const uint32_t raw = tc::smem_addr(dyn);
    unsigned char* base = dyn + ((1024u - (raw & 1023u)) & 1023u);
    for (int t = 0; t < kTiles; t++) pp.a[t] = base + t * kABytes;
    pp.stage0 = tc::smem_addr(base + kTiles * kABytes);
    for (int k = tid; k < (kLayers - 1) * kHid; k += blockDim.x) {
        st.bias[k] = md.b[k / kHid][k % kHid];
        st.hbias[k] = 0.5f * st.bias[k];
    }
    if (tid < kOut) st.bias[(kLayers - 1) * kHid + tid] = md.b[kLayers - 1][tid];
    for (int k = tid; k < 3 * kFeat; k += blockDim.x) st.freq[k] = md.freq[k];
    pp.full = tc::smem_addr(&st.bars[0]);
    pp.empty = tc::smem_addr(&st.bars[kStages]);
    pp.accf = tc::smem_addr(&st.bars[2 * kStages]);
    pp.aready = tc::smem_addr(&st.bars[2 * kStages + 1]);
    pp.done = tc::smem_addr(&st.bars[2 * kStages + 2]);
    pp.lim = wait_limit ? wait_limit : kWaitLimit;
    pp.abort = &st.abort;
    pp.stop = &st.stop;
    pp.bias = st.bias;
    pp.hbias = st.hbias;
    pp.freq = st.freq;
    if (tid == 0) {
        st.abort = 0;
        st.stop = 0;
        for (int s = 0; s < kStages; s++) {
            tc::mbar_init(pp.full + 8 * s, 32);
            tc::mbar_init(pp.empty + 8 * s, 1);
        }
        tc::mbar_init(pp.accf, 1);
        tc::mbar_init(pp.aready, kB);
        tc::mbar_init(pp.done, 1);
        tc::mbar_fence_init();
    }
    if ((tid >> 5) == 0) {
        tc::tmem_alloc(tc::smem_addr(&st.tmem_slot), kTmemCols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    pp.tmem = st.tmem_slot;
}

// Consumers, after their last evaluation: raise `stop` and release the
// MMA thread from its wait for the next A operands.
__device__ void consumers_finish(const Pipe& pp)
{
    consumers_sync();
    if (threadIdx.x == 0) *(volatile int*)pp.stop = 1;
    consumers_sync();
    tc::mbar_arrive(pp.aready);
}

// Every thread, at the end: frees tensor memory once the MMA thread has
// drained its MMAs and the loaders their copies.
__device__ void pipe_teardown(const Pipe& pp)
{
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(pp.tmem, kTmemCols);
}

__device__ __forceinline__ void consumers_diff_sum(const double sg[8], double* red, double* slot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        double v = sg[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp * 8 + c] = v;
    }
    consumers_sync();
    if (threadIdx.x < 8) {
        double s = 0.0;
        for (int w = 0; w < kB / 32; w++) s += red[w * 8 + threadIdx.x];
        slot[threadIdx.x] += s;
    }
    consumers_sync();
}

// Fixed-step tracking with the learned field (src/tracking.c:297-462
// schedule and diagnostics); every consumer thread runs every step so that
// the field evaluations line up; inactive and escaped particles evaluate at
// their frozen position and discard the result.  Threads 0..kB-1 own one
// particle each; then the MMA warp and the loader warps.
__global__ void __launch_bounds__(kThreads, 1) track_surrogate_kernel(mixed::MixField f, Model md,
                                                                       TrackBufs b, TrackParams q,
                                                                       uint32_t wait_limit)
{
    using namespace mixed;
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    __shared__ SmemStatic st;
    __shared__ double red[(kB / 32) * 8];
    __shared__ unsigned int hist[kSurrSmemBins];
    Pipe pp;
    pipe_setup(pp, st, smem_dyn, md, wait_limit);
    if (threadIdx.x >= kB) {
        if (threadIdx.x / 32 >= kLoaderWarp0) loader(pp, md.wpack);
        else if (threadIdx.x == kMmaWarp * 32) mma_issuer(pp, b.status);
        __syncwarp();
        pipe_teardown(pp);
        return;
    }
    const bool smem_hist = q.nbins <= kSurrSmemBins;
    const float dt = (float)q.dt;
    const int ntiles = (q.n + kB - 1) / kB;
    Cons cs;
    auto field = [&](const uint64_t* X, float* E, float* B) { field_tile(md, pp, cs, X, E, B); };
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * kB + threadIdx.x;
        const bool active = i < q.n;
        PM p = {};
        double x0[3] = {0, 0, 0}, u0[3] = {0, 0, 0}, tstart = 0.0, mu0 = 0.0;
        int nst = 1;
        bool esc = false;
        uint64_t X0[3] = {0, 0, 0};
        if (active) {
            double xs[3] = {b.x[i], b.y[i], b.z[i]};
            double sh[3] = {b.xs[i], b.ys[i], b.zs[i]};
            x0[0] = b.x0[i]; x0[1] = b.y0[i]; x0[2] = b.z0[i];
            u0[0] = b.ux0[i]; u0[1] = b.uy0[i]; u0[2] = b.uz0[i];
            tstart = b.t[i];
            nst = b.nsteps_ptl[i];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double r = (xs[k] - f.min[k]) / f.L[k];
                double fl = floor(r);
                if (f.bc_flag == 1 && (r < 0.0 || r > 1.0)) esc = true;
                p.X[k] = __double2ull_rz((r - fl) * 18446744073709551616.0);
                p.img[k] = (int)fl + (int)llrint(sh[k] / f.L[k]);
                double r0 = (x0[k] - f.min[k]) / f.L[k];
                X0[k] = __double2ull_rz((r0 - floor(r0)) * 18446744073709551616.0);
            }
            p.u[0] = (float)b.ux[i]; p.u[1] = (float)b.uy[i]; p.u[2] = (float)b.uz[i];
        }
        {
            float E[3], B[3];
            field(X0, E, B);  // field at the initial position: its mu is constant (static field)
            float uf0[3] = {(float)u0[0], (float)u0[1], (float)u0[2]};
            float bb = sqrtf(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
            float uu = sqrtf(uf0[0] * uf0[0] + uf0[1] * uf0[1] + uf0[2] * uf0[2]);
            // clamped to [-1, 1]: FP32 rounding can carry it just past, where
            // the pitch angle's arc cosine would be NaN
            mu0 = (double)fminf(1.0f, fmaxf(-1.0f, (B[0] * uf0[0] + B[1] * uf0[1] + B[2] * uf0[2]) / (bb * uu)));
        }
        int esc_pre = esc ? 1 : 0;
        int esc_after = esc_pre;
        int ntp = q.ntp0, tstep = 1;
        double sg[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (active && esc_pre) atomicSub(&b.remain[1], 1);
        double* slot_base = b.dpart + (size_t)blockIdx.x * q.nsdc * 8;
        int done = 0;
        int to_frame = q.einterval - q.sstep % q.einterval;
        int to_diff = kDiffInterval - q.sstep % kDiffInterval;
        if (to_frame == q.einterval) to_frame = 0;
        if (to_diff == kDiffInterval) to_diff = 0;
        for (int j = q.sstep; j <= q.estep; j++) {
            const bool at_diff = to_diff == 0, at_frame = to_frame == 0;
            to_diff = at_diff ? kDiffInterval - 1 : to_diff - 1;
            to_frame = at_frame ? q.einterval - 1 : to_frame - 1;
            sg[0] = 0.0; sg[4] = 0.0; sg[5] = 0.0;
            const bool push = active && (esc_pre == 0 || f.bc_flag == 0);
            PM pn = p;
            bool e2 = false;
            wirz_f32(f, pn, dt, field, e2);  // every consumer thread evaluates
            if (push) {
                p = pn;
                if (e2) esc_after = 1;
                nst += 1;
                done += 1;
            }
            if (at_diff) {  // block-uniform: one more field evaluation
                float E[3], B[3];
                field(p.X, E, B);
                if (push && esc_after == 0) {
                    double t = tstart + done * q.dt;
                    double tt = t * 2 + q.dt;
                    double dd[3];
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        double pos = (double)p.X[k] * 5.421010862427522e-20 + p.img[k];
                        dd[k] = x0[k] - (f.min[k] + f.L[k] * pos);
                    }
                    double dxx = dd[0] * dd[0] / tt, dyy = dd[1] * dd[1] / tt, dzz = dd[2] * dd[2] / tt;
                    double du0 = u0[0] - p.u[0], du1 = u0[1] - p.u[1], du2 = u0[2] - p.u[2];
                    double g1 = sqrt(1.0 + (double)p.u[0] * p.u[0] + (double)p.u[1] * p.u[1] + (double)p.u[2] * p.u[2]);
                    double g0 = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
                    float bb = sqrtf(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
                    float uu = sqrtf(p.u[0] * p.u[0] + p.u[1] * p.u[1] + p.u[2] * p.u[2]);
                    double mu = (double)fminf(1.0f, fmaxf(-1.0f, (B[0] * p.u[0] + B[1] * p.u[1] + B[2] * p.u[2]) / (bb * uu)));
                    double th = (double)acosf((float)mu) * (180.0 / 3.14159265358979323846);
                    double th0 = (double)acosf((float)mu0) * (180.0 / 3.14159265358979323846);
                    sg[1] = dxx; sg[2] = dyy; sg[3] = dzz;
                    sg[0] = dxx + dyy + dzz;
                    sg[4] = (du0 * du0 + du1 * du1 + du2 * du2) / tt;
                    sg[5] = (mu - mu0) * (mu - mu0) / tt;
                    sg[6] = (th - th0) * (th - th0) / tt;
                    sg[7] = (g1 - g0) * (g1 - g0) / tt;
                }
            }
            if (active && esc_pre == 0 && esc_after == 1 && f.bc_flag == 1 && ntp < q.nt_out)
                atomicAdd(&b.espect_esc[ntp * q.nbins + energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
            if (at_frame) {
                if (ntp < q.nt_out) {
                    bool take = active && esc_after == 0;
                    if (smem_hist) {
                        consumers_sync();
                        for (int k = threadIdx.x; k < q.nbins; k += kB) hist[k] = 0u;
                        consumers_sync();
                        if (take) atomicAdd(&hist[energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
                        consumers_sync();
                        for (int k = threadIdx.x; k < q.nbins; k += kB)
                            if (hist[k]) atomicAdd(&b.espect[ntp * q.nbins + k], hist[k]);
                    } else if (take) {
                        atomicAdd(&b.espect[ntp * q.nbins + energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
                    }
                }
                ntp++;
            }
            if (at_diff) {
                consumers_diff_sum(sg, red, slot_base + (size_t)tstep * 8);
                tstep++;
            }
            if (active && esc_after && at_diff && tstep < q.nsdc) atomicSub(&b.remain[tstep], 1);
            esc_pre = esc_after;
        }
        if (active && !*(volatile int*)&st.abort) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double xk = f.min[k] + f.L[k] * ((double)p.X[k] * 5.421010862427522e-20);
                if (k == 0) b.x[i] = xk;
                else if (k == 1) b.y[i] = xk;
                else b.z[i] = xk;
            }
            b.xs[i] = p.img[0] * f.L[0]; b.ys[i] = p.img[1] * f.L[1]; b.zs[i] = p.img[2] * f.L[2];
            b.ux[i] = p.u[0]; b.uy[i] = p.u[1]; b.uz[i] = p.u[2];
            b.t[i] = tstart + done * q.dt;
            b.nsteps_ptl[i] = nst;
        }
        consumers_sync();
    }
    consumers_finish(pp);
    pipe_teardown(pp);
}

// Model field at n positions through the in-kernel (per-block) evaluation path.
__global__ void __launch_bounds__(kThreads, 1) field_eval_kernel(Model md, const uint32_t* __restrict__ U,
                                                                  int n, float* __restrict__ out, int* status,
                                                                  uint32_t wait_limit)
{
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    __shared__ SmemStatic st;
    Pipe pp;
    pipe_setup(pp, st, smem_dyn, md, wait_limit);
    if (threadIdx.x >= kB) {
        if (threadIdx.x / 32 >= kLoaderWarp0) loader(pp, md.wpack);
        else if (threadIdx.x == kMmaWarp * 32) mma_issuer(pp, status);
        __syncwarp();
        pipe_teardown(pp);
        return;
    }
    Cons cs;
    for (int tile = blockIdx.x; tile * kB < n; tile += gridDim.x) {
        int i = tile * kB + threadIdx.x;
        uint64_t X[3] = {0, 0, 0};
        if (i < n)
            for (int k = 0; k < 3; k++) X[k] = (uint64_t)U[3 * i + k] << 32;
        float E[3], B[3];
        field_tile(md, pp, cs, X, E, B);
        if (i < n && !*(volatile int*)&st.abort) {
            out[6 * i] = B[0]; out[6 * i + 1] = B[1]; out[6 * i + 2] = B[2];
            out[6 * i + 3] = E[0]; out[6 * i + 4] = E[1]; out[6 * i + 5] = E[2];
        }
    }
    consumers_finish(pp);
    pipe_teardown(pp);
}

// Packs the BF16 weights [out_pad][in] of every layer into the chunk layout above.
__global__ void pack_weights_kernel(const __nv_bfloat16* w0, const __nv_bfloat16* w1, const __nv_bfloat16* w2,
                                    const __nv_bfloat16* w3, const __nv_bfloat16* w4, unsigned char* pack)
{
    const __nv_bfloat16* ws[kLayers] = {w0, w1, w2, w3, w4};
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (int l = 0; l < kLayers; l++) {
        const int n_elem = layer_out_pad(l) * layer_in(l);
        if (i < n_elem) {
            const int n = i / layer_in(l), k = i % layer_in(l);
            *reinterpret_cast<__nv_bfloat16*>(pack + pack_offset(l, n, k)) = ws[l][i];
            return;
        }
        i -= n_elem;
    }
}

cudaError_t pack_weights(const __nv_bfloat16* const w[kLayers], unsigned char* pack, cudaStream_t s)
{
    int total = 0;
    for (int l = 0; l < kLayers; l++) total += layer_out_pad(l) * layer_in(l);
    pack_weights_kernel<<<(total + 255) / 256, 256, 0, s>>>(w[0], w[1], w[2], w[3], w[4], pack);
    return cudaGetLastError();
}

cudaError_t launch_track_surrogate(const mixed::MixField& f, const Model& md, const TrackBufs& b,
                                   const TrackParams& q, int grid, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(track_surrogate_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemDyn);
    if (e != cudaSuccess) return e;
    track_surrogate_kernel<<<grid, kThreads, kSmemDyn, s>>>(f, md, b, q, g.wait_limit);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace tp

using namespace tp;

// Polls before a hand-over wait of the tensor-core pipeline gives up (0: the
// default, about 4 million); a small value makes the waits run out, for tests
// of the timeout path.
extern "C" int tp_set_wait_limit(unsigned int polls)
{
    g.wait_limit = polls;
    return 0;
}

// Model field at n positions evaluated by the block-wide kernel path used in tracking.
extern "C" int tp_mlp_eval_kernel(int n, const unsigned int* u, float* out6)
{
    mlp::Model md;
    if (!ensure_init() || !mlp::mlp_model(md)) return -1;
    if (n <= 0) return 0;
    uint32_t* dU;
    float* dO;
    if (!cuda_ok(cudaMalloc(&dU, sizeof(uint32_t) * 3 * n), "u") ||
        !cuda_ok(cudaMalloc(&dO, sizeof(float) * 6 * n), "out")) return -1;
    cudaStream_t s = g.stream;
    cudaMemcpyAsync(dU, u, sizeof(uint32_t) * 3 * n, cudaMemcpyHostToDevice, s);
    bool ok = cuda_ok(cudaFuncSetAttribute(mlp::field_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)mlp::kSmemDyn), "smem attr");
    if (ok) {
        int grid = (n + mlp::kB - 1) / mlp::kB;
        if (grid > g.num_sms) grid = g.num_sms;
        mlp::field_eval_kernel<<<grid, mlp::kThreads, mlp::kSmemDyn, s>>>(md, dU, n, dO, g.d_status, g.wait_limit);
        ok = cuda_ok(cudaGetLastError(), "field eval");
    }
    if (ok) {
        cudaMemcpyAsync(out6, dO, sizeof(float) * 6 * n, cudaMemcpyDeviceToHost, s);
        ok = cuda_ok(cudaStreamSynchronize(s), "field eval sync");
    }
    cudaFree(dU);
    cudaFree(dO);
    return ok ? 0 : -1;
}
