// track_surrogate.cu -- tracking with the learned field model: the FP32 Wirz
// push of the mixed path, with every field evaluation done for the 128
// particles of a block at once as a chain of BF16 tensor-core GEMMs
// (mma.sync m16n8k16, FP32 accumulation) through shared memory.
//
// Block layout: 4 warps, warp w owns rows [32w, 32w + 32) = its own 32
// particles, so activations never cross warps; weights stream from L2 into a
// shared chunk of 64 output neurons at a time and are shared by all warps.
#include <cstring>

#include "../../include/tp_gpu.h"
#include "mlp_common.cuh"
#include "tp_internal.h"
#include "wirz_f32.cuh"

namespace tp {
namespace mlp {

constexpr int kB = 128;            // particles (rows) per block
constexpr int kLD = kHid + 8;      // activation row stride (bf16), conflict-free fragments
constexpr int kWRows = 64;         // weight rows staged per chunk
constexpr size_t kSmemH = sizeof(__nv_bfloat16) * kB * kLD;
constexpr size_t kSmemW = sizeof(__nv_bfloat16) * kWRows * kLD;
constexpr size_t kSmemY = sizeof(float) * kB * 8;
constexpr size_t kSmemTotal = 2 * kSmemH + kSmemW + kSmemY;

struct Smem {
    __nv_bfloat16* h0;
    __nv_bfloat16* h1;
    __nv_bfloat16* w;
    float* y;
};

// All 128 threads call this together; each passes its own position and
// receives the model's E and B there.
__device__ __noinline__ void field_block(const Model& md, const int* sfreq, const Smem& sm,
                                         const uint64_t X[3], float E[3], float B[3])
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    // features of this thread's particle: row tid of h1
    {
        __nv_bfloat16* xr = sm.h1 + tid * kLD;
        uint32_t U0 = (uint32_t)(X[0] >> 32), U1 = (uint32_t)(X[1] >> 32), U2 = (uint32_t)(X[2] >> 32);
        for (int j = 0; j < kFeat; j++) {
            uint32_t ph = (uint32_t)sfreq[3 * j] * U0 + (uint32_t)sfreq[3 * j + 1] * U1 +
                          (uint32_t)sfreq[3 * j + 2] * U2;
            float s, c;
            __sincosf(mixed::rev_to_rad(ph), &s, &c);
            xr[j] = __float2bfloat16(s);
            xr[kFeat + j] = __float2bfloat16(c);
        }
    }
    __syncwarp();
    const __nv_bfloat16* hin = sm.h1;
    __nv_bfloat16* hout = sm.h0;
    for (int l = 0; l < kLayers; l++) {
        const int K = layer_in(l), Np = layer_out_pad(l);
        const __nv_bfloat16* W = md.w[l];
        const float* bias = md.b[l];
        const bool last = l == kLayers - 1;
        for (int nc = 0; nc < Np; nc += kWRows) {
            const int nrows = Np - nc < kWRows ? Np - nc : kWRows;
            __syncthreads();  // the weight chunk buffer is free
            const int per_row = K / 8;
            for (int c = tid; c < nrows * per_row; c += kB) {
                int r = c / per_row, kk = (c - r * per_row) * 8;
                *reinterpret_cast<uint4*>(sm.w + r * kLD + kk) =
                    __ldg(reinterpret_cast<const uint4*>(W + (size_t)(nc + r) * K + kk));
            }
            __syncthreads();
            float acc[2][8][4];
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 8; j++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
            const int ntl = nrows / 8;
            for (int k0 = 0; k0 < K; k0 += 16) {
                uint32_t af[2][4];
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const __nv_bfloat16* r0 = hin + (warp * 32 + i * 16 + g) * kLD + k0 + 2 * t;
                    af[i][0] = *reinterpret_cast<const uint32_t*>(r0);
                    af[i][1] = *reinterpret_cast<const uint32_t*>(r0 + 8 * kLD);
                    af[i][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
                    af[i][3] = *reinterpret_cast<const uint32_t*>(r0 + 8 * kLD + 8);
                }
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    if (j < ntl) {
                        const __nv_bfloat16* wr = sm.w + (j * 8 + g) * kLD + k0 + 2 * t;
                        uint32_t bfr[2] = {*reinterpret_cast<const uint32_t*>(wr),
                                           *reinterpret_cast<const uint32_t*>(wr + 8)};
                        mma_bf16(acc[0][j], af[0], bfr);
                        mma_bf16(acc[1][j], af[1], bfr);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    if (j >= ntl) continue;
                    const int row = warp * 32 + i * 16 + g;
                    const int col = nc + j * 8 + 2 * t;
                    if (!last) {
                        float b0 = __ldg(bias + col), b1 = __ldg(bias + col + 1);
                        *reinterpret_cast<uint32_t*>(hout + row * kLD + col) =
                            pack_bf16(silu(acc[i][j][0] + b0), silu(acc[i][j][1] + b1));
                        *reinterpret_cast<uint32_t*>(hout + (row + 8) * kLD + col) =
                            pack_bf16(silu(acc[i][j][2] + b0), silu(acc[i][j][3] + b1));
                    } else {
                        if (col < kOut) {
                            sm.y[row * 8 + col] = acc[i][j][0] + __ldg(bias + col);
                            sm.y[(row + 8) * 8 + col] = acc[i][j][2] + __ldg(bias + col);
                        }
                        if (col + 1 < kOut) {
                            sm.y[row * 8 + col + 1] = acc[i][j][1] + __ldg(bias + col + 1);
                            sm.y[(row + 8) * 8 + col + 1] = acc[i][j][3] + __ldg(bias + col + 1);
                        }
                    }
                }
        }
        if (!last) {
            const __nv_bfloat16* tmp = hin;
            hin = hout;
            hout = const_cast<__nv_bfloat16*>(tmp);
        }
    }
    __syncwarp();
    const float* yr = sm.y + tid * 8;
    B[0] = yr[0] * md.out_scale[0] + md.out_shift[0];
    B[1] = yr[1] * md.out_scale[1] + md.out_shift[1];
    B[2] = yr[2] * md.out_scale[2] + md.out_shift[2];
    E[0] = yr[3] * md.out_scale[3] + md.out_shift[3];
    E[1] = yr[4] * md.out_scale[4] + md.out_shift[4];
    E[2] = yr[5] * md.out_scale[5] + md.out_shift[5];
}

// Fixed-step tracking with the learned field (src/tracking.c:297-462
// schedule and diagnostics); every thread runs every step so that the
// block-wide field evaluations line up; inactive and escaped particles
// evaluate at their frozen position and discard the result.
__global__ void __launch_bounds__(kB, 1) track_surrogate_kernel(mixed::MixField f, Model md,
                                                                 TrackBufs b, TrackParams q)
{
    using namespace mixed;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[(kB / 32) * 8];
    __shared__ unsigned int hist[kMaxSmemBins];
    __shared__ int sfreq[3 * kFeat];
    Smem sm;
    sm.h0 = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    sm.h1 = reinterpret_cast<__nv_bfloat16*>(smem_raw + kSmemH);
    sm.w = reinterpret_cast<__nv_bfloat16*>(smem_raw + 2 * kSmemH);
    sm.y = reinterpret_cast<float*>(smem_raw + 2 * kSmemH + kSmemW);
    for (int k = threadIdx.x; k < 3 * kFeat; k += blockDim.x) sfreq[k] = md.freq[k];
    __syncthreads();
    const bool smem_hist = q.nbins <= kMaxSmemBins;
    const float dt = (float)q.dt;
    auto field = [&](const uint64_t* X, float* E, float* B) { field_block(md, sfreq, sm, X, E, B); };
    for (int tile = blockIdx.x; tile < q.ntiles; tile += gridDim.x) {
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
            mu0 = (double)((B[0] * uf0[0] + B[1] * uf0[1] + B[2] * uf0[2]) / (bb * uu));
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
            wirz_f32(f, pn, dt, field, e2);  // block-wide: every thread evaluates
            if (push) {
                p = pn;
                if (e2) esc_after = 1;
                nst += 1;
                done += 1;
            }
            if (at_diff) {  // block-uniform: one more block-wide field evaluation
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
                    double mu = (double)((B[0] * p.u[0] + B[1] * p.u[1] + B[2] * p.u[2]) / (bb * uu));
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
                        __syncthreads();
                        for (int k = threadIdx.x; k < q.nbins; k += blockDim.x) hist[k] = 0u;
                        __syncthreads();
                        if (take) atomicAdd(&hist[energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
                        __syncthreads();
                        for (int k = threadIdx.x; k < q.nbins; k += blockDim.x)
                            if (hist[k]) atomicAdd(&b.espect[ntp * q.nbins + k], hist[k]);
                    } else if (take) {
                        atomicAdd(&b.espect[ntp * q.nbins + energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
                    }
                }
                ntp++;
            }
            if (at_diff) {
                block_diff_sum(sg, red, slot_base + (size_t)tstep * 8);
                tstep++;
            }
            if (active && esc_after && at_diff && tstep < q.nsdc) atomicSub(&b.remain[tstep], 1);
            esc_pre = esc_after;
        }
        if (active) {
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
        __syncthreads();
    }
}

// Model field at n positions through the in-kernel (per-block) evaluation path.
__global__ void __launch_bounds__(kB, 1) field_eval_kernel(Model md, const uint32_t* __restrict__ U,
                                                           int n, float* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sfreq[3 * kFeat];
    Smem sm;
    sm.h0 = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    sm.h1 = reinterpret_cast<__nv_bfloat16*>(smem_raw + kSmemH);
    sm.w = reinterpret_cast<__nv_bfloat16*>(smem_raw + 2 * kSmemH);
    sm.y = reinterpret_cast<float*>(smem_raw + 2 * kSmemH + kSmemW);
    for (int k = threadIdx.x; k < 3 * kFeat; k += blockDim.x) sfreq[k] = md.freq[k];
    __syncthreads();
    for (int tile = blockIdx.x; tile * kB < n; tile += gridDim.x) {
        int i = tile * kB + threadIdx.x;
        uint64_t X[3] = {0, 0, 0};
        if (i < n)
            for (int k = 0; k < 3; k++) X[k] = (uint64_t)U[3 * i + k] << 32;
        float E[3], B[3];
        field_block(md, sfreq, sm, X, E, B);
        if (i < n) {
            out[6 * i] = B[0]; out[6 * i + 1] = B[1]; out[6 * i + 2] = B[2];
            out[6 * i + 3] = E[0]; out[6 * i + 4] = E[1]; out[6 * i + 5] = E[2];
        }
        __syncthreads();
    }
}

cudaError_t launch_track_surrogate(const mixed::MixField& f, const Model& md, const TrackBufs& b,
                                   const TrackParams& q, int grid, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(track_surrogate_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTotal);
    if (e != cudaSuccess) return e;
    track_surrogate_kernel<<<grid, kB, kSmemTotal, s>>>(f, md, b, q);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace tp

using namespace tp;

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
                                           (int)mlp::kSmemTotal), "smem attr");
    if (ok) {
        int grid = (n + mlp::kB - 1) / mlp::kB;
        if (grid > g.num_sms) grid = g.num_sms;
        mlp::field_eval_kernel<<<grid, mlp::kB, mlp::kSmemTotal, s>>>(md, dU, n, dO);
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
