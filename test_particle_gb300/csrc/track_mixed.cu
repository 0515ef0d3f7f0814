// track_mixed.cu -- mixed-precision tracking: FP32 push and field evaluation,
// 64-bit fixed-point positions, FP64 diffusion accumulations.
//
// Position: each axis holds X = frac((x - min) / L) * 2^64 as an unsigned
// 64-bit integer plus a signed period count.  Integer addition wraps exactly
// at the box, so periodic boundaries cost nothing and never round, and the
// fixed point carries 64 bits where an FP64 coordinate carries 53.  Field
// evaluation reads the top 32 bits: a grid cell index and fraction come from
// one 32x32->64 multiply, and a plane-wave phase 2 pi n.x/L is the exact
// integer n.X mod 2^32, so phases never lose accuracy to large arguments.
//
// The push is the Wirz scheme of the reference (src/tracking.c:749-892) in
// rotation form: the perpendicular frame comes from h x u (no cancellation for
// u nearly along B), 1 - cos(a) is formed as 2 sin^2(a/2), and the momentum is
// rotated in u-space so gamma is never re-derived from |v| -> 1.
#include "tp_kernels_mixed.h"
#include "wirz_f32.cuh"

namespace tp {
namespace mixed {

// pitch-angle cosine of u against the local field, FP32 field, returned in double
template <int SYS>
__device__ __forceinline__ double pitch_mu(const MixField& f, const uint64_t X[3], const float u[3],
                                           const ModePair* smodes, FieldCache& fc)
{
    float E[3], B[3];
    field_mixed<SYS>(f, X, E, B, smodes, fc);
    float bb = sqrtf(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    float uu = sqrtf(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    // FP32 rounding can carry a cosine of u nearly along B just past +-1,
    // where its arc cosine (the pitch angle) would be NaN: clamp it
    const float c = (B[0] * u[0] + B[1] * u[1] + B[2] * u[2]) / (bb * uu);
    return (double)fminf(1.0f, fmaxf(-1.0f, c));
}

// Persistent fixed-step tracking in mixed precision: the same schedule and
// diagnostics as the FP64 kernel (src/tracking.c:297-462); the mode table of
// the plane-wave field is staged once per block in shared memory.
// Per-particle data that only the diffusion steps (every 100 steps) touch --
// the initial state, its pitch cosine, the start time and the last diffusion
// singles -- lives in shared memory, [row][thread], so the step loop keeps
// only the push state and the cell cache in registers.
enum : int { DG_SG = 0, DG_X0 = 8, DG_U0 = 11, DG_T0 = 14, DG_MU0 = 15, DG_G0 = 16, DG_ROWS = 17 };

// Resident blocks of 128 threads per SM the gridded kernel is compiled for
// (its registers: 4 blocks allow 128 a thread).
#ifndef TP_MIXED_PIC_MINBLOCKS
#define TP_MIXED_PIC_MINBLOCKS 4
#endif


// The diffusion singles of one particle at a diffusion step
// (calc_diff_coeff, src/diagnostics.c:659-705), FP64 accumulation, into its
// rows of dg; one FP64 reciprocal of 2t + dt instead of eight divisions (the
// FP64 pipe runs at a small fraction of the FP32 rate).  The pitch angle
// needs the field at the particle, evaluated with the particle's cell cache.
// (Compiled as a separate function, with a cache of its own, this costs the
// step loop spills at its call site instead of saving registers: measured
// by -Xptxas -v, 24-32 B at 4 blocks per SM, 132-152 B at 5.)
template <int SYS>
__device__ __forceinline__ void diff_singles_body(const MixField& f, const PM& p, const ModePair* smodes,
                                                  FieldCache& fc, double (*dg)[kBlock], int tx, int done, double qdt)
{
    double t = dg[DG_T0][tx] + done * qdt;
    double itt = 1.0 / (t * 2 + qdt);
    double dd[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double pos = (double)p.X[k] * 5.421010862427522e-20 + p.img[k];
        dd[k] = dg[DG_X0 + k][tx] - (f.min[k] + f.L[k] * pos);
    }
    const double u00 = dg[DG_U0][tx], u01 = dg[DG_U0 + 1][tx], u02 = dg[DG_U0 + 2][tx];
    const double mu0 = dg[DG_MU0][tx];
    double dxx = dd[0] * dd[0] * itt, dyy = dd[1] * dd[1] * itt, dzz = dd[2] * dd[2] * itt;
    double du0 = u00 - p.u[0], du1 = u01 - p.u[1], du2 = u02 - p.u[2];
    double g1 = sqrt(1.0 + (double)p.u[0] * p.u[0] + (double)p.u[1] * p.u[1] + (double)p.u[2] * p.u[2]);
    double g0 = dg[DG_G0][tx];
    double mu = pitch_mu<SYS>(f, p.X, p.u, smodes, fc);
    double th = (double)acosf((float)mu) * (180.0 / 3.14159265358979323846);
    double th0 = (double)acosf((float)mu0) * (180.0 / 3.14159265358979323846);
    dg[DG_SG + 1][tx] = dxx; dg[DG_SG + 2][tx] = dyy; dg[DG_SG + 3][tx] = dzz;
    dg[DG_SG + 0][tx] = dxx + dyy + dzz;
    dg[DG_SG + 4][tx] = (du0 * du0 + du1 * du1 + du2 * du2) * itt;
    dg[DG_SG + 5][tx] = (mu - mu0) * (mu - mu0) * itt;
    dg[DG_SG + 6][tx] = (th - th0) * (th - th0) * itt;
    dg[DG_SG + 7][tx] = (g1 - g0) * (g1 - g0) * itt;
}


// Persistent fixed-step tracking in mixed precision: the same schedule and
// diagnostics as the FP64 kernel (src/tracking.c:297-462); the mode table of
// the plane-wave field is staged once per block in shared memory.
template <int SYS>
__global__ void __launch_bounds__(kBlock, SYS == TP_SYS_PIC ? TP_MIXED_PIC_MINBLOCKS : 4)
    track_mixed_kernel(MixField f, TrackBufs b, TrackParams q)
{
    __shared__ double red[(kBlock / 32) * 8];
    __shared__ unsigned int hist[kMaxSmemBins];
    __shared__ double dg[DG_ROWS][kBlock];
    extern __shared__ ModePair smodes[];
    if (SYS == TP_SYS_MODESUM) {
        for (int m = threadIdx.x; m < (f.nmodes + 1) / 2; m += blockDim.x) smodes[m] = f.modes[m];
        __syncthreads();
    }
    const int tx = threadIdx.x;
    const bool smem_hist = q.nbins <= kMaxSmemBins;
    const float dt = (float)q.dt;
    for (int tile = blockIdx.x; tile < q.ntiles; tile += gridDim.x) {
        const int slot = tile * kBlock + tx;
        const bool active = slot < q.n;
        const int i = active && q.idx ? q.idx[slot] : slot;  // the particle of this lane
        PM p = {};
        FieldCache fc;
        int nst = 1;
        bool esc = false;
#pragma unroll
        for (int r = 0; r < DG_ROWS; r++) dg[r][tx] = 0.0;
        if (active) {
            double xs[3] = {b.x[i], b.y[i], b.z[i]};
            double sh[3] = {b.xs[i], b.ys[i], b.zs[i]};
            double x0[3] = {b.x0[i], b.y0[i], b.z0[i]};
            double u0[3] = {b.ux0[i], b.uy0[i], b.uz0[i]};
            dg[DG_T0][tx] = b.t[i];
            nst = b.nsteps_ptl[i];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double r = (xs[k] - f.min[k]) / f.L[k];
                double fl = floor(r);
                if (f.bc_flag == 1 && (r < 0.0 || r > 1.0)) esc = true;
                p.X[k] = __double2ull_rz((r - fl) * 18446744073709551616.0);
                p.img[k] = (int)fl + (int)llrint(sh[k] / f.L[k]);
                dg[DG_X0 + k][tx] = x0[k];
                dg[DG_U0 + k][tx] = u0[k];
            }
            p.u[0] = (float)b.ux[i]; p.u[1] = (float)b.uy[i]; p.u[2] = (float)b.uz[i];
            dg[DG_G0][tx] = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
            // mu of the initial state: the field at the initial position is static
            uint64_t X0[3];
            float uf0[3] = {(float)u0[0], (float)u0[1], (float)u0[2]};
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double r = (x0[k] - f.min[k]) / f.L[k];
                X0[k] = __double2ull_rz((r - floor(r)) * 18446744073709551616.0);
            }
            dg[DG_MU0][tx] = pitch_mu<SYS>(f, X0, uf0, smodes, fc);
            if (q.resumed && b.sg_carry) {
                // continue exactly where the previous segment stopped: the
                // 64-bit fixed-point position and period counts, the start
                // time and the steps taken (t = t0 + steps * dt)
                const double* cr = b.sg_carry + (size_t)i * kSegCarry;
#pragma unroll
                for (int c = 0; c < 8; c++) dg[DG_SG + c][tx] = cr[c];
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    p.X[k] = (uint64_t)__double_as_longlong(cr[8 + k]);
                    p.img[k] = (int)cr[11 + k];
                }
                dg[DG_T0][tx] = cr[14];
            }
        }
        int esc_pre = esc ? 1 : 0;
        int esc_after = esc_pre;
        int ntp = q.ntp0, tstep = 1 + q.row0;
        if (active && esc_pre && !q.resumed) atomicSub(&b.remain[1], 1);
        double* slot_base = b.dpart + (size_t)blockIdx.x * q.nsdc * 8;
        int done = 0;
        if (active && q.resumed && b.sg_carry) done = (int)b.sg_carry[(size_t)i * kSegCarry + 15];
        // countdowns to the next diagnostic steps (j % einterval, j % 100)
        int to_frame = q.einterval - q.sstep % q.einterval;
        int to_diff = kDiffInterval - q.sstep % kDiffInterval;
        if (to_frame == q.einterval) to_frame = 0;
        if (to_diff == kDiffInterval) to_diff = 0;
        for (int j = q.sstep; j <= q.estep; j++) {
            const bool at_diff = to_diff == 0, at_frame = to_frame == 0;
            to_diff = at_diff ? kDiffInterval - 1 : to_diff - 1;
            to_frame = at_frame ? q.einterval - 1 : to_frame - 1;
            if (active && (esc_pre == 0 || f.bc_flag == 0)) {
                bool e2 = false;
                wirz_f32(f, p, dt, [&](const uint64_t* X, float* E, float* B) {
                    field_mixed<SYS>(f, X, E, B, smodes, fc);
                }, e2);
                if (e2) esc_after = 1;
                nst += 1;
                done += 1;
                if (esc_after == 0 && at_diff) {
                    diff_singles_body<SYS>(f, p, smodes, fc, dg, tx, done, q.dt);
                }
            }
            if (active && esc_pre == 0 && esc_after == 1 && f.bc_flag == 1 && ntp < q.nt_out)
                atomicAdd(&b.espect_esc[ntp * q.nbins + energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
            if (at_frame) {
                if (ntp < q.nt_out) {
                    bool take = active && esc_after == 0;
                    if (smem_hist) {
                        __syncthreads();
                        for (int k = tx; k < q.nbins; k += blockDim.x) hist[k] = 0u;
                        __syncthreads();
                        if (take) atomicAdd(&hist[energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
                        __syncthreads();
                        for (int k = tx; k < q.nbins; k += blockDim.x)
                            if (hist[k]) atomicAdd(&b.espect[ntp * q.nbins + k], hist[k]);
                    } else if (take) {
                        atomicAdd(&b.espect[ntp * q.nbins + energy_bin_f(b.ebin_thr, q.nbins, p.u)], 1u);
                    }
                }
                ntp++;
            }
            if (at_diff) {
                // drr, dpp and duu are the only singles the reference clears
                // every step (src/tracking.c:334-336); the others keep their
                // last values for particles that no longer move
                if (!(active && (esc_pre == 0 || f.bc_flag == 0) && esc_after == 0)) {
                    dg[DG_SG + 0][tx] = 0.0; dg[DG_SG + 4][tx] = 0.0; dg[DG_SG + 5][tx] = 0.0;
                }
                double sg[8];
#pragma unroll
                for (int c = 0; c < 8; c++) sg[c] = dg[DG_SG + c][tx];
                block_diff_sum(sg, red, slot_base + (size_t)tstep * 8);
                tstep++;
            }
            if (active && esc_after && at_diff && tstep < q.nsdc)
                atomicSub(&b.remain[tstep], 1);
            esc_pre = esc_after;
        }
        if (active) {
            double xs[3];
#pragma unroll
            for (int k = 0; k < 3; k++) xs[k] = f.min[k] + f.L[k] * ((double)p.X[k] * 5.421010862427522e-20);
            b.x[i] = xs[0]; b.y[i] = xs[1]; b.z[i] = xs[2];
            b.xs[i] = p.img[0] * f.L[0]; b.ys[i] = p.img[1] * f.L[1]; b.zs[i] = p.img[2] * f.L[2];
            b.ux[i] = p.u[0]; b.uy[i] = p.u[1]; b.uz[i] = p.u[2];
            b.t[i] = dg[DG_T0][tx] + done * q.dt;
            b.nsteps_ptl[i] = nst;
            if (b.status && !(isfinite(p.u[0]) && isfinite(p.u[1]) && isfinite(p.u[2])))
                atomicOr(b.status, ST_NONFINITE);
            if (b.sg_carry) {
                double* cr = b.sg_carry + (size_t)i * kSegCarry;
#pragma unroll
                for (int c = 0; c < 8; c++) cr[c] = dg[DG_SG + c][tx];
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    cr[8 + k] = __longlong_as_double((long long)p.X[k]);
                    cr[11 + k] = (double)p.img[k];
                }
                cr[14] = dg[DG_T0][tx];
                cr[15] = (double)done;
            }
            if (b.esc_out) b.esc_out[i] = esc_after;
        }
    }
}

// The FP32 field of the mixed path at given points (tests and callers that
// want the field the throughput path sees): each position is turned into
// 64-bit fixed point exactly as the tracking kernel turns a particle's, and
// the result is written as (Bx, By, Bz, Ex, Ey, Ez), the order of emfields.
template <int SYS>
__global__ void emf_mixed_batch_kernel(MixField f, int n, const double* __restrict__ xyz,
                                       float* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t X[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double r = (xyz[3 * i + k] - f.min[k]) / f.L[k];
        X[k] = __double2ull_rz((r - floor(r)) * 18446744073709551616.0);
    }
    FieldCache fc;
    float E[3], B[3];
    // the mode table is read from global memory here (the tracking kernel
    // stages it in shared memory; the arithmetic is the same)
    field_mixed<SYS>(f, X, E, B, f.modes, fc);
    out[6 * i + 0] = B[0]; out[6 * i + 1] = B[1]; out[6 * i + 2] = B[2];
    out[6 * i + 3] = E[0]; out[6 * i + 4] = E[1]; out[6 * i + 5] = E[2];
}

cudaError_t launch_emf_batch(const MixField& f, int n, const double* xyz, float* out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const unsigned g = (unsigned)((n + 127) / 128);
    switch (f.system_type) {
    case TP_SYS_TEST: emf_mixed_batch_kernel<TP_SYS_TEST><<<g, 128, 0, s>>>(f, n, xyz, out); break;
    case TP_SYS_FORCEFREE: emf_mixed_batch_kernel<TP_SYS_FORCEFREE><<<g, 128, 0, s>>>(f, n, xyz, out); break;
    case TP_SYS_PIC: emf_mixed_batch_kernel<TP_SYS_PIC><<<g, 128, 0, s>>>(f, n, xyz, out); break;
    case TP_SYS_MODESUM: emf_mixed_batch_kernel<TP_SYS_MODESUM><<<g, 128, 0, s>>>(f, n, xyz, out); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// --------------------------------------------------------------- launchers
template <int SYS>
static cudaError_t launch_sys(const MixField& f, const TrackBufs& b, const TrackParams& q, int grid,
                              cudaStream_t s)
{
    size_t smem = SYS == TP_SYS_MODESUM ? sizeof(ModePair) * (size_t)((f.nmodes + 1) / 2) : 0;
    if (smem > 0) {  // static plus dynamic shared memory may pass the 48 KB default
        cudaError_t e = cudaFuncSetAttribute(track_mixed_kernel<SYS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    track_mixed_kernel<SYS><<<grid, kBlock, smem, s>>>(f, b, q);
    return cudaGetLastError();
}

cudaError_t launch_track(const MixField& f, const TrackBufs& b, const TrackParams& q, int grid,
                         cudaStream_t s)
{
    switch (f.system_type) {
    case TP_SYS_TEST: return launch_sys<TP_SYS_TEST>(f, b, q, grid, s);
    case TP_SYS_FORCEFREE: return launch_sys<TP_SYS_FORCEFREE>(f, b, q, grid, s);
    case TP_SYS_PIC: return launch_sys<TP_SYS_PIC>(f, b, q, grid, s);
    case TP_SYS_MODESUM: return launch_sys<TP_SYS_MODESUM>(f, b, q, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

int track_max_blocks_per_sm(int system_type, int nmodes)
{
    int nb = 0;
    size_t smem = system_type == TP_SYS_MODESUM ? sizeof(ModePair) * (size_t)((nmodes + 1) / 2) : 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (system_type) {
    case TP_SYS_TEST: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_TEST>, kBlock, 0); break;
    case TP_SYS_FORCEFREE: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_FORCEFREE>, kBlock, 0); break;
    case TP_SYS_PIC: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_PIC>, kBlock, 0); break;
    case TP_SYS_MODESUM:
        if (smem > 0)
            cudaFuncSetAttribute(track_mixed_kernel<TP_SYS_MODESUM>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_MODESUM>, kBlock, smem);
        break;
    default: break;
    }
    return e == cudaSuccess ? nb : 0;
}

// Interleaved node layout for the gathers: per node {Ex,Ey,Ez,Bx,By,Bz,0,0}
// (32 bytes, one sector) built from the reference's AoS float E and B arrays.
__global__ void interleave_kernel(const float* __restrict__ e, const float* __restrict__ bf,
                                  size_t n, float4* __restrict__ eb)
{
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    eb[2 * i] = make_float4(e ? e[3 * i] : 0.f, e ? e[3 * i + 1] : 0.f, e ? e[3 * i + 2] : 0.f, bf[3 * i]);
    eb[2 * i + 1] = make_float4(bf[3 * i + 1], bf[3 * i + 2], 0.f, 0.f);
}

cudaError_t launch_interleave(const float* e, const float* bf, size_t n, float4* eb, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    interleave_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(e, bf, n, eb);
    return cudaGetLastError();
}

}  // namespace mixed
}  // namespace tp
