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
#include "tp_mixed.cuh"
#include "tp_kernels_mixed.h"

namespace tp {
namespace mixed {

struct PM {
    uint64_t X[3];
    int img[3];
    float u[3];
};

__device__ __forceinline__ float fx_to_float(uint64_t d)  // signed fixed-point delta -> box fraction
{
    return (float)(int64_t)d * 5.42101086242752217e-20f;  // 2^-64
}

__device__ __forceinline__ int64_t float_to_fx(float fr)  // box fraction -> signed fixed point
{
    return __float2ll_rn(fr * 18446744073709551616.0f);
}

// Adds a displacement (in box fractions) to a position, counting periods.
__device__ __forceinline__ void advance(uint64_t& X, int& img, float fr)
{
    int64_t d = float_to_fx(fr);
    uint64_t nx = X + (uint64_t)d;
    if (d > 0 && nx < X) img++;
    else if (d < 0 && nx > X) img--;
    X = nx;
}

template <int SYS>
__device__ __forceinline__ void wirz_mixed(const MixField& f, PM& p, float dt, const ModeF* smodes,
                                           FieldCache& fc, bool& escaped)
{
    const float cm = f.cm;
    float E[3], B[3];
    field_mixed<SYS>(f, p.X, E, B, smodes, fc);
    float Btot = sqrtf(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    float iB = 1.0f / Btot;
    float h[3] = {B[0] * iB, B[1] * iB, B[2] * iB};
    const float hk = 0.5f * cm * dt;
    float um[3] = {p.u[0] + hk * E[0], p.u[1] + hk * E[1], p.u[2] + hk * E[2]};
    float gam = sqrtf(1.0f + um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
    float ig = 1.0f / gam;
    // frame at the start point
    float w[3] = {h[1] * um[2] - h[2] * um[1], h[2] * um[0] - h[0] * um[2], h[0] * um[1] - h[1] * um[0]};
    float uperp = sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    float iu = uperp > 0.0f ? 1.0f / uperp : 0.0f;
    float hr[3] = {w[0] * iu, w[1] * iu, w[2] * iu};
    float hp[3] = {hr[1] * h[2] - hr[2] * h[1], hr[2] * h[0] - hr[0] * h[2], hr[0] * h[1] - hr[1] * h[0]};
    float upar = um[0] * h[0] + um[1] * h[1] + um[2] * h[2];
    float theta = cm * Btot * ig * dt;
    float s4, c4;
    __sincosf(0.25f * theta, &s4, &c4);
    float sin_h = 2.0f * s4 * c4, omc_h = 2.0f * s4 * s4;  // sin(theta/2), 1 - cos(theta/2)
    float R = uperp / (cm * Btot);
    float a1 = 0.5f * dt * upar * ig, a2 = R * sin_h, a3 = -R * omc_h;
    float dpre[3];
#pragma unroll
    for (int k = 0; k < 3; k++) dpre[k] = (h[k] * a1 + hp[k] * a2 + hr[k] * a3) * f.invL[k];
    uint64_t Xp[3] = {p.X[0], p.X[1], p.X[2]};
#pragma unroll
    for (int k = 0; k < 3; k++) Xp[k] += (uint64_t)float_to_fx(dpre[k]);
    field_mixed<SYS>(f, Xp, E, B, smodes, fc);
    Btot = sqrtf(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    iB = 1.0f / Btot;
    h[0] = B[0] * iB; h[1] = B[1] * iB; h[2] = B[2] * iB;
    w[0] = h[1] * um[2] - h[2] * um[1];
    w[1] = h[2] * um[0] - h[0] * um[2];
    w[2] = h[0] * um[1] - h[1] * um[0];
    uperp = sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    iu = uperp > 0.0f ? 1.0f / uperp : 0.0f;
    hr[0] = w[0] * iu; hr[1] = w[1] * iu; hr[2] = w[2] * iu;
    hp[0] = hr[1] * h[2] - hr[2] * h[1];
    hp[1] = hr[2] * h[0] - hr[0] * h[2];
    hp[2] = hr[0] * h[1] - hr[1] * h[0];
    upar = um[0] * h[0] + um[1] * h[1] + um[2] * h[2];
    theta = cm * Btot * ig * dt;
    float s2, c2;
    __sincosf(0.5f * theta, &s2, &c2);
    float sn = 2.0f * s2 * c2, omc = 2.0f * s2 * s2;  // sin(theta), 1 - cos(theta)
    float cs = 1.0f - omc;
#pragma unroll
    for (int k = 0; k < 3; k++) p.u[k] = h[k] * upar + uperp * (cs * hp[k] - sn * hr[k]) + hk * E[k];
    R = uperp / (cm * Btot);
    a1 = dt * upar * ig;
    a2 = R * sn;
    a3 = -R * omc;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float d = (h[k] * a1 + hp[k] * a2 + hr[k] * a3) * f.invL[k];
        if (f.bc_flag == 1) {
            // open boundary: leaving the box is an escape, not a wrap
            int before = p.img[k];
            advance(p.X[k], p.img[k], d);
            if (p.img[k] != before) escaped = true;
        } else {
            advance(p.X[k], p.img[k], d);
        }
    }
}

__device__ __forceinline__ int energy_bin_f(const double* thr, int nbins, const float u[3])
{
    double e = (double)(sqrtf(1.0f + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) - 1.0f);
    if (!(e < INFINITY)) return 0;
    int lo = 0, hi = nbins - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(thr + mid - 1) <= e) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// pitch-angle cosine of u against the local field, FP32 field, returned in double
template <int SYS>
__device__ __forceinline__ double pitch_mu(const MixField& f, const uint64_t X[3], const float u[3],
                                           const ModeF* smodes, FieldCache& fc)
{
    float E[3], B[3];
    field_mixed<SYS>(f, X, E, B, smodes, fc);
    float bb = sqrtf(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    float uu = sqrtf(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    return (double)((B[0] * u[0] + B[1] * u[1] + B[2] * u[2]) / (bb * uu));
}

__device__ __forceinline__ void block_diff_sum(const double sg[8], double* red, double* slot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        double v = sg[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp * 8 + c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double s = 0.0;
        for (int w = 0; w < nwarps; w++) s += red[w * 8 + threadIdx.x];
        slot[threadIdx.x] += s;
    }
    __syncthreads();
}

// Persistent fixed-step tracking in mixed precision: the same schedule and
// diagnostics as the FP64 kernel (src/tracking.c:297-462); the mode table of
// the plane-wave field is staged once per block in shared memory.
template <int SYS>
__global__ void __launch_bounds__(kBlock) track_mixed_kernel(MixField f, TrackBufs b, TrackParams q)
{
    __shared__ double red[(kBlock / 32) * 8];
    __shared__ unsigned int hist[kMaxSmemBins];
    extern __shared__ ModeF smodes[];
    if (SYS == TP_SYS_MODESUM) {
        for (int m = threadIdx.x; m < f.nmodes; m += blockDim.x) smodes[m] = f.modes[m];
        __syncthreads();
    }
    const bool smem_hist = q.nbins <= kMaxSmemBins;
    const float dt = (float)q.dt;
    for (int tile = blockIdx.x; tile < q.ntiles; tile += gridDim.x) {
        const int i = tile * kBlock + threadIdx.x;
        const bool active = i < q.n;
        PM p = {};
        FieldCache fc;
        double x0[3] = {0, 0, 0}, u0[3] = {0, 0, 0}, tstart = 0.0, mu0 = 0.0;
        int nst = 1;
        bool esc = false;
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
            }
            p.u[0] = (float)b.ux[i]; p.u[1] = (float)b.uy[i]; p.u[2] = (float)b.uz[i];
            // mu of the initial state: the field at the initial position is static
            uint64_t X0[3];
            float uf0[3] = {(float)u0[0], (float)u0[1], (float)u0[2]};
#pragma unroll
            for (int k = 0; k < 3; k++) {
                double r = (x0[k] - f.min[k]) / f.L[k];
                X0[k] = __double2ull_rz((r - floor(r)) * 18446744073709551616.0);
            }
            mu0 = pitch_mu<SYS>(f, X0, uf0, smodes, fc);
        }
        int esc_pre = esc ? 1 : 0;
        int esc_after = esc_pre;
        int ntp = q.ntp0, tstep = 1;
        double sg[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (active && esc_pre) atomicSub(&b.remain[1], 1);
        double* slot_base = b.dpart + (size_t)blockIdx.x * q.nsdc * 8;
        int done = 0;
        for (int j = q.sstep; j <= q.estep; j++) {
            sg[0] = 0.0; sg[4] = 0.0; sg[5] = 0.0;
            if (active && (esc_pre == 0 || f.bc_flag == 0)) {
                bool e2 = false;
                wirz_mixed<SYS>(f, p, dt, smodes, fc, e2);
                if (e2) esc_after = 1;
                nst += 1;
                done += 1;
                if (esc_after == 0 && j % kDiffInterval == 0) {
                    // calc_diff_coeff, src/diagnostics.c:659-705, FP64 accumulation
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
                    double mu = pitch_mu<SYS>(f, p.X, p.u, smodes, fc);
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
            if (j % q.einterval == 0) {
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
            if (j % kDiffInterval == 0) {
                block_diff_sum(sg, red, slot_base + (size_t)tstep * 8);
                tstep++;
            }
            if (active && esc_after && j % kDiffInterval == 0 && tstep < q.nsdc)
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
            b.t[i] = tstart + done * q.dt;
            b.nsteps_ptl[i] = nst;
        }
    }
}

// --------------------------------------------------------------- launchers
template <int SYS>
static cudaError_t launch_sys(const MixField& f, const TrackBufs& b, const TrackParams& q, int grid,
                              cudaStream_t s)
{
    size_t smem = SYS == TP_SYS_MODESUM ? sizeof(ModeF) * (size_t)f.nmodes : 0;
    if (smem > 48 * 1024) {
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
    size_t smem = system_type == TP_SYS_MODESUM ? sizeof(ModeF) * (size_t)nmodes : 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (system_type) {
    case TP_SYS_TEST: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_TEST>, kBlock, 0); break;
    case TP_SYS_FORCEFREE: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_FORCEFREE>, kBlock, 0); break;
    case TP_SYS_PIC: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_PIC>, kBlock, 0); break;
    case TP_SYS_MODESUM:
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(track_mixed_kernel<TP_SYS_MODESUM>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_mixed_kernel<TP_SYS_MODESUM>, kBlock, smem);
        break;
    default: break;
    }
    return e == cudaSuccess ? nb : 0;
}

// Interleaved node layout for the gathers: per node {Ex,Ey,Ez,0},{Bx,By,Bz,0}
// (32 bytes, one sector) built from the reference's AoS float E and B arrays.
__global__ void interleave_kernel(const float* __restrict__ e, const float* __restrict__ bf,
                                  size_t n, float4* __restrict__ eb)
{
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    eb[2 * i] = make_float4(e ? e[3 * i] : 0.f, e ? e[3 * i + 1] : 0.f, e ? e[3 * i + 2] : 0.f, 0.f);
    eb[2 * i + 1] = make_float4(bf[3 * i], bf[3 * i + 1], bf[3 * i + 2], 0.f);
}

cudaError_t launch_interleave(const float* e, const float* bf, size_t n, float4* eb, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    interleave_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(e, bf, n, eb);
    return cudaGetLastError();
}

}  // namespace mixed
}  // namespace tp
