// wirz_f32.cuh -- the FP32 Wirz push on 64-bit fixed-point positions and
// the per-block diagnostic reductions shared by the mixed-precision kernels.
#pragma once
#include "tp_mixed.cuh"

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

// Box fraction -> signed 64-bit fixed point (fr * 2^64) with 32-bit
// conversions only (64-bit float-to-integer conversions run on the FP64 pipe,
// a 64th of the FP32 rate on this part).  |fr| < 0.5: fr * 2^64 = hi * 2^32 +
// lo with hi = floor(fr * 2^32) and lo = the fraction below it times 2^32,
// two's complement without a sign branch.
__device__ __forceinline__ int64_t float_to_fx(float fr)
{
    const float a = fr * 4294967296.0f;
    const float fh = floorf(a);
    const uint32_t hi = (uint32_t)__float2int_rz(fh);
    const uint32_t lo = __float2uint_rz((a - fh) * 4294967296.0f);
    return (int64_t)(((uint64_t)hi << 32) | lo);
}

// Adds a displacement (in box fractions) to a position, counting periods:
// the period count takes the carry out of the 64-bit sum, less one for a
// negative displacement.
__device__ __forceinline__ void advance(uint64_t& X, int& img, float fr)
{
    const int64_t d = float_to_fx(fr);
    const uint64_t nx = X + (uint64_t)d;
    img += (int)(nx < X) - (int)(d < 0);
    X = nx;
}

// One Wirz push; field(X, E, B) evaluates the field at a fixed-point position.
template <class FieldFn>
__device__ __forceinline__ void wirz_f32(const MixField& f, PM& p, float dt, FieldFn&& field,
                                         bool& escaped)
{
    // Norms and their inverses come from one rsqrt each (a single SFU
    // operation, a few ulp): the FP32 path's error budget is set by FP32
    // rounding of the push, not by these.
    const float cm = f.cm, icm = 1.0f / f.cm;
    float E[3], B[3];
    field(p.X, E, B);
    float B2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
    float iB = rsqrtf(B2);
    float Btot = B2 * iB;
    float h[3] = {B[0] * iB, B[1] * iB, B[2] * iB};
    const float hk = 0.5f * cm * dt;
    float um[3] = {p.u[0] + hk * E[0], p.u[1] + hk * E[1], p.u[2] + hk * E[2]};
    float ig = rsqrtf(1.0f + um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);  // 1 / gamma
    // frame at the start point
    float w[3] = {h[1] * um[2] - h[2] * um[1], h[2] * um[0] - h[0] * um[2], h[0] * um[1] - h[1] * um[0]};
    float w2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    float iu = w2 > 0.0f ? rsqrtf(w2) : 0.0f;
    float uperp = w2 * iu;
    float hr[3] = {w[0] * iu, w[1] * iu, w[2] * iu};
    float hp[3] = {hr[1] * h[2] - hr[2] * h[1], hr[2] * h[0] - hr[0] * h[2], hr[0] * h[1] - hr[1] * h[0]};
    float upar = um[0] * h[0] + um[1] * h[1] + um[2] * h[2];
    float theta = cm * Btot * ig * dt;
    float s4, c4;
    __sincosf(0.25f * theta, &s4, &c4);
    float sin_h = 2.0f * s4 * c4, omc_h = 2.0f * s4 * s4;  // sin(theta/2), 1 - cos(theta/2)
    float R = uperp * iB * icm;  // uperp / (cm |B|)
    float a1 = 0.5f * dt * upar * ig, a2 = R * sin_h, a3 = -R * omc_h;
    float dpre[3];
#pragma unroll
    for (int k = 0; k < 3; k++) dpre[k] = (h[k] * a1 + hp[k] * a2 + hr[k] * a3) * f.invL[k];
    // The midpoint is only sampled, and the field evaluations read the top 32
    // bits of a position: a 32-bit fixed-point step is enough there.
    uint64_t Xp[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        Xp[k] = (uint64_t)((uint32_t)(p.X[k] >> 32) + (uint32_t)__float2int_rn(dpre[k] * 4294967296.0f)) << 32;
    field(Xp, E, B);
    B2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
    iB = rsqrtf(B2);
    Btot = B2 * iB;
    h[0] = B[0] * iB; h[1] = B[1] * iB; h[2] = B[2] * iB;
    w[0] = h[1] * um[2] - h[2] * um[1];
    w[1] = h[2] * um[0] - h[0] * um[2];
    w[2] = h[0] * um[1] - h[1] * um[0];
    w2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    iu = w2 > 0.0f ? rsqrtf(w2) : 0.0f;
    uperp = w2 * iu;
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
    R = uperp * iB * icm;
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

}  // namespace mixed
}  // namespace tp
