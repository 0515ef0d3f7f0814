// track_fp64.cu -- FP64 tracking path: the Wirz push, boundary conditions,
// energy binning and diffusion coefficients in the reference's arithmetic,
// and the persistent fixed-step tracking kernel with fused diagnostics.
//
// Built twice: with -fmad=false as the parity path (TP_FP64_NS = fp64) and
// with -fmad=true as the fast FP64 path (TP_FP64_NS = fp64fast, -DTP_FAST).
#include "fields_fp64.cuh"
#include "tp_kernels.h"

#ifndef TP_FP64_NS
#define TP_FP64_NS fp64
#endif

namespace tp {
namespace TP_FP64_NS {

struct P64 {
    double x, y, z, ux, uy, uz, t, xs, ys, zs;
};

// tracking_wirz, src/tracking.c:749-892 (c0_norm = 1)
template <int SYS>
__device__ __forceinline__ void wirz(const DevField& f, P64& p, double dt, int* status)
{
    const double cm = f.charge_mass;
    double e[6];
    double t0 = p.t;
    double gama = sqrt(1.0 + p.ux * p.ux + p.uy * p.uy + p.uz * p.uz);
    emf64<SYS>(f, p.x, p.y, p.z, t0, e, status);
    double Btot = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    double iBtot = 1.0 / Btot;
    double dth = dt * 0.5;
    double dm0 = p.ux + cm * dth * e[3];
    double dm1 = p.uy + cm * dth * e[4];
    double dm2 = p.uz + cm * dth * e[5];
    gama = sqrt(1.0 + dm0 * dm0 + dm1 * dm1 + dm2 * dm2);
    double igama = 1.0 / gama;
    double vm0 = dm0 * igama, vm1 = dm1 * igama, vm2 = dm2 * igama;
    double h0 = e[0] * iBtot, h1 = e[1] * iBtot, h2 = e[2] * iBtot;
    double vdothp = 0.0;
    vdothp += vm0 * h0;
    vdothp += vm1 * h1;
    vdothp += vm2 * h2;
    double q0 = vm0 - vdothp * h0, q1 = vm1 - vdothp * h1, q2 = vm2 - vdothp * h2;
    double vperp = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
    double hp0 = (vm0 - vdothp * h0) / vperp;
    double hp1 = (vm1 - vdothp * h1) / vperp;
    double hp2 = (vm2 - vdothp * h2) / vperp;
    double hr0 = h1 * hp2 - h2 * hp1;
    double hr1 = h2 * hp0 - h0 * hp2;
    double hr2 = h0 * hp1 - h1 * hp0;
    double gyroR = vperp * gama * 1.0 * iBtot / cm;
    double omegac = cm * Btot * igama;
    double dtheta = omegac * dt;
    double sind = sin(dtheta * 0.5), cosd = cos(dtheta * 0.5);
    double tmp1 = dth * vdothp * 1.0, tmp2 = gyroR * sind, tmp3 = -gyroR * (1.0 - cosd);
    double px = p.x + h0 * tmp1 + hp0 * tmp2 + hr0 * tmp3;
    double py = p.y + h1 * tmp1 + hp1 * tmp2 + hr1 * tmp3;
    double pz = p.z + h2 * tmp1 + hp2 * tmp2 + hr2 * tmp3;
    emf64<SYS>(f, px, py, pz, t0 + dth, e, status);
    Btot = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    iBtot = 1.0 / Btot;
    h0 = e[0] * iBtot; h1 = e[1] * iBtot; h2 = e[2] * iBtot;
    vdothp = 0.0;
    vdothp += vm0 * h0;
    vdothp += vm1 * h1;
    vdothp += vm2 * h2;
    q0 = vm0 - vdothp * h0; q1 = vm1 - vdothp * h1; q2 = vm2 - vdothp * h2;
    vperp = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
    hp0 = (vm0 - vdothp * h0) / vperp;
    hp1 = (vm1 - vdothp * h1) / vperp;
    hp2 = (vm2 - vdothp * h2) / vperp;
    hr0 = h1 * hp2 - h2 * hp1;
    hr1 = h2 * hp0 - h0 * hp2;
    hr2 = h0 * hp1 - h1 * hp0;
    omegac = cm * Btot * igama;
    dtheta = omegac * dt;
    sind = sin(dtheta);
    cosd = cos(dtheta);
    double vp0 = h0 * vdothp + vperp * (cosd * hp0 - sind * hr0);
    double vp1 = h1 * vdothp + vperp * (cosd * hp1 - sind * hr1);
    double vp2 = h2 * vdothp + vperp * (cosd * hp2 - sind * hr2);
    double bm = 0.0;  // get_delta_vec, src/tracking.c:1066-1078
    bm += vp0 * vp0;
    bm += vp1 * vp1;
    bm += vp2 * vp2;
    double g2 = 1.0 / sqrt(1.0 - bm);
    p.ux = g2 * vp0 + cm * dth * e[3];
    p.uy = g2 * vp1 + cm * dth * e[4];
    p.uz = g2 * vp2 + cm * dth * e[5];
    vdothp = 0.0;
    vdothp += vp0 * h0;
    vdothp += vp1 * h1;
    vdothp += vp2 * h2;
    q0 = vp0 - vdothp * h0; q1 = vp1 - vdothp * h1; q2 = vp2 - vdothp * h2;
    vperp = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
    gyroR = vperp * gama * 1.0 * iBtot / cm;
    tmp1 = dt * vdothp * 1.0;
    tmp2 = gyroR * sind;
    tmp3 = -gyroR * (1.0 - cosd);
    p.x += h0 * tmp1 + hp0 * tmp2 + hr0 * tmp3;
    p.y += h1 * tmp1 + hp1 * tmp2 + hr1 * tmp3;
    p.z += h2 * tmp1 + hp2 * tmp2 + hr2 * tmp3;
    p.t += dt;
}

// particle_bc, src/tracking.c:1172-1221
__device__ __forceinline__ void particle_bc(const DevField& f, P64& p, int& iescape)
{
    double xdim = f.xmax - f.xmin, ydim = f.ymax - f.ymin, zdim = f.zmax - f.zmin;
    if (f.bc_flag == 0) {
        if (p.x > f.xmax) { p.x -= xdim; p.xs += xdim; }
        if (p.y > f.ymax) { p.y -= ydim; p.ys += ydim; }
        if (p.z > f.zmax) { p.z -= zdim; p.zs += zdim; }
        if (p.x < f.xmin) { p.x += xdim; p.xs -= xdim; }
        if (p.y < f.ymin) { p.y += ydim; p.ys -= ydim; }
        if (p.z < f.zmin) { p.z += zdim; p.zs -= zdim; }
    } else if (f.bc_flag == 1) {
        if ((p.x > f.xmax) || (p.y > f.ymax) || (p.z > f.zmax) || (p.x < f.xmin) ||
            (p.y < f.ymin) || (p.z < f.zmin))
            iescape = 1;
    } else if (f.bc_flag == 2) {
        iescape = 0;
    }
}

// ptl_energy_fixed binning, src/diagnostics.c:187-205, done exactly by
// comparing against thresholds the host derived from the reference formula:
// the bin is the number of thresholds <= e.  NaN, e <= 0 and e = +inf give
// bin 0 as the reference does on x86.
__device__ __forceinline__ int energy_bin(const double* thr, int nbins, double ux, double uy,
                                          double uz)
{
    double gama = sqrt(1.0 + ux * ux + uy * uy + uz * uz);
    double e = gama - 1.0;
    if (!(e < INFINITY)) return 0;
    int lo = 0, hi = nbins - 1;  // answer in [0, nbins-1]
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;  // is thr[mid-1] <= e ?
        if (__ldg(thr + mid - 1) <= e) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// calc_diff_coeff, src/diagnostics.c:659-705 (pow(v, 2) taken as v * v).
// Output order: drr, dxx, dyy, dzz, dpp, duu, daa, dee.
template <int SYS>
__device__ __forceinline__ void calc_diff(const DevField& f, const P64& p0, const P64& p,
                                          double dt, double o[8], int* status)
{
    double t = p.t * 2 + dt;
    double a = p0.x - (p.x + p.xs), b = p0.y - (p.y + p.ys), c = p0.z - (p.z + p.zs);
    double dxx = a * a / t, dyy = b * b / t, dzz = c * c / t;
    double drr = dxx + dyy + dzz;
    double d0 = p0.ux - p.ux, d1 = p0.uy - p.uy, d2 = p0.uz - p.uz;
    double dpp = (d0 * d0 + d1 * d1 + d2 * d2) / t;
    double gamma = sqrt(1.0 + p.ux * p.ux + p.uy * p.uy + p.uz * p.uz);
    double gamma0 = sqrt(1.0 + p0.ux * p0.ux + p0.uy * p0.uy + p0.uz * p0.uz);
    double dg = gamma - gamma0;
    double dee = dg * dg / t;
    double e[6], e0[6];
    emf64<SYS>(f, p.x, p.y, p.z, p.t, e, status);
    emf64<SYS>(f, p0.x, p0.y, p0.z, p0.t, e0, status);
    double abs_b = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    double abs_u = sqrt(p.ux * p.ux + p.uy * p.uy + p.uz * p.uz);
    double mu = (e[0] * p.ux + e[1] * p.uy + e[2] * p.uz) / (abs_b * abs_u);
    abs_b = sqrt(e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2]);
    abs_u = sqrt(p0.ux * p0.ux + p0.uy * p0.uy + p0.uz * p0.uz);
    double mu0 = (e0[0] * p0.ux + e0[1] * p0.uy + e0[2] * p0.uz) / (abs_b * abs_u);
    double dmu = mu - mu0;
    double duu = dmu * dmu / t;
    double theta = acos(mu) * 180 / TP_PI;
    double theta0 = acos(mu0) * 180 / TP_PI;
    double dth = theta - theta0;
    double daa = dth * dth / t;
    o[0] = drr; o[1] = dxx; o[2] = dyy; o[3] = dzz;
    o[4] = dpp; o[5] = duu; o[6] = daa; o[7] = dee;
}

__device__ __forceinline__ void load(const TrackBufs& b, int i, P64& p)
{
    p.x = b.x[i]; p.y = b.y[i]; p.z = b.z[i];
    p.ux = b.ux[i]; p.uy = b.uy[i]; p.uz = b.uz[i];
    p.t = b.t[i]; p.xs = b.xs[i]; p.ys = b.ys[i]; p.zs = b.zs[i];
}

__device__ __forceinline__ void store(const TrackBufs& b, int i, const P64& p)
{
    b.x[i] = p.x; b.y[i] = p.y; b.z[i] = p.z;
    b.ux[i] = p.ux; b.uy[i] = p.uy; b.uz[i] = p.uz;
    b.t[i] = p.t; b.xs[i] = p.xs; b.ys[i] = p.ys; b.zs[i] = p.zs;
}

// Deterministic block sum of the eight per-particle diffusion values into this
// block's slice of the partial-sum scratch: warp tree, then warps in order.
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

// Persistent fixed-step tracking, restating particle_tracking_multi_steps_openmp
// and _single_step_openmp (src/tracking.c:297-462): one thread owns one
// particle for all estep steps; blocks walk tiles of kBlock particles.  All
// threads of a block run the same step sequence, so the diagnostic steps
// (every einterval steps for the spectrum, every 100 for the diffusion sums)
// are block-uniform and reduce through shared memory.
template <int SYS>
__global__ void __launch_bounds__(kBlock) track_kernel(DevField f, TrackBufs b, TrackParams q)
{
    __shared__ double red[(kBlock / 32) * 8];
    __shared__ unsigned int hist[kMaxSmemBins];
    const bool smem_hist = q.nbins <= kMaxSmemBins;
    for (int tile = blockIdx.x; tile < q.ntiles; tile += gridDim.x) {
        const int slot = tile * kBlock + threadIdx.x;
        const bool active = slot < q.n;
        const int i = active && q.idx ? q.idx[slot] : slot;  // the particle of this lane
        P64 p = {}, p0 = {};
        int nst = 1;
        if (active) {
            load(b, i, p);
            p0.x = b.x0[i]; p0.y = b.y0[i]; p0.z = b.z0[i];
            p0.ux = b.ux0[i]; p0.uy = b.uy0[i]; p0.uz = b.uz0[i]; p0.t = b.t0[i];
            nst = b.nsteps_ptl[i];
        }
        int esc_pre = 0;
        if (active) particle_bc(f, p, esc_pre);
        int esc_after = esc_pre;
        int ntp = q.ntp0, tstep = 1 + q.row0;
        double sg[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (active && q.resumed && b.sg_carry) {
#pragma unroll
            for (int c = 0; c < 8; c++) sg[c] = b.sg_carry[(size_t)i * kSegCarry + c];
        }
        if (active && esc_pre && !q.resumed) atomicSub(&b.remain[1], 1);
        double* slot_base = b.dpart + (size_t)blockIdx.x * q.nsdc * 8;
        int npts = 1;
        long toff = 0;
        if (active && q.traj_every > 0) {
            npts = b.ntraj_points[i];
            toff = i > 0 ? (long)b.ntraj_accum[i - 1] : 0;
        }
        for (int j = q.sstep; j <= q.estep; j++) {
            sg[0] = 0.0; sg[4] = 0.0; sg[5] = 0.0;  // src/tracking.c:334-336
            if (active && (esc_pre == 0 || f.bc_flag == 0)) {
                wirz<SYS>(f, p, q.dt, b.status);
                particle_bc(f, p, esc_after);
                nst += 1;
                if (esc_after == 0 && j % kDiffInterval == 0)
                    calc_diff<SYS>(f, p0, p, q.dt, sg, b.status);
                if (q.traj_every > 0 && j % q.traj_every == 0) {
                    // trajectory point, src/tracking.c:440-447
                    long off = toff + npts;
                    if (off >= 0 && off < b.ntraj_total) {
                        double* r = b.ptl_time + 11 * off;
                        r[0] = p.x; r[1] = p.y; r[2] = p.z; r[3] = b.qm[i];
                        r[4] = p.ux; r[5] = p.uy; r[6] = p.uz; r[7] = p.t;
                        r[8] = p.xs; r[9] = p.ys; r[10] = p.zs;
                    } else {
                        atomicOr(b.status, ST_BAD_INDEX);
                    }
                    npts++;
                }
            }
            if (active && esc_pre == 0 && esc_after == 1 && f.bc_flag == 1 && ntp < q.nt_out)
                atomicAdd(&b.espect_esc[ntp * q.nbins +
                                        energy_bin(b.ebin_thr, q.nbins, p.ux, p.uy, p.uz)], 1u);
            if (j % q.einterval == 0) {  // block-uniform
                if (ntp < q.nt_out) {
                    bool take = active && esc_after == 0;
                    if (smem_hist) {
                        __syncthreads();
                        for (int k = threadIdx.x; k < q.nbins; k += blockDim.x) hist[k] = 0u;
                        __syncthreads();
                        if (take) atomicAdd(&hist[energy_bin(b.ebin_thr, q.nbins, p.ux, p.uy, p.uz)], 1u);
                        __syncthreads();
                        for (int k = threadIdx.x; k < q.nbins; k += blockDim.x)
                            if (hist[k]) atomicAdd(&b.espect[ntp * q.nbins + k], hist[k]);
                    } else if (take) {
                        atomicAdd(&b.espect[ntp * q.nbins +
                                            energy_bin(b.ebin_thr, q.nbins, p.ux, p.uy, p.uz)], 1u);
                    }
                }
                ntp++;
            }
            if (j % kDiffInterval == 0) {  // block-uniform
                block_diff_sum(sg, red, slot_base + (size_t)tstep * 8);
                tstep++;
            }
            if (active && esc_after && j % kDiffInterval == 0 && tstep < q.nsdc)
                atomicSub(&b.remain[tstep], 1);
            esc_pre = esc_after;
        }
        if (active) {
            // the index again from the list rather than held through the loop
            const int ie = q.idx ? q.idx[tile * kBlock + threadIdx.x] : tile * kBlock + threadIdx.x;
            store(b, ie, p);
            b.nsteps_ptl[ie] = nst;
            if (q.traj_every > 0) b.ntraj_points[ie] = npts;
            if (b.sg_carry) {
#pragma unroll
                for (int c = 0; c < 8; c++) b.sg_carry[(size_t)ie * kSegCarry + c] = sg[c];
            }
            if (b.esc_out) b.esc_out[ie] = esc_after;
        }
    }
}

// Fixed-order sum of the per-block partials: dsum[c * nsdc + s] (component-major).
__global__ void reduce_dpart_kernel(const double* dpart, int nblocks, int nsdc, double* dsum)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;  // k = s * 8 + c
    if (k >= nsdc * 8) return;
    double s = 0.0;
    for (int bidx = 0; bidx < nblocks; bidx++) s += dpart[(size_t)bidx * nsdc * 8 + k];
    dsum[(k & 7) * nsdc + (k >> 3)] = s;
}

// ---------------------------------------------------------------- batch utilities
__global__ void emf_batch_kernel(DevField f, int n, const double* xyzt, double* out, int* status)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double e[6];
    emf64_dispatch(f, xyzt[4 * i], xyzt[4 * i + 1], xyzt[4 * i + 2], xyzt[4 * i + 3], e, status);
    for (int k = 0; k < 6; k++) out[6 * i + k] = e[k];
}

template <int SYS>
__global__ void wirz_steps_kernel(DevField f, int n, double* st, int nsteps, double dt,
                                  int* iescape, int* status)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* r = st + (size_t)11 * i;  // particles record, include/particle_info.h:6-12
    P64 p = {r[0], r[1], r[2], r[4], r[5], r[6], r[7], r[8], r[9], r[10]};
    int esc = iescape ? iescape[i] : 0;
    for (int s = 0; s < nsteps; s++) {
        wirz<SYS>(f, p, dt, status);
        if (iescape) particle_bc(f, p, esc);  // no iescape: tracking_wirz alone
    }
    r[0] = p.x; r[1] = p.y; r[2] = p.z; r[4] = p.ux; r[5] = p.uy; r[6] = p.uz;
    r[7] = p.t; r[8] = p.xs; r[9] = p.ys; r[10] = p.zs;
    if (iescape) iescape[i] = esc;
}

__global__ void ebin_kernel(const double* thr, int nbins, int n, const double* st, int* bins)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* r = st + (size_t)11 * i;
    bins[i] = energy_bin(thr, nbins, r[4], r[5], r[6]);
}

template <int SYS>
__global__ void diffc_kernel(DevField f, int n, const double* st0, const double* st, double dt,
                             double* out, int* status)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* r = st + (size_t)11 * i;
    const double* r0 = st0 + (size_t)11 * i;
    P64 p = {r[0], r[1], r[2], r[4], r[5], r[6], r[7], r[8], r[9], r[10]};
    P64 p0 = {r0[0], r0[1], r0[2], r0[4], r0[5], r0[6], r0[7], r0[8], r0[9], r0[10]};
    double o[8];
    calc_diff<SYS>(f, p0, p, dt, o, status);
    for (int k = 0; k < 8; k++) out[8 * i + k] = o[k];
}

__global__ void trilinear_kernel(DevField f, int n, const double* xyzt, long* corners,
                                 double* weights)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Tri64 r;
    trilinear64(f, xyzt[4 * i], xyzt[4 * i + 1], xyzt[4 * i + 2], xyzt[4 * i + 3], r);
    for (int k = 0; k < 8; k++) {
        corners[8 * i + k] = r.c[k];
        weights[8 * i + k] = r.w[k];
    }
}

// particle_bc on a batch of particles records
__global__ void bc_kernel(DevField f, int n, double* st, int* iescape)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* r = st + (size_t)11 * i;
    P64 p = {r[0], r[1], r[2], r[4], r[5], r[6], r[7], r[8], r[9], r[10]};
    int esc = iescape[i];
    particle_bc(f, p, esc);
    r[0] = p.x; r[1] = p.y; r[2] = p.z; r[8] = p.xs; r[9] = p.ys; r[10] = p.zs;
    iescape[i] = esc;
}

// get_{float,double}_{b,e,velocity}_at_point (src/magnetic_field.c:555-622,
// src/electric_field.c:370-437, src/velocity_field.c:555-622).  which:
// 0 B float, 1 E float, 2 v float, 3 B double, 4 E double, 5 v double.
__global__ void point_interp_kernel(DevField f, int which, int n, const double* xyzt,
                                    double* out, int* status)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Tri64 r;
    trilinear64(f, xyzt[4 * i], xyzt[4 * i + 1], xyzt[4 * i + 2], xyzt[4 * i + 3], r);
    if (which <= 2) {
        const float *c = which == 0 ? f.bc_f : which == 1 ? f.ec_f : f.vc_f;
        const float *a = which == 0 ? f.ba_f : which == 1 ? f.ea_f : f.va_f;
        const float *b = which == 0 ? f.bb_f : which == 1 ? f.eb_f : f.vb_f;
        float v[3] = {0.f, 0.f, 0.f};
        if ((f.multi_tframe == 0 && c) || (f.multi_tframe != 0 && a && b))
            interp_f3(f, r, c, a, b, v, status);
        else
            atomicOr(status, ST_BAD_INDEX);
        out[3 * i] = v[0]; out[3 * i + 1] = v[1]; out[3 * i + 2] = v[2];
    } else {
        const double *c = which == 3 ? f.bc_d : which == 4 ? f.ec_d : f.vc_d;
        const double *a = which == 3 ? f.ba_d : which == 4 ? f.ea_d : f.va_d;
        const double *b = which == 3 ? f.bb_d : which == 4 ? f.eb_d : f.vb_d;
        double v[3] = {0.0, 0.0, 0.0};
        if ((f.multi_tframe == 0 && c) || (f.multi_tframe != 0 && a && b))
            interp_d3(f, r, c, a, b, v, status);
        else
            atomicOr(status, ST_BAD_INDEX);
        out[3 * i] = v[0]; out[3 * i + 1] = v[1]; out[3 * i + 2] = v[2];
    }
}

// ---------------------------------------------------------------- Poincare map
// Field lines of the gridded B (get_magnetic_field, src/emfields.c:76-96:
// the float B grid for systems 3 and 4) traced with the fixed-step RK4 of
// next_location (src/poincare_map.c:243-290) on the unit vector of B, the
// stage points wrapped into the box (field_boundary, :296-321), and the
// crossings of the plane pos[face] = seed[face] recorded as the first point
// after a sign change (:158-181).  One thread per seed.
__device__ __forceinline__ void pm_boundary(const DevField& f, double& x, double& y, double& z)
{
    double xdim = f.xmax - f.xmin, ydim = f.ymax - f.ymin, zdim = f.zmax - f.zmin;
    if (x > f.xmax) x -= xdim;
    if (y > f.ymax) y -= ydim;
    if (z > f.zmax) z -= zdim;
    if (x < f.xmin) x += xdim;
    if (y < f.ymin) y += ydim;
    if (z < f.zmin) z += zdim;
}

__device__ __forceinline__ void pm_unit_b(const DevField& f, double x, double y, double z, double b[3],
                                          int* status)
{
    Tri64 r;
    trilinear64(f, x, y, z, 0.0, r);
    float v[3];
    interp_f3(f, r, f.bc_f, f.ba_f, f.bb_f, v, status);
    double bx = v[0], by = v[1], bz = v[2];
    double ib = 1.0 / sqrt(bx * bx + by * by + bz * bz);
    b[0] = bx * ib;
    b[1] = by * ib;
    b[2] = bz * ib;
}

__device__ __forceinline__ void pm_next(const DevField& f, double& px, double& py, double& pz, double h,
                                        int* status)
{
    double b1[3], b2[3], b3[3], b4[3], xt, yt, zt;
    pm_boundary(f, px, py, pz);
    pm_unit_b(f, px, py, pz, b1, status);
    xt = px + 0.5 * h * b1[0];
    yt = py + 0.5 * h * b1[1];
    zt = pz + 0.5 * h * b1[2];
    pm_boundary(f, xt, yt, zt);
    pm_unit_b(f, xt, yt, zt, b2, status);
    xt = px + 0.5 * h * b2[0];
    yt = py + 0.5 * h * b2[1];
    zt = pz + 0.5 * h * b2[2];
    pm_boundary(f, xt, yt, zt);
    pm_unit_b(f, xt, yt, zt, b3, status);
    xt = px + h * b3[0];
    yt = py + h * b3[1];
    zt = pz + h * b3[2];
    pm_boundary(f, xt, yt, zt);
    pm_unit_b(f, xt, yt, zt, b4, status);
    px += (h / 6) * (b1[0] + 2 * b2[0] + 2 * b3[0] + b4[0]);
    py += (h / 6) * (b1[1] + 2 * b2[1] + 2 * b3[1] + b4[1]);
    pz += (h / 6) * (b1[2] + 2 * b2[2] + 2 * b3[2] + b4[2]);
}

// outputs [n][ncross + 1] per coordinate; entries a seed does not reach keep
// the reference's fill value 2 * max of the axis
__global__ void poincare_kernel(DevField f, int n, const double* __restrict__ seeds, int face, double h,
                                double lmax, int ncross, double* xo, double* yo, double* zo, int* found,
                                int* status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t row = (size_t)i * (ncross + 1);
    for (int k = 0; k <= ncross; k++) {
        xo[row + k] = f.xmax * 2;
        yo[row + k] = f.ymax * 2;
        zo[row + k] = f.zmax * 2;
    }
    double pos[3] = {seeds[3 * i], seeds[3 * i + 1], seeds[3 * i + 2]};
    const double init = pos[face];
    xo[row] = pos[0]; yo[row] = pos[1]; zo[row] = pos[2];
    int icross = 1;
    double length = 0.0;
    while (icross <= ncross) {
        double cross = 1.0;
        while (cross > 0 && length < lmax) {  // at most lmax / h steps in all
            double pre = pos[face];
            pm_next(f, pos[0], pos[1], pos[2], h, status);
            cross = (pre - init) * (pos[face] - init);
            length += h;
        }
        if (length < lmax) {
            xo[row + icross] = pos[0];
            yo[row + icross] = pos[1];
            zo[row + icross] = pos[2];
            ++icross;
        } else {
            break;
        }
    }
    found[i] = icross - 1;
}

cudaError_t launch_poincare(const DevField& f, int n, const double* seeds, int face, double h, double lmax,
                            int ncross, double* xo, double* yo, double* zo, int* found, int* status,
                            cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    poincare_kernel<<<(n + 127) / 128, 128, 0, s>>>(f, n, seeds, face, h, lmax, ncross, xo, yo, zo, found,
                                                    status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- host launchers
cudaError_t launch_bc(const DevField& f, int n, double* st, int* iescape, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    bc_kernel<<<(n + 127) / 128, 128, 0, s>>>(f, n, st, iescape);
    return cudaGetLastError();
}

cudaError_t launch_point_interp(const DevField& f, int which, int n, const double* xyzt,
                                double* out, int* status, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    point_interp_kernel<<<(n + 127) / 128, 128, 0, s>>>(f, which, n, xyzt, out, status);
    return cudaGetLastError();
}

template <int SYS>
static cudaError_t launch_track_sys(const DevField& f, const TrackBufs& b, const TrackParams& q,
                                    int grid, cudaStream_t s)
{
    track_kernel<SYS><<<grid, kBlock, 0, s>>>(f, b, q);
    return cudaGetLastError();
}

cudaError_t launch_track(const DevField& f, const TrackBufs& b, const TrackParams& q, int grid,
                         cudaStream_t s)
{
    switch (f.system_type) {
    case TP_SYS_TEST: return launch_track_sys<TP_SYS_TEST>(f, b, q, grid, s);
    case TP_SYS_WLCS: return launch_track_sys<TP_SYS_WLCS>(f, b, q, grid, s);
    case TP_SYS_FORCEFREE: return launch_track_sys<TP_SYS_FORCEFREE>(f, b, q, grid, s);
    case TP_SYS_MHD: return launch_track_sys<TP_SYS_MHD>(f, b, q, grid, s);
    case TP_SYS_PIC: return launch_track_sys<TP_SYS_PIC>(f, b, q, grid, s);
    case TP_SYS_MODESUM: return launch_track_sys<TP_SYS_MODESUM>(f, b, q, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

int track_max_blocks_per_sm(int system_type)
{
    int nb = 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (system_type) {
    case TP_SYS_TEST: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_kernel<TP_SYS_TEST>, kBlock, 0); break;
    case TP_SYS_WLCS: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_kernel<TP_SYS_WLCS>, kBlock, 0); break;
    case TP_SYS_FORCEFREE: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_kernel<TP_SYS_FORCEFREE>, kBlock, 0); break;
    case TP_SYS_MHD: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_kernel<TP_SYS_MHD>, kBlock, 0); break;
    case TP_SYS_PIC: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_kernel<TP_SYS_PIC>, kBlock, 0); break;
    case TP_SYS_MODESUM: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, track_kernel<TP_SYS_MODESUM>, kBlock, 0); break;
    default: break;
    }
    return e == cudaSuccess ? nb : 0;
}

cudaError_t launch_reduce_dpart(const double* dpart, int nblocks, int nsdc, double* dsum,
                                cudaStream_t s)
{
    int n = nsdc * 8;
    reduce_dpart_kernel<<<(n + 127) / 128, 128, 0, s>>>(dpart, nblocks, nsdc, dsum);
    return cudaGetLastError();
}

cudaError_t launch_emf_batch(const DevField& f, int n, const double* xyzt, double* out,
                             int* status, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    emf_batch_kernel<<<(n + 127) / 128, 128, 0, s>>>(f, n, xyzt, out, status);
    return cudaGetLastError();
}

cudaError_t launch_wirz_steps(const DevField& f, int n, double* st, int nsteps, double dt,
                              int* iescape, int* status, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    int g = (n + 127) / 128;
    switch (f.system_type) {
    case TP_SYS_TEST: wirz_steps_kernel<TP_SYS_TEST><<<g, 128, 0, s>>>(f, n, st, nsteps, dt, iescape, status); break;
    case TP_SYS_WLCS: wirz_steps_kernel<TP_SYS_WLCS><<<g, 128, 0, s>>>(f, n, st, nsteps, dt, iescape, status); break;
    case TP_SYS_FORCEFREE: wirz_steps_kernel<TP_SYS_FORCEFREE><<<g, 128, 0, s>>>(f, n, st, nsteps, dt, iescape, status); break;
    case TP_SYS_MHD: wirz_steps_kernel<TP_SYS_MHD><<<g, 128, 0, s>>>(f, n, st, nsteps, dt, iescape, status); break;
    case TP_SYS_PIC: wirz_steps_kernel<TP_SYS_PIC><<<g, 128, 0, s>>>(f, n, st, nsteps, dt, iescape, status); break;
    case TP_SYS_MODESUM: wirz_steps_kernel<TP_SYS_MODESUM><<<g, 128, 0, s>>>(f, n, st, nsteps, dt, iescape, status); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_ebins(const double* thr, int nbins, int n, const double* st, int* bins,
                         cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    ebin_kernel<<<(n + 127) / 128, 128, 0, s>>>(thr, nbins, n, st, bins);
    return cudaGetLastError();
}

cudaError_t launch_diffc(const DevField& f, int n, const double* st0, const double* st,
                         double dt, double* out, int* status, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    int g = (n + 127) / 128;
    switch (f.system_type) {
    case TP_SYS_TEST: diffc_kernel<TP_SYS_TEST><<<g, 128, 0, s>>>(f, n, st0, st, dt, out, status); break;
    case TP_SYS_WLCS: diffc_kernel<TP_SYS_WLCS><<<g, 128, 0, s>>>(f, n, st0, st, dt, out, status); break;
    case TP_SYS_FORCEFREE: diffc_kernel<TP_SYS_FORCEFREE><<<g, 128, 0, s>>>(f, n, st0, st, dt, out, status); break;
    case TP_SYS_MHD: diffc_kernel<TP_SYS_MHD><<<g, 128, 0, s>>>(f, n, st0, st, dt, out, status); break;
    case TP_SYS_PIC: diffc_kernel<TP_SYS_PIC><<<g, 128, 0, s>>>(f, n, st0, st, dt, out, status); break;
    case TP_SYS_MODESUM: diffc_kernel<TP_SYS_MODESUM><<<g, 128, 0, s>>>(f, n, st0, st, dt, out, status); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_trilinear(const DevField& f, int n, const double* xyzt, long* corners,
                             double* weights, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    trilinear_kernel<<<(n + 127) / 128, 128, 0, s>>>(f, n, xyzt, corners, weights);
    return cudaGetLastError();
}

}  // namespace TP_FP64_NS
}  // namespace tp
