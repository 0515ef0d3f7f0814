// session.cu -- device-resident tracking sessions: particle state in HBM as
// SoA, one persistent tracking launch per run, diagnostics reduced on the GPU.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "../../include/tp_gpu.h"
#include "tp_internal.h"
#include "tp_kernels.h"
#include "tp_kernels_mixed.h"
#include "tp_session.h"
#include "mlp_common.cuh"

namespace tp {
namespace mlp {
cudaError_t launch_track_surrogate(const mixed::MixField& f, const Model& md, const TrackBufs& b,
                                   const TrackParams& q, int grid, cudaStream_t s);
}  // namespace mlp
}  // namespace tp

namespace tp {

__global__ void fill_int_kernel(int* p, int n, int v)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

static void fill_int(int* p, int n, int v, cudaStream_t s)
{
    if (n > 0) fill_int_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, n, v);
}

// ---------------------------------------------------------------- open-boundary segments
// Between the segments of an open-boundary run the particles still inside the
// box are compacted into an index list, in list order and independent of
// timing: per-block counts, one block that scans them and sums the departed
// particles' carried diffusion singles in block order, then the scatter.
constexpr int kCmpBlock = 1024;
// singles the reference keeps adding for a particle that no longer moves
// (dxx, dyy, dzz, daa, dee; drr, dpp, duu are cleared every step,
// src/tracking.c:334-336)
__constant__ int kStaleComp[5] = {1, 2, 3, 6, 7};

// exclusive scan over a block of kCmpBlock threads; total = the block's sum
__device__ __forceinline__ int block_excl_scan(int v, int* sh, int& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = sh[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    const int before = (warp > 0 ? sh[warp - 1] : 0) + x - v;
    total = sh[31];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(kCmpBlock) seg_count_kernel(const int* idx, int n, const int* esc,
                                                              const double* sg, int* cnt, double* part)
{
    __shared__ int sh[32];
    __shared__ double red[32][5];
    const int k = blockIdx.x * kCmpBlock + threadIdx.x;
    int keep = 0;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (k < n) {
        const int i = idx ? idx[k] : k;
        if (esc[i] == 0) {
            keep = 1;
        } else {
#pragma unroll
            for (int c = 0; c < 5; c++) v[c] = sg[(size_t)i * kSegCarry + kStaleComp[c]];
        }
    }
    int total;
    block_excl_scan(keep, sh, total);
    if (threadIdx.x == 0) cnt[blockIdx.x] = total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 5; c++) {
        double x = v[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][c] = x;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double t = 0.0;
        for (int w = 0; w < 32; w++) t += red[w][threadIdx.x];
        part[(size_t)blockIdx.x * 5 + threadIdx.x] = t;
    }
}

// One block: offsets of the kept particles per count block, the new count,
// and the departed particles' contributions to the diffusion rows row_lo ..
// row_hi (their singles, added at every later diffusion step) and to the
// remaining counts (one departure per later diffusion step), into `extra`,
// a slot of partial sums laid out like one tracking block's.
__global__ void __launch_bounds__(kCmpBlock) seg_scan_kernel(const int* cnt, const double* part, int nblk,
                                                             int n, int* off, int* n_next, double* extra,
                                                             int* remain, int nsdc, int row_lo, int row_hi)
{
    __shared__ int sh[32];
    int carry = 0;
    for (int b0 = 0; b0 < nblk; b0 += kCmpBlock) {
        const int b = b0 + threadIdx.x;
        const int v = b < nblk ? cnt[b] : 0;
        int total;
        const int pre = block_excl_scan(v, sh, total);
        if (b < nblk) off[b] = carry + pre;
        carry += total;
    }
    // one thread per component sums the blocks in order; one thread per row
    __shared__ double S[5];
    if (threadIdx.x < 5) {
        double t = 0.0;
        for (int b = 0; b < nblk; b++) t += part[(size_t)b * 5 + threadIdx.x];
        S[threadIdx.x] = t;
    }
    if (threadIdx.x == 0) *n_next = carry;
    __syncthreads();
    const int departed = n - carry;
    for (int r = row_lo + (int)threadIdx.x; r <= row_hi && r < nsdc; r += kCmpBlock) {
#pragma unroll
        for (int c = 0; c < 5; c++) extra[(size_t)r * 8 + kStaleComp[c]] += S[c];
        if (r + 1 < nsdc) remain[r + 1] -= departed;
    }
}

__global__ void __launch_bounds__(kCmpBlock) seg_scatter_kernel(const int* idx, int n, const int* esc,
                                                                const int* off, int* idx_out)
{
    __shared__ int sh[32];
    const int k = blockIdx.x * kCmpBlock + threadIdx.x;
    int keep = 0, i = 0;
    if (k < n) {
        i = idx ? idx[k] : k;
        keep = esc[i] == 0;
    }
    int total;
    const int pos = block_excl_scan(keep, sh, total);
    if (keep) idx_out[off[blockIdx.x] + pos] = i;
}

Session::~Session()
{
    for (Scratch* sc : {&soa, &soa0, &aos, &nsteps, &spec, &rem, &dpart, &dsum, &traj, &trajacc,
                        &trajpts, &cmp})
        sc->release();
    for (cudaEvent_t e : {ev0, ev1, evb, eve})
        if (e) cudaEventDestroy(e);
}

bool Session::reserve(int n)
{
    if (!ensure_init()) return false;
    if (!ev0) {
        cudaEventCreate(&ev0);
        cudaEventCreate(&ev1);
        cudaEventCreate(&evb);
        cudaEventCreate(&eve);
    }
    if (n <= cap) return true;
    size_t rec = sizeof(double) * 11 * (size_t)n;
    if (!soa.get(rec) || !soa0.get(rec) || !aos.get(rec) || !nsteps.get(sizeof(int) * (size_t)n))
        return false;
    cap = n;
    return true;
}

bool Session::load(const particles* ptl_init, const particles* ptl, int n_)
{
    if (!reserve(n_)) return false;
    n = n_;
    cudaStream_t s = g.stream;
    double* a = (double*)aos.ptr;
    if (n > 0) {
        if (!cuda_ok(cudaMemcpyAsync(a, ptl_init, sizeof(particles) * n, cudaMemcpyHostToDevice, s),
                     "load init")) return false;
        aos_to_soa(a, n, (double*)soa0.ptr, cap, s);
        if (!cuda_ok(cudaMemcpyAsync(a, ptl, sizeof(particles) * n, cudaMemcpyHostToDevice, s),
                     "load ptl")) return false;
        aos_to_soa(a, n, (double*)soa.ptr, cap, s);
    }
    loaded = true;
    return cuda_ok(cudaGetLastError(), "load");
}

bool Session::run(const RunSpec& rs, tp_run_info* info)
{
    if (!loaded) {
        set_error(1, "session: particles not loaded");
        return false;
    }
    if (rs.estep < rs.sstep || rs.einterval < 1 || rs.nt_out < 1) {
        set_error(6, "bad step range: sstep %d estep %d einterval %d nt_out %d", rs.sstep, rs.estep,
                  rs.einterval, rs.nt_out);
        return false;
    }
    // the kernels index the spectra [nt_out][nbins] with 32-bit integers
    if (rs.nbins < 1 || (long long)rs.nt_out * rs.nbins > INT_MAX) {
        set_error(6, "spectra of %d frames x %d bins: not supported", rs.nt_out, rs.nbins);
        return false;
    }
    DevField f;
    mixed::MixField mf;
    int nmodes = 0;
    const bool is_mixed = rs.precision == TP_PREC_MIXED;
    const bool is_surr = rs.precision == TP_PREC_SURROGATE;
    mlp::Model md;
    if (is_surr) {
        if (system_type != TP_SYS_MODESUM) {
            set_error(1, "the learned field model stands in for the mode-sum field (system type 5)");
            return false;
        }
        if (!build_mixfield(system_type, mf, &nmodes) || !mlp::mlp_model(md)) return false;
    } else if (is_mixed) {
        if (!build_mixfield(system_type, mf, &nmodes)) return false;
    } else if (!build_field(system_type, f)) {
        return false;
    }
    if (!ensure_thresholds(rs.nbins)) return false;
    cudaStream_t s = g.stream;
    nt_out = rs.nt_out;
    nbins = rs.nbins;
    nsdc = rs.estep / kDiffInterval + 1;
    const int ntiles = (n + kBlock - 1) / kBlock;
    int bps = 0;
    if (rs.precision == TP_PREC_FP64) bps = fp64::track_max_blocks_per_sm(system_type);
    else if (rs.precision == TP_PREC_FP64_FAST) bps = fp64fast::track_max_blocks_per_sm(system_type);
    else if (is_mixed) bps = mixed::track_max_blocks_per_sm(system_type, nmodes);
    else if (is_surr) bps = 1;
    else {
        set_error(1, "precision %d not available for system type %d", rs.precision, system_type);
        return false;
    }
    if (bps < 1) bps = 1;
    int grid = g.num_sms * bps;
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    // open boundaries: segments of seg steps with the departed particles
    // dropped.  Automatic mode: only when the tiles take more than one wave of
    // the grid (within one wave an idle lane costs nothing), about 8 segments
    // for the mixed path and 32 for the FP64 paths, whose steps cost ~60x more
    // against the fixed cost of a segment (measured on an open 128^3 box).
    const bool automatic = g.compact_steps < 0;
    // (64-bit: a segment length set near INT_MAX must not wrap when rounded up)
    long long seg_ll = !automatic ? (long long)g.compact_steps
                                  : (long long)std::max(kDiffInterval, rs.estep / (is_mixed ? 8 : 32));
    seg_ll = (seg_ll + kDiffInterval - 1) / kDiffInterval * kDiffInterval;
    const bool segs = bc_flag == 1 && g.compact_steps != 0 && rs.traj_every == 0 && !is_surr &&
                      rs.sstep == 1 && (long long)rs.estep > seg_ll && n > 0 &&
                      (!automatic || ntiles > grid);
    const int seg = (int)std::min<long long>(seg_ll, rs.estep);  // < estep whenever segs
    const int nslot = grid + (segs ? 1 : 0);  // the last slot takes the departed particles' rows
    size_t nspec = (size_t)nt_out * nbins;
    unsigned* d_spec = (unsigned*)spec.get(sizeof(unsigned) * 2 * nspec);
    int* d_rem = (int*)rem.get(sizeof(int) * nsdc);
    double* d_dpart = (double*)dpart.get(sizeof(double) * 8 * (size_t)nsdc * nslot);
    double* d_dsum = (double*)dsum.get(sizeof(double) * 8 * (size_t)nsdc);
    if (!d_spec || !d_rem || !d_dpart || !d_dsum) return false;
    const size_t nblk_max = ((size_t)n + kCmpBlock - 1) / kCmpBlock;
    double *c_sg = nullptr, *c_part = nullptr;
    int *c_idx0 = nullptr, *c_idx1 = nullptr, *c_esc = nullptr, *c_cnt = nullptr, *c_off = nullptr,
        *c_n = nullptr;
    if (segs) {
        char* c = (char*)cmp.get(sizeof(double) * ((size_t)kSegCarry * n + 5 * nblk_max) +
                                 sizeof(int) * (3 * (size_t)n + 2 * nblk_max + 1));
        if (!c) return false;
        c_sg = (double*)c;
        c_part = c_sg + (size_t)kSegCarry * n;
        c_idx0 = (int*)(c_part + 5 * nblk_max);
        c_idx1 = c_idx0 + n;
        c_esc = c_idx1 + n;
        c_cnt = c_esc + n;
        c_off = c_cnt + nblk_max;
        c_n = c_off + nblk_max;
    }
    cudaEventRecord(evb, s);
    cudaMemsetAsync(d_spec, 0, sizeof(unsigned) * 2 * nspec, s);
    cudaMemsetAsync(d_rem, 0, sizeof(int) * nsdc, s);
    cudaMemsetAsync(d_dpart, 0, sizeof(double) * 8 * (size_t)nsdc * nslot, s);
    if (rs.reset_nsteps) fill_int((int*)nsteps.ptr, n, 1, s);

    TrackBufs b;
    memset(&b, 0, sizeof(b));
    double* S = (double*)soa.ptr;
    double* S0 = (double*)soa0.ptr;
    long st = cap;
    b.x = S; b.y = S + st; b.z = S + 2 * st; b.qm = S + 3 * st;
    b.ux = S + 4 * st; b.uy = S + 5 * st; b.uz = S + 6 * st; b.t = S + 7 * st;
    b.xs = S + 8 * st; b.ys = S + 9 * st; b.zs = S + 10 * st;
    b.x0 = S0; b.y0 = S0 + st; b.z0 = S0 + 2 * st;
    b.ux0 = S0 + 4 * st; b.uy0 = S0 + 5 * st; b.uz0 = S0 + 6 * st; b.t0 = S0 + 7 * st;
    b.nsteps_ptl = (int*)nsteps.ptr;
    b.ebin_thr = g.d_thr;
    b.espect = d_spec;
    b.espect_esc = d_spec + nspec;
    b.remain = d_rem;
    b.dpart = d_dpart;
    b.status = g.d_status;
    if (rs.traj_every > 0) {
        b.ptl_time = (double*)traj.ptr;
        b.ntraj_accum = (const int*)trajacc.ptr;
        b.ntraj_points = (int*)trajpts.ptr;
        b.ntraj_total = traj_total;
    }
    TrackParams q;
    memset(&q, 0, sizeof(q));
    q.n = n;
    q.estep = rs.estep;
    q.einterval = rs.einterval;
    q.nt_out = nt_out;
    q.nbins = nbins;
    q.nsdc = nsdc;
    q.ntp0 = (int)floor(rs.sstep / (double)rs.einterval);
    q.ntiles = ntiles;
    q.sstep = rs.sstep;
    q.traj_every = rs.traj_every;
    q.dt = rs.dt;
    auto launch = [&](const TrackParams& qq, int gr) {
        return rs.precision == TP_PREC_FP64 ? fp64::launch_track(f, b, qq, gr, s)
             : is_mixed ? mixed::launch_track(mf, b, qq, gr, s)
             : is_surr  ? mlp::launch_track_surrogate(mf, md, b, qq, gr, s)
                        : fp64fast::launch_track(f, b, qq, gr, s);
    };
    int launches = 1;
    cudaEventRecord(ev0, s);
    if (!segs) {
        if (!cuda_ok(launch(q, grid), "track launch")) return false;
    } else {
        b.sg_carry = c_sg;
        b.esc_out = c_esc;
        double* extra = d_dpart + (size_t)grid * nsdc * 8;
        int n_act = n;
        const int* cur = nullptr;
        int* nxt = c_idx0;
        launches = 0;
        for (int s0 = rs.sstep;;) {
            const int e0 = (int)std::min<long long>(rs.estep, (long long)s0 + seg - 1);
            TrackParams qs = q;
            qs.sstep = s0;
            qs.estep = e0;
            qs.n = n_act;
            qs.ntiles = (n_act + kBlock - 1) / kBlock;
            qs.row0 = (s0 - 1) / kDiffInterval;
            qs.resumed = s0 > rs.sstep;
            qs.idx = cur;
            // frame index: the reference's start value plus the frames already taken
            if (qs.resumed) qs.ntp0 = q.ntp0 + (s0 - 1) / rs.einterval;
            if (!cuda_ok(launch(qs, std::min(grid, qs.ntiles)), "track launch")) return false;
            launches++;
            if (e0 >= rs.estep) break;
            const int nblk = (n_act + kCmpBlock - 1) / kCmpBlock;
            seg_count_kernel<<<nblk, kCmpBlock, 0, s>>>(cur, n_act, c_esc, c_sg, c_cnt, c_part);
            seg_scan_kernel<<<1, kCmpBlock, 0, s>>>(c_cnt, c_part, nblk, n_act, c_off, c_n, extra, d_rem,
                                                    nsdc, e0 / kDiffInterval + 1, rs.estep / kDiffInterval);
            seg_scatter_kernel<<<nblk, kCmpBlock, 0, s>>>(cur, n_act, c_esc, c_off, nxt);
            int h_n = 0;
            cudaMemcpyAsync(&h_n, c_n, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (!cuda_ok(cudaStreamSynchronize(s), "segment compaction")) return false;
            launches += 3;
            if (h_n < 0 || h_n > n_act) {
                set_error(1, "segment compaction: %d of %d particles", h_n, n_act);
                return false;
            }
            if (h_n == 0) break;  // every particle has left; its later rows are in `extra`
            n_act = h_n;
            cur = nxt;
            nxt = nxt == c_idx0 ? c_idx1 : c_idx0;
            s0 = e0 + 1;
        }
    }
    cudaEventRecord(ev1, s);
    if (!cuda_ok(fp64::launch_reduce_dpart(d_dpart, nslot, nsdc, d_dsum, s), "reduce")) return false;
    cudaEventRecord(eve, s);
    if (!cuda_ok(cudaStreamSynchronize(s), "track")) return false;
    float ms = 0.f, ms_step = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventElapsedTime(&ms_step, evb, eve);
    last_ms = ms;
    if (info) {
        info->estep = rs.estep;
        info->einterval = rs.einterval;
        info->nsdc = nsdc;
        info->nt_out = nt_out;
        info->nbins = nbins;
        info->grid = grid;
        info->blocks_per_sm = bps;
        info->kernel_ms = ms;
        info->step_ms = ms_step;
        info->launches = launches + (rs.reset_nsteps ? 2 : 1);
        info->pushes = (double)n * (rs.estep - rs.sstep + 1);
    }
    return true;
}

bool Session::fetch(particles* ptl, int* nsteps_ptl, double* espect, double* espect_escape,
                    double* dsum_out, int* remain)
{
    cudaStream_t s = g.stream;
    if (ptl && n > 0) {
        soa_to_aos((const double*)soa.ptr, n, cap, (double*)aos.ptr, s);
        cudaMemcpyAsync(ptl, aos.ptr, sizeof(particles) * n, cudaMemcpyDeviceToHost, s);
    }
    if (nsteps_ptl && n > 0)
        cudaMemcpyAsync(nsteps_ptl, nsteps.ptr, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    size_t nspec = (size_t)nt_out * nbins;
    std::vector<unsigned> hs;
    if ((espect || espect_escape) && nspec) {
        hs.resize(2 * nspec);
        cudaMemcpyAsync(hs.data(), spec.ptr, sizeof(unsigned) * 2 * nspec, cudaMemcpyDeviceToHost, s);
    }
    if (dsum_out && nsdc)
        cudaMemcpyAsync(dsum_out, dsum.ptr, sizeof(double) * 8 * nsdc, cudaMemcpyDeviceToHost, s);
    if (remain && nsdc)
        cudaMemcpyAsync(remain, rem.ptr, sizeof(int) * nsdc, cudaMemcpyDeviceToHost, s);
    if (!cuda_ok(cudaStreamSynchronize(s), "fetch")) return false;
    if (espect)
        for (size_t k = 0; k < nspec; k++) espect[k] = (double)hs[k];
    if (espect_escape)
        for (size_t k = 0; k < nspec; k++) espect_escape[k] = (double)hs[nspec + k];
    return true;
}

bool Session::set_traj(const int* ntraj_accum, const particles* ptl_time, int* points)
{
    if (n <= 0) return true;
    traj_total = ntraj_accum[n - 1];
    if (traj_total < 0) traj_total = 0;
    if (!traj.get(sizeof(particles) * (size_t)(traj_total > 0 ? traj_total : 1)) ||
        !trajacc.get(sizeof(int) * (size_t)n) || !trajpts.get(sizeof(int) * (size_t)n))
        return false;
    cudaStream_t s = g.stream;
    if (traj_total > 0 && ptl_time)
        cudaMemcpyAsync(traj.ptr, ptl_time, sizeof(particles) * traj_total, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(trajacc.ptr, ntraj_accum, sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (points) cudaMemcpyAsync(trajpts.ptr, points, sizeof(int) * n, cudaMemcpyHostToDevice, s);
    else fill_int((int*)trajpts.ptr, n, 1, s);
    return cuda_ok(cudaGetLastError(), "traj");
}

bool Session::get_traj(particles* ptl_time, int* points)
{
    cudaStream_t s = g.stream;
    if (ptl_time && traj_total > 0)
        cudaMemcpyAsync(ptl_time, traj.ptr, sizeof(particles) * traj_total, cudaMemcpyDeviceToHost, s);
    if (points && n > 0) cudaMemcpyAsync(points, trajpts.ptr, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    return cuda_ok(cudaStreamSynchronize(s), "traj fetch");
}

Session& cached_session()
{
    static Session* s = new Session();
    return *s;
}

// estep, einterval as particle_tracking_fixed_time_step derives them (src/tracking.c:103-109)
bool derive_steps(double dt, int nt_out, int& estep, int& einterval)
{
    if (!(dt > 0.0) || nt_out < 1) {
        set_error(6, "bad dt %g or nt_out %d", dt, nt_out);
        return false;
    }
    estep = (int)(simul_domain.tmax / dt);
    if (estep < 1) {
        set_error(6, "tmax %g / dt %g gives no steps", simul_domain.tmax, dt);
        return false;
    }
    einterval = estep / nt_out;
    if (einterval < 1) {
        set_error(6, "fewer steps (%d) than diagnostic frames (%d)", estep, nt_out);
        return false;
    }
    return true;
}

}  // namespace tp

using namespace tp;

struct tp_session {
    Session s;
};

extern "C" tp_session* tp_session_create(int nptl)
{
    tp_session* s = new tp_session();
    if (!s->s.reserve(nptl)) {
        delete s;
        return nullptr;
    }
    return s;
}

extern "C" void tp_session_destroy(tp_session* s) { delete s; }

extern "C" int tp_session_load(tp_session* s, const particles* ptl_init, const particles* ptl)
{
    return s && s->s.load(ptl_init, ptl, s->s.cap) ? 0 : -1;
}

extern "C" int tp_session_track(tp_session* s, int precision, double dt, int nt_out, int nbins,
                                tp_run_info* info)
{
    if (!s) return -1;
    RunSpec rs;
    if (!derive_steps(dt, nt_out, rs.estep, rs.einterval)) return -1;
    rs.precision = precision;
    rs.dt = dt;
    rs.nt_out = nt_out;
    rs.nbins = nbins;
    return s->s.run(rs, info) ? 0 : -1;
}

extern "C" int tp_session_fetch(tp_session* s, particles* ptl, int* nsteps_ptl, double* espect,
                                double* espect_escape, double* dsum, int* remain)
{
    return s && s->s.fetch(ptl, nsteps_ptl, espect, espect_escape, dsum, remain) ? 0 : -1;
}

extern "C" int tp_track_host(int precision, int nptl, double dt, int nt_out, int nbins,
                             const particles* ptl_init, particles* ptl, int* nsteps_ptl,
                             double* espect, double* espect_escape, double* dsum, int* remain,
                             tp_run_info* info)
{
    Session& s = cached_session();
    RunSpec rs;
    if (!derive_steps(dt, nt_out, rs.estep, rs.einterval)) return -1;
    rs.precision = precision;
    rs.dt = dt;
    rs.nt_out = nt_out;
    rs.nbins = nbins;
    if (!s.load(ptl_init, ptl, nptl)) return -1;
    if (!s.run(rs, info)) return -1;
    if (!s.fetch(ptl, nsteps_ptl, espect, espect_escape, dsum, remain)) return -1;
    if (remain)  // the kernel counts departures; the reference starts from nptl
        for (int k = 0; k < s.nsdc; k++) remain[k] += nptl;
    return 0;
}
