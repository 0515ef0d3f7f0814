// noalloc.cu -- tp_track_mixed_noalloc: the mixed-precision tracking kernel
// for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool or allocator (which owns every device allocation of
// the process), and embedded or real-time hosts that forbid allocation after
// start-up.  They own their particle and output buffers; this entry point
// adds nothing to them.  The kernel's scratch -- the per-block partial sums
// of the diffusion coefficients, the exact energy-bin edges and, when the
// caller passes no status word of its own, a status word -- lives in the
// file-scope device array below instead of in cudaMalloc'd memory.
//
// The array is kNoallocScratchBytes (4 MiB) on every GPU that loads the
// library and stays allocated until the process exits.  Every call shares
// it and it keeps the last call's contents; each call clears what must start
// at zero.  Calls on the same device that overlap on the GPU (other streams,
// other host threads) race on it: serialise them.  The bin edges travel to
// the device as kernel arguments, so no host buffer outlives a call.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/tp_gpu.h"
#include "tp_kernels.h"
#include "tp_kernels_mixed.h"

namespace tp {
namespace noalloc {

constexpr size_t kNoallocScratchBytes = 4u << 20;
constexpr size_t kScratchDoubles = kNoallocScratchBytes / sizeof(double);
constexpr int kMaxDevices = 64;
constexpr int kMaxBins = 4096;

// The scratch of the variant.  Host code must not pass this name to a kernel:
// on the host it names a stand-in, not the device address (see scratch_ptr).
static __device__ __align__(256) double tp_noalloc_scratch[kScratchDoubles];

// Device address of the array for the current device, looked up once per
// device with that device current (the first call on a device).  The lookup
// table is shared by host threads, hence the lock (a std::mutex allocates
// nothing).
static double* g_scratch_addr[kMaxDevices];
static bool g_scratch_ready[kMaxDevices];
static std::mutex g_scratch_lock;

static cudaError_t scratch_ptr(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_lock);
    if (!g_scratch_ready[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, tp_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<double*>(p);
        g_scratch_ready[dev] = true;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

__global__ void fill_kernel(int* p, int n, int v)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void add_kernel(int* p, int n, int v)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] += v;
}

// The bin edges reach the device by value, as the argument of a small
// kernel, a chunk of kEdgeChunk edges per launch: the launch copies its
// arguments, so the edges need neither a host staging buffer that must stay
// valid until the copy runs nor a device allocation.
constexpr int kEdgeChunk = 256;
struct EdgeChunk {
    double v[kEdgeChunk];
};

__global__ void put_edges_kernel(double* dst, EdgeChunk c, int n)
{
    int i = threadIdx.x;
    if (i < n) dst[i] = c.v[i];
}

// The reference's bin of an energy (src/diagnostics.c:193-203, x86 semantics
// for invalid conversions) and its exact edges by bisection on the bit
// pattern, written into thr[0 .. nbins-2].
static int ref_bin(double e, int nbins, double lmin, double lde)
{
    double v = floor((log10(e) - lmin) / lde);
    int ib = (!(v == v) || v < -2147483648.0 || v > 2147483647.0) ? INT_MIN : (int)v;
    if (ib < 0) ib = 0;
    else if (ib > nbins - 1) ib = nbins - 1;
    return ib;
}

static bool edges(int nbins, double emin, double emax, double* thr)
{
    double lmin = log10(emin), lde = (log10(emax) - lmin) / (nbins - 2);
    if (!(lde > 0.0) || !std::isfinite(lmin)) return false;
    unsigned long long top;
    double dmax = DBL_MAX;
    memcpy(&top, &dmax, sizeof(top));
    for (int b = 1; b < nbins; b++) {
        unsigned long long lo = 0, hi = top;
        double dh;
        memcpy(&dh, &hi, sizeof(dh));
        if (ref_bin(dh, nbins, lmin, lde) < b) return false;
        while (hi - lo > 1) {
            unsigned long long mid = lo + (hi - lo) / 2;
            double dm;
            memcpy(&dm, &mid, sizeof(dm));
            if (ref_bin(dm, nbins, lmin, lde) >= b) hi = mid;
            else lo = mid;
        }
        memcpy(&thr[b - 1], &hi, sizeof(double));
    }
    return true;
}

}  // namespace noalloc
}  // namespace tp

using namespace tp;

extern "C" int tp_track_mixed_noalloc(const tp_noalloc_args* a)
{
    using namespace noalloc;
    if (!a) return TP_NOALLOC_EINVAL;
    const int n = a->n;
    if (n < 1 || a->estep < 1 || a->nt_out < 1 || a->nbins < 3 || a->nbins > kMaxBins ||
        !(a->dt > 0.0) || (a->bc_flag != 0 && a->bc_flag != 1) || !a->d_state || !a->d_state0 ||
        !a->d_nsteps || !a->d_espect || !a->d_espect_escape || !a->d_dsum || !a->d_remain)
        return TP_NOALLOC_EINVAL;
    const int einterval = a->estep / a->nt_out;
    if (einterval < 1) return TP_NOALLOC_EINVAL;
    // the kernel indexes the spectra [nt_out][nbins] with 32-bit integers
    if ((long long)a->nt_out * a->nbins > INT_MAX) return TP_NOALLOC_EINVAL;
    if (a->system_type != TP_SYS_FORCEFREE && a->system_type != TP_SYS_PIC) return TP_NOALLOC_EINVAL;
    if (a->system_type == TP_SYS_PIC && (!a->d_grid || a->nx < 2 || a->ny < 2 || a->nz < 2 ||
                                         (unsigned long long)a->nx * a->ny * a->nz >= 0xffffffffull))
        return TP_NOALLOC_EINVAL;
    // alignment: a grid node is read with one 32-byte load, and every other
    // buffer is read and written as its element type
    auto misaligned = [](const void* p, uintptr_t al) { return ((uintptr_t)p & (al - 1)) != 0; };
    if ((a->system_type == TP_SYS_PIC && misaligned(a->d_grid, 32)) || misaligned(a->d_state, 8) ||
        misaligned(a->d_state0, 8) || misaligned(a->d_dsum, 8) || misaligned(a->d_nsteps, 4) ||
        misaligned(a->d_espect, 4) || misaligned(a->d_espect_escape, 4) || misaligned(a->d_remain, 4) ||
        misaligned(a->d_status, 4))
        return TP_NOALLOC_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(a->stream);

    // field description (host structure, no device memory of its own)
    mixed::MixField mf;
    memset(&mf, 0, sizeof(mf));
    mf.system_type = a->system_type;
    mf.bc_flag = a->bc_flag;
    mf.cm = (float)a->charge_mass;
    for (int k = 0; k < 3; k++) {
        mf.min[k] = a->lo[k];
        mf.L[k] = a->hi[k] - a->lo[k];
        if (!(mf.L[k] > 0.0)) return TP_NOALLOC_EINVAL;
        mf.invL[k] = (float)(1.0 / mf.L[k]);
    }
    if (a->system_type == TP_SYS_FORCEFREE) {
        mf.A = (float)a->abc[0]; mf.Bc = (float)a->abc[1]; mf.C = (float)a->abc[2];
        mf.B0 = (float)a->B0;
        mf.lam = (float)a->lambda0;
        mf.abc_fixed = 1;
        for (int k = 0; k < 3; k++) {
            double m = a->lambda0 * mf.L[k] / (2.0 * M_PI), r = nearbyint(m);
            if (r < 1.0 || r > 4294967295.0 || fabs(m - r) > 1e-9 * fabs(m)) mf.abc_fixed = 0;
            else mf.abc_m[k] = (uint32_t)r;
            double rev = a->lambda0 * a->lo[k] / (2.0 * M_PI);
            rev -= floor(rev);
            mf.abc_off[k] = (uint32_t)(uint64_t)llround(rev * 4294967296.0);
            mf.lmin[k] = (float)(a->lambda0 * a->lo[k]);
            mf.lL[k] = (float)(a->lambda0 * mf.L[k]);
        }
    } else {
        mf.nx = a->nx; mf.ny = a->ny; mf.nz = a->nz;
        mf.interp_ref = !a->interp_corrected;
        mf.eb = reinterpret_cast<const float4*>(a->d_grid);
    }

    // launch geometry, then the scratch layout: [edges | status | partial sums]
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
        return TP_NOALLOC_ECUDA;
    int bps = mixed::track_max_blocks_per_sm(a->system_type, 0);
    if (bps < 1) bps = 1;
    const int ntiles = (n + kBlock - 1) / kBlock;
    const int nsdc = a->estep / kDiffInterval + 1;
    const size_t thr_slots = ((size_t)(a->nbins - 1) + 31) / 32 * 32;
    const size_t head = thr_slots + 32;  // edges, then a 256-byte slot for a status word
    int grid = nsm * bps;
    if (grid > ntiles) grid = ntiles;
    while (grid > 1 && head + (size_t)grid * nsdc * 8 > kScratchDoubles) grid--;
    if (head + (size_t)grid * nsdc * 8 > kScratchDoubles) return TP_NOALLOC_ETOOBIG;

    double* scr = nullptr;
    if (scratch_ptr(&scr) != cudaSuccess) return TP_NOALLOC_ECUDA;
    double* d_thr = scr;
    // the kernel's status bits (TP_ST_*) go to the caller's word when it
    // passes one, else to a slot of the scratch that nobody reads
    int* d_status = a->d_status ? a->d_status : reinterpret_cast<int*>(scr + thr_slots);
    double* d_dpart = scr + head;

    double thr[kMaxBins];  // on the stack: edges for this call only
    if (!edges(a->nbins, a->emin, a->emax, thr)) return TP_NOALLOC_EINVAL;
    const size_t nspec = (size_t)a->nt_out * a->nbins;
    cudaError_t e = cudaSuccess;
    for (int c0 = 0; c0 < a->nbins - 1 && e == cudaSuccess; c0 += kEdgeChunk) {
        EdgeChunk ch;
        const int m = std::min(kEdgeChunk, a->nbins - 1 - c0);
        memcpy(ch.v, thr + c0, sizeof(double) * m);
        put_edges_kernel<<<1, kEdgeChunk, 0, s>>>(d_thr + c0, ch, m);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_dpart, 0, sizeof(double) * 8 * (size_t)nsdc * grid, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->d_espect, 0, sizeof(unsigned) * nspec, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->d_espect_escape, 0, sizeof(unsigned) * nspec, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->d_remain, 0, sizeof(int) * nsdc, s);
    if (e != cudaSuccess) return TP_NOALLOC_ECUDA;
    fill_kernel<<<(n + 255) / 256, 256, 0, s>>>(a->d_nsteps, n, 1);

    TrackBufs b;
    memset(&b, 0, sizeof(b));
    double* S = a->d_state;
    const double* S0 = a->d_state0;
    const long st = n;
    b.x = S; b.y = S + st; b.z = S + 2 * st; b.qm = S + 3 * st;
    b.ux = S + 4 * st; b.uy = S + 5 * st; b.uz = S + 6 * st; b.t = S + 7 * st;
    b.xs = S + 8 * st; b.ys = S + 9 * st; b.zs = S + 10 * st;
    b.x0 = S0; b.y0 = S0 + st; b.z0 = S0 + 2 * st;
    b.ux0 = S0 + 4 * st; b.uy0 = S0 + 5 * st; b.uz0 = S0 + 6 * st; b.t0 = S0 + 7 * st;
    b.nsteps_ptl = a->d_nsteps;
    b.ebin_thr = d_thr;
    b.espect = a->d_espect;
    b.espect_esc = a->d_espect_escape;
    b.remain = a->d_remain;
    b.dpart = d_dpart;
    b.status = d_status;
    TrackParams q;
    memset(&q, 0, sizeof(q));
    q.n = n;
    q.estep = a->estep;
    q.einterval = einterval;
    q.nt_out = a->nt_out;
    q.nbins = a->nbins;
    q.nsdc = nsdc;
    q.ntp0 = (int)floor(1.0 / (double)einterval);
    q.ntiles = ntiles;
    q.sstep = 1;
    q.dt = a->dt;
    if (mixed::launch_track(mf, b, q, grid, s) != cudaSuccess) return TP_NOALLOC_ECUDA;
    if (fp64::launch_reduce_dpart(d_dpart, grid, nsdc, a->d_dsum, s) != cudaSuccess)
        return TP_NOALLOC_ECUDA;
    // remain counts departures on the device; report particles remaining
    add_kernel<<<(nsdc + 255) / 256, 256, 0, s>>>(a->d_remain, nsdc, n);
    return cudaGetLastError() == cudaSuccess ? 0 : TP_NOALLOC_ECUDA;
}
