// capi.cu -- the C ABI of libtpgpu.so: the reference's tracking entry points
// and globals, device mirrors of the host field arrays, tracking sessions.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/tp_gpu.h"
#include "tp_kernels.h"
#include "tp_internal.h"

// ---------------------------------------------------------------- reference globals
extern "C" {
grids simul_grid;
domain simul_domain;
int system_type;
int multi_tframe;
int bc_flag;
int data_type;
double charge_mass;
param_ff param;
wlcs *config;
int nwlcs, iBessel;
double normI;
bfields_float *maga_float, *magb_float, *magc_float;
bfields_double *maga_double, *magb_double, *magc_double;
efields_float *efa_float, *efb_float, *efc_float;
efields_double *efa_double, *efb_double, *efc_double;
vfields_float *va_float, *vb_float, *vc_float;
vfields_double *va_double, *vb_double, *vc_double;
double B0, E0, v0;
// src/diagnostics.c:32 -- the caller's diagnostics.c normally defines these
__attribute__((weak)) double emin, emax, logemin, logemax, logde;
}

namespace tp {

Ctx g;

void set_error(int code, const char* fmt, ...)
{
    g.status = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g.err, sizeof(g.err), fmt, ap);
    va_end(ap);
}

bool cuda_ok(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return true;
    set_error(2, "%s: %s", what, cudaGetErrorString(e));
    return false;
}

// The reference reports errors with printf + exit(1); the reference-named
// entry points keep that contract.
void die_if_error(const char* where)
{
    if (g.status != 0) {
        printf("ERROR in %s: %s\n", where, g.err);
        fflush(stdout);
        exit(1);
    }
}

bool ensure_init()
{
    if (g.inited) return true;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error(3, "no CUDA device available: the GB300 tracking library has no CPU path");
        return false;
    }
    if (!cuda_ok(cudaSetDevice(g.device), "cudaSetDevice")) return false;
    if (!cuda_ok(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking), "stream")) return false;
    if (!cuda_ok(cudaMalloc(&g.d_status, sizeof(int)), "status")) return false;
    cudaMemsetAsync(g.d_status, 0, sizeof(int), g.stream);
    cudaDeviceGetAttribute(&g.num_sms, cudaDevAttrMultiProcessorCount, g.device);
    g.inited = true;
    return true;
}

// ---------------------------------------------------------------- device mirrors
bool Mirror::sync(const void* host, size_t b, cudaStream_t s)
{
    if (!host || b == 0) {
        src = nullptr;
        return true;
    }
    if (device_only) return true;
    if (host == src && b == bytes && !dirty) return true;
    if (b > cap) {
        if (dev) cudaFree(dev);
        dev = nullptr;
        cap = 0;
        if (!cuda_ok(cudaMalloc(&dev, b), "field mirror alloc")) return false;
        cap = b;
    }
    if (!cuda_ok(cudaMemcpyAsync(dev, host, b, cudaMemcpyHostToDevice, s), "field upload"))
        return false;
    src = host;
    bytes = b;
    dirty = false;
    g.upload_gen++;
    return true;
}

void Mirror::release()
{
    if (dev) cudaFree(dev);
    dev = nullptr;
    cap = bytes = 0;
    src = nullptr;
    dirty = true;
    device_only = false;
}

static size_t ncell() { return (size_t)simul_grid.nx * simul_grid.ny * simul_grid.nz; }

// Builds the device field description from the reference globals, uploading
// what the given system type reads.
bool build_field(int stype, DevField& f)
{
    if (!ensure_init()) return false;
    memset(&f, 0, sizeof(f));
    f.system_type = stype;
    f.multi_tframe = multi_tframe;
    f.interp_corrected = g.interp_corrected;
    f.ellint_corrected = g.ellint_corrected;
    f.bc_flag = bc_flag;
    f.nx = simul_grid.nx; f.ny = simul_grid.ny; f.nz = simul_grid.nz;
    f.gdx = simul_grid.dx; f.gdy = simul_grid.dy; f.gdz = simul_grid.dz; f.gdt = simul_grid.dt;
    f.charge_mass = charge_mass;
    f.xmin = simul_domain.xmin; f.xmax = simul_domain.xmax;
    f.ymin = simul_domain.ymin; f.ymax = simul_domain.ymax;
    f.zmin = simul_domain.zmin; f.zmax = simul_domain.zmax;
    f.ffA = g.ffA; f.ffB = g.ffB; f.ffC = g.ffC;
    f.B0 = param.B0;
    f.lambda0 = param.lambda0;
    cudaStream_t s = g.stream;
    size_t n3 = ncell() * 3;
    bool mt = multi_tframe != 0;
    auto dd = [&](Mirror& m, const void* h, size_t elem) -> const void* {
        if (!m.sync(h, h ? n3 * elem : 0, s)) return nullptr;
        return m.device_only ? m.dev : (h ? m.dev : nullptr);
    };
    if (stype == TP_SYS_FORCEFREE) {
        if (!mt) f.vc_d = (const double*)dd(g.m_vc_d, vc_double, sizeof(double));
        else {
            f.va_d = (const double*)dd(g.m_va_d, va_double, sizeof(double));
            f.vb_d = (const double*)dd(g.m_vb_d, vb_double, sizeof(double));
        }
    } else if (stype == TP_SYS_MHD || stype == TP_SYS_PIC) {
        if (!mt) {
            f.bc_f = (const float*)dd(g.m_bc_f, magc_float, sizeof(float));
            if (stype == TP_SYS_MHD) f.vc_f = (const float*)dd(g.m_vc_f, vc_float, sizeof(float));
            else f.ec_f = (const float*)dd(g.m_ec_f, efc_float, sizeof(float));
        } else {
            f.ba_f = (const float*)dd(g.m_ba_f, maga_float, sizeof(float));
            f.bb_f = (const float*)dd(g.m_bb_f, magb_float, sizeof(float));
            if (stype == TP_SYS_MHD) {
                f.va_f = (const float*)dd(g.m_va_f, va_float, sizeof(float));
                f.vb_f = (const float*)dd(g.m_vb_f, vb_float, sizeof(float));
            } else {
                f.ea_f = (const float*)dd(g.m_ea_f, efa_float, sizeof(float));
                f.eb_f = (const float*)dd(g.m_eb_f, efb_float, sizeof(float));
            }
        }
        bool have = mt ? (f.ba_f && f.bb_f && (stype == TP_SYS_MHD ? (f.va_f && f.vb_f) : (f.ea_f && f.eb_f)))
                       : (f.bc_f && (stype == TP_SYS_MHD ? f.vc_f != nullptr : f.ec_f != nullptr));
        if (!have) {
            if (g.status == 0) set_error(4, "system %d needs its gridded fields allocated and filled", stype);
            return false;
        }
    } else if (stype == TP_SYS_WLCS) {
        if (nwlcs > 0 && !config) {
            set_error(4, "wire-loop system without a configuration (read_wlcs not called)");
            return false;
        }
        g.m_cfg.dirty = true;  // tiny; always refreshed
        f.cfg = (const wlcs*)(nwlcs > 0 ? dd0(g.m_cfg, config, sizeof(wlcs) * nwlcs, s) : nullptr);
        f.nwlcs = nwlcs;
        f.iBessel = iBessel;
    } else if (stype == TP_SYS_MODESUM) {
        f.nmodes = (int)g.modes.size();
        f.modes = (const tp_mode*)(f.nmodes ? dd0(g.m_modes, g.modes.data(), sizeof(tp_mode) * f.nmodes, s) : nullptr);
        f.B0 = g.mode_B0;
    } else if (stype != TP_SYS_TEST) {
        set_error(5, "wrong system type %d", stype);
        return false;
    }
    return g.status == 0;
}

const void* dd0(Mirror& m, const void* h, size_t b, cudaStream_t s)
{
    if (!m.sync(h, b, s)) return nullptr;
    return m.dev;
}

// Device field with every grid the *_at_point functions may read.
bool build_field_points(DevField& f)
{
    if (!build_field(TP_SYS_TEST, f)) return false;
    cudaStream_t s = g.stream;
    size_t n3 = ncell() * 3;
    auto dd = [&](Mirror& m, const void* h, size_t elem) -> const void* {
        if (!h) return m.device_only ? m.dev : nullptr;
        return dd0(m, h, n3 * elem, s);
    };
    f.bc_f = (const float*)dd(g.m_bc_f, magc_float, 4); f.ba_f = (const float*)dd(g.m_ba_f, maga_float, 4);
    f.bb_f = (const float*)dd(g.m_bb_f, magb_float, 4); f.ec_f = (const float*)dd(g.m_ec_f, efc_float, 4);
    f.ea_f = (const float*)dd(g.m_ea_f, efa_float, 4); f.eb_f = (const float*)dd(g.m_eb_f, efb_float, 4);
    f.vc_f = (const float*)dd(g.m_vc_f, vc_float, 4); f.va_f = (const float*)dd(g.m_va_f, va_float, 4);
    f.vb_f = (const float*)dd(g.m_vb_f, vb_float, 4);
    f.bc_d = (const double*)dd(g.m_bc_d, magc_double, 8); f.ba_d = (const double*)dd(g.m_ba_d, maga_double, 8);
    f.bb_d = (const double*)dd(g.m_bb_d, magb_double, 8); f.ec_d = (const double*)dd(g.m_ec_d, efc_double, 8);
    f.ea_d = (const double*)dd(g.m_ea_d, efa_double, 8); f.eb_d = (const double*)dd(g.m_eb_d, efb_double, 8);
    f.vc_d = (const double*)dd(g.m_vc_d, vc_double, 8); f.va_d = (const double*)dd(g.m_va_d, va_double, 8);
    f.vb_d = (const double*)dd(g.m_vb_d, vb_double, 8);
    return g.status == 0;
}

// ---------------------------------------------------------------- spectrum thresholds
// The reference's bin of an energy (src/diagnostics.c:193-203), with x86
// semantics for an invalid float-to-int conversion (NaN, +-inf -> INT_MIN).
static int ref_bin(double e, int nbins, double lmin, double lde)
{
    double v = floor((log10(e) - lmin) / lde);
    int ib;
    if (!(v == v) || v < -2147483648.0 || v > 2147483647.0) ib = INT_MIN;
    else ib = (int)v;
    if (ib < 0) ib = 0;
    else if (ib > nbins - 1) ib = nbins - 1;
    return ib;
}

static double bits_to_d(unsigned long long u)
{
    double d;
    memcpy(&d, &u, sizeof(d));
    return d;
}

static unsigned long long d_to_bits(double d)
{
    unsigned long long u;
    memcpy(&u, &d, sizeof(u));
    return u;
}

// Exact bin edges: thr[b-1] = smallest double e with ref_bin(e) >= b.
bool compute_thresholds(int nbins, double lmin, double lde, std::vector<double>& thr)
{
    if (nbins < 3) {
        set_error(6, "nbins must be at least 3 (got %d)", nbins);
        return false;
    }
    if (!(lde > 0.0) || !std::isfinite(lmin)) {
        set_error(6, "bad spectrum range: logemin %g, logde %g", lmin, lde);
        return false;
    }
    thr.assign(nbins - 1, 0.0);
    const unsigned long long top = d_to_bits(DBL_MAX);
    for (int b = 1; b < nbins; b++) {
        unsigned long long lo = 0, hi = top;  // ref_bin(+0) = 0 < b, ref_bin(max) = nbins-1 >= b
        if (ref_bin(bits_to_d(hi), nbins, lmin, lde) < b) {
            set_error(6, "spectrum bins not reachable");
            return false;
        }
        while (hi - lo > 1) {
            unsigned long long mid = lo + (hi - lo) / 2;
            if (ref_bin(bits_to_d(mid), nbins, lmin, lde) >= b) hi = mid;
            else lo = mid;
        }
        thr[b - 1] = bits_to_d(hi);
    }
    return true;
}

bool ensure_thresholds(int nbins)
{
    if (g.thr_nbins == nbins && g.thr_logemin == logemin && g.thr_logde == logde && g.d_thr)
        return true;
    std::vector<double> thr;
    if (!compute_thresholds(nbins, logemin, logde, thr)) return false;
    if (g.d_thr) cudaFree(g.d_thr);
    g.d_thr = nullptr;
    if (!cuda_ok(cudaMalloc(&g.d_thr, sizeof(double) * (nbins - 1)), "thresholds")) return false;
    if (!cuda_ok(cudaMemcpyAsync(g.d_thr, thr.data(), sizeof(double) * (nbins - 1),
                                 cudaMemcpyHostToDevice, g.stream), "thresholds")) return false;
    cudaStreamSynchronize(g.stream);
    g.thr_nbins = nbins;
    g.thr_logemin = logemin;
    g.thr_logde = logde;
    return true;
}

// ---------------------------------------------------------------- scratch buffers
void* Scratch::get(size_t b)
{
    if (b <= cap) return ptr;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    if (cudaMalloc(&ptr, b) != cudaSuccess) {
        set_error(7, "device allocation of %zu bytes failed", b);
        return nullptr;
    }
    cap = b;
    return ptr;
}

void Scratch::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

// ---------------------------------------------------------------- AoS <-> SoA
__global__ void aos_to_soa_kernel(const double* __restrict__ aos, int n, double* __restrict__ soa,
                                  long stride)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* r = aos + (size_t)11 * i;
#pragma unroll
    for (int k = 0; k < 11; k++) soa[k * stride + i] = r[k];
}

__global__ void soa_to_aos_kernel(const double* __restrict__ soa, int n, long stride,
                                  double* __restrict__ aos)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* r = aos + (size_t)11 * i;
#pragma unroll
    for (int k = 0; k < 11; k++) r[k] = soa[k * stride + i];
}

void aos_to_soa(const double* d_aos, int n, double* d_soa, long stride, cudaStream_t s)
{
    if (n > 0) aos_to_soa_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_aos, n, d_soa, stride);
}

void soa_to_aos(const double* d_soa, int n, long stride, double* d_aos, cudaStream_t s)
{
    if (n > 0) soa_to_aos_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_soa, n, stride, d_aos);
}

}  // namespace tp

using namespace tp;

// ---------------------------------------------------------------- library API
extern "C" int tp_init(int device)
{
    if (g.inited && device == g.device) return 0;
    if (g.inited) {
        set_error(1, "tp_init: device already selected (%d)", g.device);
        return -1;
    }
    g.device = device;
    return ensure_init() ? 0 : -1;
}

extern "C" int tp_last_status(void) { return g.status; }
extern "C" const char* tp_last_error(void) { return g.err; }
extern "C" void tp_clear_status(void)
{
    g.status = 0;
    g.err[0] = 0;
}

// Status bits raised by kernels since the last call (read and cleared).
extern "C" int tp_device_status(void)
{
    if (!ensure_init()) return -1;
    int h = 0;
    cudaMemcpyAsync(&h, g.d_status, sizeof(int), cudaMemcpyDeviceToHost, g.stream);
    cudaMemsetAsync(g.d_status, 0, sizeof(int), g.stream);
    cudaStreamSynchronize(g.stream);
    return h;
}

extern "C" void tp_set_abc(double A, double B, double C)
{
    g.ffA = A;
    g.ffB = B;
    g.ffC = C;
}

extern "C" void tp_set_interp_corrected(int on) { g.interp_corrected = on ? 1 : 0; }
extern "C" void tp_set_ellint_corrected(int on) { g.ellint_corrected = on ? 1 : 0; }
extern "C" void tp_set_compaction(int steps) { g.compact_steps = steps < 0 ? -1 : steps; }

extern "C" int tp_set_modes(int nmodes, const tp_mode* modes, double Bz0)
{
    if (nmodes < 0 || (nmodes > 0 && !modes)) {
        set_error(1, "tp_set_modes: bad arguments");
        return -1;
    }
    g.modes.assign(modes, modes + nmodes);
    // 32-bit fixed-point phase offset, round(phase / 2pi * 2^32) mod 2^32
    for (auto& m : g.modes)
        m.pad = (int)(unsigned int)(long long)llround(m.phase / (2.0 * M_PI) * 4294967296.0);
    g.mode_B0 = Bz0;
    g.m_modes.dirty = true;
    g.modes_gen++;
    return 0;
}

extern "C" void tp_set_spectrum(int nbins, double e_min, double e_max)
{
    emin = e_min;
    emax = e_max;
    logemin = log10(emin);
    logemax = log10(emax);
    logde = (logemax - logemin) / (nbins - 2);
}

// The host arrays are authoritative again: device-only copies (synthesised
// fields) are dropped and everything is re-uploaded at the next use.
extern "C" void tp_mark_fields_dirty(void)
{
    for (Mirror* m : g.all_mirrors()) {
        if (m->device_only) m->release();
        m->dirty = true;
    }
}

extern "C" int tp_energy_thresholds(int nbins, double* thr)
{
    std::vector<double> t;
    if (!compute_thresholds(nbins, logemin, logde, t)) return -1;
    memcpy(thr, t.data(), sizeof(double) * t.size());
    return 0;
}

// Upload n AoS records, run fn(device AoS), download them back.
template <class F>
static int with_device_records(int n, particles* host, bool copy_back, F fn)
{
    if (!ensure_init()) return -1;
    if (n <= 0) return 0;
    double* d = (double*)g.s_batch_a.get(sizeof(particles) * (size_t)n);
    if (!d) return -1;
    if (!cuda_ok(cudaMemcpyAsync(d, host, sizeof(particles) * n, cudaMemcpyHostToDevice, g.stream),
                 "upload")) return -1;
    if (!fn(d)) return -1;
    if (copy_back &&
        !cuda_ok(cudaMemcpyAsync(host, d, sizeof(particles) * n, cudaMemcpyDeviceToHost, g.stream),
                 "download")) return -1;
    return cuda_ok(cudaStreamSynchronize(g.stream), "sync") ? 0 : -1;
}

extern "C" int tp_get_emf_batch(int n, const double* xyzt, double* emf6)
{
    DevField f;
    if (!build_field(system_type, f)) return -1;
    if (n <= 0) return 0;
    double* d_in = (double*)g.s_batch_a.get(sizeof(double) * 4 * (size_t)n);
    double* d_out = (double*)g.s_batch_b.get(sizeof(double) * 6 * (size_t)n);
    if (!d_in || !d_out) return -1;
    cudaMemcpyAsync(d_in, xyzt, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, g.stream);
    if (!cuda_ok(fp64::launch_emf_batch(f, n, d_in, d_out, g.d_status, g.stream), "emf")) return -1;
    cudaMemcpyAsync(emf6, d_out, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, g.stream);
    return cuda_ok(cudaStreamSynchronize(g.stream), "emf sync") ? 0 : -1;
}

extern "C" int tp_wirz_steps(int n, particles* ptl, double dt, int nsteps, int* iescape)
{
    DevField f;
    if (!build_field(system_type, f)) return -1;
    int* d_esc = (int*)g.s_batch_b.get(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!d_esc) return -1;
    if (n > 0) cudaMemcpyAsync(d_esc, iescape, sizeof(int) * n, cudaMemcpyHostToDevice, g.stream);
    int rc = with_device_records(n, ptl, true, [&](double* d) {
        return cuda_ok(fp64::launch_wirz_steps(f, n, d, nsteps, dt, d_esc, g.d_status, g.stream), "wirz");
    });
    if (rc == 0 && n > 0) {
        cudaMemcpyAsync(iescape, d_esc, sizeof(int) * n, cudaMemcpyDeviceToHost, g.stream);
        cudaStreamSynchronize(g.stream);
    }
    return rc;
}

extern "C" int tp_energy_bins(int n, const particles* ptl, int nbins, int* bins)
{
    if (!ensure_init() || !ensure_thresholds(nbins)) return -1;
    if (n <= 0) return 0;
    int* d_bins = (int*)g.s_batch_b.get(sizeof(int) * (size_t)n);
    if (!d_bins) return -1;
    int rc = with_device_records(n, (particles*)ptl, false, [&](double* d) {
        return cuda_ok(fp64::launch_ebins(g.d_thr, nbins, n, d, d_bins, g.stream), "ebins");
    });
    if (rc == 0) {
        cudaMemcpyAsync(bins, d_bins, sizeof(int) * n, cudaMemcpyDeviceToHost, g.stream);
        cudaStreamSynchronize(g.stream);
    }
    return rc;
}

extern "C" int tp_calc_diff_coeff_batch(int n, const particles* ptl_init, const particles* ptl,
                                        double dt, double* out8)
{
    DevField f;
    if (!build_field(system_type, f)) return -1;
    if (n <= 0) return 0;
    double* d0 = (double*)g.s_batch_a.get(sizeof(particles) * (size_t)n * 2);
    double* d_out = (double*)g.s_batch_b.get(sizeof(double) * 8 * (size_t)n);
    if (!d0 || !d_out) return -1;
    double* d1 = d0 + (size_t)11 * n;
    cudaMemcpyAsync(d0, ptl_init, sizeof(particles) * n, cudaMemcpyHostToDevice, g.stream);
    cudaMemcpyAsync(d1, ptl, sizeof(particles) * n, cudaMemcpyHostToDevice, g.stream);
    if (!cuda_ok(fp64::launch_diffc(f, n, d0, d1, dt, d_out, g.d_status, g.stream), "diffc")) return -1;
    cudaMemcpyAsync(out8, d_out, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, g.stream);
    return cuda_ok(cudaStreamSynchronize(g.stream), "diffc sync") ? 0 : -1;
}

extern "C" int tp_trilinear_batch(int n, const double* xyzt, long* corners8, double* weights8)
{
    DevField f;
    if (!build_field(TP_SYS_TEST, f)) return -1;
    if (n <= 0) return 0;
    double* d_in = (double*)g.s_batch_a.get(sizeof(double) * 4 * (size_t)n);
    char* d_out = (char*)g.s_batch_b.get((sizeof(long) + sizeof(double)) * 8 * (size_t)n);
    if (!d_in || !d_out) return -1;
    long* d_c = (long*)d_out;
    double* d_w = (double*)(d_out + sizeof(long) * 8 * (size_t)n);
    cudaMemcpyAsync(d_in, xyzt, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, g.stream);
    if (!cuda_ok(fp64::launch_trilinear(f, n, d_in, d_c, d_w, g.stream), "trilinear")) return -1;
    cudaMemcpyAsync(corners8, d_c, sizeof(long) * 8 * n, cudaMemcpyDeviceToHost, g.stream);
    cudaMemcpyAsync(weights8, d_w, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, g.stream);
    return cuda_ok(cudaStreamSynchronize(g.stream), "trilinear sync") ? 0 : -1;
}

// free_{b,e,v}field: drop the device mirrors of the released host arrays
extern "C" void tp_internal_fields_released(int which)
{
    if (which == 0) {
        for (Mirror* m : {&g.m_bc_f, &g.m_ba_f, &g.m_bb_f, &g.m_bc_d, &g.m_ba_d, &g.m_bb_d}) m->release();
    } else if (which == 1) {
        for (Mirror* m : {&g.m_ec_f, &g.m_ea_f, &g.m_eb_f, &g.m_ec_d, &g.m_ea_d, &g.m_eb_d}) m->release();
    } else {
        for (Mirror* m : {&g.m_vc_f, &g.m_va_f, &g.m_vb_f, &g.m_vc_d, &g.m_va_d, &g.m_vb_d}) m->release();
    }
}
