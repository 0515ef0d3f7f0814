// mixed_host.cu -- host set-up of the mixed-precision field description:
// fixed-point box geometry, FP32 node-interleaved grids, FP32 mode table.
#include <cmath>
#include <cstring>

#include "../../include/tp_gpu.h"
#include "tp_internal.h"
#include "tp_kernels_mixed.h"

namespace tp {

__global__ void interleave_v_kernel(const double* __restrict__ v, size_t n, float4* __restrict__ out)
{
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = make_float4((float)v[3 * i], (float)v[3 * i + 1], (float)v[3 * i + 2], 0.f);
}

static bool integral_multiple(double v, uint32_t& m)
{
    double r = std::nearbyint(v);
    if (r < 1.0 || r > 4294967295.0 || std::fabs(v - r) > 1e-9 * std::fabs(v)) return false;
    m = (uint32_t)r;
    return true;
}

// revolutions -> 32-bit fixed point, mod 2^32
static uint32_t rev_fixed(double rev)
{
    double fr = rev - std::floor(rev);
    return (uint32_t)(uint64_t)std::llround(fr * 4294967296.0);
}

bool build_mixfield(int stype, mixed::MixField& mf, int* nmodes_out)
{
    DevField f;
    if (!build_field(stype, f)) return false;
    memset(&mf, 0, sizeof(mf));
    mf.system_type = stype;
    mf.bc_flag = bc_flag;
    if (bc_flag != 0 && bc_flag != 1) {
        set_error(10, "the mixed-precision path supports periodic (0) and open (1) boundaries");
        return false;
    }
    if (multi_tframe != 0) {
        set_error(10, "the mixed-precision path supports single-frame fields only");
        return false;
    }
    mf.cm = (float)charge_mass;
    double mn[3] = {simul_domain.xmin, simul_domain.ymin, simul_domain.zmin};
    double mx[3] = {simul_domain.xmax, simul_domain.ymax, simul_domain.zmax};
    for (int k = 0; k < 3; k++) {
        mf.min[k] = mn[k];
        mf.L[k] = mx[k] - mn[k];
        if (!(mf.L[k] > 0.0)) {
            set_error(10, "empty domain along axis %d", k);
            return false;
        }
        mf.invL[k] = (float)(1.0 / mf.L[k]);
    }
    cudaStream_t s = g.stream;
    if (stype == TP_SYS_FORCEFREE) {
        mf.A = (float)g.ffA; mf.Bc = (float)g.ffB; mf.C = (float)g.ffC; mf.B0 = (float)param.B0;
        double lam = param.lambda0;
        mf.lam = (float)lam;
        mf.abc_fixed = 1;
        for (int k = 0; k < 3; k++) {
            if (!integral_multiple(lam * mf.L[k] / (2.0 * M_PI), mf.abc_m[k])) mf.abc_fixed = 0;
            mf.abc_off[k] = rev_fixed(lam * mn[k] / (2.0 * M_PI));
            mf.lmin[k] = (float)(lam * mn[k]);
            mf.lL[k] = (float)(lam * mf.L[k]);
        }
        if (f.vc_d) {
            mf.nx = simul_grid.nx; mf.ny = simul_grid.ny; mf.nz = simul_grid.nz;
            if (mf.nx < 2 || mf.ny < 2 || mf.nz < 2) {
                set_error(10, "gridded fields need at least 2 nodes per axis");
                return false;
            }
            mf.interp_ref = !g.interp_corrected;
            size_t n = (size_t)mf.nx * mf.ny * mf.nz;
            if (n >= 0xffffffffull) {
                set_error(10, "the mixed-precision path indexes grids of fewer than 2^32 - 1 nodes");
                return false;
            }
            float4* v4 = (float4*)g.s_mix_v.get(sizeof(float4) * n);
            if (!v4) return false;
            interleave_v_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f.vc_d, n, v4);
            if (!cuda_ok(cudaGetLastError(), "interleave v")) return false;
            mf.vgrid = v4;
        }
    } else if (stype == TP_SYS_PIC) {
        mf.nx = simul_grid.nx; mf.ny = simul_grid.ny; mf.nz = simul_grid.nz;
        if (mf.nx < 2 || mf.ny < 2 || mf.nz < 2) {
            set_error(10, "gridded fields need at least 2 nodes per axis");
            return false;
        }
        mf.interp_ref = !g.interp_corrected;
        double cells[3] = {mf.L[0] / simul_grid.dx, mf.L[1] / simul_grid.dy, mf.L[2] / simul_grid.dz};
        int nn[3] = {mf.nx, mf.ny, mf.nz};
        for (int k = 0; k < 3; k++)
            if (std::fabs(cells[k] - (nn[k] - 1)) > 1e-6 * nn[k]) {
                set_error(10, "mixed path needs grid spacing (max - min) / (n - 1) on every axis");
                return false;
            }
        size_t n = (size_t)mf.nx * mf.ny * mf.nz;
        if (n >= 0xffffffffull) {
            set_error(10, "the mixed-precision path indexes grids of fewer than 2^32 - 1 nodes");
            return false;
        }
        if (g.eb_src_e != f.ec_f || g.eb_src_b != f.bc_f || g.eb_n != n || g.eb_gen != g.upload_gen) {
            float4* eb = (float4*)g.s_mix_eb.get(sizeof(float4) * 2 * n);
            if (!eb) return false;
            if (!cuda_ok(mixed::launch_interleave(f.ec_f, f.bc_f, n, eb, s), "interleave eb")) return false;
            g.eb_src_e = f.ec_f;
            g.eb_src_b = f.bc_f;
            g.eb_n = n;
            g.eb_gen = g.upload_gen;
        }
        mf.eb = (const float4*)g.s_mix_eb.ptr;
    } else if (stype == TP_SYS_MODESUM) {
        int nm = (int)g.modes.size();
        int npair = (nm + 1) / 2;
        if (sizeof(mixed::ModePair) * (size_t)npair > 200 * 1024) {
            set_error(10, "at most %d plane-wave modes fit in shared memory",
                      (int)(200 * 1024 / sizeof(mixed::ModePair)) * 2);
            return false;
        }
        std::vector<mixed::ModePair> mfv(npair);
        memset(mfv.data(), 0, sizeof(mixed::ModePair) * npair);
        for (int m = 0; m < nm; m++) {
            const tp_mode& md = g.modes[m];
            mixed::ModePair& o = mfv[m / 2];
            const int h = m & 1;
            // round(phase / 2pi * 2^32) mod 2^32 is kept in the mode's pad word
            o.nph[h] = make_int4(md.n[0], md.n[1], md.n[2], md.pad);
            const float v[6] = {(float)md.amp_b[0], (float)md.amp_b[1], (float)md.amp_b[2],
                                (float)md.amp_e[0], (float)md.amp_e[1], (float)md.amp_e[2]};
            unsigned long long pk[3];  // (b0,b1) (b2,e0) (e1,e2), first of a pair in the low half
            for (int k = 0; k < 3; k++) {
                uint32_t lo, hi;
                memcpy(&lo, &v[2 * k], 4);
                memcpy(&hi, &v[2 * k + 1], 4);
                pk[k] = (unsigned long long)lo | ((unsigned long long)hi << 32);
            }
            if (h == 0) {
                o.amp[0].x = pk[0]; o.amp[0].y = pk[1]; o.amp[1].x = pk[2];
            } else {
                o.amp[1].y = pk[0]; o.amp[2].x = pk[1]; o.amp[2].y = pk[2];
            }
        }
        mixed::ModePair* d = (mixed::ModePair*)g.s_mix_modes.get(sizeof(mixed::ModePair) * (npair > 0 ? npair : 1));
        if (!d) return false;
        if (nm) cudaMemcpyAsync(d, mfv.data(), sizeof(mixed::ModePair) * npair, cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
        mf.nmodes = nm;
        mf.modes = d;
        mf.mB0 = (float)g.mode_B0;
    } else if (stype != TP_SYS_TEST) {
        set_error(10, "the mixed-precision path covers system types 0, 2, 4 and 5 (got %d)", stype);
        return false;
    }
    if (nmodes_out) *nmodes_out = mf.nmodes;
    return g.status == 0;
}

}  // namespace tp

using namespace tp;

// The mixed path's FP32 field at n points (xyz: n*3 doubles) as n*6 floats
// (Bx, By, Bz, Ex, Ey, Ez), for the current system type (0, 2, 4 or 5).
extern "C" int tp_get_emf_mixed_batch(int n, const double* xyz, float* emf6)
{
    mixed::MixField mf;
    if (!build_mixfield(system_type, mf, nullptr)) return -1;
    if (n <= 0) return 0;
    double* d_in = (double*)g.s_batch_a.get(sizeof(double) * 3 * (size_t)n);
    float* d_out = (float*)g.s_batch_b.get(sizeof(float) * 6 * (size_t)n);
    if (!d_in || !d_out) return -1;
    cudaMemcpyAsync(d_in, xyz, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, g.stream);
    if (!cuda_ok(mixed::launch_emf_batch(mf, n, d_in, d_out, g.stream), "emf mixed")) return -1;
    cudaMemcpyAsync(emf6, d_out, sizeof(float) * 6 * (size_t)n, cudaMemcpyDeviceToHost, g.stream);
    return cuda_ok(cudaStreamSynchronize(g.stream), "emf mixed sync") ? 0 : -1;
}
