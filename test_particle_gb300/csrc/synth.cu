// synth.cu -- synthetic gridded fields on the device: B = B0 z + sum of
// plane-wave modes, v = sum of plane-wave modes, E = -v x B at every node,
// written as the reference's AoS float E and B arrays (x fastest,
// src/magnetic_field.c:31-35) that become the device copies of the field.
//
// Node (i, j, k) sits at xmin + i dx; a mode n has phase
// 2 pi (n_x i / nx + n_y j / ny + n_z k / nz) + phase, so the grid is
// periodic in node index with period (nx, ny, nz), the periodicity the
// reference's interpolation assumes past the last node
// (src/interpolation.c:61-90).  Phases are exact in 64-bit fixed point.
#include <cstdint>

#include "../../include/tp_gpu.h"
#include "tp_internal.h"

namespace tp {

struct SynthMode {
    int n[3];
    uint32_t pad;
    uint64_t ph;
    double amp[3];
};

__device__ __forceinline__ void synth_sum(const SynthMode* m, int nm, uint64_t ui, uint64_t uj,
                                          uint64_t uk, double out[3])
{
    out[0] = out[1] = out[2] = 0.0;
    for (int q = 0; q < nm; q++) {
        uint64_t ph = (uint64_t)(int64_t)m[q].n[0] * ui + (uint64_t)(int64_t)m[q].n[1] * uj +
                      (uint64_t)(int64_t)m[q].n[2] * uk + m[q].ph;
        double c = cos((double)(int64_t)ph * 3.4061215800865545e-19);  // 2 pi / 2^64
        out[0] += m[q].amp[0] * c;
        out[1] += m[q].amp[1] * c;
        out[2] += m[q].amp[2] * c;
    }
}

__global__ void synth_kernel(const SynthMode* mb, int nb, const SynthMode* mv, int nv, double B0z,
                             int nx, int ny, int nz, float* e, float* b)
{
    size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t n = (size_t)nx * ny * nz;
    if (idx >= n) return;
    int i = (int)(idx % nx);
    int j = (int)((idx / nx) % ny);
    int k = (int)(idx / ((size_t)nx * ny));
    // i / nx as 64-bit fixed point: floor(i * 2^64 / nx)
    uint64_t ui = (uint64_t)(((unsigned __int128)i << 64) / (unsigned)nx);
    uint64_t uj = (uint64_t)(((unsigned __int128)j << 64) / (unsigned)ny);
    uint64_t uk = (uint64_t)(((unsigned __int128)k << 64) / (unsigned)nz);
    double B[3], V[3];
    synth_sum(mb, nb, ui, uj, uk, B);
    synth_sum(mv, nv, ui, uj, uk, V);
    B[2] += B0z;
    b[3 * idx] = (float)B[0];
    b[3 * idx + 1] = (float)B[1];
    b[3 * idx + 2] = (float)B[2];
    e[3 * idx] = (float)(-(V[1] * B[2] - V[2] * B[1]));
    e[3 * idx + 1] = (float)(-(V[2] * B[0] - V[0] * B[2]));
    e[3 * idx + 2] = (float)(-(V[0] * B[1] - V[1] * B[0]));
}

static bool upload_modes(const tp_mode* m, int n, Scratch& sc, SynthMode*& d)
{
    std::vector<SynthMode> h(n > 0 ? n : 1);
    for (int q = 0; q < n; q++) {
        for (int k = 0; k < 3; k++) {
            h[q].n[k] = m[q].n[k];
            h[q].amp[k] = m[q].amp_b[k];
        }
        h[q].pad = 0;
        double rev = m[q].phase / (2.0 * M_PI);
        rev -= floor(rev);
        h[q].ph = (uint64_t)(uint32_t)llround(rev * 4294967296.0) << 32;
    }
    d = (SynthMode*)sc.get(sizeof(SynthMode) * h.size());
    if (!d) return false;
    return cuda_ok(cudaMemcpyAsync(d, h.data(), sizeof(SynthMode) * h.size(), cudaMemcpyHostToDevice,
                                   g.stream), "synth modes");
}

}  // namespace tp

using namespace tp;

// Fills the device copies of the PIC grids (system 4) from mode tables; the
// device copy becomes authoritative (no upload from the host arrays).  When
// host_e / host_b are given, the float AoS arrays are also copied there.
extern "C" int tp_synth_pic_fields(int nmodes_b, const tp_mode* modes_b, int nmodes_v,
                                   const tp_mode* modes_v, double B0z, float* host_e, float* host_b)
{
    if (!ensure_init()) return -1;
    int nx = simul_grid.nx, ny = simul_grid.ny, nz = simul_grid.nz;
    size_t n = (size_t)nx * ny * nz;
    if (n == 0) {
        set_error(1, "tp_synth_pic_fields: empty grid");
        return -1;
    }
    static Scratch sb, sv;
    SynthMode *db = nullptr, *dv = nullptr;
    if (!upload_modes(modes_b, nmodes_b, sb, db) || !upload_modes(modes_v, nmodes_v, sv, dv)) return -1;
    size_t bytes = sizeof(float) * 3 * n;
    for (Mirror* m : {&g.m_ec_f, &g.m_bc_f}) {
        if (m->cap < bytes) {
            if (m->dev) cudaFree(m->dev);
            m->dev = nullptr;
            m->cap = 0;
            if (!cuda_ok(cudaMalloc(&m->dev, bytes), "synth grid alloc")) return -1;
            m->cap = bytes;
        }
        m->bytes = bytes;
        m->device_only = true;
        m->dirty = false;
    }
    synth_kernel<<<(unsigned)((n + 255) / 256), 256, 0, g.stream>>>(
        db, nmodes_b, dv, nmodes_v, B0z, nx, ny, nz, (float*)g.m_ec_f.dev, (float*)g.m_bc_f.dev);
    if (!cuda_ok(cudaGetLastError(), "synth launch")) return -1;
    g.upload_gen++;
    if (host_e) cudaMemcpyAsync(host_e, g.m_ec_f.dev, bytes, cudaMemcpyDeviceToHost, g.stream);
    if (host_b) cudaMemcpyAsync(host_b, g.m_bc_f.dev, bytes, cudaMemcpyDeviceToHost, g.stream);
    return cuda_ok(cudaStreamSynchronize(g.stream), "synth") ? 0 : -1;
}

// Returns the PIC grid copies to host-array mode (uploads from magc_float / efc_float).
extern "C" void tp_release_device_fields(void)
{
    for (Mirror* m : g.all_mirrors()) m->release();
}
