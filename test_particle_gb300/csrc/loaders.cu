// loaders.cu -- PIC-style E and B read from the reference's binary field
// files straight into device memory.
//
// The reference reads bx_<ct>.gda, by_, bz_ and ex_, ey_, ez_ (nx*ny*nz FP32
// each, x fastest) into host arrays of {x,y,z} records scaled by B0 or E0
// (src/magnetic_field.c:442-534, src/electric_field.c:257-349, single time
// frame, float data).  Here each file streams through two pinned staging
// buffers to the device (reading the next piece while the previous one
// copies), and a kernel scatters the component into the same record layout
// with the same scaling, in device memory only: the tracking kernels, the
// mixed path's interleaved grid and the single-point functions then use the
// device copy, and the host arrays stay untouched (tp_fetch_device_fields
// copies them back when a caller needs them).
#include <cstdio>
#include <cstring>

#include "../../include/tp_gpu.h"
#include "tp_internal.h"

using namespace tp;

// scale globals of the reference's field modules (magnetic_field.c:38, electric_field.c:38)
extern "C" double B0, E0;

namespace {

constexpr size_t kPiece = (size_t)16 << 20;  // floats per staging piece (64 MB)

__global__ void scatter_kernel(const float* __restrict__ comp, size_t n, double scale, int k,
                               float* __restrict__ rec)
{
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) rec[3 * i + k] = (float)((double)comp[i] * scale);  // data[i] * B0, as the reference
}

struct Staging {
    float* host[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    ~Staging()
    {
        for (int b = 0; b < 2; b++) {
            if (host[b]) cudaFreeHost(host[b]);
            if (done[b]) cudaEventDestroy(done[b]);
        }
    }
};

// One component file into dcomp (n floats), double-buffered.
bool read_component(const char* fname, size_t n, float* dcomp, Staging& st, cudaStream_t s)
{
    FILE* fp = fopen(fname, "rb");
    if (!fp) {
        set_error(7, "Unable to open file %s", fname);
        return false;
    }
    size_t done = 0;
    int b = 0;
    bool ok = true;
    while (done < n && ok) {
        size_t m = n - done < kPiece ? n - done : kPiece;
        ok = cuda_ok(cudaEventSynchronize(st.done[b]), "staging");  // its previous copy has finished
        if (!ok) break;
        if (fread(st.host[b], sizeof(float), m, fp) != m) {
            set_error(7, "file %s holds fewer than %zu values", fname, n);
            ok = false;
            break;
        }
        ok = cuda_ok(cudaMemcpyAsync(dcomp + done, st.host[b], sizeof(float) * m, cudaMemcpyHostToDevice, s),
                     "field upload") &&
             cuda_ok(cudaEventRecord(st.done[b], s), "staging event");
        done += m;
        b ^= 1;
    }
    fclose(fp);
    return ok;
}

bool device_records(Mirror& m, size_t bytes)
{
    if (m.cap < bytes) {
        if (m.dev) cudaFree(m.dev);
        m.dev = nullptr;
        m.cap = 0;
        if (!cuda_ok(cudaMalloc(&m.dev, bytes), "field grid alloc")) return false;
        m.cap = bytes;
    }
    m.bytes = bytes;
    m.device_only = true;
    m.dirty = false;
    return true;
}

}  // namespace

// The current simul_grid's PIC-style fields (system type 4) from
// <filepath>{bx,by,bz,ex,ey,ez}_<ct>.gda, scaled by B0 and E0, into device
// memory (the reference's read_bfields_binary + read_efields_binary for one
// time frame of float data).  Returns 0, or -1 with tp_last_error set.
extern "C" int tp_read_pic_fields_binary(const char* filepath, int ct)
{
    if (!ensure_init()) return -1;
    if (multi_tframe != 0) {
        set_error(7, "tp_read_pic_fields_binary reads one time frame (multi_tframe 0)");
        return -1;
    }
    const size_t n = (size_t)simul_grid.nx * simul_grid.ny * simul_grid.nz;
    if (simul_grid.nx < 1 || simul_grid.ny < 1 || simul_grid.nz < 1 || !filepath) {
        set_error(7, "tp_read_pic_fields_binary: empty grid or no path");
        return -1;
    }
    cudaStream_t s = g.stream;
    Staging st;
    static Scratch comp;
    float* dcomp = (float*)comp.get(sizeof(float) * n);
    if (!dcomp) return -1;
    const size_t piece = n < kPiece ? n : kPiece;
    for (int b = 0; b < 2; b++)
        if (!cuda_ok(cudaMallocHost(&st.host[b], sizeof(float) * piece), "pinned staging") ||
            !cuda_ok(cudaEventCreateWithFlags(&st.done[b], cudaEventDisableTiming), "staging event") ||
            !cuda_ok(cudaEventRecord(st.done[b], s), "staging event"))
            return -1;
    if (!device_records(g.m_bc_f, sizeof(float) * 3 * n) || !device_records(g.m_ec_f, sizeof(float) * 3 * n))
        return -1;
    const char* names[6] = {"bx_", "by_", "bz_", "ex_", "ey_", "ez_"};
    for (int c = 0; c < 6; c++) {
        char fname[4096];
        snprintf(fname, sizeof(fname), "%s%s%d%s", filepath, names[c], ct, ".gda");
        if (!read_component(fname, n, dcomp, st, s)) {
            g.m_bc_f.release();
            g.m_ec_f.release();
            return -1;
        }
        float* rec = (float*)(c < 3 ? g.m_bc_f.dev : g.m_ec_f.dev);
        scatter_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dcomp, n, c < 3 ? B0 : E0, c % 3, rec);
        if (!cuda_ok(cudaGetLastError(), "field scatter")) return -1;
    }
    g.upload_gen++;
    return cuda_ok(cudaStreamSynchronize(s), "field read") ? 0 : -1;
}

// Copies the device-resident PIC-style fields (from tp_read_pic_fields_binary
// or tp_synth_pic_fields) to host arrays of nx*ny*nz {x,y,z} float records.
extern "C" int tp_fetch_device_fields(float* host_e, float* host_b)
{
    if (!ensure_init()) return -1;
    if (!g.m_bc_f.device_only || !g.m_ec_f.device_only || !g.m_bc_f.dev || !g.m_ec_f.dev) {
        set_error(7, "no device-resident PIC fields to fetch");
        return -1;
    }
    cudaStream_t s = g.stream;
    if (host_e) cudaMemcpyAsync(host_e, g.m_ec_f.dev, g.m_ec_f.bytes, cudaMemcpyDeviceToHost, s);
    if (host_b) cudaMemcpyAsync(host_b, g.m_bc_f.dev, g.m_bc_f.bytes, cudaMemcpyDeviceToHost, s);
    return cuda_ok(cudaStreamSynchronize(s), "fetch fields") ? 0 : -1;
}
