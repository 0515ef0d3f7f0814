// loaders.cu -- PIC-style E and B read from the reference's binary and HDF5
// field files straight into device memory.
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
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>

#include "../../include/tp_gpu.h"
#include "../../include/tp_h5.h"
#include "h5lite.h"
#include "tp_internal.h"

using namespace tp;

// scale globals of the reference's field modules (magnetic_field.c:38, electric_field.c:38)
extern "C" double B0, E0;

namespace {

constexpr size_t kPiece = (size_t)16 << 20;  // floats per staging piece (64 MB)

// The three components of a field (comp + k * n) into its {x,y,z} records,
// scaled: data[i] * B0 into float, as the reference.  Each thread writes a
// whole 12-byte record, so a warp writes 384 contiguous bytes.
// With a power-of-two scale the product is exact in double, so one FP32
// multiply rounds it to the same float without the FP64 pipe (a small
// fraction of the FP32 rate on this part); other scales take the reference's
// double product.
template <bool POW2>
__device__ __forceinline__ float scaled(float v, double scale)
{
    return POW2 ? v * (float)scale : (float)((double)v * scale);
}

// A power of two (1 included) whose products and reciprocal stay normal.
inline bool pow2_scale(double scale)
{
    int ex = 0;
    return scale != 0.0 && std::fabs(std::frexp(scale, &ex)) == 0.5 && ex > -100 && ex < 100;
}

template <bool POW2>
__global__ void scatter3_kernel(const float* __restrict__ comp, size_t n, double scale, float* __restrict__ rec)
{
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) {
#pragma unroll
        for (int k = 0; k < 3; k++) rec[3 * i + k] = scaled<POW2>(comp[k * n + i], scale);
    }
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

// One component file into dcomp (n floats), double-buffered; each piece is
// read on several threads (one thread copies from the page cache at a few
// GB/s).
bool read_component(const char* fname, size_t n, float* dcomp, Staging& st, cudaStream_t s)
{
    const int fd = open(fname, O_RDONLY);
    if (fd < 0) {
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
        if (!tph5::read_at(fd, st.host[b], sizeof(float) * m, sizeof(float) * (uint64_t)done)) {
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
    close(fd);
    return ok;
}

// One raw HDF5 value (es bytes, big-endian or not) as the float the
// reference's H5Dread with a float memory type gives: doubles rounded to
// nearest, as a C cast.
__device__ __forceinline__ float h5_value(const unsigned char* __restrict__ p, int es, bool be)
{
    if (es == 4) {
        unsigned int w = *(const unsigned int*)p;
        if (be) w = __byte_perm(w, 0, 0x0123);
        return __uint_as_float(w);
    }
    unsigned long long w = *(const unsigned long long*)p;
    if (be) {
        const unsigned int lo = (unsigned int)w, hi = (unsigned int)(w >> 32);
        w = ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123);
    }
    return (float)__longlong_as_double((long long)w);
}

// The raw components of one field in device memory: component k's
// [nx][ny][nz] values (es[k] bytes each, big-endian when be[k]) at raw[k].
struct Raw3 {
    const unsigned char* raw[3];
    int es[3];
    int be[3];
};

// The reference's C-to-Fortran reorder (src/magnetic_field.c:656-665) of the
// three components of a field at once: the value at [i][j][k] of each file
// array goes to record (k * ny + j) * nx + i, scaled.  32 x 32 tiles of
// (i, k) at one j through shared memory: the reads along k are coalesced and
// each thread writes a whole 12-byte record, so a warp writes 384 contiguous
// bytes (no partial sectors).  Block (32, 8); grid (ceil(nz / 32),
// ceil(nx / 32), ny).
template <bool POW2, bool F32LE>  // F32LE: every component little-endian float (the usual file)
__global__ void __launch_bounds__(256) h5_transpose3_kernel(Raw3 in, int nx, int ny, int nz, double scale,
                                                           float* __restrict__ rec)
{
    __shared__ float tile[3][32][33];
    const int k0 = blockIdx.x * 32, i0 = blockIdx.y * 32, j = blockIdx.z;
#pragma unroll
    for (int c = 0; c < 3; c++)
        for (int r = threadIdx.y; r < 32; r += 8) {
            const int i = i0 + r, kk = k0 + threadIdx.x;
            if (i < nx && kk < nz) {
                const size_t q = ((size_t)i * ny + j) * nz + kk;
                tile[c][r][threadIdx.x] = F32LE ? reinterpret_cast<const float*>(in.raw[c])[q]
                                                : h5_value(in.raw[c] + q * in.es[c], in.es[c], in.be[c] != 0);
            }
        }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int kk = k0 + r, i = i0 + threadIdx.x;
        if (i < nx && kk < nz) {
            float* o = rec + 3 * (((size_t)kk * ny + j) * nx + i);
#pragma unroll
            for (int c = 0; c < 3; c++) o[c] = scaled<POW2>(tile[c][threadIdx.x][r], scale);
        }
    }
}

// The inverse, for writing a PIC field file: each record (k * ny + j) * nx + i
// of a field to [i][j][k] of three C-order [nx][ny][nz] float arrays
// (out + c * n), divided by the scale (in double, rounded to float; for a
// power-of-two scale as an FP32 product with its exact reciprocal, the same
// value without the FP64 pipe).  Whole records read (384 contiguous bytes a
// warp), tiles of (i, k) at one j; block (32, 8), grid (ceil(nx / 32),
// ceil(nz / 32), ny).
template <bool POW2>
__global__ void __launch_bounds__(256) h5_untranspose3_kernel(const float* __restrict__ rec, int nx, int ny, int nz,
                                                             double scale, float* __restrict__ out)
{
    const float inv = (float)(1.0 / scale);
    const size_t n = (size_t)nx * ny * nz;
    __shared__ float tile[3][32][33];
    const int i0 = blockIdx.x * 32, kb = blockIdx.y * 32, j = blockIdx.z;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int kk = kb + r, i = i0 + threadIdx.x;
        if (i < nx && kk < nz) {
            const float* q = rec + 3 * (((size_t)kk * ny + j) * nx + i);
#pragma unroll
            for (int c = 0; c < 3; c++) tile[c][r][threadIdx.x] = q[c];
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 3; c++)
        for (int r = threadIdx.y; r < 32; r += 8) {
            const int i = i0 + r, kk = kb + threadIdx.x;
            if (i < nx && kk < nz) {
                const float v = tile[c][threadIdx.x][r];
                out[c * n + ((size_t)i * ny + j) * nz + kk] = POW2 ? v * inv : (float)((double)v / scale);
            }
        }
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
    float* dcomp = (float*)comp.get(sizeof(float) * 3 * n);
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
        // the component waits in its slot until the field's three are in
        if (!read_component(fname, n, dcomp + (size_t)(c % 3) * n, st, s)) {
            g.m_bc_f.release();
            g.m_ec_f.release();
            return -1;
        }
        if (c % 3 != 2) continue;
        float* rec = (float*)(c < 3 ? g.m_bc_f.dev : g.m_ec_f.dev);
        const double scale = c < 3 ? B0 : E0;
        if (pow2_scale(scale)) scatter3_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dcomp, n, scale, rec);
        else scatter3_kernel<false><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dcomp, n, scale, rec);
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

// tp_read_pic_fields_h5: read_pic_bfields_float_h5 / read_pic_efields_float_h5
// (src/magnetic_field.c:632-692, src/electric_field.c:447-507) into device
// memory.  Each dataset's [0, nx) x [0, ny) x [0, nz) block streams from the
// file in whole i-planes through two pinned buffers (reading the next piece
// while the previous one copies); once a field's three components are on the
// device, one transpose kernel writes its whole records.
static int read_pic_fields_h5_impl(const char* fname, const char* gname, int with_e)
{
    if (!ensure_init()) return -1;
    if (multi_tframe != 0) {
        set_error(7, "tp_read_pic_fields_h5 reads one time frame (multi_tframe 0)");
        return -1;
    }
    const int nx = simul_grid.nx, ny = simul_grid.ny, nz = simul_grid.nz;
    if (nx < 1 || ny < 1 || nz < 1 || ny > 65535 || (nx + 31) / 32 > 65535 || !fname) {
        set_error(7, "tp_read_pic_fields_h5: grid %d x %d x %d or no file name", nx, ny, nz);
        return -1;
    }
    const size_t n = (size_t)nx * ny * nz;
    tph5::File f;
    if (!f.open(fname)) {
        set_error(7, "%s", f.error().c_str());
        return -1;
    }
    const char* names[6] = {"cbx", "cby", "cbz", "ex", "ey", "ez"};
    tph5::Dataset ds[6];
    const int ncomp = with_e ? 6 : 3;
    size_t es_max = 4;
    for (int c = 0; c < ncomp; c++) {
        if (!f.dataset(gname, names[c], ds[c])) {
            set_error(7, "%s", f.error().c_str());
            return -1;
        }
        const tph5::Dataset& d = ds[c];
        if (d.dims.size() != 3 || d.dims[0] < (uint64_t)nx || d.dims[1] < (uint64_t)ny || d.dims[2] < (uint64_t)nz) {
            set_error(7, "%s: dataset %s is not an array of at least %d x %d x %d", fname, names[c], nx, ny, nz);
            return -1;
        }
        if (d.type.cls != 1) {
            set_error(7, "%s: dataset %s is not floating point", fname, names[c]);
            return -1;
        }
        if (d.type.size > es_max) es_max = d.type.size;
    }
    cudaStream_t s = g.stream;
    static Scratch raw_dev;
    unsigned char* draw = (unsigned char*)raw_dev.get(3 * es_max * n);
    if (!draw) return -1;
    const size_t plane = (size_t)ny * nz;
    Staging st;
    const size_t piece_planes = std::max<size_t>(1, std::min<size_t>(nx, (sizeof(float) * kPiece) / (es_max * plane)));
    for (int b = 0; b < 2; b++)
        if (!cuda_ok(cudaMallocHost(&st.host[b], es_max * plane * piece_planes), "pinned staging") ||
            !cuda_ok(cudaEventCreateWithFlags(&st.done[b], cudaEventDisableTiming), "staging event") ||
            !cuda_ok(cudaEventRecord(st.done[b], s), "staging event"))
            return -1;
    if (!device_records(g.m_bc_f, sizeof(float) * 3 * n) || !device_records(g.m_ec_f, sizeof(float) * 3 * n))
        return -1;
    auto fail = [&]() {
        g.m_bc_f.release();
        g.m_ec_f.release();
        return -1;
    };
    if (!with_e && !cuda_ok(cudaMemsetAsync(g.m_ec_f.dev, 0, sizeof(float) * 3 * n, s), "E records")) return fail();
    Raw3 in;
    int b = 0;
    for (int c = 0; c < ncomp; c++) {
        const tph5::Dataset& d = ds[c];
        const size_t es = d.type.size;
        unsigned char* slot = draw + (size_t)(c % 3) * es_max * n;  // waits here until the field's three are in
        for (size_t i0 = 0; i0 < (size_t)nx; i0 += piece_planes) {
            const size_t m = std::min(piece_planes, (size_t)nx - i0);
            if (!cuda_ok(cudaEventSynchronize(st.done[b]), "staging")) return fail();
            const uint64_t off[3] = {i0, 0, 0}, cnt[3] = {m, (uint64_t)ny, (uint64_t)nz};
            if (!f.read(d, off, cnt, st.host[b])) {
                set_error(7, "%s", f.error().c_str());
                return fail();
            }
            if (!cuda_ok(cudaMemcpyAsync(slot + i0 * plane * es, st.host[b], m * plane * es, cudaMemcpyHostToDevice, s),
                         "field upload") ||
                !cuda_ok(cudaEventRecord(st.done[b], s), "staging event"))
                return fail();
            b ^= 1;
        }
        in.raw[c % 3] = slot;
        in.es[c % 3] = (int)es;
        in.be[c % 3] = d.type.atom.big_endian ? 1 : 0;
        if (c % 3 != 2) continue;
        float* rec = (float*)(c < 3 ? g.m_bc_f.dev : g.m_ec_f.dev);
        const dim3 grid((unsigned)((nz + 31) / 32), (unsigned)((nx + 31) / 32), (unsigned)ny), block(32, 8);
        const double scale = c < 3 ? B0 : E0;
        const bool p2 = pow2_scale(scale);
        const bool f32le = in.es[0] == 4 && in.es[1] == 4 && in.es[2] == 4 && !in.be[0] && !in.be[1] && !in.be[2];
        if (p2 && f32le) h5_transpose3_kernel<true, true><<<grid, block, 0, s>>>(in, nx, ny, nz, scale, rec);
        else if (p2) h5_transpose3_kernel<true, false><<<grid, block, 0, s>>>(in, nx, ny, nz, scale, rec);
        else if (f32le) h5_transpose3_kernel<false, true><<<grid, block, 0, s>>>(in, nx, ny, nz, scale, rec);
        else h5_transpose3_kernel<false, false><<<grid, block, 0, s>>>(in, nx, ny, nz, scale, rec);
        if (!cuda_ok(cudaGetLastError(), "field transpose")) return fail();
    }
    g.upload_gen++;
    return cuda_ok(cudaStreamSynchronize(s), "field read") ? 0 : fail();
}

extern "C" int tp_read_pic_fields_h5(const char* fname, const char* gname, int with_e)
{
    try {
        return read_pic_fields_h5_impl(fname, gname, with_e);
    } catch (const std::exception& e) {  // e.g. an allocation for a corrupted extent
        set_error(7, "tp_read_pic_fields_h5: %s", e.what());
    } catch (...) {
        set_error(7, "tp_read_pic_fields_h5 failed");
    }
    return -1;
}

// tp_save_pic_fields_h5: the device-resident PIC fields as the reference's
// PIC HDF5 file (the datasets tp_read_pic_fields_h5 reads), float, the
// records divided by B0 (E0).  Each field's three components are reordered on
// the GPU into C-order arrays, then each streams to the file in whole
// i-planes through two pinned buffers (the next piece copied while the
// previous one is written).
static int save_pic_fields_h5_impl(const char* fname, const char* gname, int with_e)
{
    if (!ensure_init()) return -1;
    const int nx = simul_grid.nx, ny = simul_grid.ny, nz = simul_grid.nz;
    if (!fname || !gname || nx < 1 || ny < 1 || nz < 1 || ny > 65535 || (nz + 31) / 32 > 65535) {
        set_error(7, "tp_save_pic_fields_h5: grid %d x %d x %d or no file / group name", nx, ny, nz);
        return -1;
    }
    if (!g.m_bc_f.device_only || !g.m_bc_f.dev || (with_e && (!g.m_ec_f.device_only || !g.m_ec_f.dev))) {
        set_error(7, "no device-resident PIC fields to save");
        return -1;
    }
    std::string grp = gname;
    while (!grp.empty() && grp[0] == '/') grp.erase(0, 1);
    const size_t n = (size_t)nx * ny * nz, plane = (size_t)ny * nz;
    tph5::Plan plan;
    tph5::WGroup wg;
    wg.name = grp;
    const char* names[6] = {"cbx", "cby", "cbz", "ex", "ey", "ez"};
    const int ncomp = with_e ? 6 : 3;
    for (int c = 0; c < ncomp; c++)
        wg.dsets.push_back({names[c], tph5::Type::ieee(4, false), {(uint64_t)nx, (uint64_t)ny, (uint64_t)nz}});
    plan.groups.push_back(wg);
    if (!plan.plan()) {
        set_error(7, "%s: %s", fname, plan.err.c_str());
        return -1;
    }
    std::string err;
    int fd = tph5::open_for_write(fname, err);
    if (fd < 0 || !tph5::write_meta(fd, plan, err)) {
        if (fd >= 0) close(fd);
        set_error(7, "%s", err.c_str());
        return -1;
    }
    cudaStream_t s = g.stream;
    static Scratch out_dev;
    float* dout = (float*)out_dev.get(sizeof(float) * 3 * n);
    Staging st;
    const size_t piece_planes = std::max<size_t>(1, std::min<size_t>(nx, kPiece / plane));
    bool ok = dout != nullptr;
    for (int b = 0; b < 2 && ok; b++)
        ok = cuda_ok(cudaMallocHost(&st.host[b], sizeof(float) * plane * piece_planes), "pinned staging") &&
             cuda_ok(cudaEventCreateWithFlags(&st.done[b], cudaEventDisableTiming), "staging event");
    for (int c = 0; c < ncomp && ok; c++) {
        if (c % 3 == 0) {  // the field's three components, reordered at once
            const float* rec = (const float*)(c < 3 ? g.m_bc_f.dev : g.m_ec_f.dev);
            const dim3 grid((unsigned)((nx + 31) / 32), (unsigned)((nz + 31) / 32), (unsigned)ny), block(32, 8);
            const double scale = c < 3 ? B0 : E0;
            if (pow2_scale(scale)) h5_untranspose3_kernel<true><<<grid, block, 0, s>>>(rec, nx, ny, nz, scale, dout);
            else h5_untranspose3_kernel<false><<<grid, block, 0, s>>>(rec, nx, ny, nz, scale, dout);
            ok = cuda_ok(cudaGetLastError(), "field reorder");
        }
        const float* src = dout + (size_t)(c % 3) * n;
        const tph5::WDataset& d = plan.groups[0].dsets[c];
        const size_t npieces = ((size_t)nx + piece_planes - 1) / piece_planes;
        auto enqueue = [&](size_t q) {
            const size_t i0 = q * piece_planes, m = std::min(piece_planes, (size_t)nx - i0);
            return cuda_ok(cudaMemcpyAsync(st.host[q & 1], src + i0 * plane, sizeof(float) * m * plane,
                                           cudaMemcpyDeviceToHost, s), "field download") &&
                   cuda_ok(cudaEventRecord(st.done[q & 1], s), "staging event");
        };
        if (ok) ok = enqueue(0);
        for (size_t q = 0; q < npieces && ok; q++) {
            if (q + 1 < npieces) ok = enqueue(q + 1);  // the next piece copies while this one is written
            ok = ok && cuda_ok(cudaEventSynchronize(st.done[q & 1]), "staging");
            const size_t i0 = q * piece_planes, m = std::min(piece_planes, (size_t)nx - i0);
            if (ok && !tph5::write_elements(fd, d, i0 * plane, m * plane, st.host[q & 1], err)) {
                set_error(7, "%s: %s", fname, err.c_str());
                ok = false;
            }
        }
    }
    ok = cuda_ok(cudaStreamSynchronize(s), "field save") && ok;
    close(fd);
    return ok ? 0 : -1;
}

extern "C" int tp_save_pic_fields_h5(const char* fname, const char* gname, int with_e)
{
    try {
        return save_pic_fields_h5_impl(fname, gname, with_e);
    } catch (const std::exception& e) {
        set_error(7, "tp_save_pic_fields_h5: %s", e.what());
    } catch (...) {
        set_error(7, "tp_save_pic_fields_h5 failed");
    }
    return -1;
}
