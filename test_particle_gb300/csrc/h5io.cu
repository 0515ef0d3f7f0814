// h5io.cu -- the reference's HDF5 files read and written by the library
// (h5lite.cpp), without libhdf5.
//
//   read_data_serial_{double,float}_h5, read_data_serial_{float,double}_binary:
//       the reference's data_io.c (src/data_io.c:22-120) with its signatures,
//       so a program linked against this library needs no data_io.o and no
//       libhdf5 to read its field files;
//   tp_h5_read / tp_h5_info: the same reads with an error status;
//   tp_save_particles_fields / tp_read_particles: particles_fields_init.h5 and
//       particle_diagnostics.h5 (src/diagnostics.c:290-387,
//       src/particle_info.c:376-488), the fields at the particles evaluated on
//       the GPU by the library's FP64 get_emf;
//   tp_h5_write_particles_fields: the writer alone, with the fields given;
//   tp_trajectory_diagnostics: the reference's trajectory diagnostics in one
//       process (src/diagnostics.c:403-568), from particles_fields_init.h5 to
//       particle_diagnostics.h5;
//   tp_h5_write_poincare: data/poincare_map.h5 (src/poincare_map.c:185-235).
// Several ranks writing one file each call with their own records: the file's
// layout depends only on the totals, so the rank holding the first record
// writes the metadata and every rank writes its records where they belong,
// with no exchange; the file is complete once every rank has returned.
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <atomic>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/tp_gpu.h"
#include "../../include/tp_h5.h"
#include "h5lite.h"
#include "tp_internal.h"

using namespace tp;

namespace {

const std::vector<std::string> kPtlNames = {"x", "y", "z", "qm", "ux", "uy", "uz", "t"};
const std::vector<std::string> kEmfNames = {"Bx", "By", "Bz", "Ex", "Ey", "Ez"};

// body(lo, hi) over [0, n) in up to 8 contiguous ranges of at least `grain`
// items, on threads (the calling thread takes the first range, and the rest
// when no thread can be started).  body must not throw.
template <class F>
void parallel_ranges(size_t n, size_t grain, F body)
{
    const size_t nt = std::min<size_t>(8, std::max<size_t>(1, n / std::max<size_t>(grain, 1)));
    if (nt <= 1) {
        body((size_t)0, n);
        return;
    }
    const size_t per = (n + nt - 1) / nt;
    std::vector<std::thread> th;
    size_t inline_from = n;
    for (size_t t = 1; t < nt && t * per < n; t++) {
        const size_t lo = t * per, hi = std::min(n, lo + per);
        try {
            th.emplace_back([body, lo, hi]() { body(lo, hi); });
        } catch (...) {
            inline_from = lo;
            break;
        }
    }
    body((size_t)0, std::min(per, n));
    for (size_t lo = inline_from; lo < n; lo += per) body(lo, std::min(n, lo + per));
    for (std::thread& t : th) t.join();
}

// The two datasets of a particles_fields file of ntot records.
tph5::Plan particles_plan(unsigned long long ntot)
{
    tph5::Plan p;
    tph5::WGroup g;
    g.name = "particles_fields";
    g.dsets.push_back({"particles", tph5::Type::compound_f64(kPtlNames, true), {ntot}});
    g.dsets.push_back({"fields", tph5::Type::compound_f64(kEmfNames, true), {ntot}});
    p.groups.push_back(g);
    p.plan();
    return p;
}

// A C entry point's body: exceptions (an allocation that failed for a
// corrupted extent, say) become an error status, never cross the C ABI.
template <class F>
int guarded(const char* what, F body)
{
    try {
        return body();
    } catch (const std::exception& e) {
        set_error(7, "%s: %s", what, e.what());
    } catch (...) {
        set_error(7, "%s failed", what);
    }
    return -1;
}

struct Fd {
    int fd = -1;
    ~Fd()
    {
        if (fd >= 0) close(fd);
    }
};

bool h5_read_as(const char* fname, const char* gname, const char* dset, int rank, const unsigned long long* count,
                const unsigned long long* offset, int elem_bytes, void* data)
{
    if (!fname || !dset || rank < 0 || rank > 32 || (rank > 0 && (!count || !offset)) ||
        (elem_bytes != 4 && elem_bytes != 8)) {
        set_error(7, "tp_h5_read: bad arguments");
        return false;
    }
    tph5::File f;
    tph5::Dataset ds;
    if (!f.open(fname) || !f.dataset(gname, dset, ds)) {
        set_error(7, "%s", f.error().c_str());
        return false;
    }
    if ((int)ds.dims.size() != rank) {
        set_error(7, "%s: dataset '%s' has rank %zu, not %d", fname, dset, ds.dims.size(), rank);
        return false;
    }
    if (ds.type.cls != 0 && ds.type.cls != 1) {
        set_error(7, "%s: dataset '%s' is not of a numeric type", fname, dset);
        return false;
    }
    uint64_t n = 1;
    std::vector<uint64_t> o(rank), c(rank);
    for (int d = 0; d < rank; d++) {
        o[d] = offset[d];
        c[d] = count[d];
        if (o[d] > ds.dims[d] || c[d] > ds.dims[d] - o[d]) {
            set_error(7, "%s: selection beyond the dataset's extent in dimension %d", fname, d);
            return false;
        }
        n *= c[d];
    }
    std::vector<uint8_t> raw(n * ds.type.size);
    if (!f.read(ds, o.data(), c.data(), raw.data())) {
        set_error(7, "%s", f.error().c_str());
        return false;
    }
    if (elem_bytes == 8) tph5::raw_to_double(ds.type, raw.data(), n, (double*)data);
    else tph5::raw_to_float(ds.type, raw.data(), n, (float*)data);
    return true;
}

}  // namespace

static int tp_h5_read_impl(const char* fname, const char* gname, const char* dset, int rank,
                          const unsigned long long* count, const unsigned long long* offset, int elem_bytes,
                          void* data)
{
    return h5_read_as(fname, gname, dset, rank, count, offset, elem_bytes, data) ? 0 : -1;
}

static int tp_h5_info_impl(const char* fname, const char* gname, const char* dset, int* rank,
                          unsigned long long* dims, int* type_class, int* type_size)
{
    tph5::File f;
    tph5::Dataset ds;
    if (!fname || !dset || !f.open(fname) || !f.dataset(gname, dset, ds)) {
        set_error(7, "%s", fname ? f.error().c_str() : "tp_h5_info: no file name");
        return -1;
    }
    if (ds.dims.size() > 32) {
        set_error(7, "%s: rank above 32", fname);
        return -1;
    }
    if (rank) *rank = (int)ds.dims.size();
    if (dims)
        for (size_t d = 0; d < ds.dims.size(); d++) dims[d] = ds.dims[d];
    if (type_class) *type_class = ds.type.cls;
    if (type_size) *type_size = (int)ds.type.size;
    return 0;
}

// src/data_io.c:22-47 and :52-75.  libhdf5 prints its error stack and the
// reference carries on; these print the reason and leave data untouched.
extern "C" void read_data_serial_double_h5(int rank, unsigned long long* count, unsigned long long* offset,
                                           char* fname, char* gname, char* dset_name, double* data)
{
    if (guarded("read_data_serial_double_h5",
                [&]() { return h5_read_as(fname, gname, dset_name, rank, count, offset, 8, data) ? 0 : -1; }) != 0)
        fprintf(stderr, "HDF5 read: %s\n", g.err);
}

extern "C" void read_data_serial_float_h5(int rank, unsigned long long* count, unsigned long long* offset,
                                          char* fname, char* gname, char* dset_name, float* data)
{
    if (guarded("read_data_serial_float_h5",
                [&]() { return h5_read_as(fname, gname, dset_name, rank, count, offset, 4, data) ? 0 : -1; }) != 0)
        fprintf(stderr, "HDF5 read: %s\n", g.err);
}

// src/data_io.c:90-120: the file's values from element `offset` on.
template <class T>
static void read_binary(const char* fname, long offset, long size, T* data)
{
    FILE* fp = fopen(fname, "r");
    if (!fp) {
        printf("Unable to open file %s!\n", fname);
        exit(1);
    }
    fseek(fp, offset * (long)sizeof(T), SEEK_SET);
    size_t got = fread(data, sizeof(T), (size_t)size, fp);
    (void)got;  // a short file leaves the rest untouched, as the reference
    fclose(fp);
}

extern "C" void read_data_serial_float_binary(char* fname, long offset, long size, float* data)
{
    read_binary(fname, offset, size, data);
}

extern "C" void read_data_serial_double_binary(char* fname, long offset, long size, double* data)
{
    read_binary(fname, offset, size, data);
}

static int tp_h5_write_particles_fields_impl(const char* fname, int write_meta, unsigned long long ntot,
                                            unsigned long long offset, int nptl, const particles* ptl,
                                            const emfields* emf)
{
    if (!fname || nptl < 0 || offset + (unsigned long long)nptl > ntot || (nptl > 0 && (!ptl || !emf))) {
        set_error(7, "tp_h5_write_particles_fields: bad arguments");
        return -1;
    }
    tph5::Plan p = particles_plan(ntot);
    std::string err;
    Fd fd;
    fd.fd = tph5::open_for_write(fname, err);
    if (fd.fd < 0 || (write_meta && !tph5::write_meta(fd.fd, p, err))) {
        set_error(7, "%s", err.c_str());
        return -1;
    }
    const tph5::WDataset* dp = p.find("particles_fields", "particles");
    const tph5::WDataset* de = p.find("particles_fields", "fields");
    // ranges of the records on several threads, each converting and writing
    // blocks of its own (the byte-order conversion and the copies into the
    // page cache both run at a few GB/s per thread)
    constexpr size_t kBlock = 65536;
    std::atomic<bool> failed{false};
    std::mutex err_lock;
    parallel_ranges((size_t)nptl, kBlock, [&](size_t lo, size_t hi) {
        std::string e;
        try {
            std::vector<uint8_t> buf(kBlock * 64);
            for (size_t i0 = lo; i0 < hi && !failed; i0 += kBlock) {
                const size_t m = std::min(kBlock, hi - i0);
                for (size_t i = 0; i < m; i++) {
                    const particles& q = ptl[i0 + i];
                    const double v[8] = {q.x, q.y, q.z, q.qm, q.ux, q.uy, q.uz, q.t};
                    for (int c = 0; c < 8; c++) tph5::put_f64(&buf[64 * i + 8 * c], v[c], true);
                }
                if (!tph5::write_elements(fd.fd, *dp, offset + i0, m, buf.data(), e)) break;
                for (size_t i = 0; i < m; i++) {
                    const emfields& q = emf[i0 + i];
                    const double v[6] = {q.Bx, q.By, q.Bz, q.Ex, q.Ey, q.Ez};
                    for (int c = 0; c < 6; c++) tph5::put_f64(&buf[48 * i + 8 * c], v[c], true);
                }
                if (!tph5::write_elements(fd.fd, *de, offset + i0, m, buf.data(), e)) break;
            }
        } catch (const std::exception& x) {
            e = x.what();
        }
        if (!e.empty()) {
            std::lock_guard<std::mutex> lk(err_lock);
            if (err.empty()) err = e;
            failed = true;
        }
    });
    if (!err.empty()) {
        set_error(7, "%s: %s", fname, err.c_str());
        return -1;
    }
    return 0;
}

// save_particles_fields, src/diagnostics.c:290-387: this rank's nptl records
// at offset naccumulate[mpi_rank - 1] (0 for rank 0) of ntot, with the fields
// at each record's (x, y, z, t) from the library's FP64 get_emf.
static int tp_save_particles_fields_impl(int mpi_rank, int nptl, particles* ptl, int ntot, int* naccumulate,
                                        char* fname, int system_type_arg)
{
    (void)system_type_arg;  // the reference passes it through unused
    if (mpi_rank < 0 || nptl < 0 || ntot < 0 || (mpi_rank > 0 && !naccumulate)) {
        set_error(7, "tp_save_particles_fields: bad arguments");
        return -1;
    }
    const unsigned long long off = mpi_rank == 0 ? 0ull : (unsigned long long)naccumulate[mpi_rank - 1];
    std::vector<emfields> emf((size_t)nptl);
    if (nptl > 0) {
        std::vector<double> xyzt(4 * (size_t)nptl);
        for (int i = 0; i < nptl; i++) {
            xyzt[4 * (size_t)i] = ptl[i].x;
            xyzt[4 * (size_t)i + 1] = ptl[i].y;
            xyzt[4 * (size_t)i + 2] = ptl[i].z;
            xyzt[4 * (size_t)i + 3] = ptl[i].t;
        }
        static_assert(sizeof(emfields) == 6 * sizeof(double), "emfields is six doubles");
        if (tp_get_emf_batch(nptl, xyzt.data(), (double*)emf.data()) != 0) return -1;
    }
    return tp_h5_write_particles_fields(fname, off == 0, (unsigned long long)ntot, off, nptl, ptl, emf.data());
}

// read_particles, src/particle_info.c:376-443: records [offset, offset + nptl)
// of /particles_fields/particles into x, y, z, qm, ux, uy, uz, t of ptl (the
// other members are left as they are), converted from the file's type.
static int tp_read_particles_impl(int mpi_rank, int nptl, int* nptl_accumulate, particles* ptl, char* fname)
{
    if (mpi_rank < 0 || nptl < 0 || (mpi_rank > 0 && !nptl_accumulate) || !fname || (nptl > 0 && !ptl)) {
        set_error(7, "tp_read_particles: bad arguments");
        return -1;
    }
    tph5::File f;
    tph5::Dataset ds;
    if (!f.open(fname) || !f.dataset("/particles_fields", "particles", ds)) {
        set_error(7, "%s", f.error().c_str());
        return -1;
    }
    if (ds.dims.size() != 1 || ds.type.cls != 6) {
        set_error(7, "%s: /particles_fields/particles is not a 1-D compound dataset", fname);
        return -1;
    }
    const tph5::Member* mem[8] = {nullptr};
    for (const tph5::Member& m : ds.type.members)
        for (int c = 0; c < 8; c++)
            if (m.name == kPtlNames[c]) {
                if (m.type.cls < 0) {
                    set_error(7, "%s: member %s is not numeric", fname, m.name.c_str());
                    return -1;
                }
                if ((uint64_t)m.offset + m.type.size > ds.type.size) {
                    set_error(7, "%s: member %s lies outside the record", fname, m.name.c_str());
                    return -1;
                }
                mem[c] = &m;
            }
    const uint64_t off = mpi_rank == 0 ? 0 : (uint64_t)nptl_accumulate[mpi_rank - 1];
    // blocks of about 32 MiB (read on several threads by the reader), each
    // converted on several threads
    const uint64_t block = std::max<uint64_t>(65536, ((uint64_t)32 << 20) / ds.type.size);
    std::vector<uint8_t> raw(std::min<uint64_t>(block, std::max(nptl, 1)) * ds.type.size);
    for (uint64_t i0 = 0; i0 < (uint64_t)nptl; i0 += block) {
        uint64_t m = (uint64_t)nptl - i0 < block ? (uint64_t)nptl - i0 : block;
        uint64_t o = off + i0;
        if (!f.read(ds, &o, &m, raw.data())) {
            set_error(7, "%s", f.error().c_str());
            return -1;
        }
        const size_t es = ds.type.size;
        parallel_ranges((size_t)m, 65536, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; i++) {
                double* rec = (double*)&ptl[i0 + i];
                const uint8_t* src = &raw[i * es];
                // particles: x, y, z, qm, ux, uy, uz, t are its first eight doubles
                for (int c = 0; c < 8; c++)
                    if (mem[c]) rec[c] = tph5::decode(mem[c]->type, src + mem[c]->offset);
            }
        });
    }
    return 0;
}

// data/poincare_map.h5: /poincare_map/{xpos,ypos,zpos} [npoints_total][ncross + 1]
// native doubles; this rank's rows [nshift, nshift + npoints).
static int tp_h5_write_poincare_impl(const char* fname, int npoints_total, int ncross, int nshift, int npoints,
                                    const double* xpos, const double* ypos, const double* zpos)
{
    if (!fname || npoints_total < 0 || ncross < 0 || nshift < 0 || npoints < 0 || nshift + npoints > npoints_total ||
        (npoints > 0 && (!xpos || !ypos || !zpos))) {
        set_error(7, "tp_h5_write_poincare: bad arguments");
        return -1;
    }
    tph5::Plan p;
    tph5::WGroup g;
    g.name = "poincare_map";
    const std::vector<uint64_t> dims = {(uint64_t)npoints_total, (uint64_t)ncross + 1};
    for (const char* n : {"xpos", "ypos", "zpos"}) g.dsets.push_back({n, tph5::Type::ieee(8, false), dims});
    p.groups.push_back(g);
    p.plan();
    std::string err;
    Fd fd;
    fd.fd = tph5::open_for_write(fname, err);
    if (fd.fd < 0 || (nshift == 0 && !tph5::write_meta(fd.fd, p, err))) {
        set_error(7, "%s", err.c_str());
        return -1;
    }
    const size_t m = (size_t)npoints * (ncross + 1);
    std::vector<uint8_t> buf(8 * m);
    const double* src[3] = {xpos, ypos, zpos};
    for (int c = 0; c < 3 && err.empty(); c++) {
        for (size_t i = 0; i < m; i++) tph5::put_f64(&buf[8 * i], src[c][i], false);
        tph5::write_elements(fd.fd, p.groups[0].dsets[c], (uint64_t)nshift * (ncross + 1), m, buf.data(), err);
    }
    if (!err.empty()) {
        set_error(7, "%s: %s", fname, err.c_str());
        return -1;
    }
    return 0;
}

// trajectory_diagnostics, src/diagnostics.c:504-568, with
// sort_particles_energy (:403-437) and init_ptl_traj (:455-481), for one
// process.  The particles are sorted by energy (gamma - 1 of their final
// state; particles of equal energy keep their array order, where the
// reference's quicksort may order them differently), their initial states
// reloaded from data/particles_fields_init.h5 in that order, and
// nptl_traj_tot of them chosen at a uniform interval from the highest energy
// down; they are tracked again with trajectory records every nsteps_output
// steps (scaled up as the reference does when a particle took more than 1e6
// steps), and the records are written with their fields to
// data/particle_diagnostics.h5.  The arrays are updated as the reference
// updates them (ptl and nsteps_ptl_tracking sorted; nsteps_ptl_tracking then
// as particle_tracking_hybrid leaves it).
static int trajectory_diagnostics_impl(int mpi_rank, int mpi_size, int nptl, double dt, double pmass,
                                       int nptl_traj_tot, int system_type_arg, particles* ptl, int* nptl_accumulate,
                                       int* nsteps_ptl_tracking, int nbins, int nt_out, int* nsteps_output,
                                       int bc_flag, int tracking_method, particles* ptl_init)
{
    (void)nptl_accumulate;
    if (mpi_size != 1 || mpi_rank != 0) {
        set_error(7, "tp_trajectory_diagnostics runs in one process (the reference's own "
                     "trajectory_diagnostics gathers the ranks' counts over MPI)");
        return -1;
    }
    if (nptl < 1 || nptl_traj_tot < 1 || nptl_traj_tot > nptl || !ptl || !nsteps_ptl_tracking || !nsteps_output ||
        *nsteps_output < 1 || !ptl_init) {
        set_error(7, "tp_trajectory_diagnostics: bad arguments");
        return -1;
    }
    // sort_particles_energy
    std::vector<double> ene((size_t)nptl);
    for (int i = 0; i < nptl; i++)
        ene[i] = sqrt(1.0 + ptl[i].ux * ptl[i].ux + ptl[i].uy * ptl[i].uy + ptl[i].uz * ptl[i].uz) - 1.0;
    std::vector<int> idx((size_t)nptl);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int u, int v) { return ene[u] < ene[v]; });
    std::vector<particles> init((size_t)nptl);
    memset(init.data(), 0, sizeof(particles) * (size_t)nptl);
    char init_name[] = "data/particles_fields_init.h5";
    if (tp_read_particles(0, nptl, nullptr, init.data(), init_name) != 0) return -1;
    std::vector<int> nst(nsteps_ptl_tracking, nsteps_ptl_tracking + nptl);
    for (int i = 0; i < nptl; i++) {
        ptl[i] = init[idx[i]];
        nsteps_ptl_tracking[i] = nst[idx[i]];
    }
    // init_ptl_traj (one process: particle_broadcast gives it every trajectory particle)
    const int nptl_traj = nptl_traj_tot;
    const int interval = nptl / nptl_traj;
    int ntraj_max = 0;
    for (int i = 0; i < nptl_traj; i++) ntraj_max = std::max(ntraj_max, nsteps_ptl_tracking[i]);  // as the reference
    if (ntraj_max > 1.0e6) *nsteps_output = (int)((*nsteps_output) * ((double)ntraj_max) / 1.0e6);
    std::vector<int> ntraj_accum((size_t)nptl_traj);
    std::vector<particles> ptl_traj((size_t)nptl_traj);
    long long ntraj = 0;
    for (int i = 0, j = nptl - 1; i < nptl_traj; i++, j -= interval) {
        ntraj_accum[i] = (nsteps_ptl_tracking[j] - 1) / (*nsteps_output) + 1;
        ntraj += ntraj_accum[i];
        ptl_traj[i] = ptl[j];
    }
    if (ntraj > 2147483647LL) {
        set_error(7, "tp_trajectory_diagnostics: %lld trajectory points", ntraj);
        return -1;
    }
    for (int i = 1; i < nptl_traj; i++) ntraj_accum[i] += ntraj_accum[i - 1];
    std::vector<particles> ptl_time((size_t)ntraj);
    memset(ptl_time.data(), 0, sizeof(particles) * (size_t)ntraj);
    for (int i = 0; i < nptl_traj; i++) ptl_time[i == 0 ? 0 : ntraj_accum[i - 1]] = ptl_traj[i];
    particle_tracking_hybrid(0, nptl_traj, dt, nbins, nt_out, bc_flag, *nsteps_output, pmass, ntraj_accum.data(),
                             tracking_method, 1, ptl_init, nsteps_ptl_tracking, ptl_traj.data(), ptl_time.data());
    int acc[1] = {(int)ntraj};
    char out_name[] = "data/particle_diagnostics.h5";
    return tp_save_particles_fields(0, (int)ntraj, ptl_time.data(), (int)ntraj, acc, out_name, system_type_arg);
}

extern "C" int tp_h5_read(const char* fname, const char* gname, const char* dset, int rank,
                          const unsigned long long* count, const unsigned long long* offset, int elem_bytes,
                          void* data)
{
    return guarded("tp_h5_read",
                   [&]() { return tp_h5_read_impl(fname, gname, dset, rank, count, offset, elem_bytes, data); });
}

extern "C" int tp_h5_info(const char* fname, const char* gname, const char* dset, int* rank,
                          unsigned long long* dims, int* type_class, int* type_size)
{
    return guarded("tp_h5_info",
                   [&]() { return tp_h5_info_impl(fname, gname, dset, rank, dims, type_class, type_size); });
}

extern "C" int tp_h5_write_particles_fields(const char* fname, int write_meta, unsigned long long ntot,
                                            unsigned long long offset, int nptl, const particles* ptl,
                                            const emfields* emf)
{
    return guarded("tp_h5_write_particles_fields",
                   [&]() {
                       return tp_h5_write_particles_fields_impl(fname, write_meta, ntot, offset, nptl, ptl, emf);
                   });
}

extern "C" int tp_save_particles_fields(int mpi_rank, int nptl, particles* ptl, int ntot, int* naccumulate,
                                        char* fname, int system_type_arg)
{
    return guarded("tp_save_particles_fields",
                   [&]() {
                       return tp_save_particles_fields_impl(mpi_rank, nptl, ptl, ntot, naccumulate, fname,
                                                            system_type_arg);
                   });
}

extern "C" int tp_read_particles(int mpi_rank, int nptl, int* nptl_accumulate, particles* ptl, char* fname)
{
    return guarded("tp_read_particles",
                   [&]() { return tp_read_particles_impl(mpi_rank, nptl, nptl_accumulate, ptl, fname); });
}

extern "C" int tp_h5_write_poincare(const char* fname, int npoints_total, int ncross, int nshift, int npoints,
                                    const double* xpos, const double* ypos, const double* zpos)
{
    return guarded("tp_h5_write_poincare",
                   [&]() {
                       return tp_h5_write_poincare_impl(fname, npoints_total, ncross, nshift, npoints, xpos, ypos,
                                                        zpos);
                   });
}

extern "C" int tp_trajectory_diagnostics(int mpi_rank, int mpi_size, int nptl, double dt, double pmass,
                                         int nptl_traj_tot, int system_type_arg, particles* ptl, int* nptl_accumulate,
                                         int* nsteps_ptl_tracking, int nbins, int nt_out, int* nsteps_output,
                                         int bc_flag, int tracking_method, particles* ptl_init)
{
    return guarded("tp_trajectory_diagnostics", [&]() {
        return trajectory_diagnostics_impl(mpi_rank, mpi_size, nptl, dt, pmass, nptl_traj_tot, system_type_arg, ptl,
                                           nptl_accumulate, nsteps_ptl_tracking, nbins, nt_out, nsteps_output,
                                           bc_flag, tracking_method, ptl_init);
    });
}
