// ref_api.cu -- the reference's tracking / field entry points, by name and
// signature, running on the GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sys/time.h>
#include <vector>

#include "../../include/tp_gpu.h"
#include "tp_internal.h"
#include "tp_kernels.h"
#include "tp_session.h"

using namespace tp;

// Provided by the caller's diagnostics.c (src/diagnostics.c:221-248, 723-782);
// host_config.cpp holds single-rank fallbacks with the same output format.
extern "C" void collect_espectrum(int mpi_rank, int nbins, int nt_out, double* espectrum,
                                  double* espect_tot, char* fname);
extern "C" void collect_diff_coeffs(int mpi_rank, int nsteps_dcoeffs, double* drr, double* dxx,
                                    double* dyy, double* dzz, double* dpp, double* duu,
                                    double* daa, double* dee, char* fname, int* nptl_remain);

// ---------------------------------------------------------------- setters
extern "C" void set_variables_tracking(grids* sgrid, domain* sdomain, int stype, int mt)
{
    memcpy(&simul_grid, sgrid, sizeof(grids));
    memcpy(&simul_domain, sdomain, sizeof(domain));
    system_type = stype;
    multi_tframe = mt;
}

extern "C" void set_ptl_params_tracking(int pbc, double qm)
{
    bc_flag = pbc;
    charge_mass = qm;
}

extern "C" void set_variables_emfields(int stype) { system_type = stype; }

extern "C" void set_variabls_interpolation(grids* sgrid, domain* sdomain, int mt)
{
    memcpy(&simul_grid, sgrid, sizeof(grids));
    memcpy(&simul_domain, sdomain, sizeof(domain));
    multi_tframe = mt;
}

extern "C" void set_variables_ff(grids* sgrid, domain* sdomain)
{
    memcpy(&simul_grid, sgrid, sizeof(grids));
    memcpy(&simul_domain, sdomain, sizeof(domain));
}

// ---------------------------------------------------------------- single-point fields
static void emf_point(int stype, double x, double y, double z, double t, emfields* emf,
                      const char* who)
{
    DevField f;
    double xyzt[4] = {x, y, z, t}, out[6];
    if (!build_field(stype, f)) die_if_error(who);
    double* d_in = (double*)g.s_batch_a.get(sizeof(double) * 4);
    double* d_out = (double*)g.s_batch_b.get(sizeof(double) * 6);
    if (!d_in || !d_out) die_if_error(who);
    cudaMemcpyAsync(d_in, xyzt, sizeof(xyzt), cudaMemcpyHostToDevice, g.stream);
    cuda_ok(fp64::launch_emf_batch(f, 1, d_in, d_out, g.d_status, g.stream), who);
    cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDeviceToHost, g.stream);
    cuda_ok(cudaStreamSynchronize(g.stream), who);
    die_if_error(who);
    emf->Bx = out[0]; emf->By = out[1]; emf->Bz = out[2];
    emf->Ex = out[3]; emf->Ey = out[4]; emf->Ez = out[5];
}

extern "C" void get_emf(double x, double y, double z, double t, struct emfields* emf)
{
    if (system_type < 0 || system_type > TP_SYS_MODESUM) {
        printf("ERROR: wrong system type.\n");
        exit(1);
    }
    emf_point(system_type, x, y, z, t, emf, "get_emf");
}

extern "C" void get_magnetic_field(double x, double y, double z, double t, struct emfields* emf)
{
    if (system_type != TP_SYS_MHD && system_type != TP_SYS_PIC) {
        printf("ERROR: wrong system type.\n");
        exit(1);
    }
    emf_point(system_type, x, y, z, t, emf, "get_magnetic_field");
    emf->Ex = 0.0; emf->Ey = 0.0; emf->Ez = 0.0;
}

extern "C" void getemf_test(double x, double y, double z, double t, struct emfields* emf)
{ emf_point(TP_SYS_TEST, x, y, z, t, emf, "getemf_test"); }
extern "C" void getemf_mhd_test_particle(double x, double y, double z, double t, struct emfields* emf)
{ emf_point(TP_SYS_MHD, x, y, z, t, emf, "getemf_mhd_test_particle"); }
extern "C" void getemf_pic_test_particle(double x, double y, double z, double t, struct emfields* emf)
{ emf_point(TP_SYS_PIC, x, y, z, t, emf, "getemf_pic_test_particle"); }
extern "C" void get_bfield_mhd_test_particle(double x, double y, double z, double t, struct emfields* emf)
{
    emf_point(TP_SYS_MHD, x, y, z, t, emf, "get_bfield_mhd_test_particle");
    emf->Ex = 0.0; emf->Ey = 0.0; emf->Ez = 0.0;
}
extern "C" void get_bfield_pic_test_particle(double x, double y, double z, double t, struct emfields* emf)
{
    emf_point(TP_SYS_PIC, x, y, z, t, emf, "get_bfield_pic_test_particle");
    emf->Ex = 0.0; emf->Ey = 0.0; emf->Ez = 0.0;
}
extern "C" void getemf_ff(double x, double y, double z, double t, struct emfields* emf)
{ emf_point(TP_SYS_FORCEFREE, x, y, z, t, emf, "getemf_ff"); }
extern "C" void getemf_wlcs(double x, double y, double z, double t, struct emfields* emf)
{ emf_point(TP_SYS_WLCS, x, y, z, t, emf, "getemf_wlcs"); }

// getb_ff: the ABC field alone.  B does not depend on the velocity grid, so
// it is the B of the full force-free evaluation; the grid pointers are left
// alone (clearing them for the call would drop the grids' device copies and
// make the next call upload them again).
extern "C" void getb_ff(double x, double y, double z, double t, struct bfields* bmf)
{
    emfields e;
    emf_point(TP_SYS_FORCEFREE, x, y, z, t, &e, "getb_ff");
    bmf->Bx = e.Bx; bmf->By = e.By; bmf->Bz = e.Bz;
}

static void point_interp(int which, double x, double y, double z, double t, double out[3],
                         const char* who)
{
    DevField f;
    double xyzt[4] = {x, y, z, t};
    if (!build_field_points(f)) die_if_error(who);
    double* d_in = (double*)g.s_batch_a.get(sizeof(double) * 4);
    double* d_out = (double*)g.s_batch_b.get(sizeof(double) * 3);
    if (!d_in || !d_out) die_if_error(who);
    cudaMemcpyAsync(d_in, xyzt, sizeof(xyzt), cudaMemcpyHostToDevice, g.stream);
    cuda_ok(fp64::launch_point_interp(f, which, 1, d_in, d_out, g.d_status, g.stream), who);
    cudaMemcpyAsync(out, d_out, sizeof(double) * 3, cudaMemcpyDeviceToHost, g.stream);
    cuda_ok(cudaStreamSynchronize(g.stream), who);
    die_if_error(who);
}

// gete_ff: E = -v x B with the caller's B (src/force_free.c:78-86); the
// velocity interpolation runs on the GPU, the cross product of the returned
// values is the same three lines as the reference.
extern "C" void gete_ff(double x, double y, double z, double t, struct bfields* bmf,
                        struct efields* elf)
{
    double v[3];
    point_interp(5, x, y, z, t, v, "gete_ff");
    elf->Ex = bmf->By * v[2] - bmf->Bz * v[1];
    elf->Ey = bmf->Bz * v[0] - bmf->Bx * v[2];
    elf->Ez = bmf->Bx * v[1] - bmf->By * v[0];
}

#define TP_POINT_FN(name, which, T)                                                        \
    extern "C" void name(double x, double y, double z, double t, T* a, T* b, T* c)         \
    {                                                                                      \
        double v[3];                                                                       \
        point_interp(which, x, y, z, t, v, #name);                                         \
        *a = (T)v[0]; *b = (T)v[1]; *c = (T)v[2];                                          \
    }
TP_POINT_FN(get_float_bfield_at_point, 0, float)
TP_POINT_FN(get_float_efield_at_point, 1, float)
TP_POINT_FN(get_float_velocity_at_point, 2, float)
TP_POINT_FN(get_double_bfield_at_point, 3, double)
TP_POINT_FN(get_double_efield_at_point, 4, double)
TP_POINT_FN(get_double_velocity_at_point, 5, double)

extern "C" void get_trilinar_parameters(double x, double y, double z, double t, long int* corners,
                                        double* weights, double* dt)
{
    double xyzt[4] = {x, y, z, t};
    if (tp_trilinear_batch(1, xyzt, corners, weights) != 0) die_if_error("get_trilinar_parameters");
    if (multi_tframe == 0) *dt = 0.0;
    else {
        int it1 = (int)floor(t / simul_grid.dt);  // src/interpolation.c:98-100
        *dt = t / simul_grid.dt - it1;
    }
}

// grid_indices, src/interpolation.c:36-105: index arithmetic of one point
// (host side: integer bookkeeping for the caller, not part of any GPU loop).
extern "C" void grid_indices(double x, double y, double z, double t, int* ix1, int* iy1,
                             int* iz1, int* it1, int* ix2, int* iy2, int* iz2, int* it2,
                             double* dx, double* dy, double* dz, double* dt)
{
    const grids& G = simul_grid;
    const domain& D = simul_domain;
    *ix1 = (int)floor((x - D.xmin) / G.dx);
    *iy1 = (int)floor((y - D.ymin) / G.dy);
    *iz1 = (int)floor((z - D.zmin) / G.dz);
    *ix2 = *ix1 + 1; *iy2 = *iy1 + 1; *iz2 = *iz1 + 1;
    *dx = (x - D.xmin) / G.dx - (*ix1);
    *dy = (y - D.ymin) / G.dy - (*iy1);
    *dz = (z - D.zmin) / G.dz - (*iz1);
    if (x > D.xmax) { *ix1 = G.nx - 1; *ix2 = 0; *dx = x / G.dx - (G.nx - 1); }
    if (y > D.ymax) { *iy1 = G.ny - 1; *iy2 = 0; *dy = y / G.dy - (G.ny - 1); }
    if (z > D.zmax) { *iz1 = G.nz - 1; *iz2 = 0; *dz = z / G.dz - (G.nz - 1); }
    if (x < D.xmin) { *ix1 = G.nx - 1; *ix2 = 0; *dx = x / G.dx + 1.0; }
    if (y < D.ymin) { *iy1 = G.ny - 1; *iy2 = 0; *dy = y / G.dy + 1.0; }
    if (z < D.zmin) { *iz1 = G.nz - 1; *iz2 = 0; *dz = z / G.dz + 1.0; }
    if (multi_tframe == 0) {
        *it1 = 0; *it2 = 0; *dt = 0.0;
    } else if (multi_tframe == 1) {
        *it1 = (int)floor(t / G.dt);
        *it2 = *it1 + 1;
        *dt = t / G.dt - (*it1);
    } else {
        printf("ERROR: wrong choice of time slices.\n");
        exit(1);
    }
}

// ---------------------------------------------------------------- single particle
extern "C" void tracking_wirz(struct particles* ptl, double dt)
{
    DevField f;
    if (!build_field(system_type, f)) die_if_error("tracking_wirz");
    double* d = (double*)g.s_batch_a.get(sizeof(particles));
    if (!d) die_if_error("tracking_wirz");
    cudaMemcpyAsync(d, ptl, sizeof(particles), cudaMemcpyHostToDevice, g.stream);
    cuda_ok(fp64::launch_wirz_steps(f, 1, d, 1, dt, nullptr, g.d_status, g.stream), "tracking_wirz");
    cudaMemcpyAsync(ptl, d, sizeof(particles), cudaMemcpyDeviceToHost, g.stream);
    cuda_ok(cudaStreamSynchronize(g.stream), "tracking_wirz");
    die_if_error("tracking_wirz");
}

extern "C" void particle_bc(particles* ptl, int* iescape)
{
    DevField f;
    if (!build_field(TP_SYS_TEST, f)) die_if_error("particle_bc");
    double* d = (double*)g.s_batch_a.get(sizeof(particles) + 16);
    if (!d) die_if_error("particle_bc");
    int* d_esc = (int*)(d + 11);
    cudaMemcpyAsync(d, ptl, sizeof(particles), cudaMemcpyHostToDevice, g.stream);
    cudaMemcpyAsync(d_esc, iescape, sizeof(int), cudaMemcpyHostToDevice, g.stream);
    cuda_ok(fp64::launch_bc(f, 1, d, d_esc, g.stream), "particle_bc");
    cudaMemcpyAsync(ptl, d, sizeof(particles), cudaMemcpyDeviceToHost, g.stream);
    cudaMemcpyAsync(iescape, d_esc, sizeof(int), cudaMemcpyDeviceToHost, g.stream);
    cuda_ok(cudaStreamSynchronize(g.stream), "particle_bc");
    die_if_error("particle_bc");
}

// ---------------------------------------------------------------- tracking loops
// Host bookkeeping of one GPU run in the reference's array shapes.
struct RunOut {
    std::vector<double> espect, espect_esc, dsum;
    std::vector<int> remain;
};

static bool run_range(int nptl, const RunSpec& rs, particles* ptl_init, particles* ptl,
                      int* nsteps_ptl, int* ntraj_accum, int* traj_points, particles* ptl_time,
                      RunOut& o, double* wall_ms)
{
    Session& s = cached_session();
    if (!s.load(ptl_init, ptl, nptl)) return false;
    if (rs.traj_every > 0 && !s.set_traj(ntraj_accum, ptl_time, traj_points)) return false;
    if (!rs.reset_nsteps && nsteps_ptl && nptl > 0)
        cudaMemcpyAsync(s.nsteps.ptr, nsteps_ptl, sizeof(int) * nptl, cudaMemcpyHostToDevice, g.stream);
    tp_run_info info;
    if (!s.run(rs, &info)) return false;
    size_t nspec = (size_t)rs.nt_out * rs.nbins;
    o.espect.assign(nspec, 0.0);
    o.espect_esc.assign(nspec, 0.0);
    o.dsum.assign((size_t)8 * s.nsdc, 0.0);
    o.remain.assign(s.nsdc, 0);
    if (!s.fetch(ptl, nsteps_ptl, o.espect.data(), o.espect_esc.data(), o.dsum.data(),
                 o.remain.data())) return false;
    if (rs.traj_every > 0 && !s.get_traj(ptl_time, traj_points)) return false;
    if (wall_ms) *wall_ms = info.kernel_ms;
    return true;
}

extern "C" void particle_tracking_fixed_time_step(int mpi_rank, int nptl, double dt, int nbins,
        int nt_out, int traj_diagnose, int nsteps_output, double pmass, int* ntraj_accum,
        particles* ptl_init, int* nsteps_ptl_tracking, particles* ptl, double* espectrum,
        double* espect_tot, double* espect_escape, double* espect_private,
        double* espect_escape_private, particles* ptl_time)
{
    (void)pmass; (void)espect_tot; (void)espect_private; (void)espect_escape_private;
    RunSpec rs;
    if (!derive_steps(dt, nt_out, rs.estep, rs.einterval)) die_if_error("particle_tracking_fixed_time_step");
    if (mpi_rank == 0) {
        printf("Energy output time interval %d\n", rs.einterval);
        printf("Time step for diffusion coefficients: %d\n", rs.estep / kDiffInterval + 1);
    }
    rs.precision = TP_PREC_FP64;
    rs.dt = dt;
    rs.nt_out = nt_out;
    rs.nbins = nbins;
    rs.traj_every = traj_diagnose == 1 ? nsteps_output : 0;
    RunOut o;
    if (!run_range(nptl, rs, ptl_init, ptl, nsteps_ptl_tracking, ntraj_accum, nullptr, ptl_time, o,
                   nullptr))
        die_if_error("particle_tracking_fixed_time_step");
    size_t nspec = (size_t)nt_out * nbins;
    for (size_t k = 0; k < nspec; k++) {
        espectrum[k] += o.espect[k];
        if (bc_flag == 1) espect_escape[k] += o.espect_esc[k];
    }
    int nsdc = rs.estep / kDiffInterval + 1;
    if (traj_diagnose == 0) {
        std::vector<int> rem(nsdc);
        for (int k = 0; k < nsdc; k++) rem[k] = nptl + o.remain[k];
        double* d = o.dsum.data();
        collect_diff_coeffs(mpi_rank, nsdc, d, d + nsdc, d + 2 * nsdc, d + 3 * nsdc, d + 4 * nsdc,
                            d + 5 * nsdc, d + 6 * nsdc, d + 7 * nsdc, (char*)"data/diff_coeffs.dat",
                            rem.data());
    }
}

extern "C" void particle_tracking_multi_steps_openmp(int nptl, double dt, int tid, int sstep,
        int estep, int nbins, int nt_out, int einterval_t, int traj_diagnose, int nsteps_output,
        double pmass, int* ntraj_accum, particles* ptl_init, int* ntraj_diagnostics_points_array,
        particles* ptl, int* nsteps_ptl_tracking, double* espect_private,
        double* espect_escape_private, particles* ptl_time, int* nptl_remain_time, double* drr,
        double* dxx, double* dyy, double* dzz, double* dpp, double* duu, double* daa, double* dee)
{
    (void)pmass;
    RunSpec rs;
    rs.precision = TP_PREC_FP64;
    rs.dt = dt;
    rs.sstep = sstep;
    rs.estep = estep;
    rs.einterval = einterval_t;
    rs.nt_out = nt_out;
    rs.nbins = nbins;
    rs.traj_every = traj_diagnose == 1 ? nsteps_output : 0;
    rs.reset_nsteps = false;
    RunOut o;
    if (!run_range(nptl, rs, ptl_init, ptl, nsteps_ptl_tracking, ntraj_accum,
                   ntraj_diagnostics_points_array, ptl_time, o, nullptr))
        die_if_error("particle_tracking_multi_steps_openmp");
    size_t nspec = (size_t)nt_out * nbins;
    double* ep = espect_private + (size_t)tid * nspec;
    double* eep = espect_escape_private + (size_t)tid * nspec;
    for (size_t k = 0; k < nspec; k++) {
        ep[k] += o.espect[k];
        eep[k] += o.espect_esc[k];
    }
    int nsdc = estep / kDiffInterval + 1;
    double* dst[8] = {drr, dxx, dyy, dzz, dpp, duu, daa, dee};
    for (int c = 0; c < 8; c++)
        for (int k = 0; k < nsdc; k++) dst[c][k] += o.dsum[(size_t)c * nsdc + k];
    for (int k = 0; k < nsdc; k++) nptl_remain_time[k] += o.remain[k];
}

extern "C" void particle_tracking_single_step_openmp(int iptl, int it, double dt, int tid,
        int einterval_t, int traj_diagnose, int nbins, int nt_out, int nsteps_output, double pmass,
        particles* ptl_init, int ntraj_offset_local, int* ntp, particles* ptl, int* iescape_pre,
        int* iescape_after, int* ntraj_diagnostics_points, int* nsteps_ptl_tracking,
        double* espect_private, double* espect_escape_private, particles* ptl_time, double* drr,
        double* dxx, double* dyy, double* dzz, double* dpp, double* duu, double* daa, double* dee)
{
    (void)pmass;
    size_t nspec = (size_t)nbins * nt_out;
    if (*iescape_pre == 0 || bc_flag == 0) {
        if (tp_wirz_steps(1, &ptl[iptl], dt, 1, iescape_after) != 0)
            die_if_error("particle_tracking_single_step_openmp");
        nsteps_ptl_tracking[iptl] += 1;
        if (*iescape_after == 0 && it % kDiffInterval == 0) {
            double o[8];
            if (tp_calc_diff_coeff_batch(1, &ptl_init[iptl], &ptl[iptl], dt, o) != 0)
                die_if_error("particle_tracking_single_step_openmp");
            *drr = o[0]; *dxx = o[1]; *dyy = o[2]; *dzz = o[3];
            *dpp = o[4]; *duu = o[5]; *daa = o[6]; *dee = o[7];
        }
        if (traj_diagnose == 1 && it % nsteps_output == 0) {
            int offset = ntraj_offset_local + (*ntraj_diagnostics_points);
            memcpy(&ptl_time[offset], &ptl[iptl], sizeof(particles));
            (*ntraj_diagnostics_points)++;
        }
    }
    if (*iescape_pre == 0 && *iescape_after == 1 && bc_flag == 1) {
        int bin;
        if (tp_energy_bins(1, &ptl[iptl], nbins, &bin) != 0) die_if_error("single_step");
        espect_escape_private[tid * nspec + (size_t)(*ntp) * nbins + bin] += 1.0;
    }
    if (it % einterval_t == 0) {
        if (*iescape_after == 0) {
            int bin;
            if (tp_energy_bins(1, &ptl[iptl], nbins, &bin) != 0) die_if_error("single_step");
            espect_private[tid * nspec + (size_t)(*ntp) * nbins + bin] += 1.0;
        }
        (*ntp)++;
    }
}

// src/tracking.c:475-493 (sum of the caller's per-thread rows)
extern "C" void gather_particle_spectra_openmp(int num_threads, int nbins, int nt_out,
        double* espectrum, double* espect_private, double* espect_escape,
        double* espect_escape_private)
{
    size_t nspec = (size_t)nbins * nt_out;
    for (int it = 0; it < nt_out; it++)
        for (int j = 0; j < nbins; j++)
            for (int k = 0; k < num_threads; k++) {
                espectrum[it * nbins + j] += espect_private[k * nspec + it * nbins + j];
                if (bc_flag == 1)
                    espect_escape[it * nbins + j] += espect_escape_private[k * nspec + it * nbins + j];
            }
}

int tp_bs_track_hybrid(int mpi_rank, int nptl, double dt, int nbins, int nt_out,
                       particles* ptl_init, int* nsteps_ptl, particles* ptl, double* espectrum,
                       double* espect_escape);

extern "C" void particle_tracking_hybrid(int mpi_rank, int nptl, double dt, int nbins, int nt_out,
        int bc_flag_arg, int nsteps_output, double pmass, int* ntraj_accum, int tracking_method,
        int traj_diagnose, particles* ptl_init, int* nsteps_ptl_tracking, particles* ptl,
        particles* ptl_time)
{
    size_t nspec = (size_t)nt_out * nbins;
    std::vector<double> espectrum(nspec, 0.0), espect_tot(nspec, 0.0), espect_escape(nspec, 0.0);
    struct timeval t1, t2;
    gettimeofday(&t1, nullptr);
    if (tracking_method == 0) {
        particle_tracking_fixed_time_step(mpi_rank, nptl, dt, nbins, nt_out, traj_diagnose,
                nsteps_output, pmass, ntraj_accum, ptl_init, nsteps_ptl_tracking, ptl,
                espectrum.data(), espect_tot.data(), espect_escape.data(), nullptr, nullptr,
                ptl_time);
    } else if (tracking_method == 1) {
        if (tp_bs_track_hybrid(mpi_rank, nptl, dt, nbins, nt_out, ptl_init, nsteps_ptl_tracking,
                               ptl, espectrum.data(), espect_escape.data()) != 0)
            die_if_error("particle_tracking_hybrid (adaptive)");
    }
    gettimeofday(&t2, nullptr);
    if (mpi_rank == 0)
        printf("Elapsed time: %lf s\n", (t2.tv_sec - t1.tv_sec) + 1e-6 * (t2.tv_usec - t1.tv_usec));
    if (traj_diagnose == 0) {
        collect_espectrum(mpi_rank, nbins, nt_out, espectrum.data(), espect_tot.data(),
                          (char*)"data/espectrum.dat");
        if (bc_flag_arg == 1) {
            std::fill(espect_tot.begin(), espect_tot.end(), 0.0);
            collect_espectrum(mpi_rank, nbins, nt_out, espect_escape.data(), espect_tot.data(),
                              (char*)"data/espect_escape.dat");
        }
    }
}
