/*
 * Pinning harness for the reference build in oracle/_ref (test infrastructure).
 *
 * Links against the reference's own objects (compiled from its sources by
 * oracle/build_ref.sh) and exposes flat entry points that tests and the
 * golden-fixture generator call through ctypes.  It only sets the
 * reference's globals and calls its functions; it computes nothing itself.
 *
 * Reference symbols driven here (paths inside the reference project):
 *   set_variables_tracking / set_ptl_params_tracking   src/tracking.c:53-65
 *   tracking_wirz                                      src/tracking.c:749-892
 *   particle_bc                                        src/tracking.c:1172-1221
 *   particle_tracking_fixed_time_step                  src/tracking.c:90-190
 *   get_emf                                            src/emfields.c:32-60
 *   get_trilinar_parameters                            src/interpolation.c:141-181
 *   ellint / getemf_wlcs                               src/wlcs.c:460-865
 *   ptl_energy_fixed / calc_diff_coeff                 src/diagnostics.c:187-205,659-705
 *   StepperBase / step                                 src/unused/StepperBS.c:103-354
 *   next_location                                      src/poincare_map.c:243-290
 */
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "constants.h"
#include "diagnostics.h"
#include "domain.h"
#include "electric_field.h"
#include "emfields.h"
#include "force_free.h"
#include "interpolation.h"
#include "magnetic_field.h"
#include "particle_info.h"
#include "tracking.h"
#include "velocity_field.h"
#include "wlcs.h"

double refh_ffA = 1.0, refh_ffB = 0.0, refh_ffC = 0.0;

extern struct param_ff param;
extern struct wlcs *config;
extern int nwlcs, iBessel;
extern double emin, emax, logemin, logemax, logde;
extern struct bfields_float *maga_float, *magb_float, *magc_float;
extern struct efields_float *efa_float, *efb_float, *efc_float;
extern struct vfields_double *va_double, *vb_double, *vc_double;
extern struct vfields_float *va_float, *vb_float, *vc_float;
extern double charge_mass;
extern int bc_flag;

void ellint(double k, double *elle, double *ellf);
void refh_orig_collect_diff_coeffs(int mpi_rank, int nsteps_dcoeffs, double *drr,
        double *dxx, double *dyy, double *dzz, double *dpp, double *duu,
        double *daa, double *dee, char *fname, int *nptl_remain);

/* Stepper pieces of src/unused/StepperBS.c (legacy header, n = 6, IMAXX = 9). */
#define REFH_IMAXX 9
void StepperBase(int *nseq, int *cost, double *hnext, int *k_targ,
        double coeff[][REFH_IMAXX], double *errfac, int *ipoint, _Bool densFlag);
void step(double htry, double *hnext0, double *xpre, double *y, double *dydx,
        int k_targ, int *nseq, double table[][6], int *cost,
        double coeff[][REFH_IMAXX], int *ipoint, double *errfac, double *dens,
        _Bool densFlag, double *dydxnew, double ysave[][6], double fsave[][6],
        double *hdid);
void derivs(double t, double *y, double *yderiv);

void refh_set_abc(double a, double b, double c)
{
    refh_ffA = a;
    refh_ffB = b;
    refh_ffC = c;
}

/* Same set-up sequence as get_system_info (src/domain.c:314-409), minus file reads. */
void refh_setup(int stype, double qm, int pbc, const domain *dom,
        const grids *grd, int mt, int vel_dtype)
{
    domain d = *dom;
    grids g = *grd;
    set_variables_emfields(stype);
    set_variables_bfield(&g, &d, 1.0, mt, sizeof(float));
    set_variables_efield(&g, &d, 1.0, mt, sizeof(float));
    set_variables_velocity(&g, &d, 1.0, mt, vel_dtype);
    set_variables_ff(&g, &d);
    set_variabls_interpolation(&g, &d, mt);
    set_variables_tracking(&g, &d, stype, mt);
    set_ptl_params_tracking(pbc, qm);
}

void refh_set_ff(double B0, double lambda0)
{
    param.B0 = B0;
    param.lambda0 = lambda0;
}

void refh_set_wlcs(int n, const struct wlcs *cfg, int ibessel)
{
    static struct wlcs *owned = NULL;
    free(owned);
    owned = (struct wlcs *)malloc(sizeof(struct wlcs) * (n > 0 ? n : 1));
    memcpy(owned, cfg, sizeof(struct wlcs) * n);
    config = owned;
    nwlcs = n;
    iBessel = ibessel;
}

/* Grid pointers: AoS {x,y,z} records, x fastest, as the reference stores them. */
void refh_set_pic_grids(void *ec, void *bc, void *ea, void *eb, void *ba, void *bb)
{
    efc_float = ec; magc_float = bc;
    efa_float = ea; efb_float = eb;
    maga_float = ba; magb_float = bb;
}

void refh_set_velocity(void *vc_d, void *va_d, void *vb_d, void *vc_f)
{
    vc_double = vc_d; va_double = va_d; vb_double = vb_d;
    vc_float = vc_f;
}

/* Same derived quantities as get_spectrum_info (src/diagnostics.c:629-631). */
void refh_set_spectrum(int nbins, double e_min, double e_max)
{
    emin = e_min;
    emax = e_max;
    logemin = log10(emin);
    logemax = log10(emax);
    logde = (logemax - logemin) / (nbins - 2);
}

void refh_get_spectrum_globals(double *out5)
{
    out5[0] = emin; out5[1] = emax; out5[2] = logemin; out5[3] = logemax;
    out5[4] = logde;
}

void refh_get_emf(int n, const double *xyzt, double *emf6)
{
    for (int i = 0; i < n; i++) {
        struct emfields e;
        get_emf(xyzt[4*i], xyzt[4*i+1], xyzt[4*i+2], xyzt[4*i+3], &e);
        emf6[6*i+0] = e.Bx; emf6[6*i+1] = e.By; emf6[6*i+2] = e.Bz;
        emf6[6*i+3] = e.Ex; emf6[6*i+4] = e.Ey; emf6[6*i+5] = e.Ez;
    }
}

void refh_trilinear(int n, const double *xyzt, long *corners8, double *weights8)
{
    for (int i = 0; i < n; i++) {
        double dt;
        get_trilinar_parameters(xyzt[4*i], xyzt[4*i+1], xyzt[4*i+2], xyzt[4*i+3],
                corners8 + 8*i, weights8 + 8*i, &dt);
    }
}

void refh_ellint(int n, const double *k, double *e_out, double *k_out)
{
    for (int i = 0; i < n; i++) ellint(k[i], &e_out[i], &k_out[i]);
}

/* nsteps pushes of each particle: tracking_wirz then particle_bc, the body of
 * particle_tracking_single_step_openmp (src/tracking.c:427-431). */
void refh_wirz_steps(int n, particles *ptl, double dt, int nsteps, int *iescape)
{
    for (int i = 0; i < n; i++) {
        for (int s = 0; s < nsteps; s++) {
            tracking_wirz(&ptl[i], dt);
            particle_bc(&ptl[i], &iescape[i]);
        }
    }
}

void refh_particle_bc(int n, particles *ptl, int *iescape)
{
    for (int i = 0; i < n; i++) particle_bc(&ptl[i], &iescape[i]);
}

void refh_ptl_energy_bins(int n, const particles *ptl, int nbins, int *bins)
{
    double *esp = (double *)calloc((size_t)nbins, sizeof(double));
    for (int i = 0; i < n; i++) {
        memset(esp, 0, sizeof(double) * nbins);
        ptl_energy_fixed(i, 0, 0, (particles *)ptl, nbins, 1,
                (double (*)[nbins])esp);
        bins[i] = -1;
        for (int b = 0; b < nbins; b++) if (esp[b] != 0.0) bins[i] = b;
    }
    free(esp);
}

void refh_calc_diff_coeff(int n, const particles *pinit, const particles *p,
        double dt, double *out8)
{
    for (int i = 0; i < n; i++) {
        double *o = out8 + 8*i;
        calc_diff_coeff((particles *)&pinit[i], (particles *)&p[i], dt,
                &o[0], &o[1], &o[2], &o[3], &o[4], &o[5], &o[6], &o[7]);
    }
}

/* Captured copy of the raw diffusion sums handed to collect_diff_coeffs. */
static double *cap_d = NULL;
static int *cap_remain = NULL;
static int cap_n = 0;

void collect_diff_coeffs(int mpi_rank, int nsteps_dcoeffs, double *drr,
        double *dxx, double *dyy, double *dzz, double *dpp, double *duu,
        double *daa, double *dee, char *fname, int *nptl_remain)
{
    (void)mpi_rank; (void)fname;
    free(cap_d);
    free(cap_remain);
    cap_n = nsteps_dcoeffs;
    cap_d = (double *)malloc(sizeof(double) * 8 * nsteps_dcoeffs);
    cap_remain = (int *)malloc(sizeof(int) * nsteps_dcoeffs);
    double *src[8] = {drr, dxx, dyy, dzz, dpp, duu, daa, dee};
    for (int c = 0; c < 8; c++)
        memcpy(cap_d + (size_t)c * nsteps_dcoeffs, src[c], sizeof(double) * nsteps_dcoeffs);
    memcpy(cap_remain, nptl_remain, sizeof(int) * nsteps_dcoeffs);
}

int refh_captured_dcoeffs(double *out, int *remain, int cap)
{
    int m = cap_n < cap ? cap_n : cap;
    for (int c = 0; c < 8; c++)
        memcpy(out + (size_t)c * m, cap_d + (size_t)c * cap_n, sizeof(double) * m);
    memcpy(remain, cap_remain, sizeof(int) * m);
    return cap_n;
}

/* Whole fixed-step run (src/tracking.c:90-190) with the spectra returned as
 * counts; espect / espect_escape are nt_out*nbins doubles, zeroed here. */
void refh_track_fixed(int nptl, double dt, int nbins, int nt_out,
        particles *ptl_init, particles *ptl, int *nsteps_ptl,
        double *espect, double *espect_escape)
{
    int nth = omp_get_max_threads();
    size_t per = (size_t)nbins * nt_out;
    double *ep = (double *)calloc((size_t)(nth + 1) * per, sizeof(double));
    double *eep = (double *)calloc((size_t)(nth + 1) * per, sizeof(double));
    double *etot = (double *)calloc(per, sizeof(double));
    memset(espect, 0, sizeof(double) * per);
    memset(espect_escape, 0, sizeof(double) * per);
    particle_tracking_fixed_time_step(0, nptl, dt, nbins, nt_out, 0, 1, 1.0,
            NULL, ptl_init, nsteps_ptl, ptl, (double (*)[nbins])espect,
            (double (*)[nbins])etot, (double (*)[nbins])espect_escape,
            (double (*)[nbins * nt_out])ep, (double (*)[nbins * nt_out])eep, NULL);
    free(ep);
    free(eep);
    free(etot);
}

/* The same run with trajectory diagnostics (src/tracking.c:90-190 with
 * traj_diagnose = 1): ptl_time holds each particle's records at
 * ntraj_accum[i-1] (the caller stores the initial state there, as
 * src/diagnostics.c:541-551 does); a record is added every nsteps_output steps. */
void refh_track_traj(int nptl, double dt, int nbins, int nt_out, int nsteps_output,
        int *ntraj_accum, particles *ptl_init, particles *ptl, int *nsteps_ptl,
        particles *ptl_time)
{
    int nth = omp_get_max_threads();
    size_t per = (size_t)nbins * nt_out;
    double *ep = (double *)calloc((size_t)(nth + 1) * per, sizeof(double));
    double *eep = (double *)calloc((size_t)(nth + 1) * per, sizeof(double));
    double *etot = (double *)calloc(per, sizeof(double));
    double *es = (double *)calloc(per, sizeof(double));
    double *ee = (double *)calloc(per, sizeof(double));
    particle_tracking_fixed_time_step(0, nptl, dt, nbins, nt_out, 1, nsteps_output, 1.0,
            ntraj_accum, ptl_init, nsteps_ptl, ptl, (double (*)[nbins])es,
            (double (*)[nbins])etot, (double (*)[nbins])ee,
            (double (*)[nbins * nt_out])ep, (double (*)[nbins * nt_out])eep, ptl_time);
    free(ep);
    free(eep);
    free(etot);
    free(es);
    free(ee);
}

/* Bulirsch-Stoer: nsteps accepted steps of one particle through the
 * reference's step() without dense output.  step() keeps its controller in
 * function-static variables, so a caller pins one particle per fresh process.
 * y = (x, y, z, beta_x, beta_y, beta_z); out receives (t, h_did, y[6]) per step. */
int refh_bs_integrate(double *y, double t0, double h0, int nsteps, double *out)
{
    int nseq[REFH_IMAXX], cost[REFH_IMAXX], ipoint[REFH_IMAXX + 1], k_targ;
    double coeff[REFH_IMAXX][REFH_IMAXX], errfac[2 * REFH_IMAXX + 2];
    double ysave[REFH_IMAXX][6], fsave[REFH_IMAXX * (2 * REFH_IMAXX + 1)][6];
    double table[8][6], dens[(2 * REFH_IMAXX + 5) * 6], dydx[6], dydxnew[6];
    double hnext, x = t0, h = h0, hdid;
    memset(fsave, 0, sizeof(fsave));
    StepperBase(nseq, cost, &hnext, &k_targ, coeff, errfac, ipoint, 0);
    derivs(x, y, dydx);
    for (int s = 0; s < nsteps; s++) {
        hnext = h;
        step(h, &hnext, &x, y, dydx, k_targ, nseq, table, cost, coeff, ipoint,
             errfac, dens, 0, dydxnew, ysave, fsave, &hdid);
        out[8*s] = x;
        out[8*s + 1] = hdid;
        for (int i = 0; i < 6; i++) out[8*s + 2 + i] = y[i];
        h = hnext;
    }
    return 0;
}

void refh_derivs(double t, double *y, double *dydx)
{
    derivs(t, y, dydx);
}

/* ---------------------------------------------------------------- Poincare
 * next_location is the RK4 field-line step of src/poincare_map.c:243-290
 * (not declared in the reference's headers). */
void next_location(double *fx, double *fy, double *fz, double dstep);

/* nsteps reference RK4 steps from each of n seeds; out[n][nsteps][3] */
void refh_next_location(int n, const double *xyz, double step, int nsteps, double *out)
{
    for (int i = 0; i < n; i++) {
        double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        for (int s = 0; s < nsteps; s++) {
            next_location(&x, &y, &z, step);
            double *o = out + ((size_t)i * nsteps + s) * 3;
            o[0] = x; o[1] = y; o[2] = z;
        }
    }
}

/* ---------------------------------------------------------------- field files
 * The reference's binary readers for one time frame of float data
 * (src/magnetic_field.c:442-534, src/electric_field.c:257-349): reads
 * <path>{bx,by,bz}_<ct>.gda scaled by B0 and {ex,ey,ez} by E0 into its own
 * arrays, copied out as nx*ny*nz {x,y,z} float records. */
void refh_read_pic_binary(grids *sgrid, domain *sdomain, char *path, int ct, double b0, double e0,
        float *out_b, float *out_e)
{
    size_t n = (size_t)sgrid->nx * sgrid->ny * sgrid->nz;
    set_variables_bfield(sgrid, sdomain, b0, 0, sizeof(float));
    initialize_bfield();
    read_bfields_binary(path, ct, sizeof(float));
    memcpy(out_b, magc_float, sizeof(float) * 3 * n);
    free_bfield();
    set_variables_efield(sgrid, sdomain, e0, 0, sizeof(float));
    initialize_efield();
    read_efields_binary(path, ct, sizeof(float));
    memcpy(out_e, efc_float, sizeof(float) * 3 * n);
    free_efield();
}
