/*
 * tp_oracle.h -- CPU restatement of the reference's test-particle hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests/, the smoke check and
 * the CPU-baseline leg of bench.py call it to check or time the product; the
 * product library never links, loads or calls it.
 *
 * Every function restates one reference function with the same floating-point
 * operation order (compiled with -ffp-contract=off, glibc libm), so that on the
 * same inputs it reproduces the reference bit for bit; tests/golden pins it
 * against the reference built from its own sources (oracle/build_ref.sh).
 */
#ifndef TP_ORACLE_H
#define TP_ORACLE_H
#include "../include/tp_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_field {
    int system_type;          /* TP_SYS_* */
    double charge_mass;       /* tracking.c global charge_mass */
    int bc_flag;              /* 0 periodic, 1 open, 2 none */
    domain dom;
    grids grd;
    int multi_tframe;
    int interp_corrected;     /* 0: reference corner weights (x/z swap), 1: corrected */
    int ellint_corrected;     /* 0: reference m>=0.9 branch, 1: corrected */
    /* force-free (ABC) */
    double ffA, ffB, ffC, B0, lambda0;
    const vfields_double *vc_d, *va_d, *vb_d;   /* system 2 velocity grid (NULL: E = 0) */
    /* MHD (system 3) */
    const vfields_float *vc_f, *va_f, *vb_f;
    const bfields_float *bc_f, *ba_f, *bb_f;
    /* PIC (system 4) */
    const efields_float *ec_f, *ea_f, *eb_f;
    /* wire-loop current systems (system 1) */
    int nwlcs, iBessel;
    const wlcs *cfg;
    /* turbulent mode sum (system 5) */
    int nmodes;
    const tp_mode *modes;
} or_field;

typedef struct or_spectrum {
    int nbins;
    double emin, emax, logemin, logemax, logde;
} or_spectrum;

void or_spectrum_init(or_spectrum *s, int nbins, double emin, double emax);

void or_get_emf(const or_field *f, double x, double y, double z, double t, emfields *emf);
void or_wirz(const or_field *f, particles *p, double dt);
void or_particle_bc(const or_field *f, particles *p, int *iescape);
void or_ellint(double k, int corrected, double *elle, double *ellk);
void or_trilinear(const or_field *f, double x, double y, double z, double t,
                  long corners[8], double weights[8], double *dt);
int or_energy_bin(const or_spectrum *s, double ux, double uy, double uz);
int or_energy_bin_e(const or_spectrum *s, double ene);  /* bin of an energy gamma - 1 */
void or_calc_diff_coeff(const or_field *f, const particles *p0, const particles *p,
                        double dt, double out8[8]);
void or_mode_sum(const or_field *f, double x, double y, double z, emfields *emf);
/* The synthetic gridded E, B (no reference counterpart: the test workload's
 * field) on the CPU, for the timed CPU baseline: B = B0z z + sum over mb,
 * v = sum over mv, E = -v x B, at node (i, j, k) with phases
 * 2 pi (n . (i/nx, j/ny, k/nz)) + phase, written as float AoS {x, y, z}. */
void or_synth_pic_fields(int nmb, const tp_mode *mb, int nmv, const tp_mode *mv, double B0z,
                         int nx, int ny, int nz, float *e, float *b, int nthreads);

/* One component of a PIC HDF5 field file ([nx][ny][nz] floats, C order) into
 * the x-fastest {x,y,z} float records, scaled: the reference's reorder loop of
 * read_pic_bfields_float_h5 / read_pic_efields_float_h5
 * (src/magnetic_field.c:656-665, src/electric_field.c:474-482), serial. */
void or_pic_records_from_c(const float *data, long nx, long ny, long nz, double scale, int comp, float *rec);

/* Batch helpers for ctypes callers. */
void or_get_emf_batch(const or_field *f, int n, const double *xyzt, double *emf6);
void or_wirz_steps(const or_field *f, int n, particles *p, double dt, int nsteps, int *iescape);
void or_energy_bins(const or_spectrum *s, int n, const particles *p, int *bins);
void or_trilinear_batch(const or_field *f, int n, const double *xyzt, long *corners8, double *weights8);

/* Fixed-step tracking with fused diagnostics, restating
 * particle_tracking_fixed_time_step / _multi_steps_openmp / _single_step_openmp
 * (src/tracking.c:90-190, 297-462).  Outputs:
 *   espect, espect_escape : nt_out*nbins counts (zeroed here)
 *   dsum                  : 8*nsteps_dc sums, component-major (drr,dxx,dyy,dzz,dpp,duu,daa,dee)
 *   remain                : nsteps_dc particle counts
 *   nsteps_ptl            : per-particle pushed-step counters (start at 1)
 * Particles [0, nptl) are processed by nthreads OpenMP threads (0: all);
 * per-thread sums are combined in thread order.  Returns estep, or a negative
 * value on bad input. */
int or_track_fixed(const or_field *f, const or_spectrum *s, int nptl, double dt,
                   int nt_out, const particles *ptl_init, particles *ptl,
                   int *nsteps_ptl, double *espect, double *espect_escape,
                   double *dsum, int *remain, int nthreads);

/* Number of steps and diagnostic intervals exactly as the reference derives them. */
int or_estep(const or_field *f, double dt);

/* Bulirsch-Stoer stepper (src/unused/StepperBS.c), re-entrant restatement:
 * each call owns its controller state.  y = (x, y, z, beta_x, beta_y, beta_z).
 * Performs nsteps accepted steps starting from step size h0; out holds
 * (t, h_did, y[6]) per step.  uform = 0 keeps the reference's derivatives. */
typedef struct or_bs_cfg {
    double atol, rtol;
    int kmaxx;        /* maximum tableau columns, reference KMAXX = 8 */
    int max_rejects;  /* per step, 0 = unlimited */
} or_bs_cfg;
int or_bs_integrate(const or_field *f, const or_bs_cfg *cfg, double *y, double t0,
                    double h0, int nsteps, double *out);
void or_bs_derivs(const or_field *f, double t, const double *y, double *dydx);
long or_bs_run_many(const or_field *f, const or_bs_cfg *cfg, int n, double *y, double h0,
                    int nsteps, int nthreads);

/* Poincare map, src/poincare_map.c */
void or_next_location(const or_field *f, double *fx, double *fy, double *fz, double dstep);
int or_poincare_point(const or_field *f, const double seed[3], int face, double step,
                      double length_max, int ncross, double *xo, double *yo, double *zo);
void or_poincare_many(const or_field *f, int n, const double *seeds, int face, double step,
                      double length_max, int ncross, double *xpos, double *ypos, double *zpos,
                      int *found, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
