/*
 * tp_gpu.h -- C ABI of libtpgpu.so, the GB300 (sm_103a) test-particle tracer.
 *
 * Part 1 re-exports, with the same names and signatures, the entry points of
 * the reference C API on the tracking hot path, so that the reference's own
 * callers (main.c, test_particle.c, domain.c, diagnostics.c, ...) link
 * against this library instead of tracking.o / emfields.o / interpolation.o /
 * force_free.o / wlcs.o and the field modules.  Every compute entry point runs
 * on the GPU; there is no CPU path.  Errors follow the reference: a message on
 * stdout and exit(1); tp_last_status()/tp_last_error() report the cause.
 *
 * Part 2 is this library's own API (tp_*): device-resident sessions, batch
 * utilities and the precision / mode switches used by the tests and benchmark.
 *
 * Reference locations are paths inside the reference project.
 */
#ifndef TP_GPU_H
#define TP_GPU_H
#include "tp_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ======================================================================
 * Part 1: reference-compatible entry points
 * ==================================================================== */

/* --- tracking (include/tracking.h:22-85, src/tracking.c) --- */
/* src/tracking.c:53-59 */
void set_variables_tracking(grids *sgrid, domain *sdomain, int stype, int mt);
/* src/tracking.c:61-65 */
void set_ptl_params_tracking(int pbc, double qm);
/* src/tracking.c:659-699: fixed-step tracking of all particles on the GPU; appends
 * nt_out spectra to data/espectrum.dat (and data/espect_escape.dat when bc_flag
 * is 1) and writes data/diff_coeffs.dat through collect_espectrum /
 * collect_diff_coeffs, which the caller's diagnostics.c provides.
 * tracking_method 1 runs the adaptive Bulirsch-Stoer stepper (the reference's
 * adaptive branch, src/tracking.c:681-684, is commented out). */
void particle_tracking_hybrid(int mpi_rank, int nptl, double dt, int nbins,
        int nt_out, int bc_flag, int nsteps_output, double pmass,
        int *ntraj_accum, int tracking_method, int traj_diagnose,
        particles *ptl_init, int *nsteps_ptl_tracking, particles *ptl,
        particles *ptl_time);
/* src/tracking.c:90-190.  The spectrum arguments are the reference's
 * double[nt_out][nbins] / double[threads+1][nbins*nt_out] arrays. */
void particle_tracking_fixed_time_step(int mpi_rank, int nptl, double dt,
        int nbins, int nt_out, int traj_diagnose, int nsteps_output, double pmass,
        int *ntraj_accum, particles *ptl_init, int *nsteps_ptl_tracking, particles *ptl,
        double *espectrum, double *espect_tot, double *espect_escape,
        double *espect_private, double *espect_escape_private, particles *ptl_time);
/* src/tracking.c:297-374: steps sstep..estep of all particles; spectra go to
 * row tid of espect_private, diffusion sums are added to drr..dee. */
void particle_tracking_multi_steps_openmp(int nptl, double dt, int tid, int sstep,
        int estep, int nbins, int nt_out, int einterval_t, int traj_diagnose,
        int nsteps_output, double pmass, int *ntraj_accum, particles *ptl_init,
        int *ntraj_diagnostics_points_array, particles *ptl,
        int *nsteps_ptl_tracking, double *espect_private,
        double *espect_escape_private, particles *ptl_time,
        int *nptl_remain_time, double *drr, double *dxx, double *dyy, double *dzz,
        double *dpp, double *duu, double *daa, double *dee);
/* src/tracking.c:416-462: one step of one particle */
void particle_tracking_single_step_openmp(int iptl, int it, double dt, int tid,
        int einterval_t, int traj_diagnose, int nbins, int nt_out, int nsteps_output,
        double pmass, particles *ptl_init, int ntraj_offset_local, int *ntp, particles *ptl,
        int *iescape_pre, int *iescape_after, int *ntraj_diagnostics_points,
        int *nsteps_ptl_tracking, double *espect_private,
        double *espect_escape_private, particles *ptl_time,
        double *drr, double *dxx, double *dyy, double *dzz, double *dpp,
        double *duu, double *daa, double *dee);
/* src/tracking.c:475-493 */
void gather_particle_spectra_openmp(int num_threads, int nbins, int nt_out,
        double *espectrum, double *espect_private,
        double *espect_escape, double *espect_escape_private);
/* src/tracking.c:749-892: one Wirz push of one particle */
void tracking_wirz(struct particles *ptl, double dt);
/* src/tracking.c:1172-1221 */
void particle_bc(particles *ptl, int *iescape);
/* src/tracking.c:1226-1255: parses init.dat */
double get_tracking_time_interval(int mpi_rank, char *config_file_name, double pmass);
/* src/tracking.c:1084-1140: scalar helpers of the reference API */
void cross_product(double beta_x, double beta_y, double beta_z, double Bx,
        double By, double Bz, double *Cx, double *Cy, double *Cz);
double getgamma(double dx, double dy, double dz);
void getdelta(double *delta_x, double *delta_y, double *delta_z,
        double beta_x, double beta_y, double beta_z);
double modulus(double x, double y, double z);

/* --- fields (include/emfields.h:28-40, src/emfields.c) --- */
void get_emf(double x, double y, double z, double t, struct emfields *emf);            /* :32-60 */
void get_magnetic_field(double x, double y, double z, double t, struct emfields *emf); /* :76-96 */
void set_variables_emfields(int stype);                                                 /* :196-199 */
void getemf_test(double x, double y, double z, double t, struct emfields *emf);        /* :210-218 */
void getemf_mhd_test_particle(double x, double y, double z, double t, struct emfields *emf); /* :107-120 */
void getemf_pic_test_particle(double x, double y, double z, double t, struct emfields *emf); /* :153-166 */
void get_bfield_mhd_test_particle(double x, double y, double z, double t, struct emfields *emf); /* :131-142 */
void get_bfield_pic_test_particle(double x, double y, double z, double t, struct emfields *emf); /* :177-188 */

/* --- interpolation (include/interpolation.h:3-10, src/interpolation.c) --- */
void set_variabls_interpolation(grids *sgrid, domain *sdomain, int mt);                /* :16-21 */
void grid_indices(double x, double y, double z, double t, int *ix1, int *iy1,
        int *iz1, int *it1, int *ix2, int *iy2, int *iz2, int *it2,
        double *dx, double *dy, double *dz, double *dt);                               /* :36-105 */
void get_trilinar_parameters(double x, double y, double z, double t,
        long int *corners, double *weights, double *dt);                               /* :141-181 */

/* --- force-free field (include/force_free.h, src/force_free.c) --- */
void getb_ff(double x, double y, double z, double t, struct bfields *bmf);             /* :138-150 */
void gete_ff(double x, double y, double z, double t, struct bfields *bmf, struct efields *elf); /* :78-86 */
void getemf_ff(double x, double y, double z, double t, struct emfields *emf);          /* :54-66 */
void get_param_ff(int mpi_rank, char *config_file_name);                               /* :99-125 */
void set_variables_ff(grids *sgrid, domain *sdomain);                                  /* :38-42 */

/* --- wire-loop current systems (include/wlcs.h, src/wlcs.c) --- */
void read_wlcs(int mpi_rank, char *config_file_name);                                  /* :53-222 */
void getemf_wlcs(double x, double y, double z, double t, struct emfields *emf_tot);    /* :814-865 */
void free_config(void);                                                                /* :227-229 */
void adjust_dt_normI(double *dt);                                                      /* :266-269 */

/* --- Poincare map (include/poincare_map.h, src/poincare_map.c) --- */
/* src/poincare_map.c:39-239: reads the "Poincare map configuration" section,
 * traces this rank's seeds on the GPU and writes the crossings through
 * tp_poincare_save (Part 2). */
int poincare_map(int mpi_rank, int mpi_size, char *config_file_name, domain *sdomain);
extern int map_for_single_point, face_cross_section, nhorizontal, nvertical, ncross;
extern double fx0, fy0, fz0, min_horizontal, max_horizontal, min_vertical, max_vertical;
extern double step_fieldline, fieldline_length_max;

/* --- gridded fields (include/{magnetic,electric,velocity}_field.h) --- */
void set_variables_bfield(grids *sgrid, domain *sdomain, double B0_field, int mt, int dtype); /* magnetic_field.c:55-63 */
void initialize_bfield(void);                                                          /* magnetic_field.c:102-116 */
void free_bfield(void);                                                                /* magnetic_field.c:144-158 */
void get_double_bfield_at_point(double x, double y, double z, double t,
        double *bx, double *by, double *bz);                                           /* magnetic_field.c:555-584 */
void get_float_bfield_at_point(double x, double y, double z, double t,
        float *bx, float *by, float *bz);                                              /* magnetic_field.c:593-622 */
void set_variables_efield(grids *sgrid, domain *sdomain, double E0_field, int mt, int dtype); /* electric_field.c:55-63 */
void initialize_efield(void);
void free_efield(void);
void get_double_efield_at_point(double x, double y, double z, double t,
        double *ex, double *ey, double *ez);                                           /* electric_field.c:370-399 */
void get_float_efield_at_point(double x, double y, double z, double t,
        float *ex, float *ey, float *ez);                                              /* electric_field.c:408-437 */
void set_variables_velocity(grids *sgrid, domain *sdomain, double v0_field, int mt, int dtype); /* velocity_field.c:55-66 */
void initialize_vfield(void);
void free_vfield(void);
void get_double_velocity_at_point(double x, double y, double z, double t,
        double *vx, double *vy, double *vz);                                           /* velocity_field.c:555-584 */
void get_float_velocity_at_point(double x, double y, double z, double t,
        float *vx, float *vy, float *vz);                                              /* velocity_field.c:593-622 */

/* Reference globals kept under their reference names (src/tracking.c:35-40,
 * src/emfields.c:16, src/force_free.c:31-33, src/wlcs.c:27-29,
 * src/magnetic_field.c:31-39, src/electric_field.c:31-39,
 * src/velocity_field.c:31-39).  The host grid arrays stay owned by the caller
 * side exactly as in the reference; the library mirrors them on the device. */
extern grids simul_grid;
extern domain simul_domain;
extern int system_type, multi_tframe, bc_flag, data_type;
extern double charge_mass;
extern param_ff param;
extern wlcs *config;
extern int nwlcs, iBessel;
extern double normI;
extern bfields_float *maga_float, *magb_float, *magc_float;
extern bfields_double *maga_double, *magb_double, *magc_double;
extern efields_float *efa_float, *efb_float, *efc_float;
extern efields_double *efa_double, *efb_double, *efc_double;
extern vfields_float *va_float, *vb_float, *vc_float;
extern vfields_double *va_double, *vb_double, *vc_double;
/* Spectrum globals of src/diagnostics.c:32 (set by get_spectrum_info). */
extern double emin, emax, logemin, logemax, logde;

/* ======================================================================
 * Part 2: library API
 * ==================================================================== */

enum {
    TP_PREC_FP64 = 0,       /* reference arithmetic (no FMA contraction): parity path */
    TP_PREC_FP64_FAST = 1,  /* FP64 with FMA contraction */
    TP_PREC_MIXED = 2,      /* FP32 push and field, 64-bit fixed-point positions */
    TP_PREC_SURROGATE = 3   /* as MIXED with the learned field model (mode-sum field) */
};

int tp_init(int device);              /* select the GPU; implicit on first use */
int tp_last_status(void);             /* 0 = ok; sticky until tp_clear_status() */
const char *tp_last_error(void);
void tp_clear_status(void);
int tp_device_status(void);           /* status bits raised by kernels since the last call (read and cleared) */
/* Device status bits: 1 a gather index outside the grid, 2 a non-finite
 * field or state, 4 an adaptive step or reject limit reached, 8 a step size
 * underflow, 16 a bounded wait of the tensor-core pipeline ran out. */

/* Reference compile-time choices made run-time switches. */
void tp_set_abc(double A, double B, double C);   /* include/force_free.h:21-26 */
void tp_set_interp_corrected(int on);            /* x/z weight swap of src/interpolation.c:173-180 */
void tp_set_ellint_corrected(int on);            /* m >= 0.9 branch of src/wlcs.c:741-804 */
/* Turbulent plane-wave mode sum (system type TP_SYS_MODESUM), B = B0 z + sum. */
int tp_set_modes(int nmodes, const tp_mode *modes, double B0);
/* Spectrum binning (src/diagnostics.c:588-640 without the file): sets
 * emin, emax, logemin, logemax, logde. */
void tp_set_spectrum(int nbins, double e_min, double e_max);
/* Mark the host grid arrays changed after their last upload. */
void tp_mark_fields_dirty(void);

/* Batch utilities, all on the GPU.  xyzt: n*4 doubles; particles: AoS records. */
int tp_get_emf_batch(int n, const double *xyzt, double *emf6);
/* The mixed-precision path's FP32 field (system types 0, 2, 4, 5) at n points
 * (xyz: n*3 doubles, turned into 64-bit fixed point as the tracking kernel
 * does), written as n*6 floats in emfields order (Bx, By, Bz, Ex, Ey, Ez). */
int tp_get_emf_mixed_batch(int n, const double *xyz, float *emf6);
int tp_wirz_steps(int n, particles *ptl, double dt, int nsteps, int *iescape);
int tp_energy_bins(int n, const particles *ptl, int nbins, int *bins);
int tp_calc_diff_coeff_batch(int n, const particles *ptl_init, const particles *ptl,
                             double dt, double *out8);
int tp_trilinear_batch(int n, const double *xyzt, long *corners8, double *weights8);
int tp_energy_thresholds(int nbins, double *thr);  /* nbins-1 exact bin edges */

/* Device-resident tracking sessions. */
typedef struct tp_session tp_session;
typedef struct tp_run_info {
    int estep, einterval, nsdc, nt_out, nbins;
    int grid, blocks_per_sm;
    double kernel_ms;          /* device time of the tracking kernel, CUDA events */
    double pushes;             /* particle pushes performed */
    double step_ms;            /* device time of the whole run incl. resets and reductions */
    int launches;              /* kernels this library launched for the run */
} tp_run_info;
tp_session *tp_session_create(int nptl);
void tp_session_destroy(tp_session *s);
int tp_session_load(tp_session *s, const particles *ptl_init, const particles *ptl);
int tp_session_track(tp_session *s, int precision, double dt, int nt_out, int nbins,
                     tp_run_info *info);
int tp_session_fetch(tp_session *s, particles *ptl, int *nsteps_ptl,
                     double *espect, double *espect_escape, double *dsum, int *remain);

/* Synthetic gridded fields (system type TP_SYS_PIC) generated on the GPU:
 * B = B0z z + sum of modes_b, v = sum of modes_v, E = -v x B at every node of
 * simul_grid, node (i,j,k) at phase 2 pi (n . (i/nx, j/ny, k/nz)) + phase.
 * The device copies become authoritative; host_e / host_b (n*3 floats each,
 * may be NULL) receive the same arrays.  tp_release_device_fields() returns
 * to uploading the host arrays. */
int tp_synth_pic_fields(int nmodes_b, const tp_mode *modes_b, int nmodes_v,
                        const tp_mode *modes_v, double B0z, float *host_e, float *host_b);
void tp_release_device_fields(void);

/* Adaptive Bulirsch-Stoer (src/unused/StepperBS.c) for the wire-loop field
 * (system type 1), batched on the GPU.  y: n * 6 doubles, (x, y, z, beta)
 * for uform 0 (the reference's equations, positions in L0, c0/L0 scaling)
 * or (x, y, z, u = gamma v) for uform 1 (c = 1).
 * tp_bs_steps: exactly nsteps accepted steps from t0 with first step h0;
 * rec receives (t, h, y[6]) per particle and step (n * nsteps * 8).
 * tp_bs_run: from t[i] to t_end with step sizes clipped to land on the
 * nt_out frame times, where the energy spectrum (nt_out * nbins counts) and
 * the diffusion sums (dframe: (nt_out + 1) * 8, row f + 1 = frame f) are
 * taken; steps_out / status_out per particle (status: TP step limit 4,
 * step-size underflow 8, non-finite state 2). */
int tp_bs_steps(int n, double *y, double t0, double h0, int nsteps, double atol,
                double rtol, int kmaxx, int uform, double *rec);
int tp_bs_run(int n, double *y, double *t, double t_end, int nt_out, int nbins,
              double h0, double atol, double rtol, int kmaxx, int uform, int max_steps,
              int *steps_out, int *status_out, double *espect, double *dframe,
              tp_run_info *info);

/* Learned field model (no reference counterpart): 64 integer-lattice Fourier
 * features of the box position, then 128 -> 256 -> 256 -> 256 -> 256 -> 6
 * with SiLU, BF16 tensor-core GEMMs with FP32 accumulation, trained with
 * AdamW on samples of the current plane-wave mode table (tp_set_modes).
 * Parameters are one flat FP32 array W0, b0, ..., W4, b4 (W_l [out][in]).
 * Positions u are box fractions in 32-bit fixed point (u * 2^32). */
int tp_mlp_param_count(void);
int tp_mlp_init(const int *freq /* 64 x 3 */, const float *weights /* NULL: seeded init */,
                unsigned long long seed);
int tp_mlp_set_output_norm(const float *mean6, const float *std6);
int tp_mlp_get_weights(float *weights);
int tp_mlp_grad(int n, const unsigned int *u, const float *t, double *loss, float *y,
                float *grads);
int tp_mlp_train(long long nsamples, int batch, int epochs, double lr, double wd,
                 unsigned long long seed, double *loss_out, double *ms_out);
int tp_mlp_eval(int n, const unsigned int *u, float *out6);
/* Same, through the block-wide evaluation the tracking kernel uses. */
int tp_mlp_eval_kernel(int n, const unsigned int *u, float *out6);
/* Polls before a hand-over wait of the tensor-core pipeline (learned field)
 * gives up; 0 restores the default (about 4 million).  A wait that runs out
 * sets status bit 16 (see tp_device_status), every other wait of the block then
 * returns at once, the block writes no particle results, drains its MMAs and
 * copies and frees its tensor memory.  For tests of that path. */
int tp_set_wait_limit(unsigned int polls);

/* One 128-row tile of D = A * B^T on the tensor cores (tcgen05.mma, BF16
 * operands given as raw 16-bit patterns, FP32 result): A[128][k], B[n][k],
 * D[128][n]; n a multiple of 16 in [16, 256], k a multiple of 64 in
 * [64, 256].  A self-check of the tensor-core path of the learned field model. */
int tp_tc_gemm_bf16(int n, int k, const unsigned short *a, const unsigned short *b, float *d);
/* D = A * B^T through the learned field model's training GEMM kernel
 * (tcgen05.mma over a ring of k-atoms, FP32 accumulation in tensor memory):
 * A[m][k], B[n][k] raw BF16, D[m][n] FP32; m a multiple of 128, n a multiple
 * of 16 in [16, 256], k a multiple of 64.  A self-check of the training path. */
int tp_tc_gemm_train_bf16(int m, int n, int k, const unsigned short *a, const unsigned short *b, float *d);

/* FMA-chain microbenchmark of a CUDA-core pipe: kind 0 FP32, 1 FP64, 2 packed
 * FP32 pairs (fma.rn.f32x2); *flops = floating-point operations per second
 * (a multiply-add counts 2), every SM busy, at the clock of the moment.  The
 * denominators of the compute-bound paths' rooflines. */
int tp_measure_fma_peak(int kind, double *flops);

/* Field lines of the gridded B (system types 3 and 4) from n seeds [n][3],
 * RK4 steps of length `step` on the unit vector of B, up to length_max in
 * all; xpos/ypos/zpos [n][ncross + 1] get the seed and the first ncross
 * crossings of the plane pos[face] = seed[face] (unreached entries: 2 * the
 * box maximum of the axis); found[n] the crossings reached.  The tracing of
 * src/poincare_map.c:101-181 for a batch of seeds. */
int tp_poincare_trace(int n, const double *seeds, int face, double step, double length_max, int ncross,
                      double *xpos, double *ypos, double *zpos, int *found);
/* Writer used by poincare_map (weak; the default writes the reference's
 * data/poincare_map.h5 through tp_h5_write_poincare, tp_h5.h). */
void tp_poincare_save(int mpi_rank, int mpi_size, int npoints_total, int ncross, int nshift,
                      int npoints, const double *xpos, const double *ypos, const double *zpos);

/* PIC-style fields (system type 4) of the current grid from the reference's
 * binary files <filepath>{bx,by,bz,ex,ey,ez}_<ct>.gda (nx*ny*nz FP32 each,
 * x fastest), scaled by B0 and E0 as read_bfields_binary /
 * read_efields_binary do (src/magnetic_field.c:442-534,
 * src/electric_field.c:257-349, one time frame), straight into device memory;
 * the host arrays magc_float / efc_float are not filled.  tp_mark_fields_dirty
 * or tp_release_device_fields return to the host arrays. */
int tp_read_pic_fields_binary(const char *filepath, int ct);
/* Copies device-resident PIC-style fields (tp_read_pic_fields_binary,
 * tp_synth_pic_fields) to host arrays of nx*ny*nz {x,y,z} float records. */
int tp_fetch_device_fields(float *host_e, float *host_b);

/* Open boundaries (bc_flag 1): fixed-step runs go in segments of `steps`
 * steps (rounded up to a multiple of the 100-step diffusion interval) and the
 * particles that left the box are dropped from the launches that follow, their
 * remaining diagnostic contributions (the last diffusion singles the reference
 * keeps adding, src/tracking.c:334-368, and the departure counts) added in
 * closed form.  0: one launch for the whole run; -1 (default): segments only
 * when the particles' tiles take more than one wave of the launch, about 8
 * for the mixed path and 32 for the FP64 paths.  Results are unchanged (the
 * mixed path carries its fixed-point state across); only the order of the
 * FP64 diffusion sums changes.  Runs with trajectory diagnostics or the
 * learned field, and runs that start after step 1, use one launch. */
void tp_set_compaction(int steps);

/* One call, host buffers in and out (reuses a cached session). */
int tp_track_host(int precision, int nptl, double dt, int nt_out, int nbins,
                  const particles *ptl_init, particles *ptl, int *nsteps_ptl,
                  double *espect, double *espect_escape, double *dsum, int *remain,
                  tp_run_info *info);

/* ---- Part 3: tracking without device allocation --------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory (a host framework whose allocator owns every device allocation of
 * the process, an embedded or real-time host that forbids allocation after
 * start-up): the caller passes every input and output as device memory; the
 * library uses only a 4 MiB file-scope device array for its scratch and calls
 * no allocating routine.  The first call on each device looks up that
 * array's address with the device current.  Calls on the same device share
 * the scratch: calls that overlap on the GPU race on it, so serialise them,
 * also across host threads; calls on different devices are independent.
 * Runs the mixed-precision tracking kernel (TP_PREC_MIXED) over steps
 * 1..estep, system type 2 (ABC field from abc, B0, lambda0) or 4
 * (node-interleaved grid), in one launch also with open boundaries (it does
 * not compact departed particles; the results equal the session's either
 * way).  The return value is 0 on success, else one of TP_NOALLOC_*; it does
 * not wait for the kernels.  Kernel-side conditions (device status bits as
 * for tp_device_status, e.g. 2 for a non-finite momentum) are reported in
 * *d_status when the caller passes one. */
enum {
    TP_NOALLOC_EINVAL = 1,   /* bad argument (pointer, size, range)           */
    TP_NOALLOC_ETOOBIG = 2,  /* estep / 100 + 1 partial-sum rows do not fit   */
    TP_NOALLOC_ECUDA = 3     /* a CUDA call failed                             */
};

typedef struct tp_noalloc_args {
    int n;                 /* particles, >= 1                                  */
    int system_type;       /* TP_SYS_FORCEFREE or TP_SYS_PIC                   */
    int estep;             /* last step (steps 1..estep)                       */
    int nt_out;            /* diagnostic frames; einterval = estep / nt_out    */
    int nbins;             /* energy bins, 3..4096                             */
    int bc_flag;           /* 0 periodic, 1 open                               */
    int interp_corrected;  /* 0: the reference's trilinear weights             */
    int nx, ny, nz;        /* grid nodes (system 4), >= 2 each                 */
    double dt, charge_mass, emin, emax;
    double lo[3], hi[3];   /* box (xmin, ymin, zmin), (xmax, ymax, zmax)       */
    double abc[3], B0, lambda0;  /* ABC field (system 2)                       */
    const float *d_grid;   /* system 4: per node {Ex,Ey,Ez,Bx,By,Bz,0,0},
                              x fastest, 32-byte aligned (one load per node)  */
    double *d_state;       /* in/out, 11 * n: the particles fields as columns
                              (x, y, z, qm, ux, uy, uz, t, xs, ys, zs)        */
    const double *d_state0;  /* 11 * n: the initial particles, same columns   */
    int *d_nsteps;         /* out, n: steps taken                              */
    unsigned int *d_espect;         /* out, nt_out * nbins counts              */
    unsigned int *d_espect_escape;  /* out, nt_out * nbins counts              */
    double *d_dsum;        /* out, 8 rows (drr, dxx, dyy, dzz, dpp, duu, daa,
                              dee) of estep / 100 + 1 diffusion sums          */
    int *d_remain;         /* out, estep / 100 + 1 particles remaining         */
    void *stream;          /* cudaStream_t, or NULL for the default stream    */
    int *d_status;         /* optional out (device int): the kernel's status
                              bits, cleared by the call; NULL: not reported   */
} tp_noalloc_args;

int tp_track_mixed_noalloc(const tp_noalloc_args *args);

#ifdef __cplusplus
}
#endif
#endif /* TP_GPU_H */
