// host_config.cpp -- host-side pieces of the reference API that the tracking
// library replaces: init.dat parsers (same labels and order), field-array
// set-up, the reference's scalar helpers, and single-rank fallbacks of the
// output writers that the caller's diagnostics.c normally provides.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/tp_gpu.h"

#define TP_LEN_MAX 200  // LEN_MAX, include/constants.h:1-3

extern "C" void tp_internal_fields_released(int which);
// field normalisations, src/magnetic_field.c:38, src/electric_field.c:38, src/velocity_field.c:38
extern "C" double B0, E0, v0;

// ---------------------------------------------------------------- init.dat parsers
static FILE* open_section(const char* fname, const char* label)
{
    FILE* fp = fopen(fname, "r");
    if (!fp) {
        printf("Failed to open %s.\n", fname);
        exit(1);
    }
    char buff[TP_LEN_MAX];
    while (fgets(buff, TP_LEN_MAX, fp) != NULL)
        if (strstr(buff, label) != NULL) break;
    return fp;
}

// src/tracking.c:1226-1255
extern "C" double get_tracking_time_interval(int mpi_rank, char* config_file_name, double pmass)
{
    FILE* fp = open_section(config_file_name, "Tracking method to use");
    double dt = 0.0;
    if (fscanf(fp, "Tracking time step (for electrons): %lf\n", &dt) != 1) {
        printf("Failed to read particle tracking time step.\n");
        exit(1);
    }
    fclose(fp);
    dt *= pmass;
    if (mpi_rank == 0) printf("Particle tracking time step is: %lf\n", dt);
    return dt;
}

// src/force_free.c:99-125
extern "C" void get_param_ff(int mpi_rank, char* config_file_name)
{
    FILE* fp = open_section(config_file_name, "Force-free field");
    if (fscanf(fp, "Normalized B(Gauss):%lf\n", &param.B0) != 1) {
        printf("Failed to read normalized B.\n");
        exit(1);
    }
    if (fscanf(fp, "1/Length scale (lambda):%lf\n", &param.lambda0) != 1) {
        printf("Failed to read length scale lambda.\n");
        exit(1);
    }
    fclose(fp);
    if (mpi_rank == 0) {
        printf("The normalized magnetic field is %lf Gauss\n", param.B0);
        printf("1/Length scale (lambda) is %lf \n", param.lambda0);
    }
}

// src/wlcs.c:53-222: number of systems and the geometry file name from
// init.dat, then one 14-number record per system, iBessel, omega, normI.
extern "C" void read_wlcs(int mpi_rank, char* config_file_name)
{
    FILE* fp = open_section(config_file_name, "Flag for the system to use");
    nwlcs = 1;
    if (fscanf(fp, "Number of WLCSs:%d\n", &nwlcs) != 1) {
        if (mpi_rank == 0) printf("Failed to read the number of WLCSs.\n");
        exit(1);
    }
    if (mpi_rank == 0) printf("Number of wire-loop-current-systems: %d\n", nwlcs);
    char cfname[TP_LEN_MAX];
    strcpy(cfname, "init8_3l.dat");
    if (fscanf(fp, "Configuration file name: %199s\n", cfname) != 1) {
        if (mpi_rank == 0) printf("Failed to read the configuration file name for wlcs.\n");
        exit(1);
    }
    if (mpi_rank == 0) printf("The configuration file name for wlcs: %s\n", cfname);
    fclose(fp);
    if (nwlcs < 1) {
        printf("Failed to read the number of WLCSs.\n");
        exit(1);
    }
    config = (wlcs*)malloc(sizeof(wlcs) * nwlcs);
    fp = fopen(cfname, "r");
    if (!fp) {
        printf("Failed to open %s.\n", cfname);
        exit(1);
    }
    char buff[TP_LEN_MAX];
    if (!fgets(buff, TP_LEN_MAX, fp)) {
        printf("Failed to read wire current.\n");
        exit(1);
    }
    static const char* what[14] = {
        "wire current", "x position of wire current", "the y position of wire current",
        "the z position of wire current", "theta Euler angle of wire current",
        "phi Euler angle of wire current", "t0 of wire current", "the loop current",
        "the radius of the loop current", "the x position of the loop center",
        "the y position of the loop center", "the z position of the loop center",
        "alpha Euler angle of the loop current", "beta Euler angle of the loop current"};
    for (int i = 0; i < nwlcs; i++) {
        double v[14];
        for (int k = 0; k < 14; k++)
            if (fscanf(fp, "%lf", &v[k]) != 1) {
                printf("Failed to read %s.\n", what[k]);
                exit(1);
            }
        wlcs& c = config[i];
        c.cur_wr = v[0]; c.x_wr = v[1]; c.y_wr = v[2]; c.z_wr = v[3];
        c.t0 = v[6]; c.cur_lp = v[7]; c.r_lp = v[8];
        c.x_lp = v[9]; c.y_lp = v[10]; c.z_lp = v[11];
        c.costheta_wr = cos(v[4]); c.sintheta_wr = sin(v[4]);
        c.cosphi_wr = cos(v[5]); c.sinphi_wr = sin(v[5]);
        c.cosalpha_lp = cos(v[12]); c.sinalpha_lp = sin(v[12]);
        c.cosbeta_lp = cos(v[13]); c.sinbeta_lp = sin(v[13]);
    }
    double omega;
    if (fscanf(fp, "%d", &iBessel) != 1) {
        printf("Failed to read iBessel.\n");
        exit(1);
    }
    if (fscanf(fp, "%lf", &omega) != 1) {
        printf("Failed to read omega (frequency of the wire currents).\n");
        exit(1);
    }
    normI = 1.0;
    if (fscanf(fp, "%lf", &normI) != 1) {
        printf("Failed to read normalization current.\n");
        exit(1);
    }
    if (mpi_rank == 0) printf("Normalization current is %10.4e.\n", normI);
    printf("normaI is %f.\n", normI);
    for (int i = 0; i < nwlcs; i++) {
        config[i].omega = omega;
        config[i].cur_wr *= normI;
        config[i].cur_lp *= normI;
    }
    fclose(fp);
    tp_mark_fields_dirty();
}

extern "C" void free_config(void)
{
    free(config);
    config = NULL;
}

// src/wlcs.c:266-269
extern "C" void adjust_dt_normI(double* dt)
{
    if (!config) {
        printf("ERROR: adjust_dt_normI needs a wire-loop configuration (read_wlcs).\n");
        exit(1);
    }
    *dt /= normI;
    *dt /= config[0].omega / 0.001;
}

// ---------------------------------------------------------------- scalar helpers
// src/tracking.c:1084-1140, same arithmetic
extern "C" void cross_product(double beta_x, double beta_y, double beta_z, double Bx, double By,
                              double Bz, double* Cx, double* Cy, double* Cz)
{
    *Cx = beta_y * Bz - beta_z * By;
    *Cy = beta_z * Bx - beta_x * Bz;
    *Cz = beta_x * By - beta_y * Bx;
}

extern "C" double getgamma(double dx, double dy, double dz)
{
    double delta = dx * dx + dy * dy + dz * dz;
    return sqrt(1.0 + delta);
}

extern "C" void getdelta(double* delta_x, double* delta_y, double* delta_z, double beta_x,
                         double beta_y, double beta_z)
{
    double beta_mag = sqrt(beta_x * beta_x + beta_y * beta_y + beta_z * beta_z);
    double gama = 1.0 / sqrt(1.0 - beta_mag * beta_mag);
    *delta_x = gama * beta_x;
    *delta_y = gama * beta_y;
    *delta_z = gama * beta_z;
}

extern "C" double modulus(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

// ---------------------------------------------------------------- field arrays
// The host arrays stay the reference's globals (filled by the caller's
// readers); the library mirrors them on the device at the next GPU call.
static int b_dtype = 4, e_dtype = 4, v_dtype = 4;

extern "C" void set_variables_bfield(grids* sgrid, domain* sdomain, double B0_field, int mt,
                                     int dtype)
{
    memcpy(&simul_grid, sgrid, sizeof(grids));
    memcpy(&simul_domain, sdomain, sizeof(domain));
    B0 = B0_field;
    multi_tframe = mt;
    data_type = b_dtype = dtype;
}

extern "C" void set_variables_efield(grids* sgrid, domain* sdomain, double E0_field, int mt,
                                     int dtype)
{
    memcpy(&simul_grid, sgrid, sizeof(grids));
    memcpy(&simul_domain, sdomain, sizeof(domain));
    E0 = E0_field;
    multi_tframe = mt;
    data_type = e_dtype = dtype;
}

extern "C" void set_variables_velocity(grids* sgrid, domain* sdomain, double v0_field, int mt,
                                       int dtype)
{
    memcpy(&simul_grid, sgrid, sizeof(grids));
    memcpy(&simul_domain, sdomain, sizeof(domain));
    v0 = v0_field;
    multi_tframe = mt;
    data_type = v_dtype = dtype;
}

static size_t n3() { return (size_t)simul_grid.nx * simul_grid.ny * simul_grid.nz; }

// src/magnetic_field.c:68-116 and the electric / velocity counterparts
#define TP_ALLOC_FIELD(dtype, T_F, T_D, a_f, b_f, c_f, a_d, b_d, c_d)        \
    do {                                                                      \
        if (dtype == (int)sizeof(float)) {                                    \
            if (multi_tframe == 1) {                                          \
                a_f = (T_F*)malloc(sizeof(T_F) * n3());                       \
                b_f = (T_F*)malloc(sizeof(T_F) * n3());                       \
            } else {                                                          \
                c_f = (T_F*)malloc(sizeof(T_F) * n3());                       \
            }                                                                 \
        } else if (dtype == (int)sizeof(double)) {                            \
            if (multi_tframe == 1) {                                          \
                a_d = (T_D*)malloc(sizeof(T_D) * n3());                       \
                b_d = (T_D*)malloc(sizeof(T_D) * n3());                       \
            } else {                                                          \
                c_d = (T_D*)malloc(sizeof(T_D) * n3());                       \
            }                                                                 \
        } else {                                                              \
            printf("ERROR: wrong data type\n");                               \
            exit(1);                                                          \
        }                                                                     \
        tp_mark_fields_dirty();                                               \
    } while (0)

extern "C" void initialize_bfield(void)
{
    TP_ALLOC_FIELD(b_dtype, bfields_float, bfields_double, maga_float, magb_float, magc_float,
                   maga_double, magb_double, magc_double);
}

extern "C" void initialize_efield(void)
{
    TP_ALLOC_FIELD(e_dtype, efields_float, efields_double, efa_float, efb_float, efc_float,
                   efa_double, efb_double, efc_double);
}

extern "C" void initialize_vfield(void)
{
    TP_ALLOC_FIELD(v_dtype, vfields_float, vfields_double, va_float, vb_float, vc_float,
                   va_double, vb_double, vc_double);
}

#define TP_FREE(p) do { free(p); p = NULL; } while (0)

extern "C" void free_bfield(void)
{
    TP_FREE(maga_float); TP_FREE(magb_float); TP_FREE(magc_float);
    TP_FREE(maga_double); TP_FREE(magb_double); TP_FREE(magc_double);
    tp_internal_fields_released(0);
}

extern "C" void free_efield(void)
{
    TP_FREE(efa_float); TP_FREE(efb_float); TP_FREE(efc_float);
    TP_FREE(efa_double); TP_FREE(efb_double); TP_FREE(efc_double);
    tp_internal_fields_released(1);
}

extern "C" void free_vfield(void)
{
    TP_FREE(va_float); TP_FREE(vb_float); TP_FREE(vc_float);
    TP_FREE(va_double); TP_FREE(vb_double); TP_FREE(vc_double);
    tp_internal_fields_released(2);
}

// ---------------------------------------------------------------- output writers
// Single-rank fallbacks of collect_espectrum / collect_diff_coeffs
// (src/diagnostics.c:221-248, 723-782), same file formats.  A caller that
// links the reference's diagnostics.c overrides them (and reduces over MPI).
extern "C" __attribute__((weak)) void collect_espectrum(int mpi_rank, int nbins, int nt_out,
        double* espectrum, double* espect_tot, char* fname)
{
    double* einterval = (double*)malloc(sizeof(double) * nbins);
    einterval[0] = emin;
    for (int i = 1; i < nbins - 1; i++)
        einterval[i] = pow(10, logemin) * (pow(10, logde * i) - pow(10, logde * (i - 1)));
    einterval[nbins - 1] = pow(10, logemin) * (pow(10, logde * nbins) - pow(10, logde * (nbins - 1)));
    memcpy(espect_tot, espectrum, sizeof(double) * nbins * nt_out);
    if (mpi_rank == 0) {
        FILE* fp = fopen(fname, "a");
        if (!fp) {
            printf("Failed to open %s.\n", fname);
            exit(1);
        }
        for (int i = 0; i < nt_out; i++) {
            for (int j = 0; j < nbins; j++) {
                espectrum[i * nbins + j] = espect_tot[i * nbins + j] / einterval[j];
                fprintf(fp, "%10.4e ", espectrum[i * nbins + j]);
            }
            fprintf(fp, "\n");
        }
        fclose(fp);
    }
    free(einterval);
}

extern "C" __attribute__((weak)) void collect_diff_coeffs(int mpi_rank, int nsteps_dcoeffs,
        double* drr, double* dxx, double* dyy, double* dzz, double* dpp, double* duu,
        double* daa, double* dee, char* fname, int* nptl_remain)
{
    if (mpi_rank != 0) return;
    FILE* fp = fopen(fname, "w");
    if (!fp) {
        printf("Failed to open %s.\n", fname);
        exit(1);
    }
    fprintf(fp, "drr        dxx        dyy        dzz        dpp");
    fprintf(fp, "        duu        daa        dee        nptl\n");
    for (int i = 0; i < nsteps_dcoeffs; i++)
        fprintf(fp, "%10.4e %10.4e %10.4e %10.4e %10.4e %10.4e %10.4e %10.4e %d\n", drr[i], dxx[i],
                dyy[i], dzz[i], dpp[i], duu[i], daa[i], dee[i], nptl_remain[i]);
    fclose(fp);
}
