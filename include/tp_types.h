/*
 * tp_types.h -- data types of the test-particle tracing path, layout-identical
 * to the reference C API so that its callers link against this library
 * unchanged.  Each block uses the reference header's own include guard, so a
 * translation unit may include this file together with the reference headers.
 *
 *   particles  include/particle_info.h:6-12   (88-byte AoS record)
 *   domain     include/domain.h:5-14
 *   grids      include/domain.h:19-24
 *   emfields   include/emfields.h:7-10
 *   bfields/efields include/emfields.h:12-26
 *   wlcs       include/wlcs.h:24-34
 *   param_ff   include/force_free.h:29-34
 *   {b,e,v}fields_{float,double} include/magnetic_field.h:1-13,
 *              include/electric_field.h:1-14, include/velocity_field.h:1-14
 */
#ifndef TP_TYPES_H
#define TP_TYPES_H

#ifndef PARTICLES_H
#define PARTICLES_H
typedef struct particles {
    double x, y, z, qm;
    double ux, uy, uz, t; /* u = gamma * v (c = 1) */
    double xshift, yshift, zshift; /* accumulated periodic shifts */
} particles;
#endif

#ifndef DOMAIN_H
#define DOMAIN_H
typedef struct domain {
    double xmin_ptl, xmax_ptl;
    double ymin_ptl, ymax_ptl;
    double zmin_ptl, zmax_ptl;
    double xmin, xmax;
    double ymin, ymax;
    double zmin, zmax;
    double tmin, tmax;
} domain;
#endif

#ifndef GRIDS_H
#define GRIDS_H
typedef struct grids {
    int nx, ny, nz, nt;
    double dx, dy, dz, dt;
} grids;
#endif

#ifndef TP_EMFIELDS_T
#define TP_EMFIELDS_T
typedef struct emfields {
    double Bx, By, Bz;
    double Ex, Ey, Ez;
} emfields;
#endif

#ifndef BFIELDS_H
#define BFIELDS_H
typedef struct bfields {
    double Bx, By, Bz;
} bfields;
#endif

#ifndef EFIELDS_H
#define EFIELDS_H
typedef struct efields {
    double Ex, Ey, Ez;
} efields;
#endif

#ifndef WLCS_H
#define WLCS_H
typedef struct wlcs {
    double x_wr, y_wr, z_wr;
    double costheta_wr, cosphi_wr;
    double sintheta_wr, sinphi_wr;
    double cur_wr, t0;
    double x_lp, y_lp, z_lp, r_lp;
    double cosalpha_lp, cosbeta_lp;
    double sinalpha_lp, sinbeta_lp;
    double cur_lp;
    double omega;
} wlcs;
#endif

#ifndef PARAM_FF_H
#define PARAM_FF_H
typedef struct param_ff {
    double B0, lambda0;
} param_ff;
#endif

#ifndef BFIELDS_FLOAT_H
#define BFIELDS_FLOAT_H
typedef struct bfields_float { float bx, by, bz; } bfields_float;
#endif
#ifndef BFIELDS_DOUBLE_H
#define BFIELDS_DOUBLE_H
typedef struct bfields_double { double bx, by, bz; } bfields_double;
#endif
#ifndef EFIELDS_FLOAT_H
#define EFIELDS_FLOAT_H
typedef struct efields_float { float ex, ey, ez; } efields_float;
#endif
#ifndef EFIELDS_DOUBLE_H
#define EFIELDS_DOUBLE_H
typedef struct efields_double { double ex, ey, ez; } efields_double;
#endif
#ifndef VFIELDS_FLOAT_H
#define VFIELDS_FLOAT_H
typedef struct vfields_float { float vx, vy, vz; } vfields_float;
#endif
#ifndef VFIELDS_DOUBLE_H
#define VFIELDS_DOUBLE_H
typedef struct vfields_double { double vx, vy, vz; } vfields_double;
#endif

/* Physical constants of the wire-loop field (include/constants.h:16-19,
 * include/wlcs.h:38-40). */
#define TP_L0 6.96E8
#define TP_I0 4.0E8
#define TP_C0 3.0E10

/* System types of get_emf (src/emfields.c:20-25), plus the turbulent
 * plane-wave mode sum that has no counterpart in the reference. */
enum {
    TP_SYS_TEST = 0,
    TP_SYS_WLCS = 1,
    TP_SYS_FORCEFREE = 2,
    TP_SYS_MHD = 3,
    TP_SYS_PIC = 4,
    TP_SYS_MODESUM = 5
};

/* One plane-wave mode of the turbulent field (no reference counterpart):
 *   dB(x) = amp_b * cos(2*pi*(n . x / L) + phase)
 *   E(x)  = amp_e * cos(2*pi*(n . x / L) + phase)
 * with n an integer lattice vector, so the field is periodic in the box.
 * amp_e = -v_a * (n/|n|) x amp_b for the stated Alfvenic convention. */
typedef struct tp_mode {
    int n[3];
    int pad;
    double amp_b[3];
    double amp_e[3];
    double phase; /* radians */
    double pad2;
} tp_mode;

#endif /* TP_TYPES_H */
