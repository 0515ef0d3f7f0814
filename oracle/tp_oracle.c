/*
 * tp_oracle.c -- CPU restatement of the reference's test-particle hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see tp_oracle.h): the checker and the timed CPU
 * baseline, never part of the product.  Build: -O2 -ffp-contract=off -fopenmp
 * (no FMA contraction, so x86 and aarch64 agree with the reference built the
 * same way).  Every function names the reference lines it restates; the
 * operation order inside each expression follows those lines.
 */
#include "tp_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TP_ELL_QUAL static const
#include "../test_particle_gb300/csrc/ellint_coeffs.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* src/diagnostics.c:629-631 */
void or_spectrum_init(or_spectrum *s, int nbins, double emin, double emax)
{
    s->nbins = nbins;
    s->emin = emin;
    s->emax = emax;
    s->logemin = log10(emin);
    s->logemax = log10(emax);
    s->logde = (s->logemax - s->logemin) / (nbins - 2);
}

/* ------------------------------------------------------------------ */
/* Interpolation: src/interpolation.c:36-181                           */
/* ------------------------------------------------------------------ */

/* grid_indices, src/interpolation.c:36-105 */
static void grid_indices(const or_field *f, double x, double y, double z, double t,
        int *ix1, int *iy1, int *iz1, int *ix2, int *iy2, int *iz2,
        double *dx, double *dy, double *dz, double *dt)
{
    const grids *g = &f->grd;
    const domain *d = &f->dom;
    int nx = g->nx, ny = g->ny, nz = g->nz;
    *ix1 = (int)floor((x - d->xmin) / g->dx);
    *iy1 = (int)floor((y - d->ymin) / g->dy);
    *iz1 = (int)floor((z - d->zmin) / g->dz);
    *ix2 = *ix1 + 1;
    *iy2 = *iy1 + 1;
    *iz2 = *iz1 + 1;
    *dx = (x - d->xmin) / g->dx - (*ix1);
    *dy = (y - d->ymin) / g->dy - (*iy1);
    *dz = (z - d->zmin) / g->dz - (*iz1);
    /* periodic wrap; the reference assumes xmin = 0 here (lines 61-90) */
    if (x > d->xmax) { *ix1 = nx - 1; *ix2 = 0; *dx = x / g->dx - (nx - 1); }
    if (y > d->ymax) { *iy1 = ny - 1; *iy2 = 0; *dy = y / g->dy - (ny - 1); }
    if (z > d->zmax) { *iz1 = nz - 1; *iz2 = 0; *dz = z / g->dz - (nz - 1); }
    if (x < d->xmin) { *ix1 = nx - 1; *ix2 = 0; *dx = x / g->dx + 1.0; }
    if (y < d->ymin) { *iy1 = ny - 1; *iy2 = 0; *dy = y / g->dy + 1.0; }
    if (z < d->zmin) { *iz1 = nz - 1; *iz2 = 0; *dz = z / g->dz + 1.0; }
    if (f->multi_tframe == 0) {
        *dt = 0.0;
    } else {
        int it1 = (int)floor(t / g->dt);
        *dt = t / g->dt - it1;
    }
}

/* index_transfer for rank 3, src/interpolation.c:119-128: ix + nx*iy + nx*ny*iz
 * with int products, as there. */
static long idx3(int nx, int ny, int ix, int iy, int iz)
{
    long index = ix;
    int shift = nx;
    index += shift * iy;
    shift *= ny;
    index += shift * iz;
    return index;
}

/* get_trilinar_parameters, src/interpolation.c:141-181 */
void or_trilinear(const or_field *f, double x, double y, double z, double t,
                  long corners[8], double w[8], double *dt)
{
    int ix1, iy1, iz1, ix2, iy2, iz2;
    double dx, dy, dz;
    int nx = f->grd.nx, ny = f->grd.ny;
    grid_indices(f, x, y, z, t, &ix1, &iy1, &iz1, &ix2, &iy2, &iz2, &dx, &dy, &dz, dt);
    corners[0] = idx3(nx, ny, ix1, iy1, iz1);
    corners[1] = idx3(nx, ny, ix1, iy1, iz2);
    corners[2] = idx3(nx, ny, ix1, iy2, iz1);
    corners[3] = idx3(nx, ny, ix2, iy1, iz1);
    corners[4] = idx3(nx, ny, ix2, iy2, iz1);
    corners[5] = idx3(nx, ny, ix2, iy1, iz2);
    corners[6] = idx3(nx, ny, ix1, iy2, iz2);
    corners[7] = idx3(nx, ny, ix2, iy2, iz2);
    if (!f->interp_corrected) {
        /* the reference's weights (lines 173-180): corners 1,3,4,6 carry the
         * weight of their x<->z mirror */
        w[0] = (1.0 - dx) * (1.0 - dy) * (1.0 - dz);
        w[1] = dx * (1.0 - dy) * (1.0 - dz);
        w[2] = (1.0 - dx) * dy * (1.0 - dz);
        w[3] = (1.0 - dx) * (1.0 - dy) * dz;
        w[4] = (1.0 - dx) * dy * dz;
        w[5] = dx * (1.0 - dy) * dz;
        w[6] = dx * dy * (1.0 - dz);
        w[7] = dx * dy * dz;
    } else {
        w[0] = (1.0 - dx) * (1.0 - dy) * (1.0 - dz);
        w[1] = (1.0 - dx) * (1.0 - dy) * dz;
        w[2] = (1.0 - dx) * dy * (1.0 - dz);
        w[3] = dx * (1.0 - dy) * (1.0 - dz);
        w[4] = dx * dy * (1.0 - dz);
        w[5] = dx * (1.0 - dy) * dz;
        w[6] = (1.0 - dx) * dy * dz;
        w[7] = dx * dy * dz;
    }
}

/* get_double_velocity_at_point, src/velocity_field.c:555-584 (the same shape
 * serves get_double_{b,e}field_at_point). */
static void interp_double3(const or_field *f, const double *c, const double *a,
        const double *b, double x, double y, double z, double t, double out[3])
{
    long cn[8];
    double w[8], dt;
    or_trilinear(f, x, y, z, t, cn, w, &dt);
    if (f->multi_tframe == 0) {
        double v0 = 0.0, v1 = 0.0, v2 = 0.0;
        for (int i = 0; i < 8; i++) {
            v0 += c[3*cn[i]+0] * w[i];
            v1 += c[3*cn[i]+1] * w[i];
            v2 += c[3*cn[i]+2] * w[i];
        }
        out[0] = v0; out[1] = v1; out[2] = v2;
    } else {
        double p[3] = {0.0, 0.0, 0.0}, q[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < 8; i++)
            for (int k = 0; k < 3; k++) {
                p[k] += a[3*cn[i]+k] * w[i];
                q[k] += b[3*cn[i]+k] * w[i];
            }
        for (int k = 0; k < 3; k++) out[k] = dt * p[k] + (1.0 - dt) * q[k];
    }
}

/* get_float_{b,e}field_at_point / get_float_velocity_at_point,
 * src/magnetic_field.c:593-622, src/electric_field.c:408-437,
 * src/velocity_field.c:593-622: float results accumulated through double. */
static void interp_float3(const or_field *f, const float *c, const float *a,
        const float *b, double x, double y, double z, double t, float out[3])
{
    long cn[8];
    double w[8], dt;
    or_trilinear(f, x, y, z, t, cn, w, &dt);
    if (f->multi_tframe == 0) {
        float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f;
        for (int i = 0; i < 8; i++) {
            v0 = (float)((double)v0 + (double)c[3*cn[i]+0] * w[i]);
            v1 = (float)((double)v1 + (double)c[3*cn[i]+1] * w[i]);
            v2 = (float)((double)v2 + (double)c[3*cn[i]+2] * w[i]);
        }
        out[0] = v0; out[1] = v1; out[2] = v2;
    } else {
        double p[3] = {0.0, 0.0, 0.0}, q[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < 8; i++)
            for (int k = 0; k < 3; k++) {
                p[k] += (double)a[3*cn[i]+k] * w[i];
                q[k] += (double)b[3*cn[i]+k] * w[i];
            }
        for (int k = 0; k < 3; k++) out[k] = (float)(dt * p[k] + (1.0 - dt) * q[k]);
    }
}

/* ------------------------------------------------------------------ */
/* Analytic fields                                                     */
/* ------------------------------------------------------------------ */

/* getb_ff / gete_ff / getemf_ff, src/force_free.c:54-86,138-150 */
static void emf_forcefree(const or_field *f, double x, double y, double z, double t,
        emfields *e)
{
    double l = f->lambda0;
    double bx = f->ffA * sin(l * z) + f->ffC * cos(l * y);
    double by = f->ffB * sin(l * x) + f->ffA * cos(l * z);
    double bz = f->ffC * sin(l * y) + f->ffB * cos(l * x);
    bx *= f->B0;
    by *= f->B0;
    bz *= f->B0;
    e->Bx = bx; e->By = by; e->Bz = bz;
    if (f->vc_d || f->va_d) {
        double v[3];
        interp_double3(f, (const double *)f->vc_d, (const double *)f->va_d,
                (const double *)f->vb_d, x, y, z, t, v);
        e->Ex = by * v[2] - bz * v[1];
        e->Ey = bz * v[0] - bx * v[2];
        e->Ez = bx * v[1] - by * v[0];
    } else {
        e->Ex = 0.0; e->Ey = 0.0; e->Ez = 0.0;
    }
}

/* transform / reverse_tran, src/wlcs.c:871-903 */
static void wl_transform(double *ax, double *ay, double *az, double c1, double s1,
        double c2, double s2)
{
    double ax1 = c2 * (*ax) + s2 * (*ay);
    double ay1 = -s2 * (*ax) + c2 * (*ay);
    double az1 = *az;
    *ax = c1 * ax1 - s1 * az1;
    *ay = ay1;
    *az = s1 * ax1 + c1 * az1;
}

static void wl_reverse(double *ax, double *ay, double *az, double c1, double s1,
        double c2, double s2)
{
    double ax1 = c1 * (*ax) + s1 * (*az);
    double ay1 = *ay;
    double az1 = -s1 * (*ax) + c1 * (*az);
    *ax = c2 * ax1 - s2 * ay1;
    *ay = s2 * ax1 + c2 * ay1;
    *az = az1;
}

/* ellint, src/wlcs.c:460-809 (Fukushima 2009 piecewise Taylor series).
 * corrected = 0 keeps the reference's m >= 0.9 branch, which expands K about
 * the complementary parameter with the wrong sign (m - 0.95 instead of
 * 0.95 - m) and its 10x K coefficient (term 19 of the m0 = 0.875 interval). */
void or_ellint(double k, int corrected, double *elle, double *ellf)
{
    double m = k * k;
    int i;
    *elle = 0.0;
    *ellf = 0.0;
    if (m < 0.8) i = (int)(m / 0.1);
    else if (m >= 0.8 && m < 0.85) i = 8;
    else if (m >= 0.85 && m < 0.9) i = 9;
    else i = 10;
    if (i >= 0 && i <= 9) {
        double m1 = m - tp_ell_m0[i], powj = 1.0;
        int nk = tp_ell_nk[i], ne = tp_ell_ne[i];
        for (int j = 0; j < nk; j++) {
            double kc = tp_ell_k[i][j];
            if (!corrected && i == 9 && j == 19) kc = TP_ELL_K9_19_REF;
            *ellf += kc * powj;
            if (j < ne) *elle += tp_ell_e[i][j] * powj;
            powj *= m1;
        }
        return;
    }
    /* m >= 0.9 (or NaN): K(m) = -ln q(1-m) K(1-m) / pi and Legendre's relation */
    double ellf1 = 0.0, q1 = 0.0, hm = 0.0, powj = 1.0;
    double m1 = corrected ? (0.95 - m) : (m - 0.95);
    for (int j = 0; j <= 10; j++) {
        ellf1 += tp_ell_k[0][j] * powj;
        powj *= m1;
    }
    m1 = 1.0 - m;
    powj = m1;
    for (int j = 1; j <= 14; j++) {
        q1 += tp_ell_q[j] * powj;
        powj *= m1;
    }
    powj = 1.0;
    m1 = 0.95 - m;
    for (int j = 0; j <= 10; j++) {
        hm += tp_ell_h[j] * powj;
        powj *= m1;
    }
    *ellf = -log(q1) * (ellf1 / M_PI);
    *elle = 1.0 / ellf1 * (M_PI / 2.0 + *ellf * hm);
}

/* getWireB, src/wlcs.c:361-401 */
static void wl_wire_static(const wlcs *c, double x, double y, double z, double B[3])
{
    double xp = x - c->x_wr, yp = y - c->y_wr, zp = z - c->z_wr;
    double rho, phi0, bphi;
    wl_transform(&xp, &yp, &zp, c->costheta_wr, c->sintheta_wr, c->cosphi_wr, c->sinphi_wr);
    rho = sqrt(xp * xp + yp * yp);
    if (rho < 0.1) rho = 0.1;
    double cos_phi0 = xp / rho;
    if (yp >= 0.0) phi0 = acos(cos_phi0);
    else phi0 = 2.0 * M_PI - acos(cos_phi0);
    bphi = 1.0 / 5.0 * (c->cur_wr * TP_I0) / (rho * TP_L0);
    B[0] = bphi * cos(phi0 + M_PI / 2.0);
    B[1] = bphi * sin(phi0 + M_PI / 2.0);
    B[2] = 0.0;
    wl_reverse(&B[0], &B[1], &B[2], c->costheta_wr, c->sintheta_wr, c->cosphi_wr, c->sinphi_wr);
}

/* getWire_Bessel, src/wlcs.c:281-355 (single-precision glibc Bessel functions) */
static void wl_wire_bessel(const wlcs *c, double x, double y, double z, double t,
        double B[3], double E[3])
{
    double xp = x - c->x_wr, yp = y - c->y_wr, zp = z - c->z_wr;
    double t1 = c->t0 + t, curI = c->cur_wr, omega = c->omega, rho, x0, phi1;
    wl_transform(&xp, &yp, &zp, c->costheta_wr, c->sintheta_wr, c->cosphi_wr, c->sinphi_wr);
    rho = sqrt(xp * xp + yp * yp);
    x0 = omega * rho * TP_L0 / TP_C0;
    double bj0 = j0f((float)x0), bj1 = j1f((float)x0);
    double by0 = y0f((float)x0), by1 = y1f((float)x0);
    double const0 = (curI * TP_I0) / (5.0 * rho * TP_L0) * M_PI / 2.0;
    double wireB = const0 * x0 * (-by1 * cos(omega * t1) + bj1 * sin(omega * t1));
    if (rho == 0.0) phi1 = M_PI / 2.0;
    else if (yp >= 0.0) phi1 = acos(xp / rho) + M_PI / 2.0;
    else phi1 = 2.0 * M_PI - acos(xp / rho) + M_PI / 2.0;
    B[0] = wireB * cos(phi1);
    B[1] = wireB * sin(phi1);
    B[2] = 0.0;
    wl_reverse(&B[0], &B[1], &B[2], c->costheta_wr, c->sintheta_wr, c->cosphi_wr, c->sinphi_wr);
    double wireE = -const0 * x0 * (by0 * sin(omega * t1) + bj0 * cos(omega * t1));
    E[0] = 0.0; E[1] = 0.0; E[2] = wireE;
    wl_reverse(&E[0], &E[1], &E[2], c->costheta_wr, c->sintheta_wr, c->cosphi_wr, c->sinphi_wr);
}

/* getLoopB, src/wlcs.c:406-449.  On the loop axis (rho_xy = 0) Brho is set to
 * 0 and then divided by rho_xy again, giving NaN in Bx, By as the reference
 * does; ellint_corrected = 1 also returns 0 there. */
static void wl_loop(const or_field *f, const wlcs *c, double x, double y, double z, double B[3])
{
    double xp = (x - c->x_lp) * TP_L0, yp = (y - c->y_lp) * TP_L0, zp = (z - c->z_lp) * TP_L0;
    double al = c->r_lp * TP_L0, curI = c->cur_lp * TP_I0;
    wl_transform(&xp, &yp, &zp, c->cosbeta_lp, c->sinbeta_lp, c->cosalpha_lp, c->sinalpha_lp);
    double Irho = 0.2 * curI;
    double rho_xy = sqrt(xp * xp + yp * yp);
    double al2 = al * al;
    double r2 = rho_xy * rho_xy + zp * zp;
    double irho1 = 1 / sqrt((al + rho_xy) * (al + rho_xy) + zp * zp);
    double irho2 = 1 / ((al - rho_xy) * (al - rho_xy) + zp * zp);
    double k = sqrt(4.0 * al * rho_xy) * irho1, elle, ellk;
    or_ellint(k, f->ellint_corrected, &elle, &ellk);
    double Brho = Irho * zp * irho1 * (-ellk + (al2 + r2) * elle * irho2) / rho_xy;
    if (rho_xy == 0.0) Brho = 0.0;
    double Bz = Irho * irho1 * (ellk - (r2 - al2) * elle * irho2);
    if (f->ellint_corrected && rho_xy == 0.0) {
        B[0] = 0.0; B[1] = 0.0;
    } else {
        Brho /= rho_xy;
        B[0] = Brho * xp;
        B[1] = Brho * yp;
    }
    B[2] = Bz;
    wl_reverse(&B[0], &B[1], &B[2], c->cosbeta_lp, c->sinbeta_lp, c->cosalpha_lp, c->sinalpha_lp);
}

/* getemf_wlcs, src/wlcs.c:814-865 */
static void emf_wlcs(const or_field *f, double x, double y, double z, double t, emfields *e)
{
    double Bx = 0.0, By = 0.0, Bz = 0.0, Ex = 0.0, Ey = 0.0, Ez = 0.0;
    for (int i = 0; i < f->nwlcs; i++) {
        double B[3], E[3];
        if (f->iBessel == 0) {
            wl_wire_static(&f->cfg[i], x, y, z, B);
            Bx += B[0]; By += B[1]; Bz += B[2];
        } else {
            wl_wire_bessel(&f->cfg[i], x, y, z, t, B, E);
            Bx += B[0]; Ex += E[0];
            By += B[1]; Ey += E[1];
            Bz += B[2]; Ez += E[2];
        }
        wl_loop(f, &f->cfg[i], x, y, z, B);
        Bx += B[0]; By += B[1]; Bz += B[2];
    }
    e->Bx = Bx; e->By = By; e->Bz = Bz;
    e->Ex = Ex; e->Ey = Ey; e->Ez = Ez;
    e->Bz += 0.0;
}

/* Turbulent plane-wave mode sum (no reference counterpart).  The phase
 * 2*pi*(n . u) + phase with u = (x - min)/L per axis is formed exactly in
 * 64-bit fixed point (wrap-around = periodicity), then converted to radians. */
static uint64_t fixed_frac(double u)
{
    double fr = u - floor(u);
    return (uint64_t)(fr * 18446744073709551616.0);
}

void or_mode_sum(const or_field *f, double x, double y, double z, emfields *e)
{
    const domain *d = &f->dom;
    uint64_t ux = fixed_frac((x - d->xmin) / (d->xmax - d->xmin));
    uint64_t uy = fixed_frac((y - d->ymin) / (d->ymax - d->ymin));
    uint64_t uz = fixed_frac((z - d->zmin) / (d->zmax - d->zmin));
    double b[3] = {0.0, 0.0, 0.0}, ef[3] = {0.0, 0.0, 0.0};
    for (int m = 0; m < f->nmodes; m++) {
        const tp_mode *md = &f->modes[m];
        uint64_t ph0 = (uint64_t)(int64_t)llround(md->phase / (2.0 * M_PI) * 4294967296.0) << 32;
        uint64_t ph = (uint64_t)(int64_t)md->n[0] * ux + (uint64_t)(int64_t)md->n[1] * uy
                    + (uint64_t)(int64_t)md->n[2] * uz + ph0;
        double th = (double)(int64_t)ph * (2.0 * M_PI / 18446744073709551616.0);
        double c = cos(th);
        for (int k = 0; k < 3; k++) {
            b[k] += md->amp_b[k] * c;
            ef[k] += md->amp_e[k] * c;
        }
    }
    e->Bx = b[0];
    e->By = b[1];
    e->Bz = f->B0 + b[2];
    e->Ex = ef[0]; e->Ey = ef[1]; e->Ez = ef[2];
}

/* Synthetic gridded fields.  Node (i, j, k) of a grid periodic in node
 * index has box coordinates u = (i/nx, j/ny, k/nz), held as exact 64-bit
 * fixed point floor(i 2^64 / nx); a mode's phase is the exact integer
 * n . U + phase0 (mod 2^64), phase0 = round(phase / 2 pi * 2^32) 2^32.  The
 * cosine of that angle is formed as the real part of a product of four unit
 * complex numbers, one per axis (exact per-axis angles) and one for phase0,
 * so a row of nodes costs two multiplies and an add per mode instead of a
 * cosine; the modes are summed per node in table order.  The product differs
 * from the cosine of the summed angle by a few ulp, which moves a handful of
 * the FP32 node values of a 512^3 grid by one FP32 ulp. */
static void synth_axis(const tp_mode *m, int nm, int axis, int n, int idx, double *re, double *im)
{
    const uint64_t u = (uint64_t)(((unsigned __int128)idx << 64) / (unsigned)n);
    for (int q = 0; q < nm; q++) {
        uint64_t ph = (uint64_t)(int64_t)m[q].n[axis] * u;
        double th = (double)(int64_t)ph * (2.0 * M_PI / 18446744073709551616.0);
        re[q] = cos(th);
        im[q] = sin(th);
    }
}

void or_pic_records_from_c(const float *data, long nx, long ny, long nz, double scale, int comp, float *rec)
{
    const long nxy = nx * ny, nyz = ny * nz;
    for (long i = 0; i != nx; ++i)
        for (long j = 0; j != ny; ++j)
            for (long k = 0; k != nz; ++k)
                rec[3 * (k * nxy + j * nx + i) + comp] = (float)(data[i * nyz + j * nz + k] * scale);
}

static uint64_t synth_phase0(double phase)
{
    double rev = phase / (2.0 * M_PI);
    rev -= floor(rev);
    return (uint64_t)(uint32_t)llround(rev * 4294967296.0) << 32;
}

void or_synth_pic_fields(int nmb, const tp_mode *mb, int nmv, const tp_mode *mv, double B0z,
                         int nx, int ny, int nz, float *e, float *b, int nthreads)
{
    const int nm = nmb + nmv;
    tp_mode *all = (tp_mode *)malloc(sizeof(tp_mode) * (size_t)(nm > 0 ? nm : 1));
    memcpy(all, mb, sizeof(tp_mode) * (size_t)nmb);
    memcpy(all + nmb, mv, sizeof(tp_mode) * (size_t)nmv);
    /* per mode: e^{i A_q(i)} along x for every i (SoA), and e^{i phase0} */
    double *xr = (double *)malloc(sizeof(double) * (size_t)nm * nx);
    double *xi = (double *)malloc(sizeof(double) * (size_t)nm * nx);
    double *p0r = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
    double *p0i = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
    for (int q = 0; q < nm; q++) {
        double th = (double)(int64_t)synth_phase0(all[q].phase) * (2.0 * M_PI / 18446744073709551616.0);
        p0r[q] = cos(th);
        p0i[q] = sin(th);
    }
    {
        double *re = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
        double *im = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
        for (int i = 0; i < nx; i++) {
            synth_axis(all, nm, 0, nx, i, re, im);
            for (int q = 0; q < nm; q++) {
                xr[(size_t)q * nx + i] = re[q];
                xi[(size_t)q * nx + i] = im[q];
            }
        }
        free(re);
        free(im);
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        double *yr = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
        double *yi = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
        double *zr = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
        double *zi = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
        double *acc = (double *)malloc(sizeof(double) * 6 * (size_t)nx);
        double *B0 = acc, *B1 = acc + nx, *B2 = acc + 2 * nx;
        double *V0 = acc + 3 * nx, *V1 = acc + 4 * nx, *V2 = acc + 5 * nx;
        int kz_last = -1;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (long row = 0; row < (long)ny * nz; row++) {
            const int j = (int)(row % ny), k = (int)(row / ny);
            if (k != kz_last) {
                synth_axis(all, nm, 2, nz, k, zr, zi);
                kz_last = k;
            }
            synth_axis(all, nm, 1, ny, j, yr, yi);
            for (int c = 0; c < 6 * nx; c++) acc[c] = 0.0;
            for (int q = 0; q < nm; q++) {
                /* w = e^{iB} e^{iC} e^{i phase0} */
                double ar = yr[q] * zr[q] - yi[q] * zi[q], ai = yr[q] * zi[q] + yi[q] * zr[q];
                double wr = ar * p0r[q] - ai * p0i[q], wi = ar * p0i[q] + ai * p0r[q];
                const double *qr = xr + (size_t)q * nx, *qi = xi + (size_t)q * nx;
                const double a0 = all[q].amp_b[0], a1 = all[q].amp_b[1], a2 = all[q].amp_b[2];
                double *o0 = q < nmb ? B0 : V0, *o1 = q < nmb ? B1 : V1, *o2 = q < nmb ? B2 : V2;
#ifdef _OPENMP
#pragma omp simd
#endif
                for (int i = 0; i < nx; i++) {
                    const double c = wr * qr[i] - wi * qi[i];
                    o0[i] += a0 * c;
                    o1[i] += a1 * c;
                    o2[i] += a2 * c;
                }
            }
            float *eo = e + 3 * (size_t)row * nx, *bo = b + 3 * (size_t)row * nx;
            for (int i = 0; i < nx; i++) {
                const double Bx = B0[i], By = B1[i], Bz = B2[i] + B0z;
                bo[3 * i] = (float)Bx;
                bo[3 * i + 1] = (float)By;
                bo[3 * i + 2] = (float)Bz;
                eo[3 * i] = (float)(-(V1[i] * Bz - V2[i] * By));
                eo[3 * i + 1] = (float)(-(V2[i] * Bx - V0[i] * Bz));
                eo[3 * i + 2] = (float)(-(V0[i] * By - V1[i] * Bx));
            }
        }
        free(yr); free(yi); free(zr); free(zi); free(acc);
    }
    free(xr); free(xi); free(p0r); free(p0i); free(all);
}

/* get_emf, src/emfields.c:32-60 (system 0: getemf_test :210-218; system 3:
 * getemf_mhd_test_particle :107-120; system 4: getemf_pic_test_particle :153-166) */
void or_get_emf(const or_field *f, double x, double y, double z, double t, emfields *e)
{
    e->Bx = 0.0; e->By = 0.0; e->Bz = 0.0;
    e->Ex = 0.0; e->Ey = 0.0; e->Ez = 0.0;
    switch (f->system_type) {
    case TP_SYS_TEST:
        e->Bz = 1.0E0;
        break;
    case TP_SYS_WLCS:
        emf_wlcs(f, x, y, z, t, e);
        break;
    case TP_SYS_FORCEFREE:
        emf_forcefree(f, x, y, z, t, e);
        break;
    case TP_SYS_MHD: {
        float v[3], b[3];
        interp_float3(f, (const float *)f->vc_f, (const float *)f->va_f,
                (const float *)f->vb_f, x, y, z, t, v);
        interp_float3(f, (const float *)f->bc_f, (const float *)f->ba_f,
                (const float *)f->bb_f, x, y, z, t, b);
        e->Bx = b[0]; e->By = b[1]; e->Bz = b[2];
        e->Ex = e->By * v[2] - e->Bz * v[1];
        e->Ey = e->Bz * v[0] - e->Bx * v[2];
        e->Ez = e->Bx * v[1] - e->By * v[0];
        break;
    }
    case TP_SYS_PIC: {
        float ev[3], b[3];
        interp_float3(f, (const float *)f->ec_f, (const float *)f->ea_f,
                (const float *)f->eb_f, x, y, z, t, ev);
        interp_float3(f, (const float *)f->bc_f, (const float *)f->ba_f,
                (const float *)f->bb_f, x, y, z, t, b);
        e->Ex = ev[0]; e->Ey = ev[1]; e->Ez = ev[2];
        e->Bx = b[0]; e->By = b[1]; e->Bz = b[2];
        break;
    }
    case TP_SYS_MODESUM:
        or_mode_sum(f, x, y, z, e);
        break;
    default:
        break;
    }
}

/* ------------------------------------------------------------------ */
/* Pusher: tracking_wirz, src/tracking.c:749-892 (c0_norm = 1)         */
/* ------------------------------------------------------------------ */
static double gamma_u(const double *u) /* get_gamma_vec, :1112-1115 */
{
    return sqrt(1.0 + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
}

static double modulus3(double x, double y, double z) /* :1137-1140 */
{
    return sqrt(x * x + y * y + z * z);
}

static void cross3(const double *a, const double *b, double *c) /* :1130-1135 */
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

void or_wirz(const or_field *f, particles *p, double dt)
{
    double vminus[3], vplus[3], delta[3], delta_m[3], hpara[3], hperp[3], hr[3];
    double r0[3] = {p->x, p->y, p->z}, pre[3];
    double cm = f->charge_mass, t0 = p->t;
    emfields emf;
    int i;
    delta[0] = p->ux; delta[1] = p->uy; delta[2] = p->uz;
    double gama = gamma_u(delta);
    or_get_emf(f, r0[0], r0[1], r0[2], t0, &emf);
    double Btot = sqrt(emf.Bx * emf.Bx + emf.By * emf.By + emf.Bz * emf.Bz);
    double iBtot = 1.0 / Btot;
    double dth = dt * 0.5;
    delta_m[0] = delta[0] + cm * dth * emf.Ex;
    delta_m[1] = delta[1] + cm * dth * emf.Ey;
    delta_m[2] = delta[2] + cm * dth * emf.Ez;
    gama = gamma_u(delta_m);
    double igama = 1.0 / gama;
    for (i = 0; i < 3; i++) vminus[i] = delta_m[i] * igama;
    hpara[0] = emf.Bx * iBtot; hpara[1] = emf.By * iBtot; hpara[2] = emf.Bz * iBtot;
    double vdothp = 0.0;
    for (i = 0; i < 3; i++) vdothp += vminus[i] * hpara[i];
    double vperp = modulus3(vminus[0] - vdothp * hpara[0], vminus[1] - vdothp * hpara[1],
                            vminus[2] - vdothp * hpara[2]);
    for (i = 0; i < 3; i++) hperp[i] = (vminus[i] - vdothp * hpara[i]) / vperp;
    cross3(hpara, hperp, hr);
    double gyroR = vperp * gama * 1.0 * iBtot / cm;
    double omegac = cm * Btot * igama;
    double dtheta = omegac * dt;
    double sind = sin(dtheta * 0.5), cosd = cos(dtheta * 0.5);
    double tmp1 = dth * vdothp * 1.0, tmp2 = gyroR * sind, tmp3 = -gyroR * (1.0 - cosd);
    for (i = 0; i < 3; i++)
        pre[i] = r0[i] + hpara[i] * tmp1 + hperp[i] * tmp2 + hr[i] * tmp3;
    or_get_emf(f, pre[0], pre[1], pre[2], t0 + dth, &emf);
    Btot = sqrt(emf.Bx * emf.Bx + emf.By * emf.By + emf.Bz * emf.Bz);
    iBtot = 1.0 / Btot;
    hpara[0] = emf.Bx * iBtot; hpara[1] = emf.By * iBtot; hpara[2] = emf.Bz * iBtot;
    vdothp = 0.0;
    for (i = 0; i < 3; i++) vdothp += vminus[i] * hpara[i];
    vperp = modulus3(vminus[0] - vdothp * hpara[0], vminus[1] - vdothp * hpara[1],
                     vminus[2] - vdothp * hpara[2]);
    for (i = 0; i < 3; i++) hperp[i] = (vminus[i] - vdothp * hpara[i]) / vperp;
    cross3(hpara, hperp, hr);
    omegac = cm * Btot * igama;
    dtheta = omegac * dt;
    sind = sin(dtheta);
    cosd = cos(dtheta);
    for (i = 0; i < 3; i++)
        vplus[i] = hpara[i] * vdothp + vperp * (cosd * hperp[i] - sind * hr[i]);
    /* get_delta_vec, :1066-1078 */
    double bm = 0.0;
    for (i = 0; i < 3; i++) bm += vplus[i] * vplus[i];
    double g2 = 1.0 / sqrt(1.0 - bm);
    for (i = 0; i < 3; i++) delta[i] = g2 * vplus[i];
    p->ux = delta[0] + cm * dth * emf.Ex;
    p->uy = delta[1] + cm * dth * emf.Ey;
    p->uz = delta[2] + cm * dth * emf.Ez;
    vdothp = 0.0;
    for (i = 0; i < 3; i++) vdothp += vplus[i] * hpara[i];
    vperp = modulus3(vplus[0] - vdothp * hpara[0], vplus[1] - vdothp * hpara[1],
                     vplus[2] - vdothp * hpara[2]);
    gyroR = vperp * gama * 1.0 * iBtot / cm;
    tmp1 = dt * vdothp * 1.0;
    tmp2 = gyroR * sind;
    tmp3 = -gyroR * (1.0 - cosd);
    p->x += hpara[0] * tmp1 + hperp[0] * tmp2 + hr[0] * tmp3;
    p->y += hpara[1] * tmp1 + hperp[1] * tmp2 + hr[1] * tmp3;
    p->z += hpara[2] * tmp1 + hperp[2] * tmp2 + hr[2] * tmp3;
    p->t += dt;
}

/* particle_bc, src/tracking.c:1172-1221 */
void or_particle_bc(const or_field *f, particles *p, int *iescape)
{
    const domain *d = &f->dom;
    double xdim = d->xmax - d->xmin, ydim = d->ymax - d->ymin, zdim = d->zmax - d->zmin;
    if (f->bc_flag == 0) {
        if (p->x > d->xmax) { p->x -= xdim; p->xshift += xdim; }
        if (p->y > d->ymax) { p->y -= ydim; p->yshift += ydim; }
        if (p->z > d->zmax) { p->z -= zdim; p->zshift += zdim; }
        if (p->x < d->xmin) { p->x += xdim; p->xshift -= xdim; }
        if (p->y < d->ymin) { p->y += ydim; p->yshift -= ydim; }
        if (p->z < d->zmin) { p->z += zdim; p->zshift -= zdim; }
    } else if (f->bc_flag == 1) {
        if ((p->x > d->xmax) || (p->y > d->ymax) || (p->z > d->zmax) ||
            (p->x < d->xmin) || (p->y < d->ymin) || (p->z < d->zmin))
            *iescape = 1;
    } else if (f->bc_flag == 2) {
        *iescape = 0;
    }
}

/* ptl_energy_fixed binning, src/diagnostics.c:187-205.  NaN and non-positive
 * energies land in bin 0 (x86 conversion of the invalid floor result). */
int or_energy_bin(const or_spectrum *s, double ux, double uy, double uz)
{
    double gama = sqrt(1.0 + ux * ux + uy * uy + uz * uz);
    return or_energy_bin_e(s, gama - 1.0);
}

int or_energy_bin_e(const or_spectrum *s, double ene)
{
    double v = floor((log10(ene) - s->logemin) / s->logde);
    int ibin;
    if (!(v == v) || v < -2147483648.0 || v > 2147483647.0) ibin = (int)0x80000000;
    else ibin = (int)v;
    if (ibin < 0) ibin = 0;
    else if (ibin > s->nbins - 1) ibin = s->nbins - 1;
    return ibin;
}

/* calc_diff_coeff, src/diagnostics.c:659-705.  Output order: drr, dxx, dyy,
 * dzz, dpp, duu, daa, dee. */
void or_calc_diff_coeff(const or_field *f, const particles *p0, const particles *p,
                        double dt, double o[8])
{
    double t = p->t * 2 + dt;
    double dxx = pow(p0->x - (p->x + p->xshift), 2) / t;
    double dyy = pow(p0->y - (p->y + p->yshift), 2) / t;
    double dzz = pow(p0->z - (p->z + p->zshift), 2) / t;
    double drr = dxx + dyy + dzz;
    double dpp = (pow(p0->ux - p->ux, 2) + pow(p0->uy - p->uy, 2) + pow(p0->uz - p->uz, 2)) / t;
    double gamma = sqrt(1.0 + p->ux * p->ux + p->uy * p->uy + p->uz * p->uz);
    double gamma0 = sqrt(1.0 + p0->ux * p0->ux + p0->uy * p0->uy + p0->uz * p0->uz);
    double dee = pow(gamma - gamma0, 2) / t;
    emfields e, e0;
    or_get_emf(f, p->x, p->y, p->z, p->t, &e);
    or_get_emf(f, p0->x, p0->y, p0->z, p0->t, &e0);
    double abs_b = sqrt(e.Bx * e.Bx + e.By * e.By + e.Bz * e.Bz);
    double abs_u = sqrt(p->ux * p->ux + p->uy * p->uy + p->uz * p->uz);
    double mu = (e.Bx * p->ux + e.By * p->uy + e.Bz * p->uz) / (abs_b * abs_u);
    abs_b = sqrt(e0.Bx * e0.Bx + e0.By * e0.By + e0.Bz * e0.Bz);
    abs_u = sqrt(p0->ux * p0->ux + p0->uy * p0->uy + p0->uz * p0->uz);
    double mu0 = (e0.Bx * p0->ux + e0.By * p0->uy + e0.Bz * p0->uz) / (abs_b * abs_u);
    double duu = pow(mu - mu0, 2) / t;
    double theta = acos(mu) * 180 / M_PI;
    double theta0 = acos(mu0) * 180 / M_PI;
    double daa = pow(theta - theta0, 2) / t;
    o[0] = drr; o[1] = dxx; o[2] = dyy; o[3] = dzz;
    o[4] = dpp; o[5] = duu; o[6] = daa; o[7] = dee;
}

/* estep = tmax / dt truncated, src/tracking.c:103 */
int or_estep(const or_field *f, double dt)
{
    return (int)(f->dom.tmax / dt);
}

/* particle_tracking_fixed_time_step + _multi_steps_openmp + _single_step_openmp,
 * src/tracking.c:90-190, 297-462, with tinterval_dcoeffs = 100 (:34). */
int or_track_fixed(const or_field *f, const or_spectrum *s, int nptl, double dt,
                   int nt_out, const particles *ptl_init, particles *ptl,
                   int *nsteps_ptl, double *espect, double *espect_escape,
                   double *dsum, int *remain, int nthreads)
{
    const int tdc = 100;
    int estep = or_estep(f, dt);
    if (estep < 1 || nt_out < 1) return -1;
    int einterval = estep / nt_out;
    if (einterval < 1) return -2;
    int nsdc = estep / tdc + 1, nbins = s->nbins;
    size_t nsp = (size_t)nt_out * nbins;
    memset(espect, 0, sizeof(double) * nsp);
    memset(espect_escape, 0, sizeof(double) * nsp);
    memset(dsum, 0, sizeof(double) * 8 * nsdc);
    for (int i = 0; i < nsdc; i++) remain[i] = nptl;
    for (int i = 0; i < nptl; i++) nsteps_ptl[i] = 1;
#ifdef _OPENMP
    int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    int nth = 1;
    (void)nthreads;
#endif
    double *tsum = (double *)calloc((size_t)nth * 8 * nsdc, sizeof(double));
    double *tsp = (double *)calloc((size_t)nth * nsp, sizeof(double));
    double *tse = (double *)calloc((size_t)nth * nsp, sizeof(double));
    int *trem = (int *)calloc((size_t)nth * nsdc, sizeof(int));
#ifdef _OPENMP
#pragma omp parallel num_threads(nth)
#endif
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        double *my_sum = tsum + (size_t)tid * 8 * nsdc;
        double *my_sp = tsp + (size_t)tid * nsp;
        double *my_se = tse + (size_t)tid * nsp;
        int *my_rem = trem + (size_t)tid * nsdc;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int i = 0; i < nptl; i++) {
            particles *p = &ptl[i];
            int esc_pre = 0, esc_after;
            or_particle_bc(f, p, &esc_pre);
            esc_after = esc_pre;
            int ntp = (int)floor(1 / (double)einterval);
            int tstep = 1;
            double sg[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (esc_pre) my_rem[1] -= 1;
            for (int j = 1; j <= estep; j++) {
                sg[0] = 0.0; sg[4] = 0.0; sg[5] = 0.0; /* drr, dpp, duu reset (:334-336) */
                if (esc_pre == 0 || f->bc_flag == 0) {
                    or_wirz(f, p, dt);
                    or_particle_bc(f, p, &esc_after);
                    nsteps_ptl[i] += 1;
                    if (esc_after == 0 && j % tdc == 0)
                        or_calc_diff_coeff(f, &ptl_init[i], p, dt, sg);
                }
                if (esc_pre == 0 && esc_after == 1 && f->bc_flag == 1 && ntp < nt_out)
                    my_se[(size_t)ntp * nbins + or_energy_bin(s, p->ux, p->uy, p->uz)] += 1.0;
                if (j % einterval == 0) {
                    if (esc_after == 0 && ntp < nt_out)
                        my_sp[(size_t)ntp * nbins + or_energy_bin(s, p->ux, p->uy, p->uz)] += 1.0;
                    ntp++;
                }
                if (j % tdc == 0) {
                    for (int c = 0; c < 8; c++) my_sum[(size_t)c * nsdc + tstep] += sg[c];
                    tstep++;
                }
                if (esc_after && j % tdc == 0 && tstep < nsdc) my_rem[tstep] -= 1;
                esc_pre = esc_after;
            }
        }
    }
    for (int t = 0; t < nth; t++) {
        for (size_t k = 0; k < (size_t)8 * nsdc; k++) dsum[k] += tsum[(size_t)t * 8 * nsdc + k];
        for (size_t k = 0; k < nsp; k++) {
            espect[k] += tsp[(size_t)t * nsp + k];
            espect_escape[k] += tse[(size_t)t * nsp + k];
        }
        for (int k = 0; k < nsdc; k++) remain[k] += trem[(size_t)t * nsdc + k];
    }
    free(tsum);
    free(tsp);
    free(tse);
    free(trem);
    return estep;
}

/* ------------------------------------------------------------------ */
/* batch helpers                                                       */
/* ------------------------------------------------------------------ */
void or_get_emf_batch(const or_field *f, int n, const double *xyzt, double *emf6)
{
    for (int i = 0; i < n; i++) {
        emfields e;
        or_get_emf(f, xyzt[4*i], xyzt[4*i+1], xyzt[4*i+2], xyzt[4*i+3], &e);
        emf6[6*i] = e.Bx; emf6[6*i+1] = e.By; emf6[6*i+2] = e.Bz;
        emf6[6*i+3] = e.Ex; emf6[6*i+4] = e.Ey; emf6[6*i+5] = e.Ez;
    }
}

void or_wirz_steps(const or_field *f, int n, particles *p, double dt, int nsteps, int *iescape)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < n; i++)
        for (int s = 0; s < nsteps; s++) {
            or_wirz(f, &p[i], dt);
            or_particle_bc(f, &p[i], &iescape[i]);
        }
}

void or_energy_bins(const or_spectrum *s, int n, const particles *p, int *bins)
{
    for (int i = 0; i < n; i++) bins[i] = or_energy_bin(s, p[i].ux, p[i].uy, p[i].uz);
}

void or_trilinear_batch(const or_field *f, int n, const double *xyzt, long *corners8, double *weights8)
{
    for (int i = 0; i < n; i++) {
        double dt;
        or_trilinear(f, xyzt[4*i], xyzt[4*i+1], xyzt[4*i+2], xyzt[4*i+3],
                     corners8 + 8*i, weights8 + 8*i, &dt);
    }
}

/* ------------------------------------------------------------------ */
/* Bulirsch-Stoer: src/unused/StepperBS.c (NR3 chapter 17 stepper)      */
/* ------------------------------------------------------------------ */
#define BS_IMAX 17
#define BS_NV 6

/* derivs, src/unused/StepperBS.c:443-471: y = (x, y, z, beta), positions in
 * units of L0, dbeta/dt = gamma^-3 * q/m * (E + beta x B). */
void or_bs_derivs(const or_field *f, double t, const double *y, double *yd)
{
    const double cl = TP_C0 / TP_L0;
    emfields emf;
    for (int i = 0; i < 3; i++) yd[i] = y[i + 3] * cl;
    or_get_emf(f, y[0], y[1], y[2], t, &emf);
    double cx = y[4] * emf.Bz - y[5] * emf.By;
    double cy = y[5] * emf.Bx - y[3] * emf.Bz;
    double cz = y[3] * emf.By - y[4] * emf.Bx;
    double beta2 = y[3] * y[3] + y[4] * y[4] + y[5] * y[5];
    double gama = 1.0 / sqrt(1.0 - beta2);
    double igama3 = 1.0 / (gama * gama * gama);
    yd[3] = igama3 * f->charge_mass * (emf.Ex + cx);
    yd[4] = igama3 * f->charge_mass * (emf.Ey + cy);
    yd[5] = igama3 * f->charge_mass * (emf.Ez + cz);
}

/* updatey (modified midpoint), src/unused/StepperBS.c:364-414, no dense output */
static void bs_midpoint(const or_field *f, double x, const double *y, const double *dydx,
        double htot, int nstep, double *yend)
{
    double ym[BS_NV], yn[BS_NV], h = htot / nstep, xnew, h2;
    for (int i = 0; i < BS_NV; i++) {
        ym[i] = y[i];
        yn[i] = y[i] + h * dydx[i];
    }
    xnew = x + h;
    or_bs_derivs(f, xnew, yn, yend);
    h2 = 2.0 * h;
    for (int nn = 1; nn < nstep; nn++) {
        for (int i = 0; i < BS_NV; i++) {
            double swap = ym[i] + h2 * yend[i];
            ym[i] = yn[i];
            yn[i] = swap;
        }
        xnew += h;
        or_bs_derivs(f, xnew, yn, yend);
    }
    for (int i = 0; i < BS_NV; i++) yend[i] = 0.5 * (ym[i] + yn[i] + h * yend[i]);
}

/* polyextr, src/unused/StepperBS.c:419-435 */
static void bs_polyextr(int k, double table[][BS_NV], double *last, double coeff[][BS_IMAX])
{
    for (int j = k - 1; j > 0; j--)
        for (int i = 0; i < BS_NV; i++)
            table[j - 1][i] = table[j][i] + coeff[k][j] * (table[j][i] - table[j - 1][i]);
    for (int i = 0; i < BS_NV; i++)
        last[i] = table[0][i] + coeff[k][0] * (table[0][i] - last[i]);
}

static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }

/* StepperBase (:103-149, densFlag false) and step (:159-354) with the
 * controller flags held per call instead of function-static.  As in the
 * reference's StepperBS (:77-83) every step starts from the initial k_targ. */
int or_bs_integrate(const or_field *f, const or_bs_cfg *cfg, double *y, double t0,
                    double h0, int nsteps, double *out)
{
    const double EPS = 2.22045e-16;
    const double STEPFAC1 = 0.65, STEPFAC2 = 0.94, STEPFAC3 = 0.02, STEPFAC4 = 4.0;
    const double KFAC1 = 0.8, KFAC2 = 0.9;
    const int KMAXX = cfg->kmaxx, IMAXX = cfg->kmaxx + 1;
    const double atol = cfg->atol, rtol = cfg->rtol;
    int nseq[BS_IMAX], cost[BS_IMAX];
    double coeff[BS_IMAX][BS_IMAX], table[BS_IMAX][BS_NV];
    if (KMAXX < 2 || IMAXX > BS_IMAX) return -1;
    for (int i = 0; i < IMAXX; i++) nseq[i] = 2 * (i + 1);
    cost[0] = nseq[0] + 1;
    for (int k = 0; k < KMAXX; k++) cost[k + 1] = cost[k] + nseq[k + 1];
    double logfact = -log10(dmax(1.0e-12, rtol)) * 0.6 + 0.5;
    const int k_targ0 = imax(1, imin(KMAXX - 1, (int)logfact));
    for (int k = 0; k < IMAXX; k++)
        for (int l = 0; l < k; l++) {
            double ratio = (double)(nseq[k]) / nseq[l];
            coeff[k][l] = 1.0 / (ratio * ratio - 1.0);
        }
    int first_step = 1, last_step = 0, reject = 0, prev_reject = 0;
    double x = t0, htry = h0, dydx[BS_NV], dydxnew[BS_NV];
    or_bs_derivs(f, x, y, dydx);
    for (int s = 0; s < nsteps; s++) {
        double hopt[BS_IMAX], work[BS_IMAX], ysav[BS_NV], yseq[BS_NV], scale[BS_NV];
        double h = htry, hnext = htry, hnew, err = 0.0, fac;
        int k_targ = k_targ0, k = 0, firstk = 1, forward = h > 0, nrej = 0;
        work[0] = 0.0;
        for (int i = 0; i < BS_NV; i++) ysav[i] = y[i];
        if (h != hnext && !first_step) last_step = 1;
        if (reject) { prev_reject = 1; last_step = 0; }
        reject = 0;
        hnew = fabs(h);
        while (firstk || reject) {
            h = forward ? hnew : -hnew;
            firstk = 0;
            reject = 0;
            if (cfg->max_rejects > 0 && nrej++ > cfg->max_rejects) return -2;
            for (k = 0; k <= k_targ + 1; k++) {
                bs_midpoint(f, x, ysav, dydx, h, nseq[k], yseq);
                if (k == 0) {
                    for (int i = 0; i < BS_NV; i++) y[i] = yseq[i];
                } else {
                    for (int i = 0; i < BS_NV; i++) table[k - 1][i] = yseq[i];
                }
                if (k != 0) {
                    bs_polyextr(k, table, y, coeff);
                    err = 0.0;
                    for (int i = 0; i < BS_NV; i++) {
                        scale[i] = atol + rtol * dmax(fabs(ysav[i]), fabs(y[i]));
                        err += pow((y[i] - table[0][i]) / scale[i], 2.0);
                    }
                    err = sqrt(err / BS_NV);
                    double expo = 1.0 / (2 * k + 1);
                    double facmin = pow(STEPFAC3, expo);
                    if (err == 0.0) {
                        fac = 1.0 / facmin;
                    } else {
                        fac = STEPFAC2 / pow(err / STEPFAC1, expo);
                        fac = dmax(facmin / STEPFAC4, dmin(1.0 / facmin, fac));
                    }
                    hopt[k] = fabs(h * fac);
                    work[k] = cost[k] / hopt[k];
                    if ((first_step || last_step) && err <= 1.0) break;
                    if (k == k_targ - 1 && !prev_reject && !first_step && !last_step) {
                        if (err <= 1.0) break;
                        else if (err > pow(nseq[k_targ] * nseq[k_targ + 1] / (nseq[0] * nseq[0]), 2.0)) {
                            reject = 1;
                            k_targ = k;
                            if (k_targ > 1 && work[k - 1] < KFAC1 * work[k]) k_targ--;
                            hnew = hopt[k_targ];
                            break;
                        }
                    }
                    if (k == k_targ) {
                        if (err <= 1.0) break;
                        else if (err > pow((double)nseq[k + 1] / nseq[0], 2.0)) {
                            reject = 1;
                            if (k_targ > 1 && work[k - 1] < KFAC1 * work[k]) k_targ--;
                            hnew = hopt[k_targ];
                            break;
                        }
                    }
                    if (k == k_targ + 1) {
                        if (err > 1.0) {
                            reject = 1;
                            if (k_targ > 1 && work[k_targ - 1] < KFAC1 * work[k_targ]) k_targ--;
                            hnew = hopt[k_targ];
                        }
                        break;
                    }
                }
            }
            if (reject) prev_reject = 1;
        }
        (void)EPS;
        or_bs_derivs(f, x + h, y, dydxnew);
        for (int i = 0; i < BS_NV; i++) dydx[i] = dydxnew[i];
        x += h;
        first_step = 0;
        int kopt;
        if (k == 1) {
            kopt = 2;
        } else if (k <= k_targ) {
            kopt = k;
            if (work[k - 1] < KFAC1 * work[k]) kopt = k - 1;
            else if (work[k] < KFAC2 * work[k - 1]) kopt = imin(k + 1, KMAXX - 1);
        } else {
            kopt = k - 1;
            if (k > 2 && work[k - 2] < KFAC1 * work[k - 1]) kopt = k - 2;
            if (work[k] < KFAC2 * work[kopt]) kopt = imin(k, KMAXX - 1);
        }
        if (prev_reject) {
            k_targ = imin(kopt, k);
            hnew = dmin(fabs(h), hopt[k_targ]);
            prev_reject = 0;
        } else {
            if (kopt <= k) {
                hnew = hopt[kopt];
            } else {
                if (k < k_targ && work[k] < KFAC2 * work[k - 1])
                    hnew = hopt[k] * cost[kopt + 1] / cost[k];
                else
                    hnew = hopt[k] * cost[kopt] / cost[k];
            }
            k_targ = kopt;
        }
        hnext = forward ? hnew : -hnew;
        out[8 * s] = x;
        out[8 * s + 1] = h;
        for (int i = 0; i < BS_NV; i++) out[8 * s + 2 + i] = y[i];
        htry = hnext;
    }
    return 0;
}

/* nsteps accepted steps of each of n particles (y: n*6 in/out), OpenMP over
 * particles; returns the total accepted steps (CPU baseline driver). */
long or_bs_run_many(const or_field *f, const or_bs_cfg *cfg, int n, double *y, double h0,
                    int nsteps, int nthreads)
{
    long total = 0;
#ifdef _OPENMP
    int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nth) reduction(+ : total)
#endif
    for (int i = 0; i < n; i++) {
        double *out = (double *)malloc(sizeof(double) * 8 * (size_t)nsteps);
        if (or_bs_integrate(f, cfg, y + 6 * (size_t)i, 0.0, h0, nsteps, out) == 0) total += nsteps;
        free(out);
    }
#ifndef _OPENMP
    (void)nthreads;
#endif
    return total;
}

/* ------------------------------------------------------------ Poincare map
 * src/poincare_map.c: field lines dx/|B| traced with fixed-step RK4 on the
 * unit vector of B from get_magnetic_field (systems 3 and 4: the float B
 * grid, src/emfields.c:76-96,122-188), periodic wrap of the evaluation points
 * only (field_boundary, :296-321, applied to the input of every stage), and
 * crossings of the plane pos[face] = seed[face] detected by a sign change of
 * (pre - init) * (cur - init) (:101-118, :165-181). */
static void or_field_boundary(const or_field *f, double *fx, double *fy, double *fz)
{
    double xdim = f->dom.xmax - f->dom.xmin, ydim = f->dom.ymax - f->dom.ymin;
    double zdim = f->dom.zmax - f->dom.zmin;
    if (*fx > f->dom.xmax) *fx -= xdim;
    if (*fy > f->dom.ymax) *fy -= ydim;
    if (*fz > f->dom.zmax) *fz -= zdim;
    if (*fx < f->dom.xmin) *fx += xdim;
    if (*fy < f->dom.ymin) *fy += ydim;
    if (*fz < f->dom.zmin) *fz += zdim;
}

static void or_unit_b(const or_field *f, double x, double y, double z, double b[3])
{
    emfields e;
    or_get_emf(f, x, y, z, 0, &e);  /* B part = get_bfield_{mhd,pic}_test_particle */
    double ib = 1.0 / sqrt(e.Bx * e.Bx + e.By * e.By + e.Bz * e.Bz);
    b[0] = e.Bx * ib;
    b[1] = e.By * ib;
    b[2] = e.Bz * ib;
}

/* next_location, src/poincare_map.c:243-290 */
void or_next_location(const or_field *f, double *fx, double *fy, double *fz, double dstep)
{
    double b1[3], b2[3], b3[3], b4[3], xt, yt, zt;
    or_field_boundary(f, fx, fy, fz);
    or_unit_b(f, *fx, *fy, *fz, b1);
    xt = *fx + 0.5 * dstep * b1[0];
    yt = *fy + 0.5 * dstep * b1[1];
    zt = *fz + 0.5 * dstep * b1[2];
    or_field_boundary(f, &xt, &yt, &zt);
    or_unit_b(f, xt, yt, zt, b2);
    xt = *fx + 0.5 * dstep * b2[0];
    yt = *fy + 0.5 * dstep * b2[1];
    zt = *fz + 0.5 * dstep * b2[2];
    or_field_boundary(f, &xt, &yt, &zt);
    or_unit_b(f, xt, yt, zt, b3);
    xt = *fx + dstep * b3[0];
    yt = *fy + dstep * b3[1];
    zt = *fz + dstep * b3[2];
    or_field_boundary(f, &xt, &yt, &zt);
    or_unit_b(f, xt, yt, zt, b4);
    *fx += (dstep / 6) * (b1[0] + 2 * b2[0] + 2 * b3[0] + b4[0]);
    *fy += (dstep / 6) * (b1[1] + 2 * b2[1] + 2 * b3[1] + b4[1]);
    *fz += (dstep / 6) * (b1[2] + 2 * b2[2] + 2 * b3[2] + b4[2]);
}

/* The crossing loop of one seed (src/poincare_map.c:158-181): pos_out[3][ncross+1]
 * (x row, y row, z row; entry 0 the seed), returns the crossings found. */
int or_poincare_point(const or_field *f, const double seed[3], int face, double step,
                      double length_max, int ncross, double *xo, double *yo, double *zo)
{
    double pos[3] = {seed[0], seed[1], seed[2]};
    double init = seed[face];
    xo[0] = seed[0]; yo[0] = seed[1]; zo[0] = seed[2];
    int icross = 1;
    double length = 0.0;
    while (icross <= ncross) {
        double cross = 1.0;
        while (cross > 0 && length < length_max) {
            double pre = pos[face];
            or_next_location(f, &pos[0], &pos[1], &pos[2], step);
            cross = (pre - init) * (pos[face] - init);
            length += step;
        }
        if (length < length_max) {
            xo[icross] = pos[0];
            yo[icross] = pos[1];
            zo[icross] = pos[2];
            ++icross;
        } else {
            break;
        }
    }
    return icross - 1;
}

/* Every seed (OpenMP); outputs [n][ncross+1] per coordinate, entries a seed
 * did not reach keep the reference's fill value 2 * max of that axis. */
void or_poincare_many(const or_field *f, int n, const double *seeds, int face, double step,
                      double length_max, int ncross, double *xpos, double *ypos, double *zpos,
                      int *found, int nthreads)
{
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n; i++) {
        double *xo = xpos + (size_t)i * (ncross + 1), *yo = ypos + (size_t)i * (ncross + 1);
        double *zo = zpos + (size_t)i * (ncross + 1);
        for (int k = 0; k <= ncross; k++) {
            xo[k] = f->dom.xmax * 2;
            yo[k] = f->dom.ymax * 2;
            zo[k] = f->dom.zmax * 2;
        }
        found[i] = or_poincare_point(f, seeds + 3 * i, face, step, length_max, ncross, xo, yo, zo);
    }
}
