// bs.cu -- batched adaptive Bulirsch-Stoer integration of many particles in
// one persistent launch (the reference's unused stepper src/unused/StepperBS.c,
// NR3 chapter 17, without dense output).
//
// One thread integrates one particle at a time and pulls the next particle
// from a global counter when it finishes, so lanes whose particles need few
// steps keep working while others take many.  The extrapolation tableau is
// FP64.  Every loop is bounded: a per-step rejection cap and a per-particle
// step cap end in a status code, never in a spin.
#include <climits>
#include <cmath>
#include <cstring>

#include "../../include/tp_gpu.h"
#include "fields_fp64.cuh"
#include "tp_internal.h"

namespace tp {
namespace bs {

constexpr int kImax = 17;
constexpr int kNv = 6;

struct BsConst {
    int nseq[kImax];
    int cost[kImax];
    double coeff[kImax][kImax];
    int kmaxx;
    int k_targ0;
    double atol, rtol;
    // host-computed powers of the step control: facmin[k] = STEPFAC3^(1/(2k+1))
    // (the reference's pow(STEPFAC3, expo)) and expo[k] = 1/(2k+1)
    double facmin[kImax], expo[kImax];
};

__constant__ BsConst c_bs;

struct BsArgs {
    int n;
    int uform;          // 0: the reference's beta form (positions in L0, c0/L0); 1: u = gamma v, c = 1
    int max_rejects;
    int max_steps;
    // production mode: integrate to t_end with nt_out frames and diagnostics
    double t_end;
    int nt_out, nbins;
    const double* ebin_thr;
    unsigned int* espect;
    double* dframe;     // (nt_out + 1) * 8 diffusion sums at the frames
    // parity mode: exactly nsteps accepted steps, per-step record (t, h, y[6])
    int nsteps;
    double* rec;
    // state
    double* y;          // n * 6
    double* t;          // n
    double* h;          // n: step size to try next
    const double* y0;   // n * 6 initial state (diffusion reference)
    int* steps;         // n: accepted steps
    int* pstatus;       // n: status bits per particle
    int* next;          // work counter
    int* status;
};

// derivs, src/unused/StepperBS.c:443-471 (uform = 0), or the relativistic
// equations of motion in u = gamma v (uform = 1): dx/dt = u / gamma,
// du/dt = q/m (E + u / gamma x B), c = 1.
__device__ __forceinline__ void derivs(const DevField& f, int uform, double t, const double* y,
                                       double* yd, int* status)
{
    double e[6];
    emf64<TP_SYS_WLCS>(f, y[0], y[1], y[2], t, e, status);
    if (uform == 0) {
        const double cl = TP_C0 / TP_L0;
        for (int i = 0; i < 3; i++) yd[i] = y[i + 3] * cl;
        double cx = y[4] * e[2] - y[5] * e[1];
        double cy = y[5] * e[0] - y[3] * e[2];
        double cz = y[3] * e[1] - y[4] * e[0];
        double beta2 = y[3] * y[3] + y[4] * y[4] + y[5] * y[5];
        double gama = 1.0 / sqrt(1.0 - beta2);
        double igama3 = 1.0 / (gama * gama * gama);
        yd[3] = igama3 * f.charge_mass * (e[3] + cx);
        yd[4] = igama3 * f.charge_mass * (e[4] + cy);
        yd[5] = igama3 * f.charge_mass * (e[5] + cz);
    } else {
        double ig = 1.0 / sqrt(1.0 + y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
        double v0 = y[3] * ig, v1 = y[4] * ig, v2 = y[5] * ig;
        yd[0] = v0; yd[1] = v1; yd[2] = v2;
        yd[3] = f.charge_mass * (e[3] + v1 * e[2] - v2 * e[1]);
        yd[4] = f.charge_mass * (e[4] + v2 * e[0] - v0 * e[2]);
        yd[5] = f.charge_mass * (e[5] + v0 * e[1] - v1 * e[0]);
    }
}

// updatey, src/unused/StepperBS.c:364-414 (modified midpoint, no dense output)
__device__ __forceinline__ void midpoint(const DevField& f, int uform, double x, const double* y,
                                         const double* dydx, double htot, int nstep, double* yend,
                                         int* status)
{
    double ym[kNv], yn[kNv];
    double h = htot / nstep;
    for (int i = 0; i < kNv; i++) {
        ym[i] = y[i];
        yn[i] = y[i] + h * dydx[i];
    }
    double xnew = x + h;
    derivs(f, uform, xnew, yn, yend, status);
    double h2 = 2.0 * h;
    for (int nn = 1; nn < nstep; nn++) {
        for (int i = 0; i < kNv; i++) {
            double swap = ym[i] + h2 * yend[i];
            ym[i] = yn[i];
            yn[i] = swap;
        }
        xnew += h;
        derivs(f, uform, xnew, yn, yend, status);
    }
    for (int i = 0; i < kNv; i++) yend[i] = 0.5 * (ym[i] + yn[i] + h * yend[i]);
}

__device__ __forceinline__ double sqr(double v) { return v * v; }
__device__ __forceinline__ double sqr_int(int v) { return (double)v * (double)v; }

struct Ctrl {
    bool first_step = true, last_step = false, reject = false, prev_reject = false;
};

// step, src/unused/StepperBS.c:159-354 without dense output; as in the
// reference's StepperBS (:77-83) each step starts from the initial k_targ.
// Returns 0, or ST_STEP_LIMIT when the rejection cap is hit.
__device__ int bs_step(const DevField& f, int uform, int max_rejects, bool nan_rejects, double& x,
                       double* y, double* dydx, double htry, double hnext_in, Ctrl& c,
                       double& hdid, double& hnext_out, int* status)
{
    const double STEPFAC1 = 0.65, STEPFAC2 = 0.94, STEPFAC4 = 4.0;  // STEPFAC3 = 0.02: c_bs.facmin
    const double KFAC1 = 0.8, KFAC2 = 0.9;
    const int KMAXX = c_bs.kmaxx;
    double table[kImax][kNv];
    double hopt[kImax], work[kImax], ysav[kNv], yseq[kNv], scale;
    double h = htry, hnew, err = 0.0, fac;
    int k_targ = c_bs.k_targ0, k = 0, nrej = 0;
    bool firstk = true, forward = h > 0;
    work[0] = 0.0;
    for (int i = 0; i < kNv; i++) ysav[i] = y[i];
    if (h != hnext_in && !c.first_step) c.last_step = true;
    if (c.reject) {
        c.prev_reject = true;
        c.last_step = false;
    }
    c.reject = false;
    hnew = fabs(h);
    while (firstk || c.reject) {
        h = forward ? hnew : -hnew;
        firstk = false;
        c.reject = false;
        if (max_rejects > 0 && nrej++ > max_rejects) return ST_STEP_LIMIT;
        for (k = 0; k <= k_targ + 1; k++) {
            midpoint(f, uform, x, ysav, dydx, h, c_bs.nseq[k], yseq, status);
            if (k == 0) {
                for (int i = 0; i < kNv; i++) y[i] = yseq[i];
            } else {
                for (int i = 0; i < kNv; i++) table[k - 1][i] = yseq[i];
            }
            if (k != 0) {
                // polyextr, src/unused/StepperBS.c:419-435
                for (int j = k - 1; j > 0; j--)
                    for (int i = 0; i < kNv; i++)
                        table[j - 1][i] = table[j][i] + c_bs.coeff[k][j] * (table[j][i] - table[j - 1][i]);
                for (int i = 0; i < kNv; i++)
                    y[i] = table[0][i] + c_bs.coeff[k][0] * (table[0][i] - y[i]);
                err = 0.0;
                for (int i = 0; i < kNv; i++) {
                    scale = c_bs.atol + c_bs.rtol * fmax(fabs(ysav[i]), fabs(y[i]));
                    // pow(q, 2.0) of the reference: the correctly rounded square, q * q
                    const double q = (y[i] - table[0][i]) / scale;
                    err += q * q;
                }
                err = sqrt(err / kNv);
                if (nan_rejects && !(err == err)) {
                    // a trial that left the domain of the equations (|beta| >= 1):
                    // reject and retry a quarter of the step; the reference
                    // accepts it because every comparison with NaN is false
                    c.reject = true;
                    hnew = 0.25 * fabs(h);
                    break;
                }
                const double expo = c_bs.expo[k];
                const double facmin = c_bs.facmin[k];
                if (err == 0.0) {
                    fac = 1.0 / facmin;
                } else {
                    fac = STEPFAC2 / pow(err / STEPFAC1, expo);
                    fac = fmax(facmin / STEPFAC4, fmin(1.0 / facmin, fac));
                }
                hopt[k] = fabs(h * fac);
                work[k] = c_bs.cost[k] / hopt[k];
                if ((c.first_step || c.last_step) && err <= 1.0) break;
                if (k == k_targ - 1 && !c.prev_reject && !c.first_step && !c.last_step) {
                    if (err <= 1.0) break;
                    // pow(integer ratio, 2.0) of the reference: an exact square
                    else if (err > sqr_int(c_bs.nseq[k_targ] * c_bs.nseq[k_targ + 1] /
                                           (c_bs.nseq[0] * c_bs.nseq[0]))) {
                        c.reject = true;
                        k_targ = k;
                        if (k_targ > 1 && work[k - 1] < KFAC1 * work[k]) k_targ--;
                        hnew = hopt[k_targ];
                        break;
                    }
                }
                if (k == k_targ) {
                    if (err <= 1.0) break;
                    else if (err > sqr((double)c_bs.nseq[k + 1] / c_bs.nseq[0])) {
                        c.reject = true;
                        if (k_targ > 1 && work[k - 1] < KFAC1 * work[k]) k_targ--;
                        hnew = hopt[k_targ];
                        break;
                    }
                }
                if (k == k_targ + 1) {
                    if (err > 1.0) {
                        c.reject = true;
                        if (k_targ > 1 && work[k_targ - 1] < KFAC1 * work[k_targ]) k_targ--;
                        hnew = hopt[k_targ];
                    }
                    break;
                }
            }
        }
        if (c.reject) c.prev_reject = true;
    }
    double dydxnew[kNv];
    derivs(f, uform, x + h, y, dydxnew, status);
    for (int i = 0; i < kNv; i++) dydx[i] = dydxnew[i];
    x += h;
    hdid = h;
    c.first_step = false;
    int kopt;
    if (k == 1) {
        kopt = 2;
    } else if (k <= k_targ) {
        kopt = k;
        if (work[k - 1] < KFAC1 * work[k]) kopt = k - 1;
        else if (work[k] < KFAC2 * work[k - 1]) kopt = min(k + 1, KMAXX - 1);
    } else {
        kopt = k - 1;
        if (k > 2 && work[k - 2] < KFAC1 * work[k - 1]) kopt = k - 2;
        if (work[k] < KFAC2 * work[kopt]) kopt = min(k, KMAXX - 1);
    }
    if (c.prev_reject) {
        k_targ = min(kopt, k);
        hnew = fmin(fabs(h), hopt[k_targ]);
        c.prev_reject = false;
    } else {
        if (kopt <= k) {
            hnew = hopt[kopt];
        } else {
            if (k < k_targ && work[k] < KFAC2 * work[k - 1])
                hnew = hopt[k] * c_bs.cost[kopt + 1] / c_bs.cost[k];
            else
                hnew = hopt[k] * c_bs.cost[kopt] / c_bs.cost[k];
        }
        k_targ = kopt;
    }
    hnext_out = forward ? hnew : -hnew;
    return 0;
}

__device__ __forceinline__ double gamma_of(int uform, const double* y)
{
    double s = y[3] * y[3] + y[4] * y[4] + y[5] * y[5];
    return uform ? sqrt(1.0 + s) : 1.0 / sqrt(1.0 - s);
}

__device__ __forceinline__ int ebin(const double* thr, int nbins, double e)
{
    if (!(e < INFINITY)) return 0;
    int lo = 0, hi = nbins - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(thr + mid - 1) <= e) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Parity mode: exactly nsteps accepted steps per particle, every step recorded.
__global__ void bs_steps_kernel(DevField f, BsArgs a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double y[kNv], dydx[kNv];
    for (int k = 0; k < kNv; k++) y[k] = a.y[kNv * i + k];
    double x = a.t[i], h = a.h[i], hnext = h, hdid = 0.0;
    Ctrl c;
    derivs(f, a.uform, x, y, dydx, a.status);
    int st = 0;
    for (int s = 0; s < a.nsteps && st == 0; s++) {
        st = bs_step(f, a.uform, a.max_rejects, false, x, y, dydx, h, h, c, hdid, hnext, a.status);
        double* r = a.rec + ((size_t)i * a.nsteps + s) * 8;
        r[0] = x;
        r[1] = hdid;
        for (int k = 0; k < kNv; k++) r[2 + k] = y[k];
        h = hnext;
    }
    for (int k = 0; k < kNv; k++) a.y[kNv * i + k] = y[k];
    a.t[i] = x;
    a.h[i] = h;
    a.pstatus[i] = st;
}

// Diffusion sums and energy bin of one particle landing on frame `frame`.
__device__ void frame_diagnostics(const DevField& f, const BsArgs& a, int frame, double x, double t0,
                                  const double* y, const double* y0)
{
    double g = gamma_of(a.uform, y);
    atomicAdd(&a.espect[frame * a.nbins + ebin(a.ebin_thr, a.nbins, g - 1.0)], 1u);
    // diffusion coefficients at the frame, src/diagnostics.c:659-705
    double tt = x * 2.0 - t0 * 2.0 + a.t_end / a.nt_out;
    double d0 = y0[0] - y[0], d1 = y0[1] - y[1], d2 = y0[2] - y[2];
    double g0 = gamma_of(a.uform, y0);
    double u[3], u0[3];
    for (int k = 0; k < 3; k++) {
        u[k] = a.uform ? y[3 + k] : g * y[3 + k];
        u0[k] = a.uform ? y0[3 + k] : g0 * y0[3 + k];
    }
    double du0 = u0[0] - u[0], du1 = u0[1] - u[1], du2 = u0[2] - u[2];
    double e[6], e0[6];
    emf64<TP_SYS_WLCS>(f, y[0], y[1], y[2], x, e, a.status);
    emf64<TP_SYS_WLCS>(f, y0[0], y0[1], y0[2], t0, e0, a.status);
    double mu = (e[0] * u[0] + e[1] * u[1] + e[2] * u[2]) /
                (sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
    double mu0 = (e0[0] * u0[0] + e0[1] * u0[1] + e0[2] * u0[2]) /
                 (sqrt(e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2]) * sqrt(u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]));
    double th = acos(mu) * 180 / TP_PI, th0 = acos(mu0) * 180 / TP_PI;
    double v[8];
    v[1] = d0 * d0 / tt; v[2] = d1 * d1 / tt; v[3] = d2 * d2 / tt;
    v[0] = v[1] + v[2] + v[3];
    v[4] = (du0 * du0 + du1 * du1 + du2 * du2) / tt;
    v[5] = (mu - mu0) * (mu - mu0) / tt;
    v[6] = (th - th0) * (th - th0) / tt;
    v[7] = (g - g0) * (g - g0) / tt;
    double* slot = a.dframe + (size_t)(frame + 1) * 8;
    for (int k = 0; k < 8; k++) atomicAdd(slot + k, v[k]);
}

// Production mode: every particle from its t to t_end; step sizes clipped to
// land on the nt_out frame times t_end * (f+1) / nt_out, where the energy
// spectrum and diffusion sums are taken.
//
// The stepper of bs_step restated as a state machine whose every turn makes
// exactly one derivs call (a midpoint substep, the derivative at the end of
// an accepted step, or the first derivative of a new particle): the lanes of
// a warp sit at different points of their own steps, but all of them run the
// field evaluation -- the bulk of the work -- together instead of one path at
// a time.  The arithmetic and its order are those of bs_step.
//
// The extrapolation that ends a midpoint sequence (the tableau, the error
// norm, the step control with its pow) is the other large block, and each
// lane reaches it on its own turn.  An FP64 instruction costs the pipe the
// same time with one active lane as with 32 on this part, so a lane whose
// sequence is complete holds its last derivative and waits (P_READY) until at
// least TP_BS_EX_NUM / TP_BS_EX_DEN of the warp's lanes are ready; then the
// ready lanes extrapolate together.  Waiting changes no particle's arithmetic
// (TP_BS_EX_NUM 0 disables it).
#ifndef TP_BS_EX_NUM
#define TP_BS_EX_NUM 1
#endif
#ifndef TP_BS_EX_DEN
#define TP_BS_EX_DEN 2
#endif
__global__ void __launch_bounds__(128) bs_track_kernel(DevField f, BsArgs a)
{
    enum : int { P_INIT, P_MID, P_FINAL, P_READY };
    const double STEPFAC1 = 0.65, STEPFAC2 = 0.94, STEPFAC4 = 4.0;
    const double KFAC1 = 0.8, KFAC2 = 0.9;
    const int KMAXX = c_bs.kmaxx;
    // particle
    int i = atomicAdd(a.next, 1);
    double y[kNv], dydx[kNv], y0[kNv];
    double x = 0.0, t0 = 0.0, hnext = 0.0, tf = 0.0;
    int st = 0, nacc = 0, frame = 0;
    Ctrl c;
    // step and attempt
    double table[kImax][kNv], hopt[kImax], work[kImax], ysav[kNv];
    double h = 0.0, hnew = 0.0, htry = 0.0, hprev = 0.0, err = 0.0;
    int k_targ = 0, k = 0, nrej = 0;
    bool forward = true, clip = false;
    // midpoint
    double ym[kNv], yn[kNv], ydr[kNv], hh = 0.0, xnew = 0.0;
    int nn = 0;
    int phase = P_INIT;
    if (i < a.n) {
        for (int q = 0; q < kNv; q++) {
            y[q] = a.y[kNv * i + q];
            y0[q] = a.y0[kNv * i + q];
        }
        x = a.t[i];
        hnext = a.h[i];
    }
    // each turn: one derivs call per lane that still has a particle
    while (i < a.n) {
        // the extrapolation runs this turn for the lanes ready for it when
        // enough of the warp's lanes are
        bool run_ex = true;
        if (TP_BS_EX_NUM > 0) {
            const unsigned act = __activemask();
            const unsigned rdy = __ballot_sync(act, phase == P_READY);
            run_ex = __popc(rdy) * TP_BS_EX_DEN >= __popc(act) * TP_BS_EX_NUM;
        }
        if (phase == P_READY && !run_ex) continue;
        // one call site, so that the lanes of a warp run it together
        double yd[kNv], ye[kNv];
        if (phase == P_READY) {
            for (int q = 0; q < kNv; q++) yd[q] = ydr[q];
        } else {
            for (int q = 0; q < kNv; q++) ye[q] = phase == P_MID ? yn[q] : y[q];
            const double xe = phase == P_MID ? xnew : phase == P_FINAL ? x + h : x;
            derivs(f, a.uform, xe, ye, yd, a.status);
        }

        bool begin_step = false;   // set up the next step of this particle
        bool finish = false;       // this particle is done (or failed)
        if (phase == P_INIT) {
            for (int q = 0; q < kNv; q++) dydx[q] = yd[q];
            t0 = x;
            c = Ctrl();
            st = 0;
            nacc = 0;
            frame = 0;
            tf = a.t_end * (frame + 1) / a.nt_out;
            begin_step = true;
        } else if (phase == P_MID || phase == P_READY) {
            if (phase == P_MID && nn + 1 < c_bs.nseq[k]) {  // the next substep of the midpoint
                const double h2 = 2.0 * hh;
                for (int q = 0; q < kNv; q++) {
                    double swap = ym[q] + h2 * yd[q];
                    ym[q] = yn[q];
                    yn[q] = swap;
                }
                xnew += hh;
                nn++;
                continue;
            }
            if (phase == P_MID && !run_ex) {  // the sequence is complete: wait for the others
                for (int q = 0; q < kNv; q++) ydr[q] = yd[q];
                phase = P_READY;
                continue;
            }
            phase = P_MID;
            double yseq[kNv];
            for (int q = 0; q < kNv; q++) yseq[q] = 0.5 * (ym[q] + yn[q] + hh * yd[q]);
            // level k of the extrapolation (the loop body of bs_step)
            int outcome = 0;  // 0: next level, 1: accept, 2: reject
            if (k == 0) {
                for (int q = 0; q < kNv; q++) y[q] = yseq[q];
            } else {
                for (int q = 0; q < kNv; q++) table[k - 1][q] = yseq[q];
                for (int j = k - 1; j > 0; j--)
                    for (int q = 0; q < kNv; q++)
                        table[j - 1][q] = table[j][q] + c_bs.coeff[k][j] * (table[j][q] - table[j - 1][q]);
                for (int q = 0; q < kNv; q++) y[q] = table[0][q] + c_bs.coeff[k][0] * (table[0][q] - y[q]);
                err = 0.0;
                for (int q = 0; q < kNv; q++) {
                    double scale = c_bs.atol + c_bs.rtol * fmax(fabs(ysav[q]), fabs(y[q]));
                    const double r = (y[q] - table[0][q]) / scale;
                    err += r * r;
                }
                err = sqrt(err / kNv);
                if (!(err == err)) {  // left the domain of the equations: retry a quarter step
                    c.reject = true;
                    hnew = 0.25 * fabs(h);
                    outcome = 2;
                } else {
                    const double expo = c_bs.expo[k], facmin = c_bs.facmin[k];
                    double fac;
                    if (err == 0.0) {
                        fac = 1.0 / facmin;
                    } else {
                        fac = STEPFAC2 / pow(err / STEPFAC1, expo);
                        fac = fmax(facmin / STEPFAC4, fmin(1.0 / facmin, fac));
                    }
                    hopt[k] = fabs(h * fac);
                    work[k] = c_bs.cost[k] / hopt[k];
                    if ((c.first_step || c.last_step) && err <= 1.0) {
                        outcome = 1;
                    } else if (k == k_targ - 1 && !c.prev_reject && !c.first_step && !c.last_step &&
                               (err <= 1.0 || err > sqr_int(c_bs.nseq[k_targ] * c_bs.nseq[k_targ + 1] /
                                                            (c_bs.nseq[0] * c_bs.nseq[0])))) {
                        if (err <= 1.0) {
                            outcome = 1;
                        } else {
                            c.reject = true;
                            k_targ = k;
                            if (k_targ > 1 && work[k - 1] < KFAC1 * work[k]) k_targ--;
                            hnew = hopt[k_targ];
                            outcome = 2;
                        }
                    } else if (k == k_targ &&
                               (err <= 1.0 || err > sqr((double)c_bs.nseq[k + 1] / c_bs.nseq[0]))) {
                        if (err <= 1.0) {
                            outcome = 1;
                        } else {
                            c.reject = true;
                            if (k_targ > 1 && work[k - 1] < KFAC1 * work[k]) k_targ--;
                            hnew = hopt[k_targ];
                            outcome = 2;
                        }
                    } else if (k == k_targ + 1) {
                        if (err > 1.0) {
                            c.reject = true;
                            if (k_targ > 1 && work[k_targ - 1] < KFAC1 * work[k_targ]) k_targ--;
                            hnew = hopt[k_targ];
                            outcome = 2;
                        } else {
                            outcome = 1;
                        }
                    }
                }
            }
            if (outcome == 0) {  // the next level's midpoint
                k++;
                hh = h / c_bs.nseq[k];
                for (int q = 0; q < kNv; q++) {
                    ym[q] = ysav[q];
                    yn[q] = ysav[q] + hh * dydx[q];
                }
                xnew = x + hh;
                nn = 0;
                continue;
            }
            if (outcome == 1) {  // accepted: the derivative at the end of the step
                phase = P_FINAL;
                continue;
            }
            // rejected: a new attempt of the same step
            c.prev_reject = true;
            h = forward ? hnew : -hnew;
            c.reject = false;
            if (a.max_rejects > 0 && nrej++ > a.max_rejects) {
                st = ST_STEP_LIMIT;
                finish = true;
            } else {
                k = 0;
                hh = h / c_bs.nseq[0];
                for (int q = 0; q < kNv; q++) {
                    ym[q] = ysav[q];
                    yn[q] = ysav[q] + hh * dydx[q];
                }
                xnew = x + hh;
                nn = 0;
                continue;
            }
        } else {  // P_FINAL: the step is accepted
            for (int q = 0; q < kNv; q++) dydx[q] = yd[q];
            x += h;
            const double hdid = h;
            c.first_step = false;
            int kopt;
            if (k == 1) {
                kopt = 2;
            } else if (k <= k_targ) {
                kopt = k;
                if (work[k - 1] < KFAC1 * work[k]) kopt = k - 1;
                else if (work[k] < KFAC2 * work[k - 1]) kopt = min(k + 1, KMAXX - 1);
            } else {
                kopt = k - 1;
                if (k > 2 && work[k - 2] < KFAC1 * work[k - 1]) kopt = k - 2;
                if (work[k] < KFAC2 * work[kopt]) kopt = min(k, KMAXX - 1);
            }
            if (c.prev_reject) {
                k_targ = min(kopt, k);
                hnew = fmin(fabs(h), hopt[k_targ]);
                c.prev_reject = false;
            } else {
                if (kopt <= k) {
                    hnew = hopt[kopt];
                } else {
                    if (k < k_targ && work[k] < KFAC2 * work[k - 1])
                        hnew = hopt[k] * c_bs.cost[kopt + 1] / c_bs.cost[k];
                    else
                        hnew = hopt[k] * c_bs.cost[kopt] / c_bs.cost[k];
                }
                k_targ = kopt;
            }
            const double hn = forward ? hnew : -hnew;
            nacc++;
            hnext = clip ? fmax(hn, hprev) : hn;
            bool bad = false;
            for (int q = 0; q < kNv; q++) bad |= !(y[q] == y[q]);
            if (bad) {
                st = ST_NONFINITE;
                finish = true;
            } else {
                if (clip && fabs(hdid - htry) <= 4.0 * 2.22e-16 * fabs(tf)) {
                    x = tf;  // landed on the frame time
                    frame_diagnostics(f, a, frame, x, t0, y, y0);
                    frame++;
                    if (frame < a.nt_out) tf = a.t_end * (frame + 1) / a.nt_out;
                }
                begin_step = true;
            }
        }
        if (begin_step) {  // the checks before a step and the start of bs_step
            if (frame >= a.nt_out) {
                finish = true;
            } else if (nacc >= a.max_steps) {
                st = ST_STEP_LIMIT;
                finish = true;
            } else {
                hprev = hnext;
                htry = hnext;
                clip = false;
                if (x + htry >= tf) {
                    htry = tf - x;
                    clip = true;
                }
                if (!(fabs(htry) > fabs(x) * 2.22045e-16)) {
                    st = ST_UNDERFLOW;
                    finish = true;
                } else {
                    h = htry;
                    k_targ = c_bs.k_targ0;
                    k = 0;
                    nrej = 0;
                    forward = h > 0;
                    work[0] = 0.0;
                    for (int q = 0; q < kNv; q++) ysav[q] = y[q];
                    if (h != hprev && !c.first_step) c.last_step = true;
                    if (c.reject) {
                        c.prev_reject = true;
                        c.last_step = false;
                    }
                    c.reject = false;
                    hnew = fabs(h);
                    // first attempt
                    h = forward ? hnew : -hnew;
                    if (a.max_rejects > 0 && nrej++ > a.max_rejects) {
                        st = ST_STEP_LIMIT;
                        finish = true;
                    } else {
                        hh = h / c_bs.nseq[0];
                        for (int q = 0; q < kNv; q++) {
                            ym[q] = ysav[q];
                            yn[q] = ysav[q] + hh * dydx[q];
                        }
                        xnew = x + hh;
                        nn = 0;
                        phase = P_MID;
                    }
                }
            }
        }
        if (finish) {
            for (int q = 0; q < kNv; q++) a.y[kNv * i + q] = y[q];
            a.t[i] = x;
            a.h[i] = hnext;
            a.steps[i] = nacc;
            a.pstatus[i] = st;
            if (st) atomicOr(a.status, st);
            i = atomicAdd(a.next, 1);
            if (i < a.n) {
                for (int q = 0; q < kNv; q++) {
                    y[q] = a.y[kNv * i + q];
                    y0[q] = a.y0[kNv * i + q];
                }
                x = a.t[i];
                hnext = a.h[i];
                phase = P_INIT;
            }
        }
    }
}

static bool set_const(double atol, double rtol, int kmaxx)
{
    BsConst h;
    memset(&h, 0, sizeof(h));
    if (kmaxx < 2 || kmaxx + 1 > kImax) {
        set_error(11, "kmaxx must lie in [2, %d]", kImax - 1);
        return false;
    }
    const int IMAXX = kmaxx + 1;
    for (int i = 0; i < IMAXX; i++) h.nseq[i] = 2 * (i + 1);
    h.cost[0] = h.nseq[0] + 1;
    for (int k = 0; k < kmaxx; k++) h.cost[k + 1] = h.cost[k] + h.nseq[k + 1];
    double logfact = -log10(fmax(1.0e-12, rtol)) * 0.6 + 0.5;
    int kt = (int)logfact;
    if (kt > kmaxx - 1) kt = kmaxx - 1;
    if (kt < 1) kt = 1;
    h.k_targ0 = kt;
    for (int k = 0; k < IMAXX; k++)
        for (int l = 0; l < k; l++) {
            double ratio = (double)(h.nseq[k]) / h.nseq[l];
            h.coeff[k][l] = 1.0 / (ratio * ratio - 1.0);
        }
    for (int k = 0; k < IMAXX; k++) {
        h.expo[k] = 1.0 / (2 * k + 1);
        h.facmin[k] = pow(0.02, h.expo[k]);  // STEPFAC3 of the step control
    }
    h.kmaxx = kmaxx;
    h.atol = atol;
    h.rtol = rtol;
    return cuda_ok(cudaMemcpyToSymbolAsync(c_bs, &h, sizeof(h), 0, cudaMemcpyHostToDevice, g.stream),
                   "bs constants");
}

}  // namespace bs
}  // namespace tp

using namespace tp;

static Scratch s_bs_y, s_bs_rec, s_bs_aux, s_bs_spec;

// Parity mode: n particles, nsteps accepted steps each; rec: n * nsteps * 8.
extern "C" int tp_bs_steps(int n, double* y, double t0, double h0, int nsteps, double atol,
                           double rtol, int kmaxx, int uform, double* rec)
{
    DevField f;
    if (!build_field(TP_SYS_WLCS, f)) return -1;
    if (!bs::set_const(atol, rtol, kmaxx)) return -1;
    if (n <= 0) return 0;
    double* dy = (double*)s_bs_y.get(sizeof(double) * 6 * (size_t)n);
    double* drec = (double*)s_bs_rec.get(sizeof(double) * 8 * (size_t)n * nsteps);
    char* aux = (char*)s_bs_aux.get((sizeof(double) * 2 + sizeof(int)) * (size_t)n);
    if (!dy || !drec || !aux) return -1;
    double* dt = (double*)aux;
    double* dh = dt + n;
    int* dst = (int*)(dh + n);
    std::vector<double> th(n, t0), hh(n, h0);
    cudaMemcpyAsync(dy, y, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, g.stream);
    cudaMemcpyAsync(dt, th.data(), sizeof(double) * n, cudaMemcpyHostToDevice, g.stream);
    cudaMemcpyAsync(dh, hh.data(), sizeof(double) * n, cudaMemcpyHostToDevice, g.stream);
    bs::BsArgs a;
    memset(&a, 0, sizeof(a));
    a.n = n; a.uform = uform; a.max_rejects = 200; a.nsteps = nsteps; a.rec = drec;
    a.y = dy; a.t = dt; a.h = dh; a.pstatus = dst; a.status = g.d_status;
    bs::bs_steps_kernel<<<(n + 63) / 64, 64, 0, g.stream>>>(f, a);
    if (!cuda_ok(cudaGetLastError(), "bs_steps")) return -1;
    cudaMemcpyAsync(rec, drec, sizeof(double) * 8 * (size_t)n * nsteps, cudaMemcpyDeviceToHost, g.stream);
    cudaMemcpyAsync(y, dy, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, g.stream);
    return cuda_ok(cudaStreamSynchronize(g.stream), "bs_steps sync") ? 0 : -1;
}

// Production mode: integrate n particles (y: n * 6, t: n, in/out) to t_end.
extern "C" int tp_bs_run(int n, double* y, double* t, double t_end, int nt_out, int nbins,
                         double h0, double atol, double rtol, int kmaxx, int uform, int max_steps,
                         int* steps_out, int* status_out, double* espect, double* dframe,
                         tp_run_info* info)
{
    DevField f;
    if (!build_field(TP_SYS_WLCS, f)) return -1;
    if (!bs::set_const(atol, rtol, kmaxx)) return -1;
    if (!ensure_thresholds(nbins)) return -1;
    if (n <= 0 || nt_out < 1) {
        set_error(1, "tp_bs_run: need particles and frames");
        return -1;
    }
    if ((long long)nt_out * nbins > INT_MAX) {  // the kernel indexes the spectrum with 32-bit integers
        set_error(1, "tp_bs_run: spectra of %d frames x %d bins: not supported", nt_out, nbins);
        return -1;
    }
    size_t nspec = (size_t)nt_out * nbins;
    double* dy = (double*)s_bs_y.get(sizeof(double) * 12 * (size_t)n);
    char* aux = (char*)s_bs_aux.get((sizeof(double) * 2 + sizeof(int) * 3) * (size_t)n + 16);
    char* spec = (char*)s_bs_spec.get(sizeof(unsigned) * nspec + sizeof(double) * 8 * (nt_out + 1));
    if (!dy || !aux || !spec) return -1;
    double* dy0 = dy + (size_t)6 * n;
    double* dt = (double*)aux;
    double* dh = dt + n;
    int* dsteps = (int*)(dh + n);
    int* dst = dsteps + n;
    int* dnext = dst + n;
    unsigned* dspec = (unsigned*)spec;
    double* dfr = (double*)(spec + sizeof(unsigned) * nspec + (8 - (sizeof(unsigned) * nspec) % 8) % 8);
    // keep the frame sums 8-byte aligned
    if (((size_t)dfr & 7) != 0) {
        set_error(1, "tp_bs_run: misaligned scratch");
        return -1;
    }
    std::vector<double> hh(n, h0);
    cudaStream_t s = g.stream;
    cudaMemcpyAsync(dy, y, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dy0, y, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dt, t, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dh, hh.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(dnext, 0, sizeof(int), s);
    cudaMemsetAsync(dspec, 0, sizeof(unsigned) * nspec, s);
    cudaMemsetAsync(dfr, 0, sizeof(double) * 8 * (nt_out + 1), s);
    bs::BsArgs a;
    memset(&a, 0, sizeof(a));
    a.n = n; a.uform = uform; a.max_rejects = 200; a.max_steps = max_steps;
    a.t_end = t_end; a.nt_out = nt_out; a.nbins = nbins; a.ebin_thr = g.d_thr;
    a.espect = dspec; a.dframe = dfr;
    a.y = dy; a.t = dt; a.h = dh; a.y0 = dy0; a.steps = dsteps; a.pstatus = dst; a.next = dnext;
    a.status = g.d_status;
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, bs::bs_track_kernel, 128, 0);
    if (bps < 1) bps = 1;
    int grid = g.num_sms * bps;
    int need = (n + 127) / 128;
    if (grid > need) grid = need;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    bs::bs_track_kernel<<<grid, 128, 0, s>>>(f, a);
    cudaEventRecord(e1, s);
    if (!cuda_ok(cudaGetLastError(), "bs_track")) return -1;
    std::vector<unsigned> hs(nspec);
    cudaMemcpyAsync(y, dy, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(t, dt, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (steps_out) cudaMemcpyAsync(steps_out, dsteps, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    if (status_out) cudaMemcpyAsync(status_out, dst, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hs.data(), dspec, sizeof(unsigned) * nspec, cudaMemcpyDeviceToHost, s);
    if (dframe) cudaMemcpyAsync(dframe, dfr, sizeof(double) * 8 * (nt_out + 1), cudaMemcpyDeviceToHost, s);
    if (!cuda_ok(cudaStreamSynchronize(s), "bs_track sync")) return -1;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (espect)
        for (size_t k = 0; k < nspec; k++) espect[k] = hs[k];
    if (info) {
        memset(info, 0, sizeof(*info));
        info->nt_out = nt_out;
        info->nbins = nbins;
        info->grid = grid;
        info->blocks_per_sm = bps;
        info->kernel_ms = ms;
        info->step_ms = ms;
        info->launches = 1;
        double tot = 0;
        if (steps_out)
            for (int i = 0; i < n; i++) tot += steps_out[i];
        info->pushes = tot;
    }
    return 0;
}

// particle_tracking_hybrid with tracking_method 1: the particles' own units
// (c = 1, u = gamma v), h0 = dt, frames over simul_domain.tmax.
int tp_bs_track_hybrid(int mpi_rank, int nptl, double dt, int nbins, int nt_out,
                       particles* ptl_init, int* nsteps_ptl, particles* ptl, double* espectrum,
                       double* espect_escape)
{
    (void)mpi_rank; (void)ptl_init; (void)espect_escape;
    if (system_type != TP_SYS_WLCS) {
        set_error(11, "adaptive stepping is provided for the wire-loop field (system type 1)");
        return -1;
    }
    std::vector<double> y((size_t)6 * nptl), t(nptl);
    for (int i = 0; i < nptl; i++) {
        y[6 * i] = ptl[i].x; y[6 * i + 1] = ptl[i].y; y[6 * i + 2] = ptl[i].z;
        y[6 * i + 3] = ptl[i].ux; y[6 * i + 4] = ptl[i].uy; y[6 * i + 5] = ptl[i].uz;
        t[i] = ptl[i].t;
    }
    std::vector<int> st(nptl);
    std::vector<double> esp((size_t)nt_out * nbins), dfr(8 * (nt_out + 1));
    if (tp_bs_run(nptl, y.data(), t.data(), simul_domain.tmax, nt_out, nbins, dt, 1e-10, 1e-10, 8, 1,
                  10000000, nsteps_ptl, st.data(), esp.data(), dfr.data(), nullptr) != 0)
        return -1;
    for (int i = 0; i < nptl; i++) {
        ptl[i].x = y[6 * i]; ptl[i].y = y[6 * i + 1]; ptl[i].z = y[6 * i + 2];
        ptl[i].ux = y[6 * i + 3]; ptl[i].uy = y[6 * i + 4]; ptl[i].uz = y[6 * i + 5];
        ptl[i].t = t[i];
    }
    for (size_t k = 0; k < esp.size(); k++) espectrum[k] += esp[k];
    return 0;
}
