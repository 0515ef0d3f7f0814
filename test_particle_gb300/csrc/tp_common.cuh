// tp_common.cuh -- device-side parameter blocks shared by the tracking kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tp_types.h"

namespace tp {

// Field description handed to every kernel by value.  Pointers are device
// addresses; grids are the reference's AoS {x,y,z} records, x fastest
// (src/magnetic_field.c:31-35, src/electric_field.c:31-35).
struct DevField {
    int system_type;
    int multi_tframe;
    int interp_corrected;   // 0: reference corner weights, 1: corrected
    int ellint_corrected;   // 0: reference m >= 0.9 branch, 1: corrected
    int bc_flag;
    int nx, ny, nz;
    double charge_mass;
    double xmin, xmax, ymin, ymax, zmin, zmax;
    double gdx, gdy, gdz, gdt;
    // force-free (ABC)
    double ffA, ffB, ffC, B0, lambda0;
    const double *vc_d, *va_d, *vb_d;
    // MHD / PIC float grids
    const float *vc_f, *va_f, *vb_f;
    const float *bc_f, *ba_f, *bb_f;
    const float *ec_f, *ea_f, *eb_f;
    // double-precision B / E grids (reachable only through the *_at_point API)
    const double *bc_d, *ba_d, *bb_d;
    const double *ec_d, *ea_d, *eb_d;
    // wire-loop current systems
    int nwlcs, iBessel;
    const wlcs *cfg;
    // plane-wave mode sum
    int nmodes;
    const tp_mode *modes;
};

// Output / scratch buffers of one tracking launch.
struct TrackBufs {
    // particle state, SoA, in/out
    double *x, *y, *z, *ux, *uy, *uz, *t, *xs, *ys, *zs;
    // initial state (ptl_init) for the diffusion coefficients
    const double *x0, *y0, *z0, *ux0, *uy0, *uz0, *t0;
    int *nsteps_ptl;
    const double *ebin_thr;       // nbins - 1 ascending energy thresholds
    unsigned int *espect;         // nt_out * nbins counts
    unsigned int *espect_esc;     // nt_out * nbins counts (open boundary)
    int *remain;                  // nsdc
    double *dpart;                // gridDim.x * nsdc * 8 per-block partial sums (scratch)
    // open-boundary runs in segments (null otherwise): per-particle state
    // carried from one segment to the next (kSegCarry doubles: the diffusion
    // singles, then what the mixed kernel needs to resume exactly), and the
    // escape flag at the end of the segment
    double *sg_carry;
    int *esc_out;
    int *status;                  // error word
    // trajectory diagnostics (traj_every > 0): particles records written every
    // traj_every steps at ptl_time[offset(i) + point], offset(i) = ntraj_accum[i-1]
    const double *qm;             // per-particle q/m, copied into trajectory records
    double *ptl_time;             // AoS particles records
    const int *ntraj_accum;
    int *ntraj_points;            // per-particle running point count (starts at 1)
    long ntraj_total;             // records available in ptl_time
};

struct TrackParams {
    int n;
    int estep;
    int einterval;
    int nt_out;
    int nbins;
    int nsdc;        // estep / 100 + 1
    int ntp0;        // floor(1 / einterval), as the reference starts its frame index
    int ntiles;
    int sstep;       // first step index (the reference starts at 1)
    int traj_every;  // nsteps_output when trajectory diagnostics are on, else 0
    double dt;
    // a segment of an open-boundary run (all zero for a whole run): diffusion
    // rows used before it, whether it continues a run (no initial escape
    // accounting), and the list of the q.n particles still inside the box
    int row0;
    int resumed;
    const int* idx;
};

constexpr int kDiffInterval = 100;  // tinterval_dcoeffs, src/tracking.c:34
constexpr int kBlock = 128;         // threads per block of the tracking kernels
constexpr int kSegCarry = 16;      // doubles per particle carried between segments
constexpr int kMaxSmemBins = 4096;  // per-frame block histogram in shared memory

// status bits
enum : int {
    ST_OK = 0,
    ST_BAD_INDEX = 1,     // a gather index fell outside the grid (access skipped)
    ST_NONFINITE = 2,
    ST_STEP_LIMIT = 4,    // adaptive stepper hit its per-particle step cap
    ST_UNDERFLOW = 8,     // adaptive step size underflow
    ST_TIMEOUT = 16,      // a bounded wait on the tensor-core pipeline gave up
};

}  // namespace tp
