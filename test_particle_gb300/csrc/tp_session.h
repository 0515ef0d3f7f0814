// tp_session.h -- the device-resident tracking session behind the C ABI.
#pragma once
#include "../../include/tp_gpu.h"
#include "tp_internal.h"

namespace tp {

struct RunSpec {
    int precision = TP_PREC_FP64;
    double dt = 0.0;
    int sstep = 1;
    int estep = 0;
    int einterval = 1;
    int nt_out = 1;
    int nbins = 3;
    int traj_every = 0;      // nsteps_output when trajectory diagnostics are on
    bool reset_nsteps = true;
};

struct Session {
    int cap = 0;             // particle capacity; SoA stride
    int n = 0;
    bool loaded = false;
    // SoA in the AoS field order x,y,z,qm,ux,uy,uz,t,xshift,yshift,zshift
    Scratch soa, soa0, aos, nsteps;
    Scratch spec, rem, dpart, dsum;
    Scratch traj, trajacc, trajpts;
    Scratch cmp;             // open-boundary segments: index lists, flags, carried singles
    long traj_total = 0;
    int nt_out = 0, nbins = 0, nsdc = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evb = nullptr, eve = nullptr;
    float last_ms = 0.f;
    ~Session();
    bool reserve(int n);
    bool load(const particles* ptl_init, const particles* ptl, int n);
    bool run(const RunSpec& rs, tp_run_info* info);
    // remain: departures counted on the device (negative numbers)
    bool fetch(particles* ptl, int* nsteps_ptl, double* espect, double* espect_escape,
               double* dsum, int* remain);
    bool set_traj(const int* ntraj_accum, const particles* ptl_time, int* points);
    bool get_traj(particles* ptl_time, int* points);
};

Session& cached_session();
bool derive_steps(double dt, int nt_out, int& estep, int& einterval);

}  // namespace tp
