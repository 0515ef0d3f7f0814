// tp_kernels.h -- host-side launchers exported by each kernel translation unit.
#pragma once
#include "tp_common.cuh"

namespace tp {

#define TP_DECLARE_FP64_LAUNCHERS(NS)                                                          \
    namespace NS {                                                                             \
    cudaError_t launch_track(const DevField& f, const TrackBufs& b, const TrackParams& q,      \
                             int grid, cudaStream_t s);                                        \
    int track_max_blocks_per_sm(int system_type);                                              \
    cudaError_t launch_reduce_dpart(const double* dpart, int nblocks, int nsdc, double* dsum,  \
                                    cudaStream_t s);                                           \
    cudaError_t launch_emf_batch(const DevField& f, int n, const double* xyzt, double* out,    \
                                 int* status, cudaStream_t s);                                 \
    cudaError_t launch_wirz_steps(const DevField& f, int n, double* st, int nsteps, double dt, \
                                  int* iescape, int* status, cudaStream_t s);                  \
    cudaError_t launch_ebins(const double* thr, int nbins, int n, const double* st, int* bins, \
                             cudaStream_t s);                                                  \
    cudaError_t launch_diffc(const DevField& f, int n, const double* st0, const double* st,    \
                             double dt, double* out, int* status, cudaStream_t s);             \
    cudaError_t launch_trilinear(const DevField& f, int n, const double* xyzt, long* corners,  \
                                 double* weights, cudaStream_t s);                             \
    cudaError_t launch_bc(const DevField& f, int n, double* st, int* iescape, cudaStream_t s); \
    cudaError_t launch_point_interp(const DevField& f, int which, int n, const double* xyzt,   \
                                    double* out, int* status, cudaStream_t s);                 \
    cudaError_t launch_poincare(const DevField& f, int n, const double* seeds, int face,       \
                                double h, double lmax, int ncross, double* xo, double* yo,     \
                                double* zo, int* found, int* status, cudaStream_t s);          \
    }

TP_DECLARE_FP64_LAUNCHERS(fp64)
TP_DECLARE_FP64_LAUNCHERS(fp64fast)

}  // namespace tp
