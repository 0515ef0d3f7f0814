// bs.cu -- batched adaptive Bulirsch-Stoer stepper (placeholder entry until the kernel lands).
#include "../../include/tp_gpu.h"
#include "tp_internal.h"

int tp_bs_track_hybrid(int mpi_rank, int nptl, double dt, int nbins, int nt_out,
                       particles* ptl_init, int* nsteps_ptl, particles* ptl, double* espectrum,
                       double* espect_escape)
{
    (void)mpi_rank; (void)nptl; (void)dt; (void)nbins; (void)nt_out; (void)ptl_init;
    (void)nsteps_ptl; (void)ptl; (void)espectrum; (void)espect_escape;
    tp::set_error(9, "adaptive stepping is not available in this build");
    return -1;
}
