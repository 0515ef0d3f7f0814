// tp_kernels_mixed.h -- host launchers of the mixed-precision unit.
#pragma once
#include "tp_mixed.cuh"

namespace tp {
namespace mixed {
cudaError_t launch_track(const MixField& f, const TrackBufs& b, const TrackParams& q, int grid,
                         cudaStream_t s);
int track_max_blocks_per_sm(int system_type, int nmodes);
cudaError_t launch_interleave(const float* e, const float* bf, size_t n, float4* eb, cudaStream_t s);
cudaError_t launch_emf_batch(const MixField& f, int n, const double* xyz, float* out, cudaStream_t s);
}  // namespace mixed
}  // namespace tp
