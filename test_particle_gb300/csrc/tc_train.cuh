// tc_train.cuh -- host launchers of the tensor-core training GEMMs (tc_train.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace tp {
namespace tct {
size_t smem_bytes(int n, int ring);
}
namespace tctrain {

// Z, H = silu(X W^T + b) of a hidden layer: X [M][kin] (row stride lda), W [256][kin];
// Z, H row-major [M][256], H also transposed into HT [256][M].  M a multiple of 128.
cudaError_t forward_hidden(const __nv_bfloat16* X, int lda, const __nv_bfloat16* W, int kin, int M,
                           const float* b, __nv_bfloat16* Z, __nv_bfloat16* H, __nv_bfloat16* HT, int* status,
                           cudaStream_t s);

// Y = H3 W4^T + b: H3 [M][256], W4 [16][256] (rows past the 6 outputs zero); Y FP32 [M][6].
cudaError_t forward_out(const __nv_bfloat16* H3, const __nv_bfloat16* W4, int M, const float* b, float* Y,
                        int* status, cudaStream_t s);

// G = (Gin WT^T) * silu'(Zprev): Gin [M][kout] (row stride ldg), WT [256][kout] (the
// layer's weights transposed); G row-major [M][256] and transposed into GT [256][M].
cudaError_t backward_data(const __nv_bfloat16* Gin, int ldg, const __nv_bfloat16* WT, int kout, int M,
                          const __nv_bfloat16* Zprev, __nv_bfloat16* G, __nv_bfloat16* GT, int* status,
                          cudaStream_t s);

// gr[256][kin] += GT XT^T over nsamp samples: GT [256][nsamp], XT [kin][nsamp]; split-K
// partial sums in `partial` (splits x 256 x kin FP32) reduced into gr.
cudaError_t backward_weights(const __nv_bfloat16* GT, const __nv_bfloat16* XT, int kin, int nsamp,
                             float* partial, int splits, float* gr, int* status, cudaStream_t s);

// D[M][N] = A[M][K] B[N][K]^T in FP32 (self-check).
cudaError_t gemm_f32(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, float* D, int* status,
                     cudaStream_t s);

}  // namespace tctrain
}  // namespace tp
