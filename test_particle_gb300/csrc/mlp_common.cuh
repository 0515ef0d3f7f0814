// mlp_common.cuh -- the learned field model: Fourier features of the position
// followed by an MLP (128 -> 256 -> 256 -> 256 -> 256 -> 6, SiLU), BF16
// weights and activations on the tensor cores with FP32 accumulation.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace tp {
namespace mlp {

constexpr int kFeat = 64;          // lattice frequencies
constexpr int kIn = 2 * kFeat;     // sin and cos features
constexpr int kHid = 256;
constexpr int kOut = 6;            // Bx, By, Bz, Ex, Ey, Ez
constexpr int kOutPad = 16;        // output rows padded to a tensor-core tile
constexpr int kLayers = 5;

__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int layer_out(int l) { return l == kLayers - 1 ? kOut : kHid; }
__host__ __device__ constexpr int layer_out_pad(int l) { return l == kLayers - 1 ? kOutPad : kHid; }

// Device view of the trained model used for inference.
struct Model {
    const __nv_bfloat16* w[kLayers];  // [out_pad][in] row-major, BF16
    const float* b[kLayers];          // [out] FP32
    const int* freq;                  // [kFeat][3] integer lattice frequencies
    const unsigned char* wpack;       // weights in the tensor-core chunk layout (kPackBytes)
    float out_scale[kOut], out_shift[kOut];  // y = net * scale + shift
};

// Bytes of the packed weights: 32 chunks per evaluation (see track_surrogate.cu).
constexpr size_t kPackBytes = 466944;

// Device view of the trained model (host side; false and an error if untrained).
bool mlp_model(Model& md);

// Packs the BF16 weights of every layer for the tensor-core inference.
cudaError_t pack_weights(const __nv_bfloat16* const w[kLayers], unsigned char* pack, cudaStream_t s);

__device__ __forceinline__ float silu(float z)
{
    // z * sigmoid(z) = 0.5 z (1 + tanh(z / 2)): one MUFU op per element
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return 0.5f * z * (1.0f + t);
}

__device__ __forceinline__ float silu_grad(float z)
{
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    float s = 0.5f * (1.0f + t);  // sigmoid(z)
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

}  // namespace mlp
}  // namespace tp
