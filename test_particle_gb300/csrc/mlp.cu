// mlp.cu -- training and inference of the learned field model: the forward,
// data-gradient and hidden weight-gradient GEMMs on the 5th-generation tensor
// cores (tc_train.cu: tcgen05.mma, FP32 accumulation in tensor memory, fused
// bias / SiLU / SiLU-derivative epilogues), Fourier features, MSE loss, the
// bias gradients and the output layer's 6 x 256 weight gradient as
// reductions on the CUDA cores, AdamW.
//
// The model maps a position u in the periodic box (u = (x - min) / L) to the
// six field components: 64 integer-lattice frequencies f_j give the features
// sin(2 pi f_j . u), cos(2 pi f_j . u) (exact phases in 32-bit fixed point),
// then 128 -> 256 -> 256 -> 256 -> 256 -> 6 with SiLU.  Outputs are trained
// on normalised components (zero mean, unit variance per component).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/tp_gpu.h"
#include "mlp_common.cuh"
#include "tc_train.cuh"
#include "tp_internal.h"
#include "tp_mixed.cuh"

namespace tp {
namespace mlp {

// ---------------------------------------------------------------- features
// X[b][j] = sin(2 pi f_j . u_b), X[b][64 + j] = cos(...) with u in 32-bit fixed
// point, as BF16 [n][128]; with XT, also transposed [128][n] (the
// weight-gradient operand).  Eight features at a time: the row is written in
// 16-byte pieces, the transposed copy one column at a time (a warp writes 32
// consecutive samples of a column).
__global__ void features_kernel(const uint32_t* __restrict__ U, int n, const int* __restrict__ freq,
                                __nv_bfloat16* __restrict__ X, __nv_bfloat16* __restrict__ XT = nullptr)
{
    __shared__ int fs[3 * kFeat];
    for (int k = threadIdx.x; k < 3 * kFeat; k += blockDim.x) fs[k] = freq[k];
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t U0 = U[3 * i], U1 = U[3 * i + 1], U2 = U[3 * i + 2];
    uint4* row = reinterpret_cast<uint4*>(X + (size_t)i * kIn);
#pragma unroll 1
    for (int j0 = 0; j0 < kFeat; j0 += 8) {
        uint32_t sp[4], cp[4];
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
            float s0, c0, s1, c1;
            const int j = j0 + q;
            const uint32_t ph0 = (uint32_t)fs[3 * j] * U0 + (uint32_t)fs[3 * j + 1] * U1 + (uint32_t)fs[3 * j + 2] * U2;
            const uint32_t ph1 = (uint32_t)fs[3 * j + 3] * U0 + (uint32_t)fs[3 * j + 4] * U1 +
                                 (uint32_t)fs[3 * j + 5] * U2;
            __sincosf(mixed::rev_to_rad(ph0), &s0, &c0);
            __sincosf(mixed::rev_to_rad(ph1), &s1, &c1);
            sp[q / 2] = pack_bf16(s0, s1);
            cp[q / 2] = pack_bf16(c0, c1);
        }
        row[j0 / 8] = make_uint4(sp[0], sp[1], sp[2], sp[3]);
        row[(kFeat + j0) / 8] = make_uint4(cp[0], cp[1], cp[2], cp[3]);
        if (XT) {
            unsigned short* xt = reinterpret_cast<unsigned short*>(XT);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                xt[(size_t)(j0 + q) * n + i] = (unsigned short)(sp[q / 2] >> (16 * (q & 1)));
                xt[(size_t)(kFeat + j0 + q) * n + i] = (unsigned short)(cp[q / 2] >> (16 * (q & 1)));
            }
        }
    }
}

// ---------------------------------------------------------------- samples
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform positions (32-bit fixed point per axis) and the exact FP64 mode-sum
// field there (the plane-wave sum of fields_fp64.cuh in the same phase form).
__global__ void samples_kernel(uint64_t seed, long long first, int n, const tp_mode* __restrict__ modes,
                               int nmodes, double B0z, uint32_t* __restrict__ U, float* __restrict__ T)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t id = (uint64_t)(first + i);
    uint32_t u[3];
    for (int k = 0; k < 3; k++) u[k] = (uint32_t)(mix64(seed ^ (id * 3 + k) * 0xD1342543DE82EF95ull) >> 32);
    double b[3] = {0, 0, 0}, e[3] = {0, 0, 0};
    for (int m = 0; m < nmodes; m++) {
        const tp_mode& md = modes[m];
        uint64_t ph = (uint64_t)(int64_t)md.n[0] * ((uint64_t)u[0] << 32) +
                      (uint64_t)(int64_t)md.n[1] * ((uint64_t)u[1] << 32) +
                      (uint64_t)(int64_t)md.n[2] * ((uint64_t)u[2] << 32) +
                      ((uint64_t)(uint32_t)md.pad << 32);
        double c = cos((double)(int64_t)ph * 3.4061215800865545e-19);
        for (int k = 0; k < 3; k++) {
            b[k] += md.amp_b[k] * c;
            e[k] += md.amp_e[k] * c;
        }
    }
    b[2] += B0z;
    for (int k = 0; k < 3; k++) {
        U[3 * i + k] = u[k];
        T[6 * i + k] = (float)b[k];
        T[6 * i + 3 + k] = (float)e[k];
    }
}

// ---------------------------------------------------------------- loss, biases, AdamW
// dY = 2 (y - t_n) / (n * 6) with t_n the normalised target; BF16 dY padded with
// zeros to kDYld columns (one k-atom of the output layer's data-gradient GEMM);
// the kernel writes the first 8, the rest are zeroed once
constexpr int kDYld = 64;
constexpr int kWgradSplits = 80;  // most split-K parts of a weight-gradient GEMM
__global__ void loss_kernel(const float* __restrict__ Y, const float* __restrict__ T, int n,
                            const float* __restrict__ mean, const float* __restrict__ istd,
                            __nv_bfloat16* __restrict__ dY, float* __restrict__ dYf,
                            double* __restrict__ loss)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const float scale = 2.0f / ((float)n * kOut);
        float g[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int c = 0; c < kOut; c++) {
            float r = Y[(size_t)i * kOut + c] - (T[(size_t)i * kOut + c] - mean[c]) * istd[c];
            l += r * r;
            g[c] = r * scale;
            if (dYf) dYf[(size_t)i * kOut + c] = g[c];
        }
        // columns 8.. of dY stay zero from its allocation (mlp_reserve)
        *reinterpret_cast<uint4*>(dY + (size_t)i * kDYld) =
            make_uint4(pack_bf16(g[0], g[1]), pack_bf16(g[2], g[3]), pack_bf16(g[4], g[5]), pack_bf16(g[6], g[7]));
    }
    for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)l);
}

// db[c] += sum_rows G[row][c] (BF16 rows of width ld)
// db[c] += sum over the n samples of GT[c][*] (the gradient transposed, one row
// per feature, so every block reads one contiguous row); one block per
// feature, a fixed summation order.
__global__ void bias_grad_kernel(const __nv_bfloat16* __restrict__ GT, int n, float* __restrict__ db)
{
    __shared__ float red[8];
    const uint4* row = reinterpret_cast<const uint4*>(GT + (size_t)blockIdx.x * n);
    float s = 0.f;
    for (int i = threadIdx.x; i < n / 8; i += blockDim.x) {  // 8 values per 16-byte load
        const uint4 v = row[i];
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[q]));
            s += f.x + f.y;
        }
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        db[blockIdx.x] += t;
    }
}

// The output layer's gradients from the FP32 loss gradient dYf [n][6] and the
// last hidden activations H3 [n][256]: dW4[o][k] += sum_r dYf[r][o] H3[r][k],
// db4[o] += sum_r dYf[r][o].  A block takes kOutRows consecutive samples:
// thread k owns column k of H3 and keeps six sums; FP32 atomics add the
// block's partial sums.
constexpr int kOutRows = 128;
__global__ void __launch_bounds__(256) out_grad_kernel(const float* __restrict__ dYf,
                                                       const __nv_bfloat16* __restrict__ H3, int n,
                                                       float* __restrict__ dW4, float* __restrict__ db4)
{
    __shared__ float dy[kOutRows * kOut];
    const int r0 = blockIdx.x * kOutRows, nr = min(kOutRows, n - r0);
    for (int i = threadIdx.x; i < nr * kOut; i += blockDim.x) dy[i] = dYf[(size_t)r0 * kOut + i];
    __syncthreads();
    const int k = threadIdx.x;
    float acc[kOut] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int r = 0; r < nr; r++) {
        const float h = __bfloat162float(H3[(size_t)(r0 + r) * kHid + k]);
#pragma unroll
        for (int o = 0; o < kOut; o++) acc[o] = fmaf(dy[r * kOut + o], h, acc[o]);
    }
#pragma unroll
    for (int o = 0; o < kOut; o++) atomicAdd(&dW4[o * kHid + k], acc[o]);
    if (k < kOut) {
        float t = 0.f;
        for (int r = 0; r < nr; r++) t += dy[r * kOut + k];
        atomicAdd(&db4[k], t);
    }
}

struct Adam {
    float lr, b1, b2, eps, wd, c1, c2;  // c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t)
};

__global__ void adamw_kernel(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                             float* __restrict__ v, int n, Adam a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = gr[i];
    float mi = a.b1 * m[i] + (1.f - a.b1) * g;
    float vi = a.b2 * v[i] + (1.f - a.b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float upd = (mi * a.c1) / (sqrtf(vi * a.c2) + a.eps);
    p[i] = p[i] - a.lr * (upd + a.wd * p[i]);
}

// BF16 copies of layer weights: W [out_pad][in] and its transpose [in][out_pad]
__global__ void to_bf16_kernel(const float* __restrict__ w, int out, int out_pad, int in,
                               __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= out_pad * in) return;
    int o = i / in, k = i % in;
    __nv_bfloat16 v = __float2bfloat16(o < out ? w[(size_t)o * in + k] : 0.f);
    wb[i] = v;
    if (wt) wt[(size_t)k * out_pad + o] = v;
}

// The output layer's weights transposed and padded to one k-atom: WT4 [256][64],
// WT4[k][o] = W4[o][k] for o < kOut, zero beyond.
__global__ void wt4_pad_kernel(const __nv_bfloat16* __restrict__ wt4, __nv_bfloat16* __restrict__ wt4p)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kHid * kDYld) return;
    int k = i / kDYld, o = i % kDYld;
    wt4p[i] = o < kOutPad ? wt4[(size_t)k * kOutPad + o] : __float2bfloat16(0.f);
}

}  // namespace mlp

// ---------------------------------------------------------------- host model
using namespace mlp;

struct MlpState {
    bool ready = false;
    int freq_h[kFeat * 3];
    // parameters (FP32 master), gradients, Adam moments: one flat buffer each
    size_t nparam = 0;
    size_t woff[kLayers], boff[kLayers];
    float *p = nullptr, *gr = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wb[kLayers] = {}, *wt[kLayers] = {};
    __nv_bfloat16* wt4p = nullptr;          // [256][64] output weights transposed, padded
    unsigned char* wpack = nullptr;         // kPackBytes, tensor-core inference layout
    int* freq = nullptr;
    float out_mean[kOut] = {0}, out_std[kOut] = {1, 1, 1, 1, 1, 1};
    float *d_mean = nullptr, *d_istd = nullptr;
    long step = 0;
    // batch workspaces
    int cap = 0;
    __nv_bfloat16* X = nullptr;             // [cap][128]
    __nv_bfloat16 *Z[4] = {}, *H[4] = {};   // [cap][256]
    __nv_bfloat16 *G0 = nullptr, *G1 = nullptr;  // [cap][256] backward scratch
    __nv_bfloat16* dY = nullptr;            // [cap][kDYld]
    __nv_bfloat16* XT = nullptr;            // [128][n] features transposed
    __nv_bfloat16* HT[4] = {};              // [256][n] activations transposed
    __nv_bfloat16* GT = nullptr;            // [256][n] pre-activation gradient transposed
    float* partial = nullptr;               // split-K partial weight gradients
    float* Y = nullptr;                     // [cap][6]
    float* dYf = nullptr;                   // [cap][6]
    double* loss = nullptr;
};

static MlpState M;

static bool mlp_alloc_params()
{
    if (M.p) return true;
    size_t off = 0;
    for (int l = 0; l < kLayers; l++) {
        M.woff[l] = off;
        off += (size_t)layer_out(l) * layer_in(l);
        M.boff[l] = off;
        off += layer_out(l);
    }
    M.nparam = off;
    size_t b = sizeof(float) * off;
    if (!cuda_ok(cudaMalloc(&M.p, b), "mlp params") || !cuda_ok(cudaMalloc(&M.gr, b), "mlp grads") ||
        !cuda_ok(cudaMalloc(&M.m, b), "mlp m") || !cuda_ok(cudaMalloc(&M.v, b), "mlp v"))
        return false;
    for (int l = 0; l < kLayers; l++) {
        size_t e = (size_t)layer_out_pad(l) * layer_in(l);
        if (!cuda_ok(cudaMalloc(&M.wb[l], sizeof(__nv_bfloat16) * e), "mlp wb") ||
            !cuda_ok(cudaMalloc(&M.wt[l], sizeof(__nv_bfloat16) * e), "mlp wt"))
            return false;
    }
    return cuda_ok(cudaMalloc(&M.wpack, kPackBytes), "mlp wpack") &&
           cuda_ok(cudaMalloc(&M.wt4p, sizeof(__nv_bfloat16) * kHid * kDYld), "mlp wt4p") &&
           cuda_ok(cudaMalloc(&M.partial, sizeof(float) * (size_t)kWgradSplits * kHid * kHid), "mlp partial") &&
           cuda_ok(cudaMalloc(&M.freq, sizeof(int) * 3 * kFeat), "mlp freq") &&
           cuda_ok(cudaMalloc(&M.d_mean, sizeof(float) * kOut), "mlp mean") &&
           cuda_ok(cudaMalloc(&M.d_istd, sizeof(float) * kOut), "mlp std") &&
           cuda_ok(cudaMalloc(&M.loss, sizeof(double)), "mlp loss");
}

// workspaces for batches of up to n samples (rounded up to a whole 128-row tile)
static bool mlp_reserve(int n)
{
    n = (n + 127) / 128 * 128;
    if (n <= M.cap) return true;
    auto fr = [](void* p) { if (p) cudaFree(p); };
    fr(M.X); fr(M.G0); fr(M.G1); fr(M.dY); fr(M.Y); fr(M.dYf); fr(M.XT); fr(M.GT);
    for (int l = 0; l < 4; l++) { fr(M.Z[l]); fr(M.H[l]); fr(M.HT[l]); }
    size_t h = sizeof(__nv_bfloat16) * (size_t)n * kHid;
    bool ok = cuda_ok(cudaMalloc(&M.X, sizeof(__nv_bfloat16) * (size_t)n * kIn), "X") &&
              cuda_ok(cudaMalloc(&M.XT, sizeof(__nv_bfloat16) * (size_t)n * kIn), "XT") &&
              cuda_ok(cudaMalloc(&M.G0, h), "G0") && cuda_ok(cudaMalloc(&M.G1, h), "G1") &&
              cuda_ok(cudaMalloc(&M.GT, h), "GT") &&
              cuda_ok(cudaMalloc(&M.dY, sizeof(__nv_bfloat16) * (size_t)n * kDYld), "dY") &&
              cuda_ok(cudaMalloc(&M.Y, sizeof(float) * (size_t)n * kOut), "Y") &&
              cuda_ok(cudaMalloc(&M.dYf, sizeof(float) * (size_t)n * kOut), "dYf");
    for (int l = 0; l < 4 && ok; l++)
        ok = cuda_ok(cudaMalloc(&M.Z[l], h), "Z") && cuda_ok(cudaMalloc(&M.H[l], h), "H") &&
             cuda_ok(cudaMalloc(&M.HT[l], h), "HT");
    // the padding columns of dY (beyond the 8 the loss kernel writes) stay zero
    if (ok) ok = cuda_ok(cudaMemsetAsync(M.dY, 0, sizeof(__nv_bfloat16) * (size_t)n * kDYld, g.stream), "dY zero");
    if (ok) M.cap = n;
    return ok;
}

static bool mlp_refresh_bf16()
{
    cudaStream_t s = g.stream;
    for (int l = 0; l < kLayers; l++) {
        int e = layer_out_pad(l) * layer_in(l);
        to_bf16_kernel<<<(e + 255) / 256, 256, 0, s>>>(M.p + M.woff[l], layer_out(l), layer_out_pad(l),
                                                       layer_in(l), M.wb[l], M.wt[l]);
    }
    wt4_pad_kernel<<<(kHid * kDYld + 255) / 256, 256, 0, s>>>(M.wt[kLayers - 1], M.wt4p);
    if (!cuda_ok(pack_weights(M.wb, M.wpack, s), "pack weights")) return false;
    float istd[kOut];
    for (int c = 0; c < kOut; c++) istd[c] = 1.0f / M.out_std[c];
    cudaMemcpyAsync(M.d_mean, M.out_mean, sizeof(float) * kOut, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(M.d_istd, istd, sizeof(float) * kOut, cudaMemcpyHostToDevice, s);
    return cuda_ok(cudaGetLastError(), "bf16 refresh");
}

// forward of n samples from features X (rows up to the next multiple of 128
// are computed too and ignored): fills Z/H (and H transposed) and Y
// (normalised outputs), on the tensor cores
static bool mlp_forward(int n)
{
    cudaStream_t s = g.stream;
    const int np = (n + 127) / 128 * 128;
    const __nv_bfloat16* in = M.X;
    int ldin = kIn;
    for (int l = 0; l < 4; l++) {
        if (!cuda_ok(tctrain::forward_hidden(in, ldin, M.wb[l], layer_in(l), np, M.p + M.boff[l], M.Z[l],
                                             M.H[l], M.HT[l], g.d_status, s),
                     "fwd gemm")) return false;
        in = M.H[l];
        ldin = kHid;
    }
    return cuda_ok(tctrain::forward_out(in, M.wb[4], np, M.p + M.boff[4], M.Y, g.d_status, s), "out gemm");
}

// backward of n samples (a multiple of 128) after mlp_forward and the loss
// kernel: fills M.gr.  Data gradients and the hidden layers' weight gradients
// on the tensor cores; bias gradients and the output layer's weight gradient
// as reductions.
static bool mlp_backward(int n)
{
    cudaStream_t s = g.stream;
    cudaMemsetAsync(M.gr, 0, sizeof(float) * M.nparam, s);
    // output layer: dW4 = dY^T H3, db4 = sum dY, dH3 = dY W4 (times silu'(Z3))
    {
        out_grad_kernel<<<(n + kOutRows - 1) / kOutRows, 256, 0, s>>>(M.dYf, M.H[3], n, M.gr + M.woff[4],
                                                                       M.gr + M.boff[4]);
        if (!cuda_ok(tctrain::backward_data(M.dY, kDYld, M.wt4p, kDYld, n, M.Z[3], M.G0, M.GT, g.d_status, s),
                     "dH3"))
            return false;
    }
    __nv_bfloat16 *gcur = M.G0, *gnext = M.G1;
    for (int l = 3; l >= 0; l--) {
        const __nv_bfloat16* xt = l == 0 ? M.XT : M.HT[l - 1];
        const int kin = layer_in(l);
        // split K (the samples) so that the two 128-row tiles fill the SMs, at
        // least four k-atoms per split
        const int splits = std::max(1, std::min({kWgradSplits, 76, n / 256}));
        if (!cuda_ok(tctrain::backward_weights(M.GT, xt, kin, n, M.partial, splits, M.gr + M.woff[l], g.d_status,
                                               s),
                     "dW"))
            return false;
        bias_grad_kernel<<<kHid, 256, 0, s>>>(M.GT, n, M.gr + M.boff[l]);
        if (l > 0) {
            if (!cuda_ok(tctrain::backward_data(gcur, kHid, M.wt[l], kHid, n, M.Z[l - 1], gnext, M.GT, g.d_status,
                                                s),
                         "dH"))
                return false;
            __nv_bfloat16* tmp = gcur;
            gcur = gnext;
            gnext = tmp;
        }
    }
    return true;
}

static bool mlp_loss(int n, const float* T, double* loss_out)
{
    cudaStream_t s = g.stream;
    cudaMemsetAsync(M.loss, 0, sizeof(double), s);
    loss_kernel<<<(n + 255) / 256, 256, 0, s>>>(M.Y, T, n, M.d_mean, M.d_istd, M.dY, M.dYf, M.loss);
    if (loss_out) {
        cudaMemcpyAsync(loss_out, M.loss, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (!cuda_ok(cudaStreamSynchronize(s), "loss")) return false;
        *loss_out /= (double)n * kOut;
    }
    return cuda_ok(cudaGetLastError(), "loss");
}

bool mlp::mlp_model(Model& md)
{
    if (!M.ready) {
        set_error(12, "the learned field model is not trained (tp_mlp_train)");
        return false;
    }
    for (int l = 0; l < kLayers; l++) {
        md.w[l] = M.wb[l];
        md.b[l] = M.p + M.boff[l];
    }
    md.freq = M.freq;
    md.wpack = M.wpack;
    for (int c = 0; c < kOut; c++) {
        md.out_scale[c] = M.out_std[c];
        md.out_shift[c] = M.out_mean[c];
    }
    return true;
}

}  // namespace tp

using namespace tp;

// Initialise the model: frequencies (kFeat x 3 lattice vectors) and weights
// (flat FP32 layout W0, b0, ..., W4, b4 with W_l [out][in]); NULL weights:
// seeded He-uniform initialisation.
extern "C" int tp_mlp_init(const int* freq, const float* weights, unsigned long long seed)
{
    if (!ensure_init() || !mlp_alloc_params()) return -1;
    memcpy(M.freq_h, freq, sizeof(int) * 3 * kFeat);
    cudaMemcpyAsync(M.freq, freq, sizeof(int) * 3 * kFeat, cudaMemcpyHostToDevice, g.stream);
    std::vector<float> h(M.nparam, 0.f);
    if (weights) {
        memcpy(h.data(), weights, sizeof(float) * M.nparam);
    } else {
        uint64_t st = seed * 2654435761ull + 1;
        auto rnd = [&]() {
            st ^= st << 13; st ^= st >> 7; st ^= st << 17;
            return (double)(st >> 11) * (1.0 / 9007199254740992.0);
        };
        for (int l = 0; l < kLayers; l++) {
            double lim = std::sqrt(6.0 / layer_in(l));
            if (l == kLayers - 1) lim *= 0.5;
            for (size_t k = 0; k < (size_t)layer_out(l) * layer_in(l); k++)
                h[M.woff[l] + k] = (float)((2.0 * rnd() - 1.0) * lim);
        }
    }
    cudaMemcpyAsync(M.p, h.data(), sizeof(float) * M.nparam, cudaMemcpyHostToDevice, g.stream);
    cudaMemsetAsync(M.m, 0, sizeof(float) * M.nparam, g.stream);
    cudaMemsetAsync(M.v, 0, sizeof(float) * M.nparam, g.stream);
    M.step = 0;
    M.ready = true;
    return mlp_refresh_bf16() && cuda_ok(cudaStreamSynchronize(g.stream), "mlp init") ? 0 : -1;
}

extern "C" int tp_mlp_param_count(void)
{
    int n = 0;
    for (int l = 0; l < kLayers; l++) n += layer_out(l) * layer_in(l) + layer_out(l);
    return n;
}

extern "C" int tp_mlp_set_output_norm(const float* mean, const float* stdv)
{
    for (int c = 0; c < kOut; c++) {
        M.out_mean[c] = mean[c];
        M.out_std[c] = stdv[c];
    }
    return M.ready && mlp_refresh_bf16() ? 0 : -1;
}

extern "C" int tp_mlp_get_weights(float* weights)
{
    if (!M.ready) return -1;
    cudaMemcpyAsync(weights, M.p, sizeof(float) * M.nparam, cudaMemcpyDeviceToHost, g.stream);
    return cuda_ok(cudaStreamSynchronize(g.stream), "get weights") ? 0 : -1;
}

// One forward + backward on given samples (u: n*3 box fractions as 32-bit fixed
// point, t: n*6 targets); returns the loss, the normalised outputs and the FP32
// gradients in the flat parameter layout.  For gradient checks.
extern "C" int tp_mlp_grad(int n, const unsigned int* u, const float* t, double* loss, float* y,
                           float* grads)
{
    if (n < 128 || n % 128) {
        set_error(12, "tp_mlp_grad: n must be a positive multiple of 128");
        return -1;
    }
    if (!M.ready || !mlp_reserve(n)) return -1;
    cudaStream_t s = g.stream;
    uint32_t* dU;
    float* dT;
    if (!cuda_ok(cudaMalloc(&dU, sizeof(uint32_t) * 3 * n), "u") ||
        !cuda_ok(cudaMalloc(&dT, sizeof(float) * 6 * n), "t")) return -1;
    cudaMemcpyAsync(dU, u, sizeof(uint32_t) * 3 * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dT, t, sizeof(float) * 6 * n, cudaMemcpyHostToDevice, s);
    features_kernel<<<(n + 127) / 128, 128, 0, s>>>(dU, n, M.freq, M.X, M.XT);
    bool ok = mlp_forward(n) && mlp_loss(n, dT, loss) && mlp_backward(n);
    if (ok) {
        if (y) cudaMemcpyAsync(y, M.Y, sizeof(float) * 6 * n, cudaMemcpyDeviceToHost, s);
        if (grads) cudaMemcpyAsync(grads, M.gr, sizeof(float) * M.nparam, cudaMemcpyDeviceToHost, s);
        ok = cuda_ok(cudaStreamSynchronize(s), "grad");
    }
    cudaFree(dU);
    cudaFree(dT);
    return ok ? 0 : -1;
}

// Train on nsamples field samples of the current mode table (tp_set_modes),
// drawn uniformly in the box from `seed` and evaluated with the FP64 mode sum.
// Output normalisation comes from the samples.  lr: peak AdamW rate with a
// cosine decay over epochs * (nsamples / batch) steps.  Returns the final
// mean loss (normalised units) in *loss_out and the device time in *ms_out.
extern "C" int tp_mlp_train(long long nsamples, int batch, int epochs, double lr, double wd,
                            unsigned long long seed, double* loss_out, double* ms_out)
{
    if (!M.ready) {
        set_error(12, "tp_mlp_init first");
        return -1;
    }
    if (g.modes.empty()) {
        set_error(12, "no mode table to learn (tp_set_modes)");
        return -1;
    }
    if (batch < 128 || batch % 128 || nsamples < batch) {
        set_error(12, "batch must be a positive multiple of 128 not above nsamples");
        return -1;
    }
    cudaStream_t s = g.stream;
    DevField f;
    if (!build_field(TP_SYS_MODESUM, f) || !mlp_reserve(batch)) return -1;
    uint32_t* dU = nullptr;
    float* dT = nullptr;
    if (!cuda_ok(cudaMalloc(&dU, sizeof(uint32_t) * 3 * (size_t)nsamples), "train u") ||
        !cuda_ok(cudaMalloc(&dT, sizeof(float) * 6 * (size_t)nsamples), "train t")) return -1;
    for (long long off = 0; off < nsamples; off += 1 << 22) {
        int cnt = (int)std::min<long long>(1 << 22, nsamples - off);
        samples_kernel<<<(cnt + 127) / 128, 128, 0, s>>>(seed, off, cnt, f.modes, f.nmodes, f.B0,
                                                         dU + 3 * off, dT + 6 * off);
    }
    // output normalisation from the training targets
    {
        std::vector<float> ht(6 * std::min<long long>(nsamples, 1 << 20));
        cudaMemcpyAsync(ht.data(), dT, sizeof(float) * ht.size(), cudaMemcpyDeviceToHost, s);
        if (!cuda_ok(cudaStreamSynchronize(s), "samples")) return -1;
        size_t cnt = ht.size() / 6;
        for (int c = 0; c < kOut; c++) {
            double a = 0, b = 0;
            for (size_t i = 0; i < cnt; i++) {
                a += ht[6 * i + c];
                b += (double)ht[6 * i + c] * ht[6 * i + c];
            }
            a /= cnt;
            double var = b / cnt - a * a;
            M.out_mean[c] = (float)a;
            M.out_std[c] = (float)std::sqrt(var > 1e-30 ? var : 1e-30);
        }
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    long long nb = nsamples / batch;
    long long total = nb * epochs;
    double loss = 0.0;
    bool ok = mlp_refresh_bf16();
    for (long long it = 0; it < total && ok; it++) {
        long long bi = it % nb;
        features_kernel<<<(batch + 127) / 128, 128, 0, s>>>(dU + 3 * bi * batch, batch, M.freq, M.X, M.XT);
        const bool last = it == total - 1;
        ok = mlp_forward(batch) && mlp_loss(batch, dT + 6 * bi * batch, last ? &loss : nullptr) &&
             mlp_backward(batch);
        if (!ok) break;
        M.step++;
        Adam a;
        double frac = (double)it / (double)total;
        a.lr = (float)(lr * 0.5 * (1.0 + std::cos(M_PI * frac)));
        a.b1 = 0.9f;
        a.b2 = 0.999f;
        a.eps = 1e-8f;
        a.wd = (float)wd;
        a.c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)M.step)));
        a.c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)M.step)));
        adamw_kernel<<<(int)((M.nparam + 255) / 256), 256, 0, s>>>(M.p, M.gr, M.m, M.v, (int)M.nparam, a);
        ok = mlp_refresh_bf16();
    }
    cudaEventRecord(e1, s);
    ok = ok && cuda_ok(cudaStreamSynchronize(s), "train");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(dU);
    cudaFree(dT);
    if (loss_out) *loss_out = loss;
    if (ms_out) *ms_out = ms;
    return ok ? 0 : -1;
}

// Model field at n positions (u: n*3 32-bit fixed point) through the training
// forward pass; out: n*6 physical components.
extern "C" int tp_mlp_eval(int n, const unsigned int* u, float* out)
{
    if (n <= 0) return 0;
    if (!M.ready || !mlp_reserve(n < 128 ? 128 : n)) return -1;
    cudaStream_t s = g.stream;
    uint32_t* dU;
    if (!cuda_ok(cudaMalloc(&dU, sizeof(uint32_t) * 3 * n), "u")) return -1;
    cudaMemcpyAsync(dU, u, sizeof(uint32_t) * 3 * n, cudaMemcpyHostToDevice, s);
    features_kernel<<<(n + 127) / 128, 128, 0, s>>>(dU, n, M.freq, M.X);
    bool ok = mlp_forward(n);
    std::vector<float> y(6 * (size_t)n);
    if (ok) {
        cudaMemcpyAsync(y.data(), M.Y, sizeof(float) * 6 * n, cudaMemcpyDeviceToHost, s);
        ok = cuda_ok(cudaStreamSynchronize(s), "eval");
    }
    cudaFree(dU);
    if (!ok) return -1;
    for (int i = 0; i < n; i++)
        for (int c = 0; c < kOut; c++) out[6 * i + c] = y[6 * i + c] * M.out_std[c] + M.out_mean[c];
    return 0;
}
