// Learned subgrid closure (closure.cu): a 12 -> 64 -> 64 -> 2 MLP with BF16
// weights and FP32 accumulation.  Inference and the backward pass's
// contractions run on the 5th-generation tensor cores (tcgen05.mma,
// accumulators in TMEM); the delta nonlinearities and Adam run on the CUDA
// cores.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace samgpu {

constexpr int kMlpIn = 12;   // invariants per point
constexpr int kMlpK1 = 16;   // padded input width (one K = 16 MMA step)
constexpr int kMlpH = 64;    // hidden width
constexpr int kMlpOut = 2;   // C_nu, C_kappa
constexpr int kMlpN3 = 16;   // padded output width (N = 16 MMA)
constexpr int kMlpK2 = 80;   // hidden width plus the bias inputs (K = 5 x 16)
// The biases ride in the MMAs: each FP32 bias b is split exactly into three
// BF16 parts (b = hi + mid + lo) stored as weight columns that multiply
// inputs fixed at 1.0 (input columns 12..14 of the features, hidden columns
// 64..66 of the operand tiles).
constexpr int kMlpOne = 12;  // first constant-1 input column
// FP32 parameter vector: W1 (64 x 12), b1, W2 (64 x 64), b2, W3 (2 x 64), b3
constexpr int kMlpOffW1 = 0;
constexpr int kMlpOffB1 = kMlpOffW1 + kMlpH * kMlpIn;
constexpr int kMlpOffW2 = kMlpOffB1 + kMlpH;
constexpr int kMlpOffB2 = kMlpOffW2 + kMlpH * kMlpH;
constexpr int kMlpOffW3 = kMlpOffB2 + kMlpH;
constexpr int kMlpOffB3 = kMlpOffW3 + kMlpOut * kMlpH;
constexpr int kMlpParams = kMlpOffB3 + kMlpOut;  // 5122
// The outputs are coefficients C = kMlpScale * softplus(o).
constexpr float kMlpScale = 0.02f;
constexpr int kMlpTile = 128;  // points per MMA tile (M = 128)

// Device copy of the network as the tensor cores read it: BF16 weights in
// row-major [n][k], the bias parts in columns 12..14 of w1 and 64..66 of w2
// and w3, the output padded to 16 rows (padding zero).
struct MlpDev {
  __nv_bfloat16 w1[kMlpH * kMlpK1];
  __nv_bfloat16 w2[kMlpH * kMlpK2];
  __nv_bfloat16 w3[kMlpN3 * kMlpK2];
};

// Training buffers of one minibatch (device).
struct MlpBatch {
  __nv_bfloat16* h1;  // [n][64] layer-1 activations (after ReLU)
  __nv_bfloat16* h2;  // [n][64]
  float* o;           // [n][2] raw outputs
};

// params (FP32, kMlpParams) -> the BF16 device form
void mlp_pack(const float* params, MlpDev* dev, cudaStream_t s);
// x16: [n][16] BF16 inputs, columns 12..14 equal to 1.0 and 15 zero
// (16-byte aligned; loaded by TMA); coef: [n]
// (C_nu, C_kappa); batch (may be null) receives the activations for the
// backward pass; err is set on a wait timeout.  Returns the number of CTAs
// launched, or -1 when the tensor map cannot be built (nothing launched).
int mlp_forward(const __nv_bfloat16* x16, long long n, const MlpDev* dev, float2* coef, const MlpBatch* batch,
                int* err, cudaStream_t s);
// Gradient of L = mean over points and both outputs of (C - y)^2, written
// to grad (kMlpParams floats), and the loss sum into loss[0]; part holds
// mlp_partials(n) floats.
// tensor_cores: the three contractions as tcgen05 MMAs (k_mlp_bwd_tc; err
// is set on a wait timeout), else the CUDA-core kernel (k_mlp_bwd).
long long mlp_partials(long long n);
void mlp_backward(const __nv_bfloat16* x16, const float2* y, long long n, const MlpDev* dev, const MlpBatch& batch,
                  float* part, float* grad, float* loss, int* err, bool tensor_cores, cudaStream_t s);
// One Adam step on params (m, v moments), then the BF16 repack.
void mlp_adam(float* params, float* m, float* v, const float* grad, int step, float lr, MlpDev* dev,
              cudaStream_t s);
// FP32 features [n][12] -> BF16 [n][16] (columns 12..14 = 1.0, 15 = 0)
void mlp_features_bf16(const float* f, __nv_bfloat16* x16, long long n, cudaStream_t s);
// Self-test of one tensor-core tile: D(128 x 64) = A(128 x 16) B(64 x 16)^T
// in BF16 with FP32 accumulation, for the known-answer test of the MMA path.
void mlp_mma_selftest(const __nv_bfloat16* a, const __nv_bfloat16* b, float* d, int* err, cudaStream_t s);

}  // namespace samgpu
