// Per-node MLP of the learned Newton warm start: forward, backward and Adam
// kernels (BF16 weights, FP32 activations and accumulation).
//
//   z1 = x W1 + b1, h1 = silu(z1)       x: kMlpIn features (normalised)
//   z2 = h1 W2 + b2, h2 = silu(z2)
//   y  = h2 W3 + b3                      kMlpOut outputs (normalised)
//
// Parameter vector (FP32 master copy, gradients, Adam moments):
//   W1 [in x hidden] row-major (k, j) at k*hidden + j, b1, W2, b2, W3, b3.
// The kernels read the weights from a BF16 copy of the same vector and the
// biases from the FP32 copy.  Gradients are accumulated per CTA in fixed
// tile order and summed over CTAs in fixed order, so training is
// bit-reproducible for a given sample order.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace eb {

constexpr int kMlpIn = 48;
constexpr int kMlpHidden = 128;
constexpr int kMlpOut = 6;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpIn * kMlpHidden;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden * kMlpOut;
constexpr int kMlpParams = kOffB3 + kMlpOut;  // 23,558

struct MlpDev {
  const float* P;           // FP32 parameters (biases are read from here)
  const __nv_bfloat16* W;   // BF16 copy of the parameters (weights are read from here)
};

// Y[r] = mlp(X[r]) for r < n (row-major, kMlpIn / kMlpOut floats per row).
cudaError_t mlp_forward(const MlpDev& m, const float* X, int64_t n, float* Y, cudaStream_t s);

// Training workspace on the device.
struct MlpTrainer {
  float *P = nullptr, *G = nullptr, *M1 = nullptr, *M2 = nullptr;  // params, gradient, Adam moments
  __nv_bfloat16* W = nullptr;                                      // BF16 copy
  float* gpart = nullptr;                                          // per-CTA partial gradients
  double* loss = nullptr;                                          // per-CTA partial losses (+ accumulator)
  int grid = 0;
  int64_t step = 0;
};

cudaError_t mlp_trainer_init(MlpTrainer& t, const float* params_host, cudaStream_t s);
void mlp_trainer_free(MlpTrainer& t);
// Loss (mean squared error over rows[0..n) and outputs) and its gradient in t.G;
// rows == nullptr: rows 0..n-1.  *loss_dev (device) receives the loss.
cudaError_t mlp_loss_grad(MlpTrainer& t, const float* X, const float* T, const int* rows, int64_t n, double* loss_dev,
                          cudaStream_t s);
// One Adam step on t.P from t.G; refreshes the BF16 copy.
cudaError_t mlp_adam(MlpTrainer& t, float lr, cudaStream_t s);
// BF16 copy of an FP32 parameter vector.
cudaError_t mlp_to_bf16(const float* P, __nv_bfloat16* W, cudaStream_t s);

}  // namespace eb
