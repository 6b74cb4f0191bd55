// Learned Newton warm start on the device: per-node features, the predicted
// step increment, training-sample capture and per-simulation residual norms.
#pragma once
#include <cuda_bf16.h>

#include "eb_internal.cuh"
#include "eb_mlp.cuh"

namespace eb {

constexpr int kWsRaw = 39;  // raw features per node (the network input is padded to kMlpIn)

struct WsDev {
  const int* nb;          // n_nodes x 2: first two beam neighbours (the node itself when missing)
  const int* surf_on;     // per sim: 1 when the simulation has a contact surface
  float* F;               // n_nodes x kWsRaw raw features at the step's start
  float* X;               // n_nodes x kMlpIn normalised features
  float* Y;               // n_nodes x kMlpOut network outputs
  const float* in_shift;  // kMlpIn
  const float* in_scale;  // kMlpIn
  const float* out_scale; // kMlpOut
};

// Raw and normalised features of the nodes of active simulations (committed state).
void launch_ws_features(const Dev& d, const WsDev& w, cudaStream_t s);
// dD (free DOFs of active simulations) = Δt Ḋ + ½Δt² D̈ + Δt² out_scale ⊙ Y.
void launch_ws_apply(const Dev& d, const WsDev& w, cudaStream_t s);
// Appends one sample per node with (node + phase) % stride == 0 to the ring
// (slots cursor + node / stride, modulo cap): raw features at the step's start
// and the raw target (converged increment − kinematic part) / Δt²; simulations
// outside `mask` write NaN targets.
void launch_ws_capture(const Dev& d, const WsDev& w, const int* mask, int64_t phase, int stride, int64_t cursor,
                       int64_t cap, float* sF, float* sT, cudaStream_t s);
// out[s] = Σ r² over the free DOFs of active simulation s (fixed order).
void launch_ws_rnorm(const Dev& d, double* out, cudaStream_t s);

}  // namespace eb
