// Banded LU preconditioner for the per-simulation GMRES.
//
// The reference factorises Ktan_free exactly with MKL PARDISO on every
// Newton iteration (src/linearsolvers.jl:15-23).  Here each simulation's
// tangent is permuted (reverse Cuthill-McKee on the node graph, 6 DOFs per
// node), copied into LAPACK-style band storage in FP32 and factorised by one
// CTA (blocked right-looking LU, no pivoting: the dynamic tangent carries the
// positive mass term 1/(βΔt²)M on its diagonal).  The FP32 factors are the
// GMRES preconditioner; GMRES itself measures and drives the FP64 residual,
// so the factorisation's rounding only costs an iteration or two.
//
// Band storage of simulation s (N = 6 n_s DOFs, half bandwidth b, ld = 2b+1):
// entry (i, j) with |i - j| <= b at A[(b + i - j) + ld * j], column-major.
#pragma once
#include "eb_internal.cuh"

namespace eb {

struct BandDev {
  float* A;                 // concatenated band storage
  const int64_t* off;       // per sim: offset of its band in A
  const int* bw;            // per sim: half bandwidth b in DOFs (0: no band, block-Jacobi)
  const int* pos;           // per global node: position in its simulation's band order
  const int* node_at;       // per (node_off[s] + position): global node id
  float* work;              // per DOF scratch (permuted vector)
  float* Linv;              // per panel: inverse of the unit-lower diagonal block (column-major)
  float* Uinv;              // per panel: inverse of the upper diagonal block (column-major)
  const int* refactor;      // per sim: 1 = refill and refactorise before this solve
};

constexpr int kPanel = 32;  // panel width of the blocked factorisation and solves

// Offset of simulation s's diagonal-block inverses: one kPanel x kPanel
// block per panel, with kPanel spare rows per simulation for the last panel.
__host__ __device__ __forceinline__ int64_t inv_base(int64_t n0, int s) {
  return (6 * n0 + (int64_t)kPanel * s) * kPanel;
}

__device__ __forceinline__ float& band_at(float* A, int b, int64_t ld, int i, int j) {
  return A[(int64_t)(b + i - j) + ld * (int64_t)j];
}

// z = M⁻¹ v on the CTA owning simulation s: gather into band order, forward
// substitution with unit L, backward substitution with U, scatter back.  The
// diagonal blocks are applied through their precomputed inverses (a 32x32
// product per block), the off-diagonal band by a row-parallel update.
// `xs` (may be null) is shared-memory room for the n permuted entries.
template <typename TV, typename TZ>
__device__ void band_solve(const BandDev& B, int s, int64_t n0, int n, const TV* __restrict__ v, TZ* __restrict__ z,
                           float* xs = nullptr) {
  const int b = B.bw[s];
  const int64_t ld = 2 * b + 1;
  float* A = B.A + B.off[s];
  float* x = xs ? xs : B.work + 6 * n0;
  const float* Li = B.Linv + inv_base(n0, s);
  const float* Ui = B.Uinv + inv_base(n0, s);
  __shared__ float yb[kPanel];
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int node = B.node_at[n0 + r / 6];           // global id of the node at position r/6
    x[r] = (float)v[6 * (node - n0) + r % 6];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // forward: L y = x (unit diagonal)
  for (int k0 = 0; k0 < n; k0 += kPanel) {
    const int kb = min(kPanel, n - k0);
    if (warp == 0) {
      const float* L = Li + (int64_t)k0 * kPanel;
      float acc = 0.f;
      for (int t = 0; t < kb; ++t) acc += L[t * kPanel + lane] * x[k0 + t];
      __syncwarp();
      if (lane < kb) {
        x[k0 + lane] = acc;
        yb[lane] = acc;
      }
    }
    __syncthreads();
    const int r1 = min(n, k0 + kb + b);
    for (int i = k0 + kb + threadIdx.x; i < r1; i += blockDim.x) {
      float acc = 0.f;
      const int t0 = max(k0, i - b);
      for (int t = t0; t < k0 + kb; ++t) acc += band_at(A, b, ld, i, t) * yb[t - k0];
      x[i] -= acc;
    }
    __syncthreads();
  }
  // backward: U x = y
  for (int k0 = ((n - 1) / kPanel) * kPanel; k0 >= 0; k0 -= kPanel) {
    const int kb = min(kPanel, n - k0);
    if (warp == 0) {
      const float* U = Ui + (int64_t)k0 * kPanel;
      float acc = 0.f;
      for (int t = 0; t < kb; ++t) acc += U[t * kPanel + lane] * x[k0 + t];
      __syncwarp();
      if (lane < kb) {
        x[k0 + lane] = acc;
        yb[lane] = acc;
      }
    }
    __syncthreads();
    const int r0 = max(0, k0 - b);
    for (int i = r0 + threadIdx.x; i < k0; i += blockDim.x) {
      float acc = 0.f;
      const int t1 = min(k0 + kb, i + b + 1);
      for (int t = k0; t < t1; ++t) acc += band_at(A, b, ld, i, t) * yb[t - k0];
      x[i] -= acc;
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int node = B.node_at[n0 + r / 6];
    z[6 * (node - n0) + r % 6] = (TZ)x[r];
  }
  __syncthreads();
}

void launch_band_fill(const Dev& d, const BandDev& B, const int* blk_row, cudaStream_t s);
cudaError_t launch_band_lu(const Dev& d, const BandDev& B, int max_b, cudaStream_t s);

}  // namespace eb
