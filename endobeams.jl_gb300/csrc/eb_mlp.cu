// Per-node MLP kernels (see eb_mlp.cuh) and the C-ABI training/evaluation
// entry points.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/endobeams_gb300.h"
#include "eb_mlp.cuh"

int eb_internal_fail(int code, const char* msg);

namespace eb {
namespace {

constexpr int kTile = 32;      // rows per tile
constexpr int kThr = 256;      // threads per CTA
constexpr int kLdX = 52;       // shared row stride of the input tile (floats)
constexpr int kLdH = 132;      // shared row stride of hidden activations (floats)
constexpr int kOutP = 8;       // padded output width

static_assert(kMlpIn == 48 && kMlpHidden == 128 && kMlpOut == 6, "kernel tiling assumes 48-128-128-6");

struct Smem {
  __nv_bfloat16 W1[kMlpIn * kMlpHidden];
  __nv_bfloat16 W2[kMlpHidden * kMlpHidden];
  __nv_bfloat16 W2T[kMlpHidden * kMlpHidden];  // W2 transposed (backward only)
  __nv_bfloat16 W3[kMlpHidden * kOutP];
  float b1[kMlpHidden], b2[kMlpHidden], b3[kOutP];
  float x[kTile * kLdX];
  float z1[kTile * kLdH], h1[kTile * kLdH], z2[kTile * kLdH], h2[kTile * kLdH];
  float dy[kTile * kOutP];
  double red[kThr / 32];
};

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s + z * s * (1.f - s);
}

// z = in W + b over one tile (K inputs per row), h = silu(z).  Thread t owns
// rows 4 (t / 32) .. +3 and neurons 4 (t % 32) .. +3.
template <int K, int LDI>
__device__ __forceinline__ void dense_silu(const float* in, const __nv_bfloat16* Ws, const float* b, float* z, float* h) {
  const int tm = threadIdx.x >> 5, tn = threadIdx.x & 31;
  float acc[4][4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float bc = b[4 * tn + c];
#pragma unroll
    for (int a = 0; a < 4; ++a) acc[a][c] = bc;
  }
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    const __nv_bfloat162* wp = reinterpret_cast<const __nv_bfloat162*>(Ws + k * kMlpHidden + 4 * tn);
    const float2 w01 = __bfloat1622float2(wp[0]);
    const float2 w23 = __bfloat1622float2(wp[1]);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const float xv = in[(4 * tm + a) * LDI + k];
      acc[a][0] = fmaf(xv, w01.x, acc[a][0]);
      acc[a][1] = fmaf(xv, w01.y, acc[a][1]);
      acc[a][2] = fmaf(xv, w23.x, acc[a][2]);
      acc[a][3] = fmaf(xv, w23.y, acc[a][3]);
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    float* zr = z + (4 * tm + a) * kLdH + 4 * tn;
    float* hr = h + (4 * tm + a) * kLdH + 4 * tn;
    *reinterpret_cast<float4*>(zr) = make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
    *reinterpret_cast<float4*>(hr) =
        make_float4(silu(acc[a][0]), silu(acc[a][1]), silu(acc[a][2]), silu(acc[a][3]));
  }
}

// One CTA processes tiles blockIdx.x, blockIdx.x + gridDim.x, ... of 32 rows.
// TRAIN: targets T, gradient partials per CTA in gpart, loss partial in lpart.
template <bool TRAIN>
__global__ void __launch_bounds__(kThr, 1)
    k_mlp(MlpDev m, const float* __restrict__ X, const int* __restrict__ rows, int64_t n,
          const float* __restrict__ T, float* __restrict__ Y, float* __restrict__ gpart, double* __restrict__ lpart,
          float gscale) {
  extern __shared__ __align__(16) unsigned char smraw[];
  Smem& S = *reinterpret_cast<Smem*>(smraw);
  const int t = threadIdx.x;
  // ---- weights into shared memory
  for (int i = t; i < kMlpIn * kMlpHidden; i += kThr) S.W1[i] = m.W[kOffW1 + i];
  for (int i = t; i < kMlpHidden * kMlpHidden; i += kThr) {
    const __nv_bfloat16 w = m.W[kOffW2 + i];
    S.W2[i] = w;
    if (TRAIN) S.W2T[(i % kMlpHidden) * kMlpHidden + i / kMlpHidden] = w;
  }
  for (int i = t; i < kMlpHidden * kOutP; i += kThr) {
    const int k = i / kOutP, o = i % kOutP;
    S.W3[i] = o < kMlpOut ? m.W[kOffW3 + k * kMlpOut + o] : __float2bfloat16_rn(0.f);
  }
  if (t < kMlpHidden) {
    S.b1[t] = m.P[kOffB1 + t];
    S.b2[t] = m.P[kOffB2 + t];
  }
  if (t < kOutP) S.b3[t] = t < kMlpOut ? m.P[kOffB3 + t] : 0.f;

  // gradient accumulators (TRAIN)
  float g2[8][8], g1[3][8], g3[4];
  float gb = 0.f;  // b1 (t < 128)
  float gb2 = 0.f; // b2 (t < 128)
  float gb3 = 0.f; // b3 (t < 8)
  double loss = 0.0;
  if (TRAIN) {
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int c = 0; c < 8; ++c) g2[a][c] = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 8; ++c) g1[a][c] = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c) g3[c] = 0.f;
  }
  __syncthreads();

  const int64_t ntiles = (n + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t r0 = tile * kTile;
    // ---- input tile
    for (int e = t; e < kTile * kMlpIn; e += kThr) {
      const int i = e / kMlpIn, k = e % kMlpIn;
      const int64_t r = r0 + i;
      float v = 0.f;
      if (r < n) {
        const int64_t row = rows ? (int64_t)rows[r] : r;
        v = X[row * kMlpIn + k];
      }
      S.x[i * kLdX + k] = v;
    }
    __syncthreads();
    dense_silu<kMlpIn, kLdX>(S.x, S.W1, S.b1, S.z1, S.h1);
    __syncthreads();
    dense_silu<kMlpHidden, kLdH>(S.h1, S.W2, S.b2, S.z2, S.h2);
    __syncthreads();
    // ---- output layer: thread (row t / 8, output t % 8)
    {
      const int i = t >> 3, o = t & 7;
      float acc = S.b3[o];
#pragma unroll 8
      for (int k = 0; k < kMlpHidden; ++k) acc = fmaf(S.h2[i * kLdH + k], __bfloat162float(S.W3[k * kOutP + o]), acc);
      const int64_t r = r0 + i;
      if (!TRAIN) {
        if (r < n && o < kMlpOut) Y[r * kMlpOut + o] = acc;
      } else {
        float d = 0.f;
        if (r < n && o < kMlpOut) {
          const int64_t row = rows ? (int64_t)rows[r] : r;
          const float tv = T[row * kMlpOut + o];
          if (tv == tv) d = acc - tv;  // NaN target: row carries no sample
        }
        loss += (double)d * (double)d;
        S.dy[i * kOutP + o] = d * gscale;
      }
    }
    if (TRAIN) {
      __syncthreads();
      // ---- dW3, db3
      {
        const int k = t >> 1, o0 = (t & 1) * 4;
#pragma unroll 4
        for (int i = 0; i < kTile; ++i) {
          const float hv = S.h2[i * kLdH + k];
#pragma unroll
          for (int c = 0; c < 4; ++c) g3[c] = fmaf(hv, S.dy[i * kOutP + o0 + c], g3[c]);
        }
        if (t < kOutP)
          for (int i = 0; i < kTile; ++i) gb3 += S.dy[i * kOutP + t];
      }
      // ---- dz2 = (dy W3ᵀ) ⊙ silu'(z2), in place in z2
      {
        const int tm = t >> 5, tn = t & 31;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = 4 * tm + a, j = 4 * tn + c;
            float s = 0.f;
#pragma unroll
            for (int o = 0; o < kMlpOut; ++o) s = fmaf(S.dy[i * kOutP + o], __bfloat162float(S.W3[j * kOutP + o]), s);
            S.z2[i * kLdH + j] = s * dsilu(S.z2[i * kLdH + j]);
          }
      }
      __syncthreads();
      // ---- dW2, db2 (reads h1, dz2)
      {
        const int tk = t >> 4, tj = t & 15;
#pragma unroll 2
        for (int i = 0; i < kTile; ++i) {
          const float4 ha = *reinterpret_cast<const float4*>(S.h1 + i * kLdH + 8 * tk);
          const float4 hb = *reinterpret_cast<const float4*>(S.h1 + i * kLdH + 8 * tk + 4);
          const float4 da = *reinterpret_cast<const float4*>(S.z2 + i * kLdH + 8 * tj);
          const float4 db = *reinterpret_cast<const float4*>(S.z2 + i * kLdH + 8 * tj + 4);
          const float hv[8] = {ha.x, ha.y, ha.z, ha.w, hb.x, hb.y, hb.z, hb.w};
          const float dv[8] = {da.x, da.y, da.z, da.w, db.x, db.y, db.z, db.w};
#pragma unroll
          for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int c = 0; c < 8; ++c) g2[a][c] = fmaf(hv[a], dv[c], g2[a][c]);
        }
        if (t < kMlpHidden)
          for (int i = 0; i < kTile; ++i) gb2 += S.z2[i * kLdH + t];
      }
      // ---- dz1 = (dz2 W2ᵀ) ⊙ silu'(z1), in place in z1 (reads dz2, z1; no other reader of z1)
      {
        const int tm = t >> 5, tn = t & 31;
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[a][c] = 0.f;
#pragma unroll 4
        for (int j = 0; j < kMlpHidden; ++j) {
          const __nv_bfloat162* wp = reinterpret_cast<const __nv_bfloat162*>(S.W2T + j * kMlpHidden + 4 * tn);
          const float2 w01 = __bfloat1622float2(wp[0]);
          const float2 w23 = __bfloat1622float2(wp[1]);
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const float dv = S.z2[(4 * tm + a) * kLdH + j];
            acc[a][0] = fmaf(dv, w01.x, acc[a][0]);
            acc[a][1] = fmaf(dv, w01.y, acc[a][1]);
            acc[a][2] = fmaf(dv, w23.x, acc[a][2]);
            acc[a][3] = fmaf(dv, w23.y, acc[a][3]);
          }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            float* zp = S.z1 + (4 * tm + a) * kLdH + 4 * tn + c;
            *zp = acc[a][c] * dsilu(*zp);
          }
      }
      __syncthreads();
      // ---- dW1, db1 (reads x, dz1)
      {
        const int tk = t >> 4, tj = t & 15;
#pragma unroll 2
        for (int i = 0; i < kTile; ++i) {
          const float4 da = *reinterpret_cast<const float4*>(S.z1 + i * kLdH + 8 * tj);
          const float4 db = *reinterpret_cast<const float4*>(S.z1 + i * kLdH + 8 * tj + 4);
          const float dv[8] = {da.x, da.y, da.z, da.w, db.x, db.y, db.z, db.w};
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float xv = S.x[i * kLdX + 3 * tk + a];
#pragma unroll
            for (int c = 0; c < 8; ++c) g1[a][c] = fmaf(xv, dv[c], g1[a][c]);
          }
        }
        if (t < kMlpHidden)
          for (int i = 0; i < kTile; ++i) gb += S.z1[i * kLdH + t];
      }
    }
    __syncthreads();
  }

  if (TRAIN) {
    float* G = gpart + (int64_t)blockIdx.x * kMlpParams;
    {
      const int tk = t >> 4, tj = t & 15;
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int c = 0; c < 8; ++c) G[kOffW2 + (8 * tk + a) * kMlpHidden + 8 * tj + c] = g2[a][c];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 8; ++c) G[kOffW1 + (3 * tk + a) * kMlpHidden + 8 * tj + c] = g1[a][c];
    }
    {
      const int k = t >> 1, o0 = (t & 1) * 4;
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (o0 + c < kMlpOut) G[kOffW3 + k * kMlpOut + o0 + c] = g3[c];
    }
    if (t < kMlpHidden) {
      G[kOffB1 + t] = gb;
      G[kOffB2 + t] = gb2;
    }
    if (t < kMlpOut) G[kOffB3 + t] = gb3;
    // loss: fixed-order block reduction
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, off);
    if ((t & 31) == 0) S.red[t >> 5] = loss;
    __syncthreads();
    if (t == 0) {
      double sum = 0.0;
      for (int w = 0; w < kThr / 32; ++w) sum += S.red[w];
      lpart[blockIdx.x] = sum;
    }
  }
}

// g[p] = Σ_c gpart[c][p] in CTA order; loss = Σ_c lpart[c] · lscale.
__global__ void k_mlp_reduce(const float* __restrict__ gpart, int grid, float* __restrict__ g,
                             const double* __restrict__ lpart, double* __restrict__ loss, double lscale) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kMlpParams) {
    float s = 0.f;
    for (int c = 0; c < grid; ++c) s += gpart[(int64_t)c * kMlpParams + p];
    g[p] = s;
  }
  if (p == 0 && loss) {
    double s = 0.0;
    for (int c = 0; c < grid; ++c) s += lpart[c];
    *loss = s * lscale;
  }
}

__global__ void k_mlp_adam(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m1,
                           float* __restrict__ m2, __nv_bfloat16* __restrict__ W, float lr, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParams) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float gp = g[p];
  const float a = b1 * m1[p] + (1.f - b1) * gp;
  const float v = b2 * m2[p] + (1.f - b2) * gp * gp;
  m1[p] = a;
  m2[p] = v;
  const float w = P[p] - lr * (a * c1) / (sqrtf(v * c2) + eps);
  P[p] = w;
  W[p] = __float2bfloat16_rn(w);
}

__global__ void k_mlp_bf16(const float* __restrict__ P, __nv_bfloat16* __restrict__ W) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kMlpParams) W[p] = __float2bfloat16_rn(P[p]);
}

int grid_for(int64_t n) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tiles = (n + kTile - 1) / kTile;
  return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, sms));
}

template <bool TRAIN>
cudaError_t set_smem() {
  static bool done = false;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_mlp<TRAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem));
  if (e == cudaSuccess) done = true;
  return e;
}

}  // namespace

cudaError_t mlp_forward(const MlpDev& m, const float* X, int64_t n, float* Y, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = set_smem<false>();
  if (e != cudaSuccess) return e;
  k_mlp<false><<<grid_for(n), kThr, sizeof(Smem), s>>>(m, X, nullptr, n, nullptr, Y, nullptr, nullptr, 0.f);
  return cudaGetLastError();
}

cudaError_t mlp_to_bf16(const float* P, __nv_bfloat16* W, cudaStream_t s) {
  k_mlp_bf16<<<(kMlpParams + 255) / 256, 256, 0, s>>>(P, W);
  return cudaGetLastError();
}

cudaError_t mlp_trainer_init(MlpTrainer& t, const float* params_host, cudaStream_t s) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  t.grid = sms;
  const size_t pb = sizeof(float) * kMlpParams;
  cudaError_t e;
  if ((e = cudaMalloc(&t.P, pb)) || (e = cudaMalloc(&t.G, pb)) || (e = cudaMalloc(&t.M1, pb)) ||
      (e = cudaMalloc(&t.M2, pb)) || (e = cudaMalloc(&t.W, sizeof(__nv_bfloat16) * kMlpParams)) ||
      (e = cudaMalloc(&t.gpart, pb * (size_t)t.grid)) || (e = cudaMalloc(&t.loss, sizeof(double) * (t.grid + 1))))
    return e;
  if ((e = cudaMemcpyAsync(t.P, params_host, pb, cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemsetAsync(t.M1, 0, pb, s)) || (e = cudaMemsetAsync(t.M2, 0, pb, s)))
    return e;
  t.step = 0;
  return mlp_to_bf16(t.P, t.W, s);
}

void mlp_trainer_free(MlpTrainer& t) {
  cudaFree(t.P); cudaFree(t.G); cudaFree(t.M1); cudaFree(t.M2); cudaFree(t.W); cudaFree(t.gpart); cudaFree(t.loss);
  t = MlpTrainer{};
}

cudaError_t mlp_loss_grad(MlpTrainer& t, const float* X, const float* T, const int* rows, int64_t n, double* loss_dev,
                          cudaStream_t s) {
  cudaError_t e = set_smem<true>();
  if (e != cudaSuccess) return e;
  const int grid = std::min(t.grid, grid_for(n));
  const float gscale = 2.f / (float)((double)n * kMlpOut);
  MlpDev m{t.P, t.W};
  k_mlp<true><<<grid, kThr, sizeof(Smem), s>>>(m, X, rows, n, T, nullptr, t.gpart, t.loss, gscale);
  k_mlp_reduce<<<(kMlpParams + 255) / 256, 256, 0, s>>>(t.gpart, grid, t.G, t.loss, loss_dev,
                                                        1.0 / ((double)n * kMlpOut));
  return cudaGetLastError();
}

cudaError_t mlp_adam(MlpTrainer& t, float lr, cudaStream_t s) {
  t.step += 1;
  const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)t.step)));
  const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)t.step)));
  k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(t.P, t.G, t.M1, t.M2, t.W, lr, c1, c2);
  return cudaGetLastError();
}

}  // namespace eb

// ---------------------------------------------------------------- C ABI
using namespace eb;

namespace {
struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { cudaFree(p); }
  template <typename T>
  cudaError_t put(const T* h, size_t n) {
    cudaError_t e = cudaMalloc(&p, sizeof(T) * (n ? n : 1));
    if (e == cudaSuccess && n) e = cudaMemcpy(p, h, sizeof(T) * n, cudaMemcpyHostToDevice);
    return e;
  }
  cudaError_t make(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 1); }
  template <typename T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

int cuda_fail(cudaError_t e, const char* what) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return eb_internal_fail(EB_ERR_CUDA, buf);
}
#define MCK(x, what)                          \
  do {                                        \
    cudaError_t _e = (x);                     \
    if (_e != cudaSuccess) return cuda_fail(_e, what); \
  } while (0)
}  // namespace

extern "C" {

int eb_mlp_forward(const float* params, const float* X, int64_t n, float* Y) {
  if (!params || n < 0 || (n > 0 && (!X || !Y))) return eb_internal_fail(EB_ERR_ARG, "eb_mlp_forward: bad arguments");
  DevBuf P, W, Xd, Yd;
  MCK(P.put(params, kMlpParams), "eb_mlp_forward");
  MCK(W.make(sizeof(__nv_bfloat16) * kMlpParams), "eb_mlp_forward");
  MCK(Xd.put(X, (size_t)n * kMlpIn), "eb_mlp_forward");
  MCK(Yd.make(sizeof(float) * (size_t)n * kMlpOut), "eb_mlp_forward");
  MCK(mlp_to_bf16(P.as<float>(), W.as<__nv_bfloat16>(), 0), "eb_mlp_forward");
  MlpDev m{P.as<float>(), W.as<__nv_bfloat16>()};
  MCK(mlp_forward(m, Xd.as<float>(), n, Yd.as<float>(), 0), "eb_mlp_forward");
  MCK(cudaMemcpy(Y, Yd.p, sizeof(float) * (size_t)n * kMlpOut, cudaMemcpyDeviceToHost), "eb_mlp_forward");
  return EB_OK;
}

int eb_mlp_loss_grad(const float* params, const float* X, const float* T, int64_t n, double* loss, float* grad) {
  if (!params || !X || !T || n <= 0 || !loss || !grad)
    return eb_internal_fail(EB_ERR_ARG, "eb_mlp_loss_grad: bad arguments");
  MlpTrainer tr;
  struct Guard {
    MlpTrainer& t;
    ~Guard() { mlp_trainer_free(t); }
  } guard{tr};
  DevBuf Xd, Td;
  MCK(mlp_trainer_init(tr, params, 0), "eb_mlp_loss_grad");
  MCK(Xd.put(X, (size_t)n * kMlpIn), "eb_mlp_loss_grad");
  MCK(Td.put(T, (size_t)n * kMlpOut), "eb_mlp_loss_grad");
  MCK(mlp_loss_grad(tr, Xd.as<float>(), Td.as<float>(), nullptr, n, tr.loss + tr.grid, 0), "eb_mlp_loss_grad");
  MCK(cudaMemcpy(grad, tr.G, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost), "eb_mlp_loss_grad");
  MCK(cudaMemcpy(loss, tr.loss + tr.grid, sizeof(double), cudaMemcpyDeviceToHost), "eb_mlp_loss_grad");
  return EB_OK;
}

int eb_mlp_train(float* params, const float* X, const float* T, int64_t n, int32_t epochs, int32_t batch, float lr,
                 uint64_t seed, double* loss_per_epoch) {
  if (!params || !X || !T || n <= 0 || epochs < 0 || batch <= 0 || !(lr > 0))
    return eb_internal_fail(EB_ERR_ARG, "eb_mlp_train: bad arguments");
  if (n > INT32_MAX) return eb_internal_fail(EB_ERR_ARG, "eb_mlp_train: too many samples");
  MlpTrainer tr;
  struct Guard {
    MlpTrainer& t;
    ~Guard() { mlp_trainer_free(t); }
  } guard{tr};
  DevBuf Xd, Td, Rd, Ld;
  MCK(mlp_trainer_init(tr, params, 0), "eb_mlp_train");
  MCK(Xd.put(X, (size_t)n * kMlpIn), "eb_mlp_train");
  MCK(Td.put(T, (size_t)n * kMlpOut), "eb_mlp_train");
  MCK(Rd.make(sizeof(int) * (size_t)n), "eb_mlp_train");
  const int64_t nb = (n + batch - 1) / batch;
  MCK(Ld.make(sizeof(double) * (size_t)std::max<int64_t>(1, nb)), "eb_mlp_train");
  std::vector<int> perm((size_t)n);
  std::mt19937_64 rng(seed);
  std::vector<double> bl((size_t)nb);
  for (int ep = 0; ep < epochs; ++ep) {
    for (int64_t i = 0; i < n; ++i) perm[(size_t)i] = (int)i;
    for (int64_t i = n - 1; i > 0; --i) {  // Fisher-Yates with the seeded engine
      const int64_t j = (int64_t)(rng() % (uint64_t)(i + 1));
      std::swap(perm[(size_t)i], perm[(size_t)j]);
    }
    MCK(cudaMemcpy(Rd.p, perm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice), "eb_mlp_train");
    for (int64_t b = 0; b < nb; ++b) {
      const int64_t r0 = b * batch, m = std::min<int64_t>(batch, n - r0);
      MCK(mlp_loss_grad(tr, Xd.as<float>(), Td.as<float>(), Rd.as<int>() + r0, m, Ld.as<double>() + b, 0),
          "eb_mlp_train");
      MCK(mlp_adam(tr, lr, 0), "eb_mlp_train");
    }
    MCK(cudaMemcpy(bl.data(), Ld.p, sizeof(double) * (size_t)nb, cudaMemcpyDeviceToHost), "eb_mlp_train");
    if (loss_per_epoch) {
      double s = 0.0;
      for (int64_t b = 0; b < nb; ++b) s += bl[(size_t)b];
      loss_per_epoch[ep] = s / (double)nb;
    }
  }
  MCK(cudaMemcpy(params, tr.P, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost), "eb_mlp_train");
  return EB_OK;
}

}  // extern "C"
