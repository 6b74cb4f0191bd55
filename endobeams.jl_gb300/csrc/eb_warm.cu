// Learned Newton warm start kernels (see eb_warm.cuh).
#include "eb_warm.cuh"

namespace eb {
namespace {

using ebd::V3;
using ebd::M3;

__device__ __forceinline__ V3 ld3(const double* a, int64_t n, int64_t i) {
  return ebd::v3(a[i], a[n + i], a[2 * n + i]);
}

// Signed distance and its gradient at x for simulation surface S (0 without a surface).
// Grid points outside the SDF's box are clamped onto it.
__device__ __forceinline__ double surface_phi(const SurfaceDev& S, int on, V3 x, V3* g) {
  if (!on) {
    *g = ebd::v3(0, 0, 0);
    return 0.0;
  }
  if (S.kind == 0) {
    V3 a = x - ebd::v3(S.cx, S.cy, S.cz);
    const double na = ebd::norm(a);
    *g = na > 0 ? (1 / na) * a : ebd::v3(0, 0, 0);
    return na - S.R;
  }
  V3 c = ebd::v3(fmin(fmax(x.x, S.x0), S.x0 + S.xl), fmin(fmax(x.y, S.y0), S.y0 + S.yl),
                 fmin(fmax(x.z, S.z0), S.z0 + S.zl));
  M3 h;
  return ebd::sdf_eval(S, c, g, &h);
}

__global__ void k_ws_features(Dev d, WsDev w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  const int s = d.node_sim[i];
  if (!d.active[s]) return;
  const int64_t n = d.n_nodes;
  const SurfaceDev& S = d.surf[s];
  const int on = w.surf_on[s];
  float f[kWsRaw];
  const V3 ui = ld3(d.u, n, i), vi = ld3(d.ud, n, i), ai = ld3(d.udd, n, i);
  const V3 wdi = ld3(d.wd, n, i), wddi = ld3(d.wdd, n, i);
  V3 gi;
  const double phii = surface_phi(S, on, ld3(d.X0, n, i) + ui, &gi);
  const V3 blk[5] = {ui, vi, ai, wdi, wddi};
  int k = 0;
#pragma unroll
  for (int b = 0; b < 5; ++b) {
    f[k++] = (float)blk[b].x;
    f[k++] = (float)blk[b].y;
    f[k++] = (float)blk[b].z;
  }
  f[k++] = (float)phii;
  f[k++] = (float)gi.x;
  f[k++] = (float)gi.y;
  f[k++] = (float)gi.z;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int64_t j = w.nb[2 * i + q];
    const V3 uj = ld3(d.u, n, j), vj = ld3(d.ud, n, j);
    V3 gj;
    const double phij = surface_phi(S, on, ld3(d.X0, n, j) + uj, &gj);
    const V3 du = uj - ui, dv = vj - vi;
    f[k++] = (float)du.x; f[k++] = (float)du.y; f[k++] = (float)du.z;
    f[k++] = (float)dv.x; f[k++] = (float)dv.y; f[k++] = (float)dv.z;
    f[k++] = (float)phij;
    f[k++] = (float)gj.x; f[k++] = (float)gj.y; f[k++] = (float)gj.z;
  }
  float* F = w.F + i * kWsRaw;
  float* X = w.X + i * kMlpIn;
#pragma unroll
  for (int c = 0; c < kWsRaw; ++c) {
    F[c] = f[c];
    X[c] = (f[c] - w.in_shift[c]) / w.in_scale[c];
  }
#pragma unroll
  for (int c = kWsRaw; c < kMlpIn; ++c) X[c] = 0.f;
}

__global__ void k_ws_apply(Dev d, WsDev w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  const int s = d.node_sim[i];
  if (!d.active[s]) return;
  const int64_t n = d.n_nodes;
  const double dt = d.dt[s], h2 = dt * dt;
  const V3 v[2] = {ld3(d.ud, n, i), ld3(d.wd, n, i)};
  const V3 a[2] = {ld3(d.udd, n, i), ld3(d.wdd, n, i)};
  const float* y = w.Y + i * kMlpOut;
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const double vv[3] = {v[b].x, v[b].y, v[b].z}, aa[3] = {a[b].x, a[b].y, a[b].z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int k = 3 * b + c;
      const int64_t dof = 6 * i + k;
      if (d.fixed[dof]) continue;
      d.dD[dof] = dt * vv[c] + 0.5 * h2 * aa[c] + h2 * (double)w.out_scale[k] * (double)y[k];
    }
  }
}

__global__ void k_ws_capture(Dev d, WsDev w, const int* mask, int64_t phase, int stride, int64_t cursor, int64_t cap,
                             float* sF, float* sT) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  if ((i + phase) % stride != 0) return;
  const int64_t slot = (cursor + i / stride) % cap;
  const int s = d.node_sim[i];
  float* T = sT + slot * kMlpOut;
  float* F = sF + slot * kWsRaw;
  for (int c = 0; c < kWsRaw; ++c) F[c] = w.F[i * kWsRaw + c];
  if (!mask[s]) {
    for (int c = 0; c < kMlpOut; ++c) T[c] = __int_as_float(0x7fc00000);  // NaN: no sample
    return;
  }
  const int64_t n = d.n_nodes;
  const double dt = d.dt[s], h2 = dt * dt;
  M3 dR;
#pragma unroll
  for (int k = 0; k < 9; ++k) dR.a[k] = d.dR[k * n + i];
  const V3 th = ebd::toangle(dR);
  const V3 du = ld3(d.u, n, i) - ld3(d.un, n, i);
  const V3 kin_u = dt * ld3(d.udn, n, i) + (0.5 * h2) * ld3(d.uddn, n, i);
  const V3 kin_w = dt * ld3(d.wdn, n, i) + (0.5 * h2) * ld3(d.wddn, n, i);
  const V3 ru = (1 / h2) * (du - kin_u), rw = (1 / h2) * (th - kin_w);
  T[0] = (float)ru.x; T[1] = (float)ru.y; T[2] = (float)ru.z;
  T[3] = (float)rw.x; T[4] = (float)rw.y; T[5] = (float)rw.z;
}

__global__ void k_ws_rnorm(Dev d, double* out) {
  const int s = blockIdx.x;
  if (!d.active[s]) return;
  const int64_t o = 6 * d.sim_node_off[s], e = 6 * d.sim_node_off[s + 1];
  double acc = 0.0;
  for (int64_t k = o + threadIdx.x; k < e; k += blockDim.x)
    if (!d.fixed[k]) acc += d.r[k] * d.r[k];
  __shared__ double red[32];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) sum += red[q];
    out[s] = sum;
  }
}

}  // namespace

void launch_ws_features(const Dev& d, const WsDev& w, cudaStream_t s) {
  if (d.n_nodes) k_ws_features<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, w);
}
void launch_ws_apply(const Dev& d, const WsDev& w, cudaStream_t s) {
  if (d.n_nodes) k_ws_apply<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, w);
}
void launch_ws_capture(const Dev& d, const WsDev& w, const int* mask, int64_t phase, int stride, int64_t cursor,
                       int64_t cap, float* sF, float* sT, cudaStream_t s) {
  if (d.n_nodes) k_ws_capture<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, w, mask, phase, stride, cursor, cap, sF, sT);
}
void launch_ws_rnorm(const Dev& d, double* out, cudaStream_t s) {
  if (d.n_sims) k_ws_rnorm<<<d.n_sims, 256, 0, s>>>(d, out);
}

}  // namespace eb
