// Band assembly and blocked band LU (see eb_band.cuh).
#include <map>
#include <mutex>
#include <utility>

#include "eb_band.cuh"

namespace eb {

// Thread per (block, entry): copies Ktan into the permuted FP32 band; fixed
// DOFs become identity rows/columns (the free-DOF system of
// extract_free_dofs!, src/utils_solver.jl:94-102, embedded in the full size).
__global__ void k_band_fill(Dev d, BandDev B, const int* __restrict__ blk_row) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nnzb * 36) return;
  const int blk = (int)(t / 36), k = (int)(t % 36);
  const int s = d.blk_sim[blk];
  if (!d.active[s] || !B.refactor[s]) return;
  const int b = B.bw[s];
  if (b == 0) return;
  const int row = blk_row[blk], colnode = d.col[blk];
  const int r = k % 6, c = k / 6;
  const int i = 6 * B.pos[row] + r, j = 6 * B.pos[colnode] + c;
  const int64_t gr = 6 * (int64_t)row + r, gc = 6 * (int64_t)colnode + c;
  double v = d.Kt[t];
  if (d.fixed[gr] || d.fixed[gc]) v = (gr == gc) ? 1.0 : 0.0;
  const int n = (int)(6 * (d.sim_node_off[s + 1] - d.sim_node_off[s]));
  band_view(B, s, n).at(i, j) = (float)v;
}

// Zeroes the bands of the simulations about to be refactorised (one CTA per simulation).
__global__ void k_band_zero(Dev d, BandDev B) {
  const int s = blockIdx.x;
  if (!d.active[s] || !B.refactor[s] || B.bw[s] == 0) return;
  if (threadIdx.x == 0 && B.lu_fail) B.lu_fail[s] = 0;
  float* A = B.A + B.off[s];
  const int64_t len = band_floats(6 * (d.sim_node_off[s + 1] - d.sim_node_off[s]), B.bw[s]);
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) A[i] = 0.f;
}

void launch_band_fill(const Dev& d, const BandDev& B, const int* blk_row, cudaStream_t s) {
  k_band_zero<<<d.n_sims, 512, 0, s>>>(d, B);
  if (d.nnzb) k_band_fill<<<nblocks(d.nnzb * 36, 256), 256, 0, s>>>(d, B, blk_row);
}

// Blocked right-looking LU without pivoting of one simulation's band (one CTA
// of kLuThreads threads).  Per panel of kPanel columns:
//   1. panel (rows k0 .. k0+kb+b) factorised in shared memory, column = lane;
//   2. U12 = L11⁻¹ A12, one thread per column of U12 (independent columns);
//   3. A22 -= L21 U12 on 8x8 register tiles, A22 read and written in place;
//   4. inverses of the unit-lower L11 and upper U11 stored for the solves.
constexpr int kLuThreads = 256;

__global__ void __launch_bounds__(kLuThreads) k_band_lu(Dev d, BandDev B) {
  const int s = B.order[blockIdx.x];
  if (!d.active[s] || !B.refactor[s]) return;
  const int b = B.bw[s];
  if (b == 0) return;
  const int64_t n0 = d.sim_node_off[s];
  const int n = (int)(6 * (d.sim_node_off[s + 1] - n0));
  const BandView V = band_view(B, s, n);
  float* Li = B.Linv + inv_base(n0, s);  // per panel: kPanel x kPanel, column-major
  float* Ui = B.Uinv + inv_base(n0, s);
  extern __shared__ float smf[];
  const int ldp = kPanel + b;             // odd: column stride avoids bank conflicts
  float* P = smf;                         // panel, ldp x kPanel column-major
  float* U = P + ldp * kPanel;            // U12, kPanel x b row-major
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nw = kLuThreads / 32;
  for (int k0 = 0; k0 < n; k0 += kPanel) {
    const int kb = min(kPanel, n - k0);
    const int hp = min(n - k0, kb + b);
    const int q = min(n - k0 - kb, b);
    // ---- load the panel and U12: warp per column, lanes along the rows (a band column is
    // contiguous in rows, so each warp access is one 128-byte line; q > 0 implies kb = 32)
    for (int c = warp; c < kb; c += nw)
      for (int r = lane; r < hp; r += 32) {
        const int i = k0 + r, j = k0 + c;
        P[r + ldp * c] = (i - j <= b && j - i <= b) ? V.at(i, j) : 0.f;
      }
    for (int c = warp; c < q; c += nw) {
      const int i = k0 + lane, j = k0 + kb + c;
      U[lane * b + c] = (j - i <= b) ? V.at(i, j) : 0.f;
    }
    __syncthreads();
    // ---- 1. panel LU (column c = lane)
    for (int t = 0; t < kb; ++t) {
      const float ip = 1.f / P[t + ldp * t];
      for (int r = t + 1 + threadIdx.x; r < hp; r += kLuThreads) P[r + ldp * t] *= ip;
      __syncthreads();
      if (lane > t && lane < kb) {
        const float ut = P[t + ldp * lane];
        for (int r = t + 1 + warp; r < hp; r += nw) P[r + ldp * lane] -= P[r + ldp * t] * ut;
      }
      __syncthreads();
    }
    // ---- 2. U12 = L11⁻¹ A12 (thread per column)
    for (int c = threadIdx.x; c < q; c += kLuThreads) {
      float col[kPanel];
#pragma unroll
      for (int r = 0; r < kPanel; ++r) col[r] = r < kb ? U[r * b + c] : 0.f;
#pragma unroll
      for (int r = 1; r < kPanel; ++r) {
        float acc = col[r];
#pragma unroll
        for (int t = 0; t < r; ++t) acc -= P[r + ldp * t] * col[t];
        col[r] = acc;
      }
#pragma unroll
      for (int r = 0; r < kPanel; ++r)
        if (r < kb) U[r * b + c] = col[r];
    }
    // ---- 4. inverses of L11 (unit lower) and U11 (upper), row-major kPanel x kPanel
    if (warp == 0) {
      // column `lane` of L11⁻¹: solve L z = e_lane
      float z[kPanel];
#pragma unroll
      for (int r = 0; r < kPanel; ++r) {
        float acc = (r == lane) ? 1.f : 0.f;
#pragma unroll
        for (int t = 0; t < r; ++t) acc -= (r < kb && t < kb ? P[r + ldp * t] : 0.f) * z[t];
        z[r] = acc;
      }
      float* L = Li + (int64_t)k0 * kPanel;
#pragma unroll
      for (int r = 0; r < kPanel; ++r) L[lane * kPanel + r] = z[r];
    } else if (warp == 1) {
      // column `lane` of U11⁻¹: solve U z = e_lane (identity beyond kb)
      float z[kPanel];
#pragma unroll
      for (int r = kPanel - 1; r >= 0; --r) {
        float acc = (r == lane) ? 1.f : 0.f;
#pragma unroll
        for (int t = r + 1; t < kPanel; ++t) acc -= (r < kb && t < kb ? P[r + ldp * t] : 0.f) * z[t];
        z[r] = r < kb ? acc / P[r + ldp * r] : acc;
      }
      float* Uv = Ui + (int64_t)k0 * kPanel;
#pragma unroll
      for (int r = 0; r < kPanel; ++r) Uv[lane * kPanel + r] = z[r];
    }
    __syncthreads();
    // ---- 3. trailing update A22 -= L21 U12 on 8x8 register tiles with strided rows and
    // columns (thread (ti, tj) owns rows ti + a R and columns tj + c R, R = ceil(q / 8)):
    // consecutive lanes read consecutive panel rows (no bank conflicts), share the U12
    // row (broadcast) and update consecutive band entries (coalesced).
    // The tile's band entries are loaded before the product loop so their global-memory
    // latency overlaps the FMAs.
    // Rows and columns past q are read from shared memory without guards (the
    // allocation is padded) and their products discarded.
    const int R = (q + 7) >> 3;
    for (int tile = threadIdx.x; tile < R * R; tile += kLuThreads) {
      const int ti = tile % R, tj = tile / R;
      unsigned rv = 0u, cv = 0u;  // valid rows / columns of the tile
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        rv |= (ti + a * R < q ? 1u : 0u) << a;
        cv |= (tj + a * R < q ? 1u : 0u) << a;
      }
      float acc[8][8], old[8][8];
#pragma unroll
      for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int a = 0; a < 8; ++a)
          old[a][c] = ((rv >> a) & (cv >> c) & 1u) ? V.at(k0 + kb + ti + a * R, k0 + kb + tj + c * R) : 0.f;
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[a][c] = 0.f;
      const float* pp = P + kb + ti;  // row ti + a R of column t at pp[a R + ldp t]
      const float* up = U + tj;       // column tj + c R of row t at up[c R + b t]
#pragma unroll 2
      for (int t = 0; t < kb; ++t) {
        float l[8], u[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) l[a] = pp[a * R];
#pragma unroll
        for (int c = 0; c < 8; ++c) u[c] = up[c * R];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int c = 0; c < 8; ++c) acc[a][c] = fmaf(l[a], u[c], acc[a][c]);
        pp += ldp;
        up += b;
      }
#pragma unroll
      for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int a = 0; a < 8; ++a)
          if ((rv >> a) & (cv >> c) & 1u) V.at(k0 + kb + ti + a * R, k0 + kb + tj + c * R) = old[a][c] - acc[a][c];
    }
    // ---- write back the panel and U12, warp per column as they were loaded
    for (int c = warp; c < kb; c += nw)
      for (int r = lane; r < hp; r += 32) {
        const int i = k0 + r, j = k0 + c;
        if (i - j <= b && j - i <= b) V.at(i, j) = P[r + ldp * c];
      }
    for (int c = warp; c < q; c += nw) {
      const int i = k0 + lane, j = k0 + kb + c;
      if (j - i <= b) V.at(i, j) = U[lane * b + c];
    }
    __syncthreads();
  }
}

cudaError_t raise_smem_limit(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> limit;  // (kernel, device) -> bytes set
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = limit[{func, dev}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

cudaError_t launch_band_lu(const Dev& d, const BandDev& B, int max_b, cudaStream_t s) {
  if (max_b <= 0) return cudaSuccess;
  // panel, U12 and 8 floats of padding for the unguarded reads past q
  const size_t smem = sizeof(float) * ((size_t)kPanel * (kPanel + 2 * (size_t)max_b) + 8);
  cudaError_t e = raise_smem_limit((const void*)k_band_lu, smem);
  if (e != cudaSuccess) return e;
  k_band_lu<<<d.n_sims, kLuThreads, smem, s>>>(d, B);
  return cudaGetLastError();
}

}  // namespace eb
