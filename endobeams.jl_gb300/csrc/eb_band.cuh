// Banded LU preconditioner for the per-simulation GMRES.
//
// The reference factorises Ktan_free exactly with MKL PARDISO on every
// Newton iteration (src/linearsolvers.jl:15-23).  Here each simulation's
// tangent is permuted (reverse Cuthill-McKee on the node graph, 6 DOFs per
// node), copied into band storage in FP32 and factorised by one CTA
// (blocked right-looking LU, no pivoting: the dynamic tangent carries the
// positive mass term 1/(βΔt²)M on its diagonal).  The FP32 factors are the
// GMRES preconditioner; GMRES itself measures and drives the FP64 residual,
// so the factorisation's rounding only costs an iteration or two.
//
// Band storage of simulation s (N = 6 n_s DOFs, half bandwidth b), two
// column-major parts so that each triangular sweep streams one contiguous
// block of 32 columns:
//   U part (i <= j): U[(b + i - j) + (b + 1) j]      starts at off[s]
//   L part (i >  j): L[(i - j - 1) + b j]            starts at off[s] + ustride(N, b)
// Both parts are padded to multiples of 32 floats plus 32 spare floats, so
// 16-byte-rounded bulk copies of a trailing block stay inside the allocation.
#pragma once
#include "eb_internal.cuh"

namespace eb {

struct BandDev {
  float* A;                 // concatenated band storage
  const int64_t* off;       // per sim: offset of its U part in A (L part follows)
  const int* bw;            // per sim: half bandwidth b in DOFs (0: no band, block-Jacobi)
  const int* pos;           // per global node: position in its simulation's band order
  const int* node_at;       // per (node_off[s] + position): global node id
  float* work;              // per DOF scratch (permuted vector)
  float* Linv;              // per panel: inverse of the unit-lower diagonal block (column-major)
  float* Uinv;              // per panel: inverse of the upper diagonal block (column-major)
  const int* refactor;      // per sim: 1 = refill and refactorise before this solve
  const int* order;         // CTA b of the per-simulation kernels works on simulation order[b]
                            // (largest first, so the last wave holds the smallest simulations)
};

constexpr int kPanel = 32;  // panel width of the blocked factorisation and solves

__host__ __device__ __forceinline__ int64_t pad32(int64_t x) { return ((x + 31) / 32) * 32 + 32; }
__host__ __device__ __forceinline__ int64_t ustride(int64_t n, int b) { return pad32(n * (int64_t)(b + 1)); }
__host__ __device__ __forceinline__ int64_t band_floats(int64_t n, int b) {
  return ustride(n, b) + pad32(n * (int64_t)b);
}

// Offset of simulation s's diagonal-block inverses: one kPanel x kPanel
// block per panel, with kPanel spare rows per simulation for the last panel.
__host__ __device__ __forceinline__ int64_t inv_base(int64_t n0, int s) {
  return (6 * n0 + (int64_t)kPanel * s) * kPanel;
}

struct BandView {
  float* U;
  float* L;
  int b;
  __device__ __forceinline__ float& at(int i, int j) const {
    return i > j ? L[(int64_t)(i - j - 1) + (int64_t)b * j] : U[(int64_t)(b + i - j) + (int64_t)(b + 1) * j];
  }
};

__device__ __forceinline__ BandView band_view(const BandDev& B, int s, int n) {
  const int b = B.bw[s];
  float* U = B.A + B.off[s];
  return BandView{U, U + ustride(n, b), b};
}

// ---------------------------------------------------------------- bulk async copies (TMA engine)
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// global -> shared bulk copy completing on `bar`; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait for the phase `parity` of `bar` (each try waits up to ~10 µs);
// returns false after ~1.3 s without completion.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int it = 0; it < (1 << 17); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(10000u)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Shared-memory staging of a simulation's band blocks (double buffered).
struct Stage {
  float* buf[2];    // 32 columns of one band part: 32 (b_max + 1) floats each
  float* inv[2];    // the matching 32x32 diagonal-block inverse
  uint64_t* bar;    // two mbarriers
  int* fail;        // shared flag: a wait ran out (staging is then abandoned)
  int* pend;        // shared, thread 0 only: parity of the copy in flight per buffer, -1 none
  uint32_t extra;   // bytes expected beyond the copies on the first block (timeout-path test; normally 0)
};

// Thread 0, at kernel end after a failed wait: waits (bounded) for copies still in flight.
__device__ __forceinline__ void stage_drain(const Stage* st) {
  if (!st || threadIdx.x != 0) return;
  for (int sb = 0; sb < 2; ++sb)
    if (st->pend[sb] >= 0) mbar_wait(&st->bar[sb], (uint32_t)st->pend[sb]);
}

// z = M⁻¹ v on the CTA owning simulation s: gather into band order, forward
// substitution with unit L, backward substitution with U, scatter back.  The
// diagonal blocks are applied through their precomputed inverses (a 32x32
// product per block), the off-diagonal band by a row-parallel update.
// `xs` (may be null) is shared-memory room for the n permuted entries.
// With `st` non-null, each block's 32 band columns and its inverse are
// streamed into shared memory by bulk async copies one block ahead; `ph`
// holds the two barriers' next phase bits and is advanced here.
template <typename TV, typename TZ>
__device__ void band_solve(const BandDev& B, int s, int64_t n0, int n, const TV* __restrict__ v, TZ* __restrict__ z,
                           float* xs, const Stage* st, uint32_t* ph) {
  const BandView V = band_view(B, s, n);
  const int b = V.b;
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
  const int nblk = (n + kPanel - 1) / kPanel;
  // issue the bulk copies of block jb of the L (lower) or U part into buffer `sb`
  auto issue = [&](int jb, int sb, bool lower) {
    const int k0 = jb * kPanel;
    const int kb = min(kPanel, n - k0);
    const int64_t colw = lower ? b : b + 1;
    const float* src = lower ? V.L + (int64_t)b * k0 : V.U + (int64_t)(b + 1) * k0;
    const uint32_t bytes = (uint32_t)(((int64_t)kb * colw * 4 + 15) & ~(int64_t)15);
    const float* isrc = (lower ? Li : Ui) + (int64_t)k0 * kPanel;
    fence_async_smem();
    mbar_expect_tx(&st->bar[sb], bytes + 4096u + (jb == 0 && lower ? st->extra : 0u));
    bulk_g2s(st->buf[sb], src, bytes, &st->bar[sb]);
    bulk_g2s(st->inv[sb], isrc, 4096u, &st->bar[sb]);
    st->pend[sb] = (int)ph[sb];
  };
  // all threads wait for buffer sb; thread 0 clears its pending mark
  auto await = [&](int sb) {
    if (!*st->fail) {
      if (!mbar_wait(&st->bar[sb], ph[sb]) && !mbar_wait(&st->bar[sb], ph[sb])) *st->fail = 1;
      else if (threadIdx.x == 0) st->pend[sb] = -1;
    }
    ph[sb] ^= 1u;
  };
  const bool staged = st && !*st->fail;  // uniform: read after the barrier above
  // ---- forward: L y = x (unit diagonal)
  if (staged && threadIdx.x == 0) {
    issue(0, 0, true);
    if (nblk > 1) issue(1, 1, true);
  }
  for (int jb = 0; jb < nblk; ++jb) {
    const int k0 = jb * kPanel;
    const int kb = min(kPanel, n - k0);
    const int sb = jb & 1;
    const float* Lc = nullptr;
    const float* Lin = Li + (int64_t)k0 * kPanel;
    if (staged) {
      await(sb);
      Lc = st->buf[sb];
      Lin = st->inv[sb];
    }
    if (warp == 0) {
      float acc = 0.f;
      for (int t = 0; t < kb; ++t) acc += Lin[t * kPanel + lane] * x[k0 + t];
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
      if (Lc)
        for (int t = t0; t < k0 + kb; ++t) acc += Lc[(int64_t)(t - k0) * b + (i - t - 1)] * yb[t - k0];
      else
        for (int t = t0; t < k0 + kb; ++t) acc += V.at(i, t) * yb[t - k0];
      x[i] -= acc;
    }
    __syncthreads();
    if (staged && threadIdx.x == 0 && jb + 2 < nblk && !*st->fail) issue(jb + 2, sb, true);
  }
  // ---- backward: U x = y
  if (staged && threadIdx.x == 0 && !*st->fail) {
    issue(nblk - 1, 0, false);
    if (nblk > 1) issue(nblk - 2, 1, false);
  }
  for (int q = 0; q < nblk; ++q) {
    const int jb = nblk - 1 - q;
    const int k0 = jb * kPanel;
    const int kb = min(kPanel, n - k0);
    const int sb = q & 1;
    const float* Uc = nullptr;
    const float* Uin = Ui + (int64_t)k0 * kPanel;
    if (staged) {
      await(sb);
      Uc = st->buf[sb];
      Uin = st->inv[sb];
    }
    if (warp == 0) {
      float acc = 0.f;
      for (int t = 0; t < kb; ++t) acc += Uin[t * kPanel + lane] * x[k0 + t];
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
      if (Uc)
        for (int t = k0; t < t1; ++t) acc += Uc[(int64_t)(t - k0) * (b + 1) + (b + i - t)] * yb[t - k0];
      else
        for (int t = k0; t < t1; ++t) acc += V.at(i, t) * yb[t - k0];
      x[i] -= acc;
    }
    __syncthreads();
    if (staged && threadIdx.x == 0 && q + 2 < nblk && !*st->fail) issue(nblk - 1 - (q + 2), sb, false);
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
