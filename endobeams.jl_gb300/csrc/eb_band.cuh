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

constexpr int kPanel = 32;     // panel width of the blocked factorisation and solves
constexpr int kWindow = 1024;  // shared ring of solve-vector rows (covers half bandwidths up to 960)

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

// One warp: xb[0..kb) <- Binv xb (Binv a 32x32 column-major diagonal-block
// inverse), also copied to yb.  Fully unrolled so the loads run ahead of the
// FMA chain.
__device__ __forceinline__ void diag_block(const float* Binv, float* xb, int kb, int lane, float* yb) {
  float acc = 0.f;
#pragma unroll
  for (int t = 0; t < kPanel; ++t)
    if (t < kb) acc = fmaf(Binv[t * kPanel + lane], xb[t], acc);
  __syncwarp();
  if (lane < kb) {
    xb[lane] = acc;
    yb[lane] = acc;
  }
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
  // Without `xs`, the sweeps keep the rows they touch in a shared ring of W >= b + 64
  // entries (row i in slot i mod W) and exchange 32 rows with global memory per block,
  // so the sequential chain reads and writes only shared memory.
  __shared__ float xw[kWindow];
  int W = kPanel * 2;
  while (W < b + 2 * kPanel) W <<= 1;
  const bool win = !xs && W <= kWindow;
  const int wm = W - 1;
  auto X = [&](int i) -> float& { return win ? xw[i & wm] : x[i]; };
  if (win) {
    for (int r = threadIdx.x; r < min(n, W); r += blockDim.x) xw[r & wm] = x[r];
    __syncthreads();
  }
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
      if (!*st->fail) {  // after a wait ran out, the rest of the sweep reads global memory
        Lc = st->buf[sb];
        Lin = st->inv[sb];
      }
    }
    if (warp == 0) diag_block(Lin, &X(k0), kb, lane, yb);
    __syncthreads();
    // rows below the block, up to 4 per thread with independent accumulators; each row
    // sums its in-band terms in increasing t (the same order staged or not)
    const int r1 = min(n, k0 + kb + b);
    for (int i0 = k0 + kb + (int)threadIdx.x; i0 < r1; i0 += 4 * (int)blockDim.x) {
      int ii[4];
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int q = 0; q < 4; ++q) ii[q] = i0 + q * (int)blockDim.x;
#pragma unroll 8
      for (int t = 0; t < kPanel; ++t) {
        if (t >= kb) break;
        const float y = yb[t];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int d = ii[q] - (k0 + t);  // >= 1: the row is below the column
          if (ii[q] < r1 && d <= b) {
            const float lv = Lc ? Lc[(int64_t)t * b + (d - 1)] : V.at(ii[q], k0 + t);
            acc[q] = fmaf(lv, y, acc[q]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (ii[q] < r1) X(ii[q]) -= acc[q];
    }
    if (win && (int)threadIdx.x < kb) {  // rows k0.. leave the ring, rows k0 + W.. enter
      const int t = threadIdx.x;
      x[k0 + t] = xw[(k0 + t) & wm];
      if (k0 + W + t < n) xw[(k0 + t) & wm] = x[k0 + W + t];
    }
    __syncthreads();
    if (staged && threadIdx.x == 0 && jb + 2 < nblk && !*st->fail) issue(jb + 2, sb, true);
  }
  // ---- backward: U x = y
  if (win) {
    for (int r = max(0, n - W) + threadIdx.x; r < n; r += blockDim.x) xw[r & wm] = x[r];
    __syncthreads();
  }
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
      if (!*st->fail) {
        Uc = st->buf[sb];
        Uin = st->inv[sb];
      }
    }
    if (warp == 0) diag_block(Uin, &X(k0), kb, lane, yb);
    __syncthreads();
    // rows above the block (same scheme as the forward sweep)
    const int r0 = max(0, k0 - b);
    for (int i0 = r0 + (int)threadIdx.x; i0 < k0; i0 += 4 * (int)blockDim.x) {
      int ii[4];
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int q = 0; q < 4; ++q) ii[q] = i0 + q * (int)blockDim.x;
#pragma unroll 8
      for (int t = 0; t < kPanel; ++t) {
        if (t >= kb) break;
        const float y = yb[t];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int d = (k0 + t) - ii[q];  // >= 1: the row is above the column
          if (ii[q] < k0 && d <= b) {
            const float uv = Uc ? Uc[(int64_t)t * (b + 1) + (b - d)] : V.at(ii[q], k0 + t);
            acc[q] = fmaf(uv, y, acc[q]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (ii[q] < k0) X(ii[q]) -= acc[q];
    }
    if (win && (int)threadIdx.x < kb) {  // rows k0.. leave the ring, rows k0 - W.. enter
      const int t = threadIdx.x;
      x[k0 + t] = xw[(k0 + t) & wm];
      if (k0 - W + t >= 0) xw[(k0 + t) & wm] = x[k0 - W + t];
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
