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
  float* A;                 // concatenated band storage (FP32: filled and factorised in place)
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
  int* lu_fail;             // per sim: 1 = the tensor-core factorisation stopped (a bounded wait ran out)
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

// Shared-memory staging of a simulation's band blocks: two buffers of band
// columns (32 columns of one band part) and two of 32x32 diagonal-block
// inverses, each pair on its own two mbarriers.
struct Stage {
  float* buf[2];    // 32 columns of one band part: 32 (b_max + 1) floats each
  float* inv[2];    // 32x32 diagonal-block inverses
  uint64_t* bar;    // four mbarriers: bar[0..1] band buffers, bar[2..3] inverse buffers
  int* fail;        // shared flag: a wait ran out (staging is then abandoned)
  int* pend;        // shared, thread 0 only: parity of the copy in flight per barrier, -1 none
  uint32_t extra;   // bytes expected beyond the copy of the first inverse (timeout-path test; normally 0)
};

// Thread 0, at kernel end after a failed wait: waits (bounded) for copies still in flight.
__device__ __forceinline__ void stage_drain(const Stage* st) {
  if (!st || threadIdx.x != 0) return;
  for (int k = 0; k < 4; ++k)
    if (st->pend[k] >= 0) mbar_wait(&st->bar[k], (uint32_t)st->pend[k]);
}

// Explicit shared-memory loads.  The staging buffers are reached through generic pointers,
// and a generic load that lands in shared memory is scoreboarded like a global one.
__device__ __forceinline__ float lds_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ float4 lds_f32x4(uint32_t a) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a)
               : "memory");
  return v;
}

// Σ_t col[t stride] y[t] over a full block (32 columns, none clipped by the band edge) as
// a0 + a1, a0 over even t and a1 over odd t in increasing t: the operations of the general
// loop below, unrolled so that the 32 shared loads of a row are in flight together.  `col`
// and `y` (16-byte aligned) are in shared memory.
__device__ __forceinline__ float row_dot32(const float* col, int stride, const float* y) {
  const uint32_t c = smem_u32(col), ya = smem_u32(y), sb = 4u * (uint32_t)stride;
  float a0 = 0.f, a1 = 0.f;
#pragma unroll
  for (int t4 = 0; t4 < kPanel / 4; ++t4) {
    const float4 w = lds_f32x4(ya + 16u * t4);
    a0 = fmaf(lds_f32(c + (4 * t4) * sb), w.x, a0);
    a1 = fmaf(lds_f32(c + (4 * t4 + 1) * sb), w.y, a1);
    a0 = fmaf(lds_f32(c + (4 * t4 + 2) * sb), w.z, a0);
    a1 = fmaf(lds_f32(c + (4 * t4 + 3) * sb), w.w, a1);
  }
  return a0 + a1;
}

// z = M⁻¹ v on the CTA owning simulation s: gather into band order, forward
// substitution with unit L, backward substitution with U, scatter back.
//
// Each sweep is a look-ahead pipeline over 32-row blocks with one CTA barrier
// per block.  At step s of the forward sweep warp 0 applies block s-1 to the
// rows of block s ("near" rows) and solves block s with its precomputed
// diagonal inverse, while the other warps apply block s-1 to the rows below
// block s ("far" rows); every row receives its block contributions in
// increasing block order, so the result does not depend on timing.  The
// backward sweep is the mirror image.  `xs` (may be null) is shared-memory
// room for the n permuted entries; without it the rows the sweeps touch live
// in a shared ring.  With `st` non-null, band columns and inverses are
// streamed into shared memory by bulk async copies one step ahead; bit k of
// `ph` is barrier k's next phase and is advanced here.  Everything the sweeps
// keep per thread (stage pointers, phase bits) is selected without indexing,
// so it stays in registers: no local-memory load sits on the block chain.
template <typename TV, typename TZ>
__device__ __forceinline__ void band_solve(const BandDev& B, int s, int64_t n0, int n, const TV* __restrict__ v,
                                           TZ* __restrict__ z, float* xs, const Stage* st, uint32_t& ph) {
  const BandView V = band_view(B, s, n);
  const int b = V.b;
  float* x = xs ? xs : B.work + 6 * n0;
  const float* Li = B.Linv + inv_base(n0, s);
  const float* Ui = B.Uinv + inv_base(n0, s);
  __shared__ __align__(16) float yb[2][kPanel];  // y of the last two blocks
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int node = B.node_at[n0 + r / 6];           // global id of the node at position r/6
    x[r] = (float)v[6 * (node - n0) + r % 6];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (n + kPanel - 1) / kPanel;
  // Without `xs`, the rows the sweeps touch live in a shared ring of W >= b + 64
  // entries (row i in slot i mod W); warp 0 exchanges each finished block with
  // global memory (the refill value is stored into the ring one step later).
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
  const Stage S = st ? *st : Stage{};
  auto sbuf = [&](int k) { return (k & 1) ? S.buf[1] : S.buf[0]; };
  auto sinv = [&](int k) { return (k & 1) ? S.inv[1] : S.inv[0]; };
  auto phb = [&](int k) { return (ph >> k) & 1u; };
  // bulk copies: band columns of block jb (L or U part) into buffer sb, or its inverse into buffer sb
  auto issue_cols = [&](int jb, int sb, bool lower) {
    const int k0 = jb * kPanel;
    const int kb = min(kPanel, n - k0);
    const int64_t colw = lower ? b : b + 1;
    const float* src = lower ? V.L + (int64_t)b * k0 : V.U + (int64_t)(b + 1) * k0;
    const uint32_t bytes = (uint32_t)(((int64_t)kb * colw * 4 + 15) & ~(int64_t)15);
    fence_async_smem();
    mbar_expect_tx(S.bar + sb, bytes);
    bulk_g2s(sbuf(sb), src, bytes, S.bar + sb);
    S.pend[sb] = (int)phb(sb);
  };
  auto issue_inv = [&](int jb, int sb, bool lower, uint32_t extra) {
    const float* isrc = (lower ? Li : Ui) + (int64_t)jb * kPanel * kPanel;
    fence_async_smem();
    mbar_expect_tx(S.bar + 2 + sb, 4096u + extra);
    bulk_g2s(sinv(sb), isrc, 4096u, S.bar + 2 + sb);
    S.pend[2 + sb] = (int)phb(2 + sb);
  };
  auto await = [&](int k) {  // k: barrier index 0..3
    if (!*S.fail) {
      if (!mbar_wait(S.bar + k, phb(k)) && !mbar_wait(S.bar + k, phb(k))) *S.fail = 1;
      else if (threadIdx.x == 0) S.pend[k] = -1;
    }
    ph ^= 1u << k;
  };
  const bool staged = st && !*S.fail;  // uniform: read after the barrier above
  // the copies are issued by the CTA's last thread, off warp 0's chain
  const bool issuer = threadIdx.x == blockDim.x - 1;

  for (int sweep = 0; sweep < 2; ++sweep) {
    const bool fwd = sweep == 0;
    const float* Ig = fwd ? Li : Ui;
    if (!fwd && win) {
      for (int r = max(0, n - W) + threadIdx.x; r < n; r += blockDim.x) xw[r & wm] = x[r];
      __syncthreads();
    }
    // block visited at step q (forward: q, backward: nblk - 1 - q)
    auto blk = [&](int q) { return fwd ? q : nblk - 1 - q; };
    if (staged && issuer && !*S.fail) {
      issue_inv(blk(0), 0, fwd, fwd ? S.extra : 0u);
      if (nblk > 1) {
        issue_inv(blk(1), 1, fwd, 0u);
        issue_cols(blk(0), 0, fwd);
      }
    }
    float pv = 0.f;       // warp 0: ring refill value loaded at the previous step
    int pslot = -1;
    for (int q = 0; q < nblk; ++q) {
      const int jb = blk(q);
      const int k0 = jb * kPanel;
      const int kb = min(kPanel, n - k0);
      // the block applied at this step (previous in sweep order) and its columns
      const int pj = q > 0 ? blk(q - 1) : -1;
      const int pk0 = pj * kPanel;
      const int pkb = q > 0 ? min(kPanel, n - pk0) : 0;
      const float* Pc = nullptr;                                  // staged columns of block pj
      const float* Inv = Ig + (int64_t)k0 * kPanel;               // inverse of block jb
      if (staged) {
        if (q > 0) await((q - 1) & 1);
        if (warp == 0) await(2 + (q & 1));
        else ph ^= 1u << (2 + (q & 1));  // the other threads only follow the inverse barriers' phases
        if (!*S.fail) {
          if (q > 0) Pc = sbuf(q - 1);
          Inv = sinv(q);
        }
      }
      const float* yp = yb[(q + 1) & 1];  // y of block pj (written at step q - 1)
      if (warp == 0) {
        if (pslot >= 0) xw[pslot] = pv;  // refill from the previous step
        pslot = -1;
        // near rows: the rows of block jb receive block pj
        if (q > 0 && lane < kb) {
          const int i = k0 + lane;
          float a0 = 0.f, a1 = 0.f;
          if (fwd) {  // L(i, pk0 + t), d = i - pk0 - t in [1, b]
            const int tlo = max(0, i - pk0 - b);
            int t = tlo;
            if (Pc && tlo == 0 && pkb == kPanel) {
              a0 = row_dot32(Pc + (i - pk0 - 1), b - 1, yp);
            } else if (Pc) {
              const float* col = Pc + (i - pk0 - 1);
              for (; t + 1 < pkb; t += 2) {
                a0 = fmaf(col[t * (b - 1)], yp[t], a0);
                a1 = fmaf(col[(t + 1) * (b - 1)], yp[t + 1], a1);
              }
              if (t < pkb) a0 = fmaf(col[t * (b - 1)], yp[t], a0);
            } else {
              for (; t + 1 < pkb; t += 2) {
                a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
                a1 = fmaf(V.at(i, pk0 + t + 1), yp[t + 1], a1);
              }
              if (t < pkb) a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
            }
          } else {  // U(i, pk0 + t), d = pk0 + t - i in [1, b]
            const int thi = min(pkb, i + b - pk0 + 1);
            int t = 0;
            if (Pc && thi == kPanel) {
              a0 = row_dot32(Pc + (b - pk0 + i), b, yp);
            } else if (Pc) {
              const float* col = Pc + (b - pk0 + i);
              for (; t + 1 < thi; t += 2) {
                a0 = fmaf(col[t * b], yp[t], a0);
                a1 = fmaf(col[(t + 1) * b], yp[t + 1], a1);
              }
              if (t < thi) a0 = fmaf(col[t * b], yp[t], a0);
            } else {
              for (; t + 1 < thi; t += 2) {
                a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
                a1 = fmaf(V.at(i, pk0 + t + 1), yp[t + 1], a1);
              }
              if (t < thi) a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
            }
          }
          X(i) -= a0 + a1;
        }
        __syncwarp();
        // diagonal block: y = Inv x over the block's rows (two accumulators)
        float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
        float* xb = &X(k0);
#pragma unroll
        for (int t = 0; t < kPanel; t += 4) {
          if (t < kb) d0 = fmaf(Inv[t * kPanel + lane], xb[t], d0);
          if (t + 1 < kb) d1 = fmaf(Inv[(t + 1) * kPanel + lane], xb[t + 1], d1);
          if (t + 2 < kb) d2 = fmaf(Inv[(t + 2) * kPanel + lane], xb[t + 2], d2);
          if (t + 3 < kb) d3 = fmaf(Inv[(t + 3) * kPanel + lane], xb[t + 3], d3);
        }
        __syncwarp();
        if (lane < kb) {
          const float y = (d0 + d1) + (d2 + d3);
          xb[lane] = y;
          yb[q & 1][lane] = y;
          if (win) {  // the block is final: write it back, load the row that takes its slot
            x[k0 + lane] = y;
            const int nr = fwd ? k0 + W + lane : k0 - W + lane;
            if (nr >= 0 && nr < n) {
              pv = x[nr];
              pslot = (k0 + lane) & wm;
            }
          }
        }
      } else if (q > 0) {
        // far rows receive block pj (threads of warps 1.. only)
        const int tid = threadIdx.x - 32, nth = blockDim.x - 32;
        if (fwd) {
          const int r1 = min(n, pk0 + pkb + b);
          for (int i = pk0 + 2 * kPanel + tid; i < r1; i += nth) {
            const int tlo = max(0, i - pk0 - b);
            float a0 = 0.f, a1 = 0.f;
            int t = tlo;
            if (Pc && tlo == 0 && pkb == kPanel) {
              a0 = row_dot32(Pc + (i - pk0 - 1), b - 1, yp);
            } else if (Pc) {
              const float* col = Pc + (i - pk0 - 1);
              for (; t + 1 < pkb; t += 2) {
                a0 = fmaf(col[t * (b - 1)], yp[t], a0);
                a1 = fmaf(col[(t + 1) * (b - 1)], yp[t + 1], a1);
              }
              if (t < pkb) a0 = fmaf(col[t * (b - 1)], yp[t], a0);
            } else {
              for (; t + 1 < pkb; t += 2) {
                a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
                a1 = fmaf(V.at(i, pk0 + t + 1), yp[t + 1], a1);
              }
              if (t < pkb) a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
            }
            X(i) -= a0 + a1;
          }
        } else {
          const int r0 = max(0, pk0 - b);
          for (int i = r0 + tid; i < pk0 - kPanel; i += nth) {
            const int thi = min(pkb, i + b - pk0 + 1);
            float a0 = 0.f, a1 = 0.f;
            int t = 0;
            if (Pc && thi == kPanel) {
              a0 = row_dot32(Pc + (b - pk0 + i), b, yp);
            } else if (Pc) {
              const float* col = Pc + (b - pk0 + i);
              for (; t + 1 < thi; t += 2) {
                a0 = fmaf(col[t * b], yp[t], a0);
                a1 = fmaf(col[(t + 1) * b], yp[t + 1], a1);
              }
              if (t < thi) a0 = fmaf(col[t * b], yp[t], a0);
            } else {
              for (; t + 1 < thi; t += 2) {
                a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
                a1 = fmaf(V.at(i, pk0 + t + 1), yp[t + 1], a1);
              }
              if (t < thi) a0 = fmaf(V.at(i, pk0 + t), yp[t], a0);
            }
            X(i) -= a0 + a1;
          }
        }
      }
      __syncthreads();
      // buffers freed at this step: band columns of block pj, inverse of block jb
      if (staged && issuer && !*S.fail) {
        if (q + 1 <= nblk - 2) issue_cols(blk(q + 1), (q + 1) & 1, fwd);
        if (q + 2 <= nblk - 1) issue_inv(blk(q + 2), q & 1, fwd, 0u);
      }
    }
    if (warp == 0 && pslot >= 0) xw[pslot] = pv;
    if (!win) continue;
    __syncthreads();
  }
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int node = B.node_at[n0 + r / 6];
    z[6 * (node - n0) + r % 6] = (TZ)x[r];
  }
  __syncthreads();
}

void launch_band_fill(const Dev& d, const BandDev& B, const int* blk_row, cudaStream_t s);
cudaError_t launch_band_lu(const Dev& d, const BandDev& B, int max_b, cudaStream_t s);
// The same factorisation with the trailing updates on the tensor cores (eb_band_tc.cu); its
// shared memory for the widest band of the launch is band_lu_tc_smem(max_b).
cudaError_t launch_band_lu_tc(const Dev& d, const BandDev& B, int max_b, int* lu_fail, cudaStream_t s);
size_t band_lu_tc_smem(int max_b);
constexpr size_t kLuTcSmemLimit = 227 * 1024;  // the opt-in shared memory of one CTA (the kernel has no static part)

}  // namespace eb
