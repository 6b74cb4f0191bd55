// Band LU with the trailing update on the fifth-generation tensor cores.
//
// Same factorisation as k_band_lu (eb_band.cu): blocked right-looking LU
// without pivoting of one simulation's FP32 band, one CTA per simulation,
// panels of 32 columns.  Per panel:
//   1. the panel (rows k0 .. k0+32+q) is factorised in shared memory (FP32);
//   2. U12 = L11⁻¹ A12, one thread per column, written back to the band and,
//      split into BF16 pairs (hi + lo), into the B operand in shared memory;
//   3. the L11 / U11 inverses for the triangular solves;
//   4. A22 -= L21 U12 (q x q, K = 32) on the tensor cores: L21 is split into
//      three BF16 parts (hi + mid + lo = the FP32 value) 128 rows at a time (A
//      operand), U12 likewise (B operand), and each 128 x 128 output tile is the
//      sum of the six BF16 products above FP32's rounding level (mm, lh, hl,
//      mh, hm, hh, smallest first) accumulated in FP32 in tensor memory — the
//      rounding of an FP32 product (a two-part split, three products, left the
//      factors ~1e-5 off and cost 60% more GMRES iterations); the epilogue warps
//      read the tile from tensor memory and update the band in global memory
//      (each warp's 32 lanes are 32 consecutive rows, so every column's update
//      is one coalesced 128-byte access).  Tile t+1's MMAs run on the tensor
//      core while the warps update tile t (two accumulators).
// The MMA completion waits are bounded: when one runs out the simulation's
// flag in `lu_fail` is set, the kernel waits (bounded) for its MMAs still in
// flight, releases its tensor memory and stops; the solver then reports the
// step not converged and the handle goes back to the FP32 kernel.
#include "../../include/endobeams_gb300.h"
#include "eb_band.cuh"
#include "eb_umma.cuh"

namespace eb {

namespace {

constexpr int kTcThreads = 512;  // 16 warps: warp w updates tile lanes 32 (w % 4) .., columns 32 (w / 4) ..
constexpr int kTile = 128;       // M = N = 128 per MMA
constexpr uint32_t kTmemCols = 2 * kTile;
constexpr int kOpBytes = kTile * 64;  // one 128-row, 32-wide-K BF16 operand tile (hi or lo)
constexpr int kU12 = 3 * kOpBytes / (33 * 4);  // U12 columns staged at a time in the A operand buffers (186)

// Shared memory of one CTA for half bandwidth b (bytes): mbarriers and the tensor-memory slot,
// the FP32 panel ((32 + b) x 32, odd column stride), the B operand (three parts, q <= b columns
// rounded up to 128) and one A operand chunk (three parts).
__host__ __device__ inline size_t tc_ldp(int b) { return (size_t)kPanel + b; }
__host__ __device__ inline size_t tc_npad(int b) { return ((size_t)b + kTile - 1) / kTile * kTile; }
__host__ __device__ inline size_t tc_smem_bytes(int b) {
  return 1024 + sizeof(float) * tc_ldp(b) * kPanel + 3 * 64 * tc_npad(b) + 3 * (size_t)kOpBytes;
}

// Eight consecutive K values of one operand row, split into parts, stored at `off` of each part.
__device__ __forceinline__ void store_pair(char* hi, char* lo, uint32_t off, const float (&x)[8]) {
  __nv_bfloat16 h[8], l[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) umma::split_bf16(x[j], h[j], l[j]);
  *reinterpret_cast<uint4*>(hi + off) = *reinterpret_cast<const uint4*>(h);
  *reinterpret_cast<uint4*>(lo + off) = *reinterpret_cast<const uint4*>(l);
}
__device__ __forceinline__ void store_triple(char* const (&part)[3], uint32_t off, const float (&x)[8]) {
  __nv_bfloat16 h[8], m[8], l[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) umma::split3_bf16(x[j], h[j], m[j], l[j]);
  *reinterpret_cast<uint4*>(part[0] + off) = *reinterpret_cast<const uint4*>(h);
  *reinterpret_cast<uint4*>(part[1] + off) = *reinterpret_cast<const uint4*>(m);
  *reinterpret_cast<uint4*>(part[2] + off) = *reinterpret_cast<const uint4*>(l);
}

// The six products of two three-part splits above FP32's rounding level, smallest first, for
// one K step (byte offset ko into every part); the first accumulates onto D only if acc.
__device__ __forceinline__ void mma_split3(uint32_t dt, const uint32_t (&a)[3], const uint32_t (&b)[3], uint32_t ko,
                                           uint32_t idesc, uint32_t acc) {
  constexpr int pa[6] = {1, 2, 0, 1, 0, 0};  // A part: mid, lo, hi, mid, hi, hi
  constexpr int pb[6] = {1, 0, 2, 0, 1, 0};  // B part: mid, hi, lo, hi, mid, hi
#pragma unroll
  for (int t = 0; t < 6; ++t)
    umma::mma_bf16(dt, umma::smem_desc(a[pa[t]] + ko, 128, 512), umma::smem_desc(b[pb[t]] + ko, 128, 512), idesc,
                   t == 0 ? acc : 1u);
}

}  // namespace

__global__ void __launch_bounds__(kTcThreads) k_band_lu_tc(Dev d, BandDev B, int* lu_fail) {
  const int s = B.order[blockIdx.x];
  if (!d.active[s] || !B.refactor[s]) return;
  const int b = B.bw[s];
  if (b == 0) return;
  const int64_t n0 = d.sim_node_off[s];
  const int n = (int)(6 * (d.sim_node_off[s + 1] - n0));
  const BandView V = band_view(B, s, n);
  float* Li = B.Linv + inv_base(n0, s);
  float* Ui = B.Uinv + inv_base(n0, s);
  extern __shared__ __align__(1024) char smc[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smc);          // two MMA-completion barriers
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smc + 64);   // tensor-memory base address
  const int ldp = (int)tc_ldp(b);
  float* P = reinterpret_cast<float*>(smc + 1024);                        // panel, ldp x 32 column-major
  const size_t npad = tc_npad(b);
  char* const Bp[3] = {reinterpret_cast<char*>(P + (size_t)ldp * kPanel),  // B operand: q columns (N), K = 32
                       reinterpret_cast<char*>(P + (size_t)ldp * kPanel) + 64 * npad,
                       reinterpret_cast<char*>(P + (size_t)ldp * kPanel) + 128 * npad};
  char* const Ap[3] = {Bp[2] + 64 * npad, Bp[2] + 64 * npad + kOpBytes,  // A operand chunk: 128 rows (M)
                       Bp[2] + 64 * npad + 2 * kOpBytes};
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nw = kTcThreads / 32;

  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_async_smem();
  }
  if (warp == 0) umma::tmem_alloc(tslot, kTmemCols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = umma::idesc_bf16_f32(kTile, kTile);
  uint32_t phase[2] = {0u, 0u};  // next completion parity of each accumulator's barrier
  int pending[2] = {0, 0};       // thread 0: commits not yet waited for
  bool failed = false;

  for (int k0 = 0; k0 < n && !failed; k0 += kPanel) {
    const int kb = min(kPanel, n - k0);
    const int hp = min(n - k0, kb + b);
    const int q = min(n - k0 - kb, b);
    // ---- load the panel: warp per column, lanes along the rows (a band column is contiguous in
    // rows, so each warp access is one 128-byte line)
    for (int c = warp; c < kb; c += nw)
      for (int r = lane; r < hp; r += 32) {
        const int i = k0 + r, j = k0 + c;
        P[r + ldp * c] = (i - j <= b && j - i <= b) ? V.at(i, j) : 0.f;
      }
    __syncthreads();
    // ---- 1. panel LU: warp w owns columns w and w + 16, its lanes run along the rows.  At
    // column t every owner of a later column subtracts column t's multipliers times its row-t
    // entry, and the owner of column t + 1 then scales that column by its pivot itself (same
    // warp), so one block barrier per column publishes the next multipliers.  Each entry sees
    // the same operations in the same order as a column-by-column elimination.
    if (warp == 0 && kb > 0) {
      const float ip = 1.f / P[0];
      for (int r = 1 + lane; r < hp; r += 32) P[r] *= ip;
    }
    for (int t = 0; t < kb; ++t) {
      __syncthreads();  // column t's multipliers and row t are final
      for (int c = warp; c < kb; c += nw) {
        if (c <= t) continue;
        const float ut = P[t + ldp * c];
        for (int r = t + 1 + lane; r < hp; r += 32) P[r + ldp * c] -= P[r + ldp * t] * ut;
        if (c == t + 1) {
          __syncwarp();
          const float ip = 1.f / P[c + ldp * c];
          for (int r = c + 1 + lane; r < hp; r += 32) P[r + ldp * c] *= ip;
        }
      }
    }
    __syncthreads();
    // inverses of L11 (unit lower, which = 0) and U11 (upper, which = 1), one column per lane,
    // by column-oriented substitution: the updates of one step are independent, so the
    // dependent chain is 32 steps long instead of 496 multiply-adds
    auto inverses = [&](int which) {
      float z[kPanel];
#pragma unroll
      for (int r = 0; r < kPanel; ++r) z[r] = (r == lane) ? 1.f : 0.f;
      if (which == 0) {
#pragma unroll
        for (int t = 0; t < kPanel - 1; ++t)
#pragma unroll
          for (int r = t + 1; r < kPanel; ++r) z[r] -= (r < kb && t < kb ? P[r + ldp * t] : 0.f) * z[t];
      } else {
#pragma unroll
        for (int t = kPanel - 1; t >= 0; --t) {
          if (t < kb) z[t] = z[t] / P[t + ldp * t];
#pragma unroll
          for (int r = 0; r < t; ++r) z[r] -= (r < kb && t < kb ? P[r + ldp * t] : 0.f) * z[t];
        }
      }
      float* dst = (which == 0 ? Li : Ui) + (int64_t)k0 * kPanel;
#pragma unroll
      for (int r = 0; r < kPanel; ++r) dst[lane * kPanel + r] = z[r];
    };
    // ---- 2. U12 = L11⁻¹ A12 (q > 0 implies kb = 32), into the band and B, kU12 columns at a
    // time through the (idle) A operand buffer: each column is loaded and stored by one warp
    // (32 rows, one 128-byte line), solved by one thread from shared memory (stride 33: no bank
    // conflicts).  Entries of A12 with j - i > b lie outside the band: zero, not written back.
    float* S = reinterpret_cast<float*>(Ap[0]);
    for (int cs = 0; cs < q; cs += kU12) {
      const int cn = min(kU12, q - cs);
      for (int c = warp; c < cn; c += nw) {
        const int j = k0 + kPanel + cs + c, i = k0 + lane;
        S[lane + 33 * c] = (j - i <= b) ? V.at(i, j) : 0.f;
      }
      __syncthreads();
      // the first chunk's solves occupy threads below kU12 (warps 0-5); the two top warps
      // compute the panel inverses meanwhile
      static_assert(kU12 <= kTcThreads - 64, "inverse warps must be idle in the U12 solve");
      if (cs == 0 && warp >= nw - 2) inverses(warp - (nw - 2));
      for (int c = threadIdx.x; c < cn; c += kTcThreads) {
        float col[kPanel];
#pragma unroll
        for (int r = 0; r < kPanel; ++r) col[r] = S[r + 33 * c];
        // forward substitution column by column: the 31 - t updates of step t are independent
#pragma unroll
        for (int t = 0; t < kPanel - 1; ++t)
#pragma unroll
          for (int r = t + 1; r < kPanel; ++r) col[r] -= P[r + ldp * t] * col[t];
#pragma unroll
        for (int r = 0; r < kPanel; ++r) S[r + 33 * c] = col[r];
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          float x[8];
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) x[jj] = col[8 * g + jj];
          store_triple(Bp, umma::kmajor_offset(cs + c, 8 * g), x);
        }
      }
      __syncthreads();
      for (int c = warp; c < cn; c += nw) {
        const int j = k0 + kPanel + cs + c, i = k0 + lane;
        if (j - i <= b) V.at(i, j) = S[lane + 33 * c];
      }
      __syncthreads();
    }
    // B columns past q (up to the 128-column tile) are zero
    for (int c = q + threadIdx.x; c < (int)((q + kTile - 1) / kTile * kTile); c += kTcThreads) {
      const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int g = 0; g < 4; ++g) store_triple(Bp, umma::kmajor_offset(c, 8 * g), z);
    }
    // ---- 3. without U12 work (last panel) the inverses run here, on warps 0 and 1
    if (q <= 0 && warp < 2) inverses(warp);
    // ---- write back the panel (L11, U11, L21), warp per column as it was loaded
    for (int c = warp; c < kb; c += nw)
      for (int r = lane; r < hp; r += 32) {
        const int i = k0 + r, j = k0 + c;
        if (i - j <= b && j - i <= b) V.at(i, j) = P[r + ldp * c];
      }
    __syncthreads();
    if (q <= 0) continue;
    // ---- 4. A22 -= L21 U12 on the tensor cores, 128 x 128 tiles, M chunk by M chunk
    const int mt = (q + kTile - 1) / kTile, nt = mt;
    for (int mc = 0; mc < mt && !failed; ++mc) {
      // A operand: rows 128 mc .. of L21 (panel rows 32 + m), split into BF16 pairs; rows past q are zero
      for (int u = threadIdx.x; u < kTile * 4; u += kTcThreads) {
        const int ml = u % kTile, g = u / kTile, m = kTile * mc + ml;
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = m < q ? P[(kPanel + m) + ldp * (8 * g + j)] : 0.f;
        store_triple(Ap, umma::kmajor_offset(ml, 8 * g), x);
      }
      umma::fence_proxy_async();  // operand writes visible to the tensor core
      umma::fence_before_sync();
      __syncthreads();
      umma::fence_after_sync();
      // tile (mc, nc) accumulates in tensor-memory columns 128 (nc % 2) ..
      auto issue = [&](int nc) {
        const uint32_t dt = tmem + (uint32_t)(kTile * (nc & 1));
        const uint32_t a[3] = {umma::smem_addr(Ap[0]), umma::smem_addr(Ap[1]), umma::smem_addr(Ap[2])};
        const uint32_t bb[3] = {umma::smem_addr(Bp[0] + (size_t)nc * kOpBytes),
                                umma::smem_addr(Bp[1] + (size_t)nc * kOpBytes),
                                umma::smem_addr(Bp[2] + (size_t)nc * kOpBytes)};
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) mma_split3(dt, a, bb, 256u * ks, idesc, ks);  // K = 32 as two K = 16 steps
        umma::commit(&bar[nc & 1]);
        pending[nc & 1] += 1;
      };
      if (threadIdx.x == 0) issue(0);
      const int quarter = warp & 3, group = warp >> 2;
      const int m = kTile * mc + 32 * quarter + lane;
      const int i = k0 + kPanel + m;
      for (int nc = 0; nc < nt; ++nc) {
        const int buf = nc & 1;
        // row i, columns jb .. jb + 31 of this warp's part of tile nc: the columns left of the
        // diagonal (j < i) are in the L part at L + (i - 1) + (b - 1) j, the others in the U part
        // at U + b + i + b j, so each address is one multiply-add from two row bases.  The old
        // values are loaded before the MMA wait: their latency overlaps the tensor-core work.
        const int c0 = 32 * group;
        const int jb = k0 + kPanel + kTile * nc + c0;
        const int cmax = m < q ? min(32, q - (kTile * nc + c0)) : 0;
        const int sp = min(max(i - jb, 0), 32);
        float* pL = V.L + ((int64_t)i - 1 + (int64_t)(b - 1) * jb);
        float* pU = V.U + ((int64_t)b + i + (int64_t)b * jb);
        float old[32];
#pragma unroll
        for (int c = 0; c < 32; ++c)
          old[c] = c < cmax ? (c < sp ? pL[(int64_t)(b - 1) * c] : pU[(int64_t)b * c]) : 0.f;
        const bool done = mbar_wait(&bar[buf], phase[buf]);
        if (threadIdx.x == 0 && done) pending[buf] -= 1;
        phase[buf] ^= 1u;
        // this barrier also orders every thread's accumulator read of tile nc - 1 (same buffer
        // as tile nc + 1) before the MMAs of tile nc + 1 are issued; all threads get the same
        // answer from it, so they leave the loop together
        umma::fence_before_sync();
        const int timed_out = __syncthreads_or(!done);
        umma::fence_after_sync();
        if (timed_out) {
          failed = true;
          break;
        }
        // the next tile's MMAs run while this one is written back (its accumulator was
        // released by the barrier that ended tile nc - 1)
        if (threadIdx.x == 0 && nc + 1 < nt) issue(nc + 1);
        float acc[32];
        umma::ld_32cols(tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(kTile * buf + c0), acc);
#pragma unroll
        for (int c = 0; c < 32; ++c)
          if (c < cmax) (c < sp ? pL[(int64_t)(b - 1) * c] : pU[(int64_t)b * c]) = old[c] - acc[c];
        // no barrier here: a warp goes on to load the next tile's old values (other columns)
        // while the others still store this one
      }
    }
    __syncthreads();
  }
  if (failed) {
    // a completion wait ran out: wait (bounded) for the MMAs still in flight before the
    // tensor memory is released
    if (threadIdx.x == 0) {
      for (int k = 0; k < 2; ++k)
        while (pending[k] > 0) {
          mbar_wait(&bar[k], phase[k]);
          phase[k] ^= 1u;
          pending[k] -= 1;
        }
      lu_fail[s] = 1;
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::tmem_dealloc(tmem, kTmemCols);
}

size_t band_lu_tc_smem(int max_b) { return tc_smem_bytes(max_b); }

cudaError_t launch_band_lu_tc(const Dev& d, const BandDev& B, int max_b, int* lu_fail, cudaStream_t s) {
  if (max_b <= 0) return cudaSuccess;
  const size_t smem = tc_smem_bytes(max_b);
  cudaError_t e = raise_smem_limit((const void*)k_band_lu_tc, smem);
  if (e != cudaSuccess) return e;
  k_band_lu_tc<<<d.n_sims, kTcThreads, smem, s>>>(d, B, lu_fail);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- single-tile self-test
// One CTA of 128 threads: D (128 x N) = A (128 x 32) B (N x 32)ᵀ with the operands rounded to
// BF16 (split = 0) or split into BF16 pairs with the three-product sum of the band LU (split = 1).
__global__ void k_umma_selftest(const float* __restrict__ A, const float* __restrict__ Bm, int N, int split,
                                float* __restrict__ D, int* status) {
  extern __shared__ __align__(1024) char smc[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smc);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smc + 64);
  char* const Ap[3] = {smc + 1024, smc + 1024 + kOpBytes, smc + 1024 + 2 * kOpBytes};
  char* const Bp[3] = {Ap[2] + kOpBytes, Ap[2] + 3 * kOpBytes, Ap[2] + 5 * kOpBytes};  // N <= 256 rows each
  char* Ahi = Ap[0];
  char* Alo = Ap[1];
  char* Bhi = Bp[0];
  char* Blo = Bp[1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int u = threadIdx.x; u < kTile * 4; u += blockDim.x) {
    const int r = u % kTile, g = u / kTile;
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = A[r * 32 + 8 * g + j];
    if (split == 2) store_triple(Ap, umma::kmajor_offset(r, 8 * g), x);
    else store_pair(Ahi, Alo, umma::kmajor_offset(r, 8 * g), x);
  }
  for (int u = threadIdx.x; u < N * 4; u += blockDim.x) {
    const int r = u % N, g = u / N;
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = Bm[r * 32 + 8 * g + j];
    if (split == 2) store_triple(Bp, umma::kmajor_offset(r, 8 * g), x);
    else store_pair(Bhi, Blo, umma::kmajor_offset(r, 8 * g), x);
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    fence_async_smem();
  }
  if (warp == 0) umma::tmem_alloc(tslot, 256);
  umma::fence_proxy_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  if (threadIdx.x == 0) {
    const uint32_t idesc = umma::idesc_bf16_f32(kTile, N);
    const uint32_t a_hi = umma::smem_addr(Ahi), a_lo = umma::smem_addr(Alo);
    const uint32_t b_hi = umma::smem_addr(Bhi), b_lo = umma::smem_addr(Blo);
    const uint32_t a3[3] = {umma::smem_addr(Ap[0]), umma::smem_addr(Ap[1]), umma::smem_addr(Ap[2])};
    const uint32_t b3[3] = {umma::smem_addr(Bp[0]), umma::smem_addr(Bp[1]), umma::smem_addr(Bp[2])};
    for (int ks = 0; ks < 2; ++ks) {
      const uint32_t o = 256u * ks;
      if (split == 2) {
        mma_split3(tmem, a3, b3, o, idesc, ks);
        continue;
      }
      umma::mma_bf16(tmem, umma::smem_desc(a_hi + o, 128, 512), umma::smem_desc(b_hi + o, 128, 512), idesc, ks);
      if (split) {
        umma::mma_bf16(tmem, umma::smem_desc(a_hi + o, 128, 512), umma::smem_desc(b_lo + o, 128, 512), idesc, 1);
        umma::mma_bf16(tmem, umma::smem_desc(a_lo + o, 128, 512), umma::smem_desc(b_hi + o, 128, 512), idesc, 1);
      }
    }
    umma::commit(&bar[0]);
  }
  const bool ok = mbar_wait(&bar[0], 0);
  umma::fence_after_sync();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 32) {
      float acc[32];
      umma::ld_32cols(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, acc);
      const int r = 32 * warp + lane;
#pragma unroll
      for (int c = 0; c < 32; ++c) D[(int64_t)r * N + c0 + c] = acc[c];
    }
  } else if (threadIdx.x == 0) {
    *status = 1;
    mbar_wait(&bar[0], 0);  // bounded second wait for the MMAs in flight
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

}  // namespace eb

extern "C" int eb_umma_selftest(const float* A, const float* B, int32_t N, int32_t split, float* D) {
  using namespace eb;
  if (!A || !B || !D || !(N == 64 || N == 128 || N == 256) || split < 0 || split > 2) return EB_ERR_ARG;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* dst = nullptr;
  int st = 0;
  cudaError_t e = cudaSuccess;
  const size_t smem = 1024 + 3 * (size_t)kOpBytes + 6 * (size_t)kOpBytes;
  if ((e = cudaMalloc(&dA, sizeof(float) * 128 * 32)) == cudaSuccess &&
      (e = cudaMalloc(&dB, sizeof(float) * (size_t)N * 32)) == cudaSuccess &&
      (e = cudaMalloc(&dD, sizeof(float) * 128 * (size_t)N)) == cudaSuccess &&
      (e = cudaMalloc(&dst, sizeof(int))) == cudaSuccess &&
      (e = cudaMemcpy(dA, A, sizeof(float) * 128 * 32, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemcpy(dB, B, sizeof(float) * (size_t)N * 32, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemset(dst, 0, sizeof(int))) == cudaSuccess &&
      (e = cudaFuncSetAttribute(k_umma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) ==
          cudaSuccess) {
    k_umma_selftest<<<1, 128, smem>>>(dA, dB, N, split, dD, dst);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(D, dD, sizeof(float) * 128 * (size_t)N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost);
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dst);
  if (e != cudaSuccess) return EB_ERR_CUDA;
  return st ? EB_ERR_CUDA : EB_OK;
}
