// Linear solve of the Newton step, replacing MKL PARDISO (src/linearsolvers.jl,
// called from solve_free_dofs!, src/utils_solver.jl:107-120).
//
// Ktan_free ΔD_free = r_free is solved per simulation by right-preconditioned
// GMRES with a 6x6 block-Jacobi preconditioner (the LU of each node's
// diagonal block, fixed DOFs replaced by identity rows/columns).  Each
// simulation is owned by one CTA for the whole solve: its Krylov basis
// lives in global memory (L2-resident for the sizes of a batched run), its
// Hessenberg matrix and Givens rotations in shared memory, and every
// reduction is a fixed-order block reduction, so results do not depend on
// how many simulations share the launch.
//
// Precision: the outer loop always measures the true residual b - A x in
// FP64.  Each pass runs one GMRES(m) cycle on that residual, in FP64
// (EB_PREC_FP64) or in FP32 with FP32 matrix and preconditioner
// (EB_PREC_MIXED: iterative refinement).  A pass is therefore both the
// GMRES restart and the refinement sweep.
#include <cfloat>
#include <type_traits>

#include "eb_band.cuh"
#include "eb_gmres.cuh"

namespace eb {

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; ++q) red[q * 32 + warp] = v[q];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double x = lane < nw ? red[q * 32 + lane] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
      if (lane == 0) red[q * 32] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = red[q * 32];
  __syncthreads();
}

// y = P A x over the rows of one simulation (P zeroes fixed rows).
template <typename TA, typename TX, typename TY, typename TACC>
__device__ __forceinline__ void cta_spmv(const TA* __restrict__ A, const int* __restrict__ row_ptr,
                                         const int* __restrict__ col, int64_t n0, int n, const TX* __restrict__ x,
                                         TY* __restrict__ y, const uint8_t* __restrict__ fx) {
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int64_t node = n0 + r / 6;
    const int k = r % 6;
    TACC acc = 0;
    for (int bb = row_ptr[node]; bb < row_ptr[node + 1]; ++bb) {
      const int c = (int)(col[bb] - n0);
      const TA* Ab = A + (int64_t)bb * 36 + k;
      const TX* xc = x + 6 * c;
#pragma unroll
      for (int j = 0; j < 6; ++j) acc += (TACC)Ab[6 * j] * (TACC)xc[j];
    }
    y[r] = fx[r] ? (TY)0 : (TY)acc;
  }
}

// z = M⁻¹ v with M the block diagonal
template <typename TM, typename TV, typename TZ>
__device__ __forceinline__ void cta_prec(const TM* __restrict__ Dinv, int64_t n0, int n, const TV* __restrict__ v,
                                         TZ* __restrict__ z) {
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int nl = r / 6, k = r % 6;
    const TM* Db = Dinv + (n0 + nl) * 36 + k;
    const TV* vv = v + 6 * nl;
    TM acc = 0;
#pragma unroll
    for (int j = 0; j < 6; ++j) acc += Db[6 * j] * (TM)vv[j];
    z[r] = (TZ)acc;
  }
}

template <typename T>
__global__ void __launch_bounds__(512) k_gmres(SolverArgs a) {
  const int s = a.cta_sim[blockIdx.x];
  if (!a.active[s]) return;
  const int m = a.m;
  const int64_t n0 = a.sim_node_off[s];
  const int64_t o = 6 * n0;
  const int n = (int)(6 * (a.sim_node_off[s + 1] - n0));
  extern __shared__ double sm[];
  double* H = sm;                  // (m+1) x m, column j at H + (m+1) j
  double* cs = H + (m + 1) * m;
  double* sn = cs + m;
  double* g = sn + m;              // m+1
  double* y = g + m + 1;           // m
  double* red = y + m;             // 8 x 32
  T* V = reinterpret_cast<T*>(a.V) + (int64_t)(m + 1) * o;
  T* Zb = reinterpret_cast<T*>(a.Z) + (int64_t)m * o;  // z_j = M⁻¹ v_j at Zb + j n
  double* X = a.X + o;
  double* R = a.R64 + o;
  const double* b = a.b + o;
  const uint8_t* fx = a.fixed + o;
  const T* Am = std::is_same<T, double>::value ? reinterpret_cast<const T*>(a.Kt) : reinterpret_cast<const T*>(a.Kt32);
  const T* Dm = std::is_same<T, double>::value ? reinterpret_cast<const T*>(a.Dinv64)
                                              : reinterpret_cast<const T*>(a.Dinv32);
  using TACC = T;
  const bool use_band = a.band.bw != nullptr && a.band.bw[s] > 0;
  float* xs = a.x_in_smem ? reinterpret_cast<float*>(red + 8 * 32) : nullptr;  // permuted solve vector
  // shared-memory staging of band blocks for the triangular solves (bulk async copies)
  __shared__ __align__(8) uint64_t bars[4];
  __shared__ int stage_fail;
  __shared__ int stage_pend[4];
  Stage stage;
  const Stage* stp = nullptr;
  uint32_t ph = 0u;  // bit k: next phase of staging barrier k
  if (use_band && a.stage_floats > 0) {
    char* base = reinterpret_cast<char*>(xs ? xs + a.max_n : reinterpret_cast<float*>(red + 8 * 32));
    base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(base) + 127) & ~uintptr_t(127));
    // two band-column buffers of stage_floats = 32 (b_max + 1) floats, then the inverses
    float* f = reinterpret_cast<float*>(base);
    stage.buf[0] = f;
    stage.buf[1] = f + a.stage_floats;
    stage.inv[0] = f + 2 * (int64_t)a.stage_floats;
    stage.inv[1] = stage.inv[0] + kPanel * kPanel;
    stage.bar = bars;
    stage.fail = &stage_fail;
    stage.pend = stage_pend;
    stage.extra = (uint32_t)a.stage_test_extra;
    if (threadIdx.x == 0) {
      for (int k = 0; k < 4; ++k) {
        mbar_init(&bars[k], 1);
        stage_pend[k] = -1;
      }
      stage_fail = 0;
      fence_async_smem();
    }
    __syncthreads();
    stp = &stage;
  }

  double v1[1] = {0.0};
  const bool use_x0 = a.x0_on != nullptr && a.x0_on[s] != 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double bi = fx[i] ? 0.0 : b[i];
    X[i] = (use_x0 && !fx[i]) ? a.dD[o + i] : 0.0;
    R[i] = bi;
    v1[0] += bi * bi;
  }
  block_sum<1>(v1, red);
  const double bnorm = sqrt(v1[0]);
  double rnorm = bnorm;
  if (use_x0 && isfinite(bnorm)) {
    // initial guess: X = α x0 with α = <A x0, b> / <A x0, A x0> clipped to [0, 1], so that
    // ‖b − A X‖ <= ‖b‖ (a guess that does not help costs one FP64 product)
    cta_spmv<double, double, double, double>(a.Kt, a.row_ptr, a.col, n0, n, X, R, fx);
    __syncthreads();
    double yb[2] = {0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double bi = fx[i] ? 0.0 : b[i];
      yb[0] += R[i] * bi;
      yb[1] += R[i] * R[i];
    }
    block_sum<2>(yb, red);
    double alpha = yb[1] > 0.0 ? yb[0] / yb[1] : 0.0;
    if (!(alpha > 0.0)) alpha = 0.0;
    if (alpha > 1.0) alpha = 1.0;
    double rr0[1] = {0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double bi = fx[i] ? 0.0 : b[i];
      X[i] *= alpha;
      const double ri = bi - alpha * R[i];
      R[i] = ri;
      rr0[0] += ri * ri;
    }
    block_sum<1>(rr0, red);
    rnorm = sqrt(rr0[0]);
  }
  int its = 0, refs = 0, status = 0;
  if (!isfinite(bnorm)) status = 2;  // EB_SIM_NAN
  // the tensor-core factorisation of these factors stopped at a bounded wait: not trusted
  if (use_band && a.band.lu_fail && a.band.lu_fail[s]) status = 4;

  // relative tolerance of this solve (inexact Newton, Eisenstat-Walker choice 2)
  double rtol = a.tol;
  if (a.forcing) {
    const double prev = a.prev_bnorm[s], pe = a.prev_eta[s];
    double eta = a.forcing_max;
    if (prev > 0.0) {
      const double q = bnorm / prev;
      eta = 0.9 * q * q;
      if (0.9 * pe * pe > 0.1) eta = fmax(eta, 0.9 * pe * pe);
      eta = fmin(fmax(eta, a.tol), a.forcing_max);
    }
    rtol = eta;
    __syncthreads();  // every thread has read the previous values
    if (threadIdx.x == 0) {
      a.prev_bnorm[s] = bnorm;
      a.prev_eta[s] = eta;
    }
  }
  if (status == 0 && bnorm > 0.0) {
    const double target = rtol * bnorm;
    for (int ref = 0; ref < a.max_ref && rnorm > target && its < a.max_iter; ++ref) {
      // ---- one GMRES(m) cycle on the FP64 residual R
      const double beta = rnorm;
      const double ib = 1.0 / beta;
      for (int i = threadIdx.x; i < n; i += blockDim.x) V[i] = (T)(R[i] * ib);
      if (threadIdx.x == 0) g[0] = beta;
      __syncthreads();
      const double inner_target = fmax(a.inner_tol * beta, 0.5 * target);
      int k = 0;  // dimension of the Krylov space built in this cycle
      const int jmax = min(m, a.max_iter - its);
      for (int j = 0; j < jmax; ++j) {
        T* vj = V + (int64_t)j * n;
        T* w = V + (int64_t)(j + 1) * n;
        T* zj = Zb + (int64_t)j * n;
        if (use_band) band_solve<T, T>(a.band, s, n0, n, vj, zj, xs, stp, ph);
        else cta_prec<T, T, T>(Dm, n0, n, vj, zj);
        __syncthreads();
        cta_spmv<T, T, T, TACC>(Am, a.row_ptr, a.col, n0, n, zj, w, fx);
        __syncthreads();
        // classical Gram-Schmidt, twice
        for (int pass = 0; pass < 2; ++pass) {
          for (int i0 = 0; i0 <= j; i0 += 8) {
            TACC hl[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) hl[q] = 0;
            const int nq = min(8, j + 1 - i0);
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
              const TACC wi = (TACC)w[i];
#pragma unroll
              for (int q = 0; q < 8; ++q)
                if (q < nq) hl[q] += (TACC)V[(int64_t)(i0 + q) * n + i] * wi;
            }
            double hp[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) hp[q] = (double)hl[q];
            block_sum<8>(hp, red);
            if (threadIdx.x == 0)
              for (int q = 0; q < nq; ++q) H[(m + 1) * j + i0 + q] = (pass == 0 ? 0.0 : H[(m + 1) * j + i0 + q]) + hp[q];
            // stash this chunk's coefficients in y (free until the back-substitution)
#pragma unroll
            for (int q = 0; q < 8; ++q)
              if (threadIdx.x == q && q < nq) y[i0 + q] = hp[q];
            __syncthreads();
          }
          for (int i = threadIdx.x; i < n; i += blockDim.x) {
            TACC acc = (TACC)w[i];
            for (int q = 0; q <= j; ++q) acc -= (TACC)y[q] * (TACC)V[(int64_t)q * n + i];
            w[i] = (T)acc;
          }
          __syncthreads();
        }
        TACC nl = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) nl += (TACC)w[i] * (TACC)w[i];
        double nn[1] = {(double)nl};
        block_sum<1>(nn, red);
        const double hn = sqrt(nn[0]);
        if (hn > 0.0) {
          const T ihn = (T)(1.0 / hn);
          for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = w[i] * ihn;
        }
        if (threadIdx.x == 0) {
          double* Hj = H + (m + 1) * j;
          Hj[j + 1] = hn;
          for (int i = 0; i < j; ++i) {
            const double t = cs[i] * Hj[i] + sn[i] * Hj[i + 1];
            Hj[i + 1] = -sn[i] * Hj[i] + cs[i] * Hj[i + 1];
            Hj[i] = t;
          }
          const double den = hypot(Hj[j], Hj[j + 1]);
          const double c = den > 0.0 ? Hj[j] / den : 1.0;
          const double sv = den > 0.0 ? Hj[j + 1] / den : 0.0;
          cs[j] = c;
          sn[j] = sv;
          Hj[j] = den;
          Hj[j + 1] = 0.0;
          g[j + 1] = -sv * g[j];
          g[j] = c * g[j];
        }
        __syncthreads();
        ++its;
        k = j + 1;
        const double gres = fabs(g[j + 1]);
        if (!(gres > inner_target) || hn <= DBL_MIN || !isfinite(gres)) break;
      }
      // back-substitution H y = g (k x k upper triangular)
      if (threadIdx.x == 0) {
        for (int i = k - 1; i >= 0; --i) {
          double t = g[i];
          for (int q = i + 1; q < k; ++q) t -= H[(m + 1) * q + i] * y[q];
          y[i] = t / H[(m + 1) * i + i];
        }
      }
      __syncthreads();
      // X += M⁻¹ V y = Z y: the preconditioned basis was kept, so the update needs no further
      // preconditioner application (one band solve per cycle saved)
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double acc = 0.0;
        for (int q = 0; q < k; ++q) acc += y[q] * (double)Zb[(int64_t)q * n + i];
        X[i] += acc;
      }
      __syncthreads();
      // true FP64 residual R = b - Ktan X
      cta_spmv<double, double, double, double>(a.Kt, a.row_ptr, a.col, n0, n, X, R, fx);
      __syncthreads();
      double rr[1] = {0.0};
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double ri = (fx[i] ? 0.0 : b[i]) - R[i];
        R[i] = ri;
        rr[0] += ri * ri;
      }
      block_sum<1>(rr, red);
      rnorm = sqrt(rr[0]);
      ++refs;
      if (!isfinite(rnorm)) { status = 2; break; }
    }
    if (status == 0 && rnorm > target) status = 3;  // EB_SIM_KRYLOV_STAGNATED
  }
  __syncthreads();
  if (stp && stage_fail) {
    status = 4;  // EB_SIM_WAIT_TIMEOUT: a bulk copy did not complete in time
    stage_drain(stp);
  }

  // ΔD[free] = x; Newton norms of compute_norms_corrector (utils_solver.jl:126-151)
  double q[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double f = (a.fext1[o + i] + a.Tc1[o + i]) + a.Tk1[o + i];
    if (fx[i]) {
      q[3] += f * f;
    } else {
      const double x = (bnorm > 0.0 && status != 2) ? X[i] : 0.0;
      a.dD[o + i] = x;
      q[0] += x * x;
      q[1] += b[i] * b[i];
      q[2] += f * f;
    }
  }
  block_sum<4>(q, red);
  if (threadIdx.x == 0) {
    a.norms[5 * s + 0] = q[0];
    a.norms[5 * s + 1] = q[1];
    a.norms[5 * s + 2] = q[2];
    a.norms[5 * s + 3] = q[3];
    a.norms[5 * s + 4] = status == 4 ? -1.0 : (double)its;  // iterations of this solve (-1: a wait ran out)
    a.its[s] += its;
    a.refs[s] += refs;
    const double rel = bnorm > 0.0 ? rnorm / bnorm : 0.0;
    a.relres[s] = fmax(a.relres[s], rel);
    if (status > a.status[s]) a.status[s] = status;
  }
}

// 6x6 block-Jacobi factors: inverse of each node's diagonal block of Ktan with
// fixed DOFs replaced by identity rows/columns (Gauss-Jordan, partial pivoting).
__global__ void k_block_jacobi(const Dev d, double* Dinv64, float* Dinv32) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  if (!d.active[d.node_sim[i]]) return;
  double A[36], B[36];
  const double* blk = d.Kt + (int64_t)d.diag_blk[i] * 36;
#pragma unroll
  for (int c = 0; c < 6; ++c)
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const bool fr = d.fixed[6 * i + r], fc = d.fixed[6 * i + c];
      A[6 * c + r] = (fr || fc) ? (r == c ? 1.0 : 0.0) : blk[6 * c + r];
      B[6 * c + r] = (r == c) ? 1.0 : 0.0;
    }
  for (int c = 0; c < 6; ++c) {
    int p = c;
    double best = fabs(A[6 * c + c]);
    for (int r = c + 1; r < 6; ++r)
      if (fabs(A[6 * c + r]) > best) { best = fabs(A[6 * c + r]); p = r; }
    if (p != c)
      for (int q = 0; q < 6; ++q) {
        double t = A[6 * q + c]; A[6 * q + c] = A[6 * q + p]; A[6 * q + p] = t;
        t = B[6 * q + c]; B[6 * q + c] = B[6 * q + p]; B[6 * q + p] = t;
      }
    const double piv = A[6 * c + c];
    const double ip = piv != 0.0 ? 1.0 / piv : 0.0;
    for (int q = 0; q < 6; ++q) { A[6 * q + c] *= ip; B[6 * q + c] *= ip; }
    for (int r = 0; r < 6; ++r) {
      if (r == c) continue;
      const double f = A[6 * c + r];
      if (f == 0.0) continue;
      for (int q = 0; q < 6; ++q) { A[6 * q + r] -= f * A[6 * q + c]; B[6 * q + r] -= f * B[6 * q + c]; }
    }
  }
  double* o64 = Dinv64 + i * 36;
  float* o32 = Dinv32 + i * 36;
#pragma unroll
  for (int k = 0; k < 36; ++k) { o64[k] = B[k]; o32[k] = (float)B[k]; }
}

void launch_block_jacobi(const Dev& d, double* Dinv64, float* Dinv32, cudaStream_t s) {
  if (d.n_nodes) k_block_jacobi<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, Dinv64, Dinv32);
}

size_t gmres_smem(int m) { return sizeof(double) * ((size_t)(m + 1) * m + 4 * (size_t)m + 1 + 8 * 32); }

size_t gmres_smem_total(const SolverArgs& a) {
  return gmres_smem(a.m) + (a.x_in_smem ? sizeof(float) * (size_t)a.max_n : 0) +
         (a.stage_floats > 0 ? 128 + sizeof(float) * 2 * (size_t)a.stage_floats +
                                   sizeof(float) * 2 * kPanel * kPanel
                             : 0);
}

cudaError_t launch_gmres(const SolverArgs& a, bool fp32, int threads, cudaStream_t s) {
  const size_t smem = gmres_smem_total(a);
  // shared memory is the occupancy limit: prefer the largest carveout so two CTAs fit when they can
  cudaFuncSetAttribute(k_gmres<float>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  cudaFuncSetAttribute(k_gmres<double>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (fp32) {
    cudaError_t e = raise_smem_limit((const void*)k_gmres<float>, smem);
    if (e != cudaSuccess) return e;
    k_gmres<float><<<a.n_sims, threads, smem, s>>>(a);
  } else {
    cudaError_t e = raise_smem_limit((const void*)k_gmres<double>, smem);
    if (e != cudaSuccess) return e;
    k_gmres<double><<<a.n_sims, threads, smem, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace eb
