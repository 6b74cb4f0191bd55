// C ABI of endobeams_gb300 (declared in include/endobeams_gb300.h): handle
// construction, the HHT step orchestration and the testing entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/endobeams_gb300.h"
#include "eb_gmres.cuh"
#include "eb_internal.cuh"
#include "eb_output.cuh"
#include "eb_warm.cuh"

using namespace eb;

namespace {

thread_local char g_err[1024] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(EB_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Device allocation list owned by a handle.
struct Arena {
  std::vector<void*> ptrs;
  size_t bytes = 0;
  ~Arena() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e == cudaSuccess) {
      ptrs.push_back(*p);
      bytes += n * sizeof(T);
      e = cudaMemset(*p, 0, n * sizeof(T));
    }
    return e;
  }
  template <typename T>
  cudaError_t upload(T** p, const std::vector<T>& h) {
    cudaError_t e = alloc(p, h.size());
    if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
  }
};

// ---------------------------------------------------------------- geometry helpers (host, FP64)

// get_Rₑ⁰ (src/beams/def_beam.jl:93-116), column-major output
void initial_frame(const double* X1, const double* X2, double* R) {
  const double eps = 2.220446049250313e-16;
  double d[3] = {X2[0] - X1[0], X2[1] - X1[1], X2[2] - X1[2]};
  double l0 = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  double e[3] = {d[0] / l0, d[1] / l0, d[2] / l0};
  double v[3] = {0.0, -e[2], e[1]};  // E1 × e
  double s = std::sqrt(v[1] * v[1] + v[2] * v[2]);
  double c = e[0];
  for (int k = 0; k < 9; ++k) R[k] = 0.0;
  if (c < -(1 - 2 * eps)) {
    R[0] = -1; R[4] = 1; R[8] = -1;
    return;
  }
  R[0] = 1; R[4] = 1; R[8] = 1;
  if (c > (1 - 2 * eps)) return;
  // I + S + (1-c)/s² S², S = skew(v)
  double S[9] = {0, v[2], -v[1], -v[2], 0, v[0], v[1], -v[0], 0};  // column-major skew
  double f = (1 - c) / (s * s);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      double s2 = 0;
      for (int q = 0; q < 3; ++q) s2 += S[i + 3 * q] * S[q + 3 * j];
      R[i + 3 * j] += S[i + 3 * j] + f * s2;
    }
}

// Quadratic B-spline prefilter with the even reflection at the cell edges
// (c[0] = c[1], c[n+1] = c[n]): solves ⅛c[i-1] + ¾c[i] + ⅛c[i+1] = y[i]
// along every grid line, axis by axis, into the padded coefficient grid.
void prefilter_axis(double* c, const int64_t dims[3], int axis, std::vector<double>& work) {
  const int64_t P[3] = {dims[0] + 2, dims[1] + 2, dims[2] + 2};
  const int64_t stride = axis == 0 ? 1 : (axis == 1 ? P[0] : P[0] * P[1]);
  const int64_t n = dims[axis];
  // the other two axes: interior for axes not yet filtered, full padded range for filtered ones
  int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
  auto lo = [&](int ax) { return ax < axis ? (int64_t)0 : (int64_t)1; };
  auto hi = [&](int ax) { return ax < axis ? P[ax] : dims[ax] + 1; };
  int64_t st[3] = {1, P[0], P[0] * P[1]};
  work.resize(2 * n);
  double* cp = work.data();
  double* dp = cp + n;
  for (int64_t b = lo(o2); b < hi(o2); ++b)
    for (int64_t a = lo(o1); a < hi(o1); ++a) {
      double* y = c + a * st[o1] + b * st[o2] + stride;  // first interior point
      if (n > 1) {
        // Thomas algorithm; diagonal 7/8 at both ends, 3/4 inside, off-diagonals 1/8
        double m = 0.875;
        cp[0] = 0.125 / m;
        dp[0] = y[0] / m;
        for (int64_t i = 1; i < n; ++i) {
          const double di = (i == n - 1) ? 0.875 : 0.75;
          m = di - 0.125 * cp[i - 1];
          cp[i] = (i == n - 1) ? 0.0 : 0.125 / m;
          dp[i] = (y[i * stride] - 0.125 * dp[i - 1]) / m;
        }
        y[(n - 1) * stride] = dp[n - 1];
        for (int64_t i = n - 2; i >= 0; --i) y[i * stride] = dp[i] - cp[i] * y[(i + 1) * stride];
      }
      y[-stride] = y[0];
      y[n * stride] = y[(n - 1) * stride];
    }
}

// Reverse Cuthill-McKee order of one simulation's node graph (neighbours in
// increasing degree, root a pseudo-peripheral node of each component).
// adj holds local neighbour lists (self excluded).  Returns the half
// bandwidth in nodes of the permuted graph; pos[i] is node i's position.
int rcm_order(const std::vector<std::vector<int>>& adj, std::vector<int>& pos) {
  const int n = (int)adj.size();
  std::vector<int> order;
  order.reserve(n);
  std::vector<char> seen(n, 0);
  std::vector<int> level(n, -1), queue;
  auto bfs = [&](int root, std::vector<int>& visited) {
    visited.clear();
    visited.push_back(root);
    level[root] = 0;
    int last = 0;
    for (size_t h = 0; h < visited.size(); ++h) {
      int v = visited[h];
      for (int w : adj[v])
        if (level[w] < 0) {
          level[w] = level[v] + 1;
          last = std::max(last, level[w]);
          visited.push_back(w);
        }
    }
    return last;
  };
  std::vector<int> comp;
  for (int start = 0; start < n; ++start) {
    if (seen[start]) continue;
    int root = start;
    // pseudo-peripheral root (George-Liu iteration)
    // (levels hold the BFS from `root` at the top of every iteration)
    int ecc = bfs(root, comp);
    for (int it = 0; it < 8; ++it) {
      int best = -1;
      for (int v : comp)
        if (level[v] == ecc && (best < 0 || adj[v].size() < adj[best].size())) best = v;
      for (int v : comp) level[v] = -1;
      int e2 = bfs(best, comp);
      if (e2 <= ecc) break;
      ecc = e2;
      root = best;
    }
    for (int v : comp) level[v] = -1;
    // Cuthill-McKee from root
    queue.clear();
    queue.push_back(root);
    seen[root] = 1;
    for (size_t h = 0; h < queue.size(); ++h) {
      int v = queue[h];
      order.push_back(v);
      std::vector<int> nb;
      for (int w : adj[v])
        if (!seen[w]) nb.push_back(w);
      std::sort(nb.begin(), nb.end(), [&](int x, int y) {
        return adj[x].size() != adj[y].size() ? adj[x].size() < adj[y].size() : x < y;
      });
      for (int w : nb) {
        seen[w] = 1;
        queue.push_back(w);
      }
    }
  }
  std::reverse(order.begin(), order.end());
  pos.assign(n, 0);
  for (int k = 0; k < n; ++k) pos[order[k]] = k;
  int bw = 0;
  for (int v = 0; v < n; ++v)
    for (int w : adj[v]) bw = std::max(bw, std::abs(pos[v] - pos[w]));
  return bw;
}

// The samples (sign flipped when `negate`) in the interior of the zero-padded
// coefficient layout; the device prefilter completes it.
std::vector<double> sdf_padded(const double* values, const int64_t dims[3], bool negate) {
  const int64_t px = dims[0] + 2, py = dims[1] + 2, pz = dims[2] + 2;
  std::vector<double> c((size_t)(px * py * pz), 0.0);
  for (int64_t k = 0; k < dims[2]; ++k)
    for (int64_t j = 0; j < dims[1]; ++j)
      for (int64_t i = 0; i < dims[0]; ++i) {
        double v = values[i + dims[0] * (j + dims[1] * k)];
        c[(size_t)((i + 1) + px * ((j + 1) + py * (k + 1)))] = negate ? -v : v;
      }
  return c;
}

std::vector<double> sdf_coefficients(const double* values, const int64_t dims[3], bool negate) {
  const int64_t px = dims[0] + 2, py = dims[1] + 2, pz = dims[2] + 2;
  std::vector<double> c((size_t)(px * py * pz), 0.0);
  for (int64_t k = 0; k < dims[2]; ++k)
    for (int64_t j = 0; j < dims[1]; ++j)
      for (int64_t i = 0; i < dims[0]; ++i) {
        double v = values[i + dims[0] * (j + dims[1] * k)];
        c[(size_t)((i + 1) + px * ((j + 1) + py * (k + 1)))] = negate ? -v : v;
      }
  std::vector<double> work;
  for (int ax = 0; ax < 3; ++ax) prefilter_axis(c.data(), dims, ax, work);
  return c;
}

}  // namespace

std::vector<double> eb_sdf_samples_padded_host(const double* values, const int64_t dims[3], bool negate) {
  return sdf_padded(values, dims, negate);
}

std::vector<double> eb_sdf_coefficients_host(const double* values, const int64_t dims[3], bool negate) {
  return sdf_coefficients(values, dims, negate);
}
int eb_internal_fail(int code, const char* msg) { return fail(code, "%s", msg); }

// ---------------------------------------------------------------- phase timing
// CUDA events recorded on the handle's stream at phase boundaries; elapsed
// times are resolved at the synchronisation points eb_step already has.
struct PhaseTimer {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  std::vector<int> phase_of;
  int used = 0;
  double ms[EB_NPHASES] = {0};
  int64_t launches[EB_NPHASES] = {0};
  void init(bool enable) {
    on = enable;
    if (!on) return;
    pool.resize(96);
    phase_of.assign(96, -1);
    for (auto& e : pool) cudaEventCreate(&e);
  }
  void destroy() {
    for (auto& e : pool) cudaEventDestroy(e);
    pool.clear();
  }
  void begin(cudaStream_t s) {
    if (!on) return;
    cudaEventRecord(pool[0], s);
    used = 1;
  }
  void mark(int phase, cudaStream_t s) {
    if (!on || used >= (int)pool.size()) return;
    cudaEventRecord(pool[used], s);
    phase_of[used] = phase;
    ++used;
  }
  // While `ref` (the handle's timer-start event) is set, every phase interval is also kept as
  // (phase, start, end) in ms from it, so that the intervals of handles stepped concurrently
  // can be merged on one time axis.
  cudaEvent_t ref = nullptr;
  std::vector<float> iv;
  void keep(int phase, cudaEvent_t a, cudaEvent_t b) {
    if (!ref || iv.size() >= 3u * (1u << 20)) return;
    float t0 = 0.f, t1 = 0.f;
    if (cudaEventElapsedTime(&t0, ref, a) == cudaSuccess && cudaEventElapsedTime(&t1, ref, b) == cudaSuccess) {
      iv.push_back((float)phase);
      iv.push_back(t0);
      iv.push_back(t1);
    }
  }
  void resolve() {  // call after the stream has been synchronised
    if (!on || used < 1) return;
    for (int i = 1; i < used; ++i) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, pool[i - 1], pool[i]) == cudaSuccess) ms[phase_of[i]] += t;
      keep(phase_of[i], pool[i - 1], pool[i]);
    }
    std::swap(pool[0], pool[used - 1]);
    used = 1;
  }
};

// ---------------------------------------------------------------- handle
// Learned warm start state of a handle (device buffers owned here).
struct WsHost {
  WsDev dev{};
  int* d_nb = nullptr;         // n_nodes x 2 neighbours
  int* d_surf_on = nullptr;    // per sim
  float *F = nullptr, *X = nullptr, *Y = nullptr;
  float *norm = nullptr;       // in_shift[48], in_scale[48], out_scale[6]
  float* P = nullptr;          // network parameters (FP32)
  __nv_bfloat16* W = nullptr;  // BF16 copy
  bool model = false;
  bool features_valid = false; // F holds this step's start (eb_step ran since the last commit/rollback)
  // capture ring
  float *sF = nullptr, *sT = nullptr;
  int64_t cap = 0, cursor = 0, written = 0, phase = 0;
  int stride = 1;
  double* d_rn = nullptr;      // 2 n_sims residual norms
  std::vector<double> rn;
  std::vector<int> used;
  std::vector<int> tried;      // this step: the simulation started from the network
  std::vector<int> streak;     // consecutive rejected learned starts
  std::vector<int> skip;       // steps left before the next learned attempt (back-off)
  ~WsHost() {
    cudaFree(F); cudaFree(X); cudaFree(Y); cudaFree(norm); cudaFree(P); cudaFree(W); cudaFree(sF); cudaFree(sT);
  }
};

// A captured corrector iteration (see record_iteration) and its own timer events.
struct IterGraph {
  cudaGraphExec_t exec = nullptr;
  uint64_t gen = 0;
  bool timer_ready = false;
  PhaseTimer timer;  // events recorded by the graph; launch counts per replay
};

struct eb_handle {
  // Releases the streams, events, graphs, pinned mirrors and output writer; the arena and
  // the warm-start buffers free their device memory in their own destructors.
  ~eb_handle() {
    if (vtk) {
      std::string err;
      vtk_close(vtk, err);
    }
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    timer.destroy();
    for (auto& G : graph) {
      if (G.exec) cudaGraphExecDestroy(G.exec);
      G.timer.destroy();
    }
    if (pin_active) cudaFreeHost(pin_active);
    if (pin_refactor) cudaFreeHost(pin_refactor);
    if (pin_norms) cudaFreeHost(pin_norms);
    if (side) cudaStreamDestroy(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
  }
  bool mid_step = false;  // eb_step ran and neither eb_commit nor eb_rollback followed yet
  PhaseTimer timer;
  WsHost ws;
  // pinned host mirrors used by the captured iterations, and the graphs
  int *pin_active = nullptr, *pin_refactor = nullptr;
  double* pin_norms = nullptr;
  IterGraph graph[2];      // without / with band refactorisation
  uint64_t graph_gen = 1;  // bumped when launch parameters captured in the graphs change
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  eb_params P;
  int n_sims = 0;
  cudaStream_t stream = nullptr;
  Arena arena;
  Dev d{};
  Gauss3 gauss{};
  std::vector<int64_t> node_off, elem_off, blk_off;
  std::vector<int> has_contact;
  bool any_contact = false;
  // loads / imposed
  std::vector<int64_t> load_off, fix_off;  // per-sim offsets into the flattened lists
  std::vector<int64_t> load_dof, fix_dof;  // global dofs
  int64_t* d_load_dof = nullptr;
  int64_t* d_fix_dof = nullptr;
  double* d_vals = nullptr;                // scratch for set_loads / set_imposed
  double* d_u3 = nullptr;                  // n_nodes x 3 scratch for eb_get_displacements (first use)
  // output pipeline
  double* d_E = nullptr;                   // per element
  VtkWriter* vtk = nullptr;
  // per-sim device arrays
  int* d_mask = nullptr;
  int* d_active = nullptr;
  double *d_cK = nullptr, *d_cC = nullptr, *d_cM = nullptr, *d_dt = nullptr;
  // solver
  SolverArgs sa{};
  std::vector<SolverArgs> gclass;  // empty, or {wide-band class, two-CTAs-per-SM class}
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  double *d_Dinv64 = nullptr;
  float* d_Dinv32 = nullptr;
  double* d_norms = nullptr;
  int *d_its = nullptr, *d_refs = nullptr, *d_status = nullptr;
  int* d_pred_its = nullptr;  // per sim: GMRES iterations of this step's predictor solve
  int* d_x0_on = nullptr;     // per sim: the next solve starts from the initial guess in dD
  double* d_relres = nullptr;
  std::vector<eb_sim_stats> stats;
  std::vector<double> h_norms;
  std::vector<int> max_it;  // per simulation Newton iteration cap (params.max_iterations unless set)
  std::vector<double> tol_res, tol_disp;  // per simulation Newton tolerances (params unless set)
  // band-LU preconditioner
  bool any_band = false, any_jacobi = false;
  int max_b = 0;
  bool tc_lu = false;  // band LU trailing updates on the tensor cores
  size_t band_floats = 0;
  BandDev band{};
  int* d_blk_row = nullptr;
  std::vector<int> band_b;  // per sim half bandwidth (0: block-Jacobi)
  // factorisation reuse
  int* d_refactor = nullptr;
  std::vector<int> need_refactor, refactor_mask;
  std::vector<double> dt_at_factor, cur_dt;
  std::vector<int> its0;        // GMRES iterations of the first corrector solve after the factorisation (-1: none yet)
  std::vector<double> excess;   // iterations spent beyond its0 since the factorisation
  std::vector<double> lu_cost;  // the band LU's cost in GMRES iterations (refactor_cost * b)
  std::vector<int> cur_active;
  int64_t factorizations = 0;
};

namespace {

__global__ void k_scatter(const int64_t* idx, const double* vals, int64_t n, double* dst) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[idx[t]] = vals[t];
}

// u (structure of arrays, component k at [k n + i]) -> n x 3 row-major.
__global__ void k_interleave3(const double* __restrict__ u, int64_t n, double* __restrict__ out) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 3 * n) out[t] = u[(t % 3) * n + t / 3];
}

int upload_mask(eb_handle* h, int* dst, const int32_t* mask) {
  std::vector<int> m(h->n_sims, 1);
  if (mask)
    for (int s = 0; s < h->n_sims; ++s) m[s] = mask[s] != 0;
  CK(cudaMemcpyAsync(dst, m.data(), sizeof(int) * h->n_sims, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return EB_OK;
}

// Linear solve of the simulations active on the device; `mask` (host, n_sims)
// marks the same simulations for the refactorisation decision.
// Host part of a linear solve: which simulations refactorise their band
// (factors missing, stale because Δt changed, or slow: too many GMRES
// iterations); fills refactor_mask.
bool plan_refactor(eb_handle* h, const int* mask) {
  bool any = false;
  if (!h->any_band) return false;
  double cmax = 0.0;  // largest LU cost among the simulations that refactorise
  for (int s = 0; s < h->n_sims; ++s) {
    int r = 0;
    if (mask[s] && h->band_b[s] > 0)
      r = h->need_refactor[s] || h->dt_at_factor[s] != h->cur_dt[s] || h->P.refactor_its <= 0;
    h->refactor_mask[s] = r;
    if (r) {
      cmax = std::max(cmax, h->lu_cost[s]);
      any = true;
    }
  }
  // One launch factorises every marked simulation; its duration is set by the costliest one,
  // so simulations half-way to their own limit and no costlier join at no extra wall time.
  if (any && h->P.refactor_policy == EB_REFACTOR_COST)
    for (int s = 0; s < h->n_sims; ++s)
      if (!h->refactor_mask[s] && mask[s] && h->band_b[s] > 0 && h->its0[s] >= 0 && h->lu_cost[s] <= cmax &&
          h->excess[s] >= 0.5 * h->lu_cost[s])
        h->refactor_mask[s] = 1;
  for (int s = 0; s < h->n_sims; ++s)
    if (h->refactor_mask[s]) {
      h->need_refactor[s] = 0;
      h->dt_at_factor[s] = h->cur_dt[s];
      h->its0[s] = -1;
      h->excess[s] = 0.0;
      ++h->factorizations;
    }
  return any;
}

// Stream part of a linear solve; `refactor_src` is the host copy of the refactor mask
// (pinned when the launches are captured into a graph).
// Solver arguments of one launch: corrector solves take the Eisenstat-Walker forcing term
// (when enabled); predictor solves a fixed tolerance (forcing_max under EW).
static SolverArgs solve_args(const eb_handle* h, const SolverArgs& base, bool corrector) {
  SolverArgs a = base;
  if (base.forcing && !corrector) {
    a.forcing = 0;
    a.tol = base.forcing_max;
  }
  return a;
}

int launch_solve(eb_handle* h, bool refactor, const int* refactor_src, PhaseTimer& T, bool corrector) {
  if (h->any_jacobi) {
    launch_block_jacobi(h->d, h->d_Dinv64, h->d_Dinv32, h->stream);
    T.launches[EB_PHASE_PRECOND] += 1;
  }
  if (refactor) {
    CK(cudaMemcpyAsync(h->d_refactor, refactor_src, sizeof(int) * h->n_sims, cudaMemcpyHostToDevice, h->stream));
    launch_band_fill(h->d, h->band, h->d_blk_row, h->stream);
    if (h->tc_lu) CK(launch_band_lu_tc(h->d, h->band, h->max_b, h->band.lu_fail, h->stream));
    else CK(launch_band_lu(h->d, h->band, h->max_b, h->stream));
    T.launches[EB_PHASE_PRECOND] += 3;
  }
  CK(cudaGetLastError());
  T.mark(EB_PHASE_PRECOND, h->stream);
  const bool fp32 = h->P.precision == EB_PREC_MIXED;
  int threads = h->P.threads_per_sim > 0 ? h->P.threads_per_sim : 256;
  if (h->gclass.size() == 2) {
    // wide-band simulations on the handle's stream, the two-per-SM class beside them
    CK(cudaEventRecord(h->ev_fork, h->stream));
    CK(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
    CK(launch_gmres(solve_args(h, h->gclass[0], corrector), fp32, threads, h->stream));
    CK(launch_gmres(solve_args(h, h->gclass[1], corrector), fp32, threads, h->side));
    CK(cudaEventRecord(h->ev_join, h->side));
    CK(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
  } else {
    CK(launch_gmres(solve_args(h, h->sa, corrector), fp32, threads, h->stream));
  }
  T.mark(EB_PHASE_KRYLOV, h->stream);
  T.launches[EB_PHASE_KRYLOV] += 1;
  return EB_OK;
}

int solve(eb_handle* h, const int* mask, bool corrector) {
  const bool any = plan_refactor(h, mask);
  return launch_solve(h, any, h->refactor_mask.data(), h->timer, corrector);
}

int record_iteration(eb_handle* h, bool refactor, PhaseTimer& T);

// After a bounded bulk-copy wait ran out: band blocks are read from global memory from now on.
// ... and, after a bounded wait of the tensor-core factorisation ran out, the FP32 factorisation
// is used from now on.
void disable_staging(eb_handle* h) {
  h->sa.stage_floats = 0;
  for (SolverArgs& c : h->gclass) c.stage_floats = 0;
  h->tc_lu = false;
}

// Launches the captured corrector iteration (capturing it on first use).
int run_iteration_graph(eb_handle* h, bool refactor) {
  IterGraph& G = h->graph[refactor ? 1 : 0];
  if (!G.exec || G.gen != h->graph_gen) {
    if (G.exec) {
      cudaGraphExecDestroy(G.exec);
      G.exec = nullptr;
    }
    if (!G.timer_ready) {
      G.timer.init(h->P.timing != 0);
      G.timer_ready = true;
    }
    G.timer.used = 0;
    for (int k = 0; k < EB_NPHASES; ++k) G.timer.launches[k] = 0;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed));
    const int rc = record_iteration(h, refactor, G.timer);
    const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CK(e);
    const cudaError_t ei = cudaGraphInstantiate(&G.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ei);
    G.gen = h->graph_gen;
  }
  CK(cudaGraphLaunch(G.exec, h->stream));
  for (int k = 0; k < EB_NPHASES; ++k) h->timer.launches[k] += G.timer.launches[k];
  return EB_OK;
}

// After a replay has completed: its phase times into the handle's totals.
void resolve_graph_times(eb_handle* h, bool refactor) {
  IterGraph& G = h->graph[refactor ? 1 : 0];
  if (!G.timer.on) return;
  for (int i = 1; i < G.timer.used; ++i) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, G.timer.pool[i - 1], G.timer.pool[i]) == cudaSuccess)
      h->timer.ms[G.timer.phase_of[i]] += t;
    h->timer.keep(G.timer.phase_of[i], G.timer.pool[i - 1], G.timer.pool[i]);
  }
}

// One corrector iteration after the first (assembly, residual, solve, Newmark
// and rotation updates, norms) as stream operations; eb_step replays it from
// a CUDA graph, one per refactorisation variant.  Its host inputs and outputs
// (mask of running simulations, refactor mask, Newton norms) are pinned.
int record_iteration(eb_handle* h, bool refactor, PhaseTimer& T) {
  const Dev& d = h->d;
  cudaStream_t st = h->stream;
  const double a = h->P.alpha, b = h->P.beta, g = h->P.gamma;
  const int S = h->n_sims;
  T.begin(st);
  CK(cudaMemcpyAsync(h->d_active, h->pin_active, sizeof(int) * S, cudaMemcpyHostToDevice, st));
  T.mark(EB_PHASE_UPDATE, st);
  launch_beam(d, h->gauss, st);
  T.mark(EB_PHASE_BEAM, st);
  T.launches[EB_PHASE_BEAM] += 1;
  if (h->any_contact) {
    launch_contact(d, h->gauss, st);
    T.mark(EB_PHASE_CONTACT, st);
    T.launches[EB_PHASE_CONTACT] += 1;
  }
  launch_gather(d, a, h->any_contact, st);
  T.mark(EB_PHASE_ASSEMBLY, st);
  T.launches[EB_PHASE_ASSEMBLY] += 2;
  launch_corrector_rhs(d, a, st);
  launch_apply_bc(d, st);
  T.mark(EB_PHASE_RESIDUAL, st);
  T.launches[EB_PHASE_RESIDUAL] += 3;
  int rc = launch_solve(h, refactor, h->pin_refactor, T, true);
  if (rc) return rc;
  launch_global_corrector(d, st);
  launch_local_corrector(d, b, g, st);
  T.launches[EB_PHASE_UPDATE] += 2;
  CK(cudaMemcpyAsync(h->pin_norms, h->d_norms, sizeof(double) * 5 * S, cudaMemcpyDeviceToHost, st));
  T.mark(EB_PHASE_UPDATE, st);
  return EB_OK;
}

}  // namespace

extern "C" {

const char* eb_last_error(void) { return g_err; }

int eb_default_params(eb_params* p) {
  if (!p) return fail(EB_ERR_ARG, "eb_default_params: null");
  std::memset(p, 0, sizeof(*p));
  p->alpha = -0.05;
  p->beta = 0.25 * (1 - p->alpha) * (1 - p->alpha);
  p->gamma = 0.5 * (1 - 2 * p->alpha);
  p->tolerance_residual = 1e-5;
  p->tolerance_displacement = 1e-5;
  p->max_iterations = 20;
  p->gauss_w[0] = 5.0 / 9.0; p->gauss_w[1] = 8.0 / 9.0; p->gauss_w[2] = 5.0 / 9.0;
  p->gauss_z[0] = -std::sqrt(3.0 / 5.0); p->gauss_z[1] = 0.0; p->gauss_z[2] = std::sqrt(3.0 / 5.0);
  p->precision = EB_PREC_FP64;
  p->krylov_restart = 64;
  p->krylov_max_iter = 4000;
  p->linear_tol = 1e-10;
  p->inner_tol = 1e-4;
  p->max_refinements = 60;
  p->threads_per_sim = 0;
  p->timing = 0;
  p->preconditioner = EB_PRECOND_BAND;
  p->refactor_its = 16;
  p->stage_band = 1;
  p->warm_start = EB_WS_OFF;
  p->use_graph = 1;
  p->forcing = EB_FORCING_FIXED;
  p->forcing_max = 1e-2;
  p->refactor_policy = EB_REFACTOR_THRESHOLD;
  p->refactor_cost = 0.2;
  p->band_lu = EB_LU_FP32;
  return EB_OK;
}

int eb_rcm_order(int64_t n, const int64_t* xadj, const int32_t* adjncy, int32_t* pos, int32_t* half_bandwidth) {
  if (n < 0 || (n > 0 && (!xadj || !adjncy || !pos))) return fail(EB_ERR_ARG, "eb_rcm_order: bad arguments");
  if (n >= (int64_t)INT32_MAX) return fail(EB_ERR_ARG, "eb_rcm_order: graph too large");
  std::vector<std::vector<int>> adj((size_t)n);
  for (int64_t v = 0; v < n; ++v)
    for (int64_t k = xadj[v]; k < xadj[v + 1]; ++k) {
      const int32_t w = adjncy[k];
      if (w < 0 || w >= n) return fail(EB_ERR_ARG, "eb_rcm_order: neighbour out of range");
      if (w != v) adj[(size_t)v].push_back(w);
    }
  std::vector<int> p;
  const int bw = rcm_order(adj, p);
  for (int64_t v = 0; v < n; ++v) pos[v] = p[(size_t)v];
  if (half_bandwidth) *half_bandwidth = bw;
  return EB_OK;
}

int eb_device_memory(int64_t* free_bytes, int64_t* total_bytes) {
  size_t fr = 0, tot = 0;
  cudaError_t e = cudaMemGetInfo(&fr, &tot);
  if (e != cudaSuccess) return fail(EB_ERR_CUDA, "cudaMemGetInfo: %s", cudaGetErrorString(e));
  if (free_bytes) *free_bytes = (int64_t)fr;
  if (total_bytes) *total_bytes = (int64_t)tot;
  return EB_OK;
}

int eb_device_info(int32_t* count, char* name, int32_t name_len) {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (count) *count = (e == cudaSuccess) ? c : 0;
  if (e != cudaSuccess) return fail(EB_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
  if (name && name_len > 0) {
    cudaDeviceProp pr;
    if (c > 0 && cudaGetDeviceProperties(&pr, 0) == cudaSuccess) {
      std::snprintf(name, name_len, "%s (sm_%d%d, %d SMs)", pr.name, pr.major, pr.minor, pr.multiProcessorCount);
    } else {
      name[0] = 0;
    }
  }
  return EB_OK;
}

int eb_create(const eb_params* p, int32_t n_sims, const eb_sim_desc* sims, eb_handle** out) {
  if (!p || !sims || !out || n_sims <= 0) return fail(EB_ERR_ARG, "eb_create: bad arguments");
  *out = nullptr;
  if (p->krylov_restart < 1 || p->krylov_restart > 128) return fail(EB_ERR_ARG, "krylov_restart must be in [1,128]");
  std::unique_ptr<eb_handle> h(new eb_handle());
  h->P = *p;
  h->n_sims = n_sims;
  for (int i = 0; i < 3; ++i) { h->gauss.w[i] = p->gauss_w[i]; h->gauss.z[i] = p->gauss_z[i]; }
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&h->t0));
  CK(cudaEventCreate(&h->t1));
  h->timer.init(p->timing != 0);
  CK(cudaMallocHost(&h->pin_active, sizeof(int) * (size_t)n_sims));
  CK(cudaMallocHost(&h->pin_refactor, sizeof(int) * (size_t)n_sims));
  CK(cudaMallocHost(&h->pin_norms, sizeof(double) * 5 * (size_t)n_sims));

  // ---- sizes and offsets
  h->node_off.assign(n_sims + 1, 0);
  h->elem_off.assign(n_sims + 1, 0);
  for (int s = 0; s < n_sims; ++s) {
    const eb_sim_desc& S = sims[s];
    if (S.n_nodes <= 0 || S.n_elem <= 0 || !S.X0 || !S.conn || !S.E || !S.nu || !S.rho || !S.radius || !S.damping)
      return fail(EB_ERR_ARG, "sim %d: missing nodes, connectivity or material arrays", s);
    for (int64_t e = 0; e < S.n_elem; ++e) {
      int64_t a = S.conn[2 * e], b = S.conn[2 * e + 1];
      if (a < 0 || b < 0 || a >= S.n_nodes || b >= S.n_nodes || a == b)
        return fail(EB_ERR_ARG, "sim %d: element %lld has invalid nodes (%lld, %lld)", s, (long long)e, (long long)a,
                    (long long)b);
    }
    for (int64_t k = 0; k < S.n_fixed; ++k)
      if (S.fixed_dofs[k] < 0 || S.fixed_dofs[k] >= 6 * S.n_nodes) return fail(EB_ERR_ARG, "sim %d: fixed dof out of range", s);
    for (int64_t k = 0; k < S.n_loaded; ++k)
      if (S.loaded_dofs[k] < 0 || S.loaded_dofs[k] >= 6 * S.n_nodes) return fail(EB_ERR_ARG, "sim %d: loaded dof out of range", s);
    if (S.surface < EB_SURFACE_NONE || S.surface > EB_SURFACE_PLANE)
      return fail(EB_ERR_ARG, "sim %d: unknown surface kind %d", s, (int)S.surface);
    if (S.surface == EB_SURFACE_PLANE && (S.plane_axis < 0 || S.plane_axis > 2))
      return fail(EB_ERR_ARG, "sim %d: plane_axis must be 0, 1 or 2", s);
    if (S.surface == EB_SURFACE_SDF) {
      if (!S.sdf_values || S.sdf_dims[0] < 1 || S.sdf_dims[1] < 1 || S.sdf_dims[2] < 1)
        return fail(EB_ERR_ARG, "sim %d: SDF grid missing", s);
      if (S.sdf_spacing[0] <= 0 || S.sdf_spacing[1] <= 0 || S.sdf_spacing[2] <= 0)
        return fail(EB_ERR_ARG, "sim %d: SDF spacing must be positive", s);
      if (S.sdf_interp != EB_SDF_QUADRATIC && S.sdf_interp != EB_SDF_TRILINEAR)
        return fail(EB_ERR_ARG, "sim %d: unknown SDF interpolation %d", s, (int)S.sdf_interp);
      if (S.sdf_interp == EB_SDF_TRILINEAR && (S.sdf_dims[0] < 2 || S.sdf_dims[1] < 2 || S.sdf_dims[2] < 2))
        return fail(EB_ERR_ARG, "sim %d: a trilinear SDF needs at least 2 points per axis", s);
    }
    h->node_off[s + 1] = h->node_off[s] + S.n_nodes;
    h->elem_off[s + 1] = h->elem_off[s] + S.n_elem;
  }
  const int64_t NN = h->node_off[n_sims], NE = h->elem_off[n_sims], ND = 6 * NN;
  if (NN >= (1LL << 31) / 6 || NE >= (1LL << 29)) return fail(EB_ERR_ARG, "problem too large for 32-bit indices");

  // ---- host staging of node and element data
  std::vector<double> X0(3 * NN), u(3 * NN), ud(3 * NN), udd(3 * NN), w(3 * NN), wd(3 * NN), wdd(3 * NN);
  std::vector<double> R(9 * NN), dR(9 * NN, 0.0);
  std::vector<int> node_sim(NN);
  std::vector<int> ea(NE), ebv(NE), elem_sim(NE);
  std::vector<double> l0(NE), Re0(9 * NE), Kbar(7 * NE), Jr(3 * NE), Ar(NE), damp(NE), radius(NE), Ev(NE);
  std::vector<uint8_t> is_contact(NE, 0);
  std::vector<uint8_t> fixed(ND, 0);
  std::vector<double> fext(ND, 0.0);
  h->has_contact.assign(n_sims, 0);
  std::vector<int> has_fixed(n_sims, 0);
  std::vector<SurfaceDev> surf(n_sims);
  std::vector<ContactProps> props(n_sims);
  std::vector<int> sdf_sims;  // simulations with a voxel SDF (coefficients computed below)
  h->load_off.assign(n_sims + 1, 0);
  h->fix_off.assign(n_sims + 1, 0);

  for (int s = 0; s < n_sims; ++s) {
    const eb_sim_desc& S = sims[s];
    const int64_t no = h->node_off[s], eo = h->elem_off[s];
    auto put3 = [&](std::vector<double>& dst, const double* src) {
      for (int64_t i = 0; i < S.n_nodes; ++i)
        for (int k = 0; k < 3; ++k) dst[k * NN + no + i] = src ? src[3 * i + k] : 0.0;
    };
    put3(X0, S.X0); put3(u, S.u); put3(ud, S.ud); put3(udd, S.udd); put3(w, S.w); put3(wd, S.wd); put3(wdd, S.wdd);
    for (int64_t i = 0; i < S.n_nodes; ++i) {
      node_sim[no + i] = s;
      for (int k = 0; k < 9; ++k) {
        R[k * NN + no + i] = S.R ? S.R[9 * i + k] : ((k % 4 == 0) ? 1.0 : 0.0);
        dR[k * NN + no + i] = (k % 4 == 0) ? 1.0 : 0.0;
      }
    }
    for (int64_t e = 0; e < S.n_elem; ++e) {
      const int64_t ge = eo + e;
      const int64_t a = S.conn[2 * e], b = S.conn[2 * e + 1];
      ea[ge] = (int)(no + a);
      ebv[ge] = (int)(no + b);
      elem_sim[ge] = s;
      const double* Xa = S.X0 + 3 * a;
      const double* Xb = S.X0 + 3 * b;
      const double dx = Xa[0] - Xb[0], dy = Xa[1] - Xb[1], dz = Xa[2] - Xb[2];
      const double L = std::sqrt(dx * dx + dy * dy + dz * dz);  // def_beam.jl:136
      l0[ge] = L;
      double Rm[9];
      if (S.Re0) std::memcpy(Rm, S.Re0 + 9 * e, sizeof(Rm));
      else initial_frame(Xa, Xb, Rm);
      for (int k = 0; k < 9; ++k) Re0[k * NE + ge] = Rm[k];
      // BeamMaterialProperties / K̄ⁱⁿᵗ_beam (def_beam.jl:74-85, 135-149)
      const double E = S.E[e], nu = S.nu[e], rho = S.rho[e], r = S.radius[e];
      const double G = E / (2 * (1 + nu));
      const double A = M_PI * r * r;
      const double I22 = M_PI * std::pow(r, 4) / 4, I33 = I22, Io = I22 + I33;
      const double kb[7] = {A * E / L,     G * Io / L,        4 * E * I33 / L, 4 * E * I22 / L,
                            -G * Io / L,   2 * E * I33 / L,   2 * E * I22 / L};
      for (int k = 0; k < 7; ++k) Kbar[k * NE + ge] = kb[k];
      Jr[ge] = rho * Io; Jr[NE + ge] = rho * I22; Jr[2 * NE + ge] = rho * I33;
      Ar[ge] = rho * A;
      damp[ge] = S.damping[e];
      radius[ge] = r;
      Ev[ge] = E;
    }
    // contact
    if (S.surface != EB_SURFACE_NONE) {
      h->has_contact[s] = 1;
      h->any_contact = true;
      if (S.contact_elems && S.n_contact_elems > 0) {
        for (int64_t c = 0; c < S.n_contact_elems; ++c) {
          int64_t e = S.contact_elems[c];
          if (e < 0 || e >= S.n_elem) return fail(EB_ERR_ARG, "sim %d: contact element out of range", s);
          is_contact[eo + e] = 1;
        }
      } else {
        for (int64_t e = 0; e < S.n_elem; ++e) is_contact[eo + e] = 1;
      }
      props[s] = ContactProps{S.kn, S.mu, S.eps_t, S.eta_n};
      SurfaceDev& sf = surf[s];
      std::memset(&sf, 0, sizeof(sf));
      if (S.surface == EB_SURFACE_SPHERE) {
        sf.kind = 0;
        sf.cx = S.sphere_center[0]; sf.cy = S.sphere_center[1]; sf.cz = S.sphere_center[2];
        sf.R = S.sphere_radius;
      } else if (S.surface == EB_SURFACE_PLANE) {
        sf.kind = 2;
        sf.axis = S.plane_axis;
        sf.pos = S.plane_position;
      } else if (S.surface == EB_SURFACE_SDF) {
        sf.kind = 1;
        sf.interp = S.sdf_interp;
        sf.nx = (int)S.sdf_dims[0]; sf.ny = (int)S.sdf_dims[1]; sf.nz = (int)S.sdf_dims[2];
        sf.x0 = S.sdf_origin[0]; sf.y0 = S.sdf_origin[1]; sf.z0 = S.sdf_origin[2];
        sf.ihx = 1.0 / S.sdf_spacing[0]; sf.ihy = 1.0 / S.sdf_spacing[1]; sf.ihz = 1.0 / S.sdf_spacing[2];
        sf.xl = (double)(sf.nx - 1) * S.sdf_spacing[0];
        sf.yl = (double)(sf.ny - 1) * S.sdf_spacing[1];
        sf.zl = (double)(sf.nz - 1) * S.sdf_spacing[2];
        sdf_sims.push_back(s);
      }
    }
    // BCs and loads
    for (int64_t k = 0; k < S.n_fixed; ++k) {
      fixed[6 * no + S.fixed_dofs[k]] = 1;
      h->fix_dof.push_back(6 * no + S.fixed_dofs[k]);
    }
    has_fixed[s] = S.n_fixed > 0;
    for (int64_t k = 0; k < S.n_loaded; ++k) {
      h->load_dof.push_back(6 * no + S.loaded_dofs[k]);
      fext[6 * no + S.loaded_dofs[k]] = S.fext0 ? S.fext0[k] : 0.0;  // Forces(conf), def_structures.jl:10-31
    }
    h->fix_off[s + 1] = h->fix_off[s] + S.n_fixed;
    h->load_off[s + 1] = h->load_off[s] + S.n_loaded;
  }

  // ---- block pattern: union of the elements' node pairs (sparse_matrices.jl:6-77, in 6x6 blocks)
  std::vector<std::vector<int>> adj(NN);
  for (int64_t i = 0; i < NN; ++i) adj[i].push_back((int)i);
  for (int64_t e = 0; e < NE; ++e) {
    adj[ea[e]].push_back(ebv[e]);
    adj[ebv[e]].push_back(ea[e]);
  }
  std::vector<int> row_ptr(NN + 1, 0), col, diag_blk(NN), blk_sim;
  for (int64_t i = 0; i < NN; ++i) {
    auto& v = adj[i];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    row_ptr[i + 1] = row_ptr[i] + (int)v.size();
    for (int c : v) {
      if (c == (int)i) diag_blk[i] = (int)col.size();
      col.push_back(c);
      blk_sim.push_back(node_sim[i]);
    }
  }
  const int64_t NB = (int64_t)col.size();
  auto blk_of = [&](int r, int c) {
    auto b = std::lower_bound(col.begin() + row_ptr[r], col.begin() + row_ptr[r + 1], c);
    return (int)(b - col.begin());
  };
  // ordered contribution lists (element order) per block and per node
  std::vector<int> bcnt(NB + 1, 0), ncnt(NN + 1, 0);
  for (int64_t e = 0; e < NE; ++e) {
    const int nd[2] = {ea[e], ebv[e]};
    for (int J = 0; J < 2; ++J)
      for (int I = 0; I < 2; ++I) bcnt[blk_of(nd[I], nd[J]) + 1]++;
    ncnt[nd[0] + 1]++;
    ncnt[nd[1] + 1]++;
  }
  for (int64_t b = 0; b < NB; ++b) bcnt[b + 1] += bcnt[b];
  for (int64_t i = 0; i < NN; ++i) ncnt[i + 1] += ncnt[i];
  std::vector<int> blk_contrib(bcnt[NB]), node_contrib(ncnt[NN]);
  {
    std::vector<int> bf(bcnt.begin(), bcnt.end() - 1), nf(ncnt.begin(), ncnt.end() - 1);
    for (int64_t e = 0; e < NE; ++e) {
      const int nd[2] = {ea[e], ebv[e]};
      for (int J = 0; J < 2; ++J)
        for (int I = 0; I < 2; ++I) blk_contrib[bf[blk_of(nd[I], nd[J])]++] = (int)(4 * e + I + 2 * J);
      node_contrib[nf[nd[0]]++] = (int)(2 * e);
      node_contrib[nf[nd[1]]++] = (int)(2 * e + 1);
    }
  }
  h->blk_off.assign(n_sims + 1, 0);
  for (int s = 0; s < n_sims; ++s) h->blk_off[s + 1] = row_ptr[h->node_off[s + 1]];
  std::vector<int> blk_row(NB);
  for (int64_t i = 0; i < NN; ++i)
    for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) blk_row[k] = (int)i;

  // ---- band-LU preconditioner plan: reverse Cuthill-McKee order per simulation
  std::vector<int> pos_all(NN), node_at(NN);
  std::vector<int64_t> band_off(n_sims + 1, 0);
  h->band_b.assign(n_sims, 0);
  const int bmax = (((227 * 1024) / 4 - 8) / kPanel - kPanel) / 2;  // shared-memory limit of k_band_lu
  for (int s = 0; s < n_sims; ++s) {
    const int64_t no = h->node_off[s], n = h->node_off[s + 1] - no;
    std::vector<std::vector<int>> la(n);
    for (int64_t i = 0; i < n; ++i)
      for (int g : adj[no + i])
        if (g != (int)(no + i)) la[i].push_back((int)(g - no));
    std::vector<int> pos;
    const int w = rcm_order(la, pos);
    int b = 6 * w + 5;
    if (p->preconditioner == EB_PRECOND_BLOCK_JACOBI || b > bmax) b = 0;
    h->band_b[s] = b;
    for (int64_t i = 0; i < n; ++i) {
      pos_all[no + i] = pos[i];
      node_at[no + pos[i]] = (int)(no + i);
    }
    band_off[s + 1] = band_off[s] + (b ? band_floats(6 * n, b) : 0);
  }

  // ---- device arenas
  Arena& A = h->arena;
  Dev& d = h->d;
  d.n_sims = n_sims;
  d.n_nodes = NN;
  d.n_elem = NE;
  d.nnzb = NB;
  d.n_dof = ND;
  d.beam_threads = kThreads;
  d.contact_threads = kThreads;
  d.gmat_threads = 256;
  d.gvec_threads = 256;
  int64_t *p_node_off, *p_blk_off;
  CK(A.upload(&p_node_off, h->node_off));
  CK(A.upload(&p_blk_off, h->blk_off));
  d.sim_node_off = p_node_off;
  d.sim_blk_off = p_blk_off;
  CK(A.alloc(&h->d_active, n_sims));
  CK(A.alloc(&h->d_mask, n_sims));
  CK(A.alloc(&h->d_cK, n_sims));
  CK(A.alloc(&h->d_cC, n_sims));
  CK(A.alloc(&h->d_cM, n_sims));
  CK(A.alloc(&h->d_dt, n_sims));
  d.active = h->d_active; d.cK = h->d_cK; d.cC = h->d_cC; d.cM = h->d_cM; d.dt = h->d_dt;
  // SDF coefficient grids: simulations that pass the same grid (same values pointer,
  // dims, spacing, origin and inside flag) share one device copy; distinct grids are
  // prefiltered on host threads in chunks and uploaded as each chunk completes.
  {
    std::vector<int> owner(n_sims, -1), todo;
    for (int s : sdf_sims) {
      const eb_sim_desc& S = sims[s];
      for (int t : todo) {
        const eb_sim_desc& T = sims[t];
        if (T.sdf_values == S.sdf_values && T.sdf_inside == S.sdf_inside && T.sdf_interp == S.sdf_interp &&
            std::memcmp(T.sdf_dims, S.sdf_dims, sizeof S.sdf_dims) == 0 &&
            std::memcmp(T.sdf_origin, S.sdf_origin, sizeof S.sdf_origin) == 0 &&
            std::memcmp(T.sdf_spacing, S.sdf_spacing, sizeof S.sdf_spacing) == 0) {
          owner[s] = t;
          break;
        }
      }
      if (owner[s] < 0) {
        owner[s] = s;
        todo.push_back(s);
      }
    }
    const int nthr = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
    std::vector<std::vector<double>> chunk(nthr);
    for (size_t c0 = 0; c0 < todo.size(); c0 += nthr) {
      const size_t c1 = std::min(todo.size(), c0 + nthr);
      std::vector<std::thread> pool;
      for (size_t i = c0; i < c1; ++i)
        pool.emplace_back([&, i] {
          const eb_sim_desc& S = sims[todo[i]];
          chunk[i - c0] = sdf_padded(S.sdf_values, S.sdf_dims, S.sdf_inside == 0);
        });
      for (auto& th : pool) th.join();
      for (size_t i = c0; i < c1; ++i) {
        const eb_sim_desc& S = sims[todo[i]];
        double* c;
        CK(A.upload(&c, chunk[i - c0]));
        // the trilinear interpolant uses the samples themselves
        if (S.sdf_interp == EB_SDF_QUADRATIC)
          launch_sdf_prefilter(c, (int)S.sdf_dims[0], (int)S.sdf_dims[1], (int)S.sdf_dims[2], h->stream);
        CK(cudaGetLastError());
        surf[todo[i]].coef = c;
        std::vector<double>().swap(chunk[i - c0]);
      }
      CK(cudaStreamSynchronize(h->stream));
    }
    for (int s : sdf_sims) surf[s].coef = surf[owner[s]].coef;
  }
  SurfaceDev* p_surf;
  ContactProps* p_props;
  int* p_hf;
  CK(A.upload(&p_surf, surf));
  CK(A.upload(&p_props, props));
  CK(A.upload(&p_hf, has_fixed));
  d.surf = p_surf; d.props = p_props; d.has_fixed = p_hf;
  int* p_ns;
  CK(A.upload(&p_ns, node_sim));
  d.node_sim = p_ns;
  double* pX0;
  CK(A.upload(&pX0, X0));
  d.X0 = pX0;
  CK(A.upload(&d.u, u)); CK(A.upload(&d.ud, ud)); CK(A.upload(&d.udd, udd));
  CK(A.upload(&d.w, w)); CK(A.upload(&d.wd, wd)); CK(A.upload(&d.wdd, wdd));
  CK(A.upload(&d.R, R)); CK(A.upload(&d.dR, dR));
  CK(A.upload(&d.un, u)); CK(A.upload(&d.udn, ud)); CK(A.upload(&d.uddn, udd));
  CK(A.upload(&d.wn, w)); CK(A.upload(&d.wdn, wd)); CK(A.upload(&d.wddn, wdd));
  CK(A.upload(&d.Rn, R)); CK(A.upload(&d.dRn, dR));
  int *p_ea, *p_eb, *p_es;
  CK(A.upload(&p_ea, ea)); CK(A.upload(&p_eb, ebv)); CK(A.upload(&p_es, elem_sim));
  d.ea = p_ea; d.eb = p_eb; d.elem_sim = p_es;
  double *p_l0, *p_Re0, *p_Kb, *p_Jr, *p_Ar, *p_dm, *p_rd;
  CK(A.upload(&p_l0, l0)); CK(A.upload(&p_Re0, Re0)); CK(A.upload(&p_Kb, Kbar)); CK(A.upload(&p_Jr, Jr));
  CK(A.upload(&p_Ar, Ar)); CK(A.upload(&p_dm, damp)); CK(A.upload(&p_rd, radius));
  d.l0 = p_l0; d.Re0 = p_Re0; d.Kbar = p_Kb; d.Jr = p_Jr; d.Ar = p_Ar; d.damp = p_dm; d.radius = p_rd;
  CK(A.upload(&h->d_E, Ev));  // Young's modulus per element, for the stress output
  uint8_t* p_ic;
  CK(A.upload(&p_ic, is_contact));
  d.is_contact = p_ic;
  CK(A.alloc(&d.stK, NE * 144)); CK(A.alloc(&d.stC, NE * 144)); CK(A.alloc(&d.stM, NE * 144));
  CK(A.alloc(&d.stTi, NE * 12)); CK(A.alloc(&d.stTk, NE * 12)); CK(A.alloc(&d.stE, NE * 2));
  if (h->any_contact) {
    CK(A.alloc(&d.scK, NE * 144)); CK(A.alloc(&d.scC, NE * 144)); CK(A.alloc(&d.scT, NE * 12));
    CK(A.alloc(&d.scE, NE));
  }
  CK(A.alloc(&d.sc_on, NE));
  int *p_rp, *p_col, *p_db, *p_bs, *p_bc, *p_bcl, *p_nc, *p_ncl;
  CK(A.upload(&p_rp, row_ptr)); CK(A.upload(&p_col, col)); CK(A.upload(&p_db, diag_blk)); CK(A.upload(&p_bs, blk_sim));
  CK(A.upload(&p_bc, bcnt)); CK(A.upload(&p_bcl, blk_contrib)); CK(A.upload(&p_nc, ncnt)); CK(A.upload(&p_ncl, node_contrib));
  d.row_ptr = p_rp; d.col = p_col; d.diag_blk = p_db; d.blk_sim = p_bs; d.blk_cptr = p_bc; d.blk_contrib = p_bcl;
  d.node_cptr = p_nc; d.node_contrib = p_ncl;
  CK(A.alloc(&d.K1, NB * 36)); CK(A.alloc(&d.C1, NB * 36)); CK(A.alloc(&d.M1, NB * 36));
  CK(A.alloc(&d.Kn, NB * 36)); CK(A.alloc(&d.Cn, NB * 36)); CK(A.alloc(&d.Mn, NB * 36));
  CK(A.alloc(&d.Kt, NB * 36)); CK(A.alloc(&d.Kt32, NB * 36));
  CK(A.alloc(&d.D, ND)); CK(A.alloc(&d.Dd, ND)); CK(A.alloc(&d.Ddd, ND)); CK(A.alloc(&d.dD, ND)); CK(A.alloc(&d.r, ND));
  CK(A.upload(&d.fext1, fext)); CK(A.upload(&d.fextn, fext));
  CK(A.alloc(&d.Ti1, ND)); CK(A.alloc(&d.Tin, ND)); CK(A.alloc(&d.Tk1, ND)); CK(A.alloc(&d.Tkn, ND));
  CK(A.alloc(&d.Tc1, ND)); CK(A.alloc(&d.Tcn, ND));
  CK(A.upload(&d.fixed, fixed));
  CK(A.alloc(&d.imposed, ND));
  CK(A.upload(&h->d_load_dof, h->load_dof));
  CK(A.upload(&h->d_fix_dof, h->fix_dof));
  CK(A.alloc(&h->d_vals, std::max<size_t>(h->load_dof.size(), h->fix_dof.size()) + 1));

  // ---- solver work
  const int m = p->krylov_restart;
  const bool fp32 = p->precision == EB_PREC_MIXED;
  CK(A.alloc(&h->d_Dinv64, NN * 36));
  CK(A.alloc(&h->d_Dinv32, NN * 36));
  CK(A.alloc(&h->d_norms, 5 * (size_t)n_sims));
  CK(A.alloc(&h->d_its, n_sims)); CK(A.alloc(&h->d_refs, n_sims)); CK(A.alloc(&h->d_status, n_sims));
  CK(A.alloc(&h->d_relres, n_sims));
  SolverArgs& sa = h->sa;
  sa.n_sims = n_sims;
  sa.sim_node_off = d.sim_node_off;
  sa.active = d.active;
  sa.row_ptr = d.row_ptr;
  sa.col = d.col;
  sa.Kt = d.Kt;
  sa.Kt32 = d.Kt32;
  sa.Dinv64 = h->d_Dinv64;
  sa.Dinv32 = h->d_Dinv32;
  sa.fixed = d.fixed;
  sa.b = d.r;
  sa.dD = d.dD;
  sa.fext1 = d.fext1;
  sa.Tc1 = d.Tc1;
  sa.Tk1 = d.Tk1;
  CK(A.alloc(&sa.X, ND));
  CK(A.alloc(&sa.R64, ND));
  // Krylov basis V (m + 1 vectors) and the preconditioned basis Z (m vectors) of every simulation
  if (fp32) {
    float *V, *Z;
    CK(A.alloc(&V, (size_t)(m + 1) * ND)); CK(A.alloc(&Z, (size_t)m * ND));
    sa.V = V; sa.Z = Z;
  } else {
    double *V, *Z;
    CK(A.alloc(&V, (size_t)(m + 1) * ND)); CK(A.alloc(&Z, (size_t)m * ND));
    sa.V = V; sa.Z = Z;
  }
  sa.m = m;
  sa.max_iter = p->krylov_max_iter;
  sa.max_ref = p->max_refinements;
  sa.tol = p->linear_tol;
  sa.inner_tol = fp32 ? p->inner_tol : p->linear_tol;
  sa.norms = h->d_norms;
  sa.its = h->d_its;
  sa.refs = h->d_refs;
  sa.relres = h->d_relres;
  sa.status = h->d_status;
  if (p->forcing != EB_FORCING_FIXED && p->forcing != EB_FORCING_EW) return fail(EB_ERR_ARG, "eb_create: bad forcing mode");
  if (p->forcing == EB_FORCING_EW && !(p->forcing_max > 0 && p->forcing_max < 1))
    return fail(EB_ERR_ARG, "eb_create: forcing_max must lie in (0, 1)");
  sa.forcing = p->forcing == EB_FORCING_EW ? 1 : 0;
  sa.forcing_max = p->forcing_max;
  CK(A.alloc(&sa.prev_bnorm, n_sims));
  CK(A.alloc(&sa.prev_eta, n_sims));
  CK(A.alloc(&h->d_pred_its, n_sims));
  CK(A.alloc(&h->d_x0_on, n_sims));
  CK(cudaMemset(h->d_x0_on, 0, sizeof(int) * n_sims));
  sa.x0_on = h->d_x0_on;
  h->stats.assign(n_sims, eb_sim_stats{});
  h->h_norms.assign(5 * (size_t)n_sims, 0.0);
  h->max_it.assign(n_sims, p->max_iterations);
  h->tol_res.assign(n_sims, p->tolerance_residual);
  h->tol_disp.assign(n_sims, p->tolerance_displacement);

  // ---- band storage (falls back to block-Jacobi when it would not fit in half the free memory)
  {
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    // the band, its diagonal-block inverses and the work vector must leave 2 GB free
    const size_t inv_bytes = 2 * sizeof(float) * (size_t)inv_base(NN, n_sims);
    size_t need = sizeof(float) * (size_t)band_off[n_sims];
    const size_t margin = (size_t)2 << 30;
    if (need + inv_bytes + margin > fr) {
      std::fill(h->band_b.begin(), h->band_b.end(), 0);
      std::fill(band_off.begin(), band_off.end(), 0);
      need = 0;
    }
    for (int s = 0; s < n_sims; ++s) {
      h->max_b = std::max(h->max_b, h->band_b[s]);
      if (h->band_b[s]) h->any_band = true;
      else h->any_jacobi = true;
    }
    int64_t *p_boff;
    int *p_bw, *p_pos, *p_nat;
    CK(A.upload(&p_boff, band_off));
    CK(A.upload(&p_bw, h->band_b));
    CK(A.upload(&p_pos, pos_all));
    CK(A.upload(&p_nat, node_at));
    CK(A.upload(&h->d_blk_row, blk_row));
    h->band_floats = (size_t)band_off[n_sims];
    float *p_band, *p_work, *p_li, *p_ui;
    CK(A.alloc(&p_band, h->band_floats));
    CK(A.alloc(&p_work, ND));
    const size_t inv = h->any_band ? (size_t)inv_base(NN, n_sims) : 1;
    CK(A.alloc(&p_li, inv));
    CK(A.alloc(&p_ui, inv));
    CK(A.alloc(&h->d_refactor, n_sims));
    int* p_lu_fail;
    CK(A.alloc(&p_lu_fail, n_sims));
    CK(cudaMemset(p_lu_fail, 0, sizeof(int) * n_sims));
    // CTA order of the per-simulation kernels: decreasing n (b + 1) (band solve and LU work)
    std::vector<int> order(n_sims);
    for (int s = 0; s < n_sims; ++s) order[s] = s;
    auto cost = [&](int s) { return (h->node_off[s + 1] - h->node_off[s]) * (int64_t)(h->band_b[s] + 6); };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
    int* p_order;
    CK(A.upload(&p_order, order));
    h->band = BandDev{p_band, p_boff, p_bw, p_pos, p_nat, p_work, p_li, p_ui, h->d_refactor, p_order, p_lu_fail};
    // the tensor-core factorisation where its shared memory fits the widest band
    h->tc_lu = h->any_band && p->band_lu == EB_LU_TENSOR && band_lu_tc_smem(h->max_b) <= kLuTcSmemLimit;
    sa.band = h->band;
    sa.cta_sim = p_order;
    h->need_refactor.assign(n_sims, 1);
    h->refactor_mask.assign(n_sims, 0);
    h->its0.assign(n_sims, -1);
    h->excess.assign(n_sims, 0.0);
    h->lu_cost.assign(n_sims, 0.0);
    for (int s = 0; s < n_sims; ++s) h->lu_cost[s] = p->refactor_cost * h->band_b[s];
    h->dt_at_factor.assign(n_sims, 0.0);
    h->cur_dt.assign(n_sims, 0.0);
    h->cur_active.assign(n_sims, 0);
    int max_n = 0;
    for (int s = 0; s < n_sims; ++s) max_n = std::max<int>(max_n, (int)(6 * (h->node_off[s + 1] - h->node_off[s])));
    sa.max_n = max_n;
    sa.x_in_smem = h->any_band && gmres_smem(m) + sizeof(float) * (size_t)max_n <= 200 * 1024;
    // stage band blocks through shared memory when the two buffers fit beside the rest
    sa.stage_floats = 0;
    sa.stage_test_extra = p->stage_band == 2 ? 16 : 0;
    if (h->any_band && p->stage_band) {
      sa.stage_floats = kPanel * (h->max_b + 1);
      if (gmres_smem_total(sa) > kGmresSmemLimit) sa.stage_floats = 0;
    }
    // Occupancy classes: the staging buffers are sized for the widest band of a launch, so
    // one launch runs every CTA at the occupancy of the largest simulation.  Simulations
    // whose own staged solve fits two CTAs per SM form a second launch with its own
    // buffer size, on a second stream beside the first.
    h->gclass.clear();
    if (sa.stage_floats > 0) {
      auto args_for = [&](const std::vector<int>& sims, bool two) {
        SolverArgs c = sa;
        int bmax = 0, nmax = 0;
        for (int s2 : sims) {
          bmax = std::max(bmax, h->band_b[s2]);
          nmax = std::max<int>(nmax, (int)(6 * (h->node_off[s2 + 1] - h->node_off[s2])));
        }
        c.n_sims = (int)sims.size();
        c.max_n = nmax;
        c.stage_floats = kPanel * (bmax + 1);
        c.x_in_smem = 1;
        if (gmres_smem_total(c) > (two ? kGmresTwoPerSm : (size_t)200 * 1024)) c.x_in_smem = 0;
        if (gmres_smem_total(c) > (two ? kGmresTwoPerSm : kGmresSmemLimit)) c.stage_floats = 0;
        return c;
      };
      std::vector<int> big, small;
      for (int s2 : order) {
        SolverArgs one = sa;
        one.x_in_smem = 0;
        one.stage_floats = kPanel * (h->band_b[s2] + 1);
        (h->band_b[s2] > 0 && gmres_smem_total(one) > kGmresTwoPerSm ? big : small).push_back(s2);
      }
      if (!big.empty() && !small.empty()) {
        std::vector<int> cta(big);
        cta.insert(cta.end(), small.begin(), small.end());
        int* p_cta;
        CK(A.upload(&p_cta, cta));
        SolverArgs cb = args_for(big, false), cs = args_for(small, true);
        cb.cta_sim = p_cta;
        cs.cta_sim = p_cta + big.size();
        h->gclass = {cb, cs};
        CK(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
      }
    }
  }

  // ---- learned warm start: neighbour table and surface flags (buffers for features on first use)
  {
    std::vector<int> nb(2 * NN);
    for (int64_t i = 0; i < NN; ++i) {
      int q = 0;
      for (int c : adj[i])
        if (c != (int)i && q < 2) nb[2 * i + q++] = c;
      for (; q < 2; ++q) nb[2 * i + q] = (int)i;
    }
    CK(A.upload(&h->ws.d_nb, nb));
    CK(A.upload(&h->ws.d_surf_on, h->has_contact));
    CK(A.alloc(&h->ws.d_rn, 2 * (size_t)n_sims));
    h->ws.dev.nb = h->ws.d_nb;
    h->ws.dev.surf_on = h->ws.d_surf_on;
    h->ws.rn.assign(2 * (size_t)n_sims, 0.0);
    h->ws.used.assign(n_sims, 0);
    h->ws.tried.assign(n_sims, 0);
    h->ws.streak.assign(n_sims, 0);
    h->ws.skip.assign(n_sims, 0);
  }

  // ---- initialize_state_simulation! (inizialization.jl:37-44): beams only, matricesⁿ ← matricesⁿ⁺¹
  int rc = upload_mask(h.get(), h->d_active, nullptr);
  if (rc) return rc;
  launch_beam(d, h->gauss, h->stream);
  launch_gather(d, p->alpha, false, h->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(d.Kn, d.K1, sizeof(double) * NB * 36, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(d.Cn, d.C1, sizeof(double) * NB * 36, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(d.Mn, d.M1, sizeof(double) * NB * 36, cudaMemcpyDeviceToDevice, h->stream));
  // forcesⁿ (Tⁱⁿᵗ, Tᵏ, Tᶜ) stay zero after this call, as in the reference
  CK(cudaStreamSynchronize(h->stream));
  *out = h.release();
  return EB_OK;
}

int eb_destroy(eb_handle* h) {
  delete h;  // ~eb_handle releases everything, also on a failed eb_create
  return EB_OK;
}

int eb_set_device(int32_t device) {
  CK(cudaSetDevice(device));
  return EB_OK;
}

int eb_get_device(int32_t* device) {
  if (!device) return fail(EB_ERR_ARG, "null device");
  int d = 0;
  CK(cudaGetDevice(&d));
  *device = d;
  return EB_OK;
}

int eb_timer_start(eb_handle* h) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  CK(cudaEventRecord(h->t0, h->stream));
  h->timer.ref = h->timer.on ? h->t0 : nullptr;
  h->timer.iv.clear();
  return EB_OK;
}

int eb_timer_stop(eb_handle* h, double* ms) {
  if (!h || !ms) return fail(EB_ERR_ARG, "bad arguments");
  CK(cudaEventRecord(h->t1, h->stream));
  CK(cudaEventSynchronize(h->t1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->t0, h->t1));
  *ms = t;
  return EB_OK;
}

int eb_timer_between(eb_handle* from, eb_handle* to, double* ms) {
  if (!from || !to || !ms) return fail(EB_ERR_ARG, "bad arguments");
  CK(cudaEventSynchronize(to->t1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, from->t0, to->t1));
  *ms = t;
  return EB_OK;
}

int eb_get_phase_intervals(eb_handle* h, eb_handle* ref, int32_t phase, double* start_ms, double* end_ms,
                           int64_t cap, int64_t* count) {
  if (!h || !ref || !count || phase < 0 || phase >= EB_NPHASES || cap < 0 || (cap > 0 && (!start_ms || !end_ms)))
    return fail(EB_ERR_ARG, "bad arguments");
  float off = 0.f;
  if (ref != h) CK(cudaEventElapsedTime(&off, ref->t0, h->t0));
  int64_t n = 0;
  for (size_t i = 0; i + 2 < h->timer.iv.size(); i += 3) {
    if ((int)h->timer.iv[i] != phase) continue;
    if (n < cap) {
      start_ms[n] = (double)off + h->timer.iv[i + 1];
      end_ms[n] = (double)off + h->timer.iv[i + 2];
    }
    ++n;
  }
  *count = n;
  return EB_OK;
}

int eb_get_phase_times(eb_handle* h, double* ms, int64_t* launches, int32_t reset) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  for (int i = 0; i < EB_NPHASES; ++i) {
    if (ms) ms[i] = h->timer.ms[i];
    if (launches) launches[i] = h->timer.launches[i];
    if (reset) {
      h->timer.ms[i] = 0;
      h->timer.launches[i] = 0;
    }
  }
  return EB_OK;
}

static int set_values(eb_handle* h, int32_t sim, const double* values, const std::vector<int64_t>& off,
                      const int64_t* d_idx, double* dst) {
  if (!h || sim < 0 || sim >= h->n_sims) return fail(EB_ERR_ARG, "bad handle or sim index");
  const int64_t o = off[sim], n = off[sim + 1] - o;
  if (n == 0) return EB_OK;
  if (!values) return fail(EB_ERR_ARG, "values is null");
  CK(cudaMemcpyAsync(h->d_vals, values, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  k_scatter<<<nblocks(n, 256), 256, 0, h->stream>>>(d_idx + o, h->d_vals, n, dst);
  h->timer.launches[EB_PHASE_UPDATE] += 1;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return EB_OK;
}

int eb_set_loads(eb_handle* h, int32_t sim, const double* values) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  return set_values(h, sim, values, h->load_off, h->d_load_dof, h->d.fext1);
}

int eb_set_imposed(eb_handle* h, int32_t sim, const double* values) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  return set_values(h, sim, values, h->fix_off, h->d_fix_dof, h->d.imposed);
}

int eb_set_loads_all(eb_handle* h, const double* values) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  const int64_t n = (int64_t)h->load_dof.size();
  if (n == 0) return EB_OK;
  if (!values) return fail(EB_ERR_ARG, "values is null");
  CK(cudaMemcpyAsync(h->d_vals, values, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  k_scatter<<<nblocks(n, 256), 256, 0, h->stream>>>(h->d_load_dof, h->d_vals, n, h->d.fext1);
  h->timer.launches[EB_PHASE_UPDATE] += 1;
  CK(cudaGetLastError());
  return EB_OK;
}

int eb_get_displacements(eb_handle* h, double* u) {
  if (!h || !u) return fail(EB_ERR_ARG, "bad arguments");
  const int64_t NN = h->d.n_nodes;
  if (!h->d_u3) CK(h->arena.alloc(&h->d_u3, 3 * (size_t)NN));
  if (NN) k_interleave3<<<nblocks(3 * NN, 256), 256, 0, h->stream>>>(h->d.u, NN, h->d_u3);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(u, h->d_u3, sizeof(double) * 3 * NN, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return EB_OK;
}

// Launch-shape autotuner: times the element, contact and assembly kernels on the
// current state at each candidate block size and keeps the fastest.  Every
// candidate computes each output with the same operations in the same order (one
// thread per element / block entry / DOF), so the choice changes no result.  The
// kernels overwrite only the n+1 staging and assembly arrays, which every step
// recomputes before reading them; hence the call must come between steps.
int eb_autotune(eb_handle* h, int32_t* chosen) {
  if (!h) return fail(EB_ERR_ARG, "eb_autotune: null handle");
  if (h->mid_step) return fail(EB_ERR_STATE, "eb_autotune: call it between steps (after eb_commit or eb_rollback)");
  Dev& d = h->d;
  cudaStream_t st = h->stream;
  const int S = h->n_sims;
  std::vector<int> ones(S, 1);
  CK(cudaMemcpyAsync(h->d_active, ones.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  cudaError_t err = cudaEventCreate(&e1);
  if (err != cudaSuccess) {
    cudaEventDestroy(e0);
    CK(err);
  }
  const double alpha = h->P.alpha;
  // a candidate replaces the current shape only when it is at least 5% faster
  auto time_it = [&](int* knob, const int* cand, int nc, auto&& launch) -> cudaError_t {
    float best = INFINITY, t_cur = INFINITY;
    const int cur = *knob;
    int pick = cur;
    for (int c = 0; c < nc; ++c) {
      *knob = cand[c];
      launch();
      cudaEventRecord(e0, st);
      for (int r = 0; r < 5; ++r) launch();
      cudaEventRecord(e1, st);
      cudaError_t e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (cand[c] == cur) t_cur = ms;
      if (ms < best) {
        best = ms;
        pick = cand[c];
      }
    }
    *knob = (best < 0.95f * t_cur) ? pick : cur;
    return cudaSuccess;
  };
  static const int kElem[3] = {64, 128, 256}, kGather[3] = {128, 256, 512};
  err = time_it(&d.beam_threads, kElem, 3, [&] { launch_beam(d, h->gauss, st); });
  if (err == cudaSuccess && h->any_contact)
    err = time_it(&d.contact_threads, kElem, 3, [&] { launch_contact(d, h->gauss, st); });
  if (err == cudaSuccess)
    err = time_it(&d.gmat_threads, kGather, 3, [&] { launch_gather(d, alpha, h->any_contact, st); });
  if (err == cudaSuccess)
    err = time_it(&d.gvec_threads, kGather, 3, [&] { launch_gather(d, alpha, h->any_contact, st); });
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(err);
  h->graph_gen += 1;  // captured iterations hold the old launch shapes
  if (chosen) {
    chosen[0] = d.beam_threads;
    chosen[1] = d.contact_threads;
    chosen[2] = d.gmat_threads;
    chosen[3] = d.gvec_threads;
  }
  return EB_OK;
}

int eb_set_launch_shapes(eb_handle* h, const int32_t* shapes) {
  if (!h || !shapes) return fail(EB_ERR_ARG, "eb_set_launch_shapes: bad arguments");
  for (int k = 0; k < 4; ++k) {
    const int v = shapes[k], hi = k < 2 ? kMaxElemThreads : 1024;
    if (v < 32 || v > hi || v % 32) return fail(EB_ERR_ARG, "eb_set_launch_shapes: shape %d = %d (multiples of 32 up to %d)", k, v, hi);
  }
  h->d.beam_threads = shapes[0];
  h->d.contact_threads = shapes[1];
  h->d.gmat_threads = shapes[2];
  h->d.gvec_threads = shapes[3];
  h->graph_gen += 1;
  return EB_OK;
}

int eb_beam_output(eb_handle* h, int32_t sim, int32_t points_per_beam, double* out) {
  if (!h || !out || sim < 0 || sim >= h->n_sims) return fail(EB_ERR_ARG, "eb_beam_output: bad arguments");
  if (points_per_beam < 2) return fail(EB_ERR_ARG, "eb_beam_output: points_per_beam must be at least 2");
  const int64_t e0 = h->elem_off[sim], ne = h->elem_off[sim + 1] - e0;
  const size_t n = (size_t)beam_output_doubles(ne, points_per_beam);
  double* dbuf = nullptr;
  CK(cudaMalloc(&dbuf, sizeof(double) * n));
  launch_beam_output(h->d, h->d_E, e0, ne, points_per_beam, dbuf, h->stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dbuf, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(dbuf);
  CK(e);
  return EB_OK;
}

int eb_vtk_open(eb_handle* h, const char* const* dirs, int32_t points_per_beam) {
  if (!h || !dirs) return fail(EB_ERR_ARG, "eb_vtk_open: bad arguments");
  if (h->vtk) return fail(EB_ERR_STATE, "eb_vtk_open: output already open (eb_vtk_close first)");
  std::vector<VtkSim> sims(h->n_sims);
  std::vector<std::string> ds(h->n_sims);
  for (int s = 0; s < h->n_sims; ++s) {
    sims[s] = VtkSim{h->elem_off[s], h->elem_off[s + 1] - h->elem_off[s], h->node_off[s],
                     h->node_off[s + 1] - h->node_off[s]};
    ds[s] = dirs[s] ? dirs[s] : "";
  }
  std::string err;
  h->vtk = vtk_open(h->d, h->d_E, h->stream, sims, ds, points_per_beam, err);
  if (!h->vtk) return fail(EB_ERR_ARG, "eb_vtk_open: %s", err.c_str());
  return EB_OK;
}

int eb_vtk_write(eb_handle* h, const int32_t* mask, const int32_t* counter, const int32_t* step, const double* t) {
  if (!h || !counter || !step || !t) return fail(EB_ERR_ARG, "eb_vtk_write: bad arguments");
  if (!h->vtk) return fail(EB_ERR_STATE, "eb_vtk_write: output not open (eb_vtk_open)");
  std::string err;
  if (vtk_write(h->vtk, mask, counter, step, t, err)) return fail(EB_ERR_CUDA, "%s", err.c_str());
  return EB_OK;
}

int eb_vtk_flush(eb_handle* h) {
  if (!h) return fail(EB_ERR_ARG, "eb_vtk_flush: null handle");
  if (!h->vtk) return EB_OK;
  std::string err;
  if (vtk_flush(h->vtk, err)) return fail(EB_ERR_IO, "eb_vtk_flush: %s", err.c_str());
  return EB_OK;
}

int eb_vtk_close(eb_handle* h) {
  if (!h) return fail(EB_ERR_ARG, "eb_vtk_close: null handle");
  if (!h->vtk) return EB_OK;
  std::string err;
  const int rc = vtk_close(h->vtk, err);
  h->vtk = nullptr;
  if (rc) return fail(EB_ERR_IO, "eb_vtk_close: %s", err.c_str());
  return EB_OK;
}

// First Newton iteration from the learned start: simulations whose residual at
// the learned start exceeds the HHT predictor's right-hand side (or is not
// finite) go back to their committed node state and take the plain predictor
// (predictor.jl:1-27) instead; then their first corrector assembly is redone.
static int learned_start_check(eb_handle* h, const std::vector<int>& running, double a, double b, double g) {
  WsHost& ws = h->ws;
  const Dev& d = h->d;
  const int S = h->n_sims;
  cudaStream_t st = h->stream;
  launch_ws_rnorm(d, ws.d_rn + S, st);
  CK(cudaMemcpyAsync(ws.rn.data(), ws.d_rn, sizeof(double) * 2 * S, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::vector<int> fb(S, 0);
  bool any = false;
  for (int s = 0; s < S; ++s) {
    if (!running[s] || !ws.tried[s]) continue;
    const double r0 = ws.rn[s], r1 = ws.rn[S + s];
    fb[s] = !(std::isfinite(r1) && r1 <= r0);
    ws.used[s] = !fb[s];
    any |= fb[s] != 0;
    if (fb[s]) {
      ws.streak[s] = std::min(ws.streak[s] + 1, 6);
      ws.skip[s] = 1 << (ws.streak[s] - 1);
    } else {
      ws.streak[s] = 0;
    }
  }
  if (!any) return EB_OK;
  PhaseTimer& T = h->timer;
  CK(cudaMemcpyAsync(h->d_active, fb.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(h->d_mask, fb.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
  launch_restore_nodes(d, h->d_mask, st);
  launch_init_predictor(d, st);
  launch_predictor_rhs(d, a, b, g, st);
  launch_apply_bc(d, st);
  T.launches[EB_PHASE_PREDICTOR] += 4;
  int rc = solve(h, fb.data(), false);
  if (rc) return rc;
  launch_global_predictor(d, b, g, st);
  launch_local_predictor(d, b, g, st);
  launch_init_corrector(d, st);
  launch_beam(d, h->gauss, st);
  if (h->any_contact) launch_contact(d, h->gauss, st);
  launch_gather(d, a, h->any_contact, st);
  launch_corrector_rhs(d, a, st);
  launch_apply_bc(d, st);
  T.launches[EB_PHASE_PREDICTOR] += 9;
  CK(cudaMemcpyAsync(h->d_active, running.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
  CK(cudaGetLastError());
  return EB_OK;
}

int eb_step(eb_handle* h, const double* dt, const int32_t* active, int32_t* k_out, int32_t* status_out) {
  if (!h || !dt || !k_out) return fail(EB_ERR_ARG, "eb_step: bad arguments");
  const int S = h->n_sims;
  const eb_params& P = h->P;
  const bool learned = P.warm_start == EB_WS_LEARNED;
  const bool learned_x0 = P.warm_start == EB_WS_LEARNED_X0;
  if ((learned || learned_x0) && !h->ws.model)
    return fail(EB_ERR_STATE, "eb_step: a learned warm start is selected but no model is set");
  const double a = P.alpha, b = P.beta, g = P.gamma;
  std::vector<double> cK(S), cC(S), cM(S), dts(S);
  std::vector<int> act(S), iter(S, 0), k(S, 1);
  for (int s = 0; s < S; ++s) {
    act[s] = active ? (active[s] != 0) : 1;
    if (act[s] && !(dt[s] > 0)) return fail(EB_ERR_ARG, "eb_step: dt[%d] must be positive", s);
    dts[s] = dt[s];
    h->cur_dt[s] = dt[s];
    h->cur_active[s] = act[s];
    cK[s] = 1 + a;
    cC[s] = g / (b * dt[s]);
    cM[s] = 1 / (b * (dt[s] * dt[s]));
  }
  cudaStream_t st = h->stream;
  CK(cudaMemcpyAsync(h->d_cK, cK.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(h->d_cC, cC.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(h->d_cM, cM.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(h->d_dt, dts.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(h->d_active, act.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(h->d_its, 0, sizeof(int) * S, st));
  CK(cudaMemsetAsync(h->d_refs, 0, sizeof(int) * S, st));
  CK(cudaMemsetAsync(h->d_status, 0, sizeof(int) * S, st));
  CK(cudaMemsetAsync(h->d_relres, 0, sizeof(double) * S, st));
  const Dev& d = h->d;
  PhaseTimer& T = h->timer;
  h->mid_step = true;
  T.begin(st);

  // ---- features of the learned start / of the captured samples (committed state)
  WsHost& ws = h->ws;
  if (learned || learned_x0 || ws.cap > 0) {
    launch_ws_features(d, ws.dev, st);
    T.launches[EB_PHASE_PREDICTOR] += 1;
    ws.features_valid = true;
  }
  // ---- predictor! (predictor.jl:1-27)
  launch_init_predictor(d, st);
  launch_predictor_rhs(d, a, b, g, st);
  launch_apply_bc(d, st);
  T.mark(EB_PHASE_PREDICTOR, st);
  T.launches[EB_PHASE_PREDICTOR] += 4;
  int rc = 0;
  if (learned) {
    // Simulations whose learned starts were rejected recently back off (1, 2, 4 .. 64 steps)
    // and take the HHT predictor; the others start from the network, with the predictor's
    // right-hand side norm as the fallback threshold.
    std::vector<int> plain(S, 0);
    bool any_plain = false, any_try = false;
    for (int s = 0; s < S; ++s) {
      ws.tried[s] = act[s] && ws.skip[s] == 0;
      plain[s] = act[s] && !ws.tried[s];
      if (plain[s]) ws.skip[s] -= 1;
      any_plain |= plain[s] != 0;
      any_try |= ws.tried[s] != 0;
    }
    if (any_plain) {
      CK(cudaMemcpyAsync(h->d_active, plain.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
      rc = solve(h, plain.data(), false);
      if (rc) return rc;
    }
    if (any_try) {
      CK(cudaMemcpyAsync(h->d_active, ws.tried.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
      launch_ws_rnorm(d, ws.d_rn, st);
      CK(mlp_forward(MlpDev{ws.P, ws.W}, ws.X, d.n_nodes, ws.Y, st));
      launch_ws_apply(d, ws.dev, st);
      T.launches[EB_PHASE_PREDICTOR] += 3;
    }
    CK(cudaMemcpyAsync(h->d_active, act.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
  } else if (learned_x0) {
    // the network's increment as the initial guess of the predictor's solve (free DOFs of dD)
    CK(mlp_forward(MlpDev{ws.P, ws.W}, ws.X, d.n_nodes, ws.Y, st));
    launch_ws_apply(d, ws.dev, st);
    T.launches[EB_PHASE_PREDICTOR] += 2;
    CK(cudaMemcpyAsync(h->d_x0_on, act.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
    rc = solve(h, act.data(), false);
    if (rc) return rc;
    CK(cudaMemsetAsync(h->d_x0_on, 0, sizeof(int) * S, st));
  } else {
    rc = solve(h, act.data(), false);
    if (rc) return rc;
  }
  CK(cudaMemcpyAsync(h->d_pred_its, h->d_its, sizeof(int) * S, cudaMemcpyDeviceToDevice, st));
  launch_global_predictor(d, b, g, st);
  launch_local_predictor(d, b, g, st);
  // ---- corrector! (corrector.jl:1-59)
  launch_init_corrector(d, st);
  T.mark(EB_PHASE_PREDICTOR, st);
  T.launches[EB_PHASE_PREDICTOR] += 3;
  CK(cudaGetLastError());
  if (T.on) {
    CK(cudaStreamSynchronize(st));
    T.resolve();
  }
  if (h->sa.forcing) CK(cudaMemsetAsync(h->sa.prev_bnorm, 0, sizeof(double) * S, st));  // first corrector solve: forcing_max
  std::vector<double> res(S, INFINITY), dn(S, INFINITY);
  std::vector<int> running(S);
  const std::vector<int>& max_it = h->max_it;
  for (int s = 0; s < S; ++s) running[s] = act[s] && (1 <= max_it[s]);
  bool first = true;
  std::fill(ws.used.begin(), ws.used.end(), 0);
  while (true) {
    bool any = false;
    for (int s = 0; s < S; ++s) any |= running[s] != 0;
    if (!any) break;
    if (P.use_graph && !P.timing && !(learned && first)) {
      // the iteration as one CUDA graph launch (the learned start's first iteration, with its
      // host-side check, and iterations timed phase by phase run as separate launches)
      std::memcpy(h->pin_active, running.data(), sizeof(int) * S);
      const bool ref = plan_refactor(h, running.data());
      if (ref) std::memcpy(h->pin_refactor, h->refactor_mask.data(), sizeof(int) * S);
      rc = run_iteration_graph(h, ref);
      if (rc) return rc;
      CK(cudaStreamSynchronize(st));
      resolve_graph_times(h, ref);
      std::memcpy(h->h_norms.data(), h->pin_norms, sizeof(double) * 5 * S);
      first = false;
    } else {
    T.begin(st);
    CK(cudaMemcpyAsync(h->d_active, running.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
    T.mark(EB_PHASE_UPDATE, st);
    launch_beam(d, h->gauss, st);
    T.mark(EB_PHASE_BEAM, st);
    T.launches[EB_PHASE_BEAM] += 1;
    if (h->any_contact) {
      launch_contact(d, h->gauss, st);
      T.mark(EB_PHASE_CONTACT, st);
      T.launches[EB_PHASE_CONTACT] += 1;
    }
    launch_gather(d, a, h->any_contact, st);
    T.mark(EB_PHASE_ASSEMBLY, st);
    T.launches[EB_PHASE_ASSEMBLY] += 2;
    launch_corrector_rhs(d, a, st);
    launch_apply_bc(d, st);
    T.mark(EB_PHASE_RESIDUAL, st);
    T.launches[EB_PHASE_RESIDUAL] += 3;
    if (learned && first) {
      rc = learned_start_check(h, running, a, b, g);
      if (rc) return rc;
    }
    first = false;
    rc = solve(h, running.data(), true);
    if (rc) return rc;
    launch_global_corrector(d, st);
    launch_local_corrector(d, b, g, st);
    T.launches[EB_PHASE_UPDATE] += 2;
    CK(cudaMemcpyAsync(h->h_norms.data(), h->d_norms, sizeof(double) * 5 * S, cudaMemcpyDeviceToHost, st));
    T.mark(EB_PHASE_UPDATE, st);
    CK(cudaStreamSynchronize(st));
    T.resolve();
    }
    for (int s = 0; s < S; ++s) {
      if (!running[s]) continue;
      const double* q = &h->h_norms[5 * s];
      if (q[4] < 0) {
        // a bulk-copy wait ran out in this solve: stop this simulation's Newton loop (the step
        // reports EB_SIM_WAIT_TIMEOUT) and read band blocks from global memory from now on
        disable_staging(h);
        h->graph_gen += 1;
        running[s] = 0;
        k[s] = max_it[s] + 1;
        continue;
      }
      if (h->P.refactor_its > 0 && q[4] > h->P.refactor_its) h->need_refactor[s] = 1;
      if (h->P.refactor_policy == EB_REFACTOR_COST && h->band_b.size() && h->band_b[s] > 0) {
        // rent or buy: iterations beyond the fresh factorisation's, summed, against the LU's cost
        const int its_s = (int)q[4];
        if (h->its0[s] < 0) h->its0[s] = its_s;
        else h->excess[s] += std::max(0, its_s - h->its0[s]);
        if (h->excess[s] >= h->lu_cost[s]) h->need_refactor[s] = 1;
      }
      // compute_norms_corrector (utils_solver.jl:126-151)
      double dnorm = std::sqrt(q[0]);
      double rn = std::sqrt(q[1]);
      const double fn = std::sqrt(q[2]), en = std::sqrt(q[3]);
      if (fn + en > 1e-12) rn = rn / (fn + en);
      res[s] = rn;
      dn[s] = dnorm;
      ++iter[s];
      k[s] += 1;
      if (!std::isfinite(rn) || !std::isfinite(dnorm)) {
        // The reference's loop test (corrector.jl:15) is false for NaN norms, so it would
        // accept the step; here the simulation stops iterating and the step is reported not
        // converged (EB_SIM_NAN), so its caller rolls it back instead of committing NaNs.
        running[s] = 0;
        k[s] = max_it[s] + 1;
        continue;
      }
      running[s] = (res[s] > h->tol_res[s] || dn[s] > h->tol_disp[s]) && k[s] <= max_it[s];
    }
  }
  // ---- statistics
  std::vector<int> its(S), refs(S), status(S), pred_its(S);
  std::vector<double> rel(S);
  CK(cudaMemcpyAsync(pred_its.data(), h->d_pred_its, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(its.data(), h->d_its, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(refs.data(), h->d_refs, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(status.data(), h->d_status, sizeof(int) * S, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(rel.data(), h->d_relres, sizeof(double) * S, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int s = 0; s < S; ++s) {
    eb_sim_stats& q = h->stats[s];
    if (!act[s]) continue;
    int stt = status[s];
    if (stt != EB_SIM_WAIT_TIMEOUT && (!std::isfinite(res[s]) || !std::isfinite(dn[s]))) stt = EB_SIM_NAN;
    if (k[s] > max_it[s] && stt == EB_SIM_OK) stt = EB_SIM_NOT_CONVERGED;
    if (stt == EB_SIM_WAIT_TIMEOUT) {
      // the step's solves are not trusted: report "not converged" (the caller rolls back)
      // and read band blocks from global memory from now on
      k[s] = max_it[s] + 1;
      disable_staging(h);
      h->graph_gen += 1;
    }
    q.newton_iterations = iter[s];
    q.krylov_iterations = its[s];
    q.refinements = refs[s];
    q.status = stt;
    q.last_res_norm = res[s];
    q.last_dD_norm = dn[s];
    q.max_linear_rel_residual = rel[s];
    q.warm_start_used = learned ? ws.used[s] : 0;
    q.predictor_krylov_iterations = pred_its[s];
    q.predictor_rhs_norm = learned && ws.tried[s] ? std::sqrt(ws.rn[s]) : 0.0;
    q.start_res_norm = learned && ws.tried[s] ? std::sqrt(ws.rn[S + s]) : 0.0;
    k_out[s] = k[s];
    if (status_out) status_out[s] = stt;
  }
  return EB_OK;
}

static int commit_impl(eb_handle* h, const int32_t* mask, bool commit) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  h->mid_step = false;
  int rc = upload_mask(h, h->d_mask, mask);
  if (rc) return rc;
  WsHost& ws = h->ws;
  if (commit && ws.cap > 0 && ws.features_valid) {
    const int64_t per = (h->d.n_nodes + ws.stride - 1) / ws.stride;
    launch_ws_capture(h->d, ws.dev, h->d_mask, ws.phase, ws.stride, ws.cursor, ws.cap, ws.sF, ws.sT, h->stream);
    ws.cursor = (ws.cursor + per) % ws.cap;
    ws.written = std::min(ws.cap, ws.written + per);
    ws.phase += 1;
  }
  ws.features_valid = false;
  launch_commit(h->d, h->d_mask, commit, h->stream);
  h->timer.launches[EB_PHASE_UPDATE] += 3;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return EB_OK;
}

int eb_commit(eb_handle* h, const int32_t* mask) { return commit_impl(h, mask, true); }
int eb_rollback(eb_handle* h, const int32_t* mask) { return commit_impl(h, mask, false); }

static int get_state_impl(eb_handle* h, int32_t sim, bool at_n, double* u, double* ud, double* udd, double* w,
                          double* wd, double* wdd, double* R, double* dR) {
  if (!h || sim < 0 || sim >= h->n_sims) return fail(EB_ERR_ARG, "bad handle or sim index");
  const int64_t NN = h->d.n_nodes, o = h->node_off[sim], n = h->node_off[sim + 1] - o;
  const Dev& d = h->d;
  double* src[8] = {at_n ? d.un : d.u,   at_n ? d.udn : d.ud, at_n ? d.uddn : d.udd, at_n ? d.wn : d.w,
                    at_n ? d.wdn : d.wd, at_n ? d.wddn : d.wdd, at_n ? d.Rn : d.R,   at_n ? d.dRn : d.dR};
  double* dst[8] = {u, ud, udd, w, wd, wdd, R, dR};
  const int nc[8] = {3, 3, 3, 3, 3, 3, 9, 9};
  std::vector<double> tmp((size_t)n);
  for (int f = 0; f < 8; ++f) {
    if (!dst[f]) continue;
    for (int k = 0; k < nc[f]; ++k) {
      CK(cudaMemcpy(tmp.data(), src[f] + k * NN + o, sizeof(double) * n, cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < n; ++i) dst[f][nc[f] * i + k] = tmp[i];
    }
  }
  return EB_OK;
}

int eb_get_state(eb_handle* h, int32_t sim, double* u, double* ud, double* udd, double* w, double* wd, double* wdd,
                 double* R, double* dR) {
  return get_state_impl(h, sim, false, u, ud, udd, w, wd, wdd, R, dR);
}
int eb_get_state_n(eb_handle* h, int32_t sim, double* u, double* ud, double* udd, double* w, double* wd,
                   double* wdd, double* R, double* dR) {
  return get_state_impl(h, sim, true, u, ud, udd, w, wd, wdd, R, dR);
}

// Writes one simulation's node record into both the committed state (n) and the working
// state (n+1); fields passed as NULL are left as they are.
int eb_set_state(eb_handle* h, int32_t sim, const double* u, const double* ud, const double* udd, const double* w,
                 const double* wd, const double* wdd, const double* R, const double* dR) {
  if (!h || sim < 0 || sim >= h->n_sims) return fail(EB_ERR_ARG, "eb_set_state: bad handle or sim index");
  if (h->mid_step) return fail(EB_ERR_STATE, "eb_set_state: between eb_step and eb_commit/eb_rollback");
  const int64_t NN = h->d.n_nodes, o = h->node_off[sim], n = h->node_off[sim + 1] - o;
  const Dev& d = h->d;
  double* dst[8][2] = {{d.u, d.un},   {d.ud, d.udn}, {d.udd, d.uddn}, {d.w, d.wn},
                       {d.wd, d.wdn}, {d.wdd, d.wddn}, {d.R, d.Rn},   {d.dR, d.dRn}};
  const double* src[8] = {u, ud, udd, w, wd, wdd, R, dR};
  const int nc[8] = {3, 3, 3, 3, 3, 3, 9, 9};
  std::vector<double> tmp((size_t)n);
  CK(cudaStreamSynchronize(h->stream));
  for (int f = 0; f < 8; ++f) {
    if (!src[f]) continue;
    for (int k = 0; k < nc[f]; ++k) {
      for (int64_t i = 0; i < n; ++i) tmp[i] = src[f][nc[f] * i + k];
      for (int t = 0; t < 2; ++t)
        CK(cudaMemcpy(dst[f][t] + k * NN + o, tmp.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    }
  }
  return EB_OK;
}

int eb_set_max_iterations(eb_handle* h, const int32_t* max_iterations) {
  if (!h) return fail(EB_ERR_ARG, "eb_set_max_iterations: null handle");
  for (int s = 0; s < h->n_sims; ++s) {
    const int m = max_iterations ? max_iterations[s] : h->P.max_iterations;
    if (m < 0) return fail(EB_ERR_ARG, "eb_set_max_iterations: negative cap for simulation %d", s);
  }
  for (int s = 0; s < h->n_sims; ++s) h->max_it[s] = max_iterations ? max_iterations[s] : h->P.max_iterations;
  return EB_OK;
}

int eb_set_tolerances(eb_handle* h, const double* tolerance_residual, const double* tolerance_displacement) {
  if (!h) return fail(EB_ERR_ARG, "eb_set_tolerances: null handle");
  for (int s = 0; s < h->n_sims; ++s) {
    const double r = tolerance_residual ? tolerance_residual[s] : h->P.tolerance_residual;
    const double d = tolerance_displacement ? tolerance_displacement[s] : h->P.tolerance_displacement;
    if (!(r >= 0) || !(d >= 0)) return fail(EB_ERR_ARG, "eb_set_tolerances: bad tolerance for simulation %d", s);
  }
  for (int s = 0; s < h->n_sims; ++s) {
    h->tol_res[s] = tolerance_residual ? tolerance_residual[s] : h->P.tolerance_residual;
    h->tol_disp[s] = tolerance_displacement ? tolerance_displacement[s] : h->P.tolerance_displacement;
  }
  return EB_OK;
}

int eb_get_stats(eb_handle* h, eb_sim_stats* stats) {
  if (!h || !stats) return fail(EB_ERR_ARG, "bad arguments");
  std::memcpy(stats, h->stats.data(), sizeof(eb_sim_stats) * h->n_sims);
  return EB_OK;
}

// Feature, input and output buffers of the learned start (allocated on first use).
static int ws_buffers(eb_handle* h) {
  WsHost& ws = h->ws;
  if (ws.F) return EB_OK;
  const size_t NN = (size_t)h->d.n_nodes;
  CK(cudaMalloc(&ws.F, sizeof(float) * NN * kWsRaw));
  CK(cudaMalloc(&ws.X, sizeof(float) * NN * kMlpIn));
  CK(cudaMalloc(&ws.Y, sizeof(float) * NN * kMlpOut));
  CK(cudaMalloc(&ws.norm, sizeof(float) * (2 * kMlpIn + kMlpOut)));
  CK(cudaMemset(ws.F, 0, sizeof(float) * NN * kWsRaw));
  CK(cudaMemset(ws.X, 0, sizeof(float) * NN * kMlpIn));
  CK(cudaMemset(ws.Y, 0, sizeof(float) * NN * kMlpOut));
  // identity normalisation until a model is set
  std::vector<float> nm(2 * kMlpIn + kMlpOut, 0.f);
  for (int k = kMlpIn; k < 2 * kMlpIn + kMlpOut; ++k) nm[k] = 1.f;
  CK(cudaMemcpy(ws.norm, nm.data(), sizeof(float) * nm.size(), cudaMemcpyHostToDevice));
  ws.dev.F = ws.F;
  ws.dev.X = ws.X;
  ws.dev.Y = ws.Y;
  ws.dev.in_shift = ws.norm;
  ws.dev.in_scale = ws.norm + kMlpIn;
  ws.dev.out_scale = ws.norm + 2 * kMlpIn;
  h->arena.bytes += sizeof(float) * NN * (kWsRaw + kMlpIn + kMlpOut);
  return EB_OK;
}

int eb_ws_set_model(eb_handle* h, const float* params, const float* in_shift, const float* in_scale,
                    const float* out_scale) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  WsHost& ws = h->ws;
  if (!params) {
    ws.model = false;
    return EB_OK;
  }
  if (!in_shift || !in_scale || !out_scale) return fail(EB_ERR_ARG, "eb_ws_set_model: normalisation arrays missing");
  for (int k = 0; k < kMlpIn; ++k)
    if (!(in_scale[k] != 0.f) || !std::isfinite(in_scale[k]) || !std::isfinite(in_shift[k]))
      return fail(EB_ERR_ARG, "eb_ws_set_model: in_scale must be finite and non-zero");
  for (int k = 0; k < kMlpParams; ++k)
    if (!std::isfinite(params[k])) return fail(EB_ERR_ARG, "eb_ws_set_model: non-finite parameter %d", k);
  int rc = ws_buffers(h);
  if (rc) return rc;
  if (!ws.P) {
    CK(cudaMalloc(&ws.P, sizeof(float) * kMlpParams));
    CK(cudaMalloc(&ws.W, sizeof(__nv_bfloat16) * kMlpParams));
  }
  std::vector<float> nm(2 * kMlpIn + kMlpOut);
  std::memcpy(nm.data(), in_shift, sizeof(float) * kMlpIn);
  std::memcpy(nm.data() + kMlpIn, in_scale, sizeof(float) * kMlpIn);
  std::memcpy(nm.data() + 2 * kMlpIn, out_scale, sizeof(float) * kMlpOut);
  CK(cudaMemcpyAsync(ws.norm, nm.data(), sizeof(float) * nm.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(ws.P, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, h->stream));
  CK(mlp_to_bf16(ws.P, ws.W, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  ws.model = true;
  return EB_OK;
}

int eb_ws_capture(eb_handle* h, int64_t capacity, int32_t stride) {
  if (!h || capacity < 0 || stride < 1) return fail(EB_ERR_ARG, "eb_ws_capture: bad arguments");
  WsHost& ws = h->ws;
  CK(cudaStreamSynchronize(h->stream));
  cudaFree(ws.sF);
  cudaFree(ws.sT);
  ws.sF = ws.sT = nullptr;
  ws.cap = ws.cursor = ws.written = ws.phase = 0;
  if (capacity == 0) return EB_OK;
  int rc = ws_buffers(h);
  if (rc) return rc;
  CK(cudaMalloc(&ws.sF, sizeof(float) * (size_t)capacity * kWsRaw));
  CK(cudaMalloc(&ws.sT, sizeof(float) * (size_t)capacity * kMlpOut));
  ws.cap = capacity;
  ws.stride = stride;
  return EB_OK;
}

int eb_ws_samples(eb_handle* h, int64_t first, int64_t n, float* features, float* targets, int64_t* written) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  WsHost& ws = h->ws;
  if (written) *written = ws.written;
  if (n == 0) return EB_OK;
  if (first < 0 || n < 0 || first + n > ws.cap) return fail(EB_ERR_ARG, "eb_ws_samples: range outside the ring");
  CK(cudaStreamSynchronize(h->stream));
  if (features)
    CK(cudaMemcpy(features, ws.sF + first * kWsRaw, sizeof(float) * n * kWsRaw, cudaMemcpyDeviceToHost));
  if (targets)
    CK(cudaMemcpy(targets, ws.sT + first * kMlpOut, sizeof(float) * n * kMlpOut, cudaMemcpyDeviceToHost));
  return EB_OK;
}

int eb_get_memory(eb_handle* h, int64_t* device_bytes, int32_t* band_sims) {
  if (!h) return fail(EB_ERR_ARG, "null handle");
  if (device_bytes) *device_bytes = (int64_t)h->arena.bytes;
  if (band_sims) {
    int c = 0;
    for (int b : h->band_b) c += b > 0;
    *band_sims = c;
  }
  return EB_OK;
}

int eb_get_forces(eb_handle* h, int32_t sim, double* Tint, double* Tk, double* Tc) {
  if (!h || sim < 0 || sim >= h->n_sims) return fail(EB_ERR_ARG, "bad handle or sim index");
  const int64_t o = 6 * h->node_off[sim], n = 6 * (h->node_off[sim + 1] - h->node_off[sim]);
  if (Tint) CK(cudaMemcpy(Tint, h->d.Ti1 + o, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (Tk) CK(cudaMemcpy(Tk, h->d.Tk1 + o, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (Tc) CK(cudaMemcpy(Tc, h->d.Tc1 + o, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return EB_OK;
}

}  // extern "C"
