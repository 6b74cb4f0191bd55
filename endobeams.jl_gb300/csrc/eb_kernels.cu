// Element, contact, assembly and HHT step-algebra kernels.
#include "eb_internal.cuh"

namespace eb {
using namespace ebd;

// ------------------------------------------------------------------ loads
__device__ __forceinline__ V3 node3(const double* f, int64_t n, int i) {
  return v3(f[i], f[n + i], f[2 * n + i]);
}
__device__ __forceinline__ M3 node9(const double* f, int64_t n, int i) {
  M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = f[k * n + i];
  return m;
}
__device__ __forceinline__ void store3(double* f, int64_t n, int i, V3 v) {
  f[i] = v.x; f[n + i] = v.y; f[2 * n + i] = v.z;
}
__device__ __forceinline__ void store9(double* f, int64_t n, int i, const M3& m) {
#pragma unroll
  for (int k = 0; k < 9; ++k) f[k * n + i] = m.a[k];
}
__device__ __forceinline__ V3 elem3(const double* f, int64_t ne, int64_t e) {
  return v3(f[e], f[ne + e], f[2 * ne + e]);
}

// ------------------------------------------------------------------ assemble! element pass
// One thread per element (compute_beams via assemble_beams.jl:21-48).
__global__ void __launch_bounds__(kMaxElemThreads) k_beam(Dev d, Gauss3 g) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n_elem) return;
  if (!d.active[d.elem_sim[e]]) return;
  const int a = d.ea[e], b = d.eb[e];
  const int64_t n = d.n_nodes, ne = d.n_elem;
  BeamIn in;
  in.X1 = node3(d.X0, n, a);   in.X2 = node3(d.X0, n, b);
  in.u1 = node3(d.u, n, a);    in.u2 = node3(d.u, n, b);
  in.ud1 = node3(d.ud, n, a);  in.ud2 = node3(d.ud, n, b);
  in.wd1 = node3(d.wd, n, a);  in.wd2 = node3(d.wd, n, b);
  in.udd1 = node3(d.udd, n, a); in.udd2 = node3(d.udd, n, b);
  in.wdd1 = node3(d.wdd, n, a); in.wdd2 = node3(d.wdd, n, b);
  in.R1 = node9(d.R, n, a);    in.R2 = node9(d.R, n, b);
  in.dR1 = node9(d.dR, n, a);  in.dR2 = node9(d.dR, n, b);
#pragma unroll
  for (int k = 0; k < 9; ++k) in.Re0.a[k] = d.Re0[k * ne + e];
  in.l0 = d.l0[e];
  in.Ku = d.Kbar[e];
  in.KT = v3(d.Kbar[ne + e], d.Kbar[2 * ne + e], d.Kbar[3 * ne + e]);
  in.KTT = v3(d.Kbar[4 * ne + e], d.Kbar[5 * ne + e], d.Kbar[6 * ne + e]);
  in.Jr = elem3(d.Jr, ne, e);
  in.Ar = d.Ar[e];
  in.damping = d.damp[e];
  BeamOut o{d.stK + e * 144, d.stM + e * 144, d.stC + e * 144, d.stTi + e * 12, d.stTk + e * 12, d.stE + e * 2};
  beam_element(in, g, o);
}

// One thread per contact element (compute_contact_beams via compute&assemble…:460-482).
__global__ void __launch_bounds__(kMaxElemThreads) k_contact(Dev d, Gauss3 g) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n_elem) return;
  if (!d.is_contact[e]) return;
  const int s = d.elem_sim[e];
  if (!d.active[s]) return;
  const int a = d.ea[e], b = d.eb[e];
  const int64_t n = d.n_nodes, ne = d.n_elem;
  ContactIn in;
  in.X1 = node3(d.X0, n, a);   in.X2 = node3(d.X0, n, b);
  in.u1 = node3(d.u, n, a);    in.u2 = node3(d.u, n, b);
  in.ud1 = node3(d.ud, n, a);  in.ud2 = node3(d.ud, n, b);
  in.wd1 = node3(d.wd, n, a);  in.wd2 = node3(d.wd, n, b);
  in.R1 = node9(d.R, n, a);    in.R2 = node9(d.R, n, b);
  in.dR1 = node9(d.dR, n, a);  in.dR2 = node9(d.dR, n, b);
#pragma unroll
  for (int k = 0; k < 9; ++k) in.Re0.a[k] = d.Re0[k * ne + e];
  in.l0 = d.l0[e];
  in.radius = d.radius[e];
  const SurfaceDev srf = d.surf[s];
  const ContactProps cp = d.props[s];
  ContactOut o{d.scK + e * 144, d.scC + e * 144, d.scT + e * 12, d.scE + e};
  bool any = false;
  contact_element(in, g, cp, srf, o, &any);
  d.sc_on[e] = any ? 1 : 0;
}

void launch_beam(const Dev& d, const Gauss3& g, cudaStream_t s) {
  if (d.n_elem) k_beam<<<nblocks(d.n_elem, d.beam_threads), d.beam_threads, 0, s>>>(d, g);
}
void launch_contact(const Dev& d, const Gauss3& g, cudaStream_t s) {
  if (d.n_elem) k_contact<<<nblocks(d.n_elem, d.contact_threads), d.contact_threads, 0, s>>>(d, g);
}

// ------------------------------------------------------------------ ordered block assembly
// Thread per (block, entry): the reference's `nzval[global_sparsity_map] += vec(K)`
// (assemble_beams.jl:64-66, compute&assemble…:496-497) as a fixed-order sum over
// the contributions of each block, fused with the tangent
// Ktan = (1+α)K + γ/(βΔt) C + 1/(βΔt²) M (utils_solver.jl:83).
__global__ void k_gather_mat(Dev d, double alpha, int with_contact) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nnzb * 36) return;
  const int b = (int)(t / 36), k = (int)(t % 36);
  const int s = d.blk_sim[b];
  if (!d.active[s]) return;
  const int i = k % 6, j = k / 6;
  double Ks = 0.0, Cs = 0.0, Ms = 0.0;
  const int c0 = d.blk_cptr[b], c1 = d.blk_cptr[b + 1];
  for (int c = c0; c < c1; ++c) {
    const int v = d.blk_contrib[c];
    const int64_t e = v >> 2;
    const int I = v & 1, J = (v >> 1) & 1;
    const int64_t idx = e * 144 + (6 * J + j) * 12 + (6 * I + i);
    Ks += d.stK[idx];
    Cs += d.stC[idx];
    Ms += d.stM[idx];
  }
  if (with_contact) {
    const double ca = 1 + alpha;
    for (int c = c0; c < c1; ++c) {
      const int v = d.blk_contrib[c];
      const int64_t e = v >> 2;
      if (!d.sc_on[e]) continue;
      const int I = v & 1, J = (v >> 1) & 1;
      const int64_t idx = e * 144 + (6 * J + j) * 12 + (6 * I + i);
      Ks += -d.scK[idx];
      Cs += -(ca * d.scC[idx]);
    }
  }
  d.K1[t] = Ks;
  d.C1[t] = Cs;
  d.M1[t] = Ms;
  const double kt = (d.cK[s] * Ks + d.cC[s] * Cs) + d.cM[s] * Ms;
  d.Kt[t] = kt;
  d.Kt32[t] = (float)kt;
}

// Thread per (node, dof): Tⁱⁿᵗ, Tᵏ, Tᶜ as ordered sums over incident elements
// (assemble_beams.jl:60-61, compute&assemble…:493).
__global__ void k_gather_vec(Dev d, int with_contact) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  const int i = (int)(t / 6), k = (int)(t % 6);
  if (!d.active[d.node_sim[i]]) return;
  double Ti = 0.0, Tk = 0.0, Tc = 0.0;
  const int c0 = d.node_cptr[i], c1 = d.node_cptr[i + 1];
  for (int c = c0; c < c1; ++c) {
    const int v = d.node_contrib[c];
    const int64_t e = v >> 1;
    const int I = v & 1;
    Ti += d.stTi[e * 12 + 6 * I + k];
    Tk += d.stTk[e * 12 + 6 * I + k];
  }
  if (with_contact) {
    for (int c = c0; c < c1; ++c) {
      const int v = d.node_contrib[c];
      const int64_t e = v >> 1;
      if (!d.sc_on[e]) continue;
      Tc += d.scT[e * 12 + 6 * (v & 1) + k];
    }
  }
  d.Ti1[t] = Ti;
  d.Tk1[t] = Tk;
  d.Tc1[t] = Tc;
}

void launch_gather(const Dev& d, double alpha, bool with_contact, cudaStream_t s) {
  if (d.nnzb) k_gather_mat<<<nblocks(d.nnzb * 36, d.gmat_threads), d.gmat_threads, 0, s>>>(d, alpha, with_contact ? 1 : 0);
  if (d.n_dof) k_gather_vec<<<nblocks(d.n_dof, d.gvec_threads), d.gvec_threads, 0, s>>>(d, with_contact ? 1 : 0);
}

// ------------------------------------------------------------------ predictor
// initialize_global_predictor! (utils_solver.jl:30-48)
__global__ void k_init_predictor(Dev d) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  if (!d.active[d.node_sim[i]]) return;
  const int64_t n = d.n_nodes;
  V3 u = node3(d.u, n, i), ud = node3(d.ud, n, i), udd = node3(d.udd, n, i);
  V3 wd = node3(d.wd, n, i), wdd = node3(d.wdd, n, i);
  double* D = d.D + 6 * i;
  double* Dd = d.Dd + 6 * i;
  double* Ddd = d.Ddd + 6 * i;
  double* dD = d.dD + 6 * i;
  D[0] = u.x; D[1] = u.y; D[2] = u.z; D[3] = 0.0; D[4] = 0.0; D[5] = 0.0;
  Dd[0] = ud.x; Dd[1] = ud.y; Dd[2] = ud.z; Dd[3] = wd.x; Dd[4] = wd.y; Dd[5] = wd.z;
  Ddd[0] = udd.x; Ddd[1] = udd.y; Ddd[2] = udd.z; Ddd[3] = wdd.x; Ddd[4] = wdd.y; Ddd[5] = wdd.z;
#pragma unroll
  for (int k = 0; k < 6; ++k) dD[k] = 0.0;
}

// compute_tangent_and_residuals_predictor! (utils_solver.jl:54-74), thread per (node, dof):
// Ktan from the matrices at n, r = (1+α)fⁿ⁺¹ - Tⁱⁿᵗⁿ - Tᵏⁿ - αfⁿ + Cⁿ t₁ + Mⁿ t₂ /(βΔt²).
__global__ void k_predictor_rhs(Dev d, double alpha, double beta, double gamma) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  const int i = (int)(t / 6), k = (int)(t % 6);
  const int s = d.node_sim[i];
  if (!d.active[s]) return;
  const double dt = d.dt[s];
  const double cK = d.cK[s], cC = d.cC[s], cM = d.cM[s];
  const double a1 = gamma / beta, a2 = (dt / 2 * (2 * beta - gamma)) / beta;
  const double b2 = (dt * dt) / 2;
  double r = (((1 + alpha) * d.fext1[t] - d.Tin[t]) - d.Tkn[t]) - alpha * d.fextn[t];
  double cv = 0.0, mv = 0.0;
  for (int bb = d.row_ptr[i]; bb < d.row_ptr[i + 1]; ++bb) {
    const int c = d.col[bb];
    const double* Cb = d.Cn + (int64_t)bb * 36;
    const double* Mb = d.Mn + (int64_t)bb * 36;
    const double* Kb = d.Kn + (int64_t)bb * 36;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const double vd = d.Dd[6 * c + j], va = d.Ddd[6 * c + j];
      const double t1 = a1 * vd - a2 * va;
      const double t2 = dt * vd + b2 * va;
      cv += Cb[6 * j + k] * t1;
      mv += Mb[6 * j + k] * t2;
      const double kt = (cK * Kb[6 * j + k] + cC * Cb[6 * j + k]) + cM * Mb[6 * j + k];
      d.Kt[(int64_t)bb * 36 + 6 * j + k] = kt;
      d.Kt32[(int64_t)bb * 36 + 6 * j + k] = (float)kt;
    }
  }
  r = cv + r;
  r = cM * mv + r;
  d.r[t] = r;
}

void launch_init_predictor(const Dev& d, cudaStream_t s) {
  if (d.n_nodes) k_init_predictor<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d);
}
void launch_predictor_rhs(const Dev& d, double alpha, double beta, double gamma, cudaStream_t s) {
  if (d.n_dof) k_predictor_rhs<<<nblocks(d.n_dof, 256), 256, 0, s>>>(d, alpha, beta, gamma);
}

// compute_tangent_and_residuals_corrector! residual (utils_solver.jl:87)
__global__ void k_corrector_rhs(Dev d, double alpha) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  if (!d.active[d.node_sim[t / 6]]) return;
  d.r[t] = ((1 + alpha) * ((d.fext1[t] + d.Tc1[t]) - d.Ti1[t]) - alpha * ((d.fextn[t] + d.Tcn[t]) - d.Tin[t])) -
           d.Tk1[t];
}
void launch_corrector_rhs(const Dev& d, double alpha, cudaStream_t s) {
  if (d.n_dof) k_corrector_rhs<<<nblocks(d.n_dof, 256), 256, 0, s>>>(d, alpha);
}

// apply_boundary_conditions! (utils_bcs_and_loads.jl:5-29):
// ΔD[fixed] = imposed - D[fixed]; r -= Ktan[:, fixed] ΔD[fixed].
__global__ void k_bc_delta(Dev d) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  if (!d.fixed[t]) return;
  if (!d.active[d.node_sim[t / 6]]) return;
  d.dD[t] = d.imposed[t] - d.D[t];
}
__global__ void k_bc_lift(Dev d) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  const int i = (int)(t / 6), k = (int)(t % 6);
  const int s = d.node_sim[i];
  if (!d.active[s] || !d.has_fixed[s]) return;
  double acc = 0.0;
  for (int bb = d.row_ptr[i]; bb < d.row_ptr[i + 1]; ++bb) {
    const int c = d.col[bb];
#pragma unroll
    for (int j = 0; j < 6; ++j)
      if (d.fixed[6 * c + j]) acc += d.dD[6 * c + j] * d.Kt[(int64_t)bb * 36 + 6 * j + k];
  }
  d.r[t] -= acc;
}
void launch_apply_bc(const Dev& d, cudaStream_t s) {
  if (!d.n_dof) return;
  k_bc_delta<<<nblocks(d.n_dof, 256), 256, 0, s>>>(d);
  k_bc_lift<<<nblocks(d.n_dof, 256), 256, 0, s>>>(d);
}

// compute_global_predictor! (utils_solver.jl:157-172)
__global__ void k_global_predictor(Dev d, double beta, double gamma) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  const int s = d.node_sim[t / 6];
  if (!d.active[s]) return;
  const double dt = d.dt[s];
  const double g_bdt = gamma / (beta * dt), g_b = gamma / beta, inv = 1 / (beta * (dt * dt));
  const double dt2b = (dt * (2 * beta - gamma)) / (2 * beta);
  const double Ddn = d.Dd[t], dD = d.dD[t], Ddd = d.Ddd[t];
  d.D[t] += dD;
  d.Dd[t] += (g_bdt * dD - g_b * Ddn) + dt2b * Ddd;
  d.Ddd[t] += inv * ((dD - dt * Ddn) - ((dt * dt) / 2) * Ddd);
}
void launch_global_predictor(const Dev& d, double beta, double gamma, cudaStream_t s) {
  if (d.n_dof) k_global_predictor<<<nblocks(d.n_dof, 256), 256, 0, s>>>(d, beta, gamma);
}

// angular rates of utils_solver.jl:214-215 / :239-240
__device__ __forceinline__ void rates(const M3& dR, V3 w, V3 wdn, V3 wddn, double beta, double gamma, double dt,
                                      V3* wd, V3* wdd) {
  V3 a = (gamma / (beta * dt)) * w + ((beta - gamma) / beta) * wdn + ((dt * (beta - gamma / 2)) / beta) * wddn;
  V3 b = (1 / (beta * (dt * dt))) * w - (1 / (beta * dt)) * wdn - (1 / (2 * beta) - 1) * wddn;
  *wd = dR * a;
  *wdd = dR * b;
}

// compute_local_predictor! (utils_solver.jl:197-217)
__global__ void k_local_predictor(Dev d, double beta, double gamma) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  const int s = d.node_sim[i];
  if (!d.active[s]) return;
  const int64_t n = d.n_nodes;
  const double dt = d.dt[s];
  const double* D = d.D + 6 * i;
  const double* Dd = d.Dd + 6 * i;
  const double* Ddd = d.Ddd + 6 * i;
  store3(d.u, n, i, v3(D[0], D[1], D[2]));
  store3(d.ud, n, i, v3(Dd[0], Dd[1], Dd[2]));
  store3(d.udd, n, i, v3(Ddd[0], Ddd[1], Ddd[2]));
  V3 th = v3(D[3], D[4], D[5]);
  store3(d.w, n, i, th);
  M3 dR = rotation_matrix(th);
  store9(d.dR, n, i, dR);
  store9(d.R, n, i, dR * node9(d.Rn, n, i));
  V3 wd, wdd;
  rates(dR, th, node3(d.wdn, n, i), node3(d.wddn, n, i), beta, gamma, dt, &wd, &wdd);
  store3(d.wd, n, i, wd);
  store3(d.wdd, n, i, wdd);
}
void launch_local_predictor(const Dev& d, double beta, double gamma, cudaStream_t s) {
  if (d.n_nodes) k_local_predictor<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, beta, gamma);
}

// initialize_global_corrector! (utils_solver.jl:6-24)
__global__ void k_init_corrector(Dev d) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  if (!d.active[d.node_sim[i]]) return;
  const int64_t n = d.n_nodes;
  V3 u = node3(d.u, n, i), ud = node3(d.ud, n, i), udd = node3(d.udd, n, i);
  V3 w = node3(d.w, n, i), wd = node3(d.wd, n, i), wdd = node3(d.wdd, n, i);
  double* D = d.D + 6 * i;
  double* Dd = d.Dd + 6 * i;
  double* Ddd = d.Ddd + 6 * i;
  double* dD = d.dD + 6 * i;
  D[0] = u.x; D[1] = u.y; D[2] = u.z; D[3] = w.x; D[4] = w.y; D[5] = w.z;
  Dd[0] = ud.x; Dd[1] = ud.y; Dd[2] = ud.z; Dd[3] = wd.x; Dd[4] = wd.y; Dd[5] = wd.z;
  Ddd[0] = udd.x; Ddd[1] = udd.y; Ddd[2] = udd.z; Ddd[3] = wdd.x; Ddd[4] = wdd.y; Ddd[5] = wdd.z;
#pragma unroll
  for (int k = 0; k < 6; ++k) dD[k] = 0.0;
}
void launch_init_corrector(const Dev& d, cudaStream_t s) {
  if (d.n_nodes) k_init_corrector<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d);
}

// compute_global_corrector! (utils_solver.jl:178-190)
__global__ void k_global_corrector(Dev d) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  const int s = d.node_sim[t / 6];
  if (!d.active[s]) return;
  const double dD = d.dD[t];
  d.D[t] += dD;
  d.Dd[t] += d.cC[s] * dD;
  d.Ddd[t] += d.cM[s] * dD;
}
void launch_global_corrector(const Dev& d, cudaStream_t s) {
  if (d.n_dof) k_global_corrector<<<nblocks(d.n_dof, 256), 256, 0, s>>>(d);
}

// compute_local_corrector! (utils_solver.jl:224-245); node w is not written, as in the reference.
__global__ void k_local_corrector(Dev d, double beta, double gamma) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  const int s = d.node_sim[i];
  if (!d.active[s]) return;
  const int64_t n = d.n_nodes;
  const double dt = d.dt[s];
  const double* D = d.D + 6 * i;
  const double* Dd = d.Dd + 6 * i;
  const double* Ddd = d.Ddd + 6 * i;
  const double* dD = d.dD + 6 * i;
  store3(d.u, n, i, v3(D[0], D[1], D[2]));
  store3(d.ud, n, i, v3(Dd[0], Dd[1], Dd[2]));
  store3(d.udd, n, i, v3(Ddd[0], Ddd[1], Ddd[2]));
  M3 dR = rotation_matrix(v3(dD[3], dD[4], dD[5])) * node9(d.dR, n, i);
  V3 w1 = toangle(dR);
  V3 wd, wdd;
  rates(dR, w1, node3(d.wdn, n, i), node3(d.wddn, n, i), beta, gamma, dt, &wd, &wdd);
  store9(d.dR, n, i, dR);
  store3(d.wd, n, i, wd);
  store3(d.wdd, n, i, wdd);
  store9(d.R, n, i, dR * node9(d.Rn, n, i));
}
void launch_local_corrector(const Dev& d, double beta, double gamma, cudaStream_t s) {
  if (d.n_nodes) k_local_corrector<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, beta, gamma);
}

// ------------------------------------------------------------------ commit / rollback
// update_converged! (utils_solver.jl:252-275) when commit, else update_not_converged! (:282-305).
__global__ void k_commit_nodes(Dev d, const int* mask, int commit) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_nodes) return;
  if (!mask[d.node_sim[i]]) return;
  const int64_t n = d.n_nodes;
  double* a[8] = {d.u, d.ud, d.udd, d.w, d.wd, d.wdd, d.R, d.dR};
  double* b[8] = {d.un, d.udn, d.uddn, d.wn, d.wdn, d.wddn, d.Rn, d.dRn};
  const int nc[8] = {3, 3, 3, 3, 3, 3, 9, 9};
#pragma unroll
  for (int f = 0; f < 8; ++f)
    for (int k = 0; k < nc[f]; ++k) {
      if (commit) b[f][k * n + i] = a[f][k * n + i];
      else a[f][k * n + i] = b[f][k * n + i];
    }
}
__global__ void k_commit_dofs(Dev d, const int* mask, int commit) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n_dof) return;
  if (!mask[d.node_sim[t / 6]]) return;
  if (commit) {
    d.Tin[t] = d.Ti1[t]; d.Tkn[t] = d.Tk1[t]; d.Tcn[t] = d.Tc1[t]; d.fextn[t] = d.fext1[t];
  } else {
    d.Ti1[t] = d.Tin[t]; d.Tk1[t] = d.Tkn[t]; d.Tc1[t] = d.Tcn[t]; d.fext1[t] = d.fextn[t];
  }
}
__global__ void k_commit_blocks(Dev d, const int* mask, int commit) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nnzb * 36) return;
  if (!mask[d.blk_sim[t / 36]]) return;
  if (commit) {
    d.Kn[t] = d.K1[t]; d.Cn[t] = d.C1[t]; d.Mn[t] = d.M1[t];
  } else {
    d.K1[t] = d.Kn[t]; d.C1[t] = d.Cn[t]; d.M1[t] = d.Mn[t];
  }
}
void launch_commit(const Dev& d, const int* mask, bool commit, cudaStream_t s) {
  if (d.n_nodes) k_commit_nodes<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, mask, commit ? 1 : 0);
  if (d.n_dof) k_commit_dofs<<<nblocks(d.n_dof, 256), 256, 0, s>>>(d, mask, commit ? 1 : 0);
  if (d.nnzb) k_commit_blocks<<<nblocks(d.nnzb * 36, 256), 256, 0, s>>>(d, mask, commit ? 1 : 0);
}

void launch_restore_nodes(const Dev& d, const int* mask, cudaStream_t s) {
  if (d.n_nodes) k_commit_nodes<<<nblocks(d.n_nodes), kThreads, 0, s>>>(d, mask, 0);
}

}  // namespace eb
