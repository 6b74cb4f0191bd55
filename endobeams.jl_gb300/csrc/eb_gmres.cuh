// Per-simulation GMRES solver interface (implementation in eb_gmres.cu).
#pragma once
#include "eb_band.cuh"

namespace eb {

struct SolverArgs {
  int n_sims;            // CTAs of this launch (one simulation each)
  const int* cta_sim;    // CTA -> simulation
  const int64_t* sim_node_off;
  const int* active;
  const int* row_ptr;
  const int* col;
  const double* Kt;
  const float* Kt32;
  const double* Dinv64;
  const float* Dinv32;
  const uint8_t* fixed;
  const double* b;       // right-hand side (Newton residual after the BC lift)
  double* dD;            // free components receive the solution
  const double* fext1;   // for the Newton norms
  const double* Tc1;
  const double* Tk1;
  double* X;             // n_dof work
  double* R64;           // n_dof work
  void* V;               // (m+1) n_dof Krylov basis (double or float)
  void* Z;               // m n_dof preconditioned basis z_j = M⁻¹ v_j (double or float), m n_s per simulation
  int m, max_iter, max_ref;
  double tol, inner_tol;
  double* norms;         // 5 per sim: |ΔD_free|², |r_free|², |f_free|², |f_fixed|², iterations of the solve
  int* its;              // per sim, accumulated
  int* refs;             // per sim, accumulated
  double* relres;        // per sim, max over the step
  int* status;           // per sim, max over the step
  BandDev band;          // band-LU preconditioner (bw[s] == 0: block-Jacobi for that sim)
  int x_in_smem;         // 1: the permuted solve vector lives in shared memory
  int max_n;             // largest simulation, in DOFs
  int stage_floats;      // > 0: band blocks staged in shared memory, floats per buffer (32 (b_max + 1))
  int stage_test_extra;  // > 0: the first forward block waits for bytes no copy delivers (tests the bounded wait)
  // inexact Newton: 0 fixed tolerance `tol`; 1 Eisenstat-Walker forcing term from this solve's
  // right-hand side norm and the previous corrector solve's (per simulation, on the device)
  int forcing;
  double forcing_max;
  double* prev_bnorm;    // per sim: right-hand side norm of the previous corrector solve (0: none this step)
  double* prev_eta;      // per sim: its forcing term
  const int* x0_on;      // per sim (may be null): 1 = dD holds an initial guess x0 for this solve; GMRES
                         // starts from α x0 with α in [0, 1] minimising ‖b − α A x0‖
};

void launch_block_jacobi(const Dev& d, double* Dinv64, float* Dinv32, cudaStream_t s);
cudaError_t launch_gmres(const SolverArgs& a, bool fp32, int threads, cudaStream_t s);
size_t gmres_smem(int m);
size_t gmres_smem_total(const SolverArgs& a);  // dynamic shared memory of one launch
constexpr size_t kGmresSmemLimit = 216 * 1024;  // leaves room for the kernel's static shared memory (ring, barriers)
// Dynamic shared memory up to which two CTAs share an SM (228 KB per SM, minus the kernel's
// static 4.4 KB and the 1 KB the hardware reserves, per CTA; 256 threads x 128 registers
// also allow exactly two).
constexpr size_t kGmresTwoPerSm = 108 * 1024;

}  // namespace eb
