// Internal data layout of an endobeams_gb300 handle (device side).
//
// All simulations of a handle live in one set of arenas, concatenated:
// nodes, elements, 6x6 blocks and DOFs of simulation s occupy the contiguous
// ranges [*_off[s], *_off[s+1]).  Node fields are structure-of-arrays,
// field component k of node i at [k * n_nodes + i]; DOF d of node i is
// 6 i + d (the reference's numbering, def_node_beam.jl:62-67, minus one).
//
// The global tangent is a block-sparse (BSR) matrix of 6x6 node-pair blocks,
// block values column-major (entry (i,j) at 6 j + i).  The pattern is the
// union of the elements' 12x12 footprints (sparse_matrices.jl:6-77),
// fixed for the whole run.  Element results are staged per element and
// summed into blocks by a precomputed, ordered contribution list: every sum
// has a fixed order, so assembly is bit-reproducible.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "eb_contact.cuh"

namespace eb {

using ebd::ContactProps;
using ebd::Gauss3;
using ebd::SurfaceDev;

struct Dev {
  int n_sims;
  int64_t n_nodes, n_elem, nnzb, n_dof;

  // ---- per simulation
  const int64_t* sim_node_off;  // n_sims+1
  const int64_t* sim_blk_off;   // n_sims+1
  int* active;                  // phase mask (predictor / Newton iteration)
  double* cK;                   // 1+α            (per sim, same for all)
  double* cC;                   // γ/(βΔt)
  double* cM;                   // 1/(βΔt²)
  double* dt;
  const SurfaceDev* surf;
  const ContactProps* props;
  const int* has_fixed;

  // ---- nodes
  const int* node_sim;
  const double* X0;
  double *u, *ud, *udd, *w, *wd, *wdd, *R, *dR;          // n+1
  double *un, *udn, *uddn, *wn, *wdn, *wddn, *Rn, *dRn;  // n

  // ---- elements
  const int* ea;
  const int* eb;
  const int* elem_sim;
  const double* l0;
  const double* Re0;   // [k * n_elem + e]
  const double* Kbar;  // [k * n_elem + e], k < 7
  const double* Jr;    // [k * n_elem + e], k < 3
  const double* Ar;
  const double* damp;
  const double* radius;
  const uint8_t* is_contact;  // element takes part in contact

  // ---- staging (element-major, 12x12 column-major per element)
  double *stK, *stC, *stM, *stTi, *stTk, *stE;
  double *scK, *scC, *scT, *scE;
  uint8_t* sc_on;

  // ---- block pattern and assembly plan
  const int* row_ptr;     // n_nodes+1 (global block ids)
  const int* col;         // nnzb (global node ids)
  const int* diag_blk;    // n_nodes: block id of (i,i)
  const int* blk_sim;     // nnzb: owning simulation
  const int* blk_cptr;    // nnzb+1
  const int* blk_contrib; // 4 e + (I + 2 J)
  const int* node_cptr;   // n_nodes+1
  const int* node_contrib;// 2 e + I
  double *K1, *C1, *M1, *Kn, *Cn, *Mn;  // nnzb * 36
  double* Kt;                           // tangent, FP64
  float* Kt32;                          // tangent, FP32 copy

  // ---- launch shapes (threads per block), chosen by eb_autotune among shapes whose
  // results are bitwise identical
  int beam_threads, contact_threads, gmat_threads, gvec_threads;

  // ---- DOF vectors (6 n_nodes)
  double *D, *Dd, *Ddd, *dD, *r, *fext1, *fextn, *Ti1, *Tin, *Tk1, *Tkn, *Tc1, *Tcn;
  uint8_t* fixed;    // dof is fixed
  double* imposed;   // imposed value on fixed dofs (dense, 0 elsewhere)
};

constexpr int kThreads = 128;
constexpr int kMaxElemThreads = 256;  // largest block of the element and contact kernels

inline unsigned nblocks(int64_t n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

// kernel launchers (eb_kernels.cu)
// Raises `func`'s dynamic shared-memory limit on the current device to at least `bytes` and
// never lowers it.  Handles stepped from several host threads launch the same kernel with
// different sizes; a limit set for one launch must not undercut another thread's launch.
cudaError_t raise_smem_limit(const void* func, size_t bytes);

void launch_beam(const Dev& d, const Gauss3& g, cudaStream_t s);
void launch_contact(const Dev& d, const Gauss3& g, cudaStream_t s);
void launch_gather(const Dev& d, double alpha, bool with_contact, cudaStream_t s);
void launch_init_predictor(const Dev& d, cudaStream_t s);
void launch_predictor_rhs(const Dev& d, double alpha, double beta, double gamma, cudaStream_t s);
void launch_corrector_rhs(const Dev& d, double alpha, cudaStream_t s);
void launch_apply_bc(const Dev& d, cudaStream_t s);
void launch_global_predictor(const Dev& d, double beta, double gamma, cudaStream_t s);
void launch_local_predictor(const Dev& d, double beta, double gamma, cudaStream_t s);
void launch_init_corrector(const Dev& d, cudaStream_t s);
void launch_global_corrector(const Dev& d, cudaStream_t s);
void launch_local_corrector(const Dev& d, double beta, double gamma, cudaStream_t s);
void launch_commit(const Dev& d, const int* mask, bool commit, cudaStream_t s);
// node state at n+1 <- node state at n (the node part of update_not_converged!)
void launch_restore_nodes(const Dev& d, const int* mask, cudaStream_t s);
// quadratic B-spline prefilter of a padded SDF coefficient grid (interior = samples), eb_testing.cu
void launch_sdf_prefilter(double* coef, int nx, int ny, int nz, cudaStream_t s);

}  // namespace eb
