/* endobeams_gb300 — C ABI of the GB300 (sm_103a) implementation of the
 * EndoBeams.jl per-Newton-iteration hot path.
 *
 * Conventions
 *   - Status: every entry point returns an int, 0 = EB_OK, negative = error;
 *     eb_last_error() gives the message of the last failure on this thread.
 *   - Ownership: host arrays are borrowed for the duration of the call and
 *     copied; device memory belongs to the handle and is freed by eb_destroy.
 *   - Indices are 0-based int64.  Node vectors are n x 3 row-major (node
 *     major); rotation matrices are n x 9, each 3x3 column-major.
 *   - Threads: one CUDA stream per handle; a handle is not thread-safe;
 *     different handles may be used from different threads.
 *   - Units follow the caller (the reference uses SI).
 *
 * Reference interfaces replaced (paths inside the EndoBeams.jl tree):
 *   eb_create      — NodesBeams/Beams/BeamsConfiguration/RigidInteraction
 *                    construction + setup_state_simulation + sparse_matrices_beams!
 *                    + initialize_state_simulation!  (src/beams/def_node_beam.jl:55,
 *                    src/beams/def_beam.jl:102, src/def_configurations.jl:15,
 *                    src/inizialization.jl:17-45, src/sparse_matrices.jl:80)
 *   eb_set_loads   — update_loads!            (src/utils_bcs_and_loads.jl:56-65)
 *   eb_set_imposed — update_boundary_conditions! (src/utils_bcs_and_loads.jl:42-49)
 *   eb_step        — solve_step_dynamics! = predictor! + corrector!
 *                    (src/solve_step_dynamics.jl:1-14, src/predictor.jl:1-27,
 *                    src/corrector.jl:1-59, with assemble! src/beams/assemble_beams.jl:1,
 *                    assemble_contact! src/interactions/compute&assemble_interactions_beams.jl:447
 *                    and the PARDISO solve src/linearsolvers.jl:2-28)
 *   eb_commit      — update_converged!        (src/utils_solver.jl:252-275)
 *   eb_rollback    — update_not_converged!    (src/utils_solver.jl:282-305)
 *   eb_get_state / eb_set_state — the NodeBeam fields u, u̇, ü, w, ẇ, ẅ, R, ΔR
 *                    (src/beams/def_node_beam.jl:6-48)
 *   eb_element_eval — compute_beams           (src/beams/compute_beams.jl:1-538)
 *   eb_contact_eval — compute_contact_beams   (src/interactions/compute&assemble_interactions_beams.jl:1-445)
 */
#ifndef ENDOBEAMS_GB300_H
#define ENDOBEAMS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EB_OK 0
#define EB_ERR_ARG (-1)
#define EB_ERR_CUDA (-2)
#define EB_ERR_NOMEM (-3)
#define EB_ERR_STATE (-4)
#define EB_ERR_IO (-5)

/* per-simulation status written by eb_step */
#define EB_SIM_OK 0
#define EB_SIM_NOT_CONVERGED 1     /* Newton reached max_iterations */
#define EB_SIM_NAN 2               /* non-finite residual or increment */
#define EB_SIM_KRYLOV_STAGNATED 3  /* linear solve missed its tolerance */
#define EB_SIM_WAIT_TIMEOUT 4      /* an asynchronous shared-memory copy did not complete within its wait limit */

/* linear solver precision */
#define EB_PREC_FP64 0          /* FP64 GMRES */
#define EB_PREC_MIXED 1         /* FP32 GMRES inside FP64 iterative refinement */

/* SimulationParams (src/def_params.jl:1-35), hot-path fields, plus solver knobs. */
typedef struct {
  double alpha, beta, gamma;              /* HHT parameters */
  double tolerance_residual;              /* Newton residual tolerance */
  double tolerance_displacement;          /* Newton ‖ΔD‖ tolerance */
  int32_t max_iterations;                 /* Newton iterations per step */
  double gauss_w[3], gauss_z[3];          /* 3-point Gauss rule (def_params.jl:31-33) */
  /* linear solver (replaces MKL PARDISO) */
  int32_t precision;                      /* EB_PREC_FP64 | EB_PREC_MIXED */
  int32_t krylov_restart;                 /* GMRES restart length m (<= 128) */
  int32_t krylov_max_iter;                /* total GMRES iterations per solve */
  double linear_tol;                      /* relative residual of each linear solve */
  double inner_tol;                       /* relative tolerance of the FP32 inner solve (mixed) */
  int32_t max_refinements;                /* FP64 refinement sweeps (mixed) */
  int32_t threads_per_sim;                /* CTA size of the per-simulation solver, 0 = auto */
  int32_t timing;                         /* 1: record per-phase CUDA-event times in eb_step */
  int32_t preconditioner;                 /* EB_PRECOND_* */
  int32_t refactor_its;                   /* band LU is reused until a solve needs more GMRES
                                             iterations than this or Δt changes (0: refactorise every solve) */
  int32_t stage_band;                     /* 1: the triangular solves stream band blocks into shared memory
                                             with bulk asynchronous copies (same arithmetic, same results);
                                             2: as 1, but the first block's wait expects 16 bytes that no copy
                                             delivers, so it runs out (tests EB_SIM_WAIT_TIMEOUT) */
  int32_t warm_start;                     /* EB_WS_OFF | EB_WS_LEARNED | EB_WS_LEARNED_X0 (need eb_ws_set_model) */
  int32_t use_graph;                      /* 1: each Newton iteration is one CUDA graph launch (captured once
                                             per handle and refactorisation variant); not with timing = 1,
                                             whose per-phase events need separate launches */
  int32_t forcing;                        /* EB_FORCING_FIXED: every solve to linear_tol;
                                             EB_FORCING_EW: inexact Newton, Eisenstat-Walker forcing terms */
  double forcing_max;                     /* EB_FORCING_EW: largest relative tolerance of a solve (also the
                                             predictor's); linear_tol is the smallest */
  int32_t refactor_policy;                /* EB_REFACTOR_THRESHOLD | EB_REFACTOR_COST (refactor_its stays a cap) */
  int32_t band_lu;                        /* EB_LU_FP32 | EB_LU_TENSOR */
  double refactor_cost;                   /* EB_REFACTOR_COST: GMRES iterations one band LU is worth, per
                                             DOF of half bandwidth (the LU does N b^2 work, an iteration N b) */
} eb_params;

/* Band LU engine */
#define EB_LU_FP32 0    /* FP32 on the CUDA cores */
#define EB_LU_TENSOR 1  /* panels in FP32, trailing updates on the tensor cores: operands split into three
                           BF16 parts, six BF16 products accumulated in FP32 (an FP32 product's rounding);
                           the FP32 engine where the band is too wide for its shared memory (b > ~590) */

/* When a simulation's band LU is refactorised (besides missing factors and a changed Δt) */
#define EB_REFACTOR_THRESHOLD 0  /* a solve needed more than refactor_its GMRES iterations */
#define EB_REFACTOR_COST 1       /* the GMRES iterations spent beyond those of the first solve after the
                                    factorisation, summed, reach refactor_cost * b (the LU's own cost in
                                    iterations): a rent-or-buy rule per simulation; when any simulation
                                    refactorises, those already half-way to their own limit join it */

/* Linear-solve tolerance per Newton iteration */
#define EB_FORCING_FIXED 0  /* linear_tol for every solve (the reference's direct solve, approximated) */
#define EB_FORCING_EW 1     /* η_k = 0.9 (‖F_k‖ / ‖F_k-1‖)², kept >= 0.9 η_k-1² when that exceeds 0.1,
                               clamped to [linear_tol, forcing_max]; forcing_max for a step's first
                               corrector solve and for the predictor (Eisenstat & Walker 1996, choice 2) */

/* Newton start of each step */
#define EB_WS_OFF 0      /* HHT predictor (predictor.jl:1-27) */
#define EB_WS_LEARNED_X0 2  /* the HHT predictor (predictor.jl:1-27) with the per-node MLP increment as the
                              initial guess of its linear solve (scaled by the α in [0, 1] minimising the
                              initial residual): the same Newton iterate to the linear tolerance, fewer GMRES
                              iterations when the guess is good */
#define EB_WS_LEARNED 1  /* per-node MLP increment; per simulation, the predictor again when the learned
                            start's residual exceeds the predictor's right-hand side; after k rejections
                            in a row a simulation uses the predictor for 2^(k-1) steps (at most 32)
                            before trying the network again */

/* GMRES preconditioner */
#define EB_PRECOND_BAND 0          /* FP32 band LU in reverse Cuthill-McKee order (block-Jacobi where it does not fit) */
#define EB_PRECOND_BLOCK_JACOBI 1  /* LU of each node's 6x6 diagonal block */

/* Interpolation of a voxel SDF */
#define EB_SDF_QUADRATIC 0  /* quadratic B-spline of the prefiltered samples, Reflect(OnCell()) ends
                               (Interpolations.jl as the reference uses it, def_interactions.jl:77) */
#define EB_SDF_TRILINEAR 1  /* trilinear interpolation of the samples themselves (8 taps, no prefilter;
                               gradient discontinuous across cell faces); needs >= 2 points per axis */

/* Surface kinds */
#define EB_SURFACE_NONE 0
#define EB_SURFACE_SPHERE 1  /* SphereSurface (src/interactions/def_interactions.jl:30-33) */
#define EB_SURFACE_SDF 2     /* DiscreteSignedDistanceField (def_interactions.jl:36-43,67-82) */
#define EB_SURFACE_PLANE 3   /* PlaneSurface (def_interactions.jl:24-27); the reference declares it without a
                                gap function: here gap = x[axis] - position - r, normal e_axis, the body on the
                                positive side (the sphere's convention, utils_compute_interactions_beams.jl:2-36) */

/* One simulation: the arrays of NodesBeams, Beams, BoundaryConditions, Loads and RigidInteraction. */
typedef struct {
  int64_t n_nodes, n_elem;
  const double *X0, *u, *ud, *udd, *w, *wd, *wdd; /* n x 3; NULL = zeros (X0 required) */
  const double *R;                                /* n x 9 column-major; NULL = identity */
  const int64_t *conn;                            /* n_elem x 2, 0-based node ids */
  const double *E, *nu, *rho, *radius, *damping;  /* n_elem each */
  const double *Re0;                              /* n_elem x 9 column-major; NULL = get_Rₑ⁰ */
  int64_t n_fixed;                                /* BoundaryConditions.fixed_dofs */
  const int64_t *fixed_dofs;                      /* 0-based, sorted ascending */
  int64_t n_loaded;                               /* ConcentratedForce.loaded_dofs */
  const int64_t *loaded_dofs;                     /* 0-based */
  const double *fext0;                            /* n_loaded values of force_function(0, dof) */
  /* contact (RigidInteraction) */
  int32_t surface;                                /* EB_SURFACE_* */
  double kn, mu, eps_t, eta_n;                    /* InteractionProperties (used fields) */
  int64_t n_contact_elems;                        /* BeamElementSurface; 0 with NULL list = all */
  const int64_t *contact_elems;
  double sphere_center[3], sphere_radius;
  int64_t sdf_dims[3];                            /* grid points nx, ny, nz */
  double sdf_origin[3], sdf_spacing[3];
  const double *sdf_values;                       /* nx*ny*nz, x fastest (VTK order) */
  int32_t sdf_inside;                             /* 1: use values as given, 0: negate (def_interactions.jl:71) */
  int32_t sdf_interp;                             /* EB_SDF_QUADRATIC (the reference's) | EB_SDF_TRILINEAR */
  int32_t plane_axis;                             /* PlaneSurface.axis: 0 x, 1 y, 2 z */
  double plane_position;                          /* PlaneSurface.position */
} eb_sim_desc;

typedef struct eb_handle eb_handle;

/* Solver statistics of the last eb_step, per simulation. */
typedef struct {
  int32_t newton_iterations;   /* k - 1 */
  int32_t krylov_iterations;   /* summed over the step's linear solves */
  int32_t refinements;         /* FP64 refinement sweeps (mixed precision) */
  int32_t status;              /* EB_SIM_* */
  double last_res_norm, last_dD_norm;
  double max_linear_rel_residual;  /* worst FP64 relative residual of the step's linear solves */
  int32_t warm_start_used;         /* 1: the step started from the learned increment */
  int32_t predictor_krylov_iterations; /* GMRES iterations of the step's predictor solve */
  double predictor_rhs_norm;       /* ‖r_free‖ of the HHT predictor's right-hand side (learned mode) */
  double start_res_norm;           /* ‖r_free‖ at the learned start (learned mode) */
} eb_sim_stats;

const char *eb_last_error(void);

int eb_default_params(eb_params *p);

int eb_create(const eb_params *p, int32_t n_sims, const eb_sim_desc *sims, eb_handle **out);
int eb_destroy(eb_handle *h);

/* fext at t^{n+1} for the sim's loaded dofs (values of force_function(t, dof)). */
int eb_set_loads(eb_handle *h, int32_t sim, const double *values);
/* imposed displacements for the sim's fixed dofs (n_fixed values; Encastre entries 0). */
int eb_set_imposed(eb_handle *h, int32_t sim, const double *values);
/* update_loads! for every simulation at once: the loaded-dof values of all
 * simulations concatenated in simulation order (one host-to-device copy). */
int eb_set_loads_all(eb_handle *h, const double *values);
/* Displacements u at n+1 of all simulations, concatenated in simulation order
 * (sum of n_nodes rows x 3), in one device-to-host transfer per component. */
int eb_get_displacements(eb_handle *h, double *u);

/* One HHT step (predictor + Newton corrector) for every simulation with
 * active[s] != 0 (active == NULL: all).  dt[s] per simulation.  k_out[s] is
 * the reference's return value of corrector! (iterations + 1); a step with
 * k_out[s] > max_iterations did not converge.  status_out may be NULL. */
int eb_step(eb_handle *h, const double *dt, const int32_t *active, int32_t *k_out, int32_t *status_out);

/* update_converged! / update_not_converged! for simulations with mask[s] != 0 (NULL: all). */
int eb_commit(eb_handle *h, const int32_t *mask);
int eb_rollback(eb_handle *h, const int32_t *mask);

/* Node state of one simulation at n+1 (any pointer may be NULL). */
int eb_get_state(eb_handle *h, int32_t sim, double *u, double *ud, double *udd, double *w, double *wd,
                 double *wdd, double *R, double *dR);
/* Node state at n (the last converged step). */
int eb_get_state_n(eb_handle *h, int32_t sim, double *u, double *ud, double *udd, double *w, double *wd,
                   double *wdd, double *R, double *dR);
/* Assigns one simulation's NodeBeam fields between steps (src/beams/def_node_beam.jl:6-48: the
 * reference's nodes are plain mutable records a script may change between steps): written
 * to both the committed state n and the working state n+1; NULL fields are left unchanged.
 * Layout as eb_get_state (n x 3, R and ΔR n x 9 column-major).  EB_ERR_STATE between eb_step
 * and eb_commit/eb_rollback. */
int eb_set_state(eb_handle *h, int32_t sim, const double *u, const double *ud, const double *udd, const double *w,
                 const double *wd, const double *wdd, const double *R, const double *dR);
/* Newton iteration cap per simulation (n_sims values; NULL: params.max_iterations for all).
 * The reference keeps max_iterations in each simulation's own SimulationParams
 * (src/def_params.jl:1-35, corrector.jl:15); a batch of simulations may differ in it. */
int eb_set_max_iterations(eb_handle *h, const int32_t *max_iterations);
/* Newton tolerances per simulation (n_sims values each; NULL: the params value for all) —
 * tolerance_residual / tolerance_displacement of each simulation's own SimulationParams
 * (src/def_params.jl:1-35), tested as in corrector.jl:15. */
int eb_set_tolerances(eb_handle *h, const double *tolerance_residual, const double *tolerance_displacement);
int eb_get_stats(eb_handle *h, eb_sim_stats *stats /* n_sims */);
/* Device memory the handle holds (bytes), and how many simulations use the band-LU preconditioner. */
int eb_get_memory(eb_handle *h, int64_t *device_bytes, int32_t *band_sims);
/* Assembled global vectors of one simulation at n+1 (6 n_nodes each; NULL to skip). */
int eb_get_forces(eb_handle *h, int32_t sim, double *Tint, double *Tk, double *Tc);

/* Launch-shape autotuner (no counterpart in the reference): times the element, contact and
 * assembly kernels on the current state at candidate block sizes (64/128/256 threads for the
 * element and contact kernels, 128/256/512 for the two assembly kernels) and keeps the fastest.
 * All candidates compute every value with the same operations in the same order, so results do
 * not depend on the choice.  Call between steps (after eb_commit / eb_rollback; EB_ERR_STATE
 * otherwise).  chosen (may be NULL) receives the four block sizes: element, contact, matrix
 * assembly, vector assembly. */
int eb_autotune(eb_handle *h, int32_t *chosen);
/* Sets the four block sizes directly (multiples of 32; at most 256 for the element and contact
 * kernels, 1024 for the assembly kernels). */
int eb_set_launch_shapes(eb_handle *h, const int32_t *shapes);

/* Signed distance field of a closed triangle mesh (no counterpart in the reference, whose SDFs
 * come precomputed from files, read_vtk_sdf; its vessel meshes are read by read_vtk_triangle_mesh,
 * src/IO/read_input_files.jl:81-152).  verts: n_vert x 3; tris: n_tri x 3, 0-based; grid point
 * (i, j, k) at origin + (i, j, k) * spacing, dims = (nx, ny, nz); out: nx*ny*nz values, x fastest
 * (VTK order).  |value| = distance to the nearest triangle; positive inside the mesh (generalized
 * winding number above 1/2, either orientation), negative outside: the convention of the
 * reference's SDF files for bodies inside the surface (DiscreteSignedDistanceField, inside = true). */
int eb_sdf_from_mesh(int64_t n_vert, const double *verts, int64_t n_tri, const int64_t *tris, const int64_t *dims,
                     const double *origin, const double *spacing, double *out);

/* ---- output (src/IO/visualization_beams.jl) ----
 * recompute_at_gausspts_beams! (visualization_beams.jl:122-162) of one simulation's current
 * state: points_per_beam (>= 2) points per element at z = range(-1, 1, length = points_per_beam),
 * point k = points_per_beam * e + i.  out (host) receives 11 * n_elem * points_per_beam doubles:
 * [x (3 per point) | displacement (3) | velocity (3) | strain (1 per point) | stress (1)]. */
#define EB_OUT_FIELDS 11
int eb_beam_output(eb_handle *h, int32_t sim, int32_t points_per_beam, double *out);
/* Asynchronous VTK output, replacing VTKDataBeams + write_VTK_beams (visualization_beams.jl:28-120).
 * dirs[n_sims]: output directory per simulation (NULL or "" = no output), created if missing;
 * existing files are overwritten, other files are left alone.  Each eb_vtk_write queues, for every
 * simulation with mask[s] != 0 (NULL: all) and a directory, beams_<counter[s]>.vtp (interpolated
 * beams: Stress, Strain, Displacement, Velocity; field data time = t[s], step = step[s]) and
 * beams_nodes_<counter[s]>.vtp (nodes: Displacement, In Contact, Contact Force, Contact Distance)
 * of the state at this point of the handle's stream, and returns; a writer thread writes them
 * (VTK XML PolyData, appended raw data).  eb_vtk_flush waits for the queued files and reports the
 * first write error (EB_ERR_IO); eb_vtk_close also writes each directory's simulation.pvd. */
int eb_vtk_open(eb_handle *h, const char *const *dirs, int32_t points_per_beam);
int eb_vtk_write(eb_handle *h, const int32_t *mask, const int32_t *counter, const int32_t *step, const double *t);
int eb_vtk_flush(eb_handle *h);
int eb_vtk_close(eb_handle *h);

/* Testing entry points: evaluate single elements on the device.
 * in:  n x 96 packed records (layout in the implementation notes), out: n x 458
 * (strain, kinetic, Tint[12], Tk[12], K[144], M[144], C[144]; 12x12 column-major). */
int eb_element_eval(int64_t n, const double *in, const double *gauss6, double *out);
/* Contact: surf = [kind(0 sphere,1 sdf,2 plane,3 trilinear sdf), cx, cy, cz, R, nx, ny, nz, x0, y0, z0, hx, hy, hz]
 * (plane: [2, axis, position, ...]);
 * values = SDF grid (x fastest) when kind = 1; props = [kn, mu, eps_t, eta_n];
 * out n x 301 (energy, Tc[12], Kc[144], Cc[144]); flags[n] = 1 if any Gauss point touched. */
int eb_contact_eval(int64_t n, const double *in, const double *gauss6, const double *props, const double *surf,
                    const double *values, double *out, int32_t *flags);

/* Contact evaluation that allocates no memory.  No counterpart in the
 * reference: it exists for callers that must not allocate device memory
 * during a call — hosts whose device memory is owned by their own pool
 * allocator (a Julia or PyTorch runtime that has reserved most of the GPU,
 * where a cudaMalloc behind its back fails or fragments its pool), and
 * real-time loops that forbid allocation after start-up.  Same arithmetic
 * and outputs as
 * eb_contact_eval, but every pointer named d_* is DEVICE memory supplied by
 * the caller (n x 96 inputs, the SDF grid, n x 301 outputs, n flags);
 * gauss6, props and surf are small host arrays as in eb_contact_eval.
 * The prefiltered SDF coefficients live in one fixed device array of
 * EB_NOALLOC_SDF_MAX_COEFS doubles (2.3 MB, held on every GPU that loads
 * the library until the process exits): grids with (nx+2)(ny+2)(nz+2)
 * above that (64^3 points), and grid dimensions that are not whole numbers
 * in range, are rejected with EB_ERR_ARG before anything is launched.  The
 * first call on a device (and the first after its context is re-created,
 * e.g. by cudaDeviceReset) looks up that array's device address; make that
 * first call before any stream capture.  All calls share the array and each
 * overwrites it: calls that overlap on the GPU (different streams, or
 * different host threads) race.
 * stream may be NULL (legacy default stream); the call is asynchronous. */
#define EB_NOALLOC_SDF_MAX_COEFS 287496
int eb_contact_eval_noalloc(int64_t n, const double *d_in, const double *gauss6, const double *props,
                            const double *surf, const double *d_sdf_values, double *d_out, int32_t *d_flags,
                            void *stream);

/* Tensor-core self-test (no reference counterpart): D (128 x N, row-major) = A (128 x 32) Bᵀ
 * (B: N x 32), both row-major FP32, on one CTA with the MMA, operand layout and tensor-memory
 * epilogue of the tensor-core band LU; split = 0 rounds A and B to BF16, split = 1 sums the
 * three BF16 products of their BF16 pairs, split = 2 the six products of their three-part BF16
 * splits (the band LU's arithmetic).  N is 64, 128 or 256. */
int eb_umma_selftest(const float *A, const float *B, int32_t N, int32_t split, float *D);

/* Measured FP64 FMA throughput of device 0 in TFLOP/s (independent FMA
 * chains on every SM, CUDA-event timed); the roofline denominator of the
 * FP64-bound element kernels.  No reference counterpart. */
int eb_fp64_peak(double *tflops);

/* Host only: the reverse Cuthill-McKee node order the band-LU preconditioner
 * uses (CSR adjacency, self loops ignored); pos[v] = position of node v,
 * *half_bandwidth = max |pos[v] - pos[w]| over edges.  No reference counterpart
 * (the reference hands the matrix to PARDISO, src/linearsolvers.jl:15-23). */
int eb_rcm_order(int64_t n, const int64_t *xadj, const int32_t *adjncy, int32_t *pos, int32_t *half_bandwidth);
/* Free and total memory of the current device (bytes), for sizing batches before create. */
int eb_device_memory(int64_t *free_bytes, int64_t *total_bytes);
/* Device count and name probe (for hosts that must check before create). */
int eb_device_info(int32_t *count, char *name, int32_t name_len);
/* Selects the CUDA device for handles created afterwards on this thread (no
 * reference counterpart: the reference has no device; one process per GPU). */
int eb_set_device(int32_t device);
/* The calling thread's current CUDA device (what a new host thread passes to
 * eb_set_device before it steps handles created on this one). */
int eb_get_device(int32_t *device);

/* Device timing on the handle's stream (CUDA events; no reference counterpart,
 * the reference's equivalent is TimerOutputs, src/corrector.jl:7-42).
 * eb_timer_start/stop bracket any sequence of calls; stop returns elapsed ms. */
int eb_timer_start(eb_handle *h);
int eb_timer_stop(eb_handle *h, double *ms);
/* Elapsed ms from `from`'s last eb_timer_start to `to`'s last eb_timer_stop: the
 * device span of handles stepped concurrently (one host thread each, their own
 * streams), measured between events of the two streams. */
int eb_timer_between(eb_handle *from, eb_handle *to, double *ms);
/* Per-phase device time (ms) and kernel-launch counts accumulated by eb_step
 * since the last reset (phases: EB_PHASE_*); needs eb_params.timing = 1 for
 * times, launch counts are always kept. */
#define EB_PHASE_PREDICTOR 0
#define EB_PHASE_BEAM 1
#define EB_PHASE_CONTACT 2
#define EB_PHASE_ASSEMBLY 3
#define EB_PHASE_RESIDUAL 4
#define EB_PHASE_PRECOND 5
#define EB_PHASE_KRYLOV 6
#define EB_PHASE_UPDATE 7
#define EB_NPHASES 8
int eb_get_phase_times(eb_handle *h, double *ms, int64_t *launches, int32_t reset);
/* The phase's device intervals since h's last eb_timer_start (eb_params.timing = 1), in ms
 * from ref's last eb_timer_start (ref may be h): `count` is the number of intervals, the
 * first min(count, cap) are written.  Merged over handles stepped concurrently, they give
 * the time during which any of them ran the phase. */
int eb_get_phase_intervals(eb_handle *h, eb_handle *ref, int32_t phase, double *start_ms, double *end_ms,
                           int64_t cap, int64_t *count);

/* ---------------------------------------------------------------- learned Newton warm start
 * No reference counterpart: the reference starts every Newton loop from the
 * HHT predictor (src/predictor.jl:1-27), which stays the fallback here.
 *
 * Per-node MLP: EB_WS_NIN normalised features -> 128 -> 128 -> EB_WS_NOUT,
 * SiLU activations, BF16 weights, FP32 activations and accumulation.
 * Parameter vector (EB_WS_NPARAMS floats): W1 [48 x 128] row-major, b1[128],
 * W2 [128 x 128], b2[128], W3 [128 x 6], b3[6]. */
#define EB_WS_NIN 48
#define EB_WS_NOUT 6
#define EB_WS_NPARAMS 23558
/* Standalone network kernels on host arrays (each call uploads, runs, downloads).
 * Loss = mean over rows and outputs of (y - T)^2; rows whose target is NaN add nothing. */
int eb_mlp_forward(const float *params, const float *X /* n x 48 */, int64_t n, float *Y /* n x 6 */);
int eb_mlp_loss_grad(const float *params, const float *X, const float *T /* n x 6 */, int64_t n, double *loss,
                     float *grad /* EB_WS_NPARAMS */);
/* Adam (0.9, 0.999, 1e-8) on shuffled minibatches (seeded order); params in/out. */
int eb_mlp_train(float *params, const float *X, const float *T, int64_t n, int32_t epochs, int32_t batch, float lr,
                 uint64_t seed, double *loss_per_epoch /* epochs, may be NULL */);
/* The network a batch uses when eb_params.warm_start = EB_WS_LEARNED, with its
 * normalisation: x = (f - in_shift) / in_scale over the EB_WS_NRAW raw features
 * f (inputs beyond them are 0), and for the 3 translations and 3 rotations of
 * node i:  ΔD_i = Δt Ḋ_i + Δt²/2 D̈_i + Δt² out_scale ⊙ y_i.  params NULL removes it. */
#define EB_WS_NRAW 39
int eb_ws_set_model(eb_handle *h, const float *params, const float *in_shift /* 48 */, const float *in_scale /* 48 */,
                    const float *out_scale /* 6 */);
/* Training-sample capture from the running solver: after each eb_step, eb_commit
 * stores for every node with (node + commits) % stride == 0 its raw features at
 * the step's start and the raw target (converged increment - Δt Ḋ - Δt²/2 D̈) / Δt²
 * (NaN for simulations outside the commit mask) in a device ring of `capacity`
 * samples.  capacity 0 stops capturing and frees the ring. */
int eb_ws_capture(eb_handle *h, int64_t capacity, int32_t stride);
/* Copies ring slots [first, first + n) to the host; *written = slots filled so far (<= capacity). */
int eb_ws_samples(eb_handle *h, int64_t first, int64_t n, float *features /* n x 39 */, float *targets /* n x 6 */,
                  int64_t *written);

#ifdef __cplusplus
}
#endif

#endif /* ENDOBEAMS_GB300_H */
