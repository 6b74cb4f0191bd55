// ORACLE — test infrastructure only (tests/, smoke() and bench.py's CPU
// baseline use it to check the device results).  Never linked into, or called by, the
// product library.
//
// Literal FP64 restatement of EndoBeams.jl's per-Newton-iteration hot path.
// Every function cites the reference file:line it restates.
#pragma once
#include "eb_oracle_math.hpp"

namespace orc {

// ---- rotation utilities (src/beams/utils_beams.jl) ----
M3 skew(const V3& v);                                    // utils_beams.jl:2-8
M3 rotation_matrix(const V3& th);                        // utils_beams.jl:11-32
V3 toangle(const M3& R);                                 // utils_beams.jl:90-104
M3 Ts_inv(const V3& th);                                 // utils_beams.jl:107-122
void compute_eta_mu(const V3& th, double* eta, double* mu);  // utils_beams.jl:180-198
M3 compute_Kh(const V3& th, const V3& Mbar, const M3& Tsinv, double eta, double mu);  // utils_beams.jl:201-215

struct LocalFrame {  // return tuple of local_Rₑ_and_aux, utils_beams.jl:35-87
  M3 Re;
  V3 r1, r3;  // ru₁ = -v₁', ru₂ = v₁'  (stored as vectors)
  double eta;
  M3 Gt1, Gt2, Gt3, Gt4, D3;
};
LocalFrame local_Re_and_aux(const V3& x1, const V3& x2, const M3& R1, const M3& R2, const V3& Re0E2, double ln);

// Packed per-element input record (doubles).  The same layout is used by the
// product's element-evaluation test entry point.
enum {
  EI_X1 = 0, EI_X2 = 3, EI_U1 = 6, EI_U2 = 9, EI_R1 = 12, EI_R2 = 21, EI_DR1 = 30, EI_DR2 = 39,
  EI_UD1 = 48, EI_UD2 = 51, EI_WD1 = 54, EI_WD2 = 57, EI_UDD1 = 60, EI_UDD2 = 63, EI_WDD1 = 66,
  EI_WDD2 = 69, EI_L0 = 72, EI_RE0 = 73, EI_KU = 82, EI_KT = 83, EI_KTT = 86, EI_JR = 89, EI_AR = 92,
  EI_DAMP = 93, EI_RADIUS = 94, EI_SIZE = 96
};
// Packed per-element beam output record.
enum { EO_ES = 0, EO_EK = 1, EO_TINT = 2, EO_TK = 14, EO_K = 26, EO_M = 170, EO_C = 314, EO_SIZE = 458 };
// Packed per-element contact output record.
enum { CO_E = 0, CO_TC = 1, CO_K = 13, CO_C = 157, CO_SIZE = 301 };

struct Gauss { int n; double w[3]; double z[3]; };  // def_params.jl:31-33

// compute_beams (src/beams/compute_beams.jl:1-538), exact=true, isdynamic=true.
void compute_beams(const double* in, const Gauss& g, double* out);

// ---- rigid surfaces (src/interactions/*) ----
struct Surface {
  int kind;            // 0 = SphereSurface, 1 = DiscreteSignedDistanceField (quadratic B-spline), 2 = PlaneSurface,
                       // 3 = voxel SDF interpolated trilinearly (coef = the padded samples, no prefilter)
  double center[3];    // sphere
  double radius;       // sphere
  int axis;            // plane: 0 x, 1 y, 2 z (PlaneSurface.axis)
  double position;     // plane: PlaneSurface.position along the axis
  const double* coef;  // SDF: prefiltered coefficients, (nx+2)*(ny+2)*(nz+2), x fastest
  int64_t nx, ny, nz;  // SDF grid points
  double x0[3];        // SDF origin (first grid point)
  double h[3];         // SDF spacing
};
struct ContactProps { double kn, mu, eps_t, eta_n; };  // def_interactions.jl:6-14 (used fields)

// compute_contact_beams (compute&assemble_interactions_beams.jl:1-445), exact=true.
void compute_contact_beams(const double* in, const Gauss& g, const ContactProps& cp, const Surface& s,
                           double* out);

// regularize_gap_penalty_beams / smoothstep_transition_beams
// (interactions_beams_regularization.jl:2-46)
void regularize_gap_penalty(double gap, double rb, double* p, double* dp, double* Pi);
void smoothstep_transition(double value, double pos, double rb, double* s, double* ds);

bool incontact(const V3& x, const Surface& s, double rb);                      // utils_compute…:23-36, 67-75; plane below
void contact_gap(const V3& x, const Surface& s, double rb, double* g, V3* dg, M3* d2g);  // utils_compute…:2-20, 50-64

// Quadratic B-spline SDF (Interpolations.jl 0.15.1, BSpline(Quadratic(Reflect(OnCell())))).
void sdf_prefilter(int64_t nx, int64_t ny, int64_t nz, const double* field, double* coef);
void sdf_eval(const Surface& s, const V3& x, double* val, V3* grad, M3* hess);

}  // namespace orc
