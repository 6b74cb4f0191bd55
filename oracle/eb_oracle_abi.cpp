// ORACLE — test infrastructure only.  C ABI of the CPU restatement, loaded
// by oracle/oracle.py through ctypes.  Array conventions: node vectors are
// n x 3 row-major (node-major), rotation matrices n x 9 column-major per
// node, indices 0-based int64.
#include <cstring>

#include "eb_oracle.hpp"

using namespace orc;

namespace {

Surface make_surface(const double* s, const double* coef) {
  // s = [kind, cx, cy, cz, R, nx, ny, nz, x0, y0, z0, hx, hy, hz]; plane (kind 2): [2, axis, position, ...]
  Surface f;
  f.kind = (int)s[0];
  f.axis = f.kind == 2 ? (int)s[1] : 0;
  f.position = f.kind == 2 ? s[2] : 0.0;
  f.center[0] = s[1]; f.center[1] = s[2]; f.center[2] = s[3];
  f.radius = s[4];
  f.nx = (int64_t)s[5]; f.ny = (int64_t)s[6]; f.nz = (int64_t)s[7];
  f.x0[0] = s[8]; f.x0[1] = s[9]; f.x0[2] = s[10];
  f.h[0] = s[11]; f.h[1] = s[12]; f.h[2] = s[13];
  f.coef = coef;
  return f;
}

Gauss make_gauss(const double* g) {
  Gauss q;
  q.n = 3;
  for (int i = 0; i < 3; ++i) { q.w[i] = g[i]; q.z[i] = g[3 + i]; }
  return q;
}

struct NodeArrays {
  const double *X0, *u, *ud, *udd, *wd, *wdd, *R, *dR;
};

// Gathers the packed element record of assemble_beams.jl:24-39 (and the
// contact equivalent, compute&assemble…:466-479).
void gather(const NodeArrays& na, int64_t a, int64_t b, const double* l0, const double* Re0, const double* Kbar,
            const double* Jr, const double* Ar, const double* damp, const double* radius, int64_t e, double* in) {
  std::memset(in, 0, sizeof(double) * EI_SIZE);
  std::memcpy(in + EI_X1, na.X0 + 3 * a, 24); std::memcpy(in + EI_X2, na.X0 + 3 * b, 24);
  std::memcpy(in + EI_U1, na.u + 3 * a, 24);  std::memcpy(in + EI_U2, na.u + 3 * b, 24);
  std::memcpy(in + EI_R1, na.R + 9 * a, 72);  std::memcpy(in + EI_R2, na.R + 9 * b, 72);
  std::memcpy(in + EI_DR1, na.dR + 9 * a, 72); std::memcpy(in + EI_DR2, na.dR + 9 * b, 72);
  std::memcpy(in + EI_UD1, na.ud + 3 * a, 24); std::memcpy(in + EI_UD2, na.ud + 3 * b, 24);
  std::memcpy(in + EI_WD1, na.wd + 3 * a, 24); std::memcpy(in + EI_WD2, na.wd + 3 * b, 24);
  if (na.udd) { std::memcpy(in + EI_UDD1, na.udd + 3 * a, 24); std::memcpy(in + EI_UDD2, na.udd + 3 * b, 24); }
  if (na.wdd) { std::memcpy(in + EI_WDD1, na.wdd + 3 * a, 24); std::memcpy(in + EI_WDD2, na.wdd + 3 * b, 24); }
  in[EI_L0] = l0[e];
  std::memcpy(in + EI_RE0, Re0 + 9 * e, 72);
  if (Kbar) { in[EI_KU] = Kbar[7 * e]; std::memcpy(in + EI_KT, Kbar + 7 * e + 1, 48); }
  if (Jr) std::memcpy(in + EI_JR, Jr + 3 * e, 24);
  if (Ar) in[EI_AR] = Ar[e];
  if (damp) in[EI_DAMP] = damp[e];
  if (radius) in[EI_RADIUS] = radius[e];
}

}  // namespace

extern "C" {

void orc_compute_beams_batch(int64_t n, const double* in, const double* gauss, double* out) {
  Gauss g = make_gauss(gauss);
  for (int64_t e = 0; e < n; ++e) compute_beams(in + EI_SIZE * e, g, out + EO_SIZE * e);
}

void orc_compute_contact_batch(int64_t n, const double* in, const double* gauss, const double* props,
                               const double* surf, const double* coef, double* out) {
  Gauss g = make_gauss(gauss);
  ContactProps cp{props[0], props[1], props[2], props[3]};
  Surface s = make_surface(surf, coef);
  for (int64_t e = 0; e < n; ++e) compute_contact_beams(in + EI_SIZE * e, g, cp, s, out + CO_SIZE * e);
}

void orc_sdf_prefilter(int64_t nx, int64_t ny, int64_t nz, const double* field, double* coef) {
  sdf_prefilter(nx, ny, nz, field, coef);
}

// out per point: [value, grad(3), hess(9, column-major), incontact(radius)]
void orc_sdf_eval_batch(const double* surf, const double* coef, int64_t n, const double* pts, double radius,
                        double* out) {
  Surface s = make_surface(surf, coef);
  for (int64_t i = 0; i < n; ++i) {
    V3 x = v3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    double v;
    V3 g;
    M3 h;
    sdf_eval(s, x, &v, &g, &h);
    double* o = out + 14 * i;
    o[0] = v;
    for (int k = 0; k < 3; ++k) o[1 + k] = g[k];
    for (int k = 0; k < 9; ++k) o[4 + k] = h.a[k];
    o[13] = incontact(x, s, radius) ? 1.0 : 0.0;
  }
}

// assemble! (assemble_beams.jl:1-70) followed, when n_contact > 0, by
// assemble_contact! (compute&assemble_interactions_beams.jl:447-501).
// Serial loop in element order: the deterministic version of the reference's
// (racy) threaded loop.  Outputs are zeroed first, like assemble_beams.jl:4-11.
void orc_assemble(int64_t n_nodes, int64_t n_elem, const double* X0, const double* u, const double* ud,
                  const double* udd, const double* wd, const double* wdd, const double* R, const double* dR,
                  const int64_t* conn, const double* l0, const double* Re0, const double* Kbar, const double* Jr,
                  const double* Ar, const double* damp, const double* radius, const double* gauss,
                  const int64_t* spmap, int64_t nnz, double* Knz, double* Cnz, double* Mnz, double* Tint,
                  double* Tk, double* Tc, double* energies, int64_t n_contact, const int64_t* contact_elems,
                  const double* props, double alpha, const double* surf, const double* coef) {
  Gauss g = make_gauss(gauss);
  NodeArrays na{X0, u, ud, udd, wd, wdd, R, dR};
  std::memset(Knz, 0, sizeof(double) * nnz);
  std::memset(Cnz, 0, sizeof(double) * nnz);
  std::memset(Mnz, 0, sizeof(double) * nnz);
  std::memset(Tint, 0, sizeof(double) * 6 * n_nodes);
  std::memset(Tk, 0, sizeof(double) * 6 * n_nodes);
  std::memset(Tc, 0, sizeof(double) * 6 * n_nodes);
  double in[EI_SIZE], out[EO_SIZE];
  double es = 0, ek = 0, ec = 0;
  for (int64_t e = 0; e < n_elem; ++e) {
    int64_t a = conn[2 * e], b = conn[2 * e + 1];
    gather(na, a, b, l0, Re0, Kbar, Jr, Ar, damp, radius, e, in);
    compute_beams(in, g, out);
    es += out[EO_ES];
    ek += out[EO_EK];
    for (int k = 0; k < 6; ++k) {
      Tk[6 * a + k] += out[EO_TK + k];
      Tk[6 * b + k] += out[EO_TK + 6 + k];
      Tint[6 * a + k] += out[EO_TINT + k];
      Tint[6 * b + k] += out[EO_TINT + 6 + k];
    }
    const int64_t* m = spmap + 144 * e;
    for (int k = 0; k < 144; ++k) {
      Knz[m[k]] += out[EO_K + k];
      Cnz[m[k]] += out[EO_C + k];
      Mnz[m[k]] += out[EO_M + k];
    }
  }
  if (n_contact > 0) {
    ContactProps cp{props[0], props[1], props[2], props[3]};
    Surface s = make_surface(surf, coef);
    double co[CO_SIZE];
    for (int64_t c = 0; c < n_contact; ++c) {
      int64_t e = contact_elems[c];
      int64_t a = conn[2 * e], b = conn[2 * e + 1];
      gather(na, a, b, l0, Re0, nullptr, nullptr, nullptr, nullptr, radius, e, in);
      compute_contact_beams(in, g, cp, s, co);
      ec += co[CO_E];
      for (int k = 0; k < 6; ++k) {
        Tc[6 * a + k] += co[CO_TC + k];
        Tc[6 * b + k] += co[CO_TC + 6 + k];
      }
      const int64_t* m = spmap + 144 * e;
      for (int k = 0; k < 144; ++k) {
        Knz[m[k]] += -co[CO_K + k];
        Cnz[m[k]] += -(1 + alpha) * co[CO_C + k];
      }
    }
  }
  energies[0] = es;
  energies[1] = ek;
  energies[2] = ec;
}

// recompute_at_gausspts_beams! (src/IO/visualization_beams.jl:122-162): per element,
// `pts` points at z = range(-1, 1, length = pts) along the beam, interpolated with the
// linear (axial) and cubic (bending, in the local frame) shape functions.  Output
// block of NP = n_elem * pts points: [x (3 NP) | displacement (3 NP) | velocity (3 NP) |
// strain (NP) | stress (NP)], point k = pts * e + i.
void orc_beam_output(int64_t n_elem, const double* X0, const double* u, const double* ud, const double* R,
                     const int64_t* conn, const double* l0v, const double* Re0v, const double* E, int32_t pts,
                     double* out) {
  const int64_t NP = n_elem * pts;
  double *ox = out, *od = out + 3 * NP, *ov = out + 6 * NP, *oe = out + 9 * NP, *os = out + 10 * NP;
  for (int64_t e = 0; e < n_elem; ++e) {
    const int64_t a = conn[2 * e], b = conn[2 * e + 1];
    V3 X1 = v3(X0[3 * a], X0[3 * a + 1], X0[3 * a + 2]), X2 = v3(X0[3 * b], X0[3 * b + 1], X0[3 * b + 2]);
    V3 u1 = v3(u[3 * a], u[3 * a + 1], u[3 * a + 2]), u2 = v3(u[3 * b], u[3 * b + 1], u[3 * b + 2]);
    V3 v1 = v3(ud[3 * a], ud[3 * a + 1], ud[3 * a + 2]), v2 = v3(ud[3 * b], ud[3 * b + 1], ud[3 * b + 2]);
    M3 R1, R2, Re0;
    for (int k = 0; k < 9; ++k) { R1.a[k] = R[9 * a + k]; R2.a[k] = R[9 * b + k]; Re0.a[k] = Re0v[9 * e + k]; }
    const double l0 = l0v[e];
    V3 x1 = X1 + u1, x2 = X2 + u2;
    const double ln = norm(x2 - x1);
    LocalFrame f = local_Re_and_aux(x1, x2, R1, R2, col(Re0, 1), ln);
    V3 T1 = toangle((tr(f.Re) * R1) * Re0);
    V3 T2 = toangle((tr(f.Re) * R2) * Re0);
    for (int i = 0; i < pts; ++i) {
      const int64_t k = (int64_t)pts * e + i;
      const double z = (2.0 * i - (pts - 1)) / (double)(pts - 1);
      const double xi = l0 * (z + 1) / 2;
      const double N1 = 1 - xi / l0, N2 = 1 - N1;
      const double N3 = xi * ((1 - xi / l0) * (1 - xi / l0));
      const double N4 = -(1 - xi / l0) * ((xi * xi) / l0);
      V3 ut = v3(0.0, N3 * T1[2] + N4 * T2[2], -N3 * T1[1] - N4 * T2[1]);
      V3 xg = (N1 * x1 + N2 * x2) + f.Re * ut;
      V3 dg = N1 * u1 + N2 * u2;
      V3 vg = N1 * v1 + N2 * v2;
      for (int c = 0; c < 3; ++c) { ox[3 * k + c] = xg[c]; od[3 * k + c] = dg[c]; ov[3 * k + c] = vg[c]; }
      oe[k] = 1 - ln / l0;
      os[k] = E[e] * (1 - ln / l0);
    }
  }
}

// compute_local_predictor! (utils_solver.jl:197-217).  D, Dd, Ddd are the
// global 6n vectors; node arrays are updated in place.
void orc_local_predictor(int64_t n, const double* D, const double* Dd, const double* Ddd, double* u, double* ud,
                         double* udd, double* w, double* wd, double* wdd, double* R, double* dR, const double* Rn,
                         const double* wdn, const double* wddn, double gamma, double beta, double dt) {
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      u[3 * i + k] = D[6 * i + k];
      ud[3 * i + k] = Dd[6 * i + k];
      udd[3 * i + k] = Ddd[6 * i + k];
    }
    V3 th = v3(D[6 * i + 3], D[6 * i + 4], D[6 * i + 5]);
    for (int k = 0; k < 3; ++k) w[3 * i + k] = th[k];
    M3 dRi = rotation_matrix(th);
    M3 Rni;
    std::memcpy(Rni.a, Rn + 9 * i, 72);
    M3 Ri = dRi * Rni;
    V3 wdni = v3(wdn[3 * i], wdn[3 * i + 1], wdn[3 * i + 2]);
    V3 wddni = v3(wddn[3 * i], wddn[3 * i + 1], wddn[3 * i + 2]);
    V3 wdi = dRi * (((gamma / (beta * dt)) * th + ((beta - gamma) / beta) * wdni) + ((dt * (beta - gamma / 2)) / beta) * wddni);
    V3 wddi = dRi * (((1 / (beta * (dt * dt))) * th - (1 / (beta * dt)) * wdni) - (1 / (2 * beta) - 1) * wddni);
    std::memcpy(dR + 9 * i, dRi.a, 72);
    std::memcpy(R + 9 * i, Ri.a, 72);
    for (int k = 0; k < 3; ++k) {
      wd[3 * i + k] = wdi[k];
      wdd[3 * i + k] = wddi[k];
    }
  }
}

// compute_local_corrector! (utils_solver.jl:224-245).  Node `w` is not
// written by the reference here.
void orc_local_corrector(int64_t n, const double* D, const double* Dd, const double* Ddd, const double* dD,
                         double* u, double* ud, double* udd, double* wd, double* wdd, double* R, double* dR,
                         const double* Rn, const double* wdn, const double* wddn, double gamma, double beta,
                         double dt) {
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      u[3 * i + k] = D[6 * i + k];
      ud[3 * i + k] = Dd[6 * i + k];
      udd[3 * i + k] = Ddd[6 * i + k];
    }
    M3 dRi;
    std::memcpy(dRi.a, dR + 9 * i, 72);
    dRi = rotation_matrix(v3(dD[6 * i + 3], dD[6 * i + 4], dD[6 * i + 5])) * dRi;
    V3 wdni = v3(wdn[3 * i], wdn[3 * i + 1], wdn[3 * i + 2]);
    V3 wddni = v3(wddn[3 * i], wddn[3 * i + 1], wddn[3 * i + 2]);
    V3 wn1 = toangle(dRi);
    V3 wdi = dRi * (((gamma / (beta * dt)) * wn1 + ((beta - gamma) / beta) * wdni) + ((dt * (beta - gamma / 2)) / beta) * wddni);
    V3 wddi = dRi * (((1 / (beta * (dt * dt))) * wn1 - (1 / (beta * dt)) * wdni) - (1 / (2 * beta) - 1) * wddni);
    M3 Rni;
    std::memcpy(Rni.a, Rn + 9 * i, 72);
    M3 Ri = dRi * Rni;
    std::memcpy(dR + 9 * i, dRi.a, 72);
    std::memcpy(R + 9 * i, Ri.a, 72);
    for (int k = 0; k < 3; ++k) {
      wd[3 * i + k] = wdi[k];
      wdd[3 * i + k] = wddi[k];
    }
  }
}

}  // extern "C"
