// Test infrastructure: the device element and contact arithmetic
// (endobeams.jl_gb300/csrc/eb_beam.cuh, eb_contact.cuh) compiled for the host,
// so the CPU test suite can hold the formulas to the oracle without a GPU.
// Same packed record layouts as the eb_element_eval / eb_contact_eval testing
// entry points.
#include <cstdint>

#include "../../endobeams.jl_gb300/csrc/eb_contact.cuh"

using namespace ebd;

namespace {
V3 P3(const double* p) { return v3(p[0], p[1], p[2]); }
M3 P9(const double* p) {
  M3 m;
  for (int k = 0; k < 9; ++k) m.a[k] = p[k];
  return m;
}
Gauss3 gauss(const double* g6) {
  Gauss3 g;
  for (int i = 0; i < 3; ++i) { g.w[i] = g6[i]; g.z[i] = g6[3 + i]; }
  return g;
}
}  // namespace

extern "C" void host_element_eval(int64_t n, const double* in, const double* gauss6, double* out) {
  const Gauss3 g = gauss(gauss6);
  for (int64_t e = 0; e < n; ++e) {
    const double* p = in + 96 * e;
    double* o = out + 458 * e;
    BeamIn b;
    b.X1 = P3(p + 0); b.X2 = P3(p + 3); b.u1 = P3(p + 6); b.u2 = P3(p + 9);
    b.R1 = P9(p + 12); b.R2 = P9(p + 21); b.dR1 = P9(p + 30); b.dR2 = P9(p + 39);
    b.ud1 = P3(p + 48); b.ud2 = P3(p + 51); b.wd1 = P3(p + 54); b.wd2 = P3(p + 57);
    b.udd1 = P3(p + 60); b.udd2 = P3(p + 63); b.wdd1 = P3(p + 66); b.wdd2 = P3(p + 69);
    b.l0 = p[72]; b.Re0 = P9(p + 73); b.Ku = p[82]; b.KT = P3(p + 83); b.KTT = P3(p + 86); b.Jr = P3(p + 89);
    b.Ar = p[92]; b.damping = p[93];
    BeamOut bo{o + 26, o + 170, o + 314, o + 2, o + 14, o + 0};
    beam_element(b, g, bo);
  }
}

// surf: [kind (0 sphere, 2 plane), cx|axis, cy|position, cz, R, ...]; the discrete SDF is
// covered by the GPU tests.
extern "C" void host_contact_eval(int64_t n, const double* in, const double* gauss6, const double* props,
                                  const double* surf, double* out) {
  const Gauss3 g = gauss(gauss6);
  const ContactProps cp{props[0], props[1], props[2], props[3]};
  SurfaceDev s{};
  s.kind = (int)surf[0];
  s.cx = surf[1]; s.cy = surf[2]; s.cz = surf[3]; s.R = surf[4];
  if (s.kind == 2) {
    s.axis = (int)surf[1];
    s.pos = surf[2];
  }
  for (int64_t e = 0; e < n; ++e) {
    const double* p = in + 96 * e;
    double* o = out + 301 * e;
    for (int k = 0; k < 301; ++k) o[k] = 0.0;
    ContactIn c;
    c.X1 = P3(p + 0); c.X2 = P3(p + 3); c.u1 = P3(p + 6); c.u2 = P3(p + 9);
    c.R1 = P9(p + 12); c.R2 = P9(p + 21); c.dR1 = P9(p + 30); c.dR2 = P9(p + 39);
    c.ud1 = P3(p + 48); c.ud2 = P3(p + 51); c.wd1 = P3(p + 54); c.wd2 = P3(p + 57);
    c.l0 = p[72]; c.Re0 = P9(p + 73); c.radius = p[94];
    ContactOut co{o + 13, o + 157, o + 1, o + 0};
    bool any = false;
    contact_element(c, g, cp, s, co, &any);
  }
}

// Voxel-SDF surfaces: surf[0] = 1 (quadratic B-spline, coef = prefiltered coefficients) or
// 3 (trilinear, coef = the samples), both in the padded (nx+2)(ny+2)(nz+2) layout.
extern "C" void host_contact_eval_grid(int64_t n, const double* in, const double* gauss6, const double* props,
                                       const double* surf, const double* coef, double* out) {
  const Gauss3 g = gauss(gauss6);
  const ContactProps cp{props[0], props[1], props[2], props[3]};
  SurfaceDev s{};
  s.kind = 1;
  s.interp = surf[0] == 3 ? 1 : 0;
  s.coef = coef;
  s.nx = (int)surf[5]; s.ny = (int)surf[6]; s.nz = (int)surf[7];
  s.x0 = surf[8]; s.y0 = surf[9]; s.z0 = surf[10];
  s.ihx = 1.0 / surf[11]; s.ihy = 1.0 / surf[12]; s.ihz = 1.0 / surf[13];
  s.xl = (s.nx - 1) * surf[11]; s.yl = (s.ny - 1) * surf[12]; s.zl = (s.nz - 1) * surf[13];
  for (int64_t e = 0; e < n; ++e) {
    const double* p = in + 96 * e;
    double* o = out + 301 * e;
    for (int k = 0; k < 301; ++k) o[k] = 0.0;
    ContactIn c;
    c.X1 = P3(p + 0); c.X2 = P3(p + 3); c.u1 = P3(p + 6); c.u2 = P3(p + 9);
    c.R1 = P9(p + 12); c.R2 = P9(p + 21); c.dR1 = P9(p + 30); c.dR2 = P9(p + 39);
    c.ud1 = P3(p + 48); c.ud2 = P3(p + 51); c.wd1 = P3(p + 54); c.wd2 = P3(p + 57);
    c.l0 = p[72]; c.Re0 = P9(p + 73); c.radius = p[94];
    ContactOut co{o + 13, o + 157, o + 1, o + 0};
    bool any = false;
    contact_element(c, g, cp, s, co, &any);
  }
}
