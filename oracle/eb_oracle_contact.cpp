// ORACLE — test infrastructure only.  CPU FP64 restatement of EndoBeams.jl's
// beam-to-rigid-surface contact (src/interactions/*), statement by statement.
//
// Reference quirk kept on purpose: inside the Gauss loop of
// compute_contact_beams (compute&assemble_interactions_beams.jl:100) the
// line `ηₙ, η′ₙ = smoothstep_transition_beams(ηₙ, gₙ, radius_beam)` rebinds
// the function-level local ηₙ (Julia scoping), so each in-contact Gauss point
// smooths the damping left over by the previous one.
//
// The discrete SDF follows Interpolations.jl 0.15.1 (not vendored in the
// reference; its call sites are def_interactions.jl:77-78 and
// utils_compute_interactions_beams.jl:53-55,73): quadratic B-spline,
// `Reflect(OnCell())` boundary, prefiltered so the spline interpolates the
// grid values.  Restated from the published method: per axis, the cardinal
// quadratic B-spline has weights ½(½−δ)², ¾−δ², ½(½+δ)² at offsets −1,0,+1
// from the nearest grid point, and interpolation requires
// ⅛c[i−1] + ¾c[i] + ⅛c[i+1] = y[i]; the even reflection about the cell
// edge half a spacing outside the first/last point gives c[0]=c[1] and
// c[n+1]=c[n].
#include <algorithm>
#include <vector>

#include "eb_oracle.hpp"

namespace orc {

void regularize_gap_penalty(double gap, double rb, double* p, double* dp, double* Pi) {
  // interactions_beams_regularization.jl:2-26
  double gt = rb / 4;
  double hg = gt / 2;
  if (gap <= 0) {
    *p = hg - gap;
    *dp = -1.0;
    *Pi = (gap * gap) / 2 - hg * gap + (gt * gt) / 6;
  } else {
    double aux = (gt - hg) / (gt * gt);
    *p = aux * (gap * gap) - gap + hg;
    *dp = 2 * aux * gap - 1;
    *Pi = (gt - hg) / (3 * (gt * gt)) * (gap * gap * gap) - (gap * gap) / 2 + hg * gap - (gt * gt) / 6;
  }
}

void smoothstep_transition(double value, double pos, double rb, double* s, double* ds) {
  // interactions_beams_regularization.jl:29-46
  double ul = rb / 4;
  if (pos <= 0) {
    *s = value;
    *ds = 0.0;
  } else {
    double np = (pos - ul) / ul;
    *s = np * np * (3 + 2 * np) * value;
    *ds = 6 / ul * np * (1 + np) * value;
  }
}

// ---------------- quadratic B-spline SDF ----------------

static void prefilter_line(int64_t n, double* y, int64_t stride, std::vector<double>& cp, std::vector<double>& dp) {
  // Thomas algorithm on the reduced (c[0]=c[1], c[n+1]=c[n]) interpolation system.
  if (n == 1) return;  // single point: c = y
  cp.resize(n);
  dp.resize(n);
  const double lo = 1.0 / 8.0, mid = 3.0 / 4.0, edge = 7.0 / 8.0;
  double b0 = edge;
  cp[0] = lo / b0;
  dp[0] = y[0] / b0;
  for (int64_t i = 1; i < n; ++i) {
    double bi = (i == n - 1) ? edge : mid;
    double ci = (i == n - 1) ? 0.0 : lo;
    double m = bi - lo * cp[i - 1];
    cp[i] = ci / m;
    dp[i] = (y[i * stride] - lo * dp[i - 1]) / m;
  }
  y[(n - 1) * stride] = dp[n - 1];
  for (int64_t i = n - 2; i >= 0; --i) y[i * stride] = dp[i] - cp[i] * y[(i + 1) * stride];
}

void sdf_prefilter(int64_t nx, int64_t ny, int64_t nz, const double* field, double* coef) {
  const int64_t px = nx + 2, py = ny + 2, pz = nz + 2;
  auto at = [&](int64_t i, int64_t j, int64_t k) -> double& { return coef[i + px * (j + py * k)]; };
  for (int64_t k = 0; k < pz; ++k)
    for (int64_t j = 0; j < py; ++j)
      for (int64_t i = 0; i < px; ++i) at(i, j, k) = 0.0;
  for (int64_t k = 0; k < nz; ++k)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t i = 0; i < nx; ++i) at(i + 1, j + 1, k + 1) = field[i + nx * (j + ny * k)];
  std::vector<double> cp, dp;
  // axis x, then y, then z; each pass covers the already-padded extent of earlier axes
  for (int64_t k = 1; k <= nz; ++k)
    for (int64_t j = 1; j <= ny; ++j) {
      prefilter_line(nx, &at(1, j, k), 1, cp, dp);
      at(0, j, k) = at(1, j, k);
      at(nx + 1, j, k) = at(nx, j, k);
    }
  for (int64_t k = 1; k <= nz; ++k)
    for (int64_t i = 0; i < px; ++i) {
      prefilter_line(ny, &at(i, 1, k), px, cp, dp);
      at(i, 0, k) = at(i, 1, k);
      at(i, ny + 1, k) = at(i, ny, k);
    }
  for (int64_t j = 0; j < py; ++j)
    for (int64_t i = 0; i < px; ++i) {
      prefilter_line(nz, &at(i, j, 1), px * py, cp, dp);
      at(i, j, 0) = at(i, j, 1);
      at(i, j, nz + 1) = at(i, j, nz);
    }
}

static void bweights(double t, int64_t n, int64_t* ix, double w[3], double d[3], double dd[3]) {
  int64_t i = (int64_t)std::floor(t + 0.5);
  if (i < 0) i = 0;
  if (i > n - 1) i = n - 1;
  double del = t - (double)i;
  *ix = i;
  w[0] = 0.5 * ((0.5 - del) * (0.5 - del));
  w[1] = 0.75 - del * del;
  w[2] = 0.5 * ((0.5 + del) * (0.5 + del));
  d[0] = del - 0.5;
  d[1] = -2 * del;
  d[2] = del + 0.5;
  dd[0] = 1.0;
  dd[1] = -2.0;
  dd[2] = 1.0;
}

// Trilinear interpolation of the samples (surface kind 3; sample (i,j,k) at padded (i+1,j+1,k+1)):
// in the cell [i, i+1] x [j, j+1] x [k, k+1] that holds x (cells clamped to the grid), the
// polynomial Σ w_a(fx) w_b(fy) w_c(fz) q_abc with w_0(f) = 1 - f, w_1(f) = f; its gradient and
// Hessian are those of the polynomial (∂²/∂x² = 0, mixed second derivatives from w' = ∓1).
static void sdf_eval_trilinear(const Surface& s, const V3& x, double* val, V3* grad, M3* hess) {
  int64_t n[3] = {s.nx, s.ny, s.nz};
  int64_t ix[3];
  double w[3][2], d[3][2];
  for (int a = 0; a < 3; ++a) {
    // grid coordinate formed with the inverse spacing, as the device forms it, so that both
    // select the same cell for a point on a cell face (the interpolant is continuous there,
    // its gradient is not)
    double t = (x[a] - s.x0[a]) * (1.0 / s.h[a]);
    int64_t i = (int64_t)std::floor(t);
    if (i < 0) i = 0;
    if (i > n[a] - 2) i = n[a] - 2;
    double f = t - (double)i;
    ix[a] = i + 1;
    w[a][0] = 1 - f;
    w[a][1] = f;
    d[a][0] = -1.0;
    d[a][1] = 1.0;
  }
  const int64_t px = s.nx + 2, py = s.ny + 2;
  double v = 0, g[3] = {0, 0, 0}, H01 = 0, H02 = 0, H12 = 0;
  for (int c = 0; c < 2; ++c)
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) {
        double q = s.coef[(ix[0] + a) + px * ((ix[1] + b) + py * (ix[2] + c))];
        v += w[0][a] * w[1][b] * w[2][c] * q;
        g[0] += d[0][a] * w[1][b] * w[2][c] * q;
        g[1] += w[0][a] * d[1][b] * w[2][c] * q;
        g[2] += w[0][a] * w[1][b] * d[2][c] * q;
        H01 += d[0][a] * d[1][b] * w[2][c] * q;
        H02 += d[0][a] * w[1][b] * d[2][c] * q;
        H12 += w[0][a] * d[1][b] * d[2][c] * q;
      }
  *val = v;
  if (grad) *grad = v3(g[0] / s.h[0], g[1] / s.h[1], g[2] / s.h[2]);
  if (hess) {
    M3 h = zm3();
    h(0, 1) = h(1, 0) = H01 / (s.h[0] * s.h[1]);
    h(0, 2) = h(2, 0) = H02 / (s.h[0] * s.h[2]);
    h(1, 2) = h(2, 1) = H12 / (s.h[1] * s.h[2]);
    *hess = h;
  }
}

void sdf_eval(const Surface& s, const V3& x, double* val, V3* grad, M3* hess) {
  if (s.kind == 3) {
    sdf_eval_trilinear(s, x, val, grad, hess);
    return;
  }
  int64_t n[3] = {s.nx, s.ny, s.nz};
  int64_t ix[3];
  double w[3][3], d[3][3], dd[3][3];
  for (int a = 0; a < 3; ++a) bweights((x[a] - s.x0[a]) / s.h[a], n[a], &ix[a], w[a], d[a], dd[a]);
  const int64_t px = s.nx + 2, py = s.ny + 2;
  double v = 0, g[3] = {0, 0, 0}, H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) {
        double q = s.coef[(ix[0] + a) + px * ((ix[1] + b) + py * (ix[2] + c))];
        v += w[0][a] * w[1][b] * w[2][c] * q;
        g[0] += d[0][a] * w[1][b] * w[2][c] * q;
        g[1] += w[0][a] * d[1][b] * w[2][c] * q;
        g[2] += w[0][a] * w[1][b] * d[2][c] * q;
        H[0][0] += dd[0][a] * w[1][b] * w[2][c] * q;
        H[1][1] += w[0][a] * dd[1][b] * w[2][c] * q;
        H[2][2] += w[0][a] * w[1][b] * dd[2][c] * q;
        H[0][1] += d[0][a] * d[1][b] * w[2][c] * q;
        H[0][2] += d[0][a] * w[1][b] * d[2][c] * q;
        H[1][2] += w[0][a] * d[1][b] * d[2][c] * q;
      }
  *val = v;
  if (grad) *grad = v3(g[0] / s.h[0], g[1] / s.h[1], g[2] / s.h[2]);
  if (hess) {
    M3 h;
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j) {
        double e = H[i][j] / (s.h[i] * s.h[j]);
        h(i, j) = e;
        h(j, i) = e;
      }
    *hess = h;
  }
}

static bool isinside(const V3& p, const Surface& s) {  // utils_compute_interactions_beams.jl:39-47
  bool ok = true;
  int64_t n[3] = {s.nx, s.ny, s.nz};
  for (int a = 0; a < 3; ++a) {
    double lo = s.x0[a], hi = s.x0[a] + (double)(n[a] - 1) * s.h[a];
    double l = p[a] - lo;
    ok = ok && (l >= 0 && l <= (hi - lo));
  }
  return ok;
}

// PlaneSurface (def_interactions.jl:24-27) has no gap method in the reference.  The
// one used here follows the sphere's convention (utils_compute…:2-36) with the body
// on the positive side of the plane x[axis] = position: gap = x[axis] - position - r,
// gradient e_axis, Hessian zero; contact when gap <= r/4.
bool incontact(const V3& x, const Surface& s, double rb) {
  double gbar = rb / 4;
  if (s.kind == 2) return x[s.axis] - s.position - rb <= gbar;
  if (s.kind == 0) {  // utils_compute_interactions_beams.jl:23-36
    V3 aux = x - v3(s.center[0], s.center[1], s.center[2]);
    double g = norm(aux) - s.radius - rb;
    return g <= gbar;
  }
  // utils_compute_interactions_beams.jl:67-75
  if (!isinside(x, s)) return false;
  double v;
  sdf_eval(s, x, &v, nullptr, nullptr);
  return v - rb <= gbar;
}

void contact_gap(const V3& x, const Surface& s, double rb, double* g, V3* dg, M3* d2g) {
  if (s.kind == 2) {
    *g = x[s.axis] - s.position - rb;
    *dg = v3(s.axis == 0 ? 1.0 : 0.0, s.axis == 1 ? 1.0 : 0.0, s.axis == 2 ? 1.0 : 0.0);
    *d2g = zm3();
    return;
  }
  if (s.kind == 0) {  // utils_compute_interactions_beams.jl:2-20
    V3 aux = x - v3(s.center[0], s.center[1], s.center[2]);
    double na = norm(aux);
    *g = na - s.radius - rb;
    double inv = 1 / na;
    *dg = inv * aux;
    *d2g = inv * eye3() - ((inv * inv * inv) * outer(aux, aux));
    return;
  }
  // utils_compute_interactions_beams.jl:50-64
  double v;
  V3 gr;
  M3 H;
  sdf_eval(s, x, &v, &gr, &H);
  double nn = dot(gr, gr);
  double nmaginv = 1 / std::sqrt(nn);
  gr = gr * nmaginv;
  H = (H * nmaginv) * (eye3() - outer(gr, gr) / nn);
  *g = v - rb;
  *dg = gr;
  *d2g = H;
}

// ---------------- compute_contact_beams ----------------

static V3 ld3(const double* p) { return v3(p[0], p[1], p[2]); }
static M3 ld9(const double* p) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = p[k]; return m; }
static void put(double* m, int bi, int bj, const M3& b) {
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) m[(3 * bi + i) + 12 * (3 * bj + j)] = b(i, j);
}

void compute_contact_beams(const double* in, const Gauss& gs, const ContactProps& cp, const Surface& srf,
                           double* out) {  // compute&assemble_interactions_beams.jl:1-445
  const V3 X1 = ld3(in + EI_X1), X2 = ld3(in + EI_X2);
  const V3 u1 = ld3(in + EI_U1), u2 = ld3(in + EI_U2);
  const M3 R1 = ld9(in + EI_R1), R2 = ld9(in + EI_R2), dR1 = ld9(in + EI_DR1), dR2 = ld9(in + EI_DR2);
  const V3 ud1 = ld3(in + EI_UD1), ud2 = ld3(in + EI_UD2), wd1 = ld3(in + EI_WD1), wd2 = ld3(in + EI_WD2);
  const double l0 = in[EI_L0];
  const M3 Re0 = ld9(in + EI_RE0);
  const double rb = in[EI_RADIUS];
  const double kn = cp.kn, mu = cp.mu, eps_t = cp.eps_t;
  double eta_n = cp.eta_n;  // rebound inside the Gauss loop, see file header
  const M3 I3 = eye3();

  V3 x1 = X1 + u1, x2 = X2 + u2;
  double ln = norm(x2 - x1);
  LocalFrame f = local_Re_and_aux(x1, x2, R1, R2, col(Re0, 1), ln);  // :13
  const M3& Re = f.Re;
  const M3 ReT = tr(Re);
  const V3 r3 = f.r3;
  const M3 &G1 = f.Gt1, &G2 = f.Gt2, &G3 = f.Gt3, &G4 = f.Gt4;
  M3 Rb1 = (ReT * R1) * Re0, Rb2 = (ReT * R2) * Re0;
  V3 Th1 = toangle(Rb1), Th2 = toangle(Rb2);
  V3 Ud1 = ReT * ud1, Ud2 = ReT * ud2, Wd1 = ReT * wd1, Wd2 = ReT * wd2;  // :21-24
  M3 SUd1 = skew(Ud1), SUd2 = skew(Ud2), SWd1 = skew(Wd1), SWd2 = skew(Wd2);
  M3 G1ReT = G1 * ReT, G2ReT = G2 * ReT, G4ReT = G4 * ReT;  // :31-33
  M3 ReG1 = Re * tr(G1), ReG2 = Re * tr(G2), ReG4 = Re * tr(G4);  // :35-37

  double contact_energy = 0.0;
  V3 Tc[4] = {zv3(), zv3(), zv3(), zv3()};
  M3 Kc[4][4], Cc[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) { Kc[i][j] = zm3(); Cc[i][j] = zm3(); }

  for (int ig = 0; ig < gs.n; ++ig) {  // :54
    double zg = gs.z[ig], wg = gs.w[ig];
    double xi = l0 * (zg + 1) / 2;
    double N1 = 1 - xi / l0;
    double N2 = 1 - N1;
    double N3 = xi * ((1 - xi / l0) * (1 - xi / l0));
    double N4 = -(1 - xi / l0) * ((xi * xi) / l0);
    double N5 = (1 - 3 * xi / l0) * (1 - xi / l0);
    double N6 = (3 * xi / l0 - 2) * (xi / l0);
    double N7 = N3 + N4;
    double N8 = N5 + N6 - 1;
    (void)N8;
    V3 ut = v3(0.0, N3 * Th1[2] + N4 * Th2[2], -N3 * Th1[1] + -N4 * Th2[1]);  // :70
    M3 Sut = skew(ut);
    V3 xG = (N1 * x1 + N2 * x2) + Re * ut;  // :72
    double N7l = N7 / ln, N7l2 = N7l / ln;
    M3 P1P1 = rows(0, 0, 0, 0, N7l, 0, 0, 0, N7l);
    M3 P1P2 = rows(0, 0, 0, 0, 0, N3, 0, -N3, 0);
    M3 P1P3 = -P1P1;
    M3 P1P4 = rows(0, 0, 0, 0, 0, N4, 0, -N4, 0);
    M3 H1[4];
    H1[0] = (N1 * I3 + P1P1) - Sut * G1;  // :84
    H1[1] = P1P2 - Sut * G2;
    H1[2] = (N2 * I3 + P1P3) - Sut * G3;
    H1[3] = P1P4 - Sut * G4;
    V3 h1 = ((H1[0] * Ud1 + H1[1] * Wd1) + H1[2] * Ud2) + H1[3] * Wd2;  // :89
    M3 Sh1 = skew(h1);
    M3 H1F1 = ((H1[0] * SUd1 + H1[1] * SWd1) + H1[2] * SUd2) + H1[3] * SWd2;
    V3 ud0 = Re * h1;

    if (!incontact(xG, srf, rb)) continue;  // :95

    double gn;
    V3 dg;
    M3 d2g;
    contact_gap(xG, srf, rb, &gn, &dg, &d2g);  // :97
    double pn, dpn, Pie;
    regularize_gap_penalty(gn, rb, &pn, &dpn, &Pie);
    double deta_n;
    smoothstep_transition(eta_n, gn, rb, &eta_n, &deta_n);  // :100 (rebinds eta_n)

    double udn_mag = dot(ud0, dg);
    V3 udn = udn_mag * dg;
    V3 udt = ud0 - udn;
    double udt2 = dot(udt, udt);
    contact_energy += wg * kn * Pie;  // :107
    V3 fn = (kn * pn) * dg - eta_n * udn;
    double mureg = mu / std::sqrt(udt2 + eps_t);
    V3 ft = -((kn * pn) * mureg) * udt;
    V3 fc = fn + ft;
    V3 Fc = ReT * fc;  // :116

    M3 RHR[4];
    for (int i = 0; i < 4; ++i) RHR[i] = (Re * H1[i]) * ReT;  // :118-121
    for (int i = 0; i < 4; ++i) Tc[i] += wg * (tr(RHR[i]) * fc);  // :123-126

    M3 t1[4][4], t2[4][4], t3[4][4], t4[4][4];
    for (int i = 0; i < 4; ++i) {  // :128-155
      M3 RS = Re * skew(tr(H1[i]) * Fc);
      t1[i][0] = -(RS * G1ReT);
      t1[i][1] = -(RS * G2ReT);
      t1[i][2] = -t1[i][0];
      t1[i][3] = -(RS * G4ReT);
    }
    const V3 v1 = r3;  // :157
    M3 A1Fr11 = rows(0, 0, 0, Fc[1] * v1[0], Fc[1] * v1[1], Fc[1] * v1[2], Fc[2] * v1[0], Fc[2] * v1[1], Fc[2] * v1[2]);
    M3 SFc = skew(Fc);
    M3 SFP1 = (SFc * P1P1) * ReT, SFP2 = (SFc * P1P2) * ReT, SFP4 = (SFc * P1P4) * ReT;  // :162-164
    t2[0][0] = (N7l2 * Re) * A1Fr11 - ReG1 * SFP1;  // :166
    t2[0][1] = -(ReG1 * SFP2);
    t2[0][2] = -t2[0][0];
    t2[0][3] = -(ReG1 * SFP4);
    t2[1][0] = -(ReG2 * SFP1);
    t2[1][1] = -(ReG2 * SFP2);
    t2[1][2] = -t2[1][0];
    t2[1][3] = -(ReG2 * SFP4);
    t2[2][0] = t2[0][2];
    t2[2][1] = -t2[0][1];
    t2[2][2] = t2[0][0];
    t2[2][3] = -t2[0][3];
    t2[3][0] = -(ReG4 * SFP1);
    t2[3][1] = -(ReG4 * SFP2);
    t2[3][2] = -t2[3][0];
    t2[3][3] = -(ReG4 * SFP4);
    for (int i = 0; i < 4; ++i) {  // :186-209
      M3 RHS = (Re * tr(H1[i])) * SFc;
      t3[i][0] = RHS * G1ReT;
      t3[i][1] = RHS * G2ReT;
      t3[i][2] = -t3[i][0];
      t3[i][3] = RHS * G4ReT;
    }
    M3 aux = dot(dg, ud0) * d2g + outer(dg, d2g * ud0);  // :211
    M3 A1[4];
    for (int i = 0; i < 4; ++i) A1[i] = aux * RHR[i];
    M3 RSh1 = Re * Sh1;
    M3 A2_1 = -(RSh1 * G1ReT), A2_2 = -(RSh1 * G2ReT), A2_4 = -(RSh1 * G4ReT);
    double dU2 = Ud1[1] - Ud2[1], dU3 = Ud1[2] - Ud2[2];
    M3 A1Dr1 = rows(0, 0, 0, v1[0] * dU2, v1[1] * dU2, v1[2] * dU2, v1[0] * dU3, v1[1] * dU3, v1[2] * dU3);  // :223
    M3 RSGD = Re * skew(((G1 * Ud1 + G2 * Wd1) + G3 * Ud2) + G4 * Wd2);  // :225
    M3 A3_1 = (N7l2 * Re) * A1Dr1 + (RSGD * P1P1) * ReT;
    M3 A3_2 = (RSGD * P1P2) * ReT;
    M3 A3_4 = (RSGD * P1P4) * ReT;
    M3 RH1SD = Re * H1F1;
    M3 A4_1 = RH1SD * G1ReT, A4_2 = RH1SD * G2ReT, A4_4 = RH1SD * G4ReT;
    M3 du0dd[4];
    du0dd[0] = (A2_1 + A3_1) + A4_1;  // :235
    du0dd[1] = (A2_2 + A3_2) + A4_2;
    du0dd[2] = -du0dd[0];
    du0dd[3] = (A2_4 + A3_4) + A4_4;
    M3 nn = outer(dg, dg);
    M3 dundd[4], dutdd[4], dundv[4], du0dv[4], dutdv[4];
    for (int i = 0; i < 4; ++i) {
      dundd[i] = A1[i] + nn * du0dd[i];  // :242
      dutdd[i] = du0dd[i] - dundd[i];
      dundv[i] = nn * RHR[i];
      du0dv[i] = RHR[i];
      dutdv[i] = du0dv[i] - dundv[i];
    }
    M3 auxK = ((kn * dpn) * nn + (kn * pn) * d2g) - outer(deta_n * udn, dg);  // :269
    M3 Kfn[4], Cfn[4], Kft[4], Cft[4], Kfc[4], Cfc[4];
    for (int i = 0; i < 4; ++i) {
      Kfn[i] = auxK * RHR[i] - eta_n * dundd[i];
      Cfn[i] = ((-eta_n) * nn) * du0dv[i];
    }
    M3 aux1 = outer((((-mureg) * kn) * dpn) * udt, dg);  // :290
    M3 aux2 = (((-mureg) * kn) * pn) * (I3 - (1 / (udt2 + eps_t)) * outer(udt, udt));
    for (int i = 0; i < 4; ++i) {
      Kft[i] = aux1 * RHR[i] + aux2 * dutdd[i];
      Cft[i] = aux2 * dutdv[i];
      Kfc[i] = Kfn[i] + Kft[i];
      Cfc[i] = Cfn[i] + Cft[i];
    }
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) t4[i][j] = tr(RHR[i]) * Kfc[j];  // :307-325
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        Kc[i][j] += wg * (((t1[i][j] + t2[i][j]) + t3[i][j]) + t4[i][j]);  // :332-350
        Cc[i][j] += (wg * tr(RHR[i])) * Cfc[j];                           // :352-370
      }
  }

  double l02 = l0 / 2;  // :376
  for (int i = 0; i < 4; ++i) Tc[i] = l02 * Tc[i];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      Cc[i][j] = l02 * Cc[i][j];
      Kc[i][j] = l02 * Kc[i][j];
    }
  contact_energy = l02 * contact_energy;

  V3 Tha = toangle(dR1), Thb = toangle(dR2);  // :420-437
  M3 TaT = tr(Ts_inv(Tha)), TbT = tr(Ts_inv(Thb));
  for (int j = 0; j < 4; ++j) {
    Cc[1][j] = Cc[1][j] * TaT;
    Cc[3][j] = Cc[3][j] * TbT;
  }

  out[CO_E] = contact_energy;
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 3; ++k) out[CO_TC + 3 * i + k] = Tc[i][k];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      put(out + CO_K, i, j, Kc[i][j]);  // :440
      put(out + CO_C, i, j, Cc[i][j]);  // :441
    }
}

}  // namespace orc
