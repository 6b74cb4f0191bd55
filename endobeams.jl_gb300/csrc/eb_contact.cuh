// Beam-to-rigid-surface contact element on the GPU (FP64, one thread per
// element): compute_contact_beams of
// src/interactions/compute&assemble_interactions_beams.jl:1-445 with the
// surfaces of src/interactions/utils_compute_interactions_beams.jl and the
// regularisations of interactions_beams_regularization.jl.
//
// As in the reference, the normal damping ηₙ is a function-level variable
// that the Gauss loop overwrites with its smoothstep value (:100), so an
// in-contact Gauss point sees the value left by the previous one.
#pragma once
#include "eb_beam.cuh"

namespace ebd {

struct ContactProps {
  double kn, mu, eps_t, eta_n;
};

// Rigid surface: analytic sphere, quadratic B-spline SDF on a voxel grid, or
// analytic plane.
struct SurfaceDev {
  int kind;                // 0 sphere, 1 SDF, 2 plane
  double cx, cy, cz, R;    // sphere
  int axis;                // plane: x[axis] = pos, body on the positive side
  double pos;
  const double* coef;      // (nx+2)(ny+2)(nz+2) prefiltered coefficients (interp 1: the samples), x fastest
  int interp;              // 0 quadratic B-spline (the reference's), 1 trilinear
  int nx, ny, nz;          // grid points
  double x0, y0, z0;       // first grid point
  double ihx, ihy, ihz;    // 1 / spacing
  double xl, yl, zl;       // domain extents (n-1)*h
};

struct ContactIn {
  V3 X1, X2, u1, u2, ud1, ud2, wd1, wd2;
  M3 R1, R2, dR1, dR2, Re0;
  double l0, radius;
};

struct ContactOut {
  double* K;   // 144
  double* C;   // 144
  double* T;   // 12
  double* E;   // 1
};

// interactions_beams_regularization.jl:2-26
EB_DEV void regularize_gap_penalty(double gap, double rb, double* p, double* dp, double* Pi) {
  double gt = rb / 4, hg = gt / 2;
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

// interactions_beams_regularization.jl:29-46
EB_DEV void smoothstep_transition(double value, double pos, double rb, double* s, double* ds) {
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

// Per-axis quadratic B-spline weights around the nearest grid point.
EB_DEV int bspline_axis(double t, int n, double w[3], double d[3]) {
  int i = (int)floor(t + 0.5);
  i = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
  double del = t - (double)i;
  double lo = 0.5 - del, hi = 0.5 + del;
  w[0] = 0.5 * (lo * lo);
  w[1] = 0.75 - del * del;
  w[2] = 0.5 * (hi * hi);
  d[0] = del - 0.5;
  d[1] = -2 * del;
  d[2] = del + 0.5;
  return i;
}

// Cell index (clamped to the grid's n-1 cells) and fraction along one axis.
EB_DEV int linear_axis(double t, int n, double* f) {
  int i = (int)floor(t);
  i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
  *f = t - (double)i;
  return i;
}

// Trilinear interpolant of the samples (8 taps of the padded grid, sample (i,j,k) at
// padded (i+1,j+1,k+1)): value, gradient and Hessian of the interpolating polynomial of
// the cell (its diagonal second derivatives vanish; the mixed ones do not).
EB_DEV double sdf_eval_linear(const SurfaceDev& s, V3 x, V3* grad, M3* hess) {
  double fx, fy, fz;
  const int ix = linear_axis((x.x - s.x0) * s.ihx, s.nx, &fx);
  const int iy = linear_axis((x.y - s.y0) * s.ihy, s.ny, &fy);
  const int iz = linear_axis((x.z - s.z0) * s.ihz, s.nz, &fz);
  const long px = s.nx + 2, py = s.ny + 2;
  const double* base = s.coef + ((ix + 1) + px * ((iy + 1) + py * (long)(iz + 1)));
  const double wx[2] = {1 - fx, fx}, wy[2] = {1 - fy, fy}, wz[2] = {1 - fz, fz};
  const double dd[2] = {-1.0, 1.0};
  double v = 0, gx = 0, gy = 0, gz = 0, hxy = 0, hxz = 0, hyz = 0;
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const double* row = base + px * (b + py * c);
      const double q0 = __ldg(row), q1 = __ldg(row + 1);
      const double sw = wx[0] * q0 + wx[1] * q1, sd = q1 - q0;
      v += wy[b] * wz[c] * sw;
      gx += wy[b] * wz[c] * sd;
      gy += dd[b] * wz[c] * sw;
      gz += wy[b] * dd[c] * sw;
      hxy += dd[b] * wz[c] * sd;
      hxz += wy[b] * dd[c] * sd;
      hyz += dd[b] * dd[c] * sw;
    }
  if (grad) {
    *grad = v3(gx * s.ihx, gy * s.ihy, gz * s.ihz);
    const double exy = hxy * (s.ihx * s.ihy), exz = hxz * (s.ihx * s.ihz), eyz = hyz * (s.ihy * s.ihz);
    *hess = rows(0.0, exy, exz, exy, 0.0, eyz, exz, eyz, 0.0);
  }
  return v;
}

// Value (and optionally gradient and Hessian) of the scaled quadratic
// B-spline interpolant at world point x (27 taps of the padded grid).
EB_DEV double sdf_eval(const SurfaceDev& s, V3 x, V3* grad, M3* hess) {
  if (s.interp == 1) return sdf_eval_linear(s, x, grad, hess);
  double wx[3], wy[3], wz[3], dx[3], dy[3], dz[3];
  int ix = bspline_axis((x.x - s.x0) * s.ihx, s.nx, wx, dx);
  int iy = bspline_axis((x.y - s.y0) * s.ihy, s.ny, wy, dy);
  int iz = bspline_axis((x.z - s.z0) * s.ihz, s.nz, wz, dz);
  const long px = s.nx + 2, py = s.ny + 2;
  const double* base = s.coef + (ix + px * (iy + py * (long)iz));
  double v = 0, gx = 0, gy = 0, gz = 0, hxx = 0, hyy = 0, hzz = 0, hxy = 0, hxz = 0, hyz = 0;
  const double dd[3] = {1.0, -2.0, 1.0};
  const bool full = grad != nullptr;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const double* row = base + px * (b + py * c);
      double q0 = __ldg(row), q1 = __ldg(row + 1), q2 = __ldg(row + 2);
      double sw = wx[0] * q0 + wx[1] * q1 + wx[2] * q2;   // Σ wx q
      double wyz = wy[b] * wz[c];
      v += wyz * sw;
      if (full) {
        double sd = dx[0] * q0 + dx[1] * q1 + dx[2] * q2;  // Σ dx q
        double s2 = q0 - 2 * q1 + q2;                      // Σ ddx q
        gx += wyz * sd;
        gy += dy[b] * wz[c] * sw;
        gz += wy[b] * dz[c] * sw;
        hxx += wyz * s2;
        hyy += dd[b] * wz[c] * sw;
        hzz += wy[b] * dd[c] * sw;
        hxy += dy[b] * wz[c] * sd;
        hxz += wy[b] * dz[c] * sd;
        hyz += dy[b] * dz[c] * sw;
      }
    }
  }
  if (full) {
    *grad = v3(gx * s.ihx, gy * s.ihy, gz * s.ihz);
    double exy = hxy * (s.ihx * s.ihy), exz = hxz * (s.ihx * s.ihz), eyz = hyz * (s.ihy * s.ihz);
    *hess = rows(hxx * (s.ihx * s.ihx), exy, exz, exy, hyy * (s.ihy * s.ihy), eyz, exz, eyz, hzz * (s.ihz * s.ihz));
  }
  return v;
}

EB_DEV double axis_coord(V3 x, int a) { return a == 0 ? x.x : (a == 1 ? x.y : x.z); }

// PlaneSurface (def_interactions.jl:24-27) has no gap method in the reference; the one
// here follows the sphere's convention (utils_compute…:2-36): gap = x[axis] - pos - r,
// gradient e_axis, Hessian zero, contact when gap <= r/4.
EB_DEV bool incontact(const SurfaceDev& s, V3 x, double rb) {
  double gbar = rb / 4;
  if (s.kind == 2) return axis_coord(x, s.axis) - s.pos - rb <= gbar;
  if (s.kind == 0) {  // utils_compute_interactions_beams.jl:23-36
    V3 aux = x - v3(s.cx, s.cy, s.cz);
    return norm(aux) - s.R - rb <= gbar;
  }
  // isinside (utils_compute…:39-47) && φ - r ≤ r/4 (:67-75)
  double lx = x.x - s.x0, ly = x.y - s.y0, lz = x.z - s.z0;
  bool in = lx >= 0 && lx <= s.xl && ly >= 0 && ly <= s.yl && lz >= 0 && lz <= s.zl;
  if (!in) return false;
  return sdf_eval(s, x, nullptr, nullptr) - rb <= gbar;
}

EB_DEV void contact_gap(const SurfaceDev& s, V3 x, double rb, double* g, V3* dg, M3* d2g) {
  if (s.kind == 2) {
    *g = axis_coord(x, s.axis) - s.pos - rb;
    *dg = v3(s.axis == 0 ? 1.0 : 0.0, s.axis == 1 ? 1.0 : 0.0, s.axis == 2 ? 1.0 : 0.0);
    *d2g = zm3();
    return;
  }
  if (s.kind == 0) {  // utils_compute…:2-20
    V3 aux = x - v3(s.cx, s.cy, s.cz);
    double na = norm(aux);
    *g = na - s.R - rb;
    double inv = 1 / na;
    *dg = inv * aux;
    M3 h = (-(inv * inv * inv)) * outer(aux, aux);
    h.a[0] += inv; h.a[4] += inv; h.a[8] += inv;
    *d2g = h;
    return;
  }
  // utils_compute…:50-64 (Hessian projected with the already-normalised gradient)
  V3 gr;
  M3 H;
  double v = sdf_eval(s, x, &gr, &H);
  double nn = dot(gr, gr);
  double nmaginv = 1 / sqrt(nn);
  gr = nmaginv * gr;
  M3 P = (-1.0 / nn) * outer(gr, gr);
  P.a[0] += 1; P.a[4] += 1; P.a[8] += 1;
  *g = v - rb;
  *dg = gr;
  *d2g = (nmaginv * H) * P;
}

EB_DEV void contact_element(const ContactIn& in, const Gauss3& gs, const ContactProps& cp, const SurfaceDev& srf,
                            ContactOut out, bool* any_contact) {
  const M3 I3 = eye3();
  V3 x1 = in.X1 + in.u1, x2 = in.X2 + in.u2;
  double ln = norm(x2 - x1);
  Frame f = local_frame(x1, x2, in.R1, in.R2, col(in.Re0, 1), ln);
  const M3& Re = f.Re;
  const M3 ReT = tr(Re);
  const V3 v1 = f.v1;
  const Gu G1 = f.G1;
  const Gt G2 = f.G2, G4 = f.G4;
  V3 Th1 = toangle(mulTN(Re, in.R1) * in.Re0);
  V3 Th2 = toangle(mulTN(Re, in.R2) * in.Re0);
  V3 Ud1 = mulTv(Re, in.ud1), Ud2 = mulTv(Re, in.ud2), Wd1 = mulTv(Re, in.wd1), Wd2 = mulTv(Re, in.wd2);
  V3 dU = Ud1 - Ud2;
  M3 G1ReT = Gmul(G1, ReT), G2ReT = Gmul(G2, ReT), G4ReT = Gmul(G4, ReT);
  const double rb = in.radius, l0 = in.l0, il = 1.0 / ln;
  const double kn = cp.kn, mu = cp.mu, eps_t = cp.eps_t;
  double eta_n = cp.eta_n;  // overwritten by each in-contact Gauss point (reference scoping)

  // Which Gauss points are in contact (:72, :95).  Most elements have none: they return
  // here, before the 12x12 accumulators are touched.
  bool inc[3];
  bool touched = false;
#pragma unroll
  for (int ig = 0; ig < 3; ++ig) {
    const double zg = gs.z[ig];
    double xi = l0 * (zg + 1) / 2;
    double s = xi / l0;
    double N1 = 1 - s, N2 = 1 - N1;
    double N3 = xi * ((1 - s) * (1 - s));
    double N4 = -(1 - s) * ((xi * xi) / l0);
    V3 ut = v3(0.0, N3 * Th1.z + N4 * Th2.z, -N3 * Th1.y - N4 * Th2.y);
    V3 xG = N1 * x1 + N2 * x2 + Re * ut;
    inc[ig] = incontact(srf, xG, rb);
    touched |= inc[ig];
  }
  *any_contact = touched;
  if (!touched) return;

  // Kᶜ and Cᶜ are summed over the Gauss points in the element's staging blocks (global
  // memory, this thread's own 2 x 144 doubles) rather than in 288 accumulator registers,
  // which spilled; the sums, their order and the final scaling are the same.
  double energy = 0.0;
  V3 Tc[4] = {zv3(), zv3(), zv3(), zv3()};
  for (int k = 0; k < 144; ++k) {
    out.K[k] = 0.0;
    out.C[k] = 0.0;
  }

#pragma unroll 1
  for (int ig = 0; ig < 3; ++ig) {
    if (!inc[ig]) continue;
    const double zg = gs.z[ig], wg = gs.w[ig];
    double xi = l0 * (zg + 1) / 2;
    double s = xi / l0;
    double N1 = 1 - s, N2 = 1 - N1;
    double N3 = xi * ((1 - s) * (1 - s));
    double N4 = -(1 - s) * ((xi * xi) / l0);
    double N7 = N3 + N4;
    V3 ut = v3(0.0, N3 * Th1.z + N4 * Th2.z, -N3 * Th1.y - N4 * Th2.y);
    V3 xG = N1 * x1 + N2 * x2 + Re * ut;

    double N7l = N7 * il, N7l2 = N7l * il;
    M3 Sut = skew(ut);
    M3 SutG1 = mulG(Sut, G1);
    M3 P1P2 = rows(0, 0, 0, 0, 0, N3, 0, -N3, 0);
    M3 P1P4 = rows(0, 0, 0, 0, 0, N4, 0, -N4, 0);
    M3 H1[4];
    H1[0] = diag3(N1, N1 + N7l, N1 + N7l) - SutG1;
    H1[1] = P1P2 - mulG(Sut, G2);
    H1[2] = diag3(N2, N2 - N7l, N2 - N7l) + SutG1;
    H1[3] = P1P4 - mulG(Sut, G4);
    V3 h1 = H1[0] * Ud1 + H1[1] * Wd1 + H1[2] * Ud2 + H1[3] * Wd2;
    M3 H1F1 = mulskew(H1[0], Ud1) + mulskew(H1[1], Wd1) + mulskew(H1[2], Ud2) + mulskew(H1[3], Wd2);
    V3 ud0 = Re * h1;

    double gn;
    V3 dg;
    M3 d2g;
    contact_gap(srf, xG, rb, &gn, &dg, &d2g);
    double pn, dpn, Pie;
    regularize_gap_penalty(gn, rb, &pn, &dpn, &Pie);
    double deta_n;
    smoothstep_transition(eta_n, gn, rb, &eta_n, &deta_n);

    double udn_mag = dot(ud0, dg);
    V3 udn = udn_mag * dg;
    V3 udt = ud0 - udn;
    double udt2 = dot(udt, udt);
    energy += wg * kn * Pie;
    V3 fn = (kn * pn) * dg - eta_n * udn;
    double mureg = mu / sqrt(udt2 + eps_t);
    V3 ft = (-(kn * pn) * mureg) * udt;
    V3 fc = fn + ft;
    V3 Fc = mulTv(Re, fc);

    M3 RHR[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) RHR[i] = mulNT(Re * H1[i], Re);
#pragma unroll
    for (int i = 0; i < 4; ++i) Tc[i] += wg * mulTv(RHR[i], fc);

    // t₂ factors (:157-184)
    M3 SFc = skew(Fc);
    M3 A1Fr = rows(0, 0, 0, Fc.y * v1.x, Fc.y * v1.y, Fc.y * v1.z, Fc.z * v1.x, Fc.z * v1.y, Fc.z * v1.z);
    M3 SFP1 = muld(SFc, v3(0.0, N7l, N7l)) * ReT, SFP2 = (SFc * P1P2) * ReT, SFP4 = (SFc * P1P4) * ReT;
    M3 ReG1 = mulNT(Re, full(G1)), ReG2 = mulNT(Re, full(G2)), ReG4 = mulNT(Re, full(G4));

    // ∂u̇₀/∂d (:211-238)
    M3 aux = dot(dg, ud0) * d2g + outer(dg, d2g * ud0);
    M3 Sh1 = skew(h1);
    M3 RSh1 = Re * Sh1;
    M3 A1Dr = rows(0, 0, 0, v1.x * dU.y, v1.y * dU.y, v1.z * dU.y, v1.x * dU.z, v1.y * dU.z, v1.z * dU.z);
    V3 We = Gv(G1, dU) + Gv(G2, Wd1) + Gv(G4, Wd2);
    M3 RSGD = mulskew(Re, We);  // Rₑ S(GḊ)
    M3 RH1SD = Re * H1F1;
    M3 du0[4];
    du0[0] = (RH1SD - RSh1) * G1ReT + (N7l2 * (Re * A1Dr) + muld(RSGD, v3(0.0, N7l, N7l)) * ReT);
    du0[1] = (RH1SD - RSh1) * G2ReT + (RSGD * P1P2) * ReT;
    du0[2] = -du0[0];
    du0[3] = (RH1SD - RSh1) * G4ReT + (RSGD * P1P4) * ReT;
    M3 nn = outer(dg, dg);
    M3 auxK = (kn * dpn) * nn + (kn * pn) * d2g - outer(deta_n * udn, dg);
    M3 aux1 = outer(((-mureg) * kn * dpn) * udt, dg);
    M3 aux2 = ((-mureg) * kn * pn) * (I3 - (1 / (udt2 + eps_t)) * outer(udt, udt));
    // The reference's ∂u̇ₙ/∂d = aux Rⱼ + nn D⁰ⱼ, ∂u̇ₜ/∂d = D⁰ⱼ - ∂u̇ₙ/∂d and ∂u̇ₜ/∂u̇ = Rⱼ - nn Rⱼ,
    // substituted and collected (14 products instead of 32):
    //   Kfcⱼ = A1 Rⱼ + A2 D⁰ⱼ,  Cfcⱼ = A2 Rⱼ,
    //   A1 = auxK + aux1 - (ηₙ I + aux2) aux,  A2 = aux2 - aux2 nn - ηₙ nn.
    M3 eta_aux2 = aux2;
    eta_aux2.a[0] += eta_n; eta_aux2.a[4] += eta_n; eta_aux2.a[8] += eta_n;
    const M3 A1 = (auxK + aux1) - eta_aux2 * aux;
    const M3 A2 = aux2 - (aux2 * nn + eta_n * nn);
    M3 Kfc[4], Cfc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      Kfc[j] = A1 * RHR[j] + A2 * du0[j];
      Cfc[j] = A2 * RHR[j];
    }
    // accumulate (:332-370), one row block at a time:
    //   t₁ + t₃ (:128-155, :186-209): Rₑ[-S(H₁ⁱᵀ𝓕ᶜ) + H₁ⁱᵀS(𝓕ᶜ)] Gʲ Rₑᵀ, j = 1,2,4 (t^{i3} = -t^{i1});
    //   t₂ row i from ReGᵢ and SFPⱼ.
    // H₁¹ + H₁³ = I (N₁ + N₂ = 1), so row block 3 is row block 1's complement: its t₁+t₃ and
    // t₂ are minus row 1's, and its Rₑ H₁³ Rₑᵀ = I - Rₑ H₁¹ Rₑᵀ gives Kᶜ/Cᶜ terms Kfcⱼ - t₄¹ʲ.
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i == 2) continue;  // formed with row block 0
      M3 Li = Re * (mulTN(H1[i], SFc) - skew(mulTv(H1[i], Fc)));
      const M3 t13_1 = Li * G1ReT, t13_2 = Li * G2ReT, t13_4 = Li * G4ReT;
      const M3& ReGi = (i == 1) ? ReG2 : (i == 3) ? ReG4 : ReG1;
      const M3 t2_1 = (i == 0) ? N7l2 * (Re * A1Fr) - ReG1 * SFP1 : -(ReGi * SFP1);
      const M3 t2_2 = -(ReGi * SFP2), t2_4 = -(ReGi * SFP4);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const M3 t4 = mulTN(RHR[i], Kfc[j]);
        const M3 t13v = (j == 0) ? t13_1 : (j == 1) ? t13_2 : (j == 2) ? -t13_1 : t13_4;
        const M3 t2v = (j == 0) ? t2_1 : (j == 1) ? t2_2 : (j == 2) ? -t2_1 : t2_4;
        const M3 tc = mulTN(RHR[i], Cfc[j]);
        const M3 t12 = t13v + t2v;
        acc_block(out.K, i, j, wg, t12 + t4);
        acc_block(out.C, i, j, wg, tc);
        if (i == 0) {
          acc_block(out.K, 2, j, wg, (Kfc[j] - t4) - t12);
          acc_block(out.C, 2, j, wg, Cfc[j] - tc);
        }
      }
    }
  }
  const double l02 = l0 / 2;
  out.E[0] = l02 * energy;
#pragma unroll
  for (int i = 0; i < 4; ++i) put_vec(out.T, i, l02 * Tc[i]);
  V3 Tha = toangle(in.dR1), Thb = toangle(in.dR2);
  M3 TaT = tr(Ts_inv(Tha)), TbT = tr(Ts_inv(Thb));
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      put_block(out.K, i, j, l02 * get_block(out.K, i, j));
      M3 c = l02 * get_block(out.C, i, j);
      if (i == 1) c = c * TaT;
      if (i == 3) c = c * TbT;
      put_block(out.C, i, j, c);
    }
}

}  // namespace ebd
