// ORACLE — test infrastructure only.  CPU FP64 restatement of the beam
// element of EndoBeams.jl, statement by statement, in the order the Julia
// source evaluates them (later statements see earlier reassignments, which
// matters in the exact-mode block at compute_beams.jl:480-506).
#include "eb_oracle.hpp"

#include <algorithm>

namespace orc {

M3 skew(const V3& v) {  // utils_beams.jl:2-8
  return rows(0.0, -v[2], v[1], v[2], 0.0, -v[0], -v[1], v[0], 0.0);
}

M3 rotation_matrix(const V3& th) {  // utils_beams.jl:11-32
  double n = norm(th);
  if (n > 10 * EPS64) {
    double s = std::sin(n), c = std::cos(n);
    M3 S = skew(th);
    return (eye3() + (s / n) * S) + (((1 - c) / (n * n)) * S) * S;
  }
  return eye3();
}

LocalFrame local_Re_and_aux(const V3& x1, const V3& x2, const M3& R1, const M3& R2, const V3& Re0E2,
                            double ln) {  // utils_beams.jl:35-87
  LocalFrame f;
  V3 v1 = (x2 - x1) / ln;
  V3 p1 = R1 * Re0E2;
  V3 p2 = R2 * Re0E2;
  V3 p = (p1 + p2) / 2.0;
  V3 v3_ = cross(v1, p);
  v3_ = v3_ / norm(v3_);
  V3 v2 = cross(v3_, v1);
  f.Re = hcat3(v1, v2, v3_);
  f.r1 = -v1;
  f.r3 = v1;
  double q1 = dot(v1, p), q2 = dot(v2, p);
  double q11 = dot(v1, p1), q12 = dot(v2, p1);
  double q21 = dot(v1, p2), q22 = dot(v2, p2);
  double eta = q1 / q2;
  double eta11 = q11 / q2, eta12 = q12 / q2, eta21 = q21 / q2, eta22 = q22 / q2;
  f.eta = eta;
  f.Gt1 = rows(0.0, 0.0, eta / ln, 0.0, 0.0, 1 / ln, 0.0, -1 / ln, 0.0);
  f.Gt3 = -f.Gt1;
  f.Gt2 = rows(eta12 / 2, -eta11 / 2, 0.0, 0, 0, 0, 0, 0, 0);
  f.Gt4 = rows(eta22 / 2, -eta21 / 2, 0.0, 0, 0, 0, 0, 0, 0);
  f.D3 = (eye3() - outer(v1, v1)) / ln;
  return f;
}

V3 toangle(const M3& R) {  // utils_beams.jl:90-104
  double c = (trace(R) - 1) / 2;
  double nv;
  if (std::fabs(c) < 1)
    nv = std::max(std::acos(c), 10 * EPS64);
  else
    nv = 10 * EPS64;
  V3 a = v3(R(2, 1) - R(1, 2), R(0, 2) - R(2, 0), R(1, 0) - R(0, 1));
  V3 n = (1 / (2 * std::sin(nv))) * a;
  return nv * n;
}

M3 Ts_inv(const V3& th) {  // utils_beams.jl:107-122
  double n = norm(th);
  if (n < 10 * EPS64) return eye3();
  M3 S = skew(th);
  double s2 = std::sin(n / 2), c2 = std::cos(n / 2);
  return (eye3() - S / 2.0) + (((s2 - n / 2 * c2) / (s2 * (n * n))) * S) * S;
}

void compute_eta_mu(const V3& thv, double* eta, double* mu) {  // utils_beams.jl:180-198
  double th = norm(thv);
  if (th < 10 * EPS64) {
    *eta = 1.0 / 12.0;
    *mu = 1.0 / 360.0;
  } else {
    double s = std::sin(th), c = std::cos(th), s2 = std::sin(th / 2);
    *eta = ((2 * s) - th * (1 + c)) / (2 * (th * th) * s);
    *mu = (th * (th + s) - 8 * (s2 * s2)) / (4 * (th * th * th * th) * (s2 * s2));
  }
}

M3 compute_Kh(const V3& th, const V3& Mb, const M3& Tsinv, double eta, double mu) {  // utils_beams.jl:201-215
  M3 thMt = outer(th, Mb);
  M3 MtT = tr(thMt);
  M3 Sth = skew(th), SM = skew(Mb);
  M3 inner = eta * (thMt - 2.0 * MtT + dot(th, Mb) * eye3()) + mu * ((Sth * Sth) * MtT) - SM / 2.0;
  return inner * Tsinv;
}

static V3 ld3(const double* p) { return v3(p[0], p[1], p[2]); }
static M3 ld9(const double* p) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = p[k]; return m; }

// Writes the 3x3 block `b` at block position (bi, bj) of a 12x12 column-major matrix.
static void put(double* m, int bi, int bj, const M3& b) {
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) m[(3 * bi + i) + 12 * (3 * bj + j)] = b(i, j);
}
static void putv(double* v, int bi, const V3& b) { for (int i = 0; i < 3; ++i) v[3 * bi + i] = b[i]; }

// Diagonal-times-matrix helpers: K̄ⁱⁿᵗΘ̅ and Jᵨ are Julia `Diagonal`s.
static M3 dmul(const V3& d, const M3& m) { return diag3(d[0], d[1], d[2]) * m; }
static V3 dmulv(const V3& d, const V3& x) { return v3(d[0] * x[0], d[1] * x[1], d[2] * x[2]); }

void compute_beams(const double* in, const Gauss& g, double* out) {  // compute_beams.jl:1-538
  const V3 X1 = ld3(in + EI_X1), X2 = ld3(in + EI_X2);
  const V3 u1 = ld3(in + EI_U1), u2 = ld3(in + EI_U2);
  const M3 R1 = ld9(in + EI_R1), R2 = ld9(in + EI_R2), dR1 = ld9(in + EI_DR1), dR2 = ld9(in + EI_DR2);
  const V3 ud1 = ld3(in + EI_UD1), ud2 = ld3(in + EI_UD2), wd1 = ld3(in + EI_WD1), wd2 = ld3(in + EI_WD2);
  const V3 udd1 = ld3(in + EI_UDD1), udd2 = ld3(in + EI_UDD2), wdd1 = ld3(in + EI_WDD1), wdd2 = ld3(in + EI_WDD2);
  const double l0 = in[EI_L0];
  const M3 Re0 = ld9(in + EI_RE0);
  const double Ku = in[EI_KU];
  const V3 KT = ld3(in + EI_KT), KTT = ld3(in + EI_KTT), Jr = ld3(in + EI_JR);
  const double Ar = in[EI_AR], damping = in[EI_DAMP];
  const M3 I3 = eye3();

  V3 x1 = X1 + u1, x2 = X2 + u2;                                    // :13-14
  double ln = norm(x2 - x1);                                        // :16
  double ubar = ln - l0;                                            // :18
  LocalFrame f = local_Re_and_aux(x1, x2, R1, R2, col(Re0, 1), ln);  // :20
  const M3& Re = f.Re;
  const M3 ReT = tr(Re);
  const V3 r1 = f.r1, r3 = f.r3;
  const double eta = f.eta;
  const M3 &G1 = f.Gt1, &G2 = f.Gt2, &G3 = f.Gt3, &G4 = f.Gt4, &D3 = f.D3;

  M3 Rb1 = (ReT * R1) * Re0, Rb2 = (ReT * R2) * Re0;  // :22-23
  V3 Th1 = toangle(Rb1), Th2 = toangle(Rb2);          // :25-26
  M3 T1 = Ts_inv(Th1), T2 = Ts_inv(Th2);              // :29-30

  M3 P11 = -G1, P21 = P11, P12 = I3 - G2, P22 = -G2, P14 = -G4, P24 = I3 - G4;  // :33-38
  V3 Bp1 = r1;                                                                // :41 (row vector)
  M3 Bp11 = P11 * ReT, Bp21 = Bp11, Bp12 = P12 * ReT, Bp22 = P22 * ReT, Bp14 = P14 * ReT, Bp24 = P24 * ReT;
  V3 B1 = Bp1;                                                                // :50
  M3 B11 = T1 * Bp11, B12 = T1 * Bp12, B14 = T1 * Bp14;                       // :51-53
  M3 B21 = T2 * Bp21, B22 = T2 * Bp22, B24 = T2 * Bp24;                       // :54-56

  double Tu = Ku * ubar;                                                      // :61
  V3 TT1 = dmulv(KT, Th1) + dmulv(KTT, Th2);                                  // :62
  V3 TT2 = dmulv(KTT, Th1) + dmulv(KT, Th2);                                  // :63
  double strain_energy = (ubar * Tu + dot(Th1, TT1) + dot(Th2, TT2)) / 2;     // :65

  V3 Ti1 = B1 * Tu + tr(B11) * TT1 + tr(B21) * TT2;  // :68
  V3 Ti2 = tr(B12) * TT1 + tr(B22) * TT2;            // :69
  V3 Ti3 = -Ti1;                                     // :70
  V3 Ti4 = tr(B14) * TT1 + tr(B24) * TT2;            // :71

  double Nb = Tu;                    // :77
  V3 Mp1 = tr(T1) * TT1;             // :78
  V3 Mp2 = tr(T2) * TT2;             // :79
  V3 Qs1 = tr(P11) * Mp1 + tr(P21) * Mp2;  // :82
  V3 Qs2 = tr(P12) * Mp1 + tr(P22) * Mp2;  // :83
  V3 Qs4 = tr(P14) * Mp1 + tr(P24) * Mp2;  // :84
  M3 Q1 = skew(Qs1), Q2 = skew(Qs2), Q4 = skew(Qs4);  // :87-89
  V3 a = v3(0.0, eta * (Mp1[0] + Mp2[0]) / ln + (Mp1[1] + Mp2[1]) / ln, (Mp1[2] + Mp2[2]) / ln);  // :91
  M3 DN11 = D3 * Nb;  // :94
  M3 QG11 = Q1 * G1, QG12 = Q1 * G2, QG14 = Q1 * G4, QG22 = Q2 * G2, QG24 = Q2 * G4, QG44 = Q4 * G4;  // :97-102
  V3 EGa1 = Re * (tr(G1) * a);  // :106
  M3 EGar11 = outer(EGa1, r1);  // :109
  M3 Km11 = (DN11 - (Re * QG11) * ReT) + EGar11;  // :112
  M3 Km12 = -((Re * QG12) * ReT);
  M3 Km14 = -((Re * QG14) * ReT);
  M3 Km22 = -((Re * QG22) * ReT);
  M3 Km24 = -((Re * QG24) * ReT);
  M3 Km44 = -((Re * QG44) * ReT);

  double eta1, mu1, eta2, mu2;
  compute_eta_mu(Th1, &eta1, &mu1);  // :121
  compute_eta_mu(Th2, &eta2, &mu2);  // :122
  M3 Kh1 = compute_Kh(Th1, TT1, T1, eta1, mu1);  // :127
  M3 Kh2 = compute_Kh(Th2, TT2, T2, eta2, mu2);  // :128

  M3 Kt11 = ((tr(Bp11) * Kh1) * Bp11 + (tr(Bp21) * Kh2) * Bp21) + Km11;  // :131
  M3 Kt12 = ((tr(Bp11) * Kh1) * Bp12 + (tr(Bp21) * Kh2) * Bp22) + Km12;
  M3 Kt14 = ((tr(Bp11) * Kh1) * Bp14 + (tr(Bp21) * Kh2) * Bp24) + Km14;
  M3 Kt22 = ((tr(Bp12) * Kh1) * Bp12 + (tr(Bp22) * Kh2) * Bp22) + Km22;
  M3 Kt24 = ((tr(Bp12) * Kh1) * Bp14 + (tr(Bp22) * Kh2) * Bp24) + Km24;
  M3 Kt44 = ((tr(Bp14) * Kh1) * Bp14 + (tr(Bp24) * Kh2) * Bp24) + Km44;

  auto BKB = [&](const M3& Ba1, const M3& Ba2, const M3& Bb1, const M3& Bb2) {  // :140-146 pattern
    return tr(Ba1) * (dmul(KT, Bb1) + dmul(KTT, Bb2)) + tr(Ba2) * (dmul(KTT, Bb1) + dmul(KT, Bb2));
  };
  M3 BKB11 = (outer(B1 * Ku, B1) + tr(B11) * (dmul(KT, B11) + dmul(KTT, B21))) +
             tr(B21) * (dmul(KTT, B11) + dmul(KT, B21));  // :139
  M3 BKB12 = BKB(B11, B21, B12, B22);
  M3 BKB14 = BKB(B11, B21, B14, B24);
  M3 BKB22 = BKB(B12, B22, B12, B22);
  M3 BKB24 = BKB(B12, B22, B14, B24);
  M3 BKB44 = BKB(B14, B24, B14, B24);

  M3 K11 = BKB11 + Kt11, K12 = BKB12 + Kt12, K13 = -K11, K14 = BKB14 + Kt14;  // :148-157
  M3 K22 = BKB22 + Kt22, K23 = -tr(K12), K24 = BKB24 + Kt24;
  M3 K33 = K11, K34 = -K14, K44 = BKB44 + Kt44;

  double* Kout = out + EO_K;  // :159
  put(Kout, 0, 0, K11); put(Kout, 1, 0, tr(K12)); put(Kout, 2, 0, tr(K13)); put(Kout, 3, 0, tr(K14));
  put(Kout, 0, 1, K12); put(Kout, 1, 1, K22); put(Kout, 2, 1, tr(K23)); put(Kout, 3, 1, tr(K24));
  put(Kout, 0, 2, K13); put(Kout, 1, 2, K23); put(Kout, 2, 2, K33); put(Kout, 3, 2, tr(K34));
  put(Kout, 0, 3, K14); put(Kout, 1, 3, K24); put(Kout, 2, 3, K34); put(Kout, 3, 3, K44);

  double kinetic_energy = 0.0;  // :161
  V3 Tk1 = zv3(), Tk2 = zv3(), Tk3 = zv3(), Tk4 = zv3();
  M3 M11 = zm3(), M12 = zm3(), M13 = zm3(), M14 = zm3(), M21 = zm3(), M22 = zm3(), M23 = zm3(), M24 = zm3();
  M3 M31 = zm3(), M32 = zm3(), M33 = zm3(), M34 = zm3(), M41 = zm3(), M42 = zm3(), M43 = zm3(), M44 = zm3();
  M3 C11 = zm3(), C12 = zm3(), C13 = zm3(), C14 = zm3(), C21 = zm3(), C22 = zm3(), C23 = zm3(), C24 = zm3();
  M3 C31 = zm3(), C32 = zm3(), C33 = zm3(), C34 = zm3(), C41 = zm3(), C42 = zm3(), C43 = zm3(), C44 = zm3();

  // isdynamic branch, :202-519
  V3 Ud1 = ReT * ud1, Ud2 = ReT * ud2, Wd1 = ReT * wd1, Wd2 = ReT * wd2;
  V3 Udd1 = ReT * udd1, Udd2 = ReT * udd2, Wdd1 = ReT * wdd1, Wdd2 = ReT * wdd2;
  M3 SUd1 = skew(Ud1), SUd2 = skew(Ud2), SWd1 = skew(Wd1), SWd2 = skew(Wd2);
  V3 We = ((G1 * Ud1 + G2 * Wd1) + G3 * Ud2) + G4 * Wd2;  // :219
  M3 SWe = skew(We);
  double rd = dot(r1, ud1) + dot(r3, ud2);  // :222
  const M3 Jm = diag3(Jr[0], Jr[1], Jr[2]);

  for (int ig = 0; ig < g.n; ++ig) {  // :233
    double zg = g.z[ig], wg = g.w[ig];
    double xi = l0 * (zg + 1) / 2;
    double N1 = 1 - xi / l0;
    double N2 = 1 - N1;
    double N3 = xi * ((1 - xi / l0) * (1 - xi / l0));
    double N4 = -(1 - xi / l0) * ((xi * xi) / l0);
    double N5 = (1 - 3 * xi / l0) * (1 - xi / l0);
    double N6 = (3 * xi / l0 - 2) * (xi / l0);
    double N7 = N3 + N4;
    double N8 = N5 + N6 - 1;

    V3 ut = v3(0.0, N3 * Th1[2] + N4 * Th2[2], -N3 * Th1[1] + -N4 * Th2[1]);          // :250
    V3 Thb = v3(N1 * Th1[0] + N2 * Th2[0], N5 * Th1[1] + N6 * Th2[1], N5 * Th1[2] + N6 * Th2[2]);  // :251
    M3 Sut = skew(ut), SThb = skew(Thb);
    M3 Rb = I3 + SThb;
    M3 Ir = (Rb * Jm) * tr(Rb);  // :258

    double N7l = N7 / ln, N7l2 = N7l / ln, N8l = N8 / ln, N8l2 = N8l / ln;
    M3 P1P1 = rows(0, 0, 0, 0, N7l, 0, 0, 0, N7l);
    M3 P1P2 = rows(0, 0, 0, 0, 0, N3, 0, -N3, 0);
    M3 P1P3 = -P1P1;
    M3 P1P4 = rows(0, 0, 0, 0, 0, N4, 0, -N4, 0);

    M3 H11 = (N1 * I3 + P1P1) - Sut * G1;  // :270
    M3 H12 = P1P2 - Sut * G2;
    M3 H13 = (N2 * I3 + P1P3) - Sut * G3;
    M3 H14 = P1P4 - Sut * G4;

    M3 H21 = rows(0, 0, 0, 0, 0, -N8l, 0, N8l, 0);  // :275
    M3 H22 = diag3(N1, N5, N5);
    M3 H23 = -H21;
    M3 H24 = diag3(N2, N6, N6);

    V3 udt = ((P1P1 * Ud1 + P1P2 * Wd1) + P1P3 * Ud2) + P1P4 * Wd2;  // :280
    M3 Sudt = skew(udt);
    double N7rd = N7l2 * rd;
    M3 Hd11 = diag3(0, -N7rd, -N7rd) - Sudt * G1;
    M3 Hd12 = -(Sudt * G2);
    M3 Hd14 = -(Sudt * G4);
    double N8rd = N8l2 * rd;
    M3 Hd21 = rows(0, 0, 0, 0, 0, N8rd, 0, -N8rd, 0);

    V3 h1 = ((H11 * Ud1 + H12 * Wd1) + H13 * Ud2) + H14 * Wd2;  // :292
    V3 h2 = ((H21 * Ud1 + H22 * Wd1) + H23 * Ud2) + H24 * Wd2;
    M3 Sh1 = skew(h1), Sh2 = skew(h2);

    M3 C1_1 = (SWe * H11 + Hd11) - H11 * SWe;  // :297
    M3 C1_2 = (SWe * H12 + Hd12) - H12 * SWe;
    M3 C1_3 = -C1_1;
    M3 C1_4 = (SWe * H14 + Hd14) - H14 * SWe;
    M3 C2_1 = (SWe * H21 + Hd21) - H21 * SWe;
    M3 C2_2 = SWe * H22 - H22 * SWe;
    M3 C2_3 = -C2_1;
    M3 C2_4 = SWe * H24 - H24 * SWe;

    M3 H1F1 = ((H11 * SUd1 + H12 * SWd1) + H13 * SUd2) + H14 * SWd2;  // :307
    M3 H2F1 = ((H21 * SUd1 + H22 * SWd1) + H23 * SUd2) + H24 * SWd2;

    M3 A1DrE1 = rows(0, 0, 0, Ud1[1] - Ud2[1], 0, 0, Ud1[2] - Ud2[2], 0, 0);  // :310
    M3 C3_1 = ((-(Sh1 * G1) + N7l2 * A1DrE1) + SWe * P1P1) + H1F1 * G1;
    M3 C3_2 = (-(Sh1 * G2) + SWe * P1P2) + H1F1 * G2;
    M3 C3_4 = (-(Sh1 * G4) + SWe * P1P4) + H1F1 * G4;
    M3 A2DrE1 = rows(0, 0, 0, -Ud1[2] + Ud2[2], 0, 0, Ud1[1] - Ud2[1], 0, 0);  // :315
    M3 C4_1 = (-(Sh2 * G1) + N8l2 * A2DrE1) + H2F1 * G1;
    M3 C4_2 = -(Sh2 * G2) + H2F1 * G2;
    M3 C4_4 = -(Sh2 * G4) + H2F1 * G4;

    V3 ud0 = Re * h1;  // :320
    V3 H1Edd = ((H11 * Udd1 + H12 * Wdd1) + H13 * Udd2) + H14 * Wdd2;
    V3 C1Ed = ((C1_1 * Ud1 + C1_2 * Wd1) + C1_3 * Ud2) + C1_4 * Wd2;
    V3 ReTudd0 = H1Edd + C1Ed;
    V3 W0 = h2;
    V3 wd0 = Re * W0;
    V3 H2Edd = ((H21 * Udd1 + H22 * Wdd1) + H23 * Udd2) + H24 * Wdd2;
    V3 C2Ed = ((C2_1 * Ud1 + C2_2 * Wd1) + C2_3 * Ud2) + C2_4 * Wd2;
    V3 ReTwdd0 = H2Edd + C2Ed;

    M3 SW0 = skew(W0);  // :333
    V3 IrReTwdd0 = Ir * ReTwdd0;
    M3 SW0Ir = SW0 * Ir;
    V3 SW0IrW0 = SW0Ir * W0;
    V3 Fw = IrReTwdd0 + SW0IrW0;
    M3 ArH11T = Ar * tr(H11), ArH12T = Ar * tr(H12), ArH13T = Ar * tr(H13), ArH14T = Ar * tr(H14);
    (void)ArH13T;

    V3 Tk1G = wg * (ArH11T * ReTudd0 + tr(H21) * Fw);  // :343
    Tk1 += Tk1G;
    Tk2 += wg * (ArH12T * ReTudd0 + tr(H22) * Fw);
    Tk3 += -Tk1G + (wg * Ar) * ReTudd0;
    Tk4 += wg * (ArH14T * ReTudd0 + tr(H24) * Fw);

    if (damping > 0) {  // :349
      V3 Td1G = (wg * damping) * (ArH11T * h1 + tr(H21) * (Ir * h2));
      Tk1 += Td1G;
      Tk2 += (wg * damping) * (ArH12T * h1 + tr(H22) * (Ir * h2));
      Tk3 += -Td1G + ((wg * Ar) * damping) * h1;
      Tk4 += (wg * damping) * (ArH14T * h1 + tr(H24) * (Ir * h2));
    }

    M3 M11G = wg * (ArH11T * H11 + (tr(H21) * Ir) * H21);  // :357
    M3 M12G = wg * (ArH11T * H12 + (tr(H21) * Ir) * H22);
    M3 M14G = wg * (ArH11T * H14 + (tr(H21) * Ir) * H24);
    M3 M22G = wg * (ArH12T * H12 + (tr(H22) * Ir) * H22);
    M3 M24G = wg * (ArH12T * H14 + (tr(H22) * Ir) * H24);
    M3 M44G = wg * (ArH14T * H14 + (tr(H24) * Ir) * H24);

    M11 += M11G;  // :366
    M12 += M12G;
    M13 += -M11G + wg * ArH11T;
    M14 += M14G;
    M22 += M22G;
    M23 += -tr(M12G) + wg * ArH12T;
    M24 += M24G;
    M33 += M11G + (wg * Ar) * ((I3 - H11) - tr(H11));
    M34 += -M14G + (wg * Ar) * H14;
    M44 += M44G;

    M3 SW0IrmSIrW0 = SW0Ir - skew(Ir * W0);  // :380
    M3 ArC13_1 = Ar * (C1_1 + C3_1);
    M3 ArC13_2 = Ar * (C1_2 + C3_2);
    M3 ArC13_4 = Ar * (C1_4 + C3_4);
    M3 X1m = Ir * (C2_1 + C4_1) + SW0IrmSIrW0 * H21;  // :386
    M3 X2m = Ir * (C2_2 + C4_2) + SW0IrmSIrW0 * H22;
    M3 X4m = Ir * (C2_4 + C4_4) + SW0IrmSIrW0 * H24;

    M3 C11G = wg * (tr(H11) * ArC13_1 + tr(H21) * X1m);  // :390
    M3 C12G = wg * (tr(H11) * ArC13_2 + tr(H21) * X2m);
    M3 C14G = wg * (tr(H11) * ArC13_4 + tr(H21) * X4m);
    M3 C21G = wg * (tr(H12) * ArC13_1 + tr(H22) * X1m);
    M3 C22G = wg * (tr(H12) * ArC13_2 + tr(H22) * X2m);
    M3 C24G = wg * (tr(H12) * ArC13_4 + tr(H22) * X4m);
    M3 C41G = wg * (tr(H14) * ArC13_1 + tr(H24) * X1m);
    M3 C42G = wg * (tr(H14) * ArC13_2 + tr(H24) * X2m);
    M3 C44G = wg * (tr(H14) * ArC13_4 + tr(H24) * X4m);

    C11 += C11G; C12 += C12G; C14 += C14G;  // :402
    C21 += C21G; C22 += C22G; C24 += C24G;
    C31 += -C11G + wg * ArC13_1;
    C32 += -C12G + wg * ArC13_2;
    C34 += -C14G + wg * ArC13_4;
    C41 += C41G; C42 += C42G; C44 += C44G;

    M3 Irg = (Re * Ir) * ReT;  // :418
    kinetic_energy += wg / 2 * ((Ar * dot(ud0, ud0)) + dot(wd0, Irg * wd0));
  }

  double l02 = l0 / 2;  // :423
  M3 l02Re = l02 * Re;
  Tk1 = l02Re * Tk1; Tk2 = l02Re * Tk2; Tk3 = l02Re * Tk3; Tk4 = l02Re * Tk4;
  auto sc = [&](const M3& X) { return (l02Re * X) * ReT; };
  M11 = sc(M11); M12 = sc(M12); M13 = sc(M13); M14 = sc(M14); M22 = sc(M22);
  M23 = sc(M23); M24 = sc(M24); M33 = sc(M33); M34 = sc(M34); M44 = sc(M44);
  C11 = sc(C11); C12 = sc(C12); C13 = -C11; C14 = sc(C14);  // :442
  C21 = sc(C21); C22 = sc(C22); C23 = -C21; C24 = sc(C24);
  C31 = sc(C31); C32 = sc(C32); C33 = -C31; C34 = sc(C34);
  C41 = sc(C41); C42 = sc(C42); C43 = -C41; C44 = sc(C44);
  kinetic_energy = l02 * kinetic_energy;

  if (damping > 0) {  // :461
    C11 += damping * M11; C12 += damping * M12; C13 += damping * M13; C14 += damping * M14;
    C21 += damping * tr(M12); C22 += damping * M22; C23 += damping * M23; C24 += damping * M24;
    C31 += damping * tr(M13); C32 += damping * tr(M23); C33 += damping * M33; C34 += damping * M34;
    C41 += damping * tr(M14); C42 += damping * tr(M24); C43 += damping * tr(M34); C44 += damping * M44;
  }

  // exact branch, :480-506 — sequential reassignment semantics kept
  V3 Tha = toangle(dR1), Thb2 = toangle(dR2);
  M3 Ta = Ts_inv(Tha), Tb = Ts_inv(Thb2);
  M3 TaT = tr(Ta), TbT = tr(Tb);
  M21 = tr(M12) * TaT;
  M22 = M22 * TaT;
  M23 = M23 * TaT;
  M24 = M24 * TaT;
  M31 = tr(M13);
  M32 = tr(M23);
  M41 = tr(M14) * TbT;
  M42 = tr(M24) * TbT;
  M43 = tr(M34) * TbT;
  M44 = M44 * TbT;
  C21 = C21 * TaT; C22 = C22 * TaT; C23 = C23 * TaT; C24 = C24 * TaT;
  C41 = C41 * TbT; C42 = C42 * TbT; C43 = C43 * TbT; C44 = C44 * TbT;

  out[EO_ES] = strain_energy;
  out[EO_EK] = kinetic_energy;
  double* Ti = out + EO_TINT;
  putv(Ti, 0, Ti1); putv(Ti, 1, Ti2); putv(Ti, 2, Ti3); putv(Ti, 3, Ti4);
  double* Tk = out + EO_TK;
  putv(Tk, 0, Tk1); putv(Tk, 1, Tk2); putv(Tk, 2, Tk3); putv(Tk, 3, Tk4);
  double* Mo = out + EO_M;  // :522
  put(Mo, 0, 0, M11); put(Mo, 0, 1, M12); put(Mo, 0, 2, M13); put(Mo, 0, 3, M14);
  put(Mo, 1, 0, M21); put(Mo, 1, 1, M22); put(Mo, 1, 2, M23); put(Mo, 1, 3, M24);
  put(Mo, 2, 0, M31); put(Mo, 2, 1, M32); put(Mo, 2, 2, M33); put(Mo, 2, 3, M34);
  put(Mo, 3, 0, M41); put(Mo, 3, 1, M42); put(Mo, 3, 2, M43); put(Mo, 3, 3, M44);
  double* Co = out + EO_C;  // :529
  put(Co, 0, 0, C11); put(Co, 0, 1, C12); put(Co, 0, 2, C13); put(Co, 0, 3, C14);
  put(Co, 1, 0, C21); put(Co, 1, 1, C22); put(Co, 1, 2, C23); put(Co, 1, 3, C24);
  put(Co, 2, 0, C31); put(Co, 2, 1, C32); put(Co, 2, 2, C33); put(Co, 2, 3, C34);
  put(Co, 3, 0, C41); put(Co, 3, 1, C42); put(Co, 3, 2, C43); put(Co, 3, 3, C44);
}

}  // namespace orc
