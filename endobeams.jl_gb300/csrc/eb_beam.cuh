// Corotational beam element on the GPU: one thread per element, FP64.
//
// Same quantities as compute_beams (src/beams/compute_beams.jl:1-538, the
// `exact=true, isdynamic=true` path used by assemble!): strain and kinetic
// energy, Tⁱⁿᵗ, Tᵏ (12) and Kⁱⁿᵗ, M, Cᵏ (12x12, column-major).  The
// formulas are the reference's; the evaluation exploits their structure
// (sparse Gᵀ/P/H₂ matrices, skew commutators, reuse of Bᵀ·K̄ₕ products) to
// cut FP64 instructions, which bound this kernel on GB300.
#pragma once
#include "eb_device_math.cuh"

namespace ebd {

struct BeamIn {
  V3 X1, X2, u1, u2, ud1, ud2, wd1, wd2, udd1, udd2, wdd1, wdd2;
  M3 R1, R2, dR1, dR2, Re0;
  double l0, Ku, Ar, damping;
  V3 KT, KTT, Jr;
};

struct BeamOut {  // destinations (any stride-1 buffers)
  double* K;    // 144
  double* M;    // 144
  double* C;    // 144
  double* Tint; // 12
  double* Tk;   // 12
  double* E;    // 2: strain, kinetic
};

struct Gauss3 {
  double w[3], z[3];
};

EB_DEV void put_block(double* m, int bi, int bj, const M3& b) {
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) m[(3 * bi + i) + 12 * (3 * bj + j)] = b(i, j);
}
EB_DEV void put_blockT(double* m, int bi, int bj, const M3& b) {
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) m[(3 * bi + i) + 12 * (3 * bj + j)] = b(j, i);
}
EB_DEV void put_vec(double* v, int bi, V3 x) { v[3 * bi] = x.x; v[3 * bi + 1] = x.y; v[3 * bi + 2] = x.z; }
EB_DEV M3 get_block(const double* m, int bi, int bj) {
  M3 b;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) b(i, j) = m[(3 * bi + i) + 12 * (3 * bj + j)];
  return b;
}
// block (bi, bj) of a 12x12 column-major matrix += s q (fused multiply-add per entry)
EB_DEV void acc_block(double* m, int bi, int bj, double s, const M3& q) {
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double& x = m[(3 * bi + i) + 12 * (3 * bj + j)];
      x = fma(s, q(i, j), x);
    }
}

// Element frame and auxiliaries of local_Rₑ_and_aux (utils_beams.jl:35-87).
struct Frame {
  M3 Re;
  V3 v1;
  double eta, ln;
  Gu G1;      // Gᵀ¹ ; Gᵀ³ = -Gᵀ¹
  Gt G2, G4;  // Gᵀ², Gᵀ⁴
};

EB_DEV Frame local_frame(V3 x1, V3 x2, const M3& R1, const M3& R2, V3 e2, double ln) {
  Frame f;
  f.ln = ln;
  V3 v1 = (1.0 / ln) * (x2 - x1);
  V3 p1 = R1 * e2, p2 = R2 * e2;
  V3 p = 0.5 * (p1 + p2);
  V3 v3_ = cross(v1, p);
  v3_ = (1.0 / norm(v3_)) * v3_;
  V3 v2 = cross(v3_, v1);
  f.Re = hcat3(v1, v2, v3_);
  f.v1 = v1;
  double q2 = dot(v2, p);
  double iq2 = 1.0 / q2;
  double eta = dot(v1, p) * iq2;
  double eta11 = dot(v1, p1) * iq2, eta12 = dot(v2, p1) * iq2;
  double eta21 = dot(v1, p2) * iq2, eta22 = dot(v2, p2) * iq2;
  f.eta = eta;
  double il = 1.0 / ln;
  f.G1 = Gu{eta * il, il, -il};
  f.G2 = Gt{eta12 / 2, -eta11 / 2};
  f.G4 = Gt{eta22 / 2, -eta21 / 2};
  return f;
}

// compute_K̄ₕ (utils_beams.jl:201-215)
EB_DEV M3 compute_Kh(V3 th, V3 Mb, const M3& Ts, double eta, double mu) {
  M3 MtT = outer(Mb, th);  // M̄Θ̅ᵀ
  M3 inner = eta * (outer(th, Mb) - 2.0 * MtT);
  double d = eta * dot(th, Mb);
  inner.a[0] += d; inner.a[4] += d; inner.a[8] += d;
  axpy(inner, mu, skewmul(th, skewmul(th, MtT)));
  axpy(inner, -0.5, skew(Mb));
  return inner * Ts;
}

// Gᵀ v for the GᵀΘ shape [a b 0; 0 0 0; 0 0 0]
EB_DEV V3 GTv(Gt g, V3 v) { return v3(g.a * v.x, g.b * v.x, 0.0); }

EB_DEV void beam_element(const BeamIn& in, const Gauss3& gs, BeamOut out) {
  const M3 I3 = eye3();
  // ------------------------------------------------------------ static part (:13-159)
  V3 x1 = in.X1 + in.u1, x2 = in.X2 + in.u2;
  double ln = norm(x2 - x1);
  double ubar = ln - in.l0;
  Frame f = local_frame(x1, x2, in.R1, in.R2, col(in.Re0, 1), ln);
  const M3& Re = f.Re;
  const M3 ReT = tr(Re);
  const V3 r1 = -f.v1;  // B̄⁺¹ = ru₁
  const Gu G1 = f.G1;
  const Gt G2 = f.G2, G4 = f.G4;

  V3 Th1 = toangle(mulTN(Re, in.R1) * in.Re0);
  V3 Th2 = toangle(mulTN(Re, in.R2) * in.Re0);
  M3 T1 = Ts_inv(Th1), T2 = Ts_inv(Th2);

  M3 G1ReT = Gmul(G1, ReT), G2ReT = Gmul(G2, ReT), G4ReT = Gmul(G4, ReT);
  M3 Bp11 = -G1ReT;          // P¹¹Rₑᵀ = B̄⁺¹¹ = B̄⁺²¹
  M3 Bp12 = ReT - G2ReT;     // (I-Gᵀ²)Rₑᵀ
  M3 Bp22 = -G2ReT;
  M3 Bp14 = -G4ReT;
  M3 Bp24 = ReT - G4ReT;
  M3 B11 = T1 * Bp11, B12 = T1 * Bp12, B14 = T1 * Bp14;
  M3 B21 = T2 * Bp11, B22 = T2 * Bp22, B24 = T2 * Bp24;

  double Tu = in.Ku * ubar;
  V3 TT1 = dmulv(in.KT, Th1) + dmulv(in.KTT, Th2);
  V3 TT2 = dmulv(in.KTT, Th1) + dmulv(in.KT, Th2);
  double strain_energy = (ubar * Tu + dot(Th1, TT1) + dot(Th2, TT2)) / 2;

  V3 Ti1 = Tu * r1 + mulTv(B11, TT1) + mulTv(B21, TT2);
  V3 Ti2 = mulTv(B12, TT1) + mulTv(B22, TT2);
  V3 Ti4 = mulTv(B14, TT1) + mulTv(B24, TT2);

  V3 Mp1 = mulTv(T1, TT1), Mp2 = mulTv(T2, TT2);
  V3 Mps = Mp1 + Mp2;
  V3 Qs1 = -GTv(G1, Mps);                       // P¹¹ᵀM̄⁺₁ + P²¹ᵀM̄⁺₂
  V3 Qs2 = Mp1 - GTv(G2, Mps);                  // (I-Gᵀ²)ᵀM̄⁺₁ - Gᵀ²ᵀM̄⁺₂
  V3 Qs4 = Mp2 - GTv(G4, Mps);                  // -Gᵀ⁴ᵀM̄⁺₁ + (I-Gᵀ⁴)ᵀM̄⁺₂
  M3 Q1 = skew(Qs1), Q2 = skew(Qs2), Q4 = skew(Qs4);
  double il = 1.0 / ln;
  V3 a = v3(0.0, f.eta * Mps.x * il + Mps.y * il, Mps.z * il);
  // D₃ N̄ = (I - v₁v₁ᵀ) N̄ / lₙ
  M3 Km11 = (Tu * il) * (I3 - outer(f.v1, f.v1));
  Km11 = Km11 - (Re * mulG(Q1, G1)) * ReT;
  Km11 += outer(Re * GTv(G1, a), r1);
  M3 Km12 = -((Re * mulG(Q1, G2)) * ReT);
  M3 Km14 = -((Re * mulG(Q1, G4)) * ReT);
  M3 Km22 = -((Re * mulG(Q2, G2)) * ReT);
  M3 Km24 = -((Re * mulG(Q2, G4)) * ReT);
  M3 Km44 = -((Re * mulG(Q4, G4)) * ReT);

  double eta1, mu1, eta2, mu2;
  compute_eta_mu(Th1, &eta1, &mu1);
  compute_eta_mu(Th2, &eta2, &mu2);
  M3 Kh1 = compute_Kh(Th1, TT1, T1, eta1, mu1);
  M3 Kh2 = compute_Kh(Th2, TT2, T2, eta2, mu2);

  // K̃ (:131-136) with the B̄⁺ᵀK̄ₕ left factors shared between blocks
  M3 Y11 = mulTN(Bp11, Kh1), Y21 = mulTN(Bp11, Kh2);
  M3 Kt11 = Y11 * Bp11 + Y21 * Bp11 + Km11;
  M3 Kt12 = Y11 * Bp12 + Y21 * Bp22 + Km12;
  M3 Kt14 = Y11 * Bp14 + Y21 * Bp24 + Km14;
  M3 Y12 = mulTN(Bp12, Kh1), Y22 = mulTN(Bp22, Kh2);
  M3 Kt22 = Y12 * Bp12 + Y22 * Bp22 + Km22;
  M3 Kt24 = Y12 * Bp14 + Y22 * Bp24 + Km24;
  M3 Kt44 = mulTN(Bp14, Kh1) * Bp14 + mulTN(Bp24, Kh2) * Bp24 + Km44;

  // BᵀK̄ⁱⁿᵗB (:139-146)
  M3 Z11 = dmul(in.KT, B11) + dmul(in.KTT, B21), Z21 = dmul(in.KTT, B11) + dmul(in.KT, B21);
  M3 Z12 = dmul(in.KT, B12) + dmul(in.KTT, B22), Z22 = dmul(in.KTT, B12) + dmul(in.KT, B22);
  M3 Z14 = dmul(in.KT, B14) + dmul(in.KTT, B24), Z24 = dmul(in.KTT, B14) + dmul(in.KT, B24);
  M3 K11 = outer(in.Ku * r1, r1) + mulTN(B11, Z11) + mulTN(B21, Z21) + Kt11;
  M3 K12 = mulTN(B11, Z12) + mulTN(B21, Z22) + Kt12;
  M3 K14 = mulTN(B11, Z14) + mulTN(B21, Z24) + Kt14;
  M3 K22 = mulTN(B12, Z12) + mulTN(B22, Z22) + Kt22;
  M3 K24 = mulTN(B12, Z14) + mulTN(B22, Z24) + Kt24;
  M3 K44 = mulTN(B14, Z14) + mulTN(B24, Z24) + Kt44;

  // Kⁱⁿᵗ layout of :159 (blocks below the diagonal are transposes)
  {
    // K¹³ = -K¹¹, K²³ = -K¹²ᵀ, K³³ = K¹¹, K³⁴ = -K¹⁴ (:150-156)
    double* K = out.K;
    M3 K13 = -K11, K34 = -K14, mK12 = -K12;
    put_block(K, 0, 0, K11);  put_blockT(K, 1, 0, K12);  put_blockT(K, 2, 0, K13); put_blockT(K, 3, 0, K14);
    put_block(K, 0, 1, K12);  put_block(K, 1, 1, K22);   put_block(K, 2, 1, mK12); put_blockT(K, 3, 1, K24);
    put_block(K, 0, 2, K13);  put_blockT(K, 1, 2, mK12); put_block(K, 2, 2, K11);  put_blockT(K, 3, 2, K34);
    put_block(K, 0, 3, K14);  put_block(K, 1, 3, K24);   put_block(K, 2, 3, K34);  put_block(K, 3, 3, K44);
  }

  // ------------------------------------------------------------ dynamic part (:202-519)
  V3 Ud1 = mulTv(Re, in.ud1), Ud2 = mulTv(Re, in.ud2), Wd1 = mulTv(Re, in.wd1), Wd2 = mulTv(Re, in.wd2);
  V3 Udd1 = mulTv(Re, in.udd1), Udd2 = mulTv(Re, in.udd2), Wdd1 = mulTv(Re, in.wdd1), Wdd2 = mulTv(Re, in.wdd2);
  V3 dU = Ud1 - Ud2, dUdd = Udd1 - Udd2;
  V3 We = Gv(G1, dU) + Gv(G2, Wd1) + Gv(G4, Wd2);  // Gᵀ³ = -Gᵀ¹
  double rd = dot(r1, in.ud1) - dot(r1, in.ud2);     // r³ = -r¹
  const double Ar = in.Ar, damping = in.damping;
  const V3 Jr = in.Jr;

  double kinetic = 0.0;
  V3 Tk1 = zv3(), Tk2 = zv3(), Tk3 = zv3(), Tk4 = zv3();
  // accumulators: M11 M12 M13 M14 M22 M23 M24 M33 M34 M44
  M3 Ma[10];
  // accumulators: C11 C12 C14 C21 C22 C24 C31 C32 C34 C41 C42 C44
  M3 Ca[12];
#pragma unroll
  for (int k = 0; k < 10; ++k) Ma[k] = zm3();
#pragma unroll
  for (int k = 0; k < 12; ++k) Ca[k] = zm3();

#pragma unroll 1
  for (int ig = 0; ig < 3; ++ig) {
    const double zg = gs.z[ig], wg = gs.w[ig];
    const double l0 = in.l0;
    double xi = l0 * (zg + 1) / 2;
    double s = xi / l0;
    double N1 = 1 - s;
    double N2 = 1 - N1;
    double N3 = xi * ((1 - s) * (1 - s));
    double N4 = -(1 - s) * ((xi * xi) / l0);
    double N5 = (1 - 3 * s) * (1 - s);
    double N6 = (3 * s - 2) * s;
    double N7 = N3 + N4;
    double N8 = N5 + N6 - 1;

    V3 ut = v3(0.0, N3 * Th1.z + N4 * Th2.z, -N3 * Th1.y - N4 * Th2.y);
    V3 Thb = v3(N1 * Th1.x + N2 * Th2.x, N5 * Th1.y + N6 * Th2.y, N5 * Th1.z + N6 * Th2.z);
    M3 Rb = I3 + skew(Thb);
    M3 Ir = mulNT(muld(Rb, Jr), Rb);  // R̄ Jᵨ R̄ᵀ

    double N7l = N7 * il, N7l2 = N7l * il, N8l = N8 * il, N8l2 = N8l * il;
    M3 Sut = skew(ut);
    M3 SutG1 = mulG(Sut, G1);
    M3 P1P2 = rows(0, 0, 0, 0, 0, N3, 0, -N3, 0);
    M3 P1P4 = rows(0, 0, 0, 0, 0, N4, 0, -N4, 0);
    M3 H11 = diag3(N1, N1 + N7l, N1 + N7l) - SutG1;
    M3 H12 = P1P2 - mulG(Sut, G2);
    M3 H13 = diag3(N2, N2 - N7l, N2 - N7l) + SutG1;
    M3 H14 = P1P4 - mulG(Sut, G4);
    const V3 s21 = v3(N8l, 0.0, 0.0);  // H₂¹ = skew(s21), H₂³ = -H₂¹
    const V3 d22 = v3(N1, N5, N5), d24 = v3(N2, N6, N6);

    V3 udt = v3(0.0, N7l * dU.y + N3 * Wd1.z + N4 * Wd2.z, N7l * dU.z - N3 * Wd1.y - N4 * Wd2.y);
    M3 Sudt = skew(udt);
    double N7rd = N7l2 * rd, N8rd = N8l2 * rd;
    M3 Hd11 = diag3(0.0, -N7rd, -N7rd) - mulG(Sudt, G1);
    M3 Hd12 = -mulG(Sudt, G2);
    M3 Hd14 = -mulG(Sudt, G4);

    V3 h1 = H11 * Ud1 + H12 * Wd1 + H13 * Ud2 + H14 * Wd2;
    V3 h2 = cross(s21, dU) + dmulv(d22, Wd1) + dmulv(d24, Wd2);

    M3 C11_ = skewmul(We, H11) + Hd11 - mulskew(H11, We);   // C₁¹
    M3 C12_ = skewmul(We, H12) + Hd12 - mulskew(H12, We);   // C₁²
    M3 C14_ = skewmul(We, H14) + Hd14 - mulskew(H14, We);   // C₁⁴
    // C₂¹ = [S(Ẇᵉ), S(s21)] + Ḣ₂¹ = S(Ẇᵉ × s21) + S((-N₈ṙ,0,0))
    M3 C21_ = skew(cross(We, s21) + v3(-N8rd, 0.0, 0.0));
    // C₂² = S(Ẇᵉ)D - D S(Ẇᵉ) for D = diag(d): entry (i,j) scales by d_j - d_i
    double e2 = N5 - N1, e4 = N6 - N2;
    M3 C22_ = rows(0, -We.z * e2, We.y * e2, -We.z * e2, 0, 0, We.y * e2, 0, 0);
    M3 C24_ = rows(0, -We.z * e4, We.y * e4, -We.z * e4, 0, 0, We.y * e4, 0, 0);

    M3 H1F1 = mulskew(H11, Ud1) + mulskew(H12, Wd1) + mulskew(H13, Ud2) + mulskew(H14, Wd2);
    M3 H2F1 = skewmul(s21, skew(dU)) + dmul(d22, skew(Wd1)) + dmul(d24, skew(Wd2));
    M3 Sh1 = skew(h1), Sh2 = skew(h2);

    M3 A1 = rows(0, 0, 0, N7l2 * dU.y, 0, 0, N7l2 * dU.z, 0, 0);
    M3 C31_ = mulG(H1F1 - Sh1, G1) + A1 + muld(skew(We), v3(0.0, N7l, N7l));
    M3 C32_ = mulG(H1F1 - Sh1, G2) + skewmul(We, P1P2);
    M3 C34_ = mulG(H1F1 - Sh1, G4) + skewmul(We, P1P4);
    M3 A2 = rows(0, 0, 0, -N8l2 * dU.z, 0, 0, N8l2 * dU.y, 0, 0);
    M3 C41_ = mulG(H2F1 - Sh2, G1) + A2;
    M3 C42_ = mulG(H2F1 - Sh2, G2);
    M3 C44_ = mulG(H2F1 - Sh2, G4);

    V3 ud0 = Re * h1;
    V3 ReTudd0 = (H11 * Udd1 + H12 * Wdd1 + H13 * Udd2 + H14 * Wdd2) + (C11_ * dU + C12_ * Wd1 + C14_ * Wd2);
    V3 W0 = h2;
    V3 ReTwdd0 = (cross(s21, dUdd) + dmulv(d22, Wdd1) + dmulv(d24, Wdd2)) + (C21_ * dU + C22_ * Wd1 + C24_ * Wd2);
    V3 IrW0 = Ir * W0;
    V3 Fw = Ir * ReTwdd0 + cross(W0, IrW0);

    V3 Tk1G = wg * (Ar * mulTv(H11, ReTudd0) - cross(s21, Fw));  // H₂¹ᵀ = -S(s21)
    Tk1 += Tk1G;
    Tk2 += wg * (Ar * mulTv(H12, ReTudd0) + dmulv(d22, Fw));
    Tk3 += (wg * Ar) * ReTudd0 - Tk1G;
    Tk4 += wg * (Ar * mulTv(H14, ReTudd0) + dmulv(d24, Fw));
    if (damping > 0) {
      V3 Irh2 = Ir * h2;
      V3 Td1G = (wg * damping) * (Ar * mulTv(H11, h1) - cross(s21, Irh2));
      Tk1 += Td1G;
      Tk2 += (wg * damping) * (Ar * mulTv(H12, h1) + dmulv(d22, Irh2));
      Tk3 += ((wg * Ar) * damping) * h1 - Td1G;
      Tk4 += (wg * damping) * (Ar * mulTv(H14, h1) + dmulv(d24, Irh2));
    }

    // mass blocks (:357-378)
    M3 H21TIr = -skewmul(s21, Ir);
    const double wA = wg * Ar;
    M3 M11G = wA * mulTN(H11, H11) + wg * mulskew(H21TIr, s21);
    M3 M12G = wA * mulTN(H11, H12) + wg * muld(H21TIr, d22);
    M3 M14G = wA * mulTN(H11, H14) + wg * muld(H21TIr, d24);
    M3 M22G = wA * mulTN(H12, H12) + wg * dmul(d22, muld(Ir, d22));
    M3 M24G = wA * mulTN(H12, H14) + wg * dmul(d22, muld(Ir, d24));
    M3 M44G = wA * mulTN(H14, H14) + wg * dmul(d24, muld(Ir, d24));
    Ma[0] += M11G;
    Ma[1] += M12G;
    Ma[2] += wA * tr(H11) - M11G;
    Ma[3] += M14G;
    Ma[4] += M22G;
    Ma[5] += wA * tr(H12) - tr(M12G);
    Ma[6] += M24G;
    Ma[7] += M11G + wA * ((I3 - H11) - tr(H11));
    Ma[8] += wA * H14 - M14G;
    Ma[9] += M44G;

    // gyroscopic / damping blocks (:380-416)
    M3 SWm = skewmul(W0, Ir) - skew(IrW0);
    M3 Ac1 = Ar * (C11_ + C31_), Ac2 = Ar * (C12_ + C32_), Ac4 = Ar * (C14_ + C34_);
    M3 X1 = Ir * (C21_ + C41_) + mulskew(SWm, s21);
    M3 X2 = Ir * (C22_ + C42_) + muld(SWm, d22);
    M3 X4 = Ir * (C24_ + C44_) + muld(SWm, d24);
    M3 C11G = wg * (mulTN(H11, Ac1) - skewmul(s21, X1));
    M3 C12G = wg * (mulTN(H11, Ac2) - skewmul(s21, X2));
    M3 C14G = wg * (mulTN(H11, Ac4) - skewmul(s21, X4));
    Ca[0] += C11G;
    Ca[1] += C12G;
    Ca[2] += C14G;
    Ca[3] += wg * (mulTN(H12, Ac1) + dmul(d22, X1));
    Ca[4] += wg * (mulTN(H12, Ac2) + dmul(d22, X2));
    Ca[5] += wg * (mulTN(H12, Ac4) + dmul(d22, X4));
    Ca[6] += wg * Ac1 - C11G;
    Ca[7] += wg * Ac2 - C12G;
    Ca[8] += wg * Ac4 - C14G;
    Ca[9] += wg * (mulTN(H14, Ac1) + dmul(d24, X1));
    Ca[10] += wg * (mulTN(H14, Ac2) + dmul(d24, X2));
    Ca[11] += wg * (mulTN(H14, Ac4) + dmul(d24, X4));

    kinetic += wg / 2 * (Ar * dot(ud0, ud0) + dot(W0, IrW0));
  }

  const double l02 = in.l0 / 2;
  M3 lRe = l02 * Re;
  out.E[0] = strain_energy;
  out.E[1] = l02 * kinetic;
  {
    double* T = out.Tint;
    put_vec(T, 0, Ti1); put_vec(T, 1, Ti2); put_vec(T, 2, -Ti1); put_vec(T, 3, Ti4);
    double* Tk = out.Tk;
    put_vec(Tk, 0, lRe * Tk1); put_vec(Tk, 1, lRe * Tk2); put_vec(Tk, 2, lRe * Tk3); put_vec(Tk, 3, lRe * Tk4);
  }
  // post-scaling lₒ/2 Rₑ X Rₑᵀ (:431-457)
#pragma unroll 1
  for (int k = 0; k < 10; ++k) Ma[k] = mulNT(lRe * Ma[k], Re);
#pragma unroll 1
  for (int k = 0; k < 12; ++k) Ca[k] = mulNT(lRe * Ca[k], Re);
  // exact-mode transforms (:480-506), with the damping terms (:461-478) folded in
  V3 Tha = toangle(in.dR1), Thb = toangle(in.dR2);
  M3 TaT = tr(Ts_inv(Tha)), TbT = tr(Ts_inv(Thb));
  const M3 &M11 = Ma[0], &M12 = Ma[1], &M13 = Ma[2], &M14 = Ma[3], &M22 = Ma[4], &M23 = Ma[5], &M24 = Ma[6],
           &M33 = Ma[7], &M34 = Ma[8], &M44 = Ma[9];
  double* Mo = out.M;
  double* Co = out.C;
  // row 1
  put_block(Mo, 0, 0, M11); put_block(Mo, 0, 1, M12); put_block(Mo, 0, 2, M13); put_block(Mo, 0, 3, M14);
  {
    M3 C11 = Ca[0], C12 = Ca[1], C14 = Ca[2];
    M3 C13 = -C11;
    if (damping > 0) { axpy(C11, damping, M11); axpy(C12, damping, M12); axpy(C13, damping, M13); axpy(C14, damping, M14); }
    put_block(Co, 0, 0, C11); put_block(Co, 0, 1, C12); put_block(Co, 0, 2, C13); put_block(Co, 0, 3, C14);
  }
  // row 2: M²¹ = M¹²ᵀTₐᵀ, M²ʲ = M²ʲTₐᵀ, Cᵏ²ʲ = (Cᵏ²ʲ + damping·…)Tₐᵀ
  M3 M23t = M23 * TaT;
  M3 M24t = M24 * TaT;
  put_block(Mo, 1, 0, mulTN(M12, TaT)); put_block(Mo, 1, 1, M22 * TaT); put_block(Mo, 1, 2, M23t);
  put_block(Mo, 1, 3, M24t);
  {
    M3 C21 = Ca[3], C22 = Ca[4], C24 = Ca[5];
    M3 C23 = -C21;
    if (damping > 0) {
      C21 += damping * tr(M12); axpy(C22, damping, M22); axpy(C23, damping, M23); axpy(C24, damping, M24);
    }
    put_block(Co, 1, 0, C21 * TaT); put_block(Co, 1, 1, C22 * TaT); put_block(Co, 1, 2, C23 * TaT);
    put_block(Co, 1, 3, C24 * TaT);
  }
  // row 3: M³¹ = M¹³ᵀ, M³² = (M²³Tₐᵀ)ᵀ (reassigned M²³ is read, :493)
  put_blockT(Mo, 2, 0, M13); put_blockT(Mo, 2, 1, M23t); put_block(Mo, 2, 2, M33); put_block(Mo, 2, 3, M34);
  {
    M3 C31 = Ca[6], C32 = Ca[7], C34 = Ca[8];
    M3 C33 = -C31;
    if (damping > 0) {
      C31 += damping * tr(M13); C32 += damping * tr(M23); axpy(C33, damping, M33); axpy(C34, damping, M34);
    }
    put_block(Co, 2, 0, C31); put_block(Co, 2, 1, C32); put_block(Co, 2, 2, C33); put_block(Co, 2, 3, C34);
  }
  // row 4: M⁴¹ = M¹⁴ᵀT_bᵀ, M⁴² = (M²⁴Tₐᵀ)ᵀT_bᵀ, M⁴³ = M³⁴ᵀT_bᵀ, M⁴⁴ = M⁴⁴T_bᵀ
  put_block(Mo, 3, 0, mulTN(M14, TbT)); put_block(Mo, 3, 1, mulTN(M24t, TbT)); put_block(Mo, 3, 2, mulTN(M34, TbT));
  put_block(Mo, 3, 3, M44 * TbT);
  {
    M3 C41 = Ca[9], C42 = Ca[10], C44 = Ca[11];
    M3 C43 = -C41;
    if (damping > 0) {
      C41 += damping * tr(M14); C42 += damping * tr(M24); C43 += damping * tr(M34); axpy(C44, damping, M44);
    }
    put_block(Co, 3, 0, C41 * TbT); put_block(Co, 3, 1, C42 * TbT); put_block(Co, 3, 2, C43 * TbT);
    put_block(Co, 3, 3, C44 * TbT);
  }
}

}  // namespace ebd
