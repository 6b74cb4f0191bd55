// Device-side FP64 3x3 algebra for the EndoBeams hot path on sm_103a.
//
// Storage is column-major (m(i,j) = a[i + 3j]) like Julia's StaticArrays
// `Mat33`.  Besides dense products the header carries the few structured
// products the corotational beam element evaluates many times per Gauss
// point (skew matrices, the sparse Gᵀ matrices of
// src/beams/utils_beams.jl:76-81, diagonals): on GB300 the FP64 pipe is the
// scarcest resource, so every multiply by a known zero is skipped.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define EB_DEV __device__ __forceinline__
#else
// Host compilation of the same arithmetic is used only by developer probes.
#include <cmath>
#define EB_DEV inline
using std::acos; using std::fabs; using std::fma; using std::fmax; using std::sin; using std::sqrt;
inline void sincos(double x, double* s, double* c) { *s = std::sin(x); *c = std::cos(x); }
#define __ldg(p) (*(p))
#endif

namespace ebd {

struct V3 {
  double x, y, z;
};
struct M3 {
  double a[9];
  EB_DEV double& operator()(int i, int j) { return a[i + 3 * j]; }
  EB_DEV double operator()(int i, int j) const { return a[i + 3 * j]; }
};

EB_DEV V3 v3(double x, double y, double z) { return V3{x, y, z}; }
EB_DEV V3 zv3() { return V3{0.0, 0.0, 0.0}; }
EB_DEV M3 zm3() {
  M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = 0.0;
  return m;
}
EB_DEV M3 eye3() {
  M3 m = zm3();
  m.a[0] = 1.0; m.a[4] = 1.0; m.a[8] = 1.0;
  return m;
}
EB_DEV M3 rows(double a00, double a01, double a02, double a10, double a11, double a12, double a20, double a21,
               double a22) {
  M3 m;
  m.a[0] = a00; m.a[3] = a01; m.a[6] = a02;
  m.a[1] = a10; m.a[4] = a11; m.a[7] = a12;
  m.a[2] = a20; m.a[5] = a21; m.a[8] = a22;
  return m;
}
EB_DEV M3 diag3(double a, double b, double c) { M3 m = zm3(); m.a[0] = a; m.a[4] = b; m.a[8] = c; return m; }

EB_DEV V3 operator+(V3 p, V3 q) { return v3(p.x + q.x, p.y + q.y, p.z + q.z); }
EB_DEV V3 operator-(V3 p, V3 q) { return v3(p.x - q.x, p.y - q.y, p.z - q.z); }
EB_DEV V3 operator-(V3 p) { return v3(-p.x, -p.y, -p.z); }
EB_DEV V3 operator*(double s, V3 p) { return v3(s * p.x, s * p.y, s * p.z); }
EB_DEV V3& operator+=(V3& p, V3 q) { p = p + q; return p; }

EB_DEV M3 operator+(const M3& p, const M3& q) { M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = p.a[k] + q.a[k]; return m; }
EB_DEV M3 operator-(const M3& p, const M3& q) { M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = p.a[k] - q.a[k]; return m; }
EB_DEV M3 operator-(const M3& p) { M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = -p.a[k]; return m; }
EB_DEV M3 operator*(double s, const M3& p) { M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = s * p.a[k]; return m; }
EB_DEV M3& operator+=(M3& p, const M3& q) {
#pragma unroll
  for (int k = 0; k < 9; ++k) p.a[k] += q.a[k]; return p; }
// p += s * q, one FMA per entry
EB_DEV void axpy(M3& p, double s, const M3& q) {
#pragma unroll
  for (int k = 0; k < 9; ++k) p.a[k] = fma(s, q.a[k], p.a[k]); }

EB_DEV M3 operator*(const M3& p, const M3& q) {
  M3 m;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) m(i, j) = p(i, 0) * q(0, j) + p(i, 1) * q(1, j) + p(i, 2) * q(2, j);
  return m;
}
EB_DEV V3 operator*(const M3& p, V3 q) {
  return v3(p(0, 0) * q.x + p(0, 1) * q.y + p(0, 2) * q.z, p(1, 0) * q.x + p(1, 1) * q.y + p(1, 2) * q.z,
            p(2, 0) * q.x + p(2, 1) * q.y + p(2, 2) * q.z);
}
// pᵀ q
EB_DEV M3 mulTN(const M3& p, const M3& q) {
  M3 m;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) m(i, j) = p(0, i) * q(0, j) + p(1, i) * q(1, j) + p(2, i) * q(2, j);
  return m;
}
// p qᵀ
EB_DEV M3 mulNT(const M3& p, const M3& q) {
  M3 m;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) m(i, j) = p(i, 0) * q(j, 0) + p(i, 1) * q(j, 1) + p(i, 2) * q(j, 2);
  return m;
}
// pᵀ v
EB_DEV V3 mulTv(const M3& p, V3 q) {
  return v3(p(0, 0) * q.x + p(1, 0) * q.y + p(2, 0) * q.z, p(0, 1) * q.x + p(1, 1) * q.y + p(2, 1) * q.z,
            p(0, 2) * q.x + p(1, 2) * q.y + p(2, 2) * q.z);
}
EB_DEV M3 tr(const M3& p) { M3 m;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) m(i, j) = p(j, i); return m; }
EB_DEV double dot(V3 p, V3 q) { return p.x * q.x + p.y * q.y + p.z * q.z; }
EB_DEV double norm(V3 p) { return sqrt(dot(p, p)); }
EB_DEV V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
EB_DEV M3 outer(V3 a, V3 b) {
  return rows(a.x * b.x, a.x * b.y, a.x * b.z, a.y * b.x, a.y * b.y, a.y * b.z, a.z * b.x, a.z * b.y, a.z * b.z);
}
EB_DEV double trace(const M3& p) { return p.a[0] + p.a[4] + p.a[8]; }
EB_DEV V3 col(const M3& p, int j) { return v3(p(0, j), p(1, j), p(2, j)); }
EB_DEV M3 hcat3(V3 a, V3 b, V3 c) { return rows(a.x, b.x, c.x, a.y, b.y, c.y, a.z, b.z, c.z); }
EB_DEV M3 skew(V3 v) { return rows(0.0, -v.z, v.y, v.z, 0.0, -v.x, -v.y, v.x, 0.0); }

// skew(v) * p : column j is v × p[:,j]
EB_DEV M3 skewmul(V3 v, const M3& p) {
  M3 m;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    V3 c = cross(v, col(p, j));
    m(0, j) = c.x; m(1, j) = c.y; m(2, j) = c.z;
  }
  return m;
}
// p * skew(v) : row i is p[i,:] × ... = -(v × p[i,:]ᵀ)ᵀ
EB_DEV M3 mulskew(const M3& p, V3 v) {
  M3 m;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    V3 r = v3(p(i, 0), p(i, 1), p(i, 2));
    V3 c = cross(r, v);  // (r skew(v))ᵀ = skew(v)ᵀ rᵀ = -v × r = r × v
    m(i, 0) = c.x; m(i, 1) = c.y; m(i, 2) = c.z;
  }
  return m;
}
// diag(d) * p and p * diag(d)
EB_DEV M3 dmul(V3 d, const M3& p) {
  return rows(d.x * p(0, 0), d.x * p(0, 1), d.x * p(0, 2), d.y * p(1, 0), d.y * p(1, 1), d.y * p(1, 2), d.z * p(2, 0),
              d.z * p(2, 1), d.z * p(2, 2));
}
EB_DEV M3 muld(const M3& p, V3 d) {
  return rows(p(0, 0) * d.x, p(0, 1) * d.y, p(0, 2) * d.z, p(1, 0) * d.x, p(1, 1) * d.y, p(1, 2) * d.z,
              p(2, 0) * d.x, p(2, 1) * d.y, p(2, 2) * d.z);
}
EB_DEV V3 dmulv(V3 d, V3 p) { return v3(d.x * p.x, d.y * p.y, d.z * p.z); }

// Gᵀu₁ = [0 0 g13; 0 0 g23; 0 g32 0]  (utils_beams.jl:76); Gᵀu₂ = -Gᵀu₁
struct Gu { double g13, g23, g32; };
// GᵀΘ = [a b 0; 0 0 0; 0 0 0]          (utils_beams.jl:80-81)
struct Gt { double a, b; };

EB_DEV M3 full(Gu g) { return rows(0, 0, g.g13, 0, 0, g.g23, 0, g.g32, 0); }
EB_DEV M3 full(Gt g) { return rows(g.a, g.b, 0, 0, 0, 0, 0, 0, 0); }
EB_DEV Gu neg(Gu g) { return Gu{-g.g13, -g.g23, -g.g32}; }
// p * G
EB_DEV M3 mulG(const M3& p, Gu g) {
  M3 m;
  m(0, 0) = 0.0; m(1, 0) = 0.0; m(2, 0) = 0.0;
  m(0, 1) = p(0, 2) * g.g32; m(1, 1) = p(1, 2) * g.g32; m(2, 1) = p(2, 2) * g.g32;
  m(0, 2) = p(0, 0) * g.g13 + p(0, 1) * g.g23;
  m(1, 2) = p(1, 0) * g.g13 + p(1, 1) * g.g23;
  m(2, 2) = p(2, 0) * g.g13 + p(2, 1) * g.g23;
  return m;
}
EB_DEV M3 mulG(const M3& p, Gt g) {
  M3 m;
  m(0, 0) = p(0, 0) * g.a; m(1, 0) = p(1, 0) * g.a; m(2, 0) = p(2, 0) * g.a;
  m(0, 1) = p(0, 0) * g.b; m(1, 1) = p(1, 0) * g.b; m(2, 1) = p(2, 0) * g.b;
  m(0, 2) = 0.0; m(1, 2) = 0.0; m(2, 2) = 0.0;
  return m;
}
// G * v
EB_DEV V3 Gv(Gu g, V3 v) { return v3(g.g13 * v.z, g.g23 * v.z, g.g32 * v.y); }
EB_DEV V3 Gv(Gt g, V3 v) { return v3(g.a * v.x + g.b * v.y, 0.0, 0.0); }
// Gᵀ * v
EB_DEV V3 GTv(Gu g, V3 v) { return v3(0.0, g.g32 * v.z, g.g13 * v.x + g.g23 * v.y); }
// G * p  (rows of p mixed by G)
EB_DEV M3 Gmul(Gu g, const M3& p) {
  M3 m;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    m(0, j) = g.g13 * p(2, j);
    m(1, j) = g.g23 * p(2, j);
    m(2, j) = g.g32 * p(1, j);
  }
  return m;
}
EB_DEV M3 Gmul(Gt g, const M3& p) {
  M3 m;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    m(0, j) = g.a * p(0, j) + g.b * p(1, j);
    m(1, j) = 0.0;
    m(2, j) = 0.0;
  }
  return m;
}

constexpr double EPS64 = 2.220446049250313e-16;  // eps(Float64)

// utils_beams.jl:11-32
EB_DEV M3 rotation_matrix(V3 th) {
  double n = norm(th);
  if (n > 10 * EPS64) {
    double s, c;
    sincos(n, &s, &c);
    M3 S = skew(th);
    M3 R = eye3();
    axpy(R, s / n, S);
    axpy(R, (1 - c) / (n * n), skewmul(th, S));
    return R;
  }
  return eye3();
}

// utils_beams.jl:90-104
EB_DEV V3 toangle(const M3& R) {
  double c = (trace(R) - 1) / 2;
  double nv = (fabs(c) < 1) ? fmax(acos(c), 10 * EPS64) : 10 * EPS64;
  double f = nv * (1 / (2 * sin(nv)));
  return v3(f * (R(2, 1) - R(1, 2)), f * (R(0, 2) - R(2, 0)), f * (R(1, 0) - R(0, 1)));
}

// utils_beams.jl:107-122
EB_DEV M3 Ts_inv(V3 th) {
  double n = norm(th);
  if (n < 10 * EPS64) return eye3();
  double s2, c2;
  sincos(n / 2, &s2, &c2);
  M3 S = skew(th);
  M3 T = eye3();
  axpy(T, -0.5, S);
  axpy(T, (s2 - n / 2 * c2) / (s2 * (n * n)), skewmul(th, S));
  return T;
}

// utils_beams.jl:180-198
EB_DEV void compute_eta_mu(V3 thv, double* eta, double* mu) {
  double th = norm(thv);
  if (th < 10 * EPS64) {
    *eta = 1.0 / 12.0;
    *mu = 1.0 / 360.0;
  } else {
    double s, c;
    sincos(th, &s, &c);
    double s2 = sin(th / 2);
    *eta = ((2 * s) - th * (1 + c)) / (2 * (th * th) * s);
    *mu = (th * (th + s) - 8 * (s2 * s2)) / (4 * (th * th * th * th) * (s2 * s2));
  }
}

}  // namespace ebd
