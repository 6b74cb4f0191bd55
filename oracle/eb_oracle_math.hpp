// ORACLE — test infrastructure only. Never linked into the product library.
//
// Small fixed-size FP64 linear algebra used by the CPU restatement of the
// EndoBeams.jl hot path.  Storage is column-major like Julia's StaticArrays
// (`Mat33` of src/constants.jl:1), so `m(i,j)` is `a[i + 3*j]`.
// Every operation is the plain textbook formula, evaluated left to right,
// without fused multiply-add (the build passes -ffp-contract=off), so the
// oracle gives the same bits on x86-64 and aarch64 hosts.
#pragma once
#include <cmath>
#include <cstdint>

namespace orc {

struct V3 {
  double v[3];
  double& operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};

struct M3 {
  double a[9];  // column-major
  double& operator()(int i, int j) { return a[i + 3 * j]; }
  double operator()(int i, int j) const { return a[i + 3 * j]; }
};

inline V3 v3(double x, double y, double z) { return V3{{x, y, z}}; }
inline V3 zv3() { return V3{{0.0, 0.0, 0.0}}; }
inline M3 zm3() { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = 0.0; return m; }
inline M3 eye3() { M3 m = zm3(); m(0, 0) = 1.0; m(1, 1) = 1.0; m(2, 2) = 1.0; return m; }
// Row-major literal constructor, reads like Julia's `@SMatrix [a b c; d e f; g h i]`.
inline M3 rows(double a00, double a01, double a02, double a10, double a11, double a12,
               double a20, double a21, double a22) {
  M3 m;
  m(0, 0) = a00; m(0, 1) = a01; m(0, 2) = a02;
  m(1, 0) = a10; m(1, 1) = a11; m(1, 2) = a12;
  m(2, 0) = a20; m(2, 1) = a21; m(2, 2) = a22;
  return m;
}
inline M3 diag3(double a, double b, double c) { M3 m = zm3(); m(0, 0) = a; m(1, 1) = b; m(2, 2) = c; return m; }

inline V3 operator+(const V3& x, const V3& y) { return v3(x[0] + y[0], x[1] + y[1], x[2] + y[2]); }
inline V3 operator-(const V3& x, const V3& y) { return v3(x[0] - y[0], x[1] - y[1], x[2] - y[2]); }
inline V3 operator-(const V3& x) { return v3(-x[0], -x[1], -x[2]); }
inline V3 operator*(double s, const V3& x) { return v3(s * x[0], s * x[1], s * x[2]); }
inline V3 operator*(const V3& x, double s) { return v3(x[0] * s, x[1] * s, x[2] * s); }
inline V3 operator/(const V3& x, double s) { return v3(x[0] / s, x[1] / s, x[2] / s); }
inline V3& operator+=(V3& x, const V3& y) { x = x + y; return x; }

inline M3 operator+(const M3& x, const M3& y) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = x.a[k] + y.a[k]; return m; }
inline M3 operator-(const M3& x, const M3& y) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = x.a[k] - y.a[k]; return m; }
inline M3 operator-(const M3& x) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = -x.a[k]; return m; }
inline M3 operator*(double s, const M3& x) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = s * x.a[k]; return m; }
inline M3 operator*(const M3& x, double s) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = x.a[k] * s; return m; }
inline M3 operator/(const M3& x, double s) { M3 m; for (int k = 0; k < 9; ++k) m.a[k] = x.a[k] / s; return m; }
inline M3& operator+=(M3& x, const M3& y) { x = x + y; return x; }

inline M3 operator*(const M3& x, const M3& y) {
  M3 m;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m(i, j) = x(i, 0) * y(0, j) + x(i, 1) * y(1, j) + x(i, 2) * y(2, j);
  return m;
}
inline V3 operator*(const M3& x, const V3& y) {
  return v3(x(0, 0) * y[0] + x(0, 1) * y[1] + x(0, 2) * y[2],
            x(1, 0) * y[0] + x(1, 1) * y[1] + x(1, 2) * y[2],
            x(2, 0) * y[0] + x(2, 1) * y[1] + x(2, 2) * y[2]);
}
inline M3 tr(const M3& x) { M3 m; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) m(i, j) = x(j, i); return m; }
inline double dot(const V3& x, const V3& y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; }
inline double norm(const V3& x) { return std::sqrt(dot(x, x)); }
inline V3 cross(const V3& a, const V3& b) {
  return v3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
inline M3 outer(const V3& a, const V3& b) { M3 m; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) m(i, j) = a[i] * b[j]; return m; }
inline double trace(const M3& x) { return x(0, 0) + x(1, 1) + x(2, 2); }
inline V3 col(const M3& x, int j) { return v3(x(0, j), x(1, j), x(2, j)); }
inline M3 hcat3(const V3& a, const V3& b, const V3& c) {
  M3 m; for (int i = 0; i < 3; ++i) { m(i, 0) = a[i]; m(i, 1) = b[i]; m(i, 2) = c[i]; } return m;
}

// A 1x3 row vector (Julia adjoint of a Vec3) times a 3x3 matrix / vector.
inline double rowdot(const V3& r, const V3& x) { return dot(r, x); }

const double EPS64 = 2.220446049250313e-16;  // eps(Float64)

}  // namespace orc
