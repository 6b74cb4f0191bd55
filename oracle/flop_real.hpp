// ORACLE — test infrastructure only.  A double that counts the floating-point
// operations applied to it, so the oracle's element restatements can be compiled
// over it (oracle/flop_count.cpp) to give the algorithmic FP64 operation count of
// one element evaluation, independent of any GPU code.
#pragma once
#include <cmath>
#include <cstdint>

namespace flop {

struct Counts {
  unsigned long long add = 0, mul = 0, div = 0, sqrt = 0, trans = 0;  // trans: sin, cos, acos calls
};
inline Counts g;

struct Real {
  double v;
  Real() = default;
  constexpr Real(double x) : v(x) {}
  explicit constexpr operator double() const { return v; }
  explicit operator int() const { return (int)v; }
  explicit operator long() const { return (long)v; }
  explicit operator long long() const { return (long long)v; }
  Real& operator+=(Real o) { ++g.add; v += o.v; return *this; }
  Real& operator-=(Real o) { ++g.add; v -= o.v; return *this; }
  Real& operator*=(Real o) { ++g.mul; v *= o.v; return *this; }
  Real& operator/=(Real o) { ++g.div; v /= o.v; return *this; }
};
inline Real operator+(Real a, Real b) { ++g.add; return Real(a.v + b.v); }
inline Real operator-(Real a, Real b) { ++g.add; return Real(a.v - b.v); }
inline Real operator*(Real a, Real b) { ++g.mul; return Real(a.v * b.v); }
inline Real operator/(Real a, Real b) { ++g.div; return Real(a.v / b.v); }
inline Real operator-(Real a) { return Real(-a.v); }
inline Real operator+(Real a) { return a; }
inline bool operator<(Real a, Real b) { return a.v < b.v; }
inline bool operator>(Real a, Real b) { return a.v > b.v; }
inline bool operator<=(Real a, Real b) { return a.v <= b.v; }
inline bool operator>=(Real a, Real b) { return a.v >= b.v; }
inline bool operator==(Real a, Real b) { return a.v == b.v; }
inline bool operator!=(Real a, Real b) { return a.v != b.v; }

}  // namespace flop

// The oracle calls these through std::; counted overloads for the counting build only.
namespace std {
inline flop::Real sqrt(flop::Real x) { ++flop::g.sqrt; return flop::Real(::sqrt(x.v)); }
inline flop::Real sin(flop::Real x) { ++flop::g.trans; return flop::Real(::sin(x.v)); }
inline flop::Real cos(flop::Real x) { ++flop::g.trans; return flop::Real(::cos(x.v)); }
inline flop::Real acos(flop::Real x) { ++flop::g.trans; return flop::Real(::acos(x.v)); }
inline flop::Real fabs(flop::Real x) { return flop::Real(::fabs(x.v)); }
inline flop::Real floor(flop::Real x) { return flop::Real(::floor(x.v)); }
}  // namespace std
