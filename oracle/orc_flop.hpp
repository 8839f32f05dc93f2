// ORACLE — test infrastructure only (operation counts of the oracle's formulas).
//
// A counting scalar: a double that counts every arithmetic operation applied
// to it.  orc_flopcount.cpp compiles the oracle's own headers a second time
// with `double` replaced by this type, so the counts are those of the oracle's
// formulas (which restate the reference's) evaluated on a given state, every
// branch taken as the data decide.  Conventions: add, sub, mul, div and sqrt
// one flop each (the oracle is built with -ffp-contract=off, so no fused
// operations occur); log, exp and pow counted separately (and reported with a
// fixed weight by the caller); sign flips, comparisons, fabs, min and max are
// not counted.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <vector>

namespace orc_count {

struct Counts {
  long long add = 0, mul = 0, div = 0, sqrt = 0, log = 0, exp = 0, pow = 0;
};

inline Counts& counts() {
  static Counts c;
  return c;
}

struct Flop {
  double v;
  constexpr Flop() : v(0.0) {}
  constexpr Flop(double x) : v(x) {}
  explicit constexpr operator double() const { return v; }
  Flop& operator+=(const Flop& o) { ++counts().add; v += o.v; return *this; }
  Flop& operator-=(const Flop& o) { ++counts().add; v -= o.v; return *this; }
  Flop& operator*=(const Flop& o) { ++counts().mul; v *= o.v; return *this; }
  Flop& operator/=(const Flop& o) { ++counts().div; v /= o.v; return *this; }
  Flop operator-() const { return Flop(-v); }
  Flop operator+() const { return *this; }
};

inline Flop operator+(const Flop& a, const Flop& b) { ++counts().add; return Flop(a.v + b.v); }
inline Flop operator-(const Flop& a, const Flop& b) { ++counts().add; return Flop(a.v - b.v); }
inline Flop operator*(const Flop& a, const Flop& b) { ++counts().mul; return Flop(a.v * b.v); }
inline Flop operator/(const Flop& a, const Flop& b) { ++counts().div; return Flop(a.v / b.v); }
inline bool operator<(const Flop& a, const Flop& b) { return a.v < b.v; }
inline bool operator>(const Flop& a, const Flop& b) { return a.v > b.v; }
inline bool operator<=(const Flop& a, const Flop& b) { return a.v <= b.v; }
inline bool operator>=(const Flop& a, const Flop& b) { return a.v >= b.v; }
inline bool operator==(const Flop& a, const Flop& b) { return a.v == b.v; }
inline bool operator!=(const Flop& a, const Flop& b) { return a.v != b.v; }

}  // namespace orc_count

namespace std {
inline orc_count::Flop sqrt(const orc_count::Flop& x) {
  ++orc_count::counts().sqrt;
  return orc_count::Flop(std::sqrt(x.v));
}
inline orc_count::Flop log(const orc_count::Flop& x) {
  ++orc_count::counts().log;
  return orc_count::Flop(std::log(x.v));
}
inline orc_count::Flop exp(const orc_count::Flop& x) {
  ++orc_count::counts().exp;
  return orc_count::Flop(std::exp(x.v));
}
inline orc_count::Flop pow(const orc_count::Flop& x, const orc_count::Flop& y) {
  ++orc_count::counts().pow;
  return orc_count::Flop(std::pow(x.v, y.v));
}
inline orc_count::Flop fabs(const orc_count::Flop& x) { return orc_count::Flop(std::fabs(x.v)); }
inline orc_count::Flop abs(const orc_count::Flop& x) { return orc_count::Flop(std::fabs(x.v)); }
// trigonometric functions appear only in set-up code (basis, initial data)
inline orc_count::Flop cos(const orc_count::Flop& x) { return orc_count::Flop(std::cos(x.v)); }
inline orc_count::Flop sin(const orc_count::Flop& x) { return orc_count::Flop(std::sin(x.v)); }
inline bool isfinite(const orc_count::Flop& x) { return std::isfinite(x.v); }
}  // namespace std
