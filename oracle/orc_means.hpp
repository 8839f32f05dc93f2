// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Logarithmic mean and its inverse, restated from the published method in
// H. Ranocha, M. Schlottke-Lakemper, J. Chan, A. M. Rueda-Ramirez, A. R. Winters,
// F. Hindenlang, G. J. Gassner, "Efficient implementation of modern entropy
// stable and kinetic energy preserving discontinuous Galerkin methods for
// conservation laws", ACM TOMS 49 (2023), arXiv:2112.10517, Sec. 2.2:
// with f2 = ((x - y)/(x + y))^2 evaluated as (x(x-2y)+y^2)/(x(x+2y)+y^2),
//   f2 <  1e-4:  ln_mean = (x+y) * 52.5 / (105 + f2 (35 + f2 (21 + f2 15)))
//   otherwise :  ln_mean = (y - x) / log(y / x)
// TrixiAtmo imports these as `Trixi.ln_mean`, `Trixi.inv_ln_mean`
// (src/TrixiAtmo.jl:37); Trixi.jl 0.17 is the defining (external) package.
#pragma once
#include <cmath>

namespace orc {

inline double ln_mean(double x, double y) {
  const double f2 = (x * (x - 2.0 * y) + y * y) / (x * (x + 2.0 * y) + y * y);
  if (f2 < 1.0e-4) {
    return (x + y) * 52.5 / (105.0 + f2 * (35.0 + f2 * (21.0 + f2 * 15.0)));
  }
  return (y - x) / std::log(y / x);
}

inline double inv_ln_mean(double x, double y) {
  const double f2 = (x * (x - 2.0 * y) + y * y) / (x * (x + 2.0 * y) + y * y);
  if (f2 < 1.0e-4) {
    return (105.0 + f2 * (35.0 + f2 * (21.0 + f2 * 15.0))) / (52.5 * (x + y));
  }
  return std::log(y / x) / (y - x);
}

}  // namespace orc
