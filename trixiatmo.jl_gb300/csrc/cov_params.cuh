// Parameters of the covariant shallow-water kernels: the equations' gravity
// and the volume / surface flux choices (see cov_kernels.cuh).
#pragma once

namespace tag {

struct CovParams {
  double g;
  int split;     // SplitCovariantShallowWaterEquations2D
  int volume;    // 0 weak form, 1 flux differencing
  int vol_sym;   // 0 flux_central, 1 flux_ec
  int vol_nc;    // 0 none, 1 flux_nonconservative_ec
  int surf_sym;  // 0 flux_central, 1 flux_ec
  int surf_diss; // 0 none, 1 local Lax-Friedrichs
  int surf_nc;   // 0 none, 1 flux_nonconservative_ec, 2 flux_nonconservative_surface_simplified
};

}  // namespace tag
