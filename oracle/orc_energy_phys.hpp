// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// The DG drivers' physics policies of the dry energy equations (2D:
// CompressibleEulerEnergyEquationsWithGravity2D with (flux_ranocha,
// flux_nonconservative_waruszewski_etal) / (FluxLMARS(c), flux_zero); 3D: the
// same plus source_terms_coriolis): which pointwise formulas each phase of
// orc_dg2d.hpp / orc_dg3d.hpp calls.  Shared by orc_api.cpp and the operation
// counts of orc_flopcount.cpp.
#pragma once
#include "orc_euler_energy_2d.hpp"
#include "orc_euler_energy_3d.hpp"

namespace orc {

struct EnergyPhys {
  using State = EulerEnergy2D::State;
  static constexpr int nv = 5;
  static constexpr bool has_noncons = true;
  static constexpr bool has_sources = false;
  EulerEnergy2D eq;
  double c_lmars = 340.0;
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_ranocha(a, b, n);
  }
  State volume_noncons(const State& a, const State& b, const double* n) const {
    return eq.noncons_waruszewski(a, b, n);
  }
  State surface_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_lmars(a, b, n, c_lmars);
  }
  State surface_noncons(const State&, const State&, const double*) const { return State{}; }
  State bc_structured(const State& ui, const double* n, int direction) const {
    return eq.slip_wall_structured(ui, n, direction, c_lmars);
  }
  State bc_normal(const State& ui, const double* n) const {
    return eq.slip_wall_normal(ui, n, c_lmars);
  }
  State source(const State&, const double*, double) const { return State{}; }
  void max_abs_speeds(const State& u, double& l1, double& l2) const { eq.max_abs_speeds(u, l1, l2); }
  // flux(u, normal_direction), compressible_euler_energy_with_gravity_2d.jl:154-166
  State flux(const State& u, const double* n) const {
    double rho, v1, v2, p;
    eq.cons2prim(u, rho, v1, v2, p);
    const double vn = v1 * n[0] + v2 * n[1];
    const double rvn = rho * vn;
    return {rvn, rvn * v1 + p * n[0], rvn * v2 + p * n[1], (u[3] + p) * vn, 0.0};
  }
};

struct EnergyPhys3D {
  using State = EulerEnergy3D::State;
  static constexpr int nv = 6;
  static constexpr bool has_noncons = true;
  static constexpr bool has_sources = true;
  EulerEnergy3D eq;
  double c_lmars = 340.0, omega = 0.0;
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_ranocha(a, b, n);
  }
  State volume_noncons(const State& a, const State& b, const double* n) const {
    return eq.noncons_waruszewski(a, b, n);
  }
  State surface_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_lmars(a, b, n, c_lmars);
  }
  State surface_noncons(const State&, const State&, const double*) const { return State{}; }
  State bc_normal(const State& ui, const double* n) const { return eq.slip_wall_normal(ui, n, c_lmars); }
  State source(const State& u, const double*, double) const { return eq.coriolis(u, omega); }
  void max_abs_speeds(const State& u, double* l) const { eq.max_abs_speeds(u, l); }
};

}  // namespace orc
