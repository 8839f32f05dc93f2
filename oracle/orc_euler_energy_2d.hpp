// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Pointwise physics of `CompressibleEulerEnergyEquationsWithGravity2D`,
// restated from src/equations/compressible_euler_energy_with_gravity_2d.jl
// (state u = (rho, rho_v1, rho_v2, rho_e, phi), rho_e the total energy
// without the potential, phi = g z carried as a passive variable).
#pragma once
#include <array>
#include <cmath>
#include "orc_means.hpp"

namespace orc {

struct EulerEnergy2D {
  static constexpr int nv = 5;
  using State = std::array<double, 5>;
  double c_p = 1004.0, c_v = 717.0, g = 9.81;
  double R = 287.0, gamma = 1004.0 / 717.0, inv_gamma_minus_one = 0.0;
  double p_0 = 100000.0;

  // :49-59
  EulerEnergy2D(double cp = 1004.0, double cv = 717.0, double grav = 9.81)
      : c_p(cp), c_v(cv), g(grav) {
    R = c_p - c_v;
    gamma = c_p / c_v;
    inv_gamma_minus_one = 1.0 / (gamma - 1.0);
  }

  // cons2prim, :527-536
  void cons2prim(const State& u, double& rho, double& v1, double& v2, double& p) const {
    rho = u[0];
    v1 = u[1] / rho;
    v2 = u[2] / rho;
    p = (gamma - 1.0) * (u[3] - 0.5 * (u[1] * v1 + u[2] * v2));
  }

  // prim2cons, :585-592
  State prim2cons(double rho, double v1, double v2, double p, double phi) const {
    const double rv1 = rho * v1, rv2 = rho * v2;
    return {rho, rv1, rv2, p * inv_gamma_minus_one + 0.5 * (rv1 * v1 + rv2 * v2), phi};
  }

  // flux_ranocha, :366-395
  State flux_ranocha(const State& ul, const State& ur, const double* n) const {
    double rho_ll, v1_ll, v2_ll, p_ll, rho_rr, v1_rr, v2_rr, p_rr;
    cons2prim(ul, rho_ll, v1_ll, v2_ll, p_ll);
    cons2prim(ur, rho_rr, v1_rr, v2_rr, p_rr);
    const double vn_ll = v1_ll * n[0] + v2_ll * n[1];
    const double vn_rr = v1_rr * n[0] + v2_rr * n[1];
    const double rho_mean = ln_mean(rho_ll, rho_rr);
    const double inv_rho_p_mean = p_ll * p_rr * inv_ln_mean(rho_ll * p_rr, rho_rr * p_ll);
    const double v1_avg = 0.5 * (v1_ll + v1_rr);
    const double v2_avg = 0.5 * (v2_ll + v2_rr);
    const double p_avg = 0.5 * (p_ll + p_rr);
    const double vsq_avg = 0.5 * (v1_ll * v1_rr + v2_ll * v2_rr);
    const double f1 = rho_mean * 0.5 * (vn_ll + vn_rr);
    const double f2 = f1 * v1_avg + p_avg * n[0];
    const double f3 = f1 * v2_avg + p_avg * n[1];
    const double f4 = f1 * (vsq_avg + inv_rho_p_mean * inv_gamma_minus_one) +
                      0.5 * (p_ll * vn_rr + p_rr * vn_ll);
    return {f1, f2, f3, f4, 0.0};
  }

  // flux_nonconservative_waruszewski_etal, :186-205
  State noncons_waruszewski(const State& ul, const State& ur, const double* n) const {
    const double v1_ll = ul[1] / ul[0], v1_rr = ur[1] / ur[0];
    const double v2_ll = ul[2] / ul[0], v2_rr = ur[2] / ur[0];
    const double v1_avg = 0.5 * (v1_ll + v1_rr);
    const double v2_avg = 0.5 * (v2_ll + v2_rr);
    const double rho_avg = ln_mean(ul[0], ur[0]);
    const double phi_jump = ur[4] - ul[4];
    return {0.0, n[0] * rho_avg * phi_jump, n[1] * rho_avg * phi_jump,
            n[0] * rho_avg * v1_avg * phi_jump + n[1] * rho_avg * v2_avg * phi_jump, 0.0};
  }

  // FluxLMARS, :397-430
  State flux_lmars(const State& ul, const State& ur, const double* n, double c) const {
    double rho_ll, v1_ll, v2_ll, p_ll, rho_rr, v1_rr, v2_rr, p_rr;
    cons2prim(ul, rho_ll, v1_ll, v2_ll, p_ll);
    cons2prim(ur, rho_rr, v1_rr, v2_rr, p_rr);
    const double v_ll = v1_ll * n[0] + v2_ll * n[1];
    const double v_rr = v1_rr * n[0] + v2_rr * n[1];
    const double norm_ = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double rho = 0.5 * (rho_ll + rho_rr);
    const double p = 0.5 * (p_ll + p_rr) - 0.5 * c * rho * (v_rr - v_ll) / norm_;
    const double v = 0.5 * (v_ll + v_rr) - 1.0 / (2.0 * c * rho) * (p_rr - p_ll) * norm_;
    double f1, f2, f3, f4;
    if (v >= 0) {
      f1 = ul[0] * v; f2 = ul[1] * v; f3 = ul[2] * v; f4 = ul[3] * v + p_ll * v;
    } else {
      f1 = ur[0] * v; f2 = ur[1] * v; f3 = ur[2] * v; f4 = ur[3] * v + p_rr * v;
    }
    return {f1, f2 + p * n[0], f3 + p * n[1], f4, 0.0};
  }

  // Slip wall as reached from a StructuredMesh boundary: Trixi passes the
  // (sign-corrected) contravariant vector in the `orientation` slot, so the
  // method at :102-129 runs with `orientation == 1` false and mirrors v2; the
  // flux is evaluated with the inner state on the side given by `direction`.
  // direction is 1-based as in Trixi (1 = x-, 2 = x+, 3 = y-, 4 = y+); the
  // returned flux is in the +xi/+eta sense of `normal`.
  State slip_wall_structured(const State& u_inner, const double* normal, int direction,
                             double c) const {
    State ub = {u_inner[0], u_inner[1], -u_inner[2], u_inner[3], u_inner[4]};
    if (direction % 2 == 0) return flux_lmars(u_inner, ub, normal, c);
    return flux_lmars(ub, u_inner, normal, c);
  }

  // Slip wall with an outward normal (P4estMesh path), :77-100.
  State slip_wall_normal(const State& u_inner, const double* normal_direction, double c) const {
    const double nn = std::sqrt(normal_direction[0] * normal_direction[0] +
                                normal_direction[1] * normal_direction[1]);
    const double nx = normal_direction[0] / nn, ny = normal_direction[1] / nn;
    const double u_normal = nx * u_inner[1] + ny * u_inner[2];
    State ub = {u_inner[0], u_inner[1] - 2.0 * u_normal * nx, u_inner[2] - 2.0 * u_normal * ny,
                u_inner[3], u_inner[4]};
    return flux_lmars(u_inner, ub, normal_direction, c);
  }

  // max_abs_speeds, :518-524
  void max_abs_speeds(const State& u, double& l1, double& l2) const {
    double rho, v1, v2, p;
    cons2prim(u, rho, v1, v2, p);
    const double c = std::sqrt(gamma * p / rho);
    l1 = std::fabs(v1) + c;
    l2 = std::fabs(v2) + c;
  }

  // entropy (mathematical), :602-627
  double entropy(const State& u) const {
    const double p = (gamma - 1.0) * (u[3] - 0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0]);
    const double s = std::log(p) - gamma * std::log(u[0]);
    return -s * u[0] * inv_gamma_minus_one;
  }
};

}  // namespace orc
