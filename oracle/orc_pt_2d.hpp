// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Pointwise physics of CompressibleEulerPotentialTemperatureEquationsWithGravity2D,
// restated from src/equations/compressible_euler_potential_temperature_gravity_2d.jl:
//   state u = (rho, rho_v1, rho_v2, rho_theta, phi), p = K (rho_theta)^gamma,
//   K = p_0 (R / p_0)^gamma; phi = g z is passive.
// The Stolarsky mean (Trixi, external) is restated from its definition
//   S(x, y) = (gamma - 1)/gamma (y^gamma - x^gamma) / (y^(gamma-1) - x^(gamma-1))
// (Winters et al., BIT Numer. Math. 60, 2020): for f^2 = ((y-x)/(x+y))^2 < 1e-2
// it is evaluated as (x+y)/2 R(f^2) with the first eight terms of the series
// R = (sum_j C(gamma, 2j+1)/gamma f^2j) / (sum_j C(gamma-1, 2j+1)/(gamma-1) f^2j)
// (from the binomial expansions of (1 +- f)^a), else from the definition.
#pragma once
#include <array>
#include <cmath>
#include "orc_means.hpp"

namespace orc {

// series coefficients of the Stolarsky mean for exponent gamma
inline void stolarsky_coefficients(double gamma, double* c) {
  double a[8], b[8];
  auto binom = [](double x, int m) {
    double r = 1.0;
    for (int i = 0; i < m; ++i) r = r * (x - i) / (i + 1);
    return r;
  };
  for (int j = 0; j < 8; ++j) {
    a[j] = binom(gamma, 2 * j + 1) / gamma;
    b[j] = binom(gamma - 1.0, 2 * j + 1) / (gamma - 1.0);
  }
  for (int k = 0; k < 8; ++k) {
    double s = a[k];
    for (int i = 1; i <= k; ++i) s -= b[i] * c[k - i];
    c[k] = s;
  }
}

struct PotTemp2D {
  static constexpr int nv = 5;
  using State = std::array<double, 5>;
  double c_p = 1004.0, c_v = 717.0, g = 9.80616, p_0 = 100000.0;
  double R = 287.0, gamma = 1004.0 / 717.0, K = 0.0, sc[8];
  int volume = 0;  // 0 flux_tec, 1 flux_ec, 2 flux_etec
  int nc_kind = 0;  // 0 waruszewski (ln_mean rho), 1 artiano (stolarsky rho), 2 souza (average)
  int surface = 0;  // surface flux: 0 FluxLMARS(c), 1 flux_ec
  int snc_kind = -1;  // surface nonconservative term: -1 flux_zero, else as nc_kind

  void init(double cp, double cv, double grav) {
    c_p = cp; c_v = cv; g = grav;
    R = c_p - c_v;
    gamma = c_p / c_v;
    K = p_0 * std::pow(R / p_0, gamma);
    stolarsky_coefficients(gamma, sc);
  }

  double stolarsky(double x, double y) const {
    const double s = x + y, d = y - x;
    const double t = d / s, f2 = t * t;
    if (f2 < 1e-2) {
      double r = sc[7];
      for (int k = 6; k >= 0; --k) r = r * f2 + sc[k];
      return 0.5 * s * r;
    }
    return (gamma - 1.0) / gamma * (std::pow(y, gamma) - std::pow(x, gamma)) /
           (std::pow(y, gamma - 1.0) - std::pow(x, gamma - 1.0));
  }

  // cons2prim (p = K rho_theta^gamma)
  void cons2prim(const State& u, double& rho, double& v1, double& v2, double& p) const {
    rho = u[0];
    v1 = u[1] / rho;
    v2 = u[2] / rho;
    p = K * std::pow(u[3], gamma);
  }

  // prim2cons: rho_theta = (p / p_0)^(1/gamma) p_0 / R
  State prim2cons(double rho, double v1, double v2, double p, double phi) const {
    return {rho, rho * v1, rho * v2, std::pow(p / p_0, 1.0 / gamma) * p_0 / R, phi};
  }

  // flux(u, normal_direction), with the reference's pressure(): K exp(gamma log rho_theta)
  State flux(const State& u, const double* n) const {
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double vn = v1 * n[0] + v2 * n[1];
    const double rvn = u[0] * vn;
    const double p = K * std::exp(gamma * std::log(u[3]));
    return {rvn, rvn * v1 + p * n[0], rvn * v2 + p * n[1], u[3] * vn, 0.0};
  }

  // flux_tec / flux_ec / flux_etec (:205-284)
  State volume_flux(const State& ul, const State& ur, const double* n) const {
    double rl, v1l, v2l, pl, rr, v1r, v2r, pr;
    cons2prim(ul, rl, v1l, v2l, pl);
    cons2prim(ur, rr, v1r, v2r, pr);
    const double vnl = v1l * n[0] + v2l * n[1], vnr = v1r * n[0] + v2r * n[1];
    const double v1a = 0.5 * (v1l + v1r), v2a = 0.5 * (v2l + v2r), pa = 0.5 * (pl + pr);
    double f1, f4;
    if (volume == 0) {
      f1 = ln_mean(rl, rr) * 0.5 * (vnl + vnr);
      f4 = stolarsky(ul[3], ur[3]) * 0.5 * (vnl + vnr);
    } else if (volume == 1) {
      f1 = ln_mean(rl, rr) * 0.5 * (vnl + vnr);
      f4 = f1 * inv_ln_mean(rl / ul[3], rr / ur[3]);
    } else {
      f4 = stolarsky(ul[3], ur[3]) * 0.5 * (vnl + vnr);
      f1 = f4 * ln_mean(rl / ul[3], rr / ur[3]);
    }
    return {f1, f1 * v1a + pa * n[0], f1 * v2a + pa * n[1], f4, 0.0};
  }

  // flux_nonconservative_{waruszewski_etal, artiano_etal, souza_etal} (:111-170)
  State noncons_of(const State& ul, const State& ur, const double* n, int kind) const {
    double ra;
    if (kind == 0) ra = ln_mean(ul[0], ur[0]);
    else if (kind == 1) ra = stolarsky(ul[0], ur[0]);
    else ra = 0.5 * (ul[0] + ur[0]);
    const double jump = ur[4] - ul[4];
    return {0.0, n[0] * ra * jump, n[1] * ra * jump, 0.0, 0.0};
  }
  State noncons(const State& ul, const State& ur, const double* n) const {
    return noncons_of(ul, ur, n, nc_kind);
  }

  // flux_ec (:290-321) whatever the volume flux is
  State flux_ec(const State& ul, const State& ur, const double* n) const {
    double rl, v1l, v2l, pl, rr, v1r, v2r, pr;
    cons2prim(ul, rl, v1l, v2l, pl);
    cons2prim(ur, rr, v1r, v2r, pr);
    const double vnl = v1l * n[0] + v2l * n[1], vnr = v1r * n[0] + v2r * n[1];
    const double v1a = 0.5 * (v1l + v1r), v2a = 0.5 * (v2l + v2r), pa = 0.5 * (pl + pr);
    const double f1 = ln_mean(rl, rr) * 0.5 * (vnl + vnr);
    const double f4 = f1 * inv_ln_mean(rl / ul[3], rr / ur[3]);
    return {f1, f1 * v1a + pa * n[0], f1 * v2a + pa * n[1], f4, 0.0};
  }

  // the configured surface flux and nonconservative surface term
  State surface_flux(const State& ul, const State& ur, const double* n, double a) const {
    return surface ? flux_ec(ul, ur, n) : flux_lmars(ul, ur, n, a);
  }
  State surface_noncons(const State& ul, const State& ur, const double* n) const {
    if (snc_kind < 0) return State{};
    return noncons_of(ul, ur, n, snc_kind);
  }

  // FluxLMARS (:171-193)
  State flux_lmars(const State& ul, const State& ur, const double* n, double a) const {
    double rl, v1l, v2l, pl, rr, v1r, v2r, pr;
    cons2prim(ul, rl, v1l, v2l, pl);
    cons2prim(ur, rr, v1r, v2r, pr);
    const double vl = v1l * n[0] + v2l * n[1], vr = v1r * n[0] + v2r * n[1];
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double rho = 0.5 * (rl + rr);
    const double p_int = 0.5 * (pl + pr) - 0.5 * a * rho * (vr - vl) / nrm;
    const double v_int = 0.5 * (vl + vr) - 1.0 / (2.0 * a * rho) * (pr - pl) * nrm;
    State f{};
    const State& us = v_int > 0 ? ul : ur;
    for (int v = 0; v < 4; ++v) f[v] = us[v] * v_int;
    f[1] += p_int * n[0];
    f[2] += p_int * n[1];
    f[4] = 0.0;
    return f;
  }

  // slip walls: StructuredMesh (:62-83; reached with the normal vector in the
  // `orientation` slot, so `orientation == 1` is false and rho_v2 is mirrored;
  // states ordered by the parity of the direction) and outward normal (:45-60)
  State slip_wall_structured(const State& ui, const double* n, int direction, double a) const {
    State ub = ui;
    ub[2] = -ui[2];
    if (direction % 2 == 0) return surface_flux(ui, ub, n, a);
    return surface_flux(ub, ui, n, a);
  }
  // the surface flux plus half the nonconservative term of the inner and the
  // mirrored state (zero: both carry the same phi)
  State slip_wall_normal(const State& ui, const double* n, double a) const {
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double nx = n[0] / nrm, ny = n[1] / nrm;
    const double un = nx * ui[1] + ny * ui[2];
    const State ub = {ui[0], ui[1] - 2.0 * un * nx, ui[2] - 2.0 * un * ny, ui[3], ui[4]};
    State f = surface_flux(ui, ub, n, a);
    const State g = surface_noncons(ui, ub, n);
    for (int v = 0; v < 5; ++v) f[v] += 0.5 * g[v];
    return f;
  }

  void max_abs_speeds(const State& u, double& l1, double& l2) const {
    double rho, v1, v2, p;
    cons2prim(u, rho, v1, v2, p);
    const double c = std::sqrt(gamma * p / rho);
    l1 = std::fabs(v1) + c;
    l2 = std::fabs(v2) + c;
  }
};

}  // namespace orc
