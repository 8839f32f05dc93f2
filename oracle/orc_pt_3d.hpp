// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Pointwise physics of CompressibleEulerPotentialTemperatureEquationsWithGravity3D,
// restated from src/equations/compressible_euler_potential_temperature_gravity_3d.jl:
//   state u = (rho, rho_v1, rho_v2, rho_v3, rho_theta, phi), p = K rho_theta^gamma,
//   K = p_0 (R / p_0)^gamma (constructor :53-66); phi = g z is passive.
// flux :110-125, nonconservative gravity terms :146-211, FluxLMARS :213-256,
// slip wall :83-107, flux_tec :428-458, flux_ec :468-497, flux_etec :505-533,
// max_abs_speeds :695-700; Coriolis from
// src/equations/initial_condition_compressible_euler_3d.jl:245-269.
// The Stolarsky mean is the one of orc_pt_2d.hpp.
#pragma once
#include <array>
#include <cmath>
#include "orc_means.hpp"
#include "orc_pt_2d.hpp"

namespace orc {

struct PotTemp3D {
  static constexpr int nv = 6;
  using State = std::array<double, 6>;
  double c_p = 1004.0, c_v = 717.0, g = 9.80616, p_0 = 100000.0;
  double R = 287.0, gamma = 1004.0 / 717.0, K = 0.0, sc[8];
  int volume = 0;   // 0 flux_tec, 1 flux_ec, 2 flux_etec, 3 flux_kennedy_gruber
  int nc_kind = 0;  // 0 waruszewski (ln_mean rho), 1 artiano (stolarsky rho), 2 souza (average)

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

  void cons2prim(const State& u, double& rho, double* v, double& p) const {
    rho = u[0];
    v[0] = u[1] / rho;
    v[1] = u[2] / rho;
    v[2] = u[3] / rho;
    p = K * std::pow(u[4], gamma);
  }

  // prim2cons (:535-543): rho_theta = (p / K)^(1 / gamma)
  State prim2cons(double rho, double v1, double v2, double v3, double p, double phi) const {
    return {rho, rho * v1, rho * v2, rho * v3, std::pow(p / K, 1.0 / gamma), phi};
  }

  // flux with the reference's pressure(): K exp(gamma log rho_theta)
  State flux(const State& u, const double* n) const {
    const double v1 = u[1] / u[0], v2 = u[2] / u[0], v3 = u[3] / u[0];
    const double vn = v1 * n[0] + v2 * n[1] + v3 * n[2];
    const double rvn = u[0] * vn;
    const double p = K * std::exp(gamma * std::log(u[4]));
    return {rvn, rvn * v1 + p * n[0], rvn * v2 + p * n[1], rvn * v3 + p * n[2], u[4] * vn, 0.0};
  }

  State volume_flux(const State& ul, const State& ur, const double* n) const {
    double rl, vl[3], pl, rr, vr[3], pr;
    cons2prim(ul, rl, vl, pl);
    cons2prim(ur, rr, vr, pr);
    const double vnl = vl[0] * n[0] + vl[1] * n[1] + vl[2] * n[2];
    const double vnr = vr[0] * n[0] + vr[1] * n[1] + vr[2] * n[2];
    double va[3];
    for (int k = 0; k < 3; ++k) va[k] = 0.5 * (vl[k] + vr[k]);
    const double pa = 0.5 * (pl + pr);
    double f1, f5;
    if (volume == 0) {
      f1 = ln_mean(rl, rr) * 0.5 * (vnl + vnr);
      f5 = stolarsky(ul[4], ur[4]) * 0.5 * (vnl + vnr);
    } else if (volume == 1) {
      f1 = ln_mean(rl, rr) * 0.5 * (vnl + vnr);
      f5 = f1 * inv_ln_mean(rl / ul[4], rr / ur[4]);
    } else if (volume == 3) {
      // flux_kennedy_gruber, src/equations/compressible_euler_potential_temperature_gravity_3d.jl:333-359
      const double v_dot_n_avg = va[0] * n[0] + va[1] * n[1] + va[2] * n[2];
      f1 = 0.5 * (rl + rr) * v_dot_n_avg;
      f5 = f1 * (0.5 * (ul[4] / rl + ur[4] / rr));
    } else {
      f5 = stolarsky(ul[4], ur[4]) * 0.5 * (vnl + vnr);
      f1 = f5 * ln_mean(rl / ul[4], rr / ur[4]);
    }
    return {f1, f1 * va[0] + pa * n[0], f1 * va[1] + pa * n[1], f1 * va[2] + pa * n[2], f5, 0.0};
  }

  State noncons(const State& ul, const State& ur, const double* n) const {
    double ra;
    if (nc_kind == 0) ra = ln_mean(ul[0], ur[0]);
    else if (nc_kind == 1) ra = stolarsky(ul[0], ur[0]);
    else ra = 0.5 * (ul[0] + ur[0]);
    const double jump = ur[5] - ul[5];
    return {0.0, n[0] * ra * jump, n[1] * ra * jump, n[2] * ra * jump, 0.0, 0.0};
  }

  State flux_lmars(const State& ul, const State& ur, const double* n, double a) const {
    double rl, vl[3], pl, rr, vr[3], pr;
    cons2prim(ul, rl, vl, pl);
    cons2prim(ur, rr, vr, pr);
    const double v_l = vl[0] * n[0] + vl[1] * n[1] + vl[2] * n[2];
    const double v_r = vr[0] * n[0] + vr[1] * n[1] + vr[2] * n[2];
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double rho = 0.5 * (rl + rr);
    const double p_int = 0.5 * (pl + pr) - 0.5 * a * rho * (v_r - v_l) / nrm;
    const double v_int = 0.5 * (v_l + v_r) - 1.0 / (2.0 * a * rho) * (pr - pl) * nrm;
    const State& us = v_int > 0 ? ul : ur;
    State f{};
    for (int v = 0; v < 5; ++v) f[v] = us[v] * v_int;
    f[1] += p_int * n[0];
    f[2] += p_int * n[1];
    f[3] += p_int * n[2];
    f[5] = 0.0;
    return f;
  }

  // boundary_condition_slip_wall (outward normal), :83-107
  State slip_wall_normal(const State& ui, const double* n, double a) const {
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double e[3] = {n[0] / nrm, n[1] / nrm, n[2] / nrm};
    const double un = e[0] * ui[1] + e[1] * ui[2] + e[2] * ui[3];
    const State ub = {ui[0], ui[1] - 2.0 * un * e[0], ui[2] - 2.0 * un * e[1],
                      ui[3] - 2.0 * un * e[2], ui[4], ui[5]};
    return flux_lmars(ui, ub, n, a);
  }

  State coriolis(const State& u, double omega) const {
    return {0.0, 2.0 * omega * u[2], -2.0 * omega * u[1], 0.0, 0.0, 0.0};
  }

  void max_abs_speeds(const State& u, double* l) const {
    double rho, v[3], p;
    cons2prim(u, rho, v, p);
    const double c = std::sqrt(gamma * p / rho);
    for (int k = 0; k < 3; ++k) l[k] = std::fabs(v[k]) + c;
  }
};

}  // namespace orc
