// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Pointwise physics of `CompressibleEulerEnergyEquationsWithGravity3D`,
// restated from src/equations/compressible_euler_energy_with_gravity_3d.jl
// (state u = (rho, rho_v1, rho_v2, rho_v3, rho_e, phi)), and the Coriolis
// source of src/equations/initial_condition_compressible_euler_3d.jl:245-269.
#pragma once
#include <array>
#include <cmath>
#include "orc_means.hpp"

namespace orc {

struct EulerEnergy3D {
  static constexpr int nv = 6;
  using State = std::array<double, 6>;
  double c_p = 1004.0, c_v = 717.0, g = 9.81;
  double R = 287.0, gamma = 1004.0 / 717.0, inv_gamma_minus_one = 0.0;
  double p_0 = 100000.0;

  EulerEnergy3D(double cp = 1004.0, double cv = 717.0, double grav = 9.81)
      : c_p(cp), c_v(cv), g(grav) {
    R = c_p - c_v;
    gamma = c_p / c_v;
    inv_gamma_minus_one = 1.0 / (gamma - 1.0);
  }

  // cons2prim
  void cons2prim(const State& u, double& rho, double& v1, double& v2, double& v3,
                 double& p) const {
    rho = u[0];
    v1 = u[1] / rho;
    v2 = u[2] / rho;
    v3 = u[3] / rho;
    p = (gamma - 1.0) * (u[4] - 0.5 * (u[1] * v1 + u[2] * v2 + u[3] * v3));
  }

  State prim2cons(double rho, double v1, double v2, double v3, double p, double phi) const {
    return {rho, rho * v1, rho * v2, rho * v3,
            p * inv_gamma_minus_one + 0.5 * rho * (v1 * v1 + v2 * v2 + v3 * v3), phi};
  }

  // flux_ranocha (3D), :382-415
  State flux_ranocha(const State& ul, const State& ur, const double* n) const {
    double rl, v1l, v2l, v3l, pl, rr, v1r, v2r, v3r, pr;
    cons2prim(ul, rl, v1l, v2l, v3l, pl);
    cons2prim(ur, rr, v1r, v2r, v3r, pr);
    const double vnl = v1l * n[0] + v2l * n[1] + v3l * n[2];
    const double vnr = v1r * n[0] + v2r * n[1] + v3r * n[2];
    const double rho_mean = ln_mean(rl, rr);
    const double inv_rho_p_mean = pl * pr * inv_ln_mean(rl * pr, rr * pl);
    const double v1a = 0.5 * (v1l + v1r), v2a = 0.5 * (v2l + v2r), v3a = 0.5 * (v3l + v3r);
    const double pa = 0.5 * (pl + pr);
    const double vsq = 0.5 * (v1l * v1r + v2l * v2r + v3l * v3r);
    const double f1 = rho_mean * 0.5 * (vnl + vnr);
    return {f1, f1 * v1a + pa * n[0], f1 * v2a + pa * n[1], f1 * v3a + pa * n[2],
            f1 * (vsq + inv_rho_p_mean * inv_gamma_minus_one) + 0.5 * (pl * vnr + pr * vnl), 0.0};
  }

  // flux_nonconservative_waruszewski_etal (3D), :135-159
  State noncons_waruszewski(const State& ul, const State& ur, const double* n) const {
    const double v1l = ul[1] / ul[0], v2l = ul[2] / ul[0], v3l = ul[3] / ul[0];
    const double v1r = ur[1] / ur[0], v2r = ur[2] / ur[0], v3r = ur[3] / ur[0];
    const double v1a = 0.5 * (v1l + v1r), v2a = 0.5 * (v2l + v2r), v3a = 0.5 * (v3l + v3r);
    const double ra = ln_mean(ul[0], ur[0]);
    const double j = ur[5] - ul[5];
    return {0.0, n[0] * ra * j, n[1] * ra * j, n[2] * ra * j,
            n[0] * ra * v1a * j + n[1] * ra * v2a * j + n[2] * ra * v3a * j, 0.0};
  }

  // FluxLMARS (3D), :430-466
  State flux_lmars(const State& ul, const State& ur, const double* n, double c) const {
    double rl, v1l, v2l, v3l, pl, rr, v1r, v2r, v3r, pr;
    cons2prim(ul, rl, v1l, v2l, v3l, pl);
    cons2prim(ur, rr, v1r, v2r, v3r, pr);
    const double vl = v1l * n[0] + v2l * n[1] + v3l * n[2];
    const double vr = v1r * n[0] + v2r * n[1] + v3r * n[2];
    const double norm_ = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double rho = 0.5 * (rl + rr);
    const double p = 0.5 * (pl + pr) - 0.5 * c * rho * (vr - vl) / norm_;
    const double v = 0.5 * (vl + vr) - 1.0 / (2.0 * c * rho) * (pr - pl) * norm_;
    State f;
    if (v >= 0) {
      for (int k = 0; k < 5; ++k) f[k] = v * ul[k];
      f[4] += pl * v;
    } else {
      for (int k = 0; k < 5; ++k) f[k] = v * ur[k];
      f[4] += pr * v;
    }
    f[1] += p * n[0];
    f[2] += p * n[1];
    f[3] += p * n[2];
    f[5] = 0.0;
    return f;
  }

  // boundary_condition_slip_wall (3D, outward normal), :93-116
  State slip_wall_normal(const State& ui, const double* nd, double c) const {
    const double nn = std::sqrt(nd[0] * nd[0] + nd[1] * nd[1] + nd[2] * nd[2]);
    const double n0 = nd[0] / nn, n1 = nd[1] / nn, n2 = nd[2] / nn;
    const double un = n0 * ui[1] + n1 * ui[2] + n2 * ui[3];
    State ub = {ui[0], ui[1] - 2.0 * un * n0, ui[2] - 2.0 * un * n1, ui[3] - 2.0 * un * n2,
                ui[4], ui[5]};
    return flux_lmars(ui, ub, nd, c);
  }

  // max_abs_speeds (3D), :559-564
  void max_abs_speeds(const State& u, double* l) const {
    double rho, v1, v2, v3, p;
    cons2prim(u, rho, v1, v2, v3, p);
    const double c = std::sqrt(gamma * p / rho);
    l[0] = std::fabs(v1) + c;
    l[1] = std::fabs(v2) + c;
    l[2] = std::fabs(v3) + c;
  }

  // coriolis_source, initial_condition_compressible_euler_3d.jl:245-255
  State coriolis(const State& u, double omega) const {
    return {0.0, 2.0 * omega * u[2], -2.0 * omega * u[1], 0.0, 0.0, 0.0};
  }
};

}  // namespace orc
