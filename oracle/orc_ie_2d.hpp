// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Pointwise physics of CompressibleEulerInternalEnergyEquationsWithGravity2D,
// restated from src/equations/compressible_euler_internal_energy_with_gravity_2d.jl:
//   state u = (rho, rho_v1, rho_v2, rho_e_internal, phi), p = (gamma - 1) rho_e_internal;
// flux_conservative_etec :110-136, flux_nonconservative_etec :144-165,
// flux_conservative_es :174-216, flux_nonconservative_es :224-246,
// slip wall :77-99 (flux + nonconservative flux of the mirrored state),
// prim2cons :248-255, cons2prim :257-264, max_abs_speeds :319-325.
// The physical flux (Trixi's flux for the energy variable rho_e_internal,
// (rho_e_internal + p) v . n) is the consistency reference.
#pragma once
#include <array>
#include <cmath>
#include "orc_means.hpp"

namespace orc {

struct InternalEnergy2D {
  static constexpr int nv = 5;
  using State = std::array<double, 5>;
  double c_p = 1004.0, c_v = 717.0, g = 9.81, gamma = 1004.0 / 717.0, inv_gm1 = 717.0 / 287.0;

  void init(double cp, double cv, double grav) {
    c_p = cp; c_v = cv; g = grav;
    gamma = c_p / c_v;
    inv_gm1 = 1.0 / (gamma - 1.0);
  }

  void cons2prim(const State& u, double& rho, double& v1, double& v2, double& p) const {
    rho = u[0];
    v1 = u[1] / rho;
    v2 = u[2] / rho;
    p = (gamma - 1.0) * u[3];
  }

  State prim2cons(double rho, double v1, double v2, double p, double phi) const {
    return {rho, rho * v1, rho * v2, p * inv_gm1, phi};
  }

  // physical flux of the conservative part: (rho v.n, rho v1 v.n + p n1,
  // rho v2 v.n + p n2, (rho e + p) v.n)
  State flux(const State& u, const double* n) const {
    double rho, v1, v2, p;
    cons2prim(u, rho, v1, v2, p);
    const double vn = v1 * n[0] + v2 * n[1];
    return {rho * vn, rho * v1 * vn + p * n[0], rho * v2 * vn + p * n[1], (u[3] + p) * vn, 0.0};
  }

  State flux_etec(const State& ul, const State& ur, const double* n) const {
    double rl, v1l, v2l, pl, rr, v1r, v2r, pr;
    cons2prim(ul, rl, v1l, v2l, pl);
    cons2prim(ur, rr, v1r, v2r, pr);
    const double vnl = v1l * n[0] + v2l * n[1], vnr = v1r * n[0] + v2r * n[1];
    const double vn_avg = 0.5 * (vnl + vnr);
    const double rho_mean = ln_mean(rl, rr);
    const double v1a = 0.5 * (v1l + v1r), v2a = 0.5 * (v2l + v2r);
    const double pa = 0.5 * (pl + pr);
    const double inv_rho_p_mean = pl * pr * inv_ln_mean(rl * pr, rr * pl);
    const double f1 = rho_mean * 0.5 * (vnl + vnr);
    return {f1, f1 * v1a + pa * n[0], f1 * v2a + pa * n[1],
            f1 * inv_rho_p_mean * inv_gm1 + pa * vn_avg, 0.0};
  }

  State noncons_etec(const State& ul, const State& ur, const double* n) const {
    double rl, v1l, v2l, pl, rr, v1r, v2r, pr;
    cons2prim(ul, rl, v1l, v2l, pl);
    cons2prim(ur, rr, v1r, v2r, pr);
    const double vnl = v1l * n[0] + v2l * n[1], vnr = v1r * n[0] + v2r * n[1];
    const double vn_avg = 0.5 * (vnr + vnl);
    const double gravity = ln_mean(rl, rr) * (ur[4] - ul[4]);
    return {0.0, gravity * n[0], gravity * n[1], -vn_avg * (pr - pl), 0.0};
  }

  State flux_es(const State& ul, const State& ur, const double* n) const {
    double rl, v1l, v2l, pl, rr, v1r, v2r, pr;
    cons2prim(ul, rl, v1l, v2l, pl);
    cons2prim(ur, rr, v1r, v2r, pr);
    const double vnl = v1l * n[0] + v2l * n[1], vnr = v1r * n[0] + v2r * n[1];
    const double rho_mean = ln_mean(rl, rr);
    const double cl = std::sqrt(gamma * pl / rl), cr = std::sqrt(gamma * pr / rr);
    const double a = 0.5 * (cl + cr);
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double rho_avg = 0.5 * (rl + rr);
    const double p_int = 0.5 * (pl + pr) - 0.5 * a * rho_avg * (vnr - vnl) / nrm;
    const double v_int = 0.5 * (vnl + vnr) - 1.0 / (2.0 * a * rho_avg) * (pr - pl) * nrm;
    const double pa = 0.5 * (pl + pr);
    double rho_up, f2, f3;
    if (v_int >= 0) {
      rho_up = rho_mean - 0.5 * (rr - rl);
      f2 = ul[1] * v_int;
      f3 = ul[2] * v_int;
    } else {
      rho_up = rho_mean + 0.5 * (rr - rl);
      f2 = ur[1] * v_int;
      f3 = ur[2] * v_int;
    }
    const double inv_rho_p_mean = pl * pr * inv_ln_mean(rl * pr, rr * pl);
    const double f1 = rho_up * v_int;
    return {f1, f2 + p_int * n[0], f3 + p_int * n[1], f1 * inv_rho_p_mean * inv_gm1 + pa * v_int,
            0.0};
  }

  State noncons_es(const State& ul, const State& ur, const double* n) const {
    double rl, v1l, v2l, pl, rr, v1r, v2r, pr;
    cons2prim(ul, rl, v1l, v2l, pl);
    cons2prim(ur, rr, v1r, v2r, pr);
    const double vnl = v1l * n[0] + v2l * n[1], vnr = v1r * n[0] + v2r * n[1];
    const double cl = std::sqrt(gamma * pl / rl), cr = std::sqrt(gamma * pr / rr);
    const double a = 0.5 * (cl + cr);
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double rho_avg = 0.5 * (rl + rr);
    const double v_int = 0.5 * (vnl + vnr) - 1.0 / (2.0 * a * rho_avg) * (pr - pl) * nrm;
    return {0.0, 0.0, 0.0, -v_int * (pr - pl), 0.0};
  }

  // boundary_condition_slip_wall (outward normal): the surface flux plus half
  // the nonconservative flux of the inner and the mirrored state
  State slip_wall_normal(const State& ui, const double* n) const {
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double e0 = n[0] / nrm, e1 = n[1] / nrm;
    const double un = e0 * ui[1] + e1 * ui[2];
    const State ub = {ui[0], ui[1] - 2.0 * un * e0, ui[2] - 2.0 * un * e1, ui[3], ui[4]};
    const State f = flux_es(ui, ub, n), gnc = noncons_es(ui, ub, n);
    State r;
    for (int v = 0; v < 5; ++v) r[v] = f[v] + 0.5 * gnc[v];
    return r;
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
