// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Pointwise physics of `CompressibleMoistEulerEquations2D`, restated from
// src/equations/compressible_moist_euler_2d.jl:
//   state u = (rho, rho_v1, rho_v2, rho_E, rho_qv, rho_ql)
// Gravity enters through source_terms_geopotential; phase change through the
// Fischer-Burmeister source term.
#pragma once
#include <array>
#include <cmath>
#include "orc_means.hpp"

namespace orc {

struct MoistEuler2D {
  static constexpr int nv = 6;
  using State = std::array<double, 6>;
  // constructor, :20-31
  double c_pd = 1004.0, c_vd = 717.0, c_pv = 1885.0, c_vv = 1424.0, g = 9.80616;
  double p_0 = 100000.0, R_d = 287.0, R_v = 461.0, c_pl = 4186.0, kappa = 0.0,
         gamma = 0.0, L_00 = 3147620.0;

  void init(double cpd, double cvd, double cpv, double cvv, double gravity) {
    c_pd = cpd; c_vd = cvd; c_pv = cpv; c_vv = cvv; g = gravity;
    R_d = c_pd - c_vd;
    R_v = c_pv - c_vv;
    gamma = c_pd / c_vd;
    kappa = 1.0 - 1.0 / gamma;
  }

  // get_current_condition, :383-402 -> (p, T)
  void condition(const State& u, double& p, double& T) const {
    const double rho_qd = u[0] - u[4] - u[5];
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double rho_e = u[3] - 0.5 * (u[1] * v1 + u[2] * v2);
    T = (rho_e - L_00 * u[4]) / (rho_qd * c_vd + u[4] * c_vv + u[5] * c_pl);
    p = (rho_qd * R_d + u[4] * R_v) * T;
  }

  // ratio of specific heats of the mixture (:897-902)
  double gamma_mix(const State& u) const {
    const double qv = u[4] / u[0], ql = u[5] / u[0];
    const double qd = 1.0 - qv - ql;
    return (qd * c_pd + qv * c_pv + ql * c_pl) * (1.0 / (qd * c_vd + qv * c_vv + ql * c_pl));
  }

  // flux(u, normal_direction), :63-82
  State flux(const State& u, const double* n) const {
    double p, T;
    condition(u, p, T);
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double qv = u[4] / u[0], ql = u[5] / u[0];
    const double vn = v1 * n[0] + v2 * n[1];
    const double rvn = u[0] * vn;
    return {rvn, rvn * v1 + p * n[0], rvn * v2 + p * n[1], (u[3] + p) * vn, rvn * qv, rvn * ql};
  }

  // flux_chandrashekar, :936-1003 (R_q = 0)
  State flux_chandrashekar(const State& ul, const State& ur, const double* n) const {
    const double rqd_l = ul[0] - ul[4] - ul[5], rqd_r = ur[0] - ur[4] - ur[5];
    const double v1_l = ul[1] / ul[0], v1_r = ur[1] / ur[0];
    const double v2_l = ul[2] / ul[0], v2_r = ur[2] / ur[0];
    const double re_l = ul[3] - 0.5 * (ul[1] * v1_l + ul[2] * v2_l);
    const double re_r = ur[3] - 0.5 * (ur[1] * v1_r + ur[2] * v2_r);
    const double T_l = (re_l - L_00 * ul[4]) / (rqd_l * c_vd + ul[4] * c_vv + ul[5] * c_pl);
    const double T_r = (re_r - L_00 * ur[4]) / (rqd_r * c_vd + ur[4] * c_vv + ur[5] * c_pl);
    double rqd_mean = 0, rqv_mean = 0, rql_mean = 0, iT_mean = 0;
    if (rqd_l != 0.0 && rqd_r != 0.0) rqd_mean = ln_mean(rqd_l, rqd_r);
    if (ul[4] != 0.0 && ur[4] != 0.0) rqv_mean = ln_mean(ul[4], ur[4]);
    if (ul[5] != 0.0 && ur[5] != 0.0) rql_mean = ln_mean(ul[5], ur[5]);
    const double iT_l = 1.0 / T_l, iT_r = 1.0 / T_r;
    if (iT_l != 0.0 && iT_r != 0.0) iT_mean = inv_ln_mean(iT_l, iT_r);
    const double v1a = 0.5 * (v1_l + v1_r), v2a = 0.5 * (v2_l + v2_r);
    const double v1sq = 0.5 * (v1_l * v1_l + v1_r * v1_r);
    const double v2sq = 0.5 * (v2_l * v2_l + v2_r * v2_r);
    const double rqd_avg = 0.5 * (rqd_l + rqd_r), rqv_avg = 0.5 * (ul[4] + ur[4]);
    const double iT_avg = 0.5 * (iT_l + iT_r);
    const double vdn = n[0] * v1a + n[1] * v2a;
    const double p_int = (1.0 / iT_avg) * (R_d * rqd_avg + R_v * rqv_avg);
    const double K = 0.5 * (v1sq + v2sq);
    const double f_d = rqd_mean * vdn, f_v = rqv_mean * vdn, f_l = rql_mean * vdn;
    const double f1 = f_d + f_v + f_l;
    const double f2 = f1 * v1a + n[0] * p_int;
    const double f3 = f1 * v2a + n[1] * p_int;
    const double f4 = (c_vd * iT_mean - K) * f_d + (L_00 + c_vv * iT_mean - K) * f_v +
                      (c_pl * iT_mean - K) * f_l + v1a * f2 + v2a * f3;
    return {f1, f2, f3, f4, f_v, f_l};
  }

  // FluxLMARS, :446-485
  State flux_lmars(const State& ul, const State& ur, const double* n, double a) const {
    double p_l, T_l, p_r, T_r;
    condition(ul, p_l, T_l);
    condition(ur, p_r, T_r);
    const double v_l = (ul[1] / ul[0]) * n[0] + (ul[2] / ul[0]) * n[1];
    const double v_r = (ur[1] / ur[0]) * n[0] + (ur[2] / ur[0]) * n[1];
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double rho = 0.5 * (ul[0] + ur[0]);
    const double p_int = 0.5 * (p_l + p_r) - 0.5 * a * rho * (v_r - v_l) / nrm;
    const double v_int = 0.5 * (v_l + v_r) - 1.0 / (2.0 * a * rho) * (p_r - p_l) * nrm;
    State f;
    if (v_int > 0) {
      for (int v = 0; v < 6; ++v) f[v] = ul[v] * v_int;
      f[3] += p_l * v_int;
    } else {
      for (int v = 0; v < 6; ++v) f[v] = ur[v] * v_int;
      f[3] += p_r * v_int;
    }
    f[1] += p_int * n[0];
    f[2] += p_int * n[1];
    return f;
  }

  // max_abs_speed_naive (normal direction), :893-918
  double max_abs_speed_naive(const State& ul, const State& ur, const double* n) const {
    double p_l, T_l, p_r, T_r;
    condition(ul, p_l, T_l);
    condition(ur, p_r, T_r);
    const double vl = (ul[1] / ul[0]) * n[0] + (ul[2] / ul[0]) * n[1];
    const double vr = (ur[1] / ur[0]) * n[0] + (ur[2] / ur[0]) * n[1];
    const double cl = std::sqrt(gamma_mix(ul) * p_l / ul[0]);
    const double cr = std::sqrt(gamma_mix(ur) * p_r / ur[0]);
    return std::max(std::fabs(vl), std::fabs(vr)) +
           std::max(cl, cr) * std::sqrt(n[0] * n[0] + n[1] * n[1]);
  }

  // flux_lax_friedrichs: central flux + local Lax-Friedrichs dissipation
  State flux_llf(const State& ul, const State& ur, const double* n) const {
    const State fl = flux(ul, n), fr = flux(ur, n);
    const double lam = max_abs_speed_naive(ul, ur, n);
    State f;
    for (int v = 0; v < 6; ++v) f[v] = 0.5 * (fl[v] + fr[v]) - 0.5 * lam * (ur[v] - ul[v]);
    return f;
  }

  // boundary_condition_slip_wall with an outward normal, :85-129 (pressure
  // Riemann problem, Toro 2009 section 6.3.3)
  State slip_wall(const State& ui, const double* n) const {
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double c = n[0] / nrm, s = n[1] / nrm;
    const double vn = (c * ui[1] + s * ui[2]) / ui[0];
    double p, T;
    condition(ui, p, T);
    const double qv = ui[4] / ui[0], ql = ui[5] / ui[0];
    const double qd = 1.0 - qv - ql;
    const double gm = (qd * c_pd + qv * c_pv + ql * c_pl) * (1.0 / (qd * c_vd + qv * c_vv + ql * c_pl));
    double p_star;
    if (vn <= 0) {
      const double cs = std::sqrt(gm * p / ui[0]);
      p_star = p * std::pow(1.0 + 0.5 * (gm - 1.0) * vn / cs, 2.0 * gm * (1.0 / (gm - 1.0)));
    } else {
      const double A = 2.0 / ((gm + 1.0) * ui[0]);
      const double B = p * (gm - 1.0) / (gm + 1.0);
      p_star = p + 0.5 * vn / A * (vn + std::sqrt(vn * vn + 4.0 * A * (p + B)));
    }
    return {0.0, p_star * c * nrm, p_star * s * nrm, 0.0, 0.0, 0.0};
  }

  // the StructuredMesh variant, :132-149: flux in the +xi/+eta sense
  State slip_wall_structured(const State& ui, const double* n, int direction) const {
    if (direction % 2 == 1) {
      const double m[2] = {-n[0], -n[1]};
      State f = slip_wall(ui, m);
      for (auto& x : f) x = -x;
      return f;
    }
    return slip_wall(ui, n);
  }

  // source_terms_geopotential, :320-340
  State source_geopotential(const State& u) const {
    return {0.0, 0.0, -g * u[0], -g * u[2], 0.0, 0.0};
  }

  // phase_change_term, :405-430
  double phase_change(const State& u) const {
    double p, T;
    condition(u, p, T);
    const double rho_qd = u[0] - u[4] - u[5];
    const double T_C = T - 273.15;
    const double p_vs = 611.2 * std::exp(17.62 * T_C / (243.12 + T_C));
    const double rho_star_qv = p_vs / (R_v * T);
    const double a = rho_star_qv - u[4];
    const double b = u[0] - u[4] - rho_qd;
    return a + b - std::sqrt(a * a + b * b);
  }

  // source_terms_moist_bubble, :376-380: geopotential + phase change (:433-441)
  State source_moist_bubble(const State& u) const {
    State s = source_geopotential(u);
    const double q = phase_change(u);
    s[4] += q;
    s[5] -= q;
    return s;
  }

  // source_terms_nonhydrostatic_rayleigh_sponge, :346-373: damping of the
  // velocity towards (10, 0) in the layer z_s = 9000 < z < z_top = 16000
  State source_rayleigh_sponge(const State& u, const double* x) const {
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double z = x[1], z_s = 9000.0, z_top = 16000.0, alpha = 0.5;
    double tau = 0.0;
    if (z > z_s) {
      const double s = std::sin(0.5 * (z - z_s) * (1.0 / (z_top - z_s)));
      tau = alpha * (s * s);
    }
    return {0.0, -tau * u[0] * (v1 - 10.0), -tau * u[0] * (v2 - 0.0), 0.0, 0.0, 0.0};
  }

  // the source of examples/euler/dry_air/buoyancy/elixir_gemein_nonhydrostatic_gravity_waves.jl:50-56:
  // (geopotential + phase change) + Rayleigh sponge
  State source_gravity_wave(const State& u, const double* x) const {
    State s = source_moist_bubble(u);
    const State r = source_rayleigh_sponge(u, x);
    for (int v = 0; v < 6; ++v) s[v] += r[v];
    return s;
  }

  // max_abs_speeds, :921-930
  void max_abs_speeds(const State& u, double& l1, double& l2) const {
    double p, T;
    condition(u, p, T);
    const double c = std::sqrt(gamma_mix(u) * p / u[0]);
    l1 = std::fabs(u[1] / u[0]) + c;
    l2 = std::fabs(u[2] / u[0]) + c;
  }

  // initial_condition_convergence_test_dry, :173-200
  State ic_convergence_dry(const double* x, double t) const {
    const double pi = 3.14159265358979323846;
    const double om = 2.0 * pi * 0.5;
    const double ini = 2.0 + 0.1 * std::sin(om * (x[0] + x[1] - t));
    const double mu = c_vd;
    const double T = (ini - 1.0) / c_vd;
    const double E = mu * T + 1.0;
    return {ini, ini, ini, E * ini, 0.0, 0.0};
  }

  // source_terms_convergence_test_dry, :203-241
  State source_convergence_dry(const State& u, const double* x, double t) const {
    const double pi = 3.14159265358979323846;
    const double om = 2.0 * pi * 0.5, A = 0.1;
    const double si = std::sin(om * (x[0] + x[1] - t)), co = std::cos(om * (x[0] + x[1] - t));
    const double rho = 2.0 + A * si;
    const double rho_x = om * A * co;
    const double mu = c_vd, xi = R_d;
    const double T = (rho - 1.0) / c_vd;
    const double dT = rho_x / c_vd;
    const double E = mu * T + 1.0;
    const double dE = E * rho_x + rho * mu * dT;
    const double dp = xi * (T * rho_x + rho * dT);
    State s = source_moist_bubble(u);
    s[0] += rho_x;
    s[1] += rho_x + dp;
    s[2] += s[1];
    s[3] += dE + 2.0 * dp;
    // qv = ql = 0: du5 += 0 * du1, du6 += 0 * du1
    s[4] += 0.0 * s[0];
    s[5] += 0.0 * s[0];
    return s;
  }

  // initial_condition_convergence_test_moist, :244-272
  State ic_convergence_moist(const double* x, double t) const {
    const double pi = 3.14159265358979323846;
    const double om = 2.0 * pi * 0.5;
    const double ini = 2.0 + 0.1 * std::sin(om * (x[0] + x[1] - t));
    const double qv = 100.0 / L_00, ql = qv / 10.0;
    const double mu = (1.0 - qv - ql) * c_vd + qv * c_vv + ql * c_pl;
    const double T = (ini - 1.0) / mu + 10.0 / c_vd + 40.0;
    const double E = mu * T + qv * L_00 + 1.0;
    return {ini, ini, ini, E * ini, qv * ini, ql * ini};
  }

  // source_terms_convergence_test_moist, :275-317
  State source_convergence_moist(const State& u, const double* x, double t) const {
    const double pi = 3.14159265358979323846;
    const double om = 2.0 * pi * 0.5, A = 0.1;
    const double si = std::sin(om * (x[0] + x[1] - t)), co = std::cos(om * (x[0] + x[1] - t));
    const double rho = 2.0 + A * si;
    const double rho_x = om * A * co;
    const double qv = 100.0 / L_00, ql = qv / 10.0;
    const double mu = (1.0 - qv - ql) * c_vd + qv * c_vv + ql * c_pl;
    const double xi = (1.0 - qv - ql) * R_d + qv * R_v;
    const double T = (rho - 1.0) / mu + 10.0 / c_vd + 40.0;
    const double dT = rho_x / c_vd;
    const double E = mu * T + qv * L_00 + 1.0;
    const double dE = E * rho_x + rho * mu * dT;
    const double dp = xi * (T * rho_x + rho * dT);
    const State ue = {rho, rho, rho, rho * E, rho * qv, rho * ql};
    const State a = source_moist_bubble(u), b = source_moist_bubble(ue);
    State s;
    for (int v = 0; v < 6; ++v) s[v] = a[v] - b[v];
    s[0] += rho_x;
    s[1] += rho_x + dp;
    s[2] += rho_x + dp;
    s[3] += dE + 2.0 * dp;
    s[4] += qv * rho_x;
    s[5] += ql * rho_x;
    return s;
  }
};

}  // namespace orc
