// ORACLE — test infrastructure only (CPU checker for the CUDA path).
//
// Pointwise physics of `CompressibleRainyEulerEquations2D`, restated from
// src/equations/compressible_rainy_euler_2d.jl:
//   state u = (rho_dry, rho_moist, rho_rain, rho_v1, rho_v2, energy,
//              rho_vapour, rho_cloud, temperature)
// slots 7-9 hold the solution of the saturation system, updated by the Newton
// stage limiter (src/callbacks_stage/nonlinear_solve_dg2d.jl:6-44).
#pragma once
#include <array>
#include <cmath>
#include "orc_means.hpp"

namespace orc {

struct RainyEuler2D {
  static constexpr int nv = 9;
  using State = std::array<double, 9>;
  // constants, :72-109
  double c_l = 4186.0, c_pd = 1004.0, c_vd = 717.0, c_pv = 1885.0, c_vv = 1424.0;
  double R_d = 287.0, R_v = 461.0, eps = 287.0 / 461.0;
  double ref_s_p = 610.7, ref_temp = 273.15, ref_L = 2500000.0, ref_p = 100000.0;
  double g = 9.80616, N_0 = 8000000.0, v_0 = 130.0;

  // cons2nonlinearsystemsol, :219-260 (the dry branch when moist and rain are 0)
  void nlsol(const State& u, double& rv, double& rc, double& T) const {
    const double rho = u[0] + u[1] + u[2];
    const double rinv = 1.0 / rho;
    if (u[1] == 0.0 && u[2] == 0.0) {
      const double v1 = u[3] * rinv, v2 = u[4] * rinv;
      const double ek = 0.5 * (v1 * v1 + v2 * v2) * rho;
      T = (u[5] - ek) / (c_vd * rho);
      rv = 0.0;
      rc = 0.0;
      return;
    }
    rv = u[6];
    rc = u[7];
    T = u[8];
    if (rv < 0.0 && std::fabs(rv) <= 1e-15) rv = 0.0;
    if (rc < 0.0 && std::fabs(rc) <= 1e-15) rc = 0.0;
  }

  // pressure, :328-341
  double pressure(const State& u) const {
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    return (R_d * u[0] + R_v * rv) * T;
  }

  // speed_of_sound, :332-366 (returns v_sound)
  double sound(const State& u) const {
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    const double rinv = 1.0 / (u[0] + u[1] + u[2]);
    const double p = (R_d * u[0] + R_v * rv) * T;
    const double q_v = rv / u[0];
    const double q_l = (rc + u[2]) / u[0];
    const double gamma_m = 1.0 + (R_d + R_v * q_v) / (c_vd + c_vv * q_v + c_l * q_l);
    return std::sqrt(gamma_m * p * rinv);
  }

  // terminal_velocity_rain, :380-395
  double v_rain(double rho_moist, double rho_rain) const {
    if (rho_rain > 0.0)
      return v_0 * 1.9386213994279082 *
             std::pow(rho_rain / (3.14159265358979323846 * (rho_moist + rho_rain) * N_0), 0.125);
    return 0.0;
  }

  // saturation_vapour_pressure, :397-419
  double e_s(double T) const {
    const double e = ref_s_p * std::pow(T / ref_temp, (c_pv - c_l) / R_v);
    return e * std::exp(((ref_L - (c_pv - c_l) * ref_temp) / R_v) * (1.0 / ref_temp - 1.0 / T));
  }

  // saturation_vapour_pressure_derivative, :421-446
  double e_s_T(double T) const {
    const double c1 = (c_pv - c_l) / R_v;
    const double c2 = (ref_L - (c_pv - c_l) * ref_temp) / R_v;
    double d = ref_s_p / std::pow(ref_temp, c1);
    d *= (c1 * std::pow(T, c1 - 1.0) + c2 * std::pow(T, c1 - 2.0));
    d *= std::exp(c2 * (1.0 / ref_temp - 1.0 / T));
    return d;
  }

  // flux(u, normal_direction), :504-545
  State flux(const State& u, const double* n) const {
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    const double rho = u[0] + u[1] + u[2];
    const double rinv = 1.0 / rho;
    const double v1 = u[3] * rinv, v2 = u[4] * rinv;
    const double vr = v_rain(u[1], u[2]);
    const double vn = v1 * n[0] + v2 * n[1];
    const double vrn = vr * n[1];
    const double p = (R_d * u[0] + R_v * rv) * T;
    State f{};
    f[0] = u[0] * vn;
    f[1] = u[1] * vn;
    f[2] = u[2] * (vn - vrn);
    f[3] = rho * vn * v1 + p * n[0] - u[2] * vrn * v1;
    f[4] = rho * vn * v2 + p * n[1] - u[2] * vrn * v2;
    f[5] = (u[5] + p) * vn - (c_l * T + 0.5 * (v1 * v1 + v2 * v2)) * u[2] * vrn;
    return f;
  }

  // cons2speeds-based max_abs_speed_naive (normal direction), :595-611
  double max_abs_speed_naive(const State& ul, const State& ur, const double* n) const {
    auto sp = [&](const State& u, double& vn_abs) {
      const double rinv = 1.0 / (u[0] + u[1] + u[2]);
      const double v1 = u[3] * rinv, v2 = u[4] * rinv;
      vn_abs = std::fabs(v1 * n[0] + v2 * n[1]) + std::fabs(v_rain(u[1], u[2]) * n[1]);
      return sound(u);
    };
    double vl, vr;
    const double cl = sp(ul, vl), cr = sp(ur, vr);
    return std::max(vl, vr) + std::max(cl, cr) * std::sqrt(n[0] * n[0] + n[1] * n[1]);
  }

  // flux_lax_friedrichs = central flux + local Lax-Friedrichs dissipation with
  // max_abs_speed_naive (Trixi.jl; the dissipation acts on all 9 slots)
  State flux_llf(const State& ul, const State& ur, const double* n) const {
    const State fl = flux(ul, n), fr = flux(ur, n);
    const double lam = max_abs_speed_naive(ul, ur, n);
    State f;
    for (int v = 0; v < 9; ++v) f[v] = 0.5 * (fl[v] + fr[v]) - 0.5 * lam * (ur[v] - ul[v]);
    return f;
  }

  // flux_ec_rain, :872-961
  State flux_ec_rain(const State& ul, const State& ur, const double* n) const {
    double rv_l, rc_l, T_l, rv_r, rc_r, T_r;
    nlsol(ul, rv_l, rc_l, T_l);
    nlsol(ur, rv_r, rc_r, T_r);
    const double iT_l = 1.0 / T_l, iT_r = 1.0 / T_r;
    const double ri_l = 1.0 / (ul[0] + ul[1] + ul[2]), ri_r = 1.0 / (ur[0] + ur[1] + ur[2]);
    const double v1_l = ul[3] * ri_l, v2_l = ul[4] * ri_l;
    const double v1_r = ur[3] * ri_r, v2_r = ur[4] * ri_r;
    const double vr_l = v_rain(rv_l + rc_l, ul[2]);
    const double vr_r = v_rain(rv_r + rc_r, ur[2]);
    const double v1a = 0.5 * (v1_l + v1_r), v2a = 0.5 * (v2_l + v2_r);
    const double v1sq = 0.5 * (v1_l * v1_l + v1_r * v1_r);
    const double v2sq = 0.5 * (v2_l * v2_l + v2_r * v2_r);
    const double K = 0.5 * (v1sq + v2sq);
    const double vdn = n[0] * v1a + n[1] * v2a;
    const double vrn = 0.5 * n[1] * (vr_l + vr_r);
    const double rd_avg = 0.5 * (ul[0] + ur[0]);
    const double rv_avg = 0.5 * (rv_l + rv_r);
    const double rc_avg = 0.5 * (rc_l + rc_r);
    const double rr_avg = 0.5 * (ul[2] + ur[2]);
    const double rd_log = (ul[0] != 0.0 && ur[0] != 0.0) ? ln_mean(ul[0], ur[0]) : 0.0;
    const double rv_log = (rv_l != 0.0 && rv_r != 0.0) ? ln_mean(rv_l, rv_r) : 0.0;
    (void)rc_avg;
    const double iT_avg = 0.5 * (iT_l + iT_r);
    const double iT_log = inv_ln_mean(iT_l, iT_r);
    const double p_int = (1.0 / iT_avg) * (R_d * rd_avg + R_v * rv_avg);
    const double f_v = rv_log * vdn;
    const double f_c = rc_avg * vdn;
    const double f_d = rd_log * vdn;
    const double f_r = rr_avg * (vdn - vrn);
    const double f_m = f_v + f_c;
    const double f_rho = f_d + f_m + f_r;
    const double f_m1 = f_rho * v1a + p_int * n[0];
    const double f_m2 = f_rho * v2a + p_int * n[1];
    const double f_e = (c_vd * iT_log - K) * f_d + (c_vv * iT_log - K + ref_L) * f_v +
                       (c_l * iT_log - K) * (f_c + f_r) + (v1a * f_m1 + v2a * f_m2);
    return {f_d, f_m, f_r, f_m1, f_m2, f_e, 0.0, 0.0, 0.0};
  }

  // boundary_condition_simple_slip_wall as reached from a StructuredMesh
  // (:973-994): the normal vector arrives in the `orientation` slot, so
  // `orientation == 1` is false and rho_v2 is mirrored; states ordered by the
  // parity of the (1-based) direction; flux in the +xi/+eta sense.
  State slip_wall_structured(const State& ui, const double* n, int direction) const {
    State ub = ui;
    ub[4] = -ui[4];
    if (direction % 2 == 0) return flux_llf(ui, ub, n);
    return flux_llf(ub, ui, n);
  }

  // flux_LMARS, :817-861 (a = 360, beta = 1): the upwind state times the
  // interface velocity plus the interface pressure
  State flux_lmars(const State& ul, const State& ur, const double* n) const {
    const double a = 360.0, beta = 1.0;
    const double rho_l = ul[0] + ul[1] + ul[2], rho_r = ur[0] + ur[1] + ur[2];
    const double ri_l = 1.0 / rho_l, ri_r = 1.0 / rho_r;
    const double p_l = pressure(ul), p_r = pressure(ur);
    const double v_l = (ul[3] * ri_l) * n[0] + (ul[4] * ri_l) * n[1];
    const double v_r = (ur[3] * ri_r) * n[0] + (ur[4] * ri_r) * n[1];
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double rho = 0.5 * (rho_l + rho_r);
    const double p_int = 0.5 * (p_l + p_r) - beta * 0.5 * a * rho * (v_r - v_l) / nrm;
    const double v_int = 0.5 * (v_l + v_r) - beta * 1.0 / (2.0 * a * rho) * (p_r - p_l) * nrm;
    const State& us = v_int > 0 ? ul : ur;
    const double ps = v_int > 0 ? p_l : p_r;
    return {us[0] * v_int, us[1] * v_int, 0.0, us[3] * v_int + p_int * n[0],
            us[4] * v_int + p_int * n[1], us[5] * v_int + ps * v_int, 0.0, 0.0, 0.0};
  }

  // boundary_condition_slip_wall with an outward normal, :639-686: the wall
  // pressure of the normal Riemann problem (Toro 2009, section 6.3.3)
  State slip_wall(const State& ui, const double* n) const {
    const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1]);
    const double c = n[0] / nrm, s = n[1] / nrm;
    const double rho = ui[0] + ui[1] + ui[2];
    const double rinv = 1.0 / rho;
    const double v_normal = (c * ui[3] + s * ui[4]) * rinv;
    double rv, rc, T;
    nlsol(ui, rv, rc, T);
    const double p = (R_d * ui[0] + R_v * rv) * T;
    const double q_v = rv / ui[0], q_l = (rc + ui[2]) / ui[0];
    const double gamma = 1.0 + (R_d + R_v * q_v) / (c_vd + c_vv * q_v + c_l * q_l);
    double p_star;
    if (v_normal <= 0.0) {
      const double v_sound = std::sqrt(gamma * p * rinv);
      p_star = p * std::pow(1.0 + 0.5 * (gamma - 1.0) * v_normal / v_sound,
                            2.0 * gamma * (1.0 / (gamma - 1.0)));
    } else {
      const double A = 2.0 / ((gamma + 1.0) * rho);
      const double B = p * (gamma - 1.0) / (gamma + 1.0);
      p_star = p + 0.5 * v_normal / A *
                       (v_normal + std::sqrt(v_normal * v_normal + 4.0 * A * (p + B)));
    }
    return {0.0, 0.0, 0.0, p_star * c * nrm, p_star * s * nrm, 0.0, 0.0, 0.0, 0.0};
  }

  // its StructuredMesh method, :689-705: on the negative faces (odd 1-based
  // direction) the outward-normal wall of -n, sign flipped back
  State slip_wall_pressure_structured(const State& ui, const double* n, int direction) const {
    if (direction % 2 == 1) {
      const double m[2] = {-n[0], -n[1]};
      State f = slip_wall(ui, m);
      for (double& x : f) x = -x;
      return f;
    }
    return slip_wall(ui, n);
  }

  // source_terms_no_phase_change, :580-593: gravity only
  State source_no_phase_change(const State& u) const {
    const double rho = u[0] + u[1] + u[2];
    return {0.0, 0.0, 0.0, 0.0, -g * rho, -g * u[4], 0.0, 0.0, 0.0};
  }

  // source_terms_rainy, :548-577
  State source_rainy(const State& u) const {
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    const double rho = u[0] + u[1] + u[2];
    const double rho_vs = e_s(T) / (R_v * T);
    double S_ev = (3.86e-3 - 9.41e-5 * (T - ref_temp)) * (1.0 + 9.1 * std::pow(u[2], 0.1875));
    S_ev *= (rho_vs - rv) * std::pow(u[2], 0.5);
    const double S_auto = 0.001 * rc;
    const double S_acc = 1.72 * rc * std::pow(u[2], 0.875);
    const double S_rain = S_auto + S_acc - S_ev;
    return {0.0, -S_rain, S_rain, 0.0, -rho * g, -u[4] * g, 0.0, 0.0, 0.0};
  }

  // max_abs_speeds, :588-593
  void max_abs_speeds(const State& u, double& l1, double& l2) const {
    const double rinv = 1.0 / (u[0] + u[1] + u[2]);
    const double v1 = u[3] * rinv, v2 = u[4] * rinv;
    const double c = sound(u);
    l1 = std::fabs(v1) + c;
    l2 = std::fabs(v2) + c + std::fabs(v_rain(u[1], u[2]));
  }

  // saturation_residual, :738-772
  void residual(const State& u, const double* x, double* r) const {
    const double rho = u[0] + u[1] + u[2];
    const double rinv = 1.0 / rho;
    const double v1 = u[3] * rinv, v2 = u[4] * rinv;
    double r1 = (c_vd * u[0] + c_vv * x[0] + c_l * (x[1] + u[2])) * x[2];
    r1 += x[0] * ref_L;
    r1 -= (u[5] - rho * 0.5 * (v1 * v1 + v2 * v2));
    double r2 = std::min(e_s(x[2]) / (R_v * x[2]), u[1]);
    r2 -= x[0];
    r2 *= 1.0e7;
    double r3 = u[1];
    r3 -= x[0] + x[1];
    r3 *= 1.0e7;
    r[0] = r1;
    r[1] = r2;
    r[2] = r3;
  }

  // saturation_residual_jacobian, :774-809 (row-major J[3][3])
  void jacobian(const State& u, const double* x, double* J) const {
    const double svp = e_s(x[2]);
    const double svp_t = e_s_T(x[2]);
    J[0] = c_vv * x[2] + ref_L;
    J[1] = c_l * x[2];
    J[2] = c_vd * u[0] + c_vv * x[0] + c_l * (x[1] + u[2]);
    J[3] = -10000000.0;
    J[4] = 0.0;
    J[5] = (svp / (R_v * x[2]) < u[1]) ? (svp_t * x[2] - svp) / (R_v * x[2] * x[2]) * 1.0e7 : 0.0;
    J[6] = -10000000.0;
    J[7] = -10000000.0;
    J[8] = 0.0;
  }
};

}  // namespace orc
