// Device physics of CompressibleMoistEulerEquations2D
// (reference: src/equations/compressible_moist_euler_2d.jl).
// State u = (rho, rho_v1, rho_v2, rho_E, rho_qv, rho_ql); all six variables
// are evolved.  Gravity enters through source_terms_geopotential.
#pragma once
#include "tag_common.cuh"

namespace tag {

struct PhysMoist2D {
  static constexpr int NV = 6;
  static constexpr int NA = 6;
  // rho_qd, rho_qv, rho_ql, v1/2, v2/2, 1/T, (v1^2 + v2^2)/4 (odd stride)
  static constexpr int NQ = 7;
  static constexpr int kRho = 0, kBeta = 0, kLogRho = 0, kLogBeta = 0;
  static constexpr bool kNodeLogs = false;
  static constexpr bool kHasSources = true;
  static constexpr bool kSurfaceNoncons = false;  // surface flux only (flux_zero)

  struct Params {
    double c_pd, c_vd, c_pv, c_vv, c_pl, R_d, R_v, L_00, g, c_lmars;
    int surface;  // TAG_SF_LMARS, TAG_SF_LAX_FRIEDRICHS or TAG_SF_CHANDRASHEKAR
    int source;   // 0 or a TAG_SRC_* id of the moist equations
  };

  // constructor, :20-31; params = (c_pd, c_vd, c_pv, c_vv, g, c_lmars, source)
  static Params make_params(const double* p) {
    Params q;
    q.c_pd = p[0];
    q.c_vd = p[1];
    q.c_pv = p[2];
    q.c_vv = p[3];
    q.g = p[4];
    q.c_lmars = p[5];
    q.source = (int)p[6];
    q.surface = TAG_SF_LMARS;
    q.c_pl = 4186.0;
    q.R_d = q.c_pd - q.c_vd;
    q.R_v = q.c_pv - q.c_vv;
    q.L_00 = 3147620.0;
    return q;
  }

  // get_current_condition, :383-402
  TAG_DEV static void condition(const Params& P, const double* u, double& p, double& T) {
    const double rho_qd = u[0] - u[4] - u[5];
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double rho_e = u[3] - 0.5 * (u[1] * v1 + u[2] * v2);
    T = (rho_e - P.L_00 * u[4]) / (rho_qd * P.c_vd + u[4] * P.c_vv + u[5] * P.c_pl);
    p = (rho_qd * P.R_d + u[4] * P.R_v) * T;
  }

  // mixture ratio of specific heats and sound speed (:921-930)
  TAG_DEV static double sound(const Params& P, const double* u, double p) {
    const double qv = u[4] / u[0], ql = u[5] / u[0];
    const double qd = 1.0 - qv - ql;
    const double gm = (qd * P.c_pd + qv * P.c_pv + ql * P.c_pl) *
                      (1.0 / (qd * P.c_vd + qv * P.c_vv + ql * P.c_pl));
    return sqrt(gm * p / u[0]);
  }

  TAG_DEV static void node_prims(const Params& P, const double* u, double* q, unsigned& bad) {
    double p, T;
    condition(P, u, p, T);
    const double ri = 1.0 / u[0];
    const double v1 = u[1] * ri, v2 = u[2] * ri;
    q[0] = u[0] - u[4] - u[5];
    q[1] = u[4];
    q[2] = u[5];
    q[3] = 0.5 * v1;
    q[4] = 0.5 * v2;
    q[5] = 1.0 / T;
    q[6] = 0.25 * (v1 * v1 + v2 * v2);
    if (!(u[0] > 0.0)) bad |= TAG_S_NEG_DENSITY;
    if (!(p > 0.0)) bad |= TAG_S_NEG_PRESSURE;
  }

  // flux_chandrashekar (:936-1003, R_q = 0) for one symmetric pair, on the
  // half-valued node quantities of node_prims and the averaged normal.
  TAG_DEV static void volume_pair(const Params& P, const double* a, const double* b, double n1,
                                  double n2, double* Fa, double* Fb) {
    const double v1a = a[3] + b[3], v2a = a[4] + b[4];
    const double K = a[6] + b[6];
    const double vdn = n1 * v1a + n2 * v2a;
    double rqd_mean, iT_mean;
    ln_mean_pair<false>(a[0], b[0], a[5], b[5], 0.0, 0.0, 0.0, 0.0, rqd_mean, iT_mean);
    const double rqv_mean = (a[1] != 0.0 && b[1] != 0.0) ? ln_mean_single(a[1], b[1]) : 0.0;
    const double rql_mean = (a[2] != 0.0 && b[2] != 0.0) ? ln_mean_single(a[2], b[2]) : 0.0;
    const double p_int = (P.R_d * (0.5 * (a[0] + b[0])) + P.R_v * (0.5 * (a[1] + b[1]))) /
                         (0.5 * (a[5] + b[5]));
    const double f_d = rqd_mean * vdn, f_v = rqv_mean * vdn, f_l = rql_mean * vdn;
    const double f1 = f_d + f_v + f_l;
    const double f2 = f1 * v1a + n1 * p_int;
    const double f3 = f1 * v2a + n2 * p_int;
    const double f4 = (P.c_vd * iT_mean - K) * f_d + (P.L_00 + P.c_vv * iT_mean - K) * f_v +
                      (P.c_pl * iT_mean - K) * f_l + v1a * f2 + v2a * f3;
    Fa[0] = Fb[0] = f1;
    Fa[1] = Fb[1] = f2;
    Fa[2] = Fb[2] = f3;
    Fa[3] = Fb[3] = f4;
    Fa[4] = Fb[4] = f_v;
    Fa[5] = Fb[5] = f_l;
  }

  // flux(u, normal_direction), :63-82
  TAG_DEV static void flux(const Params& P, const double* u, double n1, double n2, double* f) {
    double p, T;
    condition(P, u, p, T);
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double qv = u[4] / u[0], ql = u[5] / u[0];
    const double vn = v1 * n1 + v2 * n2;
    const double rvn = u[0] * vn;
    f[0] = rvn;
    f[1] = rvn * v1 + p * n1;
    f[2] = rvn * v2 + p * n2;
    f[3] = (u[3] + p) * vn;
    f[4] = rvn * qv;
    f[5] = rvn * ql;
  }

  // FluxLMARS, :446-485
  TAG_DEV static void lmars(const Params& P, const double* ul, const double* ur, double n1,
                            double n2, double* F) {
    const double a = P.c_lmars;
    double p_l, T_l, p_r, T_r;
    condition(P, ul, p_l, T_l);
    condition(P, ur, p_r, T_r);
    const double v_l = (ul[1] / ul[0]) * n1 + (ul[2] / ul[0]) * n2;
    const double v_r = (ur[1] / ur[0]) * n1 + (ur[2] / ur[0]) * n2;
    const double nrm = sqrt(n1 * n1 + n2 * n2);
    const double rho = 0.5 * (ul[0] + ur[0]);
    const double p_int = 0.5 * (p_l + p_r) - 0.5 * a * rho * (v_r - v_l) / nrm;
    const double v_int = 0.5 * (v_l + v_r) - 1.0 / (2.0 * a * rho) * (p_r - p_l) * nrm;
    const double* us = v_int > 0.0 ? ul : ur;
    const double ps = v_int > 0.0 ? p_l : p_r;
#pragma unroll
    for (int v = 0; v < 6; ++v) F[v] = us[v] * v_int;
    F[3] += ps * v_int;
    F[1] += p_int * n1;
    F[2] += p_int * n2;
  }

  // flux_lax_friedrichs with max_abs_speed_naive (:893-918)
  TAG_DEV static void llf(const Params& P, const double* ul, const double* ur, double n1,
                          double n2, double* F) {
    double fl[6], fr[6], p_l, T_l, p_r, T_r;
    flux(P, ul, n1, n2, fl);
    flux(P, ur, n1, n2, fr);
    condition(P, ul, p_l, T_l);
    condition(P, ur, p_r, T_r);
    const double vl = (ul[1] / ul[0]) * n1 + (ul[2] / ul[0]) * n2;
    const double vr = (ur[1] / ur[0]) * n1 + (ur[2] / ur[0]) * n2;
    const double lam = fmax(fabs(vl), fabs(vr)) +
                       fmax(sound(P, ul, p_l), sound(P, ur, p_r)) * sqrt(n1 * n1 + n2 * n2);
#pragma unroll
    for (int v = 0; v < 6; ++v) F[v] = 0.5 * (fl[v] + fr[v]) - 0.5 * lam * (ur[v] - ul[v]);
  }

  TAG_DEV static void surface_flux(const Params& P, const double* ul, const double* ur, double n1,
                                   double n2, double* F) {
    if (P.surface == TAG_SF_LAX_FRIEDRICHS) {
      llf(P, ul, ur, n1, n2, F);
    } else if (P.surface == TAG_SF_CHANDRASHEKAR) {
      double qa[NQ], qb[NQ], Fb[6];
      unsigned bad = 0;
      node_prims(P, ul, qa, bad);
      node_prims(P, ur, qb, bad);
      volume_pair(P, qa, qb, n1, n2, F, Fb);
    } else {
      lmars(P, ul, ur, n1, n2, F);
    }
  }

  // boundary_condition_slip_wall with an outward normal (:85-129): the flux of
  // the pressure Riemann problem at the wall (Toro 2009, section 6.3.3)
  TAG_DEV static void slip_wall(const Params& P, const double* ui, double n1, double n2,
                                double* F) {
    const double nrm = sqrt(n1 * n1 + n2 * n2);
    const double c = n1 / nrm, s = n2 / nrm;
    const double vn = (c * ui[1] + s * ui[2]) / ui[0];
    double p, T;
    condition(P, ui, p, T);
    const double qv = ui[4] / ui[0], ql = ui[5] / ui[0];
    const double qd = 1.0 - qv - ql;
    const double gm = (qd * P.c_pd + qv * P.c_pv + ql * P.c_pl) *
                      (1.0 / (qd * P.c_vd + qv * P.c_vv + ql * P.c_pl));
    double p_star;
    if (vn <= 0.0) {
      const double cs = sqrt(gm * p / ui[0]);
      p_star = p * pow(1.0 + 0.5 * (gm - 1.0) * vn / cs, 2.0 * gm * (1.0 / (gm - 1.0)));
    } else {
      const double A = 2.0 / ((gm + 1.0) * ui[0]);
      const double B = p * (gm - 1.0) / (gm + 1.0);
      p_star = p + 0.5 * vn / A * (vn + sqrt(vn * vn + 4.0 * A * (p + B)));
    }
    F[0] = 0.0;
    F[1] = p_star * c * nrm;
    F[2] = p_star * s * nrm;
    F[3] = F[4] = F[5] = 0.0;
  }

  // kind TAG_BC_SLIP_WALL_STRUCTURED: (n1, n2) in the +xi/+eta sense; the
  // StructuredMesh method (:132-149) is the outward-normal wall evaluated with
  // the outward normal, so the OUTWARD flux is slip_wall(+-n).  Otherwise
  // (n1, n2) is already outward.
  TAG_DEV static void boundary_flux(const Params& P, const double* ui, double n1, double n2,
                                    int face, int kind, double* F) {
    if (kind == TAG_BC_SLIP_WALL_STRUCTURED && !(face & 1)) {
      n1 = -n1;
      n2 = -n2;
    }
    slip_wall(P, ui, n1, n2, F);
  }

  // phase_change_term, :405-430
  TAG_DEV static double phase_change(const Params& P, const double* u) {
    double p, T;
    condition(P, u, p, T);
    const double rho_qd = u[0] - u[4] - u[5];
    const double T_C = T - 273.15;
    const double p_vs = 611.2 * exp(17.62 * T_C / (243.12 + T_C));
    const double a = p_vs / (P.R_v * T) - u[4];
    const double b = u[0] - u[4] - rho_qd;
    return a + b - sqrt(a * a + b * b);
  }

  // source_terms_geopotential (:320-340), + phase change for the moist bubble
  // (:376-380, :433-441)
  TAG_DEV static void bubble_source(const Params& P, const double* u, bool phase, double* s) {
    s[0] = 0.0;
    s[1] = 0.0;
    s[2] = -P.g * u[0];
    s[3] = -P.g * u[2];
    const double q = phase ? phase_change(P, u) : 0.0;
    s[4] = q;
    s[5] = -q;
  }

  TAG_DEV static void source(const Params& P, const double* u, const double* x, double t,
                             double* s) {
    if (P.source == TAG_SRC_GEOPOTENTIAL || P.source == TAG_SRC_MOIST_BUBBLE) {
      bubble_source(P, u, P.source == TAG_SRC_MOIST_BUBBLE, s);
      return;
    }
    if (P.source == TAG_SRC_MOIST_GRAVITY_WAVE) {
      // + source_terms_nonhydrostatic_rayleigh_sponge (:346-373): relax the
      // velocity to (10, 0) above z_s = 9 km with
      // tau = 1/2 sin^2((z - z_s) / (2 (z_top - z_s))), z_top = 16 km
      bubble_source(P, u, true, s);
      const double z = x[1];
      double tau = 0.0;
      if (z > 9000.0) {
        const double sn = sin(0.5 * (z - 9000.0) * (1.0 / (16000.0 - 9000.0)));
        tau = 0.5 * (sn * sn);
      }
      const double v1 = u[1] / u[0], v2 = u[2] / u[0];
      s[1] += -tau * u[0] * (v1 - 10.0);
      s[2] += -tau * u[0] * (v2 - 0.0);
      return;
    }
    if (P.source != TAG_SRC_MOIST_CONVERGENCE_DRY && P.source != TAG_SRC_MOIST_CONVERGENCE) {
#pragma unroll
      for (int v = 0; v < 6; ++v) s[v] = 0.0;
      return;
    }
    // manufactured solutions of the convergence tests (:203-241, :275-317)
    const double om = 3.14159265358979323846, A = 0.1;  // 2 pi / L with L = 2
    double si, co;
    sincos(om * (x[0] + x[1] - t), &si, &co);
    const double rho = 2.0 + A * si;
    const double rho_x = om * A * co;
    if (P.source == TAG_SRC_MOIST_CONVERGENCE_DRY) {
      const double T = (rho - 1.0) / P.c_vd;
      const double dT = rho_x / P.c_vd;
      const double E = P.c_vd * T + 1.0;
      const double dE = E * rho_x + rho * P.c_vd * dT;
      const double dp = P.R_d * (T * rho_x + rho * dT);
      bubble_source(P, u, true, s);
      s[0] += rho_x;
      s[1] += rho_x + dp;
      s[2] += s[1];
      s[3] += dE + 2.0 * dp;
      s[4] += 0.0 * s[0];
      s[5] += 0.0 * s[0];
      return;
    }
    const double qv = 100.0 / P.L_00, ql = qv / 10.0;
    const double mu = (1.0 - qv - ql) * P.c_vd + qv * P.c_vv + ql * P.c_pl;
    const double xi = (1.0 - qv - ql) * P.R_d + qv * P.R_v;
    const double T = (rho - 1.0) / mu + 10.0 / P.c_vd + 40.0;
    const double dT = rho_x / P.c_vd;
    const double E = mu * T + qv * P.L_00 + 1.0;
    const double dE = E * rho_x + rho * mu * dT;
    const double dp = xi * (T * rho_x + rho * dT);
    const double ue[6] = {rho, rho, rho, rho * E, rho * qv, rho * ql};
    double se[6];
    bubble_source(P, u, true, s);
    bubble_source(P, ue, true, se);
#pragma unroll
    for (int v = 0; v < 6; ++v) s[v] -= se[v];
    s[0] += rho_x;
    s[1] += rho_x + dp;
    s[2] += rho_x + dp;
    s[3] += dE + 2.0 * dp;
    s[4] += qv * rho_x;
    s[5] += ql * rho_x;
  }

  // max_abs_speeds, :921-930
  TAG_DEV static void max_speeds(const Params& P, const double* u, double& l1, double& l2) {
    double p, T;
    condition(P, u, p, T);
    const double c = sound(P, u, p);
    l1 = fabs(u[1] / u[0]) + c;
    l2 = fabs(u[2] / u[0]) + c;
  }
};

}  // namespace tag
