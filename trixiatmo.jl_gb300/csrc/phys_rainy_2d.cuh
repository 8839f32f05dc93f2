// Device physics of CompressibleRainyEulerEquations2D
// (reference: src/equations/compressible_rainy_euler_2d.jl).
// State u = (rho_dry, rho_moist, rho_rain, rho_v1, rho_v2, energy, rho_vapour,
// rho_cloud, temperature); slots 7-9 are the saturation-system unknowns (set by
// the Newton stage limiter).  All 9 slots are evolved: the volume flux of
// slots 7-9 is zero but the Lax-Friedrichs dissipation acts on them.
#pragma once
#include "tag_common.cuh"

namespace tag {

struct RainyConst {
  // :72-109
  static constexpr double c_l = 4186.0, c_pd = 1004.0, c_vd = 717.0, c_pv = 1885.0, c_vv = 1424.0;
  static constexpr double R_d = 287.0, R_v = 461.0;
  static constexpr double ref_s_p = 610.7, ref_temp = 273.15, ref_L = 2500000.0;
  static constexpr double g = 9.80616, N_0 = 8000000.0, v_0 = 130.0;
  static constexpr double pi = 3.14159265358979323846;
};

// saturation_vapour_pressure (:397-419),
//   e_s(T) = ref_s_p (T / ref_temp)^c1 exp(c2 (1 / ref_temp - 1 / T)),
// evaluated as ref_s_p exp(c1 log(T / ref_temp) + c2 (1 / ref_temp - 1 / T)):
// one logarithm and one exponential where the power costs both again (FP64
// transcendentals are the rainy kernels' main cost).  Relative difference to
// the reference's form: a few ulp.
constexpr double kRainyC1 = (RainyConst::c_pv - RainyConst::c_l) / RainyConst::R_v;
constexpr double kRainyC2 =
    (RainyConst::ref_L - (RainyConst::c_pv - RainyConst::c_l) * RainyConst::ref_temp) /
    RainyConst::R_v;

TAG_DEV double rainy_e_s(double T) {
  using C = RainyConst;
  return C::ref_s_p * exp(kRainyC1 * log(T / C::ref_temp) + kRainyC2 * (1.0 / C::ref_temp - 1.0 / T));
}

// saturation_vapour_pressure_derivative (:421-446) from the value e_s = e_s(T):
// the reference's ref_s_p / ref_temp^c1 (c1 T^(c1-1) + c2 T^(c1-2)) exp(...)
// equals e_s(T) (c1 + c2 / T) / T
TAG_DEV double rainy_e_s_T_from(double T, double e_s) { return e_s * (kRainyC1 + kRainyC2 / T) / T; }

TAG_DEV double rainy_e_s_T(double T) { return rainy_e_s_T_from(T, rainy_e_s(T)); }

// x^(1/8) by three correctly rounded square roots (x^0.125 to a few ulp;
// NaN for x < 0, as the power)
TAG_DEV double rainy_root8(double x) { return sqrt(sqrt(sqrt(x))); }

// terminal_velocity_rain, :380-395
TAG_DEV double rainy_v_rain(double rho_moist, double rho_rain) {
  using C = RainyConst;
  if (rho_rain > 0.0)
    return C::v_0 * 1.9386213994279082 *
           rainy_root8(rho_rain / (C::pi * (rho_moist + rho_rain) * C::N_0));
  return 0.0;
}

struct PhysRainy2D {
  static constexpr int NV = 9;
  static constexpr int NA = 9;
  // rho_d, rho_m, rho_r, v1/2, v2/2, rho_vapour, rho_cloud, T, 1/T,
  // v_rain(rho_vapour + rho_cloud, rho_r), (v1^2 + v2^2)/4
  static constexpr int NQ = 11;
  static constexpr int kRho = 0, kBeta = 0, kLogRho = 0, kLogBeta = 0;
  static constexpr bool kNodeLogs = false;
  static constexpr bool kHasSources = true;
  static constexpr bool kSurfaceNoncons = false;  // surface flux only (flux_zero)

  struct Params {
    int source_kind;  // TAG_SRC_RAINY, TAG_SRC_RAINY_CONVERGENCE or TAG_SRC_RAINY_NO_PHASE_CHANGE
    int lmars;        // surface flux: 0 flux_lax_friedrichs, 1 flux_LMARS
  };

  // params = (source kind); the surface flux is set from the configuration
  static Params make_params(const double* p, int surface_flux = TAG_SF_LAX_FRIEDRICHS) {
    Params q;
    q.source_kind = (int)p[0];
    q.lmars = surface_flux == TAG_SF_LMARS;
    return q;
  }

  // cons2nonlinearsystemsol, :219-260
  TAG_DEV static void nlsol(const double* u, double& rv, double& rc, double& T) {
    using C = RainyConst;
    const double rho = u[0] + u[1] + u[2];
    if (u[1] == 0.0 && u[2] == 0.0) {
      const double ri = 1.0 / rho;
      const double v1 = u[3] * ri, v2 = u[4] * ri;
      T = (u[5] - 0.5 * (v1 * v1 + v2 * v2) * rho) / (C::c_vd * rho);
      rv = 0.0;
      rc = 0.0;
      return;
    }
    rv = u[6];
    rc = u[7];
    T = u[8];
    if (rv < 0.0 && fabs(rv) <= 1e-15) rv = 0.0;
    if (rc < 0.0 && fabs(rc) <= 1e-15) rc = 0.0;
  }

  TAG_DEV static void node_prims(const Params&, const double* u, double* q, unsigned& bad) {
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    const double ri = 1.0 / (u[0] + u[1] + u[2]);
    const double v1 = u[3] * ri, v2 = u[4] * ri;
    q[0] = u[0];
    q[1] = u[1];
    q[2] = u[2];
    q[3] = 0.5 * v1;
    q[4] = 0.5 * v2;
    q[5] = rv;
    q[6] = rc;
    q[7] = T;
    q[8] = 1.0 / T;
    q[9] = rainy_v_rain(rv + rc, u[2]);
    q[10] = 0.25 * (v1 * v1 + v2 * v2);
    if (!(u[0] > 0.0)) bad |= TAG_S_NEG_DENSITY;
    if (!(T > 0.0)) bad |= TAG_S_NEG_PRESSURE;
  }

  // flux_ec_rain, :872-961, for one symmetric pair (no nonconservative part)
  TAG_DEV static void volume_pair(const Params&, const double* a, const double* b, double n1,
                                  double n2, double* Fa, double* Fb) {
    using C = RainyConst;
    const double v1a = a[3] + b[3], v2a = a[4] + b[4];
    const double K = a[10] + b[10];
    const double vdn = n1 * v1a + n2 * v2a;
    const double vrn = 0.5 * n2 * (a[9] + b[9]);
    const double rd_avg = 0.5 * (a[0] + b[0]);
    const double rv_avg = 0.5 * (a[5] + b[5]);
    const double rc_avg = 0.5 * (a[6] + b[6]);
    const double rr_avg = 0.5 * (a[2] + b[2]);
    // ln_mean of the dry densities, inv_ln_mean of 1/T and 1/(1/T_a + 1/T_b)
    // (= 1/(2 iT_avg), the pressure's divisor) from one shared reciprocal
    double rd_log, iT_log, i_sum;
    if (a[0] != 0.0 && b[0] != 0.0) {
      ln_mean_pair<false, true>(a[0], b[0], a[8], b[8], 0.0, 0.0, 0.0, 0.0, rd_log, iT_log,
                                &i_sum);
    } else {
      rd_log = 0.0;
      iT_log = inv_ln_mean_single(a[8], b[8]);
      i_sum = 1.0 / (a[8] + b[8]);
    }
    const double rv_log = (a[5] != 0.0 && b[5] != 0.0) ? ln_mean_single(a[5], b[5]) : 0.0;
    const double p_int = (C::R_d * rd_avg + C::R_v * rv_avg) * (2.0 * i_sum);
    const double f_v = rv_log * vdn;
    const double f_c = rc_avg * vdn;
    const double f_d = rd_log * vdn;
    const double f_r = rr_avg * (vdn - vrn);
    const double f_m = f_v + f_c;
    const double f_rho = f_d + f_m + f_r;
    const double f_m1 = f_rho * v1a + p_int * n1;
    const double f_m2 = f_rho * v2a + p_int * n2;
    const double f_e = (C::c_vd * iT_log - K) * f_d + (C::c_vv * iT_log - K + C::ref_L) * f_v +
                       (C::c_l * iT_log - K) * (f_c + f_r) + (v1a * f_m1 + v2a * f_m2);
    Fa[0] = Fb[0] = f_d;
    Fa[1] = Fb[1] = f_m;
    Fa[2] = Fb[2] = f_r;
    Fa[3] = Fb[3] = f_m1;
    Fa[4] = Fb[4] = f_m2;
    Fa[5] = Fb[5] = f_e;
    Fa[6] = Fb[6] = 0.0;
    Fa[7] = Fb[7] = 0.0;
    Fa[8] = Fb[8] = 0.0;
  }

  // flux(u, normal_direction), :504-545
  TAG_DEV static void flux(const Params&, const double* u, double n1, double n2, double* f) {
    using C = RainyConst;
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    const double rho = u[0] + u[1] + u[2];
    const double ri = 1.0 / rho;
    const double v1 = u[3] * ri, v2 = u[4] * ri;
    const double vr = rainy_v_rain(u[1], u[2]);
    const double vn = v1 * n1 + v2 * n2;
    const double vrn = vr * n2;
    const double p = (C::R_d * u[0] + C::R_v * rv) * T;
    f[0] = u[0] * vn;
    f[1] = u[1] * vn;
    f[2] = u[2] * (vn - vrn);
    f[3] = rho * vn * v1 + p * n1 - u[2] * vrn * v1;
    f[4] = rho * vn * v2 + p * n2 - u[2] * vrn * v2;
    f[5] = (u[5] + p) * vn - (C::c_l * T + 0.5 * (v1 * v1 + v2 * v2)) * u[2] * vrn;
    f[6] = f[7] = f[8] = 0.0;
  }

  // flux(u, n) together with the two speeds of max_abs_speed_naive
  // (:595-611) at the same state: |v.n| + |v_rain n2| and the speed of sound,
  // each primitive computed once
  TAG_DEV static void flux_and_speeds(const double* u, double n1, double n2, double* f,
                                      double& vabs, double& c) {
    using C = RainyConst;
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    const double rho = u[0] + u[1] + u[2];
    const double ri = 1.0 / rho;
    const double v1 = u[3] * ri, v2 = u[4] * ri;
    const double vr = rainy_v_rain(u[1], u[2]);
    const double vn = v1 * n1 + v2 * n2;
    const double vrn = vr * n2;
    const double p = (C::R_d * u[0] + C::R_v * rv) * T;
    f[0] = u[0] * vn;
    f[1] = u[1] * vn;
    f[2] = u[2] * (vn - vrn);
    f[3] = rho * vn * v1 + p * n1 - u[2] * vrn * v1;
    f[4] = rho * vn * v2 + p * n2 - u[2] * vrn * v2;
    f[5] = (u[5] + p) * vn - (C::c_l * T + 0.5 * (v1 * v1 + v2 * v2)) * u[2] * vrn;
    f[6] = f[7] = f[8] = 0.0;
    vabs = fabs(vn) + fabs(vrn);
    const double q_v = rv / u[0];
    const double q_l = (rc + u[2]) / u[0];
    const double gm = 1.0 + (C::R_d + C::R_v * q_v) / (C::c_vd + C::c_vv * q_v + C::c_l * q_l);
    c = sqrt(gm * p * ri);
  }

  // speed_of_sound (:332-366) and the normal speeds of max_abs_speed_naive (:595-611)
  TAG_DEV static double sound(const double* u) {
    using C = RainyConst;
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    const double ri = 1.0 / (u[0] + u[1] + u[2]);
    const double p = (C::R_d * u[0] + C::R_v * rv) * T;
    const double q_v = rv / u[0];
    const double q_l = (rc + u[2]) / u[0];
    const double gm = 1.0 + (C::R_d + C::R_v * q_v) / (C::c_vd + C::c_vv * q_v + C::c_l * q_l);
    return sqrt(gm * p * ri);
  }

  // pressure(u), :328-341
  TAG_DEV static double pressure(const double* u) {
    using C = RainyConst;
    double rv, rc, T;
    nlsol(u, rv, rc, T);
    return (C::R_d * u[0] + C::R_v * rv) * T;
  }

  // flux_LMARS, :817-861 (speed of sound a = 360, beta = 1): upwinded
  // transport of the whole state plus the interface pressure
  TAG_DEV static void lmars(const double* ul, const double* ur, double n1, double n2, double* F) {
    const double a = 360.0;
    const double rl = ul[0] + ul[1] + ul[2], rr = ur[0] + ur[1] + ur[2];
    const double ril = 1.0 / rl, rir = 1.0 / rr;
    const double pl = pressure(ul), pr = pressure(ur);
    const double vl = (ul[3] * ril) * n1 + (ul[4] * ril) * n2;
    const double vr = (ur[3] * rir) * n1 + (ur[4] * rir) * n2;
    const double nrm = sqrt(n1 * n1 + n2 * n2);
    const double rho = 0.5 * (rl + rr);
    const double p_int = 0.5 * (pl + pr) - 0.5 * a * rho * (vr - vl) / nrm;
    const double v_int = 0.5 * (vl + vr) - 1.0 / (2.0 * a * rho) * (pr - pl) * nrm;
    const double* us = v_int > 0.0 ? ul : ur;
    const double ps = v_int > 0.0 ? pl : pr;
    F[0] = us[0] * v_int;
    F[1] = us[1] * v_int;
    F[2] = 0.0;
    F[3] = us[3] * v_int + p_int * n1;
    F[4] = us[4] * v_int + p_int * n2;
    F[5] = us[5] * v_int + ps * v_int;
    F[6] = F[7] = F[8] = 0.0;
  }

  // boundary_condition_slip_wall with an outward normal (:639-686): the
  // pressure of the Riemann problem against the wall (Toro 2009, 6.3.3)
  TAG_DEV static void slip_wall(const double* ui, double n1, double n2, double* F) {
    using C = RainyConst;
    const double nrm = sqrt(n1 * n1 + n2 * n2);
    const double c = n1 / nrm, s = n2 / nrm;
    const double rho = ui[0] + ui[1] + ui[2];
    const double ri = 1.0 / rho;
    const double vn = (c * ui[3] + s * ui[4]) * ri;
    double rv, rc, T;
    nlsol(ui, rv, rc, T);
    const double p = (C::R_d * ui[0] + C::R_v * rv) * T;
    const double q_v = rv / ui[0];
    const double q_l = (rc + ui[2]) / ui[0];
    const double gm = 1.0 + (C::R_d + C::R_v * q_v) / (C::c_vd + C::c_vv * q_v + C::c_l * q_l);
    double p_star;
    if (vn <= 0.0) {
      const double cs = sqrt(gm * p * ri);
      p_star = p * pow(1.0 + 0.5 * (gm - 1.0) * vn / cs, 2.0 * gm * (1.0 / (gm - 1.0)));
    } else {
      const double A = 2.0 / ((gm + 1.0) * rho);
      const double B = p * (gm - 1.0) / (gm + 1.0);
      p_star = p + 0.5 * vn / A * (vn + sqrt(vn * vn + 4.0 * A * (p + B)));
    }
    F[0] = F[1] = F[2] = 0.0;
    F[3] = p_star * c * nrm;
    F[4] = p_star * s * nrm;
    F[5] = F[6] = F[7] = F[8] = 0.0;
  }

  // flux_lax_friedrichs: central flux + 0.5 max_abs_speed_naive (u_rr - u_ll);
  // or flux_LMARS
  TAG_DEV static void surface_flux(const Params& P, const double* ul, const double* ur, double n1,
                                   double n2, double* F) {
    if (P.lmars) {
      lmars(ul, ur, n1, n2, F);
      return;
    }
    double fl[9], fr[9], vl, vr, cl, cr;
    flux_and_speeds(ul, n1, n2, fl, vl, cl);
    flux_and_speeds(ur, n1, n2, fr, vr, cr);
    const double lam = fmax(vl, vr) + fmax(cl, cr) * sqrt(n1 * n1 + n2 * n2);
#pragma unroll
    for (int v = 0; v < 9; ++v) F[v] = 0.5 * (fl[v] + fr[v]) - 0.5 * lam * (ur[v] - ul[v]);
  }

  // kind TAG_BC_SIMPLE_SLIP_WALL: boundary_condition_simple_slip_wall reached
  // from a StructuredMesh (:973-994): rho_v2 mirrored, states ordered by the
  // face parity.  TAG_BC_SLIP_WALL_STRUCTURED: boundary_condition_slip_wall's
  // StructuredMesh method (:689-705), the outward-normal wall evaluated with
  // the outward normal (-n on the negative faces).  Both return the OUTWARD flux.
  TAG_DEV static void boundary_flux(const Params& P, const double* ui, double n1, double n2,
                                    int face, int kind, double* F) {
    if (kind == TAG_BC_SLIP_WALL_STRUCTURED || kind == TAG_BC_SLIP_WALL_NORMAL) {
      if (kind == TAG_BC_SLIP_WALL_STRUCTURED && !(face & 1)) {
        n1 = -n1;
        n2 = -n2;
      }
      slip_wall(ui, n1, n2, F);
      return;
    }
    double ub[9];
#pragma unroll
    for (int v = 0; v < 9; ++v) ub[v] = ui[v];
    ub[4] = -ui[4];
    if (face & 1) {
      surface_flux(P, ui, ub, n1, n2, F);
    } else {
      surface_flux(P, ub, ui, n1, n2, F);
#pragma unroll
      for (int v = 0; v < 9; ++v) F[v] = -F[v];
    }
  }

  // source_terms_rainy (:548-577), source_terms_no_phase_change (:580-593)
  // or the manufactured source of
  // examples/euler/precipitation/tests/convergence_test.jl:42-124; s[9]
  TAG_DEV static void source(const Params& P, const double* u, const double* x, double t,
                             double* s) {
    using C = RainyConst;
    if (P.source_kind == TAG_SRC_RAINY_NO_PHASE_CHANGE) {
      const double rho = u[0] + u[1] + u[2];
#pragma unroll
      for (int v = 0; v < 9; ++v) s[v] = 0.0;
      s[4] = -C::g * rho;
      s[5] = -C::g * u[4];
      return;
    }
    if (P.source_kind == TAG_SRC_RAINY) {
      double rv, rc, T;
      nlsol(u, rv, rc, T);
      const double rho = u[0] + u[1] + u[2];
      const double rho_vs = rainy_e_s(T) / (C::R_v * T);
      // rho_r^0.1875, rho_r^0.5 and rho_r^0.875 from square roots: with
      // r8 = rho_r^(1/8) and r16 = r8^(1/2), r16^3, sqrt(rho_r) and r8^7
      const double r8 = rainy_root8(u[2]), r16 = sqrt(r8);
      const double r8_2 = r8 * r8, r8_4 = r8_2 * r8_2;
      double S_ev = (3.86e-3 - 9.41e-5 * (T - C::ref_temp)) * (1.0 + 9.1 * (r16 * r16 * r16));
      S_ev *= (rho_vs - rv) * sqrt(u[2]);
      const double S_auto = 0.001 * rc;
      const double S_acc = 1.72 * rc * (r8_4 * r8_2 * r8);
      const double S_rain = S_auto + S_acc - S_ev;
      s[0] = 0.0; s[1] = -S_rain; s[2] = S_rain; s[3] = 0.0;
      s[4] = -rho * C::g; s[5] = -u[4] * C::g; s[6] = s[7] = s[8] = 0.0;
      return;
    }
    // manufactured solution (source kind TAG_SRC_RAINY_CONVERGENCE)
    const double c_help = C::v_0 * 1.9386213994279082 * pow(C::pi * C::N_0, -0.125);
    const double A = 0.1, om = 2.0 * C::pi / 2.0;
    double si, co;
    sincos(om * (x[0] + x[1] - t), &si, &co);
    const double rho = 2.0 + A * si;
    const double rho_x = om * A * co, rho_t = -rho_x;
    const double T = rho + 250.0;
    const double svp = rainy_e_s(T), dsvp = rainy_e_s_T(T);
    const double rv = svp / (C::R_v * T);
    const double rc = rho / C::c_l * 3000.0, rr = rho / C::c_l * 1000.0;
    const double rm = rv + rc, rd = rho - rm - rr;
    const double vr = rainy_v_rain(rm, rr);
    const double svp_t = rho_t * dsvp, svp_x = rho_x * dsvp;
    const double rv_t = (svp_t * T - rho_t * svp) / (C::R_v * T * T);
    const double rv_x = (svp_x * T - rho_x * svp) / (C::R_v * T * T);
    const double rc_t = rho_t / C::c_l * 3000.0, rc_x = rho_x / C::c_l * 3000.0;
    const double rr_t = rho_t / C::c_l * 1000.0, rr_x = rho_x / C::c_l * 1000.0;
    const double rm_t = rv_t + rc_t, rm_x = rv_x + rc_x;
    const double rd_t = rho_t - rm_t - rr_t, rd_x = rho_x - rm_x - rr_x;
    double e_t = (C::c_vd * rd_t + C::c_vv * rv_t + C::c_l * (rc_t + rr_t)) * T;
    e_t += (C::c_vd * rd + C::c_vv * rv + C::c_l * (rc + rr)) * rho_t;
    e_t += rv_t * C::ref_L + rho_t;
    double e_x = (C::c_vd * rd_x + C::c_vv * rv_x + C::c_l * (rc_x + rr_x)) * T;
    e_x += (C::c_vd * rd + C::c_vv * rv + C::c_l * (rc + rr)) * rho_x;
    e_x += rv_x * C::ref_L + rho_x;
    double p_x = (rd_x * C::R_d + rv_x * C::R_v) * T;
    p_x += (rd * C::R_d + rv * C::R_v) * rho_x;
    double vr_x = c_help * 0.125 * ((rr_x * rm - rr * rm_x) / ((rm + rr) * (rm + rr)));
    vr_x *= pow(rr / (rm + rr), -0.875);
    const double rrvr_x = rr_x * vr + rr * vr_x;
    s[0] = rd_t + 2.0 * rd_x;
    s[1] = rm_t + 2.0 * rm_x;
    s[2] = rr_t + 2.0 * rr_x - rrvr_x;
    s[3] = rho_x + p_x - rrvr_x;
    s[4] = rho_x + p_x - rrvr_x;
    s[5] = e_t + 2.0 * (e_x + p_x) - (C::c_l * rho_x * rr * vr) - (C::c_l * T + 1.0) * rrvr_x;
    s[6] = s[7] = s[8] = 0.0;
    (void)u;
  }

  // max_abs_speeds, :588-593
  TAG_DEV static void max_speeds(const Params&, const double* u, double& l1, double& l2) {
    const double ri = 1.0 / (u[0] + u[1] + u[2]);
    const double c = sound(u);
    l1 = fabs(u[3] * ri) + c;
    l2 = fabs(u[4] * ri) + c + fabs(rainy_v_rain(u[1], u[2]));
  }
};

}  // namespace tag
