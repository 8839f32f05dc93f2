// Device physics of CompressibleEulerPotentialTemperatureEquationsWithGravity2D
// (reference: src/equations/compressible_euler_potential_temperature_gravity_2d.jl).
// State u = (rho, rho_v1, rho_v2, rho_theta, phi), p = K rho_theta^gamma; phi = g z
// is passive, so kernels evolve NA = 4 variables.  Volume fluxes flux_tec /
// flux_ec / flux_etec with the nonconservative gravity term of Waruszewski et al.
// (or Artiano et al., Souza et al.); surface flux (FluxLMARS(c), flux_zero).
//
// The Stolarsky mean S(x, y) = (gamma-1)/gamma (y^g - x^g) / (y^(g-1) - x^(g-1))
// (Winters et al. 2020) is evaluated as (x+y)/2 R(f^2), f = (y-x)/(x+y), with the
// first eight terms of its series in f^2 when f^2 < 1e-2 (coefficients from the
// binomial expansions of (1 +- f)^a, computed on the host per gamma), else from
// per-node powers x^g, x^(g-1) with one division per pair.
#pragma once
#include "tag_common.cuh"

namespace tag {

struct PhysPT2D {
  static constexpr int NV = 5;
  static constexpr int NA = 4;
  // rho, v1/2, v2/2, p/2, phi/2, rho_theta, sigma = rho/rho_theta,
  // rho_theta^gamma, rho_theta^(gamma-1), rho^gamma, rho^(gamma-1) (odd stride)
  static constexpr int NQ = 11;
  static constexpr int kRho = 0, kBeta = 0, kLogRho = 0, kLogBeta = 0;
  static constexpr bool kNodeLogs = false;
  // MountainWaveSetup's Rayleigh damping when set (Params::mountain)
  static constexpr bool kHasSources = true;
  // surface flux (FluxLMARS(c), flux_zero) or (flux_ec, a nonconservative
  // gravity term); the interface kernel adds the per-side term when snc >= 0
  static constexpr bool kSurfaceNoncons = true;

  struct Params {
    double gamma, K, c_lmars, stol_fac;  // stol_fac = (gamma - 1) / gamma
    double sc[8];                        // Stolarsky series coefficients
    int volume;                          // 0 flux_tec, 1 flux_ec, 2 flux_etec,
                                         // 3 flux_kennedy_gruber (3D only)
    int nc;                              // 0 waruszewski, 1 artiano, 2 souza
    int surface;                         // 0 FluxLMARS(c), 1 flux_ec
    int snc;                             // surface gravity term: -1 none (flux_zero), else as nc
    int mountain;                        // 1: MountainWaveSetup's damping source
    double g;                            // gravity
    double mw[8];  // theta_0, u0, N, z_damping_start, z_damping_end, x_damping_start,
                   // x_damping_end, damping_rate
  };

  // params = (c_p, c_v, g, LMARS c, nonconservative kind, volume kind,
  // surface kind, surface nonconservative kind + 1)
  static Params make_params(const double* p) {
    Params q;
    const double c_p = p[0], c_v = p[1], R = c_p - c_v;
    q.gamma = c_p / c_v;
    q.K = 100000.0 * pow(R / 100000.0, q.gamma);
    q.c_lmars = p[3];
    q.stol_fac = (q.gamma - 1.0) / q.gamma;
    q.nc = (int)p[4];
    q.volume = (int)p[5];
    q.surface = (int)p[6];
    q.snc = (int)p[7] - 1;
    q.mountain = 0;
    q.g = p[2];
    for (int k = 0; k < 8; ++k) q.mw[k] = 0.0;
    double a[8], b[8];
    for (int j = 0; j < 8; ++j) {
      double ra = 1.0, rb = 1.0;
      for (int i = 0; i < 2 * j + 1; ++i) {
        ra = ra * (q.gamma - i) / (i + 1);
        rb = rb * (q.gamma - 1.0 - i) / (i + 1);
      }
      a[j] = ra / q.gamma;
      b[j] = rb / (q.gamma - 1.0);
    }
    for (int k = 0; k < 8; ++k) {
      double s = a[k];
      for (int i = 1; i <= k; ++i) s -= b[i] * q.sc[k - i];
      q.sc[k] = s;
    }
    return q;
  }

  TAG_DEV static void node_prims(const Params& P, const double* u, double* q, unsigned& bad) {
    const double rho = u[0];
    const double irho = 1.0 / rho;
    const double tg = pow(u[3], P.gamma);  // rho_theta^gamma
    q[0] = rho;
    q[1] = 0.5 * u[1] * irho;
    q[2] = 0.5 * u[2] * irho;
    q[3] = 0.5 * (P.K * tg);
    q[4] = 0.5 * u[4];
    q[5] = u[3];
    q[6] = rho / u[3];
    q[7] = tg;
    q[8] = tg / u[3];
    if (P.nc == 1) {
      const double rg = pow(rho, P.gamma);
      q[9] = rg;
      q[10] = rg * irho;
    } else {
      q[9] = q[10] = 0.0;
    }
    if (!(rho > 0.0)) bad |= TAG_S_NEG_DENSITY;
    if (!(u[3] > 0.0)) bad |= TAG_S_NEG_PRESSURE;
  }

  // Stolarsky mean of x, y with per-node powers (x^g, x^(g-1)), (y^g, y^(g-1))
  TAG_DEV static double stolarsky(const Params& P, double x, double y, double xg, double xg1,
                                  double yg, double yg1) {
    const double s = x + y, d = y - x;
    const double t = d / s, f2 = t * t;
    if (f2 < 1e-2) {
      double r = P.sc[7];
#pragma unroll
      for (int k = 6; k >= 0; --k) r = fma(r, f2, P.sc[k]);
      return 0.5 * s * r;
    }
    return P.stol_fac * (yg - xg) / (yg1 - xg1);
  }

  // One symmetric pair: the two-point flux F plus half the nonconservative
  // term G (antisymmetric in the pair): Fa = F + G/2, Fb = F - G/2.
  TAG_DEV static void volume_pair(const Params& P, const double* a, const double* b, double n1,
                                  double n2, double* Fa, double* Fb) {
    const double v1 = a[1] + b[1], v2 = a[2] + b[2];
    const double vn = n1 * v1 + n2 * v2;
    const double pa = a[3] + b[3];
    double rho_ln = 0.0, f1, f4;
    if (P.volume == 1) {
      double inv_sig;
      ln_mean_pair<false>(a[0], b[0], a[6], b[6], 0.0, 0.0, 0.0, 0.0, rho_ln, inv_sig);
      f1 = rho_ln * vn;
      f4 = f1 * inv_sig;
    } else {
      f4 = stolarsky(P, a[5], b[5], a[7], a[8], b[7], b[8]) * vn;
      if (P.volume == 0) {
        rho_ln = ln_mean_single(a[0], b[0]);
        f1 = rho_ln * vn;
      } else {
        f1 = f4 * ln_mean_single(a[6], b[6]);
      }
    }
    double ravg;
    if (P.nc == 0) ravg = (P.volume == 2) ? ln_mean_single(a[0], b[0]) : rho_ln;
    else if (P.nc == 1) ravg = stolarsky(P, a[0], b[0], a[9], a[10], b[9], b[10]);
    else ravg = 0.5 * (a[0] + b[0]);
    const double jump = 2.0 * (b[4] - a[4]);  // phi_b - phi_a (stored halved)
    const double g1 = 0.5 * n1 * ravg * jump, g2 = 0.5 * n2 * ravg * jump;
    const double F2 = f1 * v1 + pa * n1, F3 = f1 * v2 + pa * n2;
    Fa[0] = Fb[0] = f1;
    Fa[1] = F2 + g1;
    Fb[1] = F2 - g1;
    Fa[2] = F3 + g2;
    Fb[2] = F3 - g2;
    Fa[3] = Fb[3] = f4;
  }

  // flux(u, normal_direction), :84-98 (pressure() = K exp(gamma log rho_theta))
  TAG_DEV static void flux(const Params& P, const double* u, double n1, double n2, double* f) {
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double vn = v1 * n1 + v2 * n2;
    const double rvn = u[0] * vn;
    const double p = P.K * exp(P.gamma * log(u[3]));
    f[0] = rvn;
    f[1] = rvn * v1 + p * n1;
    f[2] = rvn * v2 + p * n2;
    f[3] = u[3] * vn;
  }

  // FluxLMARS (:171-193)
  TAG_DEV static void lmars(const Params& P, const double* ul, const double* ur, double n1,
                            double n2, double* F) {
    const double a = P.c_lmars;
    const double p_l = P.K * pow(ul[3], P.gamma), p_r = P.K * pow(ur[3], P.gamma);
    const double v_l = (ul[1] / ul[0]) * n1 + (ul[2] / ul[0]) * n2;
    const double v_r = (ur[1] / ur[0]) * n1 + (ur[2] / ur[0]) * n2;
    const double nrm = sqrt(n1 * n1 + n2 * n2);
    const double rho = 0.5 * (ul[0] + ur[0]);
    const double p_int = 0.5 * (p_l + p_r) - 0.5 * a * rho * (v_r - v_l) / nrm;
    const double v_int = 0.5 * (v_l + v_r) - 1.0 / (2.0 * a * rho) * (p_r - p_l) * nrm;
    const double* us = v_int > 0.0 ? ul : ur;
    F[0] = us[0] * v_int;
    F[1] = us[1] * v_int + p_int * n1;
    F[2] = us[2] * v_int + p_int * n2;
    F[3] = us[3] * v_int;
  }

  // flux_ec (:290-321) of full states
  TAG_DEV static void flux_ec(const Params& P, const double* ul, const double* ur, double n1,
                              double n2, double* F) {
    const double irl = 1.0 / ul[0], irr = 1.0 / ur[0];
    const double v1l = ul[1] * irl, v2l = ul[2] * irl, v1r = ur[1] * irr, v2r = ur[2] * irr;
    const double pl = P.K * pow(ul[3], P.gamma), pr = P.K * pow(ur[3], P.gamma);
    const double vn = 0.5 * ((v1l * n1 + v2l * n2) + (v1r * n1 + v2r * n2));
    const double pa = 0.5 * (pl + pr);
    double rho_ln, inv_sig;
    ln_mean_pair<false>(ul[0], ur[0], ul[0] / ul[3], ur[0] / ur[3], 0.0, 0.0, 0.0, 0.0, rho_ln,
                        inv_sig);
    const double f1 = rho_ln * vn;
    F[0] = f1;
    F[1] = f1 * 0.5 * (v1l + v1r) + pa * n1;
    F[2] = f1 * 0.5 * (v2l + v2r) + pa * n2;
    F[3] = f1 * inv_sig;
  }

  TAG_DEV static void surface_flux(const Params& P, const double* ul, const double* ur, double n1,
                                   double n2, double* F) {
    if (P.surface == 1)
      flux_ec(P, ul, ur, n1, n2, F);
    else
      lmars(P, ul, ur, n1, n2, F);
  }

  // the nonconservative gravity term of the surface flux, G(ul, ur) along the
  // primary's normal (zero for flux_zero)
  // MountainWaveSetup as source terms (src/equations/initial_condition_compressible_euler_2d.jl:174-200):
  // relaxation of v1 to u0, of v2 to 0 and of theta to theta_0 exp(N^2 z / g)
  // at the rate of rayleigh_damping_coefficient (:80-106), a sum of sin^2
  // ramps above z_damping_start and beyond +-x_damping_start
  TAG_DEV static void source(const Params& P, const double* u, const double* x, double,
                             double* s) {
    s[0] = s[1] = s[2] = s[3] = 0.0;
    if (!P.mountain) return;
    const double rate = P.mw[7], zs = P.mw[3], ze = P.mw[4], xs = P.mw[5], xe = P.mw[6];
    double dv = 0.0, dr = 0.0, dl = 0.0;
    if (x[1] > zs) {
      const double r = sinpi(0.5 * (x[1] - zs) / (ze - zs));
      dv = rate * (r * r);
    }
    if (!(x[0] < xs)) {
      const double r = sinpi(0.5 * (x[0] - xs) / (xe - xs));
      dr = rate * (r * r);
    }
    if (!(x[0] > -xs)) {
      const double r = sinpi(0.5 * (x[0] + xs) / (-xe + xs));
      dl = rate * (r * r);
    }
    const double damping = -(dv + dr + dl);
    const double v1 = u[1] / u[0], theta = u[3] / u[0];
    const double theta_b = P.mw[0] * exp(P.mw[2] * P.mw[2] / P.g * x[1]);
    s[1] = u[0] * (v1 - P.mw[1]) * damping;
    s[2] = u[2] * damping;
    s[3] = u[0] * (theta - theta_b) * damping;
  }

  TAG_DEV static void surface_noncons(const Params& P, const double* ul, const double* ur,
                                      double n1, double n2, double* G) {
    G[0] = G[1] = G[2] = G[3] = 0.0;
    if (P.snc < 0) return;
    double ra;
    if (P.snc == 0) {
      ra = ln_mean_single(ul[0], ur[0]);
    } else if (P.snc == 1) {
      const double xg = pow(ul[0], P.gamma), yg = pow(ur[0], P.gamma);
      ra = stolarsky(P, ul[0], ur[0], xg, xg / ul[0], yg, yg / ur[0]);
    } else {
      ra = 0.5 * (ul[0] + ur[0]);
    }
    const double jump = ur[4] - ul[4];
    G[1] = n1 * ra * jump;
    G[2] = n2 * ra * jump;
  }

  // Slip walls.  TAG_BC_SLIP_WALL_STRUCTURED (:62-83): reached with the normal
  // vector in the `orientation` slot, so rho_v2 is mirrored; states ordered by
  // the face parity; returned OUTWARD.  Otherwise (:45-60) the normal momentum
  // is mirrored about the outward normal (n1, n2).
  TAG_DEV static void boundary_flux(const Params& P, const double* ui, double n1, double n2,
                                    int face, int kind, double* F) {
    // (the wall's nonconservative term vanishes: both states carry the same phi)
    if (kind == TAG_BC_SLIP_WALL_STRUCTURED) {
      const double ub[5] = {ui[0], ui[1], -ui[2], ui[3], ui[4]};
      if (face & 1) {
        surface_flux(P, ui, ub, n1, n2, F);
      } else {
        surface_flux(P, ub, ui, n1, n2, F);
        F[0] = -F[0]; F[1] = -F[1]; F[2] = -F[2]; F[3] = -F[3];
      }
    } else {
      const double nn = sqrt(n1 * n1 + n2 * n2);
      const double nx = n1 / nn, ny = n2 / nn;
      const double un = nx * ui[1] + ny * ui[2];
      const double ub[5] = {ui[0], ui[1] - 2.0 * un * nx, ui[2] - 2.0 * un * ny, ui[3], ui[4]};
      surface_flux(P, ui, ub, n1, n2, F);
    }
  }

  // max_abs_speeds
  TAG_DEV static void max_speeds(const Params& P, const double* u, double& l1, double& l2) {
    const double rho = u[0];
    const double v1 = u[1] / rho, v2 = u[2] / rho;
    const double p = P.K * pow(u[3], P.gamma);
    const double c = sqrt(P.gamma * p / rho);
    l1 = fabs(v1) + c;
    l2 = fabs(v2) + c;
  }
};

}  // namespace tag
