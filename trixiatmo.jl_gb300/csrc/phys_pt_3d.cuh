// Device physics of CompressibleEulerPotentialTemperatureEquationsWithGravity3D
// (reference: src/equations/compressible_euler_potential_temperature_gravity_3d.jl)
// with the Coriolis source (src/equations/initial_condition_compressible_euler_3d.jl:245-269).
// State u = (rho, rho_v1, rho_v2, rho_v3, rho_theta, phi), p = K rho_theta^gamma;
// phi = g z is passive, so kernels evolve NA = 5 variables.  Volume fluxes
// flux_tec / flux_ec / flux_etec (:428-533) with the nonconservative gravity
// term of Waruszewski et al. (or Artiano et al., Souza et al.; :146-211);
// surface flux (FluxLMARS(c), flux_zero) (:213-256); slip walls (:83-107).
// The Stolarsky mean as in phys_pt_2d.cuh (series below f^2 = 1e-2, per-node
// powers above).
#pragma once
#include "phys_pt_2d.cuh"

namespace tag {

struct PhysPT3D {
  static constexpr int NV = 6;
  static constexpr int NA = 5;
  // rho, v1/2, v2/2, v3/2, p/2, phi/2, rho_theta, sigma = rho/rho_theta,
  // rho_theta^gamma, rho_theta^(gamma-1), rho^gamma, rho^(gamma-1), pad (odd stride)
  static constexpr int NQ = 13;
  static constexpr int kRho = 0, kBeta = 0, kLogRho = 0, kLogBeta = 0;
  static constexpr bool kNodeLogs = false;
  static constexpr double kLogRange = kLogMeanRange;
  static constexpr bool kHasSources = true;  // Coriolis, per (node, variable)

  struct Params {
    PhysPT2D::Params pt;  // gamma, K, LMARS c, Stolarsky series, volume / gravity-term kinds
    double omega;
  };

  // params = (c_p, c_v, g, LMARS c, nonconservative kind, volume kind, Omega)
  static Params make_params(const double* p) {
    double p2[8];
    for (int k = 0; k < 8; ++k) p2[k] = p[k];
    p2[6] = 0.0;  // surface (FluxLMARS(c), flux_zero)
    p2[7] = 0.0;
    Params q;
    q.pt = PhysPT2D::make_params(p2);
    q.omega = p[6];
    return q;
  }

  TAG_DEV static void node_prims(const Params& Q, const double* u, double* q, unsigned& bad) {
    const PhysPT2D::Params& P = Q.pt;
    const double rho = u[0];
    const double irho = 1.0 / rho;
    const double tg = pow(u[4], P.gamma);  // rho_theta^gamma
    q[0] = rho;
    q[1] = 0.5 * u[1] * irho;
    q[2] = 0.5 * u[2] * irho;
    q[3] = 0.5 * u[3] * irho;
    q[4] = 0.5 * (P.K * tg);
    q[5] = 0.5 * u[5];
    q[6] = u[4];
    q[7] = rho / u[4];
    q[8] = tg;
    q[9] = tg / u[4];
    if (P.nc == 1) {
      const double rg = pow(rho, P.gamma);
      q[10] = rg;
      q[11] = rg * irho;
    } else {
      q[10] = q[11] = 0.0;
    }
    q[12] = P.volume == 3 ? 0.5 * u[4] * irho : 0.0;  // theta / 2 (flux_kennedy_gruber)
    if (!(rho > 0.0)) bad |= TAG_S_NEG_DENSITY;
    if (!(u[4] > 0.0)) bad |= TAG_S_NEG_PRESSURE;
  }

  // One symmetric pair: the two-point flux F plus half the nonconservative
  // term G (antisymmetric in the pair): Fa = F + G/2, Fb = F - G/2.
  TAG_DEV static void volume_pair(const Params& Q, const double* a, const double* b,
                                  const double* nrm, double* Fa, double* Fb) {
    const PhysPT2D::Params& P = Q.pt;
    const double n1 = nrm[0], n2 = nrm[1], n3 = nrm[2];
    const double v1 = a[1] + b[1], v2 = a[2] + b[2], v3 = a[3] + b[3];
    const double vn = n1 * v1 + n2 * v2 + n3 * v3;
    const double pa = a[4] + b[4];
    double rho_ln = 0.0, f1, f5;
    if (P.volume == 1) {
      double inv_sig;
      ln_mean_pair<false>(a[0], b[0], a[7], b[7], 0.0, 0.0, 0.0, 0.0, rho_ln, inv_sig);
      f1 = rho_ln * vn;
      f5 = f1 * inv_sig;
    } else if (P.volume == 3) {
      // flux_kennedy_gruber (:333-359): arithmetic means of rho, v, p and theta
      f1 = 0.5 * (a[0] + b[0]) * vn;
      f5 = f1 * (a[12] + b[12]);
    } else {
      f5 = PhysPT2D::stolarsky(P, a[6], b[6], a[8], a[9], b[8], b[9]) * vn;
      if (P.volume == 0) {
        rho_ln = ln_mean_single(a[0], b[0]);
        f1 = rho_ln * vn;
      } else {
        f1 = f5 * ln_mean_single(a[7], b[7]);
      }
    }
    double ravg;
    if (P.nc == 0) ravg = (P.volume >= 2) ? ln_mean_single(a[0], b[0]) : rho_ln;
    else if (P.nc == 1) ravg = PhysPT2D::stolarsky(P, a[0], b[0], a[10], a[11], b[10], b[11]);
    else ravg = 0.5 * (a[0] + b[0]);
    const double h = ravg * (b[5] - a[5]);  // (phi_b - phi_a) / 2 rho_avg (stored halved)
    const double F2 = f1 * v1 + pa * n1, F3 = f1 * v2 + pa * n2, F4 = f1 * v3 + pa * n3;
    Fa[0] = Fb[0] = f1;
    Fa[1] = F2 + n1 * h;
    Fb[1] = F2 - n1 * h;
    Fa[2] = F3 + n2 * h;
    Fb[2] = F3 - n2 * h;
    Fa[3] = F4 + n3 * h;
    Fb[3] = F4 - n3 * h;
    Fa[4] = Fb[4] = f5;
  }

  // FluxLMARS (:213-256)
  TAG_DEV static void lmars(const Params& Q, const double* ul, const double* ur, const double* n,
                            double* F) {
    const PhysPT2D::Params& P = Q.pt;
    const double a = P.c_lmars;
    const double p_l = P.K * pow(ul[4], P.gamma), p_r = P.K * pow(ur[4], P.gamma);
    const double v_l = (ul[1] / ul[0]) * n[0] + (ul[2] / ul[0]) * n[1] + (ul[3] / ul[0]) * n[2];
    const double v_r = (ur[1] / ur[0]) * n[0] + (ur[2] / ur[0]) * n[1] + (ur[3] / ur[0]) * n[2];
    const double nrm = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double rho = 0.5 * (ul[0] + ur[0]);
    const double p_int = 0.5 * (p_l + p_r) - 0.5 * a * rho * (v_r - v_l) / nrm;
    const double v_int = 0.5 * (v_l + v_r) - 1.0 / (2.0 * a * rho) * (p_r - p_l) * nrm;
    const double* us = v_int > 0.0 ? ul : ur;
    F[0] = us[0] * v_int;
    F[1] = us[1] * v_int + p_int * n[0];
    F[2] = us[2] * v_int + p_int * n[1];
    F[3] = us[3] * v_int + p_int * n[2];
    F[4] = us[4] * v_int;
  }

  TAG_DEV static void surface_flux(const Params& Q, const double* ul, const double* ur,
                                   const double* n, double* F) {
    lmars(Q, ul, ur, n, F);
  }

  // boundary_condition_slip_wall (:83-107) with the outward normal n
  TAG_DEV static void boundary_flux(const Params& Q, const double* ui, const double* n, double* F) {
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double e0 = n[0] / nn, e1 = n[1] / nn, e2 = n[2] / nn;
    const double un = e0 * ui[1] + e1 * ui[2] + e2 * ui[3];
    const double ub[6] = {ui[0], ui[1] - 2.0 * un * e0, ui[2] - 2.0 * un * e1,
                          ui[3] - 2.0 * un * e2, ui[4], ui[5]};
    lmars(Q, ui, ub, n, F);
  }

  // coriolis_source: du2 += 2 Omega rho_v2, du3 -= 2 Omega rho_v1
  TAG_DEV static double source(const Params& Q, const double* u, int v) {
    if (v == 1) return 2.0 * Q.omega * u[2];
    if (v == 2) return -2.0 * Q.omega * u[1];
    return 0.0;
  }

  // max_abs_speeds (:695-700)
  TAG_DEV static void max_speeds(const Params& Q, const double* u, double* l) {
    const PhysPT2D::Params& P = Q.pt;
    const double irho = 1.0 / u[0];
    const double v1 = u[1] * irho, v2 = u[2] * irho, v3 = u[3] * irho;
    const double p = P.K * pow(u[4], P.gamma);
    const double c = sqrt(P.gamma * p / u[0]);
    l[0] = fabs(v1) + c;
    l[1] = fabs(v2) + c;
    l[2] = fabs(v3) + c;
  }
};

}  // namespace tag
