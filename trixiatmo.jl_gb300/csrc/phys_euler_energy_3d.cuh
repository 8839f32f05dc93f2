// Device physics of CompressibleEulerEnergyEquationsWithGravity3D
// (reference: src/equations/compressible_euler_energy_with_gravity_3d.jl) and
// the Coriolis source (src/equations/initial_condition_compressible_euler_3d.jl:245-269).
// State u = (rho, rho_v1, rho_v2, rho_v3, rho_e, phi); phi is passive, so
// kernels evolve NA = 5 active variables.
#pragma once
#include "tag_common.cuh"

namespace tag {

struct PhysEnergy3D {
  static constexpr int NV = 6;
  static constexpr int NA = 5;
  // rho/2, v1/2, v2/2, v3/2, p/2, phi/2, beta/2 = rho/(2p), log(rho/2),
  // log(beta/2) (odd stride); the halved rho and beta feed ln_mean_pair_halved
  static constexpr int NQ = 9;
  static constexpr int kRho = 0, kBeta = 6, kLogRho = 7, kLogBeta = 8;
  // the polynomial forms up to f2 = 0.09 keep every pair of a tall shell element (km-sized
  // vertical node spacing) out of the logarithms; only elements whose values
  // spread further take logarithms, once per node
  static constexpr bool kNodeLogs = true;
  static constexpr double kLogRange = kLongLogRange;
  static constexpr bool kHasSources = true;  // Coriolis, added per (node, variable)

  struct Params {
    double gamma, gm1, inv_gm1, c_lmars, quarter_c, inv_c, omega, half_inv_gm1;
  };

  static Params make_params(const double* p) {
    Params q;
    q.gamma = p[0] / p[1];
    q.gm1 = q.gamma - 1.0;
    q.inv_gm1 = 1.0 / (q.gamma - 1.0);
    q.half_inv_gm1 = 0.5 * q.inv_gm1;
    q.c_lmars = p[3];
    q.quarter_c = 0.25 * p[3];
    q.inv_c = 1.0 / p[3];
    q.omega = p[4];
    return q;
  }

  // cons2prim (:568-578) once per node with one reciprocal: rho p =
  // (gamma - 1)(rho E - |rho v|^2 / 2) needs no division, and r = 1/(rho^2 p)
  // gives 1/(2 rho) = (rho p) r / 2 and rho/(2p) = rho^3 r / 2.
  TAG_DEV static void node_prims(const Params& P, const double* u, double* q, unsigned& bad) {
    const double rho = u[0];
    const double m2 = fma(u[3], u[3], fma(u[2], u[2], u[1] * u[1]));
    const double rp = P.gm1 * fma(rho, u[4], -0.5 * m2);
    const double r = 1.0 / (rho * rp);
    const double hirho = 0.5 * (rp * r);
    q[0] = 0.5 * rho;
    q[1] = u[1] * hirho;
    q[2] = u[2] * hirho;
    q[3] = u[3] * hirho;
    q[4] = rp * hirho;
    q[5] = 0.5 * u[5];
    q[6] = q[0] * rho * (rho * r);
    if (not_positive(rho)) bad |= TAG_S_NEG_DENSITY;
    if (not_positive(q[4])) bad |= TAG_S_NEG_PRESSURE;
  }

  // flux_ranocha (3D, :382-415) + half of flux_nonconservative_waruszewski_etal
  // (3D, :135-159) for one symmetric pair; see PhysEnergy2D::volume_pair.
  // nrm is the average of the two nodes' contravariant vectors.  With h the
  // gravity term rho_mean (phi_b - phi_a) / 2, the momentum fluxes of the two
  // sides are f1 v + n (p_avg +- h), and the energy fluxes 2 E +- h vn with
  // E = f1 (v_a.v_b / 4 + inv_beta_mean / (2 (gamma - 1))) + (p_a vn_b + p_b vn_a) / 4
  // (node values halved, so E is half of flux_ranocha's energy flux).
  TAG_DEV static void volume_pair(const Params& P, const double* qa, const double* qb,
                                  const double* nrm, double* Fa, double* Fb) {
    double rho_mean, inv_rho_p_mean;
    ln_mean_pair_halved(qa[0], qb[0], qa[6], qb[6], qa[7], qb[7], qa[8], qb[8], rho_mean,
                        inv_rho_p_mean);
    const double n1 = nrm[0], n2 = nrm[1], n3 = nrm[2];
    const double v1 = qa[1] + qb[1], v2 = qa[2] + qb[2], v3 = qa[3] + qb[3];
    // halved normal velocities of both nodes: vn = 0.5 (vn_a + vn_b)
    const double vna = fma(qa[3], n3, fma(qa[2], n2, qa[1] * n1));
    const double vnb = fma(qb[3], n3, fma(qb[2], n2, qb[1] * n1));
    const double vn = vna + vnb;
    const double f1 = rho_mean * vn;
    const double h = rho_mean * (qb[5] - qa[5]);
    const double p_avg = qa[4] + qb[4];
    const double pp = p_avg + h, pm = p_avg - h;
    const double t1 = f1 * v1, t2 = f1 * v2, t3 = f1 * v3;
    Fa[0] = f1;
    Fb[0] = f1;
    Fa[1] = fma(n1, pp, t1);
    Fb[1] = fma(n1, pm, t1);
    Fa[2] = fma(n2, pp, t2);
    Fb[2] = fma(n2, pm, t2);
    Fa[3] = fma(n3, pp, t3);
    Fb[3] = fma(n3, pm, t3);
    const double vv = fma(qa[3], qb[3], fma(qa[2], qb[2], qa[1] * qb[1]));
    const double x = fma(inv_rho_p_mean, P.half_inv_gm1, vv);
    const double e = fma(f1, x, fma(qa[4], vnb, qb[4] * vna));
    const double hv = h * vn;
    Fa[4] = fma(2.0, e, hv);
    Fb[4] = fma(2.0, e, -hv);
  }

  // FluxLMARS (3D, :430-466) for the (unnormalised) normal n:
  //   p = (p_ll + p_rr)/2 - c rho (v_rr - v_ll) / (2 |n|),
  //   v = (v_ll + v_rr)/2 - (p_rr - p_ll) |n| / (2 c rho),  rho = (rho_ll + rho_rr)/2,
  // with one reciprocal for 1/rho_ll, 1/rho_rr and 1/(rho_ll + rho_rr), one
  // reciprocal square root for |n| and 1/|n|, and p = (gamma - 1)(rho e -
  // |rho v|^2 / (2 rho)).
  TAG_DEV static void lmars(const Params& P, const double* ul, const double* ur, const double* n,
                            double* F) {
    const double rho_ll = ul[0], rho_rr = ur[0];
    const double srho = rho_ll + rho_rr, prho = rho_ll * rho_rr;
    const double r = 1.0 / (prho * srho);
    const double irl = (rho_rr * srho) * r, irr = (rho_ll * srho) * r, isum = prho * r;
    const double ml = fma(ul[3], ul[3], fma(ul[2], ul[2], ul[1] * ul[1]));
    const double mr = fma(ur[3], ur[3], fma(ur[2], ur[2], ur[1] * ur[1]));
    const double pl = P.gm1 * fma(-0.5 * ml, irl, ul[4]);
    const double pr = P.gm1 * fma(-0.5 * mr, irr, ur[4]);
    const double vl = fma(ul[3], n[2], fma(ul[2], n[1], ul[1] * n[0])) * irl;
    const double vr = fma(ur[3], n[2], fma(ur[2], n[1], ur[1] * n[0])) * irr;
    const double nsq = fma(n[2], n[2], fma(n[1], n[1], n[0] * n[0]));
    const double inorm = rsqrt(nsq), norm_ = nsq * inorm;
    const double p = 0.5 * (pl + pr) - P.quarter_c * srho * (vr - vl) * inorm;
    const double v = 0.5 * (vl + vr) - P.inv_c * (pr - pl) * norm_ * isum;
    const double* us = v >= 0.0 ? ul : ur;
    const double ps = v >= 0.0 ? pl : pr;
    F[0] = v * us[0];
    F[1] = v * us[1] + p * n[0];
    F[2] = v * us[2] + p * n[1];
    F[3] = v * us[3] + p * n[2];
    F[4] = v * us[4] + ps * v;
  }

  TAG_DEV static void surface_flux(const Params& P, const double* ul, const double* ur,
                                   const double* n, double* F) {
    lmars(P, ul, ur, n, F);
  }

  // boundary_condition_slip_wall (3D), :93-116, with the outward normal n.
  TAG_DEV static void boundary_flux(const Params& P, const double* ui, const double* n, double* F) {
    const double inn = rsqrt(fma(n[2], n[2], fma(n[1], n[1], n[0] * n[0])));
    const double e0 = n[0] * inn, e1 = n[1] * inn, e2 = n[2] * inn;
    const double un = e0 * ui[1] + e1 * ui[2] + e2 * ui[3];
    const double ub[6] = {ui[0], ui[1] - 2.0 * un * e0, ui[2] - 2.0 * un * e1,
                          ui[3] - 2.0 * un * e2, ui[4], ui[5]};
    lmars(P, ui, ub, n, F);
  }

  // coriolis_source: du2 += 2 Omega rho_v2, du3 -= 2 Omega rho_v1
  TAG_DEV static double source(const Params& P, const double* u, int v) {
    if (v == 1) return 2.0 * P.omega * u[2];
    if (v == 2) return -2.0 * P.omega * u[1];
    return 0.0;
  }

  TAG_DEV static void max_speeds(const Params& P, const double* u, double* l) {
    const double irho = 1.0 / u[0];
    const double v1 = u[1] * irho, v2 = u[2] * irho, v3 = u[3] * irho;
    const double p = P.gm1 * (u[4] - 0.5 * (u[1] * v1 + u[2] * v2 + u[3] * v3));
    const double c = sqrt(P.gamma * p * irho);
    l[0] = fabs(v1) + c;
    l[1] = fabs(v2) + c;
    l[2] = fabs(v3) + c;
  }
};

}  // namespace tag
