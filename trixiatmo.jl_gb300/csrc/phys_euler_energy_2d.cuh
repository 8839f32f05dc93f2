// Device physics of CompressibleEulerEnergyEquationsWithGravity2D
// (reference: src/equations/compressible_euler_energy_with_gravity_2d.jl).
// State u = (rho, rho_v1, rho_v2, rho_e, phi); phi = g z is passive (zero flux,
// zero time derivative), so kernels evolve NA = 4 active variables.
#pragma once
#include "tag_common.cuh"

namespace tag {

struct PhysEnergy2D {
  static constexpr int NV = 5;  // stored variables per node
  static constexpr int NA = 4;  // variables with nonzero du
  // per-node quantities kept in shared memory (odd stride: no bank conflicts):
  // rho/2, v1/2, v2/2, p/2, phi/2, beta/2 = rho/(2p), log(rho/2), log(beta/2),
  // (pad); the halved rho and beta feed ln_mean_pair_halved
  static constexpr int NQ = 9;
  static constexpr int kRho = 0, kBeta = 5, kLogRho = 6, kLogBeta = 7;
  static constexpr bool kNodeLogs = false;  // 2D elements rarely leave the series range
  static constexpr bool kHasSources = false;
  static constexpr bool kSurfaceNoncons = false;  // surface flux only (flux_zero)

  struct Params {
    double gamma, gm1, inv_gm1, c_lmars, quarter_c, inv_c, half_inv_gm1;
  };

  static Params make_params(const double* p) {
    Params q;
    const double c_p = p[0], c_v = p[1];
    q.gamma = c_p / c_v;
    q.gm1 = q.gamma - 1.0;
    q.inv_gm1 = 1.0 / (q.gamma - 1.0);
    q.c_lmars = p[3];
    q.quarter_c = 0.25 * p[3];
    q.inv_c = 1.0 / p[3];
    q.half_inv_gm1 = 0.5 * q.inv_gm1;
    return q;
  }

  // cons2prim (:527-536), once per node:
  //   q = (rho/2, v1/2, v2/2, p/2, phi/2, beta/2 = rho/(2p)); flags bad states.
  // One reciprocal: rho p = (gamma - 1)(rho E - |rho v|^2 / 2) needs no
  // division, and r = 1/(rho^2 p) gives 1/(2 rho) = (rho p) r / 2 and
  // rho/(2p) = rho^3 r / 2.
  TAG_DEV static void node_prims(const Params& P, const double* u, double* q, unsigned& bad) {
    const double rho = u[0];
    const double m2 = fma(u[2], u[2], u[1] * u[1]);
    const double rp = P.gm1 * fma(rho, u[3], -0.5 * m2);
    const double r = 1.0 / (rho * rp);
    const double hirho = 0.5 * (rp * r);
    q[0] = 0.5 * rho;
    q[1] = u[1] * hirho;
    q[2] = u[2] * hirho;
    q[3] = rp * hirho;
    q[4] = 0.5 * u[4];
    q[5] = q[0] * rho * (rho * r);
    q[8] = 0.0;
    if (not_positive(rho)) bad |= TAG_S_NEG_DENSITY;
    if (not_positive(q[3])) bad |= TAG_S_NEG_PRESSURE;
  }

  // One symmetric pair of the volume integral: flux_ranocha (:366-395) plus half
  // the nonconservative flux_nonconservative_waruszewski_etal (:186-205), both
  // with the averaged contravariant vector (n1, n2).  Returns Fa = F + G/2 (to
  // node a, weighted by Dsplit[a,b]) and Fb = F - G/2 (to node b, Dsplit[b,a]);
  // G(b,a) = -G(a,b).  Written on the half-valued node quantities of
  // node_prims; p_ll p_rr inv_ln_mean(rho_ll p_rr, rho_rr p_ll) is evaluated as
  // the equal inv_ln_mean(rho_ll/p_ll, rho_rr/p_rr).  With h the gravity term
  // rho_mean (phi_b - phi_a) / 2, the momentum fluxes of the two sides are
  // f1 v + n (p_avg +- h) and the energy fluxes 2 E +- h vn, E being half of
  // flux_ranocha's energy flux.
  TAG_DEV static void volume_pair(const Params& P, const double* qa, const double* qb,
                                  double n1, double n2, double* Fa, double* Fb) {
    double rho_mean, inv_rho_p_mean;
    ln_mean_pair_halved<true, false, true>(qa[0], qb[0], qa[5], qb[5], 0.0, 0.0, 0.0, 0.0,
                                           rho_mean, inv_rho_p_mean);
    const double v1 = qa[1] + qb[1];
    const double v2 = qa[2] + qb[2];
    const double vn = fma(v2, n2, v1 * n1);  // 0.5 (vn_a + vn_b)
    const double f1 = rho_mean * vn;
    const double h = rho_mean * (qb[4] - qa[4]);
    const double p_avg = qa[3] + qb[3];
    const double pp = p_avg + h, pm = p_avg - h;
    const double t1 = f1 * v1, t2 = f1 * v2;
    Fa[0] = f1;
    Fb[0] = f1;
    Fa[1] = fma(n1, pp, t1);
    Fb[1] = fma(n1, pm, t1);
    Fa[2] = fma(n2, pp, t2);
    Fb[2] = fma(n2, pm, t2);
    // E = f1 (v_a.v_b / 4 + inv_beta_mean / (2 (gamma - 1))) + (p_a vn_b + p_b vn_a) / 4
    const double vv = fma(qa[2], qb[2], qa[1] * qb[1]);
    const double x = fma(inv_rho_p_mean, P.half_inv_gm1, vv);
    const double c1 = fma(qa[3], qb[1], qb[3] * qa[1]);
    const double c2 = fma(qa[3], qb[2], qb[3] * qa[2]);
    const double e = fma(f1, x, fma(n2, c2, n1 * c1));
    const double hv = h * vn;
    Fa[3] = fma(2.0, e, hv);
    Fb[3] = fma(2.0, e, -hv);
  }

  // FluxLMARS (:397-430) between states ul, ur for the (unnormalised) normal n:
  //   p = (p_ll + p_rr)/2 - c rho (v_rr - v_ll) / (2 |n|),
  //   v = (v_ll + v_rr)/2 - (p_rr - p_ll) |n| / (2 c rho),  rho = (rho_ll + rho_rr)/2,
  // with one reciprocal for 1/rho_ll, 1/rho_rr and 1/(rho_ll + rho_rr), one
  // reciprocal square root for |n| and 1/|n|, and p = (gamma - 1)(rho e -
  // |rho v|^2 / (2 rho)) (the FP64 pipe bounds the interface kernel too).
  TAG_DEV static void lmars(const Params& P, const double* ul, const double* ur, double n1,
                            double n2, double* F) {
    const double rho_ll = ul[0], rho_rr = ur[0];
    const double srho = rho_ll + rho_rr, prho = rho_ll * rho_rr;
    const double r = 1.0 / (prho * srho);
    const double irl = (rho_rr * srho) * r, irr = (rho_ll * srho) * r, isum = prho * r;
    const double p_ll = P.gm1 * fma(-0.5 * fma(ul[2], ul[2], ul[1] * ul[1]), irl, ul[3]);
    const double p_rr = P.gm1 * fma(-0.5 * fma(ur[2], ur[2], ur[1] * ur[1]), irr, ur[3]);
    const double v_ll = fma(ul[2], n2, ul[1] * n1) * irl;
    const double v_rr = fma(ur[2], n2, ur[1] * n1) * irr;
    const double nsq = fma(n2, n2, n1 * n1);
    const double inorm = rsqrt(nsq), norm_ = nsq * inorm;
    const double p = 0.5 * (p_ll + p_rr) - P.quarter_c * srho * (v_rr - v_ll) * inorm;
    const double v = 0.5 * (v_ll + v_rr) - P.inv_c * (p_rr - p_ll) * norm_ * isum;
    if (v >= 0.0) {
      F[0] = ul[0] * v; F[1] = ul[1] * v; F[2] = ul[2] * v; F[3] = ul[3] * v + p_ll * v;
    } else {
      F[0] = ur[0] * v; F[1] = ur[1] * v; F[2] = ur[2] * v; F[3] = ur[3] * v + p_rr * v;
    }
    F[1] += p * n1;
    F[2] += p * n2;
  }

  // Interface: surface flux (FluxLMARS, flux_zero) with the primary's outward
  // normal; F is stored for the primary and -F for the secondary.
  TAG_DEV static void surface_flux(const Params& P, const double* ul, const double* ur, double n1,
                                   double n2, double* F) {
    lmars(P, ul, ur, n1, n2, F);
  }

  // Slip wall.  kind TAG_BC_SLIP_WALL_STRUCTURED: normal (n1, n2) is the
  // sign-corrected contravariant vector in the +xi/+eta sense; the reference
  // method :102-129 mirrors v2 and orders the states by the parity of the face;
  // the returned flux is OUTWARD (negated on xi-/eta- faces).
  // kind TAG_BC_SLIP_WALL_NORMAL: (n1, n2) is the outward normal; :77-100.
  TAG_DEV static void boundary_flux(const Params& P, const double* ui, double n1, double n2,
                                    int face, int kind, double* F) {
    if (kind == TAG_BC_SLIP_WALL_STRUCTURED) {
      const double ub[5] = {ui[0], ui[1], -ui[2], ui[3], ui[4]};
      if (face & 1) {
        lmars(P, ui, ub, n1, n2, F);
      } else {
        lmars(P, ub, ui, n1, n2, F);
        F[0] = -F[0]; F[1] = -F[1]; F[2] = -F[2]; F[3] = -F[3];
      }
    } else {
      const double inn = rsqrt(fma(n2, n2, n1 * n1));
      const double nx = n1 * inn, ny = n2 * inn;
      const double un = nx * ui[1] + ny * ui[2];
      const double ub[5] = {ui[0], ui[1] - 2.0 * un * nx, ui[2] - 2.0 * un * ny, ui[3], ui[4]};
      lmars(P, ui, ub, n1, n2, F);
    }
  }

  // max_abs_speeds (:518-524)
  TAG_DEV static void max_speeds(const Params& P, const double* u, double& l1, double& l2) {
    const double irho = 1.0 / u[0];
    const double v1 = u[1] * irho, v2 = u[2] * irho;
    const double p = P.gm1 * (u[3] - 0.5 * (u[1] * v1 + u[2] * v2));
    const double c = sqrt(P.gamma * p * irho);
    l1 = fabs(v1) + c;
    l2 = fabs(v2) + c;
  }
};

}  // namespace tag
