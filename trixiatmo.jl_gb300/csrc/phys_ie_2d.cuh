// Device physics of CompressibleEulerInternalEnergyEquationsWithGravity2D
// (reference: src/equations/compressible_euler_internal_energy_with_gravity_2d.jl).
// State u = (rho, rho_v1, rho_v2, rho_e_internal, phi), p = (gamma - 1) rho_e_internal;
// phi = g z is passive, so kernels evolve NA = 4 variables.  Volume flux
// (flux_conservative_etec :110-136, flux_nonconservative_etec :144-165);
// surface flux (flux_conservative_es :174-216, flux_nonconservative_es
// :224-246), whose nonconservative part differs on the two sides of an
// interface (kSurfaceNoncons); slip walls :77-99.
#pragma once
#include "tag_common.cuh"

namespace tag {

struct PhysIE2D {
  static constexpr int NV = 5;
  static constexpr int NA = 4;
  // rho, v1/2, v2/2, p/2, phi/2, beta = rho/p, (unused logs), pad (odd stride)
  static constexpr int NQ = 9;
  static constexpr int kRho = 0, kBeta = 5, kLogRho = 6, kLogBeta = 7;
  static constexpr bool kNodeLogs = false;
  static constexpr bool kHasSources = false;
  static constexpr bool kSurfaceNoncons = true;

  struct Params {
    double gamma, gm1, inv_gm1;
  };

  // params = (c_p, c_v, g)
  static Params make_params(const double* p) {
    Params q;
    q.gamma = p[0] / p[1];
    q.gm1 = q.gamma - 1.0;
    q.inv_gm1 = 1.0 / (q.gamma - 1.0);
    return q;
  }

  TAG_DEV static void node_prims(const Params& P, const double* u, double* q, unsigned& bad) {
    const double rho = u[0];
    const double irho = 1.0 / rho;
    const double p = P.gm1 * u[3];
    q[0] = rho;
    q[1] = 0.5 * u[1] * irho;
    q[2] = 0.5 * u[2] * irho;
    q[3] = 0.5 * p;
    q[4] = 0.5 * u[4];
    q[5] = rho / p;
    q[6] = q[7] = q[8] = 0.0;
    if (!(rho > 0.0)) bad |= TAG_S_NEG_DENSITY;
    if (!(p > 0.0)) bad |= TAG_S_NEG_PRESSURE;
  }

  // flux_conservative_etec + half of flux_nonconservative_etec (antisymmetric)
  // on the halved node quantities; p_ll p_rr inv_ln_mean(rho_ll p_rr, rho_rr p_ll)
  // is evaluated as the equal inv_ln_mean(rho_ll/p_ll, rho_rr/p_rr).
  TAG_DEV static void volume_pair(const Params& P, const double* qa, const double* qb, double n1,
                                  double n2, double* Fa, double* Fb) {
    double rho_mean, inv_rho_p_mean;
    ln_mean_pair<false>(qa[0], qb[0], qa[5], qb[5], 0.0, 0.0, 0.0, 0.0, rho_mean, inv_rho_p_mean);
    const double v1 = qa[1] + qb[1], v2 = qa[2] + qb[2];  // averages
    const double vn = n1 * v1 + n2 * v2;                    // 0.5 (vn_a + vn_b)
    const double p_avg = qa[3] + qb[3];
    const double f1 = rho_mean * vn;
    const double f2 = f1 * v1 + p_avg * n1;
    const double f3 = f1 * v2 + p_avg * n2;
    const double f4 = f1 * inv_rho_p_mean * P.inv_gm1 + p_avg * vn;
    const double gr = rho_mean * (qb[4] - qa[4]);   // rho_mean (phi_b - phi_a) / 2
    const double gp = -vn * (qb[3] - qa[3]);         // -vn_avg (p_b - p_a) / 2
    Fa[0] = Fb[0] = f1;
    Fa[1] = f2 + gr * n1;
    Fb[1] = f2 - gr * n1;
    Fa[2] = f3 + gr * n2;
    Fb[2] = f3 - gr * n2;
    Fa[3] = f4 + gp;
    Fb[3] = f4 - gp;
  }

  // Trixi's flux (conservative part) for the weak form and consistency
  TAG_DEV static void flux(const Params& P, const double* u, double n1, double n2, double* f) {
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double p = P.gm1 * u[3];
    const double vn = v1 * n1 + v2 * n2;
    f[0] = u[0] * vn;
    f[1] = u[1] * vn + p * n1;
    f[2] = u[2] * vn + p * n2;
    f[3] = (u[3] + p) * vn;
  }

  // interface speed of sound and normal velocity of the es pair
  TAG_DEV static double v_interface(const Params& P, const double* ul, const double* ur,
                                    double n1, double n2, double& vnl, double& vnr, double& pl,
                                    double& pr, double& a, double& nrm) {
    const double rl = ul[0], rr = ur[0];
    pl = P.gm1 * ul[3];
    pr = P.gm1 * ur[3];
    vnl = (ul[1] / rl) * n1 + (ul[2] / rl) * n2;
    vnr = (ur[1] / rr) * n1 + (ur[2] / rr) * n2;
    const double cl = sqrt(P.gamma * pl / rl), cr = sqrt(P.gamma * pr / rr);
    a = 0.5 * (cl + cr);
    nrm = sqrt(n1 * n1 + n2 * n2);
    const double rho_avg = 0.5 * (rl + rr);
    return 0.5 * (vnl + vnr) - 1.0 / (2.0 * a * rho_avg) * (pr - pl) * nrm;
  }

  // flux_conservative_es
  TAG_DEV static void surface_flux(const Params& P, const double* ul, const double* ur, double n1,
                                   double n2, double* F) {
    double vnl, vnr, pl, pr, a, nrm;
    const double v_int = v_interface(P, ul, ur, n1, n2, vnl, vnr, pl, pr, a, nrm);
    const double rl = ul[0], rr = ur[0];
    const double rho_mean = ln_mean_single(rl, rr);
    const double rho_avg = 0.5 * (rl + rr);
    const double p_int = 0.5 * (pl + pr) - 0.5 * a * rho_avg * (vnr - vnl) / nrm;
    const double p_avg = 0.5 * (pl + pr);
    double rho_up, f2, f3;
    if (v_int >= 0.0) {
      rho_up = rho_mean - 0.5 * (rr - rl);
      f2 = ul[1] * v_int;
      f3 = ul[2] * v_int;
    } else {
      rho_up = rho_mean + 0.5 * (rr - rl);
      f2 = ur[1] * v_int;
      f3 = ur[2] * v_int;
    }
    const double inv_rho_p_mean = inv_ln_mean_single(rl / pl, rr / pr);
    const double f1 = rho_up * v_int;
    F[0] = f1;
    F[1] = f2 + p_int * n1;
    F[2] = f3 + p_int * n2;
    F[3] = f1 * inv_rho_p_mean * P.inv_gm1 + p_avg * v_int;
  }

  // flux_nonconservative_es of (ul, ur) along the primary's normal
  TAG_DEV static void surface_noncons(const Params& P, const double* ul, const double* ur,
                                      double n1, double n2, double* G) {
    double vnl, vnr, pl, pr, a, nrm;
    const double v_int = v_interface(P, ul, ur, n1, n2, vnl, vnr, pl, pr, a, nrm);
    G[0] = G[1] = G[2] = 0.0;
    G[3] = -v_int * (pr - pl);
  }

  // boundary_condition_slip_wall (outward normal): flux + 1/2 nonconservative
  // flux of the inner and the mirrored state
  TAG_DEV static void boundary_flux(const Params& P, const double* ui, double n1, double n2, int,
                                    int, double* F) {
    const double nn = sqrt(n1 * n1 + n2 * n2);
    const double nx = n1 / nn, ny = n2 / nn;
    const double un = nx * ui[1] + ny * ui[2];
    const double ub[5] = {ui[0], ui[1] - 2.0 * un * nx, ui[2] - 2.0 * un * ny, ui[3], ui[4]};
    double G[4];
    surface_flux(P, ui, ub, n1, n2, F);
    surface_noncons(P, ui, ub, n1, n2, G);
#pragma unroll
    for (int v = 0; v < 4; ++v) F[v] += 0.5 * G[v];
  }

  TAG_DEV static void max_speeds(const Params& P, const double* u, double& l1, double& l2) {
    const double rho = u[0];
    const double v1 = u[1] / rho, v2 = u[2] / rho;
    const double p = P.gm1 * u[3];
    const double c = sqrt(P.gamma * p / rho);
    l1 = fabs(v1) + c;
    l2 = fabs(v2) + c;
  }
};

}  // namespace tag
