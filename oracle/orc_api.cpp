// ORACLE — test infrastructure only. This shared library is the CPU checker
// (and the timed CPU baseline) for the CUDA path; the product library never
// links it. Its C ABI is called from tests/ and from bench.py's cpu_baseline.
//
// It restates the reference's CPU `rhs!` for
// CompressibleEulerEnergyEquationsWithGravity2D on a StructuredMesh, with
// volume_flux = (flux_ranocha, flux_nonconservative_waruszewski_etal) and
// surface_flux = (FluxLMARS(c), flux_zero) as in
// examples/euler/dry_air/buoyancy/elixir_energy_inertia_gravity_waves.jl:27-44.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "orc_basis.hpp"
#include "orc_dg2d.hpp"
#include "orc_dg3d.hpp"
#include "orc_euler_energy_2d.hpp"
#include "orc_euler_energy_3d.hpp"
#include "orc_moist_2d.hpp"
#include "orc_pt_2d.hpp"
#include "orc_pt_3d.hpp"
#include "orc_ie_2d.hpp"
#include "orc_cov_swe.hpp"
#include "orc_rainy_2d.hpp"
#include "orc_time.hpp"
#include "orc_energy_phys.hpp"

namespace orc {

struct Euler2DCase {
  EnergyPhys phys;
  Basis basis;
  Mesh2D mesh;
  std::unique_ptr<DG2D<EnergyPhys>> dg;
  size_t ndofs() const { return (size_t)mesh.nelem * basis.n * basis.n; }
};

// initial_condition_gravity_waves, src/equations/initial_condition_compressible_euler_2d.jl:11-35
inline EulerEnergy2D::State ic_gravity_waves(const EulerEnergy2D& eq, const double* x) {
  const double g = eq.g, c_p = eq.c_p, c_v = eq.c_v;
  const double x_c = 100000.0, a = 5000.0, H = 10000.0;
  const double R = c_p - c_v, T0 = 250.0;
  const double delta = g / (R * T0);
  const double DeltaT = 0.001;
  const double pi = 3.14159265358979323846;
  const double Tb = DeltaT * std::sin(pi * x[1] / H) * std::exp(-(x[0] - x_c) * (x[0] - x_c) / (a * a));
  const double ps = 100000.0;
  const double rhos = ps / (T0 * R);
  const double rho_b = rhos * (-Tb / T0);
  const double p = ps * std::exp(-delta * x[1]);
  const double rho = rhos * std::exp(-delta * x[1]) + rho_b * std::exp(-0.5 * delta * x[1]);
  return eq.prim2cons(rho, 20.0, 0.0, p, g * x[1]);
}

// Warm bubble (Wicker & Skamarock 1998) of
// examples/euler/dry_air/buoyancy/elixir_gemein_bubble.jl:20-51 written for the
// energy equations: neutral background theta_ref, cos^2 theta bubble.
inline EulerEnergy2D::State ic_warm_bubble(const EulerEnergy2D& eq, const double* x, double xc,
                                           double zc, double rc, double dtheta, double v1) {
  const double theta_ref = 300.0;
  const double kappa = eq.R / eq.c_p;
  const double r = std::sqrt((x[0] - xc) * (x[0] - xc) + (x[1] - zc) * (x[1] - zc));
  double dth = 0.0;
  if (r <= rc) {
    const double c = std::cos(3.14159265358979323846 * 0.5 * r / rc);
    dth = dtheta * c * c;
  }
  const double theta = theta_ref + dth;
  const double p = eq.p_0 * std::pow(1.0 - kappa * eq.g * x[1] / (eq.R * theta_ref), eq.c_p / eq.R);
  const double rho = p / (std::pow(p / eq.p_0, kappa) * eq.R * theta);
  const double T = p / (eq.R * rho);
  const double rho_e = rho * eq.c_v * T + 0.5 * rho * v1 * v1;
  return {rho, rho * v1, 0.0, rho_e, eq.g * x[1]};
}

// 3D case: geometry and connectivity are copied from the caller's arrays
// (built by the host mirror exactly as passed to the C ABI).
struct Euler3DCase {
  EnergyPhys3D phys;
  Basis basis;
  std::vector<double> Ja, invJ, xyz;
  Mesh3D mesh;
  std::unique_ptr<DG3D<EnergyPhys3D>> dg;
  size_t ndofs() const { return (size_t)mesh.nelem * basis.n * basis.n * basis.n; }
};

struct RainyPhys {
  using State = RainyEuler2D::State;
  static constexpr int nv = 9;
  static constexpr bool has_noncons = false;
  static constexpr bool has_sources = true;
  RainyEuler2D eq;
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_ec_rain(a, b, n);
  }
  State volume_noncons(const State&, const State&, const double*) const { return State{}; }
  // surface 0: flux_lax_friedrichs, 1: flux_LMARS
  int surface = 0;
  // StructuredMesh walls (kind 1): 0 boundary_condition_simple_slip_wall,
  // 1 boundary_condition_slip_wall (pressure Riemann problem)
  int wall = 0;
  State surface_flux(const State& a, const State& b, const double* n) const {
    return surface == 1 ? eq.flux_lmars(a, b, n) : eq.flux_llf(a, b, n);
  }
  State surface_noncons(const State&, const State&, const double*) const { return State{}; }
  State bc_structured(const State& ui, const double* n, int direction) const {
    if (wall == 1) return eq.slip_wall_pressure_structured(ui, n, direction);
    State ub = ui;
    ub[4] = -ui[4];
    return direction % 2 == 0 ? surface_flux(ui, ub, n) : surface_flux(ub, ui, n);
  }
  State bc_normal(const State& ui, const double* n) const {
    if (wall == 1) return eq.slip_wall(ui, n);
    return eq.slip_wall_structured(ui, n, 2);
  }
  // 0: source_terms_rainy; 1: convergence-test manufactured source; 2: none;
  // 3: source_terms_no_phase_change
  int source_kind = 0;
  State flux(const State& u, const double* n) const { return eq.flux(u, n); }
  State source(const State& u, const double* x, double t) const {
    if (source_kind == 2) return State{};
    if (source_kind == 3) return eq.source_no_phase_change(u);
    return source_kind == 0 ? eq.source_rainy(u) : source_convergence(x, t);
  }
  void max_abs_speeds(const State& u, double& l1, double& l2) const { eq.max_abs_speeds(u, l1, l2); }

  // source_terms_convergence_test_rainy,
  // examples/euler/precipitation/tests/convergence_test.jl:42-124
  State source_convergence(const double* x, double t) const {
    const RainyEuler2D& q = eq;
    const double c_help = q.v_0 * 1.9386213994279082 * std::pow(3.14159265358979323846 * q.N_0, -0.125);
    const double c = 2.0, A = 0.1, L = 2.0, f = 1.0 / L, om = 2.0 * 3.14159265358979323846 * f;
    const double si = std::sin(om * (x[0] + x[1] - t)), co = std::cos(om * (x[0] + x[1] - t));
    const double rho = c + A * si;
    const double rho_x = om * A * co, rho_t = -rho_x;
    const double T = rho + 250.0;
    const double svp = q.e_s(T);
    const double rv = svp / (q.R_v * T);
    const double rc = rho / q.c_l * 3000.0;
    const double rr = rho / q.c_l * 1000.0;
    const double rm = rv + rc;
    const double rd = rho - rm - rr;
    const double vr = q.v_rain(rm, rr);
    const double svp_t = rho_t * q.e_s_T(T);
    const double svp_x = rho_x * q.e_s_T(T);
    const double rv_t = (svp_t * T - rho_t * svp) / (q.R_v * T * T);
    const double rv_x = (svp_x * T - rho_x * svp) / (q.R_v * T * T);
    const double rc_t = rho_t / q.c_l * 3000.0, rc_x = rho_x / q.c_l * 3000.0;
    const double rr_t = rho_t / q.c_l * 1000.0, rr_x = rho_x / q.c_l * 1000.0;
    const double rm_t = rv_t + rc_t, rm_x = rv_x + rc_x;
    const double rd_t = rho_t - rm_t - rr_t, rd_x = rho_x - rm_x - rr_x;
    double e_t = (q.c_vd * rd_t + q.c_vv * rv_t + q.c_l * (rc_t + rr_t)) * T;
    e_t += (q.c_vd * rd + q.c_vv * rv + q.c_l * (rc + rr)) * rho_t;
    e_t += rv_t * q.ref_L + rho_t;
    double e_x = (q.c_vd * rd_x + q.c_vv * rv_x + q.c_l * (rc_x + rr_x)) * T;
    e_x += (q.c_vd * rd + q.c_vv * rv + q.c_l * (rc + rr)) * rho_x;
    e_x += rv_x * q.ref_L + rho_x;
    double p_x = (rd_x * q.R_d + rv_x * q.R_v) * T;
    p_x += (rd * q.R_d + rv * q.R_v) * rho_x;
    double vr_x = c_help * 0.125 * ((rr_x * rm - rr * rm_x) / ((rm + rr) * (rm + rr)));
    vr_x *= std::pow(rr / (rm + rr), -0.875);
    const double rrvr_x = rr_x * vr + rr * vr_x;
    State s{};
    s[0] = rd_t + 2.0 * rd_x;
    s[1] = rm_t + 2.0 * rm_x;
    s[2] = rr_t + 2.0 * rr_x - rrvr_x;
    s[3] = rho_x + p_x - rrvr_x;
    s[4] = rho_x + p_x - rrvr_x;
    s[5] = e_t + 2.0 * (e_x + p_x) - (q.c_l * rho_x * rr * vr);
    s[5] -= (q.c_l * T + 1.0) * rrvr_x;
    return s;
  }
};

// initial_condition_convergence_test_rainy, convergence_test.jl:8-40
inline RainyEuler2D::State ic_rainy_convergence(const RainyEuler2D& q, const double* x, double t) {
  const double c = 2.0, A = 0.1, L = 2.0, om = 2.0 * 3.14159265358979323846 / L;
  const double rho = c + A * std::sin(om * (x[0] + x[1] - t));
  const double T = rho + 250.0;
  const double rv = q.e_s(T) / (q.R_v * T);
  const double rc = rho / q.c_l * 3000.0;
  const double rr = rho / q.c_l * 1000.0;
  const double rm = rv + rc;
  const double rd = rho - rm - rr;
  double e = (q.c_vd * rd + q.c_vv * rv + q.c_l * (rc + rr)) * T;
  e += rv * q.ref_L + rho;
  return {rd, rm, rr, rho, rho, e, rv, rc, T};
}

struct RainyCase {
  RainyPhys phys;
  Basis basis;
  Mesh2D mesh;
  std::unique_ptr<DG2D<RainyPhys>> dg;
  size_t ndofs() const { return (size_t)mesh.nelem * basis.n * basis.n; }
};

// Newton solve of the saturation system on every node, restating
// src/callbacks_stage/nonlinear_solve_dg2d.jl:6-44 (warm start from slots 7-9,
// negative rain clamped in the stored state after the node copy is taken,
// guess -= J \ res).  mode 0: the reference's absolute criterion
// max|res| < tol; mode 1: relative criterion |res_1| < tol |E_internal|,
// |res_2|, |res_3| < tol 1e7 rho_moist.  guesses (nodes x 3, may be null)
// replace the warm start.  polish > 0 (a canonical finish that the reference
// does not have): the converged iterate is snapped to a grid fixed by the
// state (vapour, cloud: 2^-24 of the power of two above rho_moist; T: 2^-18 K)
// and `polish` updates are taken from there, kept if the criterion still
// holds, so solves from different starts return the same bits.  Returns the total
// number of Newton updates until the criterion held; iters (may be null)
// receives them per node.
inline void solve3(const double* J, const double* r, double* dx) {
  const double a = J[0], b = J[1], c = J[2], d = J[3], e = J[4], f = J[5], g = J[6], h = J[7],
               i = J[8];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  const double id = 1.0 / det;
  dx[0] = (A * r[0] + (c * h - b * i) * r[1] + (b * f - c * e) * r[2]) * id;
  dx[1] = (B * r[0] + (a * i - c * g) * r[1] + (c * d - a * f) * r[2]) * id;
  dx[2] = (C * r[0] + (b * g - a * h) * r[1] + (a * e - b * d) * r[2]) * id;
}

inline bool newton_done(const RainyEuler2D& eq, const RainyEuler2D::State& u, const double* r,
                        int mode, double tol) {
  if (mode == 0) return std::max(std::fabs(r[0]), std::max(std::fabs(r[1]), std::fabs(r[2]))) < tol;
  const double rho = u[0] + u[1] + u[2];
  const double e_int = u[5] - 0.5 * (u[3] * u[3] + u[4] * u[4]) / rho;
  const double s2 = tol * 1.0e7 * std::fabs(u[1]);
  return std::fabs(r[0]) < tol * std::fabs(e_int) && std::fabs(r[1]) <= s2 && std::fabs(r[2]) <= s2;
}

inline int newton_node(const RainyEuler2D& eq, const RainyEuler2D::State& u, double* x, int mode,
                       double tol, int maxit, int polish, bool* converged) {
  double r[3], J[9], dx[3];
  int it = 0;
  *converged = false;
  for (; it < maxit; ++it) {
    eq.residual(u, x, r);
    if (newton_done(eq, u, r, mode, tol)) {
      *converged = true;
      break;
    }
    eq.jacobian(u, x, J);
    solve3(J, r, dx);
    for (int k = 0; k < 3; ++k) x[k] -= dx[k];
  }
  if (!*converged) {
    eq.residual(u, x, r);
    *converged = newton_done(eq, u, r, mode, tol);
  }
  if (polish > 0 && *converged) {
    // canonical finish: snap to the state's grid, then `polish` updates
    double y[3] = {x[0], x[1], x[2]};
    int e;
    std::frexp(std::fabs(u[1]), &e);
    const double gm = std::ldexp(1.0, e - 24), gt = std::ldexp(1.0, -18);
    y[0] = std::rint(y[0] / gm) * gm;
    y[1] = std::rint(y[1] / gm) * gm;
    y[2] = std::rint(y[2] / gt) * gt;
    for (int p = 0; p < polish; ++p) {
      eq.residual(u, y, r);
      eq.jacobian(u, y, J);
      solve3(J, r, dx);
      for (int k = 0; k < 3; ++k) y[k] -= dx[k];
    }
    eq.residual(u, y, r);
    if (newton_done(eq, u, r, mode, tol))
      for (int k = 0; k < 3; ++k) x[k] = y[k];
  }
  return it;
}

// CompressibleMoistEulerEquations2D on a StructuredMesh.  Volume: flux
// differencing with flux_chandrashekar or the weak form; surface flux 0:
// FluxLMARS(c), 1: flux_lax_friedrichs, 2: flux_chandrashekar; sources 0: none,
// 1: source_terms_geopotential, 2: source_terms_moist_bubble, 3/4: the dry /
// moist convergence tests' sources.
struct MoistPhys {
  using State = MoistEuler2D::State;
  static constexpr int nv = 6;
  static constexpr bool has_noncons = false;
  static constexpr bool has_sources = true;
  MoistEuler2D eq;
  int surface_kind = 0, source_kind = 1;
  double c_lmars = 360.0;
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_chandrashekar(a, b, n);
  }
  State volume_noncons(const State&, const State&, const double*) const { return State{}; }
  State surface_flux(const State& a, const State& b, const double* n) const {
    if (surface_kind == 1) return eq.flux_llf(a, b, n);
    if (surface_kind == 2) return eq.flux_chandrashekar(a, b, n);
    return eq.flux_lmars(a, b, n, c_lmars);
  }
  State surface_noncons(const State&, const State&, const double*) const { return State{}; }
  State bc_structured(const State& ui, const double* n, int direction) const {
    return eq.slip_wall_structured(ui, n, direction);
  }
  State bc_normal(const State& ui, const double* n) const { return eq.slip_wall(ui, n); }
  State flux(const State& u, const double* n) const { return eq.flux(u, n); }
  State source(const State& u, const double* x, double t) const {
    switch (source_kind) {
      case 1: return eq.source_geopotential(u);
      case 2: return eq.source_moist_bubble(u);
      case 3: return eq.source_convergence_dry(u, x, t);
      case 4: return eq.source_convergence_moist(u, x, t);
      case 5: return eq.source_gravity_wave(u, x);
      default: return State{};
    }
  }
  void max_abs_speeds(const State& u, double& l1, double& l2) const { eq.max_abs_speeds(u, l1, l2); }
};

// A 2D mesh given by the host mirror's arrays (curvilinear P4estMesh, or a
// StructuredMesh with curved faces): node coordinates [E][n][n][2],
// contravariant vectors [E][n][n][2][2], inverse Jacobian [E][n][n],
// interfaces and boundary faces as for the C ABI.
Mesh2D mesh_from_arrays(int n, int nelem, const double* xy, const double* Ja, const double* invJ,
                        int nif, const int* if_e, const int* if_f, const int* if_flip, int nbd,
                        const int* bd_e, const int* bd_f, const int* bd_kind) {
  const size_t nodes = (size_t)nelem * n * n;
  Mesh2D m;
  m.n = n;
  m.nelem = nelem;
  m.xy.assign(xy, xy + nodes * 2);
  m.Ja.assign(Ja, Ja + nodes * 4);
  m.invJ.assign(invJ, invJ + nodes);
  for (int k = 0; k < nif; ++k) {
    m.if_e0.push_back(if_e[2 * k]);
    m.if_e1.push_back(if_e[2 * k + 1]);
    m.if_f0.push_back(if_f[2 * k]);
    m.if_f1.push_back(if_f[2 * k + 1]);
    m.if_flip.push_back(if_flip[k]);
  }
  for (int k = 0; k < nbd; ++k) {
    m.bd_e.push_back(bd_e[k]);
    m.bd_f.push_back(bd_f[k]);
    m.bd_kind.push_back(bd_kind[k]);
  }
  return m;
}

struct MoistCase {
  MoistPhys phys;
  Basis basis;
  Mesh2D mesh;
  std::unique_ptr<DG2D<MoistPhys>> dg;
  int ic_kind = 0;
  size_t ndofs() const { return (size_t)mesh.nelem * basis.n * basis.n; }
};

// Initial states of the moist tests.  kind 0: the warm bubble of
// examples/euler/dry_air/buoyancy/elixir_gemein_bubble.jl:20-51 (v1 = 20,
// no moisture); 1 / 2: the dry / moist convergence tests (:173-200, :244-272);
// 3: the mountain-triggered gravity wave of
// examples/euler/dry_air/buoyancy/elixir_gemein_nonhydrostatic_gravity_waves.jl:15-39
// (constant Brunt-Vaisala frequency N = 0.01 over theta_0 = T_0 = 280 K,
// v1 = 10, no moisture).
inline MoistEuler2D::State ic_moist(const MoistEuler2D& eq, int kind, const double* x, double t) {
  if (kind == 1) return eq.ic_convergence_dry(x, t);
  if (kind == 2) return eq.ic_convergence_moist(x, t);
  if (kind == 3) {
    const double z = x[1], theta_0 = 280.0, N = 0.01;
    const double theta = theta_0 * std::exp(N * N * z / eq.g);
    const double p = eq.p_0 * std::pow(1.0 + eq.g * eq.g * (1.0 / (eq.c_pd * theta_0 * (N * N))) *
                                                 (std::exp(-z * (N * N) / eq.g) - 1.0),
                                       1.0 / eq.kappa);
    const double rho = p / (std::pow(p / eq.p_0, eq.kappa) * eq.R_d * theta);
    const double T = p / (eq.R_d * rho);
    const double v1 = 10.0, v2 = 0.0;
    return {rho, rho * v1, rho * v2, rho * eq.c_vd * T + 0.5 * rho * (v1 * v1 + v2 * v2), 0.0,
            0.0};
  }
  const double xc = 10000.0, zc = 2000.0, rc = 2000.0, theta_ref = 300.0;
  const double r = std::sqrt((x[0] - xc) * (x[0] - xc) + (x[1] - zc) * (x[1] - zc));
  double dth = 0.0;
  if (r <= rc) {
    const double c = std::cos(3.14159265358979323846 * (0.5 * r / rc));
    dth = 2.0 * c * c;
  }
  const double theta = theta_ref + dth;
  const double p = eq.p_0 * std::pow(1.0 - eq.kappa * eq.g * x[1] / (eq.R_d * theta_ref),
                                     eq.c_pd / eq.R_d);
  const double rho = p / (std::pow(p / eq.p_0, eq.kappa) * eq.R_d * theta);
  const double T = p / (eq.R_d * rho);
  const double v1 = 20.0;
  return {rho, rho * v1, 0.0, rho * eq.c_vd * T + 0.5 * rho * v1 * v1, 0.0, 0.0};
}

// l2 / linf errors of a 2D StructuredMesh solution against exact(x) on the
// analysis nodes of degree 2N (Trixi's AnalysisCallback, l2 normalised by the
// domain volume).
template <int NVAR, class Exact>
void errors_2d(const Basis& b, const Mesh2D& mesh, const double* u, Exact&& exact, double* l2,
               double* linf) {
  const int n = b.n;
  const Basis a = make_lgl_basis(2 * (n - 1));
  const int na = a.n;
  const std::vector<double> V = interpolation_matrix(b.x, a.x);
  for (int v = 0; v < NVAR; ++v) { l2[v] = 0.0; linf[v] = 0.0; }
  double vol = 0.0;
  constexpr int K = NVAR + 3;
  std::vector<double> fu(n * n * K), tmp(na * n * K), fa(na * na * K);
  for (int e = 0; e < mesh.nelem; ++e) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t q = (size_t)(e * n + j) * n + i;
        for (int v = 0; v < NVAR; ++v) fu[(j * n + i) * K + v] = u[q * NVAR + v];
        fu[(j * n + i) * K + NVAR] = mesh.xy[q * 2];
        fu[(j * n + i) * K + NVAR + 1] = mesh.xy[q * 2 + 1];
        fu[(j * n + i) * K + NVAR + 2] = 1.0 / mesh.invJ[q];
      }
    for (int j = 0; j < n; ++j)
      for (int ia = 0; ia < na; ++ia)
        for (int v = 0; v < K; ++v) {
          double s = 0;
          for (int i = 0; i < n; ++i) s += V[ia * n + i] * fu[(j * n + i) * K + v];
          tmp[(j * na + ia) * K + v] = s;
        }
    for (int ja = 0; ja < na; ++ja)
      for (int ia = 0; ia < na; ++ia)
        for (int v = 0; v < K; ++v) {
          double s = 0;
          for (int j = 0; j < n; ++j) s += V[ja * n + j] * tmp[(j * na + ia) * K + v];
          fa[(ja * na + ia) * K + v] = s;
        }
    for (int ja = 0; ja < na; ++ja)
      for (int ia = 0; ia < na; ++ia) {
        const double* f = &fa[(ja * na + ia) * K];
        const double x[2] = {f[NVAR], f[NVAR + 1]};
        const auto ex = exact(x);
        const double wJ = a.w[ia] * a.w[ja] * f[NVAR + 2];
        for (int v = 0; v < NVAR; ++v) {
          const double d = ex[v] - f[v];
          l2[v] += d * d * wJ;
          linf[v] = std::max(linf[v], std::fabs(d));
        }
        vol += wJ;
      }
  }
  for (int v = 0; v < NVAR; ++v) l2[v] = std::sqrt(l2[v] / vol);
}

// CompressibleEulerPotentialTemperatureEquationsWithGravity2D on a
// StructuredMesh: volume (flux_tec | flux_ec | flux_etec, nonconservative
// gravity term), surface (FluxLMARS(c), flux_zero).
// rayleigh_damping_coefficient (src/equations/initial_condition_compressible_euler_2d.jl:80-106):
// sin^2 ramps of the vertical layer above z_s and of the lateral layers beyond +-x_s
inline double rayleigh_damping(const double* x, double rate, double zs, double ze, double xs,
                               double xe) {
  const double pi = 3.14159265358979323846;
  double dv = 0.0, dr = 0.0, dl = 0.0;
  if (x[1] > zs) {
    const double s = std::sin(pi * (0.5 * (x[1] - zs) / (ze - zs)));
    dv = rate * (s * s);
  }
  if (!(x[0] < xs)) {
    const double s = std::sin(pi * (0.5 * (x[0] - xs) / (xe - xs)));
    dr = rate * (s * s);
  }
  if (!(x[0] > -xs)) {
    const double s = std::sin(pi * (0.5 * (x[0] + xs) / (-xe + xs)));
    dl = rate * (s * s);
  }
  return dv + dr + dl;
}

struct PTPhys {
  using State = PotTemp2D::State;
  static constexpr int nv = 5;
  static constexpr bool has_noncons = true;
  static constexpr bool has_sources = true;
  PotTemp2D eq;
  double c_lmars = 340.0;
  // MountainWaveSetup's source (initial_condition_compressible_euler_2d.jl:174-200):
  // mw = (theta_0, u0, N, z_damping_start, z_damping_end, x_damping_start,
  // x_damping_end, damping_rate); off when mountain == 0
  int mountain = 0;
  double mw[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.volume_flux(a, b, n);
  }
  State volume_noncons(const State& a, const State& b, const double* n) const {
    return eq.noncons(a, b, n);
  }
  State surface_flux(const State& a, const State& b, const double* n) const {
    return eq.surface_flux(a, b, n, c_lmars);
  }
  State surface_noncons(const State& a, const State& b, const double* n) const {
    return eq.surface_noncons(a, b, n);
  }
  State bc_structured(const State& ui, const double* n, int direction) const {
    return eq.slip_wall_structured(ui, n, direction, c_lmars);
  }
  State bc_normal(const State& ui, const double* n) const {
    return eq.slip_wall_normal(ui, n, c_lmars);
  }
  State flux(const State& u, const double* n) const { return eq.flux(u, n); }
  State source(const State& u, const double* x, double) const {
    if (!mountain) return State{};
    const double v1 = u[1] / u[0], theta = u[3] / u[0];
    const double damping = -rayleigh_damping(x, mw[7], mw[3], mw[4], mw[5], mw[6]);
    const double theta_b = mw[0] * std::exp(mw[2] * mw[2] / eq.g * x[1]);
    return {0.0, u[0] * (v1 - mw[1]) * damping, u[2] * damping,
            u[0] * (theta - theta_b) * damping, 0.0};
  }
  void max_abs_speeds(const State& u, double& l1, double& l2) const { eq.max_abs_speeds(u, l1, l2); }
};

struct PTCase {
  PTPhys phys;
  Basis basis;
  Mesh2D mesh;
  std::unique_ptr<DG2D<PTPhys>> dg;
  size_t ndofs() const { return (size_t)mesh.nelem * basis.n * basis.n; }
};

// initial_condition_gravity_waves (src/equations/initial_condition_compressible_euler_2d.jl:11-35)
// for the potential-temperature equations (their prim2cons)
inline PotTemp2D::State ic_gravity_waves_pt(const PotTemp2D& eq, const double* x) {
  const double g = eq.g, R = eq.R, T0 = 250.0;
  const double x_c = 100000.0, a = 5000.0, H = 10000.0;
  const double delta = g / (R * T0);
  const double pi = 3.14159265358979323846;
  const double Tb = 0.001 * std::sin(pi * x[1] / H) * std::exp(-(x[0] - x_c) * (x[0] - x_c) / (a * a));
  const double ps = 100000.0;
  const double rhos = ps / (T0 * R);
  const double rho_b = rhos * (-Tb / T0);
  const double p = ps * std::exp(-delta * x[1]);
  const double rho = rhos * std::exp(-delta * x[1]) + rho_b * std::exp(-0.5 * delta * x[1]);
  return eq.prim2cons(rho, 20.0, 0.0, p, g * x[1]);
}

}  // namespace orc



using namespace orc;

extern "C" {

// Creates a 2D dry-Euler (energy + gravity) case on an nx x ny StructuredMesh
// of the rectangle [x0,x1] x [y0,y1]; periodic flags per direction, slip walls
// elsewhere. Returns an opaque handle.
void* orc_euler2d_create(int polydeg, int nx, int ny, double x0, double x1, double y0, double y1,
                         int periodic_x, int periodic_y, double c_p, double c_v, double g,
                         double c_lmars) {
  auto* c = new Euler2DCase();
  c->phys.eq = EulerEnergy2D(c_p, c_v, g);
  c->phys.c_lmars = c_lmars;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = structured_rectangle(c->basis, nx, ny, x0, x1, y0, y1, periodic_x != 0,
                                 periodic_y != 0, 1);
  c->dg.reset(new DG2D<EnergyPhys>(c->phys, c->basis, c->mesh));
  return c;
}

void orc_euler2d_destroy(void* h) { delete static_cast<Euler2DCase*>(h); }

int64_t orc_euler2d_ndofs(void* h) { return (int64_t) static_cast<Euler2DCase*>(h)->ndofs(); }

// Exports the basis (nodes, weights, D, Dsplit) and the mesh geometry in the
// layouts documented in orc_dg2d.hpp.
void orc_euler2d_basis(void* h, double* x, double* w, double* D, double* Dsplit) {
  auto* c = static_cast<Euler2DCase*>(h);
  const int n = c->basis.n;
  std::memcpy(x, c->basis.x.data(), n * sizeof(double));
  std::memcpy(w, c->basis.w.data(), n * sizeof(double));
  std::memcpy(D, c->basis.D.data(), n * n * sizeof(double));
  std::memcpy(Dsplit, c->basis.Dsplit.data(), n * n * sizeof(double));
}

void orc_euler2d_geometry(void* h, double* Ja, double* invJ, double* xy) {
  auto* c = static_cast<Euler2DCase*>(h);
  std::memcpy(Ja, c->mesh.Ja.data(), c->mesh.Ja.size() * sizeof(double));
  std::memcpy(invJ, c->mesh.invJ.data(), c->mesh.invJ.size() * sizeof(double));
  std::memcpy(xy, c->mesh.xy.data(), c->mesh.xy.size() * sizeof(double));
}

// which: 0 = gravity waves; 1 = warm bubble with params (xc, zc, rc, dtheta, v1)
void orc_euler2d_initial_condition(void* h, int which, const double* prm, double* u) {
  auto* c = static_cast<Euler2DCase*>(h);
  const size_t nd = c->ndofs();
  for (size_t q = 0; q < nd; ++q) {
    const double* x = &c->mesh.xy[q * 2];
    EulerEnergy2D::State s = which == 0
                                 ? ic_gravity_waves(c->phys.eq, x)
                                 : ic_warm_bubble(c->phys.eq, x, prm[0], prm[1], prm[2], prm[3], prm[4]);
    for (int v = 0; v < 5; ++v) u[q * 5 + v] = s[v];
  }
}

void orc_euler2d_rhs(void* h, const double* u, double* du, double t) {
  static_cast<Euler2DCase*>(h)->dg->rhs(u, du, t);
}

double orc_euler2d_max_dt(void* h, const double* u) {
  return static_cast<Euler2DCase*>(h)->dg->max_dt(u);
}

// `nsteps` CK2N54 steps with dt = cfl * max_dt(u) recomputed before each step
// (the StepsizeCallback pattern). k must hold ndofs*nv doubles (kept between
// calls as the 2N register). Returns the final time.
double orc_euler2d_ck_steps(void* h, double* u, double* k, double t, double cfl, int nsteps,
                            double fixed_dt) {
  auto* c = static_cast<Euler2DCase*>(h);
  const size_t N = c->ndofs() * 5;
  std::vector<double> du(N);
  for (int s = 0; s < nsteps; ++s) {
    const double dt = fixed_dt > 0 ? fixed_dt : cfl * c->dg->max_dt(u);
    ck2n54_step([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, u, k,
                du.data(), N, t, dt);
    t += dt;
  }
  return t;
}

// Runs SSPRK43 with adaptive = false from t0 to t_end, dt = cfl * max_dt(u)
// before each step and the last step shortened to land on t_end.
int orc_euler2d_ssprk43_run(void* h, double* u, double t0, double t_end, double cfl) {
  auto* c = static_cast<Euler2DCase*>(h);
  const size_t N = c->ndofs() * 5;
  std::vector<double> tmp(N), du(N), u0(N);
  double t = t0;
  int steps = 0;
  while (t < t_end) {
    double dt = cfl * c->dg->max_dt(u);
    if (t + dt > t_end) dt = t_end - t;
    ssprk43_step([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, u,
                 tmp.data(), du.data(), u0.data(), N, t, dt);
    t += dt;
    ++steps;
  }
  return steps;
}

// L2 and Linf errors against the gravity-wave initial state, evaluated as
// Trixi's AnalysisCallback does: interpolation to LGL nodes of degree
// 2*polydeg, Jacobian-weighted quadrature normalised by the total volume.
void orc_euler2d_errors_gravity_waves(void* h, const double* u, double* l2, double* linf) {
  auto* c = static_cast<Euler2DCase*>(h);
  const Basis& b = c->basis;
  const int n = b.n, N = n - 1;
  const Basis a = make_lgl_basis(2 * N);
  const int na = a.n;
  const std::vector<double> V = interpolation_matrix(b.x, a.x);
  for (int v = 0; v < 5; ++v) { l2[v] = 0.0; linf[v] = 0.0; }
  double vol = 0.0;
  std::vector<double> fu(n * n * 7), fa(na * na * 7), tmp(na * n * 7);
  for (int e = 0; e < c->mesh.nelem; ++e) {
    // pack (u[5], x, y, J) per node
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t q = (size_t)(e * n + j) * n + i;
        for (int v = 0; v < 5; ++v) fu[(j * n + i) * 7 + v] = u[q * 5 + v];
        fu[(j * n + i) * 7 + 5] = c->mesh.xy[q * 2];
        fu[(j * n + i) * 7 + 6] = c->mesh.xy[q * 2 + 1];
      }
    std::vector<double> Jl(n * n);
    for (int q = 0; q < n * n; ++q) Jl[q] = 1.0 / c->mesh.invJ[(size_t)e * n * n + q];
    // interpolate in xi then eta
    for (int j = 0; j < n; ++j)
      for (int ia = 0; ia < na; ++ia)
        for (int v = 0; v < 7; ++v) {
          double s = 0;
          for (int i = 0; i < n; ++i) s += V[ia * n + i] * fu[(j * n + i) * 7 + v];
          tmp[(j * na + ia) * 7 + v] = s;
        }
    for (int ja = 0; ja < na; ++ja)
      for (int ia = 0; ia < na; ++ia)
        for (int v = 0; v < 7; ++v) {
          double s = 0;
          for (int j = 0; j < n; ++j) s += V[ja * n + j] * tmp[(j * na + ia) * 7 + v];
          fa[(ja * na + ia) * 7 + v] = s;
        }
    std::vector<double> Jt(na * n), Ja_(na * na);
    for (int j = 0; j < n; ++j)
      for (int ia = 0; ia < na; ++ia) {
        double s = 0;
        for (int i = 0; i < n; ++i) s += V[ia * n + i] * Jl[j * n + i];
        Jt[j * na + ia] = s;
      }
    for (int ja = 0; ja < na; ++ja)
      for (int ia = 0; ia < na; ++ia) {
        double s = 0;
        for (int j = 0; j < n; ++j) s += V[ja * n + j] * Jt[j * na + ia];
        Ja_[ja * na + ia] = s;
      }
    for (int ja = 0; ja < na; ++ja)
      for (int ia = 0; ia < na; ++ia) {
        const double* f = &fa[(ja * na + ia) * 7];
        const double x[2] = {f[5], f[6]};
        const EulerEnergy2D::State ex = ic_gravity_waves(c->phys.eq, x);
        const double wJ = a.w[ia] * a.w[ja] * Ja_[ja * na + ia];
        for (int v = 0; v < 5; ++v) {
          const double d = ex[v] - f[v];
          l2[v] += d * d * wJ;
          linf[v] = std::max(linf[v], std::fabs(d));
        }
        vol += wJ;
      }
  }
  for (int v = 0; v < 5; ++v) l2[v] = std::sqrt(l2[v] / vol);
}


// ---- 3D: CompressibleEulerEnergyEquationsWithGravity3D on a hexahedral mesh
void* orc_euler3d_create(int polydeg, int nelem, const double* Ja, const double* invJ,
                         const double* xyz, int nif, const int* if_e, const int* if_f,
                         const int* if_orient, int nbd, const int* bd_e, const int* bd_f,
                         double c_p, double c_v, double g, double c_lmars, double omega) {
  auto* c = new Euler3DCase();
  c->phys.eq = EulerEnergy3D(c_p, c_v, g);
  c->phys.c_lmars = c_lmars;
  c->phys.omega = omega;
  c->basis = make_lgl_basis(polydeg);
  const int n = c->basis.n;
  const size_t nodes = (size_t)nelem * n * n * n;
  c->Ja.assign(Ja, Ja + nodes * 9);
  c->invJ.assign(invJ, invJ + nodes);
  if (xyz) c->xyz.assign(xyz, xyz + nodes * 3);
  c->mesh.n = n;
  c->mesh.nelem = nelem;
  c->mesh.Ja = c->Ja.data();
  c->mesh.invJ = c->invJ.data();
  c->mesh.xyz = xyz ? c->xyz.data() : nullptr;
  for (int k = 0; k < nif; ++k) {
    c->mesh.if_e0.push_back(if_e[2 * k]);
    c->mesh.if_e1.push_back(if_e[2 * k + 1]);
    c->mesh.if_f0.push_back(if_f[2 * k]);
    c->mesh.if_f1.push_back(if_f[2 * k + 1]);
    c->mesh.if_orient.push_back(if_orient[k]);
  }
  for (int k = 0; k < nbd; ++k) {
    c->mesh.bd_e.push_back(bd_e[k]);
    c->mesh.bd_f.push_back(bd_f[k]);
  }
  c->dg.reset(new DG3D<EnergyPhys3D>(c->phys, c->basis, c->mesh));
  return c;
}

void orc_euler3d_destroy(void* h) { delete static_cast<Euler3DCase*>(h); }

void orc_euler3d_rhs(void* h, const double* u, double* du, double t) {
  static_cast<Euler3DCase*>(h)->dg->rhs(u, du, t);
}

double orc_euler3d_max_dt(void* h, const double* u) {
  return static_cast<Euler3DCase*>(h)->dg->max_dt(u);
}

double orc_euler3d_ck_steps(void* h, double* u, double* k, double t, double cfl, int nsteps,
                            double fixed_dt) {
  auto* c = static_cast<Euler3DCase*>(h);
  const size_t N = c->ndofs() * 6;
  std::vector<double> du(N);
  for (int s = 0; s < nsteps; ++s) {
    const double dt = fixed_dt > 0 ? fixed_dt : cfl * c->dg->max_dt(u);
    ck2n54_step([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, u, k,
                du.data(), N, t, dt);
    t += dt;
  }
  return t;
}


double orc_euler3d_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                             double fixed_dt, double t_end) {
  auto* c = static_cast<Euler3DCase*>(h);
  return ssp_steps([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
                   [&](const double* uu) { return c->dg->max_dt(uu); }, [](double*) {}, u,
                   c->ndofs() * 6, t, cfl, nsteps, scheme, fixed_dt, t_end);
}

// ---- 3D potential temperature with gravity ----------------------------------
// CompressibleEulerPotentialTemperatureEquationsWithGravity3D: volume
// (flux_tec | flux_ec | flux_etec, nonconservative gravity term), surface
// (FluxLMARS(c), flux_zero), slip walls with the outward normal, Coriolis.
struct PTPhys3D {
  using State = PotTemp3D::State;
  static constexpr int nv = 6;
  static constexpr bool has_noncons = true;
  static constexpr bool has_sources = true;
  PotTemp3D eq;
  double c_lmars = 340.0, omega = 0.0;
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.volume_flux(a, b, n);
  }
  State volume_noncons(const State& a, const State& b, const double* n) const {
    return eq.noncons(a, b, n);
  }
  State surface_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_lmars(a, b, n, c_lmars);
  }
  State surface_noncons(const State&, const State&, const double*) const { return State{}; }
  State bc_normal(const State& ui, const double* n) const {
    return eq.slip_wall_normal(ui, n, c_lmars);
  }
  State source(const State& u, const double*, double) const { return eq.coriolis(u, omega); }
  void max_abs_speeds(const State& u, double* l) const { eq.max_abs_speeds(u, l); }
};

struct PT3DCase {
  PTPhys3D phys;
  Basis basis;
  std::vector<double> Ja, invJ, xyz;
  Mesh3D mesh;
  std::unique_ptr<DG3D<PTPhys3D>> dg;
  size_t ndofs() const { return (size_t)mesh.nelem * basis.n * basis.n * basis.n; }
};

void* orc_pt3d_create(int polydeg, int nelem, const double* Ja, const double* invJ,
                      const double* xyz, int nif, const int* if_e, const int* if_f,
                      const int* if_orient, int nbd, const int* bd_e, const int* bd_f, double c_p,
                      double c_v, double g, double c_lmars, double omega, int volume, int nc) {
  auto* c = new PT3DCase();
  c->phys.eq.init(c_p, c_v, g);
  c->phys.eq.volume = volume;
  c->phys.eq.nc_kind = nc;
  c->phys.c_lmars = c_lmars;
  c->phys.omega = omega;
  c->basis = make_lgl_basis(polydeg);
  const int n = c->basis.n;
  const size_t nodes = (size_t)nelem * n * n * n;
  c->Ja.assign(Ja, Ja + nodes * 9);
  c->invJ.assign(invJ, invJ + nodes);
  if (xyz) c->xyz.assign(xyz, xyz + nodes * 3);
  c->mesh.n = n;
  c->mesh.nelem = nelem;
  c->mesh.Ja = c->Ja.data();
  c->mesh.invJ = c->invJ.data();
  c->mesh.xyz = xyz ? c->xyz.data() : nullptr;
  for (int k = 0; k < nif; ++k) {
    c->mesh.if_e0.push_back(if_e[2 * k]);
    c->mesh.if_e1.push_back(if_e[2 * k + 1]);
    c->mesh.if_f0.push_back(if_f[2 * k]);
    c->mesh.if_f1.push_back(if_f[2 * k + 1]);
    c->mesh.if_orient.push_back(if_orient[k]);
  }
  for (int k = 0; k < nbd; ++k) {
    c->mesh.bd_e.push_back(bd_e[k]);
    c->mesh.bd_f.push_back(bd_f[k]);
  }
  c->dg.reset(new DG3D<PTPhys3D>(c->phys, c->basis, c->mesh));
  return c;
}

void orc_pt3d_destroy(void* h) { delete static_cast<PT3DCase*>(h); }

void orc_pt3d_rhs(void* h, const double* u, double* du, double t) {
  static_cast<PT3DCase*>(h)->dg->rhs(u, du, t);
}

double orc_pt3d_max_dt(void* h, const double* u) {
  return static_cast<PT3DCase*>(h)->dg->max_dt(u);
}

double orc_pt3d_ck_steps(void* h, double* u, double* k, double t, double cfl, int nsteps,
                         double fixed_dt) {
  auto* c = static_cast<PT3DCase*>(h);
  const size_t N = c->ndofs() * 6;
  std::vector<double> du(N);
  for (int s = 0; s < nsteps; ++s) {
    const double dt = fixed_dt > 0 ? fixed_dt : cfl * c->dg->max_dt(u);
    ck2n54_step([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, u, k,
                du.data(), N, t, dt);
    t += dt;
  }
  return t;
}

double orc_pt3d_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                          double fixed_dt, double t_end) {
  auto* c = static_cast<PT3DCase*>(h);
  return ssp_steps([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
                   [&](const double* uu) { return c->dg->max_dt(uu); }, [](double*) {}, u,
                   c->ndofs() * 6, t, cfl, nsteps, scheme, fixed_dt, t_end);
}

// Adaptive SSPRK43 (orc_time.hpp) on a 3D potential-temperature case; see
// orc_pt_ssprk43_adaptive.
double orc_pt3d_ssprk43_adaptive(void* h, double* u, double t, double t_end, const double* stops,
                                 int nstops, double abstol, double reltol, int variant,
                                 double* stats) {
  auto* c = static_cast<PT3DCase*>(h);
  AdaptiveStats st;
  const double tf = ssprk43_adaptive(
      [&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, [](double*) {}, u,
      c->ndofs() * 6, t, t_end, stops, nstops, abstol, reltol, variant, &st);
  if (stats) {
    stats[0] = (double)st.accepted;
    stats[1] = (double)st.rejected;
    stats[2] = (double)st.rhs_calls;
    stats[3] = st.dt_first;
    stats[4] = st.dt_last;
  }
  return tf;
}

// pointwise 3D fluxes for the consistency tests: kind 0 flux, 1 volume flux
// (tec / ec / etec / kennedy_gruber by `volume`), 2 nonconservative term (by
// `nc`), 3 LMARS(c)
void orc_pt3d_pointwise(int kind, int volume, int nc, double c, const double* ul,
                        const double* ur, const double* n, double* f) {
  PotTemp3D eq;
  eq.init(1004.0, 717.0, 9.80616);
  eq.volume = volume;
  eq.nc_kind = nc;
  PotTemp3D::State a, b;
  for (int v = 0; v < 6; ++v) { a[v] = ul[v]; b[v] = ur[v]; }
  PotTemp3D::State r = kind == 0 ? eq.flux(a, n)
                     : kind == 1 ? eq.volume_flux(a, b, n)
                     : kind == 2 ? eq.noncons(a, b, n)
                                 : eq.flux_lmars(a, b, n, c);
  for (int v = 0; v < 6; ++v) f[v] = r[v];
}

// the same for the 2D equations (5 variables)
void orc_pt2d_pointwise(int kind, int volume, int nc, double c, const double* ul,
                        const double* ur, const double* n, double* f) {
  PotTemp2D eq;
  eq.init(1004.0, 717.0, 9.80616);
  eq.volume = volume;
  eq.nc_kind = nc;
  PotTemp2D::State a, b;
  for (int v = 0; v < 5; ++v) { a[v] = ul[v]; b[v] = ur[v]; }
  PotTemp2D::State r = kind == 0 ? eq.flux(a, n)
                     : kind == 1 ? eq.volume_flux(a, b, n)
                     : kind == 2 ? eq.noncons(a, b, n)
                                 : eq.flux_lmars(a, b, n, c);
  for (int v = 0; v < 5; ++v) f[v] = r[v];
}

// ---- 2D rainy Euler (flux_ec_rain / flux_lax_friedrichs, source_terms_rainy,
//      simple slip walls) on a StructuredMesh rectangle
// weak_form: VolumeIntegralWeakForm (else flux differencing with flux_ec_rain);
// source_kind: 0 source_terms_rainy, 1 the convergence-test source, 2 none.
void* orc_rainy_create(int polydeg, int nx, int ny, double x0, double x1, double y0, double y1,
                       int periodic_x, int periodic_y, int weak_form, int source_kind) {
  auto* c = new RainyCase();
  c->phys.source_kind = source_kind;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = structured_rectangle(c->basis, nx, ny, x0, x1, y0, y1, periodic_x != 0,
                                 periodic_y != 0, 1);
  c->dg.reset(new DG2D<RainyPhys>(c->phys, c->basis, c->mesh));
  c->dg->weak_form = weak_form != 0;
  return c;
}

// on a mesh given by the host mirror's arrays (see mesh_from_arrays);
// surface 0 flux_lax_friedrichs / 1 flux_LMARS, wall 0 simple / 1 pressure
// Riemann slip wall on the boundary faces of kind 1
void* orc_rainy_create_mesh(int polydeg, int nelem, const double* xy, const double* Ja,
                            const double* invJ, int nif, const int* if_e, const int* if_f,
                            const int* if_flip, int nbd, const int* bd_e, const int* bd_f,
                            const int* bd_kind, int weak_form, int source_kind, int surface,
                            int wall) {
  auto* c = new RainyCase();
  c->phys.source_kind = source_kind;
  c->phys.surface = surface;
  c->phys.wall = wall;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = mesh_from_arrays(c->basis.n, nelem, xy, Ja, invJ, nif, if_e, if_f, if_flip, nbd, bd_e,
                             bd_f, bd_kind);
  c->dg.reset(new DG2D<RainyPhys>(c->phys, c->basis, c->mesh));
  c->dg->weak_form = weak_form != 0;
  return c;
}

void orc_rainy_flux_lmars(const double* ul, const double* ur, const double* n, double* f) {
  RainyEuler2D eq;
  RainyEuler2D::State a, b;
  for (int v = 0; v < 9; ++v) { a[v] = ul[v]; b[v] = ur[v]; }
  const auto r = eq.flux_lmars(a, b, n);
  for (int v = 0; v < 9; ++v) f[v] = r[v];
}

void orc_rainy_slip_wall(const double* u, const double* n, double* f) {
  RainyEuler2D eq;
  RainyEuler2D::State a;
  for (int v = 0; v < 9; ++v) a[v] = u[v];
  const auto r = eq.slip_wall(a, n);
  for (int v = 0; v < 9; ++v) f[v] = r[v];
}

void orc_rainy_geometry(void* h, double* xy) {
  auto* c = static_cast<RainyCase*>(h);
  std::memcpy(xy, c->mesh.xy.data(), c->mesh.xy.size() * sizeof(double));
}

void orc_rainy_initial_condition_convergence(void* h, double t, double* u) {
  auto* c = static_cast<RainyCase*>(h);
  const size_t nd = c->ndofs();
  for (size_t q = 0; q < nd; ++q) {
    const auto s = ic_rainy_convergence(c->phys.eq, &c->mesh.xy[q * 2], t);
    for (int v = 0; v < 9; ++v) u[q * 9 + v] = s[v];
  }
}

// l2 / linf errors against the convergence-test solution at time t (analysis
// nodes of degree 2N, as in orc_euler2d_errors_gravity_waves).
void orc_rainy_errors_convergence(void* h, const double* u, double t, double* l2, double* linf) {
  auto* c = static_cast<RainyCase*>(h);
  const Basis& b = c->basis;
  const int n = b.n;
  const Basis a = make_lgl_basis(2 * (n - 1));
  const int na = a.n;
  const std::vector<double> V = interpolation_matrix(b.x, a.x);
  for (int v = 0; v < 9; ++v) { l2[v] = 0.0; linf[v] = 0.0; }
  double vol = 0.0;
  constexpr int K = 12;  // 9 vars + x + y + J
  std::vector<double> fu(n * n * K), tmp(na * n * K), fa(na * na * K);
  for (int e = 0; e < c->mesh.nelem; ++e) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t q = (size_t)(e * n + j) * n + i;
        for (int v = 0; v < 9; ++v) fu[(j * n + i) * K + v] = u[q * 9 + v];
        fu[(j * n + i) * K + 9] = c->mesh.xy[q * 2];
        fu[(j * n + i) * K + 10] = c->mesh.xy[q * 2 + 1];
        fu[(j * n + i) * K + 11] = 1.0 / c->mesh.invJ[q];
      }
    for (int j = 0; j < n; ++j)
      for (int ia = 0; ia < na; ++ia)
        for (int v = 0; v < K; ++v) {
          double s = 0;
          for (int i = 0; i < n; ++i) s += V[ia * n + i] * fu[(j * n + i) * K + v];
          tmp[(j * na + ia) * K + v] = s;
        }
    for (int ja = 0; ja < na; ++ja)
      for (int ia = 0; ia < na; ++ia)
        for (int v = 0; v < K; ++v) {
          double s = 0;
          for (int j = 0; j < n; ++j) s += V[ja * n + j] * tmp[(j * na + ia) * K + v];
          fa[(ja * na + ia) * K + v] = s;
        }
    for (int ja = 0; ja < na; ++ja)
      for (int ia = 0; ia < na; ++ia) {
        const double* f = &fa[(ja * na + ia) * K];
        const double x[2] = {f[9], f[10]};
        const auto ex = ic_rainy_convergence(c->phys.eq, x, t);
        const double wJ = a.w[ia] * a.w[ja] * f[11];
        for (int v = 0; v < 9; ++v) {
          const double d = ex[v] - f[v];
          l2[v] += d * d * wJ;
          linf[v] = std::max(linf[v], std::fabs(d));
        }
        vol += wJ;
      }
  }
  for (int v = 0; v < 9; ++v) l2[v] = std::sqrt(l2[v] / vol);
}

void orc_rainy_destroy(void* h) { delete static_cast<RainyCase*>(h); }

void orc_rainy_rhs(void* h, const double* u, double* du, double t) {
  static_cast<RainyCase*>(h)->dg->rhs(u, du, t);
}

double orc_rainy_max_dt(void* h, const double* u) {
  return static_cast<RainyCase*>(h)->dg->max_dt(u);
}

// Newton stage limiter over n node states u[n][9] (see newton_node); returns
// the summed Newton updates and the number of nodes that did not converge in
// *nfail.  guesses[n][3], when given, replaces the warm start of slots 7-9.
long orc_rainy_newton_states(double* u, long nodes, int mode, double tol, int maxit, int polish,
                             const double* guesses, int* iters, long* nfail) {
  const RainyEuler2D eq;
  long total = 0, bad = 0;
#pragma omp parallel for reduction(+ : total, bad) schedule(static)
  for (long q = 0; q < nodes; ++q) {
    double* un = u + q * 9;
    RainyEuler2D::State s;
    for (int v = 0; v < 9; ++v) s[v] = un[v];
    double x[3] = {un[6], un[7], un[8]};
    if (guesses) {
      x[0] = guesses[q * 3];
      x[1] = guesses[q * 3 + 1];
      x[2] = guesses[q * 3 + 2];
    }
    if (un[2] < 0.0) un[2] = 0.0;
    bool conv;
    const int it = newton_node(eq, s, x, mode, tol, maxit, polish, &conv);
    if (iters) iters[q] = it;
    total += it;
    if (!conv) ++bad;
    un[6] = x[0];
    un[7] = x[1];
    un[8] = x[2];
  }
  if (nfail) *nfail = bad;
  return total;
}

// The same over all nodes of a rainy case.
long orc_rainy_newton(void* h, double* u, int mode, double tol, int maxit, int polish,
                      const double* guesses, int* iters, long* nfail) {
  auto* c = static_cast<RainyCase*>(h);
  return orc_rainy_newton_states(u, (long)c->ndofs(), mode, tol, maxit, polish, guesses, iters,
                                 nfail);
}

// CK2N54 steps with the Newton stage limiter after every stage (the
// reference's solve(ode, ...; stage_limiter! = NonlinearSolveDG(...))).
double orc_rainy_ck_steps(void* h, double* u, double* k, double t, double cfl, int nsteps,
                          double fixed_dt, int mode, double tol, int maxit, double t_end) {
  auto* c = static_cast<RainyCase*>(h);
  const size_t N = c->ndofs() * 9;
  std::vector<double> du(N);
  for (int s = 0; s < nsteps; ++s) {
    if (t_end > 0 && t >= t_end) break;
    double dt = fixed_dt > 0 ? fixed_dt : cfl * c->dg->max_dt(u);
    if (t_end > 0 && t + dt > t_end) dt = t_end - t;
    for (int st = 0; st < CK2N54::stages; ++st) {
      c->dg->rhs(u, du.data(), t + CK2N54::c[st] * dt);
      const double a = CK2N54::A[st], bb = CK2N54::B[st];
#pragma omp parallel for schedule(static)
      for (long q = 0; q < (long)N; ++q) {
        k[q] = a * k[q] + dt * du[q];
        u[q] = u[q] + bb * k[q];
      }
      long nf;
      orc_rainy_newton(h, u, mode, tol, maxit, 0, nullptr, nullptr, &nf);
    }
    t += dt;
  }
  return t;
}

// ---- 2D internal energy with gravity ------------------------------------------
// CompressibleEulerInternalEnergyEquationsWithGravity2D: volume
// (flux_conservative_etec, flux_nonconservative_etec), surface
// (flux_conservative_es, flux_nonconservative_es), slip walls with the
// outward normal (the reference's P4estMesh elixir).
struct IEPhys {
  using State = InternalEnergy2D::State;
  static constexpr int nv = 5;
  static constexpr bool has_noncons = true;
  static constexpr bool has_sources = false;
  InternalEnergy2D eq;
  State flux(const State& u, const double* n) const { return eq.flux(u, n); }
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_etec(a, b, n);
  }
  State volume_noncons(const State& a, const State& b, const double* n) const {
    return eq.noncons_etec(a, b, n);
  }
  int surface = 0;  // 0: the es pair (the elixir's), 1: the etec pair (entropy conservative)
  State surface_flux(const State& a, const State& b, const double* n) const {
    return surface ? eq.flux_etec(a, b, n) : eq.flux_es(a, b, n);
  }
  State surface_noncons(const State& a, const State& b, const double* n) const {
    return surface ? eq.noncons_etec(a, b, n) : eq.noncons_es(a, b, n);
  }
  State bc_structured(const State& ui, const double* n, int) const {
    return eq.slip_wall_normal(ui, n);
  }
  State bc_normal(const State& ui, const double* n) const { return eq.slip_wall_normal(ui, n); }
  State source(const State&, const double*, double) const { return State{}; }
  void max_abs_speeds(const State& u, double& l1, double& l2) const {
    eq.max_abs_speeds(u, l1, l2);
  }
};

struct IECase {
  IEPhys phys;
  Basis basis;
  Mesh2D mesh;
  std::unique_ptr<DG2D<IEPhys>> dg;
  size_t ndofs() const { return (size_t)mesh.nelem * basis.n * basis.n; }
};

void* orc_ie_create(int polydeg, int nx, int ny, double x0, double x1, double y0, double y1,
                    int periodic_x, int periodic_y, double c_p, double c_v, double g,
                    int surface) {
  auto* c = new IECase();
  c->phys.eq.init(c_p, c_v, g);
  c->phys.surface = surface;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = structured_rectangle(c->basis, nx, ny, x0, x1, y0, y1, periodic_x != 0,
                                 periodic_y != 0, 2);
  c->dg.reset(new DG2D<IEPhys>(c->phys, c->basis, c->mesh));
  return c;
}

void orc_ie_destroy(void* h) { delete static_cast<IECase*>(h); }

void orc_ie_rhs(void* h, const double* u, double* du, double t) {
  static_cast<IECase*>(h)->dg->rhs(u, du, t);
}

double orc_ie_max_dt(void* h, const double* u) { return static_cast<IECase*>(h)->dg->max_dt(u); }

double orc_ie_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                        double fixed_dt, double t_end) {
  auto* c = static_cast<IECase*>(h);
  return ssp_steps([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
                   [&](const double* uu) { return c->dg->max_dt(uu); }, [](double*) {}, u,
                   c->ndofs() * 5, t, cfl, nsteps, scheme, fixed_dt, t_end);
}

// pointwise fluxes for the consistency tests: kind 0 flux, 1 conservative
// etec, 2 nonconservative etec, 3 conservative es, 4 nonconservative es
void orc_ie_pointwise(int kind, const double* ul, const double* ur, const double* n, double* f) {
  InternalEnergy2D eq;
  eq.init(1004.0, 717.0, 9.81);
  InternalEnergy2D::State a, b;
  for (int v = 0; v < 5; ++v) { a[v] = ul[v]; b[v] = ur[v]; }
  const InternalEnergy2D::State r = kind == 0 ? eq.flux(a, n)
                                  : kind == 1 ? eq.flux_etec(a, b, n)
                                  : kind == 2 ? eq.noncons_etec(a, b, n)
                                  : kind == 3 ? eq.flux_es(a, b, n)
                                              : eq.noncons_es(a, b, n);
  for (int v = 0; v < 5; ++v) f[v] = r[v];
}

// SSPRK43 / SSPRK33 steps with the Newton stage limiter after every stage.
double orc_rainy_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                           double fixed_dt, double t_end, int mode, double tol, int maxit) {
  auto* c = static_cast<RainyCase*>(h);
  return ssp_steps([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
                   [&](const double* uu) { return c->dg->max_dt(uu); },
                   [&](double* v) {
                     long nf;
                     orc_rainy_newton(h, v, mode, tol, maxit, 0, nullptr, nullptr, &nf);
                   },
                   u, c->ndofs() * 9, t, cfl, nsteps, scheme, fixed_dt, t_end);
}

// Adaptive SSPRK43 (orc_time.hpp) on a rainy case with the Newton stage
// limiter (mode, tol, maxit) after every stage, as SSPRK43(; stage_limiter!)
// applies NonlinearSolveDG; stats as orc_pt_ssprk43_adaptive.
double orc_rainy_ssprk43_adaptive(void* h, double* u, double t, double t_end,
                                  const double* stops, int nstops, double abstol, double reltol,
                                  int variant, int mode, double tol, int maxit, double* stats) {
  auto* c = static_cast<RainyCase*>(h);
  AdaptiveStats st;
  const double tf = ssprk43_adaptive(
      [&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
      [&](double* v) {
        long nf;
        orc_rainy_newton(h, v, mode, tol, maxit, 0, nullptr, nullptr, &nf);
      },
      u, c->ndofs() * 9, t, t_end, stops, nstops, abstol, reltol, variant, &st);
  if (stats) {
    stats[0] = (double)st.accepted;
    stats[1] = (double)st.rejected;
    stats[2] = (double)st.rhs_calls;
    stats[3] = st.dt_first;
    stats[4] = st.dt_last;
  }
  return tf;
}

// Pointwise helpers for tests: flux_ec_rain, flux_llf, residual, Jacobian.
void orc_rainy_flux_ec(const double* ul, const double* ur, const double* n, double* f) {
  RainyEuler2D eq;
  RainyEuler2D::State a, b;
  for (int v = 0; v < 9; ++v) { a[v] = ul[v]; b[v] = ur[v]; }
  const auto r = eq.flux_ec_rain(a, b, n);
  for (int v = 0; v < 9; ++v) f[v] = r[v];
}

void orc_rainy_flux(const double* u, const double* n, double* f) {
  RainyEuler2D eq;
  RainyEuler2D::State a;
  for (int v = 0; v < 9; ++v) a[v] = u[v];
  const auto r = eq.flux(a, n);
  for (int v = 0; v < 9; ++v) f[v] = r[v];
}

double orc_rainy_saturation_vapour_pressure(double T) { return RainyEuler2D().e_s(T); }

// ---- 2D moist Euler (CompressibleMoistEulerEquations2D) -------------------
// wall_kind: 1 StructuredMesh slip wall semantics, 2 outward-normal (P4estMesh).
void* orc_moist_create(int polydeg, int nx, int ny, double x0, double x1, double y0, double y1,
                       int periodic_x, int periodic_y, int weak_form, int surface_kind,
                       int source_kind, int wall_kind, double c_lmars, double gravity,
                       int ic_kind) {
  auto* c = new MoistCase();
  c->phys.eq.init(1004.0, 717.0, 1885.0, 1424.0, gravity);
  c->phys.surface_kind = surface_kind;
  c->phys.source_kind = source_kind;
  c->phys.c_lmars = c_lmars;
  c->ic_kind = ic_kind;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = structured_rectangle(c->basis, nx, ny, x0, x1, y0, y1, periodic_x != 0,
                                 periodic_y != 0, wall_kind);
  c->dg.reset(new DG2D<MoistPhys>(c->phys, c->basis, c->mesh));
  c->dg->weak_form = weak_form != 0;
  return c;
}

// the same on a mesh given by the host mirror's arrays (see mesh_from_arrays)
void* orc_moist_create_mesh(int polydeg, int nelem, const double* xy, const double* Ja,
                            const double* invJ, int nif, const int* if_e, const int* if_f,
                            const int* if_flip, int nbd, const int* bd_e, const int* bd_f,
                            const int* bd_kind, int weak_form, int surface_kind, int source_kind,
                            double c_lmars, double gravity, int ic_kind) {
  auto* c = new MoistCase();
  c->phys.eq.init(1004.0, 717.0, 1885.0, 1424.0, gravity);
  c->phys.surface_kind = surface_kind;
  c->phys.source_kind = source_kind;
  c->phys.c_lmars = c_lmars;
  c->ic_kind = ic_kind;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = mesh_from_arrays(c->basis.n, nelem, xy, Ja, invJ, nif, if_e, if_f, if_flip, nbd, bd_e,
                             bd_f, bd_kind);
  c->dg.reset(new DG2D<MoistPhys>(c->phys, c->basis, c->mesh));
  c->dg->weak_form = weak_form != 0;
  return c;
}

void orc_moist_destroy(void* h) { delete static_cast<MoistCase*>(h); }

void orc_moist_initial_condition(void* h, double t, double* u) {
  auto* c = static_cast<MoistCase*>(h);
  const size_t nd = c->ndofs();
  for (size_t q = 0; q < nd; ++q) {
    const auto s = ic_moist(c->phys.eq, c->ic_kind, &c->mesh.xy[q * 2], t);
    for (int v = 0; v < 6; ++v) u[q * 6 + v] = s[v];
  }
}

void orc_moist_errors(void* h, const double* u, double t, double* l2, double* linf) {
  auto* c = static_cast<MoistCase*>(h);
  errors_2d<6>(c->basis, c->mesh, u,
               [&](const double* x) { return ic_moist(c->phys.eq, c->ic_kind, x, t); }, l2, linf);
}

void orc_moist_rhs(void* h, const double* u, double* du, double t) {
  static_cast<MoistCase*>(h)->dg->rhs(u, du, t);
}

double orc_moist_max_dt(void* h, const double* u) { return static_cast<MoistCase*>(h)->dg->max_dt(u); }

// CK2N54 steps at cfl (or fixed_dt), the last one shortened to land on t_end
// (> 0) as OrdinaryDiffEq does; returns the new time.
double orc_moist_ck_steps(void* h, double* u, double* k, double t, double cfl, int nsteps,
                          double fixed_dt, double t_end) {
  auto* c = static_cast<MoistCase*>(h);
  const size_t N = c->ndofs() * 6;
  std::vector<double> du(N);
  for (int s = 0; s < nsteps; ++s) {
    if (t_end > 0 && t >= t_end) break;
    double dt = fixed_dt > 0 ? fixed_dt : cfl * c->dg->max_dt(u);
    if (t_end > 0 && t + dt > t_end) dt = t_end - t;
    ck2n54_step([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, u, k,
                du.data(), N, t, dt);
    t += dt;
  }
  return t;
}

void orc_moist_flux_chandrashekar(const double* ul, const double* ur, const double* n, double* f) {
  MoistEuler2D eq;
  eq.init(1004.0, 717.0, 1885.0, 1424.0, 9.80616);
  MoistEuler2D::State a, b;
  for (int v = 0; v < 6; ++v) { a[v] = ul[v]; b[v] = ur[v]; }
  const auto r = eq.flux_chandrashekar(a, b, n);
  for (int v = 0; v < 6; ++v) f[v] = r[v];
}

void orc_moist_flux(const double* u, const double* n, double* f) {
  MoistEuler2D eq;
  eq.init(1004.0, 717.0, 1885.0, 1424.0, 9.80616);
  MoistEuler2D::State a;
  for (int v = 0; v < 6; ++v) a[v] = u[v];
  const auto r = eq.flux(a, n);
  for (int v = 0; v < 6; ++v) f[v] = r[v];
}

// ---- covariant shallow water on the cubed sphere --------------------------
// aux: [E][n][n][26] (the reference's aux_node_vars), xyz: [E][n][n][3];
// interfaces as passed to the C ABI (orientation 1 = secondary runs backward).
// flux ids: see orc::CovFluxes.
void* orc_cov_create(int polydeg, int nelem, const double* aux, const double* xyz, int nif,
                     const int* if_e, const int* if_f, const int* if_flip, double g, double omega,
                     int split, int volume, int vol_sym, int vol_nc, int surf_sym, int surf_diss,
                     int surf_nc) {
  auto* c = new CovDG();
  c->eq.g = g;
  c->eq.omega = omega;
  c->eq.split = split != 0;
  c->fx = CovFluxes{volume, vol_sym, vol_nc, surf_sym, surf_diss, surf_nc};
  c->b = make_lgl_basis(polydeg);
  c->n = polydeg + 1;
  c->nelem = nelem;
  const size_t nodes = (size_t)nelem * c->n * c->n;
  c->aux.assign(aux, aux + nodes * 26);
  c->xyz.assign(xyz, xyz + nodes * 3);
  for (int k = 0; k < nif; ++k) {
    c->if_e0.push_back(if_e[2 * k]);
    c->if_e1.push_back(if_e[2 * k + 1]);
    c->if_f0.push_back(if_f[2 * k]);
    c->if_f1.push_back(if_f[2 * k + 1]);
    c->if_flip.push_back(if_flip[k]);
  }
  return c;
}

void orc_cov_destroy(void* h) { delete static_cast<CovDG*>(h); }

void orc_cov_rhs(void* h, const double* u, double* du) { static_cast<CovDG*>(h)->rhs(u, du); }

double orc_cov_max_dt(void* h, const double* u) { return static_cast<CovDG*>(h)->max_dt(u); }

double orc_cov_ck_steps(void* h, double* u, double* k, double t, double cfl, int nsteps,
                        double fixed_dt, double t_end) {
  auto* c = static_cast<CovDG*>(h);
  const size_t N = (size_t)c->nelem * c->n * c->n * 3;
  std::vector<double> du(N);
  for (int s = 0; s < nsteps; ++s) {
    if (t_end > 0 && t >= t_end) break;
    double dt = fixed_dt > 0 ? fixed_dt : cfl * c->max_dt(u);
    if (t_end > 0 && t + dt > t_end) dt = t_end - t;
    ck2n54_step([&](const double* uu, double* dd, double) { c->rhs(uu, dd); }, u, k, du.data(), N,
                t, dt);
    t += dt;
  }
  return t;
}

double orc_cov_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                         double fixed_dt, double t_end) {
  auto* c = static_cast<CovDG*>(h);
  return ssp_steps([&](const double* uu, double* dd, double) { c->rhs(uu, dd); },
                   [&](const double* uu) { return c->max_dt(uu); }, [](double*) {}, u,
                   (size_t)c->nelem * c->n * c->n * 3, t, cfl, nsteps, scheme, fixed_dt, t_end);
}

// ---- 2D potential temperature with gravity --------------------------------
// volume: 0 flux_tec, 1 flux_ec, 2 flux_etec; nc: 0 waruszewski, 1 artiano,
// 2 souza; wall_kind: 1 StructuredMesh, 2 outward normal.
void* orc_pt_create(int polydeg, int nx, int ny, double x0, double x1, double y0, double y1,
                    int periodic_x, int periodic_y, int volume, int nc, int wall_kind,
                    double c_p, double c_v, double g, double c_lmars, int surface, int snc) {
  auto* c = new PTCase();
  c->phys.eq.init(c_p, c_v, g);
  c->phys.eq.volume = volume;
  c->phys.eq.nc_kind = nc;
  c->phys.eq.surface = surface;
  c->phys.eq.snc_kind = snc;
  c->phys.c_lmars = c_lmars;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = structured_rectangle(c->basis, nx, ny, x0, x1, y0, y1, periodic_x != 0,
                                 periodic_y != 0, wall_kind);
  c->dg.reset(new DG2D<PTPhys>(c->phys, c->basis, c->mesh));
  return c;
}

// potential temperature on such a mesh:
// node coordinates [E][n][n][2], contravariant vectors [E][n][n][2][2],
// inverse Jacobian [E][n][n], interfaces and boundary faces as for the C ABI
void* orc_pt_create_mesh(int polydeg, int nelem, const double* xy, const double* Ja,
                         const double* invJ, int nif, const int* if_e, const int* if_f,
                         const int* if_flip, int nbd, const int* bd_e, const int* bd_f,
                         const int* bd_kind, int volume, int nc, int surface, int snc, double c_p,
                         double c_v, double g, double c_lmars) {
  auto* c = new PTCase();
  c->phys.eq.init(c_p, c_v, g);
  c->phys.eq.volume = volume;
  c->phys.eq.nc_kind = nc;
  c->phys.eq.surface = surface;
  c->phys.eq.snc_kind = snc;
  c->phys.c_lmars = c_lmars;
  c->basis = make_lgl_basis(polydeg);
  c->mesh = mesh_from_arrays(c->basis.n, nelem, xy, Ja, invJ, nif, if_e, if_f, if_flip, nbd, bd_e,
                             bd_f, bd_kind);
  c->dg.reset(new DG2D<PTPhys>(c->phys, c->basis, c->mesh));
  return c;
}

// MountainWaveSetup's damping source (params as PTPhys::mw) and the states of
// the Dirichlet boundary faces (kind 4) [B][n][5]
void orc_pt_set_mountain(void* h, const double* mw, const double* bd_values) {
  auto* c = static_cast<PTCase*>(h);
  c->phys.mountain = mw != nullptr;
  if (mw)
    for (int k = 0; k < 8; ++k) c->phys.mw[k] = mw[k];
  if (bd_values) {
    const size_t nb = c->mesh.bd_e.size() * c->basis.n * 5;
    c->mesh.bd_values.assign(bd_values, bd_values + nb);
  }
  c->dg.reset(new DG2D<PTPhys>(c->phys, c->basis, c->mesh));
}

void orc_pt_destroy(void* h) { delete static_cast<PTCase*>(h); }

void orc_pt_initial_condition_gravity_waves(void* h, double* u) {
  auto* c = static_cast<PTCase*>(h);
  for (size_t q = 0; q < c->ndofs(); ++q) {
    const auto s = ic_gravity_waves_pt(c->phys.eq, &c->mesh.xy[q * 2]);
    for (int v = 0; v < 5; ++v) u[q * 5 + v] = s[v];
  }
}

void orc_pt_errors_gravity_waves(void* h, const double* u, double* l2, double* linf) {
  auto* c = static_cast<PTCase*>(h);
  errors_2d<5>(c->basis, c->mesh, u,
               [&](const double* x) { return ic_gravity_waves_pt(c->phys.eq, x); }, l2, linf);
}

void orc_pt_rhs(void* h, const double* u, double* du, double t) {
  static_cast<PTCase*>(h)->dg->rhs(u, du, t);
}

double orc_pt_max_dt(void* h, const double* u) { return static_cast<PTCase*>(h)->dg->max_dt(u); }

// SSPRK43 at a fixed CFL (adaptive = false), the last step shortened to t_end
int orc_pt_ssprk43_run(void* h, double* u, double t0, double t_end, double cfl) {
  auto* c = static_cast<PTCase*>(h);
  const size_t N = c->ndofs() * 5;
  std::vector<double> tmp(N), du(N), u0(N);
  double t = t0;
  int steps = 0;
  while (t < t_end) {
    double dt = cfl * c->dg->max_dt(u);
    if (t + dt > t_end) dt = t_end - t;
    ssprk43_step([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, u,
                 tmp.data(), du.data(), u0.data(), N, t, dt);
    t += dt;
    ++steps;
  }
  return steps;
}

double orc_pt_ck_steps(void* h, double* u, double* k, double t, double cfl, int nsteps) {
  auto* c = static_cast<PTCase*>(h);
  const size_t N = c->ndofs() * 5;
  std::vector<double> du(N);
  for (int s = 0; s < nsteps; ++s) {
    const double dt = cfl * c->dg->max_dt(u);
    ck2n54_step([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, u, k,
                du.data(), N, t, dt);
    t += dt;
  }
  return t;
}

// SSPRK43 (scheme 1) / SSPRK33 (scheme 2) steps of the energy 2D, moist,
// potential-temperature and covariant cases (orc::ssp_steps).
double orc_euler2d_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                             double fixed_dt, double t_end) {
  auto* c = static_cast<Euler2DCase*>(h);
  return ssp_steps([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
                   [&](const double* uu) { return c->dg->max_dt(uu); }, [](double*) {}, u,
                   c->ndofs() * 5, t,
                   cfl, nsteps, scheme, fixed_dt, t_end);
}

double orc_moist_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                           double fixed_dt, double t_end) {
  auto* c = static_cast<MoistCase*>(h);
  return ssp_steps([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
                   [&](const double* uu) { return c->dg->max_dt(uu); }, [](double*) {}, u,
                   c->ndofs() * 6, t,
                   cfl, nsteps, scheme, fixed_dt, t_end);
}

double orc_pt_ssp_steps(void* h, double* u, double t, double cfl, int nsteps, int scheme,
                        double fixed_dt, double t_end) {
  auto* c = static_cast<PTCase*>(h);
  return ssp_steps([&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); },
                   [&](const double* uu) { return c->dg->max_dt(uu); }, [](double*) {}, u,
                   c->ndofs() * 5, t,
                   cfl, nsteps, scheme, fixed_dt, t_end);
}

// Adaptive SSPRK43 (orc_time.hpp) on a 2D potential-temperature case from t
// to t_end with optional stops; stats = (accepted, rejected, rhs calls,
// first dt, last dt).  Returns the final time.
double orc_pt_ssprk43_adaptive(void* h, double* u, double t, double t_end, const double* stops,
                               int nstops, double abstol, double reltol, int variant,
                               double* stats) {
  auto* c = static_cast<PTCase*>(h);
  AdaptiveStats st;
  const double tf = ssprk43_adaptive(
      [&](const double* uu, double* dd, double tt) { c->dg->rhs(uu, dd, tt); }, [](double*) {}, u,
      c->ndofs() * 5, t, t_end, stops, nstops, abstol, reltol, variant, &st);
  if (stats) {
    stats[0] = (double)st.accepted;
    stats[1] = (double)st.rejected;
    stats[2] = (double)st.rhs_calls;
    stats[3] = st.dt_first;
    stats[4] = st.dt_last;
  }
  return tf;
}

// the logarithmic mean and its inverse of orc_means.hpp (Trixi's definitions)
double orc_ln_mean(double x, double y) { return ln_mean(x, y); }
double orc_inv_ln_mean(double x, double y) { return inv_ln_mean(x, y); }

double orc_pt_stolarsky(double x, double y, double gamma) {
  PotTemp2D eq;
  eq.gamma = gamma;
  stolarsky_coefficients(gamma, eq.sc);
  return eq.stolarsky(x, y);
}

}  // extern "C"
