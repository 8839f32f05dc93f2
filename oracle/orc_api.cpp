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
#include "orc_time.hpp"

namespace orc {

struct EnergyPhys {
  using State = EulerEnergy2D::State;
  static constexpr int nv = 5;
  static constexpr bool has_noncons = true;
  static constexpr bool has_sources = false;
  EulerEnergy2D eq;
  double c_lmars = 340.0;
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_ranocha(a, b, n);
  }
  State volume_noncons(const State& a, const State& b, const double* n) const {
    return eq.noncons_waruszewski(a, b, n);
  }
  State surface_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_lmars(a, b, n, c_lmars);
  }
  State surface_noncons(const State&, const State&, const double*) const { return State{}; }
  State bc_structured(const State& ui, const double* n, int direction) const {
    return eq.slip_wall_structured(ui, n, direction, c_lmars);
  }
  State bc_normal(const State& ui, const double* n) const {
    return eq.slip_wall_normal(ui, n, c_lmars);
  }
  State source(const State&, const double*, double) const { return State{}; }
  void max_abs_speeds(const State& u, double& l1, double& l2) const { eq.max_abs_speeds(u, l1, l2); }
};

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

struct EnergyPhys3D {
  using State = EulerEnergy3D::State;
  static constexpr int nv = 6;
  static constexpr bool has_noncons = true;
  static constexpr bool has_sources = true;
  EulerEnergy3D eq;
  double c_lmars = 340.0, omega = 0.0;
  State volume_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_ranocha(a, b, n);
  }
  State volume_noncons(const State& a, const State& b, const double* n) const {
    return eq.noncons_waruszewski(a, b, n);
  }
  State surface_flux(const State& a, const State& b, const double* n) const {
    return eq.flux_lmars(a, b, n, c_lmars);
  }
  State surface_noncons(const State&, const State&, const double*) const { return State{}; }
  State bc_normal(const State& ui, const double* n) const { return eq.slip_wall_normal(ui, n, c_lmars); }
  State source(const State& u, const double*, double) const { return eq.coriolis(u, omega); }
  void max_abs_speeds(const State& u, double* l) const { eq.max_abs_speeds(u, l); }
};

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

}  // extern "C"
