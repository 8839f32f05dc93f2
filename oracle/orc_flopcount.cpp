// ORACLE — test infrastructure only: algorithmic operation counts.
//
// The algorithmic work of one DOF·stage is defined as the operation count of
// the oracle's formulas (a restatement of the reference's): this translation
// unit compiles the oracle's own headers a second time with `double` replaced
// by the counting scalar of orc_flop.hpp and runs one CarpenterKennedy2N54 step
// (one max_dt, five right-hand sides with their stage updates) on a given
// state, so every branch (series or logarithm in the logarithmic means,
// upwind side in LMARS, ...) is the one the state takes.  Counts: add (incl.
// sub), mul, div, sqrt, log, exp, pow.  Built single-threaded (the OpenMP
// pragmas of the drivers are ignored).
#include "orc_flop.hpp"

#define ORC_FLOP_COUNTING
#define double orc_count::Flop
#include "orc_basis.hpp"
#include "orc_means.hpp"
#include "orc_dg2d.hpp"
#include "orc_dg3d.hpp"
#include "orc_time.hpp"
#include "orc_energy_phys.hpp"
#include "orc_cov_swe.hpp"
#undef double

using orc_count::Flop;

namespace {

std::vector<Flop> flops(const double* a, size_t n) { return std::vector<Flop>(a, a + n); }

// Phases of one step: 0 volume integral, 1 interface fluxes, 2 boundary
// fluxes, 3 surface integral + apply_jacobian + sources, 4 stage updates
// (k = A k + dt du, u += B k), 5 max_dt (once per step).
constexpr int kPhases = 6;

struct PhaseCounter {
  orc_count::Counts acc[kPhases];
  int cur = -1;
  void to(int phase) {
    if (cur >= 0) {
      const orc_count::Counts& c = orc_count::counts();
      orc_count::Counts& a = acc[cur];
      a.add += c.add; a.mul += c.mul; a.div += c.div; a.sqrt += c.sqrt;
      a.log += c.log; a.exp += c.exp; a.pow += c.pow;
    }
    orc_count::counts() = orc_count::Counts{};
    cur = phase;
  }
  void write(long long* out) {
    to(-1);
    for (int p = 0; p < kPhases; ++p) {
      const orc_count::Counts& a = acc[p];
      long long* o = out + 7 * p;
      o[0] = a.add; o[1] = a.mul; o[2] = a.div; o[3] = a.sqrt;
      o[4] = a.log; o[5] = a.exp; o[6] = a.pow;
    }
  }
};

// One CarpenterKennedy2N54 step (as orc::ck2n54_step) with the phases of each
// right-hand side counted apart.  `volume(e)`, `iface(k)`, `bound(k)`,
// `surf(e)` run one phase on du for the current state.
template <class MaxDt, class Volume, class Iface, class Bound, class Surf>
void counted_step(PhaseCounter& pc, std::vector<Flop>& u, double cfl, int nelem, int nif,
                  int nbd, std::vector<Flop>& du, MaxDt&& max_dt, Volume&& volume, Iface&& iface,
                  Bound&& bound, Surf&& surf) {
  const size_t N = u.size();
  std::vector<Flop> k(N);
  pc.to(5);
  const Flop dt = Flop(cfl) * max_dt();
  for (int s = 0; s < orc::CK2N54::stages; ++s) {
    std::fill(du.begin(), du.end(), Flop(0.0));
    pc.to(0);
    for (int e = 0; e < nelem; ++e) volume(e);
    pc.to(1);
    for (int q = 0; q < nif; ++q) iface(q);
    pc.to(2);
    for (int q = 0; q < nbd; ++q) bound(q);
    pc.to(3);
    for (int e = 0; e < nelem; ++e) surf(e);
    pc.to(4);
    const Flop a = orc::CK2N54::A[s], bb = orc::CK2N54::B[s];
    for (size_t q = 0; q < N; ++q) {
      k[q] = a * k[q] + dt * du[q];
      u[q] = u[q] + bb * k[q];
    }
  }
}

}  // namespace

extern "C" {

// counts[6][7] (phases x operations) of one CK2N54 step at CFL `cfl` of the 3D dry-Euler shell case
// (arrays as orc_euler3d_create takes them), starting from u0.
int orc_count_euler3d_step(int polydeg, int nelem, const double* Ja, const double* invJ,
                           const double* xyz, int nif, const int* if_e, const int* if_f,
                           const int* if_o, int nbd, const int* bd_e, const int* bd_f, double c_p,
                           double c_v, double g, double c_lmars, double omega, double cfl,
                           const double* u0, long long* counts) {
  orc::EnergyPhys3D phys;
  phys.eq = orc::EulerEnergy3D(c_p, c_v, g);
  phys.c_lmars = c_lmars;
  phys.omega = omega;
  const orc::Basis basis = orc::make_lgl_basis(polydeg);
  const int n = basis.n;
  const size_t nodes = (size_t)nelem * n * n * n;
  const std::vector<Flop> ja = flops(Ja, nodes * 9), ij = flops(invJ, nodes),
                          x = flops(xyz, nodes * 3);
  orc::Mesh3D mesh;
  mesh.n = n;
  mesh.nelem = nelem;
  mesh.Ja = ja.data();
  mesh.invJ = ij.data();
  mesh.xyz = x.data();
  for (int q = 0; q < nif; ++q) {
    mesh.if_e0.push_back(if_e[2 * q]);
    mesh.if_e1.push_back(if_e[2 * q + 1]);
    mesh.if_f0.push_back(if_f[2 * q]);
    mesh.if_f1.push_back(if_f[2 * q + 1]);
    mesh.if_orient.push_back(if_o[q]);
  }
  for (int q = 0; q < nbd; ++q) {
    mesh.bd_e.push_back(bd_e[q]);
    mesh.bd_f.push_back(bd_f[q]);
  }
  orc::DG3D<orc::EnergyPhys3D> dg(phys, basis, mesh);
  std::vector<Flop> u = flops(u0, nodes * 6), du(u.size());
  PhaseCounter pc;
  counted_step(pc, u, cfl, nelem, nif, nbd, du, [&] { return dg.max_dt(u.data()); },
               [&](int e) { dg.volume_integral(u.data(), du.data(), e); },
               [&](int q) { dg.interface_flux(u.data(), q); },
               [&](int q) { dg.boundary_flux(u.data(), q); },
               [&](int e) { dg.surface_jacobian_sources(u.data(), du.data(), e, Flop(0.0)); });
  pc.write(counts);
  return 0;
}

// The same for one 2D dry-Euler member on an nx x ny StructuredMesh rectangle
// (periodic in x, slip walls in y), as orc_euler2d_create builds it.
int orc_count_euler2d_step(int polydeg, int nx, int ny, double x0, double x1, double y0,
                           double y1, double c_p, double c_v, double g, double c_lmars,
                           double cfl, const double* u0, long long* counts) {
  orc::EnergyPhys phys;
  phys.eq = orc::EulerEnergy2D(c_p, c_v, g);
  phys.c_lmars = c_lmars;
  const orc::Basis basis = orc::make_lgl_basis(polydeg);
  const orc::Mesh2D mesh = orc::structured_rectangle(basis, nx, ny, Flop(x0), Flop(x1), Flop(y0),
                                                     Flop(y1), true, false);
  orc::DG2D<orc::EnergyPhys> dg(phys, basis, mesh);
  std::vector<Flop> u = flops(u0, (size_t)mesh.nelem * basis.n * basis.n * 5), du(u.size());
  PhaseCounter pc;
  counted_step(pc, u, cfl, mesh.nelem, (int)mesh.if_e0.size(), (int)mesh.bd_e.size(), du,
               [&] { return dg.max_dt(u.data()); },
               [&](int e) { dg.volume_integral(u.data(), du.data(), e); },
               [&](int q) { dg.interface_flux(u.data(), q); },
               [&](int q) { dg.boundary_flux(u.data(), q, Flop(0.0)); },
               [&](int e) { dg.surface_jacobian_sources(u.data(), du.data(), e, Flop(0.0)); });
  pc.write(counts);
  return 0;
}

// The same for one covariant shallow-water mesh (arrays as orc_cov_create
// takes them).
int orc_count_cov_step(int polydeg, int nelem, const double* aux, const double* xyz, int nif,
                       const int* if_e, const int* if_f, const int* if_flip, double g,
                       double omega, int split, int volume, int vol_sym, int vol_nc,
                       int surf_sym, int surf_diss, int surf_nc, double cfl, const double* u0,
                       long long* counts) {
  orc::CovDG c;
  c.eq.g = g;
  c.eq.omega = omega;
  c.eq.split = split != 0;
  c.fx = orc::CovFluxes{volume, vol_sym, vol_nc, surf_sym, surf_diss, surf_nc};
  c.b = orc::make_lgl_basis(polydeg);
  c.n = polydeg + 1;
  c.nelem = nelem;
  const size_t nodes = (size_t)nelem * c.n * c.n;
  c.aux = flops(aux, nodes * 26);
  c.xyz = flops(xyz, nodes * 3);
  for (int q = 0; q < nif; ++q) {
    c.if_e0.push_back(if_e[2 * q]);
    c.if_e1.push_back(if_e[2 * q + 1]);
    c.if_f0.push_back(if_f[2 * q]);
    c.if_f1.push_back(if_f[2 * q + 1]);
    c.if_flip.push_back(if_flip[q]);
  }
  std::vector<Flop> u = flops(u0, nodes * 3), du(u.size());
  if (c.sfv.size() != (size_t)nelem * 4 * c.n * 3) c.sfv.assign((size_t)nelem * 4 * c.n * 3, 0.0);
  PhaseCounter pc;
  counted_step(pc, u, cfl, nelem, nif, 0, du, [&] { return c.max_dt(u.data()); },
               [&](int e) { c.volume(u.data(), du.data(), e); },
               [&](int q) { c.interface(u.data(), q); }, [](int) {},
               [&](int e) { c.surface_jacobian_sources(u.data(), du.data(), e); });
  pc.write(counts);
  return 0;
}

}  // extern "C"
