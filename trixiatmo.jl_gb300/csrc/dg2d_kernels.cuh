// DGSEM kernels for 2D curvilinear quadrilateral meshes (StructuredMesh /
// P4estMesh{2} in Cartesian form), templated on the device physics policy and
// on the number of nodes per direction n.
//
// One stage of the semidiscretization is two launches:
//   k_interface  — prolong2interfaces + calc_interface_flux + calc_boundary_flux:
//                  one thread per (interface or boundary face, face node); writes
//                  the outward numerical flux of both sides into sfv.
//   k_element    — volume integral (flux differencing), surface integral,
//                  apply_jacobian, sources and (optionally) the 2N Runge-Kutta
//                  stage update and the CFL speed reduction, EPB elements per CTA.
// Layouts: u[e][j][i][v] (Trixi's u[v, i, j, e]); Ja[e][j][i][d][c]
// (contravariant_vectors[c, d, i, j, e]); invJ[e][j][i]; sfv[e][face][l][NA].
#pragma once
#include "tag_common.cuh"

namespace tag {

struct BasisDev {
  double Ds[kMaxNodes * kMaxNodes];  // Dsplit[a * n + b] (row a, column b)
  double winv0, winvN;               // 1 / w_0, 1 / w_N
  double Dh[kMaxNodes * kMaxNodes];  // D_hat[a * n + b] (weak form)
};

enum VolumeKind : int { kVolFluxDiff = 0, kVolWeak = 1 };

enum ElementMode : int { kModeRhs = 0, kModeStage = 1 };

struct StageArgs {
  double A, B, C;                 // stage coefficients (StageCoef)
  int ssp, save;                  // SSP (Shu-Osher) form; keep u in k at this stage
  const double* dt;               // per-member dt (device)
  double* max_speed;              // per-member CFL speed accumulator, or null
  const int* member;              // member of each element, or null (one member)
  double c_stage;                 // stage time fraction (stage mode)
  const double* t_member;         // per-member step start time (stage mode)
  double t_rhs;                   // time of an rhs evaluation (rhs mode)
  const double* xy;               // node coordinates (sources), or null
  double* sink;                   // last stage of a 3D step: the new state is also stored
                                  // here (mapped host memory), or null
};

inline void set_stage(StageArgs& st, int scheme, int stage) {
  const StageCoef c = rk_stage(scheme, stage);
  st.A = c.A;
  st.B = c.B;
  st.C = c.C;
  st.ssp = c.ssp;
  st.save = c.save;
  st.c_stage = c.c;
}

// New value of one stage variable from its old value uo and time derivative
// dv; updates the variable's k register (StageCoef's two forms).
TAG_DEV double stage_value(const StageArgs& st, double uo, double* __restrict__ kp, double dt,
                           double dv) {
  if (!st.ssp) {
    const double kn = st.A * *kp + dt * dv;
    *kp = kn;
    return uo + st.B * kn;
  }
  const double w = uo + (st.B * dt) * dv;
  if (st.save) {
    *kp = uo;
    return w;
  }
  return st.A == 0.0 ? w : st.A * *kp + st.C * w;
}

// ---------------------------------------------------------------------------
// Interface + boundary fluxes
// ---------------------------------------------------------------------------
template <class Phys, int n>
__global__ void __launch_bounds__(256) k_interface(
    typename Phys::Params P, const double* __restrict__ u, const double* __restrict__ Ja,
    const double* __restrict__ invJ, const int* __restrict__ if_e, const int* __restrict__ if_f,
    const int* __restrict__ if_flip, int nif, const int* __restrict__ bd_e,
    const int* __restrict__ bd_f, const int* __restrict__ bd_kind, int nbd,
    double* __restrict__ sfv, const double* __restrict__ bvals = nullptr) {
  constexpr int NV = Phys::NV, NA = Phys::NA;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = tid / n, l = tid % n;
  if (k < nif) {
    const int e0 = if_e[2 * k], e1 = if_e[2 * k + 1];
    const int f0 = if_f[2 * k], f1 = if_f[2 * k + 1];
    const int l1 = if_flip[k] ? n - 1 - l : l;
    int i0, j0, i1, j1;
    face_node(f0, l, n, i0, j0);
    face_node(f1, l1, n, i1, j1);
    const size_t q0 = ((size_t)e0 * n + j0) * n + i0;
    const size_t q1 = ((size_t)e1 * n + j1) * n + i1;
    double ul[NV], ur[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      ul[v] = u[q0 * NV + v];
      ur[v] = u[q1 * NV + v];
    }
    const double s = ((invJ[q0] < 0.0) ? -1.0 : 1.0) * ((f0 & 1) ? 1.0 : -1.0);
    const double n1 = s * Ja[q0 * 4 + 2 * (f0 >> 1)];
    const double n2 = s * Ja[q0 * 4 + 2 * (f0 >> 1) + 1];
    double F[NA];
    Phys::surface_flux(P, ul, ur, n1, n2, F);
    double* s0 = sfv + (((size_t)e0 * 4 + f0) * n + l) * NA;
    double* s1 = sfv + (((size_t)e1 * 4 + f1) * n + l1) * NA;
    if constexpr (Phys::kSurfaceNoncons) {
      // nonconservative surface terms, each side with its own state first:
      // primary F + G(ul, ur)/2, secondary -(F + G(ur, ul)/2)
      double G0[NA], G1[NA];
      Phys::surface_noncons(P, ul, ur, n1, n2, G0);
      Phys::surface_noncons(P, ur, ul, n1, n2, G1);
#pragma unroll
      for (int v = 0; v < NA; ++v) {
        s0[v] = F[v] + 0.5 * G0[v];
        s1[v] = -(F[v] + 0.5 * G1[v]);
      }
    } else {
#pragma unroll
      for (int v = 0; v < NA; ++v) {
        s0[v] = F[v];
        s1[v] = -F[v];
      }
    }
    return;
  }
  const int kb = k - nif;
  if (kb < nbd) {
    const int e = bd_e[kb], f = bd_f[kb], kind = bd_kind[kb];
    int i, j;
    face_node(f, l, n, i, j);
    const size_t q = ((size_t)e * n + j) * n + i;
    double ui[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) ui[v] = u[q * NV + v];
    const double sj = (invJ[q] < 0.0) ? -1.0 : 1.0;
    double n1 = sj * Ja[q * 4 + 2 * (f >> 1)];
    double n2 = sj * Ja[q * 4 + 2 * (f >> 1) + 1];
    double F[NA];
    // StructuredMesh walls: normal in the +xi/+eta sense, states ordered by
    // the face parity inside boundary_flux, result turned outward here
    if (kind == TAG_BC_SLIP_WALL_STRUCTURED || kind == TAG_BC_SIMPLE_SLIP_WALL) {
      Phys::boundary_flux(P, ui, n1, n2, f, kind, F);
#pragma unroll
      for (int v = 0; v < NA; ++v) F[v] *= sj;
    } else if (kind == TAG_BC_DIRICHLET) {
      // BoundaryConditionDirichlet (P4estMesh method): the surface flux of the
      // inner and the given state along the outward normal, plus half the
      // nonconservative surface flux
      const double so = (f & 1) ? 1.0 : -1.0;
      double ub[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) ub[v] = bvals[((size_t)kb * n + l) * NV + v];
      Phys::surface_flux(P, ui, ub, so * n1, so * n2, F);
      if constexpr (Phys::kSurfaceNoncons) {
        double G[NA];
        Phys::surface_noncons(P, ui, ub, so * n1, so * n2, G);
#pragma unroll
        for (int v = 0; v < NA; ++v) F[v] += 0.5 * G[v];
      }
    } else {
      const double so = (f & 1) ? 1.0 : -1.0;
      Phys::boundary_flux(P, ui, so * n1, so * n2, f, kind, F);
    }
    double* s0 = sfv + (((size_t)e * 4 + f) * n + l) * NA;
#pragma unroll
    for (int v = 0; v < NA; ++v) s0[v] = F[v];
  }
}

// ---------------------------------------------------------------------------
// Element kernel
// ---------------------------------------------------------------------------
template <class Phys, int n>
struct ElemSmem {
  static constexpr int NV = Phys::NV, NA = Phys::NA, NQ = Phys::NQ;
  static constexpr int nn = n * n;
  static constexpr int npl = n * (n - 1) / 2;   // pairs per line
  static constexpr int P = 2 * n * npl;         // pairs per element
  static constexpr int TPE = (P > nn) ? P : nn; // threads per element
  // doubles per element
  static constexpr int oU = 0;
  static constexpr int oQ = oU + nn * NV;
  static constexpr int oJa = oQ + nn * NQ;
  static constexpr int oC = oJa + nn * 4;        // slots [2][nn][n][NA]
  static constexpr int oL = oC + 2 * nn * n * NA; // CFL speeds [2][nn]
  static constexpr int oS = oL + 2 * nn;          // sources [nn][NA]
  static constexpr int per_elem = oS + (Phys::kHasSources ? nn * NA : 0);
  static size_t bytes(int epb) { return sizeof(double) * (size_t)per_elem * epb + sizeof(BasisDev); }
};

template <class Phys, int n, int MODE, int VOL = kVolFluxDiff>
__global__ void k_element(typename Phys::Params Pp, const BasisDev basis, double* __restrict__ u,
                          double* __restrict__ du, double* __restrict__ kreg,
                          const double* __restrict__ Ja, const double* __restrict__ invJ,
                          const double* __restrict__ sfv, int nelem, int epb, StageArgs st,
                          unsigned* __restrict__ status) {
  using S = ElemSmem<Phys, n>;
  constexpr int NV = Phys::NV, NA = Phys::NA, NQ = Phys::NQ;
  constexpr int nn = S::nn, npl = S::npl;
  extern __shared__ double smem[];
  BasisDev* sb = reinterpret_cast<BasisDev*>(smem);
  double* base = smem + sizeof(BasisDev) / sizeof(double);

  const int e_first = blockIdx.x * epb;
  const int ne = min(epb, nelem - e_first);
  const int nthr = blockDim.x;
  unsigned bad = 0;

  // --- phase 0: basis + element data to shared memory
  for (int t = threadIdx.x; t < (int)(sizeof(BasisDev) / sizeof(double)); t += nthr)
    smem[t] = reinterpret_cast<const double*>(&basis)[t];
  {
    const double* ug = u + (size_t)e_first * nn * NV;
    for (int t = threadIdx.x; t < ne * nn * NV; t += nthr) {
      const int el = t / (nn * NV), r = t % (nn * NV);
      base[el * S::per_elem + S::oU + r] = ug[t];
    }
    // contravariant vectors are kept halved: the pair normal is the sum
    const double* jg = Ja + (size_t)e_first * nn * 4;
    for (int t = threadIdx.x; t < ne * nn * 4; t += nthr) {
      const int el = t / (nn * 4), r = t % (nn * 4);
      base[el * S::per_elem + S::oJa + r] = 0.5 * jg[t];
    }
  }
  __syncthreads();

  // --- phase 1: per-node primitives; zero the self slots
  for (int t = threadIdx.x; t < ne * nn; t += nthr) {
    const int el = t / nn, node = t % nn;
    double* eb = base + el * S::per_elem;
    Phys::node_prims(Pp, eb + S::oU + node * NV, eb + S::oQ + node * NQ, bad);
    const int i = node % n, j = node / n;
    if constexpr (VOL == kVolFluxDiff) {
#pragma unroll
      for (int v = 0; v < NA; ++v) {
        eb[S::oC + ((0 * nn + node) * n + i) * NA + v] = 0.0;
        eb[S::oC + ((1 * nn + node) * n + j) * NA + v] = 0.0;
      }
    }
  }
  __syncthreads();

  // per element: can a node pair leave the series range of the logarithmic
  // means?  If so, the per-node logarithms are computed (once per node)
  if (Phys::kNodeLogs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = (nthr + 31) >> 5;
    for (int el = warp; el < ne; el += nwarps) {
      const bool logs = element_needs_logs(base + el * S::per_elem + S::oQ, nn, NQ, Phys::kRho,
                                           Phys::kBeta, kLogMeanRange);
      if (lane == 0) base[el * S::per_elem + S::oL] = logs ? 1.0 : 0.0;
    }
    __syncthreads();
  }
  if (Phys::kNodeLogs) for (int t = threadIdx.x; t < ne * nn; t += nthr) {
    const int el = t / nn, node = t % nn;
    double* eb = base + el * S::per_elem;
    double* q = eb + S::oQ + node * NQ;
    if (eb[S::oL] != 0.0) {
      q[Phys::kLogRho] = log(q[Phys::kRho]);
      q[Phys::kLogBeta] = log(q[Phys::kBeta]);
    } else {
      q[Phys::kLogRho] = 0.0;
      q[Phys::kLogBeta] = 0.0;
    }
  }
  if (Phys::kNodeLogs) __syncthreads();

  // --- phase 2 (weak form): contravariant fluxes per node,
  //     F~_d = f(u, Ja^d) into slot 0 of direction d
  if constexpr (VOL == kVolWeak) {
    for (int t = threadIdx.x; t < ne * nn * 2; t += nthr) {
      const int el = t / (nn * 2), r = t % (nn * 2);
      const int node = r >> 1, d = r & 1;
      double* eb = base + el * S::per_elem;
      const double* ja = eb + S::oJa + node * 4 + 2 * d;  // halved
      double F[NA];
      Phys::flux(Pp, eb + S::oU + node * NV, 2.0 * ja[0], 2.0 * ja[1], F);
#pragma unroll
      for (int v = 0; v < NA; ++v) eb[S::oC + ((d * nn + node) * n + 0) * NA + v] = F[v];
    }
  }
  // --- phase 2: one thread per symmetric pair (a < b) on a line, ordered by
  //     direction first, so that the warps of a CTA with several elements
  //     hold pairs of one direction (the logarithmic means' forms then agree
  //     across a warp: horizontal pairs of a stratified atmosphere take the
  //     short series, vertical ones the longer)
  if constexpr (VOL == kVolFluxDiff) for (int t = threadIdx.x; t < ne * S::P; t += nthr) {
    const int per_dir = ne * n * npl;
    const int d = t / per_dir, rd = t % per_dir;
    const int el = rd / (n * npl), r = rd % (n * npl);
    const int line = r / npl;
    int q = r % npl, a = 0;
    while (q >= n - 1 - a) { q -= n - 1 - a; ++a; }
    const int b = a + 1 + q;
    const int na_ = d == 0 ? line * n + a : a * n + line;
    const int nb_ = d == 0 ? line * n + b : b * n + line;
    double* eb = base + el * S::per_elem;
    const double* ja_a = eb + S::oJa + na_ * 4 + 2 * d;
    const double* ja_b = eb + S::oJa + nb_ * 4 + 2 * d;
    const double n1 = ja_a[0] + ja_b[0];
    const double n2 = ja_a[1] + ja_b[1];
    double Fa[NA], Fb[NA];
    Phys::volume_pair(Pp, eb + S::oQ + na_ * NQ, eb + S::oQ + nb_ * NQ, n1, n2, Fa, Fb);
    // raw pair fluxes; the D_split weights are applied in the slot reduction
    double* ca = eb + S::oC + ((d * nn + na_) * n + b) * NA;
    double* cb = eb + S::oC + ((d * nn + nb_) * n + a) * NA;
#pragma unroll
    for (int v = 0; v < NA; ++v) {
      ca[v] = Fa[v];
      cb[v] = Fb[v];
    }
  }
  // --- phase 2b: sources per node (from the state before the update)
  if constexpr (Phys::kHasSources) {
    for (int t = threadIdx.x; t < ne * nn; t += nthr) {
      const int el = t / nn, node = t % nn;
      const int e = e_first + el;
      double* eb = base + el * S::per_elem;
      double tt = st.t_rhs;
      if (MODE == kModeStage) {
        const int m = st.member ? st.member[e] : 0;
        tt = st.t_member[m] + st.c_stage * st.dt[m];
      }
      const double* x = st.xy ? st.xy + ((size_t)e * nn + node) * 2 : nullptr;
      Phys::source(Pp, eb + S::oU + node * NV, x, tt, eb + S::oS + node * NA);
    }
  }
  __syncthreads();

  // --- phase 3: per (node, variable): slot sums, surface integral, Jacobian,
  //     sources, stage update
  for (int t = threadIdx.x; t < ne * nn * NA; t += nthr) {
    const int el = t / (nn * NA), r = t % (nn * NA);
    const int node = r / NA, v = r % NA;
    const int i = node % n, j = node / n;
    const int e = e_first + el;
    double* eb = base + el * S::per_elem;
    double acc = 0.0;
    if constexpr (VOL == kVolFluxDiff) {
#pragma unroll
      for (int b = 0; b < n; ++b)
        acc = fma(sb->Ds[i * n + b], eb[S::oC + ((0 * nn + node) * n + b) * NA + v], acc);
#pragma unroll
      for (int b = 0; b < n; ++b)
        acc = fma(sb->Ds[j * n + b], eb[S::oC + ((1 * nn + node) * n + b) * NA + v], acc);
    } else {
      // weak form: du(i, j) = sum_b D_hat[i, b] F~_1(b, j) + D_hat[j, b] F~_2(i, b)
#pragma unroll
      for (int b = 0; b < n; ++b)
        acc = fma(sb->Dh[i * n + b], eb[S::oC + ((0 * nn + j * n + b) * n + 0) * NA + v], acc);
#pragma unroll
      for (int b = 0; b < n; ++b)
        acc = fma(sb->Dh[j * n + b], eb[S::oC + ((1 * nn + b * n + i) * n + 0) * NA + v], acc);
    }
    const double* se = sfv + (size_t)e * 4 * n * NA;
    if (i == 0) acc += se[(0 * n + j) * NA + v] * sb->winv0;
    if (i == n - 1) acc += se[(1 * n + j) * NA + v] * sb->winvN;
    if (j == 0) acc += se[(2 * n + i) * NA + v] * sb->winv0;
    if (j == n - 1) acc += se[(3 * n + i) * NA + v] * sb->winvN;
    const size_t gq = (size_t)e * nn + node;
    double dv = acc * (-invJ[gq]);
    if constexpr (Phys::kHasSources) dv += eb[S::oS + node * NA + v];
    if (not_finite(dv)) bad |= TAG_S_NAN;
    if (MODE == kModeRhs) {
      du[gq * NV + v] = dv;
    } else {
      const size_t kq = gq * NA + v;
      const double dt = st.dt[st.member ? st.member[e] : 0];
      const double un = stage_value(st, eb[S::oU + node * NV + v], kreg + kq, dt, dv);
      eb[S::oU + node * NV + v] = un;
      u[gq * NV + v] = un;
    }
  }
  if constexpr (MODE == kModeRhs && NV > NA) {
    // passive variables have zero time derivative
    for (int t = threadIdx.x; t < ne * nn * (NV - NA); t += nthr) {
      const int el = t / (nn * (NV - NA)), r = t % (nn * (NV - NA));
      const int node = r / (NV - NA), v = NA + r % (NV - NA);
      du[((size_t)(e_first + el) * nn + node) * NV + v] = 0.0;
    }
  }

  // --- phase 4 (last stage of a step): CFL speeds of the updated state
  if (MODE == kModeStage && st.max_speed != nullptr) {
    __syncthreads();
    // the step's result to the registered sink (host memory over the host
    // link): each element's new state is one contiguous block in shared
    // memory and in the sink, stored by consecutive threads at consecutive
    // addresses
    if (st.sink != nullptr) {
      double* o = st.sink + (size_t)e_first * nn * NV;
      for (int t = threadIdx.x; t < ne * nn * NV; t += nthr) {
        const int el = t / (nn * NV), r = t % (nn * NV);
        o[t] = base[el * S::per_elem + S::oU + r];
      }
    }
    for (int t = threadIdx.x; t < ne * nn; t += nthr) {
      const int el = t / nn, node = t % nn;
      double* eb = base + el * S::per_elem;
      double l1, l2;
      Phys::max_speeds(Pp, eb + S::oU + node * NV, l1, l2);
      const double* ja = eb + S::oJa + node * 4;  // halved
      const double ij = 2.0 * fabs(invJ[(size_t)(e_first + el) * nn + node]);
      eb[S::oL + node] = fabs(ja[0] * l1 + ja[1] * l2) * ij;
      eb[S::oL + nn + node] = fabs(ja[2] * l1 + ja[3] * l2) * ij;
    }
    __syncthreads();
    for (int el = threadIdx.x; el < ne; el += nthr) {
      double* eb = base + el * S::per_elem;
      double m1 = 0.0, m2 = 0.0;
      for (int node = 0; node < nn; ++node) {
        m1 = fmax(m1, eb[S::oL + node]);
        m2 = fmax(m2, eb[S::oL + nn + node]);
      }
      eb[S::oL] = m1 + m2;  // element's scaled speed (slot 0 reused)
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      // one atomic per run of consecutive elements of the same member
      int cur = st.member ? st.member[e_first] : 0;
      double run = 0.0;
      for (int el = 0; el < ne; ++el) {
        const int m = st.member ? st.member[e_first + el] : 0;
        if (m != cur) {
          atomic_max_nonneg(st.max_speed + cur, run);
          cur = m;
          run = 0.0;
        }
        run = fmax(run, base[el * S::per_elem + S::oL]);
      }
      atomic_max_nonneg(st.max_speed + cur, run);
    }
  }
  if (bad) atomicOr(status, bad);
}

// ---------------------------------------------------------------------------
// CFL speed reduction of a state (Trixi.max_dt) and per-step scalars
// ---------------------------------------------------------------------------
// Tile of k_max_speed: EPB elements per CTA, one thread per node.
template <int n>
struct MaxSpeedTile {
  static constexpr int nn = n * n;
  static constexpr int EPB = nn >= 256 ? 1 : 256 / nn;
  static constexpr int T = EPB * nn;
};

// One thread per node: the node's two contravariant speeds |Ja^d . lambda| / J
// go to shared memory; per element the maxima over its nodes are summed
// (Trixi's max_lambda1 + max_lambda2); one atomic per CTA when all its
// elements belong to one member, else one per element.
template <class Phys, int n>
__global__ void __launch_bounds__(MaxSpeedTile<n>::T) k_max_speed(
    typename Phys::Params Pp, const double* __restrict__ u, const double* __restrict__ Ja,
    const double* __restrict__ invJ, int nelem, const int* __restrict__ member,
    double* __restrict__ max_speed) {
  using K = MaxSpeedTile<n>;
  constexpr int NV = Phys::NV, nn = n * n;
  __shared__ double s1[K::T], s2[K::T], se[K::EPB];
  const int e0 = blockIdx.x * K::EPB;
  const int t = threadIdx.x;
  double a = 0.0, b = 0.0;
  if (e0 + t / nn < nelem) {
    const size_t q = (size_t)e0 * nn + t;
    double l1, l2;
    Phys::max_speeds(Pp, u + q * NV, l1, l2);
    const double* ja = Ja + q * 4;
    const double ij = fabs(invJ[q]);
    a = fabs(ja[0] * l1 + ja[1] * l2) * ij;
    b = fabs(ja[2] * l1 + ja[3] * l2) * ij;
  }
  s1[t] = a;
  s2[t] = b;
  __syncthreads();
  if (t < K::EPB) {
    double m1 = 0.0, m2 = 0.0;
    for (int k = 0; k < nn; ++k) {
      m1 = fmax(m1, s1[t * nn + k]);
      m2 = fmax(m2, s2[t * nn + k]);
    }
    se[t] = m1 + m2;
  }
  __syncthreads();
  if (t == 0) {
    const int ne = min(K::EPB, nelem - e0);
    const int m0 = member ? member[e0] : 0;
    bool uniform = true;
    double mx = 0.0;
    for (int k = 0; k < ne; ++k) {
      if (member && member[e0 + k] != m0) uniform = false;
      mx = fmax(mx, se[k]);
    }
    if (uniform) {
      atomic_max_nonneg(max_speed + m0, mx);
    } else {
      for (int k = 0; k < ne; ++k) atomic_max_nonneg(max_speed + member[e0 + k], se[k]);
    }
  }
}

// Start of an RK step, per member: t += previous dt; dt = cfl * 2 / (n *
// max_speed) (or the fixed dt); reset the speed accumulator for the step's
// last stage.  max_speed starts at nextfloat(0) like the reference.
static __global__ void k_begin_step(MemberScalars s, const StepCtl* ctl, int nmembers, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmembers) return;
  s.t[m] += s.dt[m];
  const double ms = s.max_speed[m] > 0.0 ? s.max_speed[m] : 4.9406564584124654e-324;
  s.dt[m] = ctl->fixed_dt > 0.0 ? ctl->fixed_dt : ctl->cfl * (2.0 / (n * ms));
  s.max_speed[m] = 0.0;
}

}  // namespace tag
