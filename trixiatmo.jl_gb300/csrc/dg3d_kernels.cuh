// DGSEM kernels for 3D curvilinear hexahedral meshes (P4estMesh{3} in
// Cartesian form), templated on the device physics policy and on the number of
// nodes per direction n.  One stage = k_interface3d + k_element3d.
//
// Volume integral schedule: every line of n nodes has n(n-1)/2 symmetric
// pairs; they are evaluated in round-robin order (the circle method of
// tournament scheduling) so that within a round the pairs of a line touch
// disjoint nodes.  Each round therefore adds D_split-weighted pair fluxes
// straight into per-direction node accumulators without atomics, and the
// summation order is fixed (bitwise reproducible).  A warp owns whole lines,
// so the rounds need only warp-level synchronisation.
// Layouts: u[e][k][j][i][v]; Ja[e][k][j][i][d][c]; invJ[e][k][j][i];
// sfv[e][face][l2][l1][NA].
#pragma once
#include "dg2d_kernels.cuh"

namespace tag {

TAG_DEV void face_node3d(int f, int l1, int l2, int n, int& i, int& j, int& k) {
  const int end = (f & 1) ? n - 1 : 0;
  const int d = f >> 1;
  i = d == 0 ? end : l1;
  j = d == 0 ? l1 : (d == 1 ? end : l2);
  k = d == 2 ? end : l2;
}

TAG_DEV void orient_map(int o, int l1, int l2, int n, int& s1, int& s2) {
  int a = (o & 1) ? l2 : l1, b = (o & 1) ? l1 : l2;
  if (o & 2) a = n - 1 - a;
  if (o & 4) b = n - 1 - b;
  s1 = a;
  s2 = b;
}

// Pair (a, b) of line-slot s in round r of the circle method on m = n rounded
// up to even positions; returns false for the bye of odd n.
TAG_DEV bool round_robin_pair(int n, int r, int s, int& a, int& b) {
  const int m = (n + 1) & ~1;
  const int mm = m - 1;
  int x, y;
  if (s == 0) {
    x = mm;
    y = r;
  } else {
    x = (r + s) % mm;
    y = (r - s + mm) % mm;
  }
  if (x >= n || y >= n) return false;
  a = min(x, y);
  b = max(x, y);
  return true;
}

template <class Phys, int n>
__global__ void __launch_bounds__(256) k_interface3d(
    typename Phys::Params P, const double* __restrict__ u, const double* __restrict__ Ja,
    const double* __restrict__ invJ, const int* __restrict__ if_e, const int* __restrict__ if_f,
    const int* __restrict__ if_o, int nif, const int* __restrict__ bd_e,
    const int* __restrict__ bd_f, int nbd, double* __restrict__ sfv) {
  constexpr int NV = Phys::NV, NA = Phys::NA, nn = n * n;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int kf = tid / nn, r = tid % nn;
  const int l1 = r % n, l2 = r / n;
  if (kf < nif) {
    const int e0 = if_e[2 * kf], e1 = if_e[2 * kf + 1];
    const int f0 = if_f[2 * kf], f1 = if_f[2 * kf + 1];
    int s1, s2, i0, j0, k0, i1, j1, k1;
    orient_map(if_o[kf], l1, l2, n, s1, s2);
    face_node3d(f0, l1, l2, n, i0, j0, k0);
    face_node3d(f1, s1, s2, n, i1, j1, k1);
    const size_t q0 = (((size_t)e0 * n + k0) * n + j0) * n + i0;
    const size_t q1 = (((size_t)e1 * n + k1) * n + j1) * n + i1;
    double ul[NV], ur[NV], nrm[3];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      ul[v] = u[q0 * NV + v];
      ur[v] = u[q1 * NV + v];
    }
    const double s = ((invJ[q0] < 0.0) ? -1.0 : 1.0) * ((f0 & 1) ? 1.0 : -1.0);
#pragma unroll
    for (int c = 0; c < 3; ++c) nrm[c] = s * Ja[(q0 * 3 + (f0 >> 1)) * 3 + c];
    double F[NA];
    Phys::surface_flux(P, ul, ur, nrm, F);
    double* a0 = sfv + ((((size_t)e0 * 6 + f0) * n + l2) * n + l1) * NA;
    double* a1 = sfv + ((((size_t)e1 * 6 + f1) * n + s2) * n + s1) * NA;
#pragma unroll
    for (int v = 0; v < NA; ++v) {
      a0[v] = F[v];
      a1[v] = -F[v];
    }
    return;
  }
  const int kb = kf - nif;
  if (kb < nbd) {
    const int e = bd_e[kb], f = bd_f[kb];
    int i, j, k;
    face_node3d(f, l1, l2, n, i, j, k);
    const size_t q = (((size_t)e * n + k) * n + j) * n + i;
    double ui[NV], nrm[3];
#pragma unroll
    for (int v = 0; v < NV; ++v) ui[v] = u[q * NV + v];
    const double s = ((invJ[q] < 0.0) ? -1.0 : 1.0) * ((f & 1) ? 1.0 : -1.0);
#pragma unroll
    for (int c = 0; c < 3; ++c) nrm[c] = s * Ja[(q * 3 + (f >> 1)) * 3 + c];
    double F[NA];
    Phys::boundary_flux(P, ui, nrm, F);
    double* a0 = sfv + ((((size_t)e * 6 + f) * n + l2) * n + l1) * NA;
#pragma unroll
    for (int v = 0; v < NA; ++v) a0[v] = F[v];
  }
}

template <class Phys, int n>
struct ElemSmem3D {
  static constexpr int NV = Phys::NV, NA = Phys::NA, NQ = Phys::NQ;
  static constexpr int nn = n * n, nnn = n * n * n;
  static constexpr int S = ((n + 1) & ~1) / 2;     // pair slots per line and round (incl. a bye)
  static constexpr int R = ((n + 1) & ~1) - 1;     // rounds
  static constexpr int LPW = 32 / S;               // whole lines per warp
  static constexpr int WPE = (3 * nn + LPW - 1) / LPW;  // warps per element in the pair phase
  static constexpr int TPE = (32 * WPE > nnn) ? 32 * WPE : nnn;  // threads per element
  static constexpr int oU = 0;
  static constexpr int oQ = oU + nnn * NV;
  static constexpr int oJa = oQ + nnn * NQ;       // contravariant vectors as stored
  static constexpr int oA = oJa + nnn * 9;        // accumulators [3][nnn][NA]
  static constexpr int oL = oA + 3 * nnn * NA;    // CFL speeds [3][nnn]
  static constexpr int per_elem = oL + 3 * nnn;
  static size_t bytes(int epb) { return sizeof(double) * (size_t)per_elem * epb + sizeof(BasisDev); }
};

template <class Phys, int n, int MODE>
__global__ void k_element3d(typename Phys::Params Pp, const BasisDev basis, double* __restrict__ u,
                            double* __restrict__ du, double* __restrict__ kreg,
                            const double* __restrict__ Ja, const double* __restrict__ invJ,
                            const double* __restrict__ sfv, int nelem, int epb, StageArgs st,
                            unsigned* __restrict__ status) {
  using S = ElemSmem3D<Phys, n>;
  constexpr int NV = Phys::NV, NA = Phys::NA, NQ = Phys::NQ;
  constexpr int nn = S::nn, nnn = S::nnn;
  extern __shared__ double smem[];
  BasisDev* sb = reinterpret_cast<BasisDev*>(smem);
  double* base = smem + sizeof(BasisDev) / sizeof(double);
  const int e_first = blockIdx.x * epb;
  const int ne = min(epb, nelem - e_first);
  const int nthr = blockDim.x;
  unsigned bad = 0;

  // The pair normal is ja_a + ja_b, twice the average the two-point fluxes
  // take; every volume pair flux is linear in the normal, so D_split is halved
  // instead (both scalings by 2 are exact: the same bits as averaging).
  for (int t = threadIdx.x; t < (int)(sizeof(BasisDev) / sizeof(double)); t += nthr) {
    const double b = reinterpret_cast<const double*>(&basis)[t];
    smem[t] = t < kMaxNodes * kMaxNodes ? 0.5 * b : b;
  }
  {
    const double* ug = u + (size_t)e_first * nnn * NV;
    for (int t = threadIdx.x; t < ne * nnn * NV; t += nthr) {
      const int el = t / (nnn * NV), r = t % (nnn * NV);
      base[el * S::per_elem + S::oU + r] = ug[t];
    }
    const double* jg = Ja + (size_t)e_first * nnn * 9;
    for (int t = threadIdx.x; t < ne * nnn * 9; t += nthr) {
      const int el = t / (nnn * 9), r = t % (nnn * 9);
      base[el * S::per_elem + S::oJa + r] = jg[t];
    }
  }
  __syncthreads();

  // per-node quantities; zero the accumulators
  for (int t = threadIdx.x; t < ne * nnn; t += nthr) {
    const int el = t / nnn, node = t % nnn;
    double* eb = base + el * S::per_elem;
    Phys::node_prims(Pp, eb + S::oU + node * NV, eb + S::oQ + node * NQ, bad);
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int v = 0; v < NA; ++v) eb[S::oA + (d * nnn + node) * NA + v] = 0.0;
  }
  __syncthreads();

  // per element: can a node pair leave the series range of the logarithmic
  // means?  If so, the per-node logarithms are computed (once per node)
  if (Phys::kNodeLogs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = (nthr + 31) >> 5;
    for (int el = warp; el < ne; el += nwarps) {
      const bool logs = element_needs_logs(base + el * S::per_elem + S::oQ, nnn, NQ, Phys::kRho,
                                           Phys::kBeta, Phys::kLogRange);
      if (lane == 0) base[el * S::per_elem + S::oL] = logs ? 1.0 : 0.0;
    }
    __syncthreads();
  }
  if (Phys::kNodeLogs) for (int t = threadIdx.x; t < ne * nnn; t += nthr) {
    const int el = t / nnn, node = t % nnn;
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

  // volume integral: each warp takes whole lines (LPW lines of one element,
  // S slots each) and runs their R rounds with only __syncwarp between rounds:
  // the pairs of one line meet the same nodes only across rounds, the lines of
  // one direction are disjoint, and each direction has its own accumulators.
  // A node's contributions arrive in round order whatever the launch shape.
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = nthr >> 5;
    const int lw = lane / S::S, slot = lane % S::S;
    for (int task = warp; task < ne * S::WPE; task += nwarps) {
      const int el = task / S::WPE;
      const int lg = (task % S::WPE) * S::LPW + lw;  // d * nn + line
      const bool on = lw < S::LPW && lg < 3 * nn;
      const int d = lg / nn, line = lg % nn;
      // line = p1 + n * p2 over the two other directions (ascending)
      const int p1 = line % n, p2 = line / n;
      double* eb = base + el * S::per_elem;
      for (int r = 0; r < S::R; ++r) {
        int a, b;
        if (on && round_robin_pair(n, r, slot, a, b)) {
          int na_, nb_;
          if (d == 0) {
            na_ = (p2 * n + p1) * n + a;
            nb_ = (p2 * n + p1) * n + b;
          } else if (d == 1) {
            na_ = (p2 * n + a) * n + p1;
            nb_ = (p2 * n + b) * n + p1;
          } else {
            na_ = (a * n + p2) * n + p1;
            nb_ = (b * n + p2) * n + p1;
          }
          const double* ja_a = eb + S::oJa + na_ * 9 + 3 * d;
          const double* ja_b = eb + S::oJa + nb_ * 9 + 3 * d;
          const double nrm[3] = {ja_a[0] + ja_b[0], ja_a[1] + ja_b[1], ja_a[2] + ja_b[2]};
          double Fa[NA], Fb[NA];
          Phys::volume_pair(Pp, eb + S::oQ + na_ * NQ, eb + S::oQ + nb_ * NQ, nrm, Fa, Fb);
          const double dab = sb->Ds[a * n + b], dba = sb->Ds[b * n + a];
          double* ca = eb + S::oA + (d * nnn + na_) * NA;
          double* cb = eb + S::oA + (d * nnn + nb_) * NA;
#pragma unroll
          for (int v = 0; v < NA; ++v) {
            ca[v] = fma(dab, Fa[v], ca[v]);
            cb[v] = fma(dba, Fb[v], cb[v]);
          }
        }
        __syncwarp();
      }
      // surface integral: the line's two end nodes lie on the element's faces
      // 2d and 2d+1; their surface fluxes (face-local index (p1, p2)) are
      // added to the same direction's accumulators, here rather than in the
      // per-node phase where they would be a divergent branch
      if (on) {
        for (int end = slot; end < 2; end += S::S) {
          const int a = end == 0 ? 0 : n - 1;
          const int nd = d == 0 ? (p2 * n + p1) * n + a
                                : (d == 1 ? (p2 * n + a) * n + p1 : (a * n + p2) * n + p1);
          const double w = end == 0 ? sb->winv0 : sb->winvN;
          const double* sf =
              sfv + ((((size_t)(e_first + el) * 6 + 2 * d + end) * n + p2) * n + p1) * NA;
          double* c = eb + S::oA + (d * nnn + nd) * NA;
#pragma unroll
          for (int v = 0; v < NA; ++v) c[v] = fma(sf[v], w, c[v]);
        }
      }
    }
  }
  __syncthreads();

  // per (node, variable): direction sums (surface integral included),
  // Jacobian, sources, stage update
  for (int t = threadIdx.x; t < ne * nnn * NA; t += nthr) {
    const int el = t / (nnn * NA), r = t % (nnn * NA);
    const int node = r / NA, v = r % NA;
    const int e = e_first + el;
    double* eb = base + el * S::per_elem;
    const double acc = eb[S::oA + (0 * nnn + node) * NA + v] +
                       eb[S::oA + (1 * nnn + node) * NA + v] + eb[S::oA + (2 * nnn + node) * NA + v];
    const size_t gq = (size_t)e * nnn + node;
    const double dv = acc * (-invJ[gq]) + Phys::source(Pp, eb + S::oU + node * NV, v);
    if (not_finite(dv)) bad |= TAG_S_NAN;
    if (MODE == kModeRhs) {
      du[gq * NV + v] = dv;
    } else {
      const size_t kq = gq * NA + v;
      const double dt = st.dt[st.member ? st.member[e] : 0];
      const double un = stage_value(st, eb[S::oU + node * NV + v], kreg + kq, dt, dv);
      // all reads of this node's old state (the Coriolis source) precede the
      // barrier below; write the new value to global memory now and to
      // shared memory after it
      u[gq * NV + v] = un;
      eb[S::oA + node * NA + v] = un;  // stage the new value (direction-0 slot is free)
    }
  }
  if (MODE == kModeRhs) {
    for (int t = threadIdx.x; t < ne * nnn * (NV - NA); t += nthr) {
      const int el = t / (nnn * (NV - NA)), r = t % (nnn * (NV - NA));
      const int node = r / (NV - NA), v = NA + r % (NV - NA);
      du[((size_t)(e_first + el) * nnn + node) * NV + v] = 0.0;
    }
  }
  if (MODE == kModeStage && st.max_speed != nullptr) {
    __syncthreads();
    for (int t = threadIdx.x; t < ne * nnn; t += nthr) {
      const int el = t / nnn, node = t % nnn;
      double* eb = base + el * S::per_elem;
      double un[NV];
#pragma unroll
      for (int v = 0; v < NA; ++v) un[v] = eb[S::oA + node * NA + v];
#pragma unroll
      for (int v = NA; v < NV; ++v) un[v] = eb[S::oU + node * NV + v];
      double lam[3];
      Phys::max_speeds(Pp, un, lam);
      const double* ja = eb + S::oJa + node * 9;
      const double ij = fabs(invJ[(size_t)(e_first + el) * nnn + node]);
#pragma unroll
      for (int d = 0; d < 3; ++d)
        eb[S::oL + d * nnn + node] =
            fabs(ja[3 * d] * lam[0] + ja[3 * d + 1] * lam[1] + ja[3 * d + 2] * lam[2]) * ij;
    }
    __syncthreads();
    // the step's result to the registered sink (host memory over the host
    // link): each element's state is one contiguous block, stored by
    // consecutive threads at consecutive addresses
    if (st.sink != nullptr) {
      double* o = st.sink + (size_t)e_first * nnn * NV;
      for (int t = threadIdx.x; t < ne * nnn * NV; t += nthr) {
        const int el = t / (nnn * NV), r = t % (nnn * NV);
        const int node = r / NV, v = r % NV;
        const double* eb = base + el * S::per_elem;
        o[t] = v < NA ? eb[S::oA + node * NA + v] : eb[S::oU + node * NV + v];
      }
    }
    // one warp per element: the per-direction maxima over its nodes on the
    // integer pipe (the speeds are non-negative, and the bit patterns of
    // non-negative doubles order like their values), then summed
    {
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = nthr >> 5;
      for (int el = warp; el < ne; el += nwarps) {
        double* eb = base + el * S::per_elem;
        long long m[3] = {0, 0, 0};
        for (int node = lane; node < nnn; node += 32)
#pragma unroll
          for (int d = 0; d < 3; ++d)
            m[d] = max(m[d], __double_as_longlong(eb[S::oL + d * nnn + node]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
          for (int d = 0; d < 3; ++d) m[d] = max(m[d], __shfl_xor_sync(0xffffffffu, m[d], o));
        if (lane == 0)
          eb[S::oL] = __longlong_as_double(m[0]) + __longlong_as_double(m[1]) +
                      __longlong_as_double(m[2]);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int cur = st.member ? st.member[e_first] : 0;
      double run = 0.0;
      for (int el = 0; el < ne; ++el) {
        const int mb = st.member ? st.member[e_first + el] : 0;
        if (mb != cur) {
          atomic_max_nonneg(st.max_speed + cur, run);
          cur = mb;
          run = 0.0;
        }
        run = fmax(run, base[el * S::per_elem + S::oL]);
      }
      atomic_max_nonneg(st.max_speed + cur, run);
    }
  }
  if (bad) atomicOr(status, bad);
}

// One warp per element (a 3D element has up to 512 nodes): the lanes stride
// over the nodes, the per-direction maxima meet by shuffles, and lane 0 adds
// the element's value into its member's running maximum.  Max is exact, so the
// result does not depend on the order.  blockDim is a multiple of 32.  With
// copy_to the kernel also stores every value it reads there: a state read
// from mapped host memory lands in device memory with its CFL speeds reduced
// in the same pass.
template <class Phys, int n>
__global__ void k_max_speed3d(typename Phys::Params Pp, const double* __restrict__ u,
                              const double* __restrict__ Ja, const double* __restrict__ invJ,
                              int nelem, const int* __restrict__ member,
                              double* __restrict__ max_speed, double* __restrict__ copy_to) {
  constexpr int NV = Phys::NV, nnn = n * n * n;
  const int lane = threadIdx.x & 31;
  const int e = (int)(((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (e >= nelem) return;  // warp-uniform
  double m[3] = {0.0, 0.0, 0.0};
  // chunks of 32 nodes; every lane takes part in each chunk (the shuffles of
  // the copying path need the whole warp), lanes past the last node idle
  for (int c0 = 0; c0 < nnn; c0 += 32) {
    const int node = c0 + lane;
    const bool on = node < nnn;
    const size_t q = (size_t)e * nnn + node;
    double un[NV];
    if (copy_to) {
      // the chunk's nodes are consecutive NV-double records: read and store
      // them lane-contiguously (the host link serves whole lines), then hand
      // each lane its node's values by shuffles
      const size_t base = ((size_t)e * nnn + c0) * NV;
      const int avail = min(32, nnn - c0) * NV;
      double r[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        const int i = lane + 32 * k;
        r[k] = i < avail ? u[base + i] : 0.0;
        if (i < avail) copy_to[base + i] = r[k];
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const int i = lane * NV + v, src = i & 31, reg = i >> 5;
        double got = 0.0;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const double x = __shfl_sync(0xffffffffu, r[k], src);
          if (k == reg) got = x;
        }
        un[v] = got;
      }
    } else if (on) {
#pragma unroll
      for (int v = 0; v < NV; ++v) un[v] = u[q * NV + v];
    }
    if (!on) continue;
    double lam[3];
    Phys::max_speeds(Pp, un, lam);
    const double* ja = Ja + q * 9;
    const double ij = fabs(invJ[q]);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      m[d] = fmax(m[d], fabs(ja[3 * d] * lam[0] + ja[3 * d + 1] * lam[1] + ja[3 * d + 2] * lam[2]) * ij);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int d = 0; d < 3; ++d) m[d] = fmax(m[d], __shfl_xor_sync(0xffffffffu, m[d], o));
  if (lane == 0) atomic_max_nonneg(max_speed + (member ? member[e] : 0), m[0] + m[1] + m[2]);
}

}  // namespace tag
