// Covariant shallow-water equations on a 2D manifold (the cubed sphere):
// device physics and kernels.
//
// Reference: src/equations/covariant_shallow_water.jl (fluxes :155-176,
// sources :216-243, speeds :246-305), covariant_shallow_water_split.jl
// (flux_ec :101-116, nonconservative fluxes :142-220, sources :273-302), the
// Lax-Friedrichs dissipation of src/equations/equations.jl:243-257, and the
// covariant DGSEM of src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl
// (weak form :98-131, flux differencing :135-234, interfaces :239-432,
// sources :435-452, apply_jacobian :461-478), max_dt of
// src/callbacks_step/stepsize_dg2d.jl:47-71.
//
// A handle holds one or more element groups; a group is a run of elements of
// one polynomial degree (an uneven ensemble has one group per run of members
// with equal degree).  Every stage is one interface launch and one element
// launch over all groups: each CTA finds its group and runs the body
// instantiated for that group's n.  The solution is u[node][3] with the
// nodes of each element contiguous; aux[node][26] is the reference's
// aux_node_vars; pk[node][16] a packed copy of what the element kernel reads.
#pragma once
#include "cov_params.cuh"
#include "dg2d_kernels.cuh"

namespace tag {

// packed per-node element data
enum CovPack : int {
  kPJ = 0, kPGc11, kPGc12, kPGc22, kPGv11, kPGv12, kPGv22, kPHs,
  kPC111, kPC112, kPC122, kPC211, kPC212, kPC222, kPF, kPInvJ, kPack = 16
};

struct CovGroup {
  int n;         // nodes per direction
  int e0, ne;    // elements [e0, e0 + ne)
  long node0;    // first node of element e0
  long sf0;      // first double of element e0 in the surface-flux array
  int if0, nif;  // interfaces [if0, if0 + nif)
  int epb;       // elements per CTA
  int blk0;      // first CTA of the group in the element launch
  int iblk0;     // first CTA of the group in the interface launch
  int basis;     // offset of the group's BasisDev in the basis array
};

constexpr int kCovMaxGroups = 64;

struct CovGroups {
  int count;
  CovGroup g[kCovMaxGroups];
};

TAG_DEV int cov_find_group(const CovGroups& G, int blk, bool iface) {
  int lo = 0;
  for (int k = 1; k < G.count; ++k)
    if ((iface ? G.g[k].iblk0 : G.g[k].blk0) <= blk) lo = k;
  return lo;
}

// packs aux (26), the Coriolis parameter f = 2 Omega z / |x| and 1/J per node
__global__ void k_cov_pack(const double* __restrict__ aux, const double* __restrict__ xyz,
                           long nodes, double omega, double* __restrict__ pk) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nodes) return;
  const double* a = aux + q * 26;
  double* p = pk + q * kPack;
  p[kPJ] = a[12];
  p[kPGc11] = a[16]; p[kPGc12] = a[17]; p[kPGc22] = a[18];
  p[kPGv11] = a[13]; p[kPGv12] = a[14]; p[kPGv22] = a[15];
  p[kPHs] = a[19];
#pragma unroll
  for (int k = 0; k < 6; ++k) p[kPC111 + k] = a[20 + k];
  const double* x = xyz + q * 3;
  p[kPF] = 2.0 * omega * x[2] / sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  p[kPInvJ] = 1.0 / a[12];
}

// ---- pointwise physics on packed data -----------------------------------------
TAG_DEV double cov_gcon(const double* p, int i, int j) {
  return (i == 0 && j == 0) ? p[kPGc11] : (i == 1 && j == 1) ? p[kPGc22] : p[kPGc12];
}

// contravariant flux component o of one node (standard or split form); ih = 1/h
TAG_DEV void cov_flux(const CovParams& P, const double* u, double ih, const double* p, int o,
                      double* f) {
  const double J = p[kPJ];
  const double m = J * u[1 + o];
  if (P.split) {
    f[0] = m;
    f[1] = m * (u[1] * ih);
    f[2] = m * (u[2] * ih);
    return;
  }
  const double vo = u[1 + o] * ih;
  const double gt = 0.5 * P.g * u[0] * u[0];
  f[0] = m;
  f[1] = J * (u[1] * vo + cov_gcon(p, 0, o) * gt);
  f[2] = J * (u[2] * vo + cov_gcon(p, 1, o) * gt);
}

// source_terms_geometric_coriolis (standard or split), after apply_jacobian
TAG_DEV void cov_source(const CovParams& P, const double* u, double ih, const double* p,
                        double* s) {
  const double hv0 = u[1], hv1 = u[2];
  const double v0 = hv0 * ih, v1 = hv1 * ih;
  const double T00 = hv0 * v0, T01 = hv0 * v1, T10 = hv1 * v0, T11 = hv1 * v1;
  double sg0, sg1;
  if (!P.split) {
    const double gt = 0.5 * P.g * u[0] * u[0];
    sg0 = p[kPC111] * (T00 + gt * p[kPGc11]) + p[kPC112] * (T01 + gt * p[kPGc12]) +
          p[kPC112] * (T10 + gt * p[kPGc12]) + p[kPC122] * (T11 + gt * p[kPGc22]);
    sg1 = p[kPC211] * (T00 + gt * p[kPGc11]) + p[kPC212] * (T01 + gt * p[kPGc12]) +
          p[kPC212] * (T10 + gt * p[kPGc12]) + p[kPC222] * (T11 + gt * p[kPGc22]);
  } else {
    // C = G_cov T, w_i = (Gamma^1 C[0,:])_i + (Gamma^2 C[1,:])_i
    const double C00 = p[kPGv11] * T00 + p[kPGv12] * T10, C01 = p[kPGv11] * T01 + p[kPGv12] * T11;
    const double C10 = p[kPGv12] * T00 + p[kPGv22] * T10, C11 = p[kPGv12] * T01 + p[kPGv22] * T11;
    const double w0 = (p[kPC111] * C00 + p[kPC112] * C01) + (p[kPC211] * C10 + p[kPC212] * C11);
    const double w1 = (p[kPC112] * C00 + p[kPC122] * C01) + (p[kPC212] * C10 + p[kPC222] * C11);
    const double s0 = p[kPC111] * T00 + p[kPC112] * T01 + p[kPC112] * T10 + p[kPC122] * T11;
    const double s1 = p[kPC211] * T00 + p[kPC212] * T01 + p[kPC212] * T10 + p[kPC222] * T11;
    sg0 = 0.5 * (s0 - (p[kPGc11] * w0 + p[kPGc12] * w1));
    sg1 = 0.5 * (s1 - (p[kPGc12] * w0 + p[kPGc22] * w1));
  }
  const double fJ = p[kPF] * p[kPJ];
  s[0] = 0.0;
  s[1] = -(sg0 + fJ * (p[kPGc12] * hv0 - p[kPGc11] * hv1));
  s[2] = -(sg1 + fJ * (p[kPGc22] * hv0 - p[kPGc12] * hv1));
}

// ---- interface fluxes ------------------------------------------------------------
// Geometry of one side of an interface node (the reference's aux layout: A
// column-major at 0..5, the contravariant basis column-major at 6..11, J at
// 12, G_11 G_12 G_22 at 13..15, G^11 G^12 G^22 at 16..18).
struct CovSide {
  double A[6], Ac[6], J, gv11, gv12, gv22, gc11, gc12, gc22;
};

TAG_DEV void cov_load_side(const double* __restrict__ a, CovSide& s) {
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    s.A[k] = a[k];
    s.Ac[k] = a[6 + k];
  }
  s.J = a[12];
  s.gv11 = a[13]; s.gv12 = a[14]; s.gv22 = a[15];
  s.gc11 = a[16]; s.gc12 = a[17]; s.gc22 = a[18];
}

// state of another node in the contravariant basis of `to`
TAG_DEV void cov_transform(const double* u, const CovSide& from, const CovSide& to, double* s) {
  double gl[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) gl[r] = from.A[r] * u[1] + from.A[3 + r] * u[2];
  s[0] = u[0];
#pragma unroll
  for (int r = 0; r < 2; ++r) s[1 + r] = to.Ac[r] * gl[0] + to.Ac[2 + r] * gl[1] + to.Ac[4 + r] * gl[2];
}

// surface flux (+ 0.5 nonconservative) along o of left state a and right
// state c, both sides' geometry `w` (the reference passes aux_vars_ll twice);
// iha = 1 / a[0], ihc = 1 / c[0]
TAG_DEV void cov_surface(const CovParams& P, const double* a, const double* c, double iha,
                         double ihc, const CovSide& w, int o, double* F) {
  const double J = w.J;
  const double gco0 = o ? w.gc12 : w.gc11;  // G^{1o}
  const double gco1 = o ? w.gc22 : w.gc12;  // G^{2o}
  const double ao = o ? a[2] : a[1], co = o ? c[2] : c[1];
  const double va1 = a[1] * iha, va2 = a[2] * iha, vc1 = c[1] * ihc, vc2 = c[2] * ihc;
  const double vao = o ? va2 : va1, vco = o ? vc2 : vc1;
  if (P.surf_sym == 1) {
    const double m = 0.5 * (J * ao + J * co);
    F[0] = m;
    F[1] = 0.5 * (va1 + vc1) * m;
    F[2] = 0.5 * (va2 + vc2) * m;
  } else if (P.split) {
    const double ma = J * ao, mc = J * co;
    F[0] = 0.5 * (ma + mc);
    F[1] = 0.5 * (ma * va1 + mc * vc1);
    F[2] = 0.5 * (ma * va2 + mc * vc2);
  } else {
    const double ga = 0.5 * P.g * a[0] * a[0], gc = 0.5 * P.g * c[0] * c[0];
    F[0] = 0.5 * (J * ao + J * co);
    F[1] = 0.5 * (J * (a[1] * vao + gco0 * ga) + J * (c[1] * vco + gco0 * gc));
    F[2] = 0.5 * (J * (a[2] * vao + gco1 * ga) + J * (c[2] * vco + gco1 * gc));
  }
  if (P.surf_diss) {
    const double goo = o ? w.gc22 : w.gc11;
    const double lam = fmax(fabs(vao) + sqrt(goo * a[0] * P.g), fabs(vco) + sqrt(goo * c[0] * P.g));
    const double s = -0.5 * J * lam;
    F[0] += s * (c[0] - a[0]);
    F[1] += s * (c[1] - a[1]);
    F[2] += s * (c[2] - a[2]);
  }
  if (P.surf_nc == 1) {
    // flux_nonconservative_ec with both geometries `w` (no topography jump)
    const double vcv0 = w.gv11 * vc1 + w.gv12 * vc2;
    const double vcv1 = w.gv12 * vc1 + w.gv22 * vc2;
    const double half_m = 0.5 * ao;
    const double ph = P.g * a[0] * c[0];
    F[1] += 0.5 * (J * (half_m * (w.gc11 * vcv0 + w.gc12 * vcv1 - vc1) + gco0 * ph));
    F[2] += 0.5 * (J * (half_m * (w.gc12 * vcv0 + w.gc22 * vcv1 - vc2) + gco1 * ph));
  } else if (P.surf_nc == 2) {
    const double ph = P.g * a[0] * c[0];
    F[1] += 0.5 * (J * (gco0 * ph));
    F[2] += 0.5 * (J * (gco1 * ph));
  }
}

// outward flux of one side (face f of its element)
// ih_mine = 1 / mine[0], ih_other = 1 / other_in_mine[0] (the transformation
// keeps h), each computed once per interface node
TAG_DEV void cov_side_flux(const CovParams& P, const double* mine, const double* other_in_mine,
                           double ih_mine, double ih_other, const CovSide& w, int f, double* F) {
  const int o = f >> 1;
  if ((f & 1) == 0) {
    cov_surface(P, other_in_mine, mine, ih_other, ih_mine, w, o, F);
    F[0] = -F[0];
    F[1] = -F[1];
    F[2] = -F[2];
  } else {
    cov_surface(P, mine, other_in_mine, ih_mine, ih_other, w, o, F);
  }
}

template <int n>
TAG_DEV void cov_interface_body(const CovParams& P, const CovGroup& G, int lblk, const double* u,
                                const double* aux, const int* if_e, const int* if_f,
                                const int* if_flip, double* sfv) {
  const int t = lblk * blockDim.x + threadIdx.x;
  const int k = t / n, l = t % n;
  if (k >= G.nif) return;
  const int kk = G.if0 + k;
  const int e0 = if_e[2 * kk], e1 = if_e[2 * kk + 1];
  const int f0 = if_f[2 * kk], f1 = if_f[2 * kk + 1];
  const int l1 = if_flip[kk] ? n - 1 - l : l;
  int i0, j0, i1, j1;
  face_node(f0, l, n, i0, j0);
  face_node(f1, l1, n, i1, j1);
  const long q0 = G.node0 + (long)(e0 - G.e0) * n * n + j0 * n + i0;
  const long q1 = G.node0 + (long)(e1 - G.e0) * n * n + j1 * n + i1;
  double ul[3], ur[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    ul[v] = u[q0 * 3 + v];
    ur[v] = u[q1 * 3 + v];
  }
  CovSide al, ar;
  cov_load_side(aux + q0 * 26, al);
  cov_load_side(aux + q1 * 26, ar);
  double rt[3], lt[3], Fp[3], Fs[3];
  cov_transform(ur, ar, al, rt);
  cov_transform(ul, al, ar, lt);
  const double ihl = 1.0 / ul[0], ihr = 1.0 / ur[0];
  cov_side_flux(P, ul, rt, ihl, ihr, al, f0, Fp);
  cov_side_flux(P, ur, lt, ihr, ihl, ar, f1, Fs);
  double* s0 = sfv + G.sf0 + ((long)(e0 - G.e0) * 4 + f0) * n * 3 + l * 3;
  double* s1 = sfv + G.sf0 + ((long)(e1 - G.e0) * 4 + f1) * n * 3 + l1 * 3;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    s0[v] = Fp[v];
    s1[v] = Fs[v];
  }
}

__global__ void __launch_bounds__(256) k_cov_interface(CovParams P, const CovGroups* __restrict__ GG,
                                                       const double* __restrict__ u,
                                                       const double* __restrict__ aux,
                                                       const int* __restrict__ if_e,
                                                       const int* __restrict__ if_f,
                                                       const int* __restrict__ if_flip,
                                                       double* __restrict__ sfv) {
  const int gi = cov_find_group(*GG, blockIdx.x, true);
  const CovGroup& G = GG->g[gi];
  const int lblk = blockIdx.x - G.iblk0;
  switch (G.n) {
    case 4: cov_interface_body<4>(P, G, lblk, u, aux, if_e, if_f, if_flip, sfv); break;
    case 6: cov_interface_body<6>(P, G, lblk, u, aux, if_e, if_f, if_flip, sfv); break;
    case 8: cov_interface_body<8>(P, G, lblk, u, aux, if_e, if_f, if_flip, sfv); break;
    case 2: cov_interface_body<2>(P, G, lblk, u, aux, if_e, if_f, if_flip, sfv); break;
    case 3: cov_interface_body<3>(P, G, lblk, u, aux, if_e, if_f, if_flip, sfv); break;
    case 5: cov_interface_body<5>(P, G, lblk, u, aux, if_e, if_f, if_flip, sfv); break;
    case 7: cov_interface_body<7>(P, G, lblk, u, aux, if_e, if_f, if_flip, sfv); break;
    default: break;
  }
}

// ---- element kernel --------------------------------------------------------------
// One thread per node (epb * n^2 <= 256 threads).  Shared memory per node:
// flux differencing: v1, v2, (G_cov v)_1, (G_cov v)_2, J hv^1, J hv^2, h, h_s, J,
// G^11, G^12, G^22, g h^2 / 2 (13 doubles, an odd stride); weak form: the two
// contravariant fluxes.
constexpr int kCovQ = 13;
__host__ __device__ constexpr int cov_elem_doubles(int n) { return n * n * kCovQ; }

// VK: 0 weak form (VolumeIntegralWeakForm), 1 flux differencing; a template
// parameter so that each volume kind gets its own register allocation
template <int n, int MODE, int VK>
TAG_DEV void cov_element_body(const CovParams& P, const CovGroup& G, int lblk,
                              const BasisDev* __restrict__ bases, double* __restrict__ u,
                              double* __restrict__ du, double* __restrict__ kreg,
                              const double* __restrict__ pk, const double* __restrict__ sfv,
                              StageArgs st, double* smem, unsigned& bad) {
  constexpr int nn = n * n;
  BasisDev* sb = reinterpret_cast<BasisDev*>(smem);
  double* q = smem + sizeof(BasisDev) / sizeof(double);
  const int el_first = lblk * G.epb;
  const int ne = min(G.epb, G.ne - el_first);
  if (ne <= 0) return;
  for (int t = threadIdx.x; t < (int)(sizeof(BasisDev) / sizeof(double)); t += blockDim.x)
    smem[t] = reinterpret_cast<const double*>(bases + G.basis)[t];
  const int el = threadIdx.x / nn, node = threadIdx.x % nn;
  const bool act = el < ne;
  const int i = node % n, j = node / n;
  const long gq = G.node0 + (long)(el_first + el) * nn + node;
  double ui[3], ih = 0.0;  // ih = 1/h, shared by the fluxes and the source
  double* qn = q + threadIdx.x * kCovQ;
  const double* __restrict__ pg = pk + gq * kPack;  // re-read where needed (L1 hit)
  if (act) {
#pragma unroll
    for (int v = 0; v < 3; ++v) ui[v] = u[gq * 3 + v];
    double p[kPack];
#pragma unroll
    for (int k = 0; k < kPack; ++k) p[k] = __ldg(pg + k);
    ih = 1.0 / ui[0];
    if constexpr (VK == 0) {
      cov_flux(P, ui, ih, p, 0, qn);
      cov_flux(P, ui, ih, p, 1, qn + 3);
    } else {
      const double v1 = ui[1] * ih, v2 = ui[2] * ih;
      qn[0] = v1;
      qn[1] = v2;
      qn[2] = p[kPGv11] * v1 + p[kPGv12] * v2;
      qn[3] = p[kPGv12] * v1 + p[kPGv22] * v2;
      qn[4] = p[kPJ] * ui[1];
      qn[5] = p[kPJ] * ui[2];
      qn[6] = ui[0];
      qn[7] = p[kPHs];
      qn[8] = p[kPJ];
      qn[9] = p[kPGc11];
      qn[10] = p[kPGc12];
      qn[11] = p[kPGc22];
      qn[12] = 0.5 * P.g * ui[0] * ui[0];
    }
  }
  __syncthreads();
  double un[3] = {0.0, 0.0, 0.0};
  if (act) {
    const double* eq = q + el * nn * kCovQ;
    double acc[3] = {0.0, 0.0, 0.0};
    if constexpr (VK == 0) {
#pragma unroll
      for (int b = 0; b < n; ++b) {
        const double d1 = sb->Dh[i * n + b], d2 = sb->Dh[j * n + b];
        const double* F1 = eq + (j * n + b) * kCovQ;
        const double* F2 = eq + (b * n + i) * kCovQ + 3;
#pragma unroll
        for (int v = 0; v < 3; ++v) acc[v] = fma(d2, F2[v], fma(d1, F1[v], acc[v]));
      }
    } else if (P.split && P.vol_sym <= 1) {
      // Split form with flux_central or flux_ec (and flux_nonconservative_ec):
      // every pair flux is a sum of products of a node-a factor and a node-b
      // factor, so each line sum sum_b D_ab f(a, b) is formed from a few
      // contractions sum_b D_ab x_b of node-b quantities (the pair terms of
      // covariant_shallow_water_split.jl:100-215 regrouped; 10 instead of
      // ~33 FP64 operations per partner node).  b = a is left out of the
      // symmetric part and kept in the nonconservative part, as in the
      // pairwise form.
      const double* qa = qn;
      const double h_a = ui[0], hs_a = qa[7], J_a = qa[8];
      const double gh = P.g * h_a;
      double nc1 = 0.0, nc2 = 0.0;
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        const double hvo_a = d ? ui[2] : ui[1];
        const double Jhvo_a = d ? qa[5] : qa[4];
        const double gco0 = d ? qa[10] : qa[9], gco1 = d ? qa[11] : qa[10];
        const int a = d ? j : i;
        double SD = 0.0, A1 = 0.0, A2 = 0.0, A3 = 0.0, A4 = 0.0, A5 = 0.0;
        double B2 = 0.0, B3 = 0.0, BH = 0.0;
#pragma unroll
        for (int b = 0; b < n; ++b) {
          const double* qb = eq + (d ? b * n + i : j * n + b) * kCovQ;
          const double Dab = sb->Ds[a * n + b];
          if (b != a) {
            const double Jb = d ? qb[5] : qb[4];
            SD += Dab;
            A1 = fma(Dab, Jb, A1);
            A2 = fma(Dab, qb[0], A2);
            A3 = fma(Dab, qb[0] * Jb, A3);
            A4 = fma(Dab, qb[1], A4);
            A5 = fma(Dab, qb[1] * Jb, A5);
          }
          if (P.vol_nc) {
            B2 = fma(Dab, qb[2], B2);
            B3 = fma(Dab, qb[3], B3);
            BH = fma(Dab, qb[6] + qb[7], BH);
          }
        }
        acc[0] += 0.5 * (Jhvo_a * SD + A1);
        if (P.vol_sym == 1) {
          // flux_ec: f = m (1, (v_a + v_b) / 2), m = (J hv_a + J hv_b) / 2
          acc[1] += 0.25 * ((qa[0] * Jhvo_a) * SD + qa[0] * A1 + Jhvo_a * A2 + A3);
          acc[2] += 0.25 * ((qa[1] * Jhvo_a) * SD + qa[1] * A1 + Jhvo_a * A4 + A5);
        } else {
          // flux_central of the split fluxes: (J hv v_a + J hv v_b) / 2
          acc[1] += 0.5 * ((Jhvo_a * qa[0]) * SD + A3);
          acc[2] += 0.5 * ((Jhvo_a * qa[1]) * SD + A5);
        }
        if (P.vol_nc) {
          const double Daa = sb->Ds[a * n + a];
          const double Sall = SD + Daa;
          const double B0 = fma(Daa, qa[0], A2), B1 = fma(Daa, qa[1], A4);
          const double half_m = 0.5 * hvo_a;
          const double ph = gh * (BH - hs_a * Sall);
          nc1 += J_a * (half_m * (qa[9] * B2 + qa[10] * B3 - B0) + gco0 * ph);
          nc2 += J_a * (half_m * (qa[10] * B2 + qa[11] * B3 - B1) + gco1 * ph);
        }
      }
      acc[1] += 0.5 * nc1;
      acc[2] += 0.5 * nc2;
    } else {
      const double* qa = qn;
      const double h_a = ui[0], hs_a = qa[7], J_a = qa[8];
      double nc1 = 0.0, nc2 = 0.0;
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        const double hvo_a = d ? ui[2] : ui[1];
        const double Jhvo_a = d ? qa[5] : qa[4];
        const double gco0 = d ? qa[10] : qa[9], gco1 = d ? qa[11] : qa[10];
        const int a = d ? j : i;
#pragma unroll
        for (int b = 0; b < n; ++b) {
          const double* qb = eq + (d ? b * n + i : j * n + b) * kCovQ;
          const double Dab = sb->Ds[a * n + b];
          if (b != a) {
            const double Jhvo_b = d ? qb[5] : qb[4];
            double f0, f1, f2;
            if (P.vol_sym == 1) {
              const double m = 0.5 * (Jhvo_a + Jhvo_b);
              f0 = m;
              f1 = 0.5 * (qa[0] + qb[0]) * m;
              f2 = 0.5 * (qa[1] + qb[1]) * m;
            } else if (P.split) {
              f0 = 0.5 * (Jhvo_a + Jhvo_b);
              f1 = 0.5 * (Jhvo_a * qa[0] + Jhvo_b * qb[0]);
              f2 = 0.5 * (Jhvo_a * qa[1] + Jhvo_b * qb[1]);
            } else {
              const double gb0 = d ? qb[10] : qb[9], gb1 = d ? qb[11] : qb[10];
              f0 = 0.5 * (Jhvo_a + Jhvo_b);
              f1 = 0.5 * ((Jhvo_a * qa[0] + J_a * gco0 * qa[12]) + (Jhvo_b * qb[0] + qb[8] * gb0 * qb[12]));
              f2 = 0.5 * ((Jhvo_a * qa[1] + J_a * gco1 * qa[12]) + (Jhvo_b * qb[1] + qb[8] * gb1 * qb[12]));
            }
            acc[0] = fma(Dab, f0, acc[0]);
            acc[1] = fma(Dab, f1, acc[1]);
            acc[2] = fma(Dab, f2, acc[2]);
          }
          if (P.vol_nc) {
            const double half_m = 0.5 * hvo_a;
            const double ph = P.g * h_a * (qb[6] + (qb[7] - hs_a));
            const double g0 = J_a * (half_m * (qa[9] * qb[2] + qa[10] * qb[3] - qb[0]) + gco0 * ph);
            const double g1 = J_a * (half_m * (qa[10] * qb[2] + qa[11] * qb[3] - qb[1]) + gco1 * ph);
            nc1 = fma(Dab, g0, nc1);
            nc2 = fma(Dab, g1, nc2);
          }
        }
      }
      acc[1] += 0.5 * nc1;
      acc[2] += 0.5 * nc2;
    }
    const double* se = sfv + G.sf0 + (long)(el_first + el) * 4 * n * 3;
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      if (i == 0) acc[v] += se[(0 * n + j) * 3 + v] * sb->winv0;
      if (i == n - 1) acc[v] += se[(1 * n + j) * 3 + v] * sb->winvN;
      if (j == 0) acc[v] += se[(2 * n + i) * 3 + v] * sb->winv0;
      if (j == n - 1) acc[v] += se[(3 * n + i) * 3 + v] * sb->winvN;
    }
    double s[3];
    {
      double p[kPack];
#pragma unroll
      for (int k = 0; k < kPack; ++k) p[k] = __ldg(pg + k);
      cov_source(P, ui, ih, p, s);
    }
    const double fac = -__ldg(pg + kPInvJ);
    const int e = G.e0 + el_first + el;
    double dv[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      dv[v] = acc[v] * fac + s[v];
      if (!isfinite(dv[v])) bad |= TAG_S_NAN;
    }
    if (!(ui[0] > 0.0)) bad |= TAG_S_NEG_DENSITY;
    if (MODE == kModeRhs) {
#pragma unroll
      for (int v = 0; v < 3; ++v) du[gq * 3 + v] = dv[v];
    } else {
      const double dt = st.dt[st.member ? st.member[e] : 0];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        un[v] = stage_value(st, ui[v], kreg + gq * 3 + v, dt, dv[v]);
        u[gq * 3 + v] = un[v];
      }
    }
  }
  if (MODE == kModeStage && st.max_speed != nullptr) {
    // the step's result to the registered sink (host memory over the host
    // link).  A warp's nodes are consecutive, so its 32 nodes x 3 values are
    // 96 consecutive doubles: lane l stores doubles l, l + 32 and l + 64,
    // fetched from their nodes' lanes, so that every store is contiguous
    if (st.sink != nullptr) {
      const int lane = threadIdx.x & 31, w_first = threadIdx.x & ~31;
      const long q0 = G.node0 + (long)el_first * nn + w_first;
      const int valid = ne * nn - w_first;  // the warp's nodes in range (may be <= 0)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int d = lane + 32 * k, src = d / 3, c = d % 3;
        const double s0 = __shfl_sync(0xffffffffu, un[0], src);
        const double s1 = __shfl_sync(0xffffffffu, un[1], src);
        const double s2 = __shfl_sync(0xffffffffu, un[2], src);
        if (src < valid) st.sink[q0 * 3 + d] = c == 0 ? s0 : (c == 1 ? s1 : s2);
      }
    }
    // CFL speeds of the updated state, scaled by n: dt = cfl 2 / (n max_e(l1 + l2))
    __syncthreads();
    if (act) {
      const double ihn = 1.0 / un[0];
      qn[0] = fabs(un[1] * ihn) + sqrt(__ldg(pg + kPGc11) * un[0] * P.g);
      qn[1] = fabs(un[2] * ihn) + sqrt(__ldg(pg + kPGc22) * un[0] * P.g);
    }
    __syncthreads();
    if (threadIdx.x < ne) {
      const double* eq = q + threadIdx.x * nn * kCovQ;
      double m1 = 0.0, m2 = 0.0;
      for (int k = 0; k < nn; ++k) {
        m1 = fmax(m1, eq[k * kCovQ]);
        m2 = fmax(m2, eq[k * kCovQ + 1]);
      }
      const int e = G.e0 + el_first + threadIdx.x;
      atomic_max_nonneg(st.max_speed + (st.member ? st.member[e] : 0), n * (m1 + m2));
    }
  }
}

// 256 threads and at least three CTAs per SM: up to 85 registers, which the
// FP64-latency-bound body uses for independent operations in flight
template <int MODE, int VK>
__global__ void __launch_bounds__(256, 3) k_cov_element(CovParams P, const CovGroups* __restrict__ GG,
                                                     const BasisDev* __restrict__ bases,
                                                     double* __restrict__ u,
                                                     double* __restrict__ du,
                                                     double* __restrict__ kreg,
                                                     const double* __restrict__ pk,
                                                     const double* __restrict__ sfv, StageArgs st,
                                                     unsigned* __restrict__ status) {
  extern __shared__ double smem[];
  const int gi = cov_find_group(*GG, blockIdx.x, false);
  const CovGroup& G = GG->g[gi];
  const int lblk = blockIdx.x - G.blk0;
  unsigned bad = 0;
  switch (G.n) {
    case 4: cov_element_body<4, MODE, VK>(P, G, lblk, bases, u, du, kreg, pk, sfv, st, smem, bad); break;
    case 6: cov_element_body<6, MODE, VK>(P, G, lblk, bases, u, du, kreg, pk, sfv, st, smem, bad); break;
    case 8: cov_element_body<8, MODE, VK>(P, G, lblk, bases, u, du, kreg, pk, sfv, st, smem, bad); break;
    case 2: cov_element_body<2, MODE, VK>(P, G, lblk, bases, u, du, kreg, pk, sfv, st, smem, bad); break;
    case 3: cov_element_body<3, MODE, VK>(P, G, lblk, bases, u, du, kreg, pk, sfv, st, smem, bad); break;
    case 5: cov_element_body<5, MODE, VK>(P, G, lblk, bases, u, du, kreg, pk, sfv, st, smem, bad); break;
    case 7: cov_element_body<7, MODE, VK>(P, G, lblk, bases, u, du, kreg, pk, sfv, st, smem, bad); break;
    default: break;
  }
  if (bad) atomicOr(status, bad);
}

// scaled CFL speed n max_e(l1 + l2) of a host-set state, per member
__global__ void k_cov_max_speed(CovParams P, const CovGroups* __restrict__ GG,
                                const double* __restrict__ u, const double* __restrict__ pk,
                                const int* __restrict__ member, double* __restrict__ max_speed,
                                int nelem) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  int gi = 0;
  for (int k = 1; k < GG->count; ++k)
    if (GG->g[k].e0 <= e) gi = k;
  const CovGroup& G = GG->g[gi];
  const int n = G.n, nn = n * n;
  const long q0 = G.node0 + (long)(e - G.e0) * nn;
  double m1 = 0.0, m2 = 0.0;
  for (int node = 0; node < nn; ++node) {
    const double* uq = u + (q0 + node) * 3;
    const double* p = pk + (q0 + node) * kPack;
    m1 = fmax(m1, fabs(uq[1] / uq[0]) + sqrt(p[kPGc11] * uq[0] * P.g));
    m2 = fmax(m2, fabs(uq[2] / uq[0]) + sqrt(p[kPGc22] * uq[0] * P.g));
  }
  atomic_max_nonneg(max_speed + (member ? member[e] : 0), n * (m1 + m2));
}

}  // namespace tag
