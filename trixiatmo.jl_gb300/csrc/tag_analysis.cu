// Device analysis kernels (integrals, entropy time derivative, error norms);
// the interface and the reference it follows are described in tag_analysis.cuh.
#include <cmath>
#include <vector>

#include "tag_analysis.cuh"
#include "cov_params.cuh"
#include "phys_euler_energy_2d.cuh"
#include "phys_euler_energy_3d.cuh"
#include "phys_moist_2d.cuh"
#include "phys_pt_2d.cuh"
#include "phys_pt_3d.cuh"
#include "phys_ie_2d.cuh"
#include "phys_rainy_2d.cuh"

namespace tag {

namespace {

constexpr int kAnThreads = 128;  // power of two (tree reductions)

// NaN-propagating max (Julia's max), so a NaN error shows in linf
TAG_DEV double nanmax(double a, double b) { return (isnan(a) || a > b) ? a : b; }

// ---- per-equation analysis functions --------------------------------------
// entropy(u), energy_total(u) and cons2entropy(u) . du as the reference
// defines them for each equation system; aux is the node's aux_node_vars
// (covariant equations) or null.
template <class Phys>
struct An;

// compressible_euler_energy_with_gravity_2d.jl: cons2entropy :539-557,
// entropy = entropy_math :602-627, energy_total :630
template <>
struct An<PhysEnergy2D> {
  using P = PhysEnergy2D::Params;
  static constexpr int NV = 5;
  static constexpr bool kEntropy = true, kEnergy = true;
  TAG_DEV static double entropy(const P& q, const double* u, const double*) {
    const double p = q.gm1 * (u[3] - 0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0]);
    const double s = log(p) - q.gamma * log(u[0]);
    return -s * u[0] * q.inv_gm1;
  }
  TAG_DEV static double energy_total(const P&, const double* u, const double*) { return u[3]; }
  TAG_DEV static double dsdt(const P& q, const double* u, const double* du, const double*) {
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double v_square = v1 * v1 + v2 * v2;
    const double p = q.gm1 * (u[3] - 0.5 * u[0] * v_square);
    const double s = log(p) - q.gamma * log(u[0]);
    const double rho_p = u[0] / p;
    const double w1 = (q.gamma - s) * q.inv_gm1 - 0.5 * rho_p * v_square;
    return w1 * du[0] + rho_p * v1 * du[1] + rho_p * v2 * du[2] - rho_p * du[3];
  }
};

// compressible_euler_energy_with_gravity_3d.jl: cons2entropy :581-601,
// entropy_math :661-673, energy_total = rho_e
template <>
struct An<PhysEnergy3D> {
  using P = PhysEnergy3D::Params;
  static constexpr int NV = 6;
  static constexpr bool kEntropy = true, kEnergy = true;
  TAG_DEV static double entropy(const P& q, const double* u, const double*) {
    const double p =
        q.gm1 * (u[4] - 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]);
    const double s = log(p) - q.gamma * log(u[0]);
    return -s * u[0] * q.inv_gm1;
  }
  TAG_DEV static double energy_total(const P&, const double* u, const double*) { return u[4]; }
  TAG_DEV static double dsdt(const P& q, const double* u, const double* du, const double*) {
    const double v1 = u[1] / u[0], v2 = u[2] / u[0], v3 = u[3] / u[0];
    const double v_square = v1 * v1 + v2 * v2 + v3 * v3;
    const double p = q.gm1 * (u[4] - 0.5 * u[0] * v_square);
    const double s = log(p) - q.gamma * log(u[0]);
    const double rho_p = u[0] / p;
    const double w1 = (q.gamma - s) * q.inv_gm1 - 0.5 * rho_p * v_square;
    return w1 * du[0] + rho_p * (v1 * du[1] + v2 * du[2] + v3 * du[3]) - rho_p * du[4];
  }
};

// compressible_euler_potential_temperature_gravity_2d.jl: cons2entropy
// :371-379, entropy = entropy_thermodynamic :381-387, energy_total :389-397
// (p_0 (R rho_theta / p_0)^gamma = K rho_theta^gamma, K = p_0 (R / p_0)^gamma)
template <>
struct An<PhysPT2D> {
  using P = PhysPT2D::Params;
  static constexpr int NV = 5;
  static constexpr bool kEntropy = true, kEnergy = true;
  TAG_DEV static double entropy(const P& q, const double* u, const double*) {
    const double p = q.K * pow(u[3], q.gamma);
    const double s = log(p) - q.gamma * log(u[0]);
    return -s * u[0] / (q.gamma - 1.0);
  }
  TAG_DEV static double energy_total(const P& q, const double* u, const double*) {
    const double p = q.K * pow(u[3], q.gamma);
    return p / (q.gamma - 1.0) + 0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0];
  }
  TAG_DEV static double dsdt(const P& q, const double* u, const double* du, const double*) {
    const double w1 = log(q.K * pow(u[3] / u[0], q.gamma)) - q.gamma;
    const double w4 = u[0] / u[3] * q.gamma;
    return w1 * du[0] + w4 * du[3];
  }
};

// compressible_euler_potential_temperature_gravity_3d.jl: cons2entropy
// :560-569, entropy :571-578, energy_total :593-603
template <>
struct An<PhysPT3D> {
  using P = PhysPT3D::Params;
  static constexpr int NV = 6;
  static constexpr bool kEntropy = true, kEnergy = true;
  TAG_DEV static double entropy(const P& q, const double* u, const double*) {
    const double p = q.pt.K * pow(u[4], q.pt.gamma);
    const double s = log(p) - q.pt.gamma * log(u[0]);
    return -s * u[0] / (q.pt.gamma - 1.0);
  }
  TAG_DEV static double energy_total(const P& q, const double* u, const double*) {
    const double p = q.pt.K * pow(u[4], q.pt.gamma);
    return p / (q.pt.gamma - 1.0) + 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0];
  }
  TAG_DEV static double dsdt(const P& q, const double* u, const double* du, const double*) {
    const double w1 = log(q.pt.K * pow(u[4] / u[0], q.pt.gamma)) - q.pt.gamma;
    const double w5 = u[0] / u[4] * q.pt.gamma;
    return w1 * du[0] + w5 * du[4];
  }
};

// compressible_euler_internal_energy_with_gravity_2d.jl: cons2entropy
// :271-280 and entropy :282-289 as defined there (no energy_total)
template <>
struct An<PhysIE2D> {
  using P = PhysIE2D::Params;
  static constexpr int NV = 5;
  static constexpr bool kEntropy = true, kEnergy = false;
  TAG_DEV static double entropy(const P& q, const double* u, const double*) {
    const double p = q.gm1 * u[3];
    const double s = log(p) - q.gamma * log(u[0]);
    return -s * u[0] / q.gm1;
  }
  TAG_DEV static double energy_total(const P&, const double*, const double*) { return 0.0; }
  TAG_DEV static double dsdt(const P& q, const double* u, const double* du, const double*) {
    const double w1 = log(u[3] * q.gm1 / pow(u[0], q.gamma)) - q.gamma;
    const double w4 = u[0] / (u[3] * q.gm1);
    return w1 * du[0] + w4 * du[3];
  }
};

// compressible_moist_euler_2d.jl: cons2entropy :513-551 (zero-density
// guards), entropy = -entropy_thermodynamic :733-757 (no guards, as there),
// energy_total = rho_E :760
template <>
struct An<PhysMoist2D> {
  using P = PhysMoist2D::Params;
  static constexpr int NV = 6;
  static constexpr bool kEntropy = true, kEnergy = true;
  TAG_DEV static double entropy(const P& q, const double* u, const double*) {
    double p, T;
    PhysMoist2D::condition(q, u, p, T);
    const double rho_qd = u[0] - u[4] - u[5], rho_qv = u[4], rho_ql = u[5];
    const double lT = log(T);
    const double s_d = q.c_vd * lT - q.R_d * log(rho_qd * q.R_d);
    const double s_v = q.c_vv * lT - q.R_v * log(rho_qv * q.R_v);
    const double s_l = q.c_pl * lT;
    return -(rho_qd * s_d + rho_qv * s_v + rho_ql * s_l);
  }
  TAG_DEV static double energy_total(const P&, const double* u, const double*) { return u[3]; }
  TAG_DEV static double dsdt(const P& q, const double* u, const double* du, const double*) {
    double p, T;
    PhysMoist2D::condition(q, u, p, T);
    const double v1 = u[1] / u[0], v2 = u[2] / u[0];
    const double v_square = v1 * v1 + v2 * v2;
    const double rho_qd = u[0] - u[4] - u[5], rho_qv = u[4], rho_ql = u[5];
    double s_d = 0.0, s_v = 0.0, s_l = 0.0;
    if (rho_qd > 0) s_d = q.c_pd * log(T) - q.R_d * log(rho_qd * q.R_d * T);
    if (rho_qv > 0) s_v = q.c_pv * log(T) - q.R_v * log(rho_qv * q.R_v * T);
    if (rho_ql > 0) s_l = q.c_pl * log(T);
    const double g_d = (q.c_pd - s_d) * T;
    const double g_v = q.L_00 + (q.c_pv - s_v) * T;
    const double g_l = (q.c_pl - s_l) * T;
    const double iT = 1.0 / T;
    return iT * ((g_d - 0.5 * v_square) * du[0] + v1 * du[1] + v2 * du[2] - du[3] +
                 (g_v - g_d) * du[4] + (g_l - g_d) * du[5]);
  }
};

// compressible_rainy_euler_2d.jl: cons2entropy :132-172 (no entropy or
// energy_total is defined for these equations)
template <>
struct An<PhysRainy2D> {
  using P = PhysRainy2D::Params;
  static constexpr int NV = 9;
  static constexpr bool kEntropy = false, kEnergy = false;
  TAG_DEV static double entropy(const P&, const double*, const double*) { return 0.0; }
  TAG_DEV static double energy_total(const P&, const double*, const double*) { return 0.0; }
  TAG_DEV static double dsdt(const P&, const double* u, const double* du, const double*) {
    using C = RainyConst;
    double rv, rc, T;
    PhysRainy2D::nlsol(u, rv, rc, T);
    const double rho_inv = 1.0 / (u[0] + u[1] + u[2]);
    const double lT = log(T), iT = 1.0 / T;
    const double v1 = u[3] * rho_inv, v2 = u[4] * rho_inv;
    const double vsq = 0.5 * (v1 * v1 + v2 * v2) * iT;
    const double rv_log = rv > 0.0 ? log(rv) : 0.0;
    const double w_d = C::c_vd * lT - C::R_d * log(u[0]) + vsq - C::c_vd - C::R_d;
    const double w_v =
        C::c_vv * lT - C::R_v * rv_log + vsq - C::c_vv - C::R_v - C::ref_L * iT;
    const double w_l = C::c_l * lT + vsq - C::c_l;
    return w_d * du[0] + (w_v + w_l) * du[1] + w_l * du[2] - v1 * iT * du[3] -
           v2 * iT * du[4] + iT * du[5];
  }
};

// covariant_shallow_water.jl: cons2entropy :128-137, entropy :155-164 (the
// total energy); aux: G_11 G_12 G_22 at 13..15, h_s at 19
struct PhysCovAn {};
template <>
struct An<PhysCovAn> {
  using P = CovParams;
  static constexpr int NV = 3;
  static constexpr bool kEntropy = true, kEnergy = false;
  TAG_DEV static void vel(const double* u, const double* a, double* vcon, double* vcov) {
    vcon[0] = u[1] / u[0];
    vcon[1] = u[2] / u[0];
    vcov[0] = a[13] * vcon[0] + a[14] * vcon[1];
    vcov[1] = a[14] * vcon[0] + a[15] * vcon[1];
  }
  TAG_DEV static double entropy(const P& q, const double* u, const double* a) {
    double vcon[2], vcov[2];
    vel(u, a, vcon, vcov);
    const double h = u[0];
    return 0.5 * (h * (vcov[0] * vcon[0] + vcov[1] * vcon[1]) + q.g * h * h) + q.g * h * a[19];
  }
  TAG_DEV static double energy_total(const P&, const double*, const double*) { return 0.0; }
  TAG_DEV static double dsdt(const P& q, const double* u, const double* du, const double* a) {
    double vcon[2], vcov[2];
    vel(u, a, vcon, vcov);
    const double w0 = q.g * (u[0] + a[19]) - 0.5 * (vcov[0] * vcon[0] + vcov[1] * vcon[1]);
    return w0 * du[0] + vcov[0] * du[1] + vcov[1] * du[2];
  }
};

constexpr int kQErrors = 100;  // internal: error norms at the solution nodes

template <int NV>
__host__ __device__ constexpr int nq_of(int Q) {
  return Q == TAG_AQ_STATE ? NV + 1 : Q == kQErrors ? 2 * NV + 1 : 2;
}

// fixed-order tree reduction of NQ columns over the block (blockDim.x a power
// of two); the result is left in red[0 .. NQ)
template <int NQ>
TAG_DEV void block_reduce(const double (&acc)[NQ], double* red, int max_lo, int max_hi) {
  const int t = threadIdx.x;
#pragma unroll
  for (int q = 0; q < NQ; ++q) red[t * NQ + q] = acc[q];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (t < s) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const double a = red[t * NQ + q], b = red[(t + s) * NQ + q];
        red[t * NQ + q] = (q >= max_lo && q < max_hi) ? nanmax(a, b) : a + b;
      }
    }
    __syncthreads();
  }
}

// One block per (chunk of a member's nodes, member): per-node integrands
// weighted by wj, summed in a fixed order; the last column is the volume.
template <class T, int Q>
__global__ void __launch_bounds__(kAnThreads)
    k_node_rows(typename T::P P, const double* __restrict__ u, const double* __restrict__ du,
                const double* __restrict__ aux, const double* __restrict__ wj,
                const double* __restrict__ uex, const long* __restrict__ mbeg,
                const long* __restrict__ mend, long chunk, double* __restrict__ rows) {
  constexpr int NV = T::NV;
  constexpr int NQ = nq_of<NV>(Q);
  __shared__ double red[kAnThreads * NQ];
  const int m = blockIdx.y, c = blockIdx.x;
  const long b = mbeg[m] + (long)c * chunk;
  const long e = min(mend[m], b + chunk);
  double acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
  for (long q = b + threadIdx.x; q < e; q += blockDim.x) {
    const double* uq = u + q * NV;
    const double* aq = aux ? aux + q * 26 : nullptr;
    const double w = wj[q];
    if constexpr (Q == TAG_AQ_STATE) {
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] += w * uq[v];
    } else if constexpr (Q == TAG_AQ_ENTROPY) {
      acc[0] += w * T::entropy(P, uq, aq);
    } else if constexpr (Q == TAG_AQ_ENERGY_TOTAL) {
      acc[0] += w * T::energy_total(P, uq, aq);
    } else if constexpr (Q == TAG_AQ_ENTROPY_TIMEDERIVATIVE) {
      acc[0] += w * T::dsdt(P, uq, du + q * NV, aq);
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const double d = uex[q * NV + v] - uq[v];
        acc[v] += w * d * d;
        acc[NV + v] = nanmax(acc[NV + v], fabs(d));
      }
    }
    acc[NQ - 1] += w;
  }
  block_reduce<NQ>(acc, red, Q == kQErrors ? NV : 0, Q == kQErrors ? 2 * NV : 0);
  if (threadIdx.x < NQ) rows[((long)m * gridDim.x + c) * NQ + threadIdx.x] = red[threadIdx.x];
}

// One block per Cartesian element: the solution and J interpolated to the
// m^DIM analysis nodes, compared with the exact solution there.
template <class T, int DIM>
__global__ void __launch_bounds__(kAnThreads)
    k_element_error_rows(int n, int m, const double* __restrict__ u,
                         const double* __restrict__ invJ, const double* __restrict__ V,
                         const double* __restrict__ wa, const double* __restrict__ uex,
                         double* __restrict__ rows) {
  constexpr int NV = T::NV, NQ = 2 * NV + 1;
  extern __shared__ double sm[];
  const int npe = DIM == 3 ? n * n * n : n * n;
  const int ma = DIM == 3 ? m * m * m : m * m;
  double* su = sm;              // [npe][NV]
  double* sJ = su + npe * NV;   // [npe]
  double* sV = sJ + npe;        // [m][n]
  double* sw = sV + m * n;      // [m]
  double* red = sw + m;         // [kAnThreads][NQ]
  const long e = blockIdx.x;
  for (int k = threadIdx.x; k < npe * NV; k += blockDim.x) su[k] = u[e * npe * NV + k];
  for (int k = threadIdx.x; k < npe; k += blockDim.x) sJ[k] = 1.0 / invJ[e * npe + k];
  for (int k = threadIdx.x; k < m * n; k += blockDim.x) sV[k] = V[k];
  for (int k = threadIdx.x; k < m; k += blockDim.x) sw[k] = wa[k];
  __syncthreads();
  double acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
  for (int a = threadIdx.x; a < ma; a += blockDim.x) {
    const int ia = a % m, ja = (a / m) % m, ka = a / (m * m);
    double ui[NV], Ji = 0.0;
#pragma unroll
    for (int v = 0; v < NV; ++v) ui[v] = 0.0;
    for (int l = 0; l < npe; ++l) {
      const int i = l % n, j = (l / n) % n, k = l / (n * n);
      double c = sV[ia * n + i] * sV[ja * n + j];
      if (DIM == 3) c *= sV[ka * n + k];
#pragma unroll
      for (int v = 0; v < NV; ++v) ui[v] += c * su[l * NV + v];
      Ji += c * sJ[l];
    }
    double wJ = sw[ia] * sw[ja] * fabs(Ji);
    if (DIM == 3) wJ *= sw[ka];
    const double* ue = uex + (e * ma + a) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double d = ue[v] - ui[v];
      acc[v] += wJ * d * d;
      acc[NV + v] = nanmax(acc[NV + v], fabs(d));
    }
    acc[2 * NV] += wJ;
  }
  block_reduce<NQ>(acc, red, NV, 2 * NV);
  if (threadIdx.x < NQ) rows[e * NQ + threadIdx.x] = red[threadIdx.x];
}

__global__ void k_reduce_rows(const double* __restrict__ rows, int nq, int max_lo, int max_hi,
                              const long* __restrict__ rbeg, const long* __restrict__ rend,
                              long stride, double* __restrict__ out) {
  extern __shared__ double red[];  // [blockDim][nq]
  const int m = blockIdx.x, t = threadIdx.x;
  const long b = rbeg ? rbeg[m] : (long)m * stride;
  const long e = rbeg ? rend[m] : b + stride;
  for (int q = 0; q < nq; ++q) red[t * nq + q] = 0.0;
  for (long r = b + t; r < e; r += blockDim.x)
    for (int q = 0; q < nq; ++q) {
      const double v = rows[r * nq + q];
      red[t * nq + q] =
          (q >= max_lo && q < max_hi) ? nanmax(red[t * nq + q], v) : red[t * nq + q] + v;
    }
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (t < s)
      for (int q = 0; q < nq; ++q) {
        const double a = red[t * nq + q], c = red[(t + s) * nq + q];
        red[t * nq + q] = (q >= max_lo && q < max_hi) ? nanmax(a, c) : a + c;
      }
    __syncthreads();
  }
  if (t < nq) out[(long)m * nq + t] = red[t];
}

__global__ void k_weights_cartesian(const double* __restrict__ invJ, const double* __restrict__ w,
                                    int n, int dim, long nodes, double* __restrict__ wj) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nodes) return;
  const int npe = dim == 3 ? n * n * n : n * n;
  const int l = (int)(q % npe);
  double c = w[l % n] * w[(l / n) % n];
  if (dim == 3) c *= w[l / (n * n)];
  wj[q] = c * fabs(1.0 / invJ[q]);
}

__global__ void k_weights_covariant(const double* __restrict__ aux, const double* __restrict__ w,
                                    int n, long node0, long count, double* __restrict__ wj) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= count) return;
  const long q = node0 + r;
  const int l = (int)(r % (n * n));
  wj[q] = w[l % n] * w[l / n] * aux[q * 26 + 12];
}

__global__ void k_coordinates(int dim, int n, int m, const double* __restrict__ xyz,
                              const double* __restrict__ V, double* __restrict__ out) {
  const long e = blockIdx.x;
  const int npe = dim == 3 ? n * n * n : n * n;
  const int ma = dim == 3 ? m * m * m : m * m;
  for (int a = threadIdx.x; a < ma; a += blockDim.x) {
    const int ia = a % m, ja = (a / m) % m, ka = a / (m * m);
    double x[3] = {0.0, 0.0, 0.0};
    for (int l = 0; l < npe; ++l) {
      const int i = l % n, j = (l / n) % n, k = l / (n * n);
      double c = V[ia * n + i] * V[ja * n + j];
      if (dim == 3) c *= V[ka * n + k];
      for (int d = 0; d < dim; ++d) x[d] += c * xyz[(e * npe + l) * dim + d];
    }
    for (int d = 0; d < dim; ++d) out[(e * ma + a) * dim + d] = x[d];
  }
}

int last_status() { return cudaGetLastError() == cudaSuccess ? TAG_OK : TAG_E_CUDA; }

template <class T>
int launch_node_rows(const AnalysisArgs& a, const double* uex, int quantity, int nchunks,
                     long chunk, double* rows, cudaStream_t s) {
  const auto& P = *static_cast<const typename T::P*>(a.params);
  const dim3 grid(nchunks, a.nmembers);
  switch (quantity) {
    case TAG_AQ_STATE:
      k_node_rows<T, TAG_AQ_STATE><<<grid, kAnThreads, 0, s>>>(P, a.u, a.du, a.aux, a.wj, uex,
                                                                a.mbeg, a.mend, chunk, rows);
      break;
    case TAG_AQ_ENTROPY:
      if (!T::kEntropy) return TAG_E_INVALID;
      k_node_rows<T, TAG_AQ_ENTROPY><<<grid, kAnThreads, 0, s>>>(P, a.u, a.du, a.aux, a.wj, uex,
                                                                  a.mbeg, a.mend, chunk, rows);
      break;
    case TAG_AQ_ENERGY_TOTAL:
      if (!T::kEnergy) return TAG_E_INVALID;
      k_node_rows<T, TAG_AQ_ENERGY_TOTAL><<<grid, kAnThreads, 0, s>>>(
          P, a.u, a.du, a.aux, a.wj, uex, a.mbeg, a.mend, chunk, rows);
      break;
    case TAG_AQ_ENTROPY_TIMEDERIVATIVE:
      k_node_rows<T, TAG_AQ_ENTROPY_TIMEDERIVATIVE><<<grid, kAnThreads, 0, s>>>(
          P, a.u, a.du, a.aux, a.wj, uex, a.mbeg, a.mend, chunk, rows);
      break;
    case kQErrors:
      k_node_rows<T, kQErrors><<<grid, kAnThreads, 0, s>>>(P, a.u, a.du, a.aux, a.wj, uex,
                                                            a.mbeg, a.mend, chunk, rows);
      break;
    default:
      return TAG_E_INVALID;
  }
  return last_status();
}

int dispatch_node_rows(const AnalysisArgs& a, const double* uex, int quantity, int nchunks,
                       long chunk, double* rows, cudaStream_t s) {
  switch (a.phys) {
    case kAnEnergy2D:
      return launch_node_rows<An<PhysEnergy2D>>(a, uex, quantity, nchunks, chunk, rows, s);
    case kAnEnergy3D:
      return launch_node_rows<An<PhysEnergy3D>>(a, uex, quantity, nchunks, chunk, rows, s);
    case kAnRainy2D:
      return launch_node_rows<An<PhysRainy2D>>(a, uex, quantity, nchunks, chunk, rows, s);
    case kAnMoist2D:
      return launch_node_rows<An<PhysMoist2D>>(a, uex, quantity, nchunks, chunk, rows, s);
    case kAnPT2D:
      return launch_node_rows<An<PhysPT2D>>(a, uex, quantity, nchunks, chunk, rows, s);
    case kAnCov:
      return launch_node_rows<An<PhysCovAn>>(a, uex, quantity, nchunks, chunk, rows, s);
    case kAnPT3D:
      return launch_node_rows<An<PhysPT3D>>(a, uex, quantity, nchunks, chunk, rows, s);
    case kAnIE2D:
      return launch_node_rows<An<PhysIE2D>>(a, uex, quantity, nchunks, chunk, rows, s);
  }
  return TAG_E_INVALID;
}

template <class T>
int launch_element_errors(int dim, int n, int m, int nelem, const double* u, const double* invJ,
                          const double* V, const double* wa, const double* uex, double* rows,
                          cudaStream_t s) {
  constexpr int NQ = 2 * T::NV + 1;
  const int npe = dim == 3 ? n * n * n : n * n;
  const size_t smem =
      sizeof(double) * ((size_t)npe * T::NV + npe + (size_t)m * n + m + (size_t)kAnThreads * NQ);
  if (smem > 48 * 1024) return TAG_E_INVALID;
  if (dim == 3)
    k_element_error_rows<T, 3><<<nelem, kAnThreads, smem, s>>>(n, m, u, invJ, V, wa, uex, rows);
  else
    k_element_error_rows<T, 2><<<nelem, kAnThreads, smem, s>>>(n, m, u, invJ, V, wa, uex, rows);
  return last_status();
}

// Legendre polynomial L_N and its derivative at x (three-term recurrence)
void legendre(int N, double x, double& L, double& dL) {
  if (N == 0) {
    L = 1.0;
    dL = 0.0;
    return;
  }
  double l0 = 1.0, l1 = x, d0 = 0.0, d1 = 1.0;
  for (int k = 1; k < N; ++k) {
    const double l2 = ((2 * k + 1) * x * l1 - k * l0) / (k + 1);
    const double d2 = d0 + (2 * k + 1) * l1;
    l0 = l1;
    l1 = l2;
    d0 = d1;
    d1 = d2;
  }
  L = l1;
  dL = d1;
}

}  // namespace

int analysis_values(int phys, int quantity) {
  static const int nv[] = {5, 6, 9, 6, 5, 3, 6, 5};
  if (phys < 0 || phys > kAnIE2D) return -1;
  switch (quantity) {
    case TAG_AQ_STATE: return nv[phys];
    case TAG_AQ_ENTROPY: return phys == kAnRainy2D ? -1 : 1;
    case TAG_AQ_ENERGY_TOTAL:
      return (phys == kAnRainy2D || phys == kAnCov || phys == kAnIE2D) ? -1 : 1;
    case TAG_AQ_ENTROPY_TIMEDERIVATIVE: return 1;
  }
  return -1;
}

int analysis_node_rows(const AnalysisArgs& a, int nchunks, long chunk, double* rows,
                       cudaStream_t s) {
  return dispatch_node_rows(a, nullptr, a.quantity, nchunks, chunk, rows, s);
}

int analysis_node_error_rows(const AnalysisArgs& a, const double* u_exact, int nchunks, long chunk,
                             double* rows, cudaStream_t s) {
  return dispatch_node_rows(a, u_exact, kQErrors, nchunks, chunk, rows, s);
}

int analysis_element_error_rows(int phys, int dim, int n, int m, int nelem, const double* u,
                                const double* invJ, const double* V, const double* wa,
                                const double* u_exact, double* rows, cudaStream_t s) {
  switch (phys) {
    case kAnEnergy2D:
      return launch_element_errors<An<PhysEnergy2D>>(dim, n, m, nelem, u, invJ, V, wa, u_exact,
                                                     rows, s);
    case kAnEnergy3D:
      return launch_element_errors<An<PhysEnergy3D>>(dim, n, m, nelem, u, invJ, V, wa, u_exact,
                                                     rows, s);
    case kAnRainy2D:
      return launch_element_errors<An<PhysRainy2D>>(dim, n, m, nelem, u, invJ, V, wa, u_exact,
                                                    rows, s);
    case kAnMoist2D:
      return launch_element_errors<An<PhysMoist2D>>(dim, n, m, nelem, u, invJ, V, wa, u_exact,
                                                    rows, s);
    case kAnPT2D:
      return launch_element_errors<An<PhysPT2D>>(dim, n, m, nelem, u, invJ, V, wa, u_exact,
                                                 rows, s);
    case kAnPT3D:
      return launch_element_errors<An<PhysPT3D>>(dim, n, m, nelem, u, invJ, V, wa, u_exact,
                                                 rows, s);
    case kAnIE2D:
      return launch_element_errors<An<PhysIE2D>>(dim, n, m, nelem, u, invJ, V, wa, u_exact,
                                                 rows, s);
  }
  return TAG_E_INVALID;
}

int analysis_reduce_rows(const double* rows, int nq, int max_lo, int max_hi, const long* rbeg,
                         const long* rend, long stride, int nmembers, double* out,
                         cudaStream_t s) {
  const int threads = 128;
  k_reduce_rows<<<nmembers, threads, sizeof(double) * threads * nq, s>>>(
      rows, nq, max_lo, max_hi, rbeg, rend, stride, out);
  return last_status();
}

int analysis_weights_cartesian(const double* invJ, const double* w, int n, int dim, long nodes,
                               double* wj, cudaStream_t s) {
  k_weights_cartesian<<<(unsigned)((nodes + 255) / 256), 256, 0, s>>>(invJ, w, n, dim, nodes, wj);
  return last_status();
}

int analysis_weights_covariant(const double* aux, const double* w, int n, long node0, long count,
                               double* wj, cudaStream_t s) {
  if (count <= 0) return TAG_OK;
  k_weights_covariant<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(aux, w, n, node0, count,
                                                                       wj);
  return last_status();
}

int analysis_coordinates(int dim, int n, int m, int nelem, const double* xyz, const double* V,
                         double* out, cudaStream_t s) {
  k_coordinates<<<nelem, kAnThreads, 0, s>>>(dim, n, m, xyz, V, out);
  return last_status();
}

// LGL nodes: the end points and the roots of L_N' (Newton from the
// Chebyshev-Gauss-Lobatto points, L_N'' from Legendre's differential
// equation); weights 2 / (N (N + 1) L_N(x_j)^2).
void lgl_nodes_weights(int N, double* x, double* w) {
  x[0] = -1.0;
  x[N] = 1.0;
  for (int j = 1; j < N; ++j) {
    double t = -std::cos(M_PI * j / N);
    for (int it = 0; it < 100; ++it) {
      double L, dL;
      legendre(N, t, L, dL);
      const double d2L = (2.0 * t * dL - N * (N + 1.0) * L) / (1.0 - t * t);
      const double dt = dL / d2L;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    x[j] = t;
  }
  for (int j = 0; j <= N / 2; ++j) {  // symmetric about 0
    const double s = 0.5 * (x[N - j] - x[j]);
    x[j] = -s;
    x[N - j] = s;
  }
  if (N % 2 == 0) x[N / 2] = 0.0;
  for (int j = 0; j <= N; ++j) {
    double L, dL;
    legendre(N, x[j], L, dL);
    w[j] = 2.0 / (N * (N + 1.0) * L * L);
  }
}

void interpolation_matrix(const double* xf, int nf, const double* xt, int nt, double* V) {
  std::vector<double> lam(nf, 1.0);
  for (int i = 0; i < nf; ++i)
    for (int k = 0; k < nf; ++k)
      if (k != i) lam[i] /= (xf[i] - xf[k]);
  for (int a = 0; a < nt; ++a) {
    int hit = -1;
    for (int i = 0; i < nf; ++i)
      if (xt[a] == xf[i]) hit = i;
    if (hit >= 0) {
      for (int i = 0; i < nf; ++i) V[a * nf + i] = i == hit ? 1.0 : 0.0;
      continue;
    }
    double den = 0.0;
    for (int i = 0; i < nf; ++i) den += lam[i] / (xt[a] - xf[i]);
    for (int i = 0; i < nf; ++i) V[a * nf + i] = lam[i] / (xt[a] - xf[i]) / den;
  }
}

}  // namespace tag
