// C ABI of libtrixiatmo_gpu.so (declared in include/trixiatmo_gpu.h): handle
// management, device memory, stage sequencing, CUDA-graph capture of the RK
// step and the elements-per-CTA autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "dg2d_kernels.cuh"
#include "cov_kernels.cuh"
#include "dg3d_kernels.cuh"
#include "newton_rainy.cuh"
#include "phys_euler_energy_2d.cuh"
#include "phys_euler_energy_3d.cuh"
#include "phys_moist_2d.cuh"
#include "phys_pt_2d.cuh"
#include "phys_pt_3d.cuh"
#include "phys_ie_2d.cuh"
#include "phys_rainy_2d.cuh"
#include "tag_analysis.cuh"
#include "output_kernels.cuh"

using namespace tag;

// NVTX ranges named after the reference's timer sections of rhs_hyperbolic!
// (src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl:16-67) and the
// stage limiter (src/callbacks_stage/nonlinear_solve_dg.jl:38), joined where
// one kernel does several of them.  Header-only NVTX: inert unless a profiler
// attaches.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
constexpr const char* kNvtxInterface = "prolong2interfaces + interface flux + boundary flux";
constexpr const char* kNvtxElement =
    "volume integral + surface integral + Jacobian + source terms";

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define TAG_CUDA(call)                                                                    \
  do {                                                                                    \
    cudaError_t err_ = (call);                                                            \
    if (err_ != cudaSuccess)                                                              \
      return fail(TAG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_));      \
  } while (0)

struct Ops;

}  // namespace

void tag::set_last_error(const std::string& msg) { g_last_error = msg; }

// Threads of an element-kernel CTA: `items` work items split `div` ways,
// rounded up to whole warps.
inline int cta_threads(int items, int div) { return ((items + div - 1) / div + 31) / 32 * 32; }

struct tag_handle_s {
  int eq = 0, n = 0, nelem = 0, nif = 0, nbd = 0, nv = 0, na = 0;
  int dim = 2, npe = 0, nface = 4, jpn = 4;  // nodes per element, faces, Ja doubles per node
  long nodes = 0;                            // solution nodes (all elements)
  int dt_n = 0;                              // n in dt = cfl 2 / (n max_speed); 1 when
                                             // the kernels reduce n-scaled speeds
  // covariant equations: element groups, geometry, packed element data
  CovParams p_cov{};

  CovGroups h_groups{};
  CovGroups* d_groups = nullptr;
  BasisDev* d_bases = nullptr;
  double *d_aux = nullptr, *d_pk = nullptr;
  int cov_blocks = 0, cov_iblocks = 0, cov_threads = 0;
  size_t cov_smem = 0;
  PhysEnergy2D::Params p_energy{};
  PhysEnergy3D::Params p_energy3d{};
  PhysRainy2D::Params p_rainy{};
  PhysMoist2D::Params p_moist{};
  PhysPT2D::Params p_pt{};
  PhysPT3D::Params p_pt3d{};
  PhysIE2D::Params p_ie{};
  // rainy: Newton stage limiter settings, MLP parameters, statistics counters
  bool has_limiter = false;
  int scheme = TAG_RK_CK2N54;  // time integrator of tag_rk_steps
  NewtonArgs newton{0, 20, 0, 0, 8, 1e-9, nullptr, nullptr, nullptr};
  float* d_mlp = nullptr;
  unsigned long long* d_counters = nullptr;
  int* d_iters = nullptr;
  // the stage limiter inside tag_rk_steps: its start (NewtonArgs::learned)
  // and counters accumulated over the run ([0] updates, [1] fallbacks,
  // [2] not converged), with the number of node solves they cover
  int newton_start = 0;
  unsigned long long* d_run_counters = nullptr;
  long long run_node_solves = 0;
  BasisDev basis{};
  cudaStream_t stream = nullptr;
  double *d_u = nullptr, *d_k = nullptr, *d_Ja = nullptr, *d_invJ = nullptr, *d_xy = nullptr,
         *d_sfv = nullptr, *d_tmp_u = nullptr, *d_tmp_du = nullptr;
  // adaptive SSPRK43: the stage value entering the last stage, error partials
  double *d_u3 = nullptr, *d_err = nullptr;
  int *d_if_e = nullptr, *d_if_f = nullptr, *d_if_flip = nullptr, *d_bd_e = nullptr,
      *d_bd_f = nullptr, *d_bd_kind = nullptr;
  // states of the TAG_BC_DIRICHLET faces [B][n][nv] (allocated when the mesh has
  // such faces; the interface kernel reads them)
  double* d_bvals = nullptr;
  bool need_bvals = false, bvals_set = false;
  int nmembers = 1;
  int* d_member = nullptr;        // [E] or null
  double* d_mscal = nullptr;      // [3 * nmembers]: t, dt, max_speed
  StepCtl* d_ctl = nullptr;
  double* h_pin = nullptr;        // pinned staging, 3 * nmembers + 2 doubles
  unsigned* d_status = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_epb = -1;
  // 3D: mapped host array that the last stage of every tag_rk_steps step also
  // stores the new state into (tag_set_state_sink); armed only while the step
  // graph is captured, so that no other stage sequence writes it
  double* sink = nullptr;
  double* graph_sink = nullptr;
  bool capturing_steps = false;
  bool speed_valid = false;
  int epb = 0;
  // threads of a CTA = its elements' work items / tile_div, rounded up to
  // whole warps (1 or 2: one or two items per thread and phase)
  int tile_div = 1;
  const Ops* ops = nullptr;
  // analysis (allocated by the first analysis call)
  bool an_ready = false;
  int an_m = 0, an_chunks = 0;
  long an_chunk = 0;
  double *d_an_wj = nullptr, *d_an_V = nullptr, *d_an_wa = nullptr, *d_an_rows = nullptr,
         *d_an_erows = nullptr, *d_an_out = nullptr, *d_an_uex = nullptr, *d_an_x = nullptr;
  long* d_an_rng = nullptr;  // [4][nmembers]: node begin, node end, element begin, element end
  size_t an_uex_cap = 0;
};

namespace {

// Launchers for one (physics, n) instantiation.
struct Ops {
  int (*interface)(tag_handle h, const double* u);
  int (*element)(tag_handle h, int mode, double* u, double* du, int stage, bool last, double t);
  int (*max_speed)(tag_handle h, const double* u);
  // optional: u from mapped host memory into d_u with the CFL speeds reduced
  int (*load_state)(tag_handle h, const double* u_mapped);
  int (*init)(int max_smem);
  size_t (*smem_bytes)(int epb);
  int threads_per_element;
  int (*max_threads)();  // per-CTA thread limit of the element kernels (registers)
};

// Largest multiple of 32 threads both element kernels (stage and rhs mode) of
// one instantiation can be launched with.
template <class K1, class K2>
int launch_thread_cap(K1 k1, K2 k2, int& cap) {
  cudaFuncAttributes a, b;
  TAG_CUDA(cudaFuncGetAttributes(&a, k1));
  TAG_CUDA(cudaFuncGetAttributes(&b, k2));
  cap = (std::min(a.maxThreadsPerBlock, b.maxThreadsPerBlock) / 32) * 32;
  return TAG_OK;
}

template <class Phys>
const typename Phys::Params& params_of(tag_handle h);
template <>
const PhysEnergy2D::Params& params_of<PhysEnergy2D>(tag_handle h) {
  return h->p_energy;
}
template <>
const PhysEnergy3D::Params& params_of<PhysEnergy3D>(tag_handle h) {
  return h->p_energy3d;
}
template <>
const PhysRainy2D::Params& params_of<PhysRainy2D>(tag_handle h) {
  return h->p_rainy;
}
template <>
const PhysMoist2D::Params& params_of<PhysMoist2D>(tag_handle h) {
  return h->p_moist;
}
template <>
const PhysPT2D::Params& params_of<PhysPT2D>(tag_handle h) {
  return h->p_pt;
}
template <>
const PhysPT3D::Params& params_of<PhysPT3D>(tag_handle h) {
  return h->p_pt3d;
}
template <>
const PhysIE2D::Params& params_of<PhysIE2D>(tag_handle h) {
  return h->p_ie;
}

template <class Phys, int n, int VOL = kVolFluxDiff>
struct OpsImpl {
  using S = ElemSmem<Phys, n>;
  static int interface(tag_handle h, const double* u) {
    const int total = (h->nif + h->nbd) * n;
    if (total == 0) return TAG_OK;
    const int threads = 256;
    if (h->need_bvals && !h->bvals_set)
      return fail(TAG_E_INVALID, "Dirichlet boundary faces without states (tag_set_boundary_values)");
    k_interface<Phys, n><<<(total + threads - 1) / threads, threads, 0, h->stream>>>(
        params_of<Phys>(h), u, h->d_Ja, h->d_invJ, h->d_if_e, h->d_if_f, h->d_if_flip, h->nif,
        h->d_bd_e, h->d_bd_f, h->d_bd_kind, h->nbd, h->d_sfv, h->d_bvals);
    TAG_CUDA(cudaGetLastError());
    return TAG_OK;
  }
  static int element(tag_handle h, int mode, double* u, double* du, int stage, bool last,
                     double t) {
    const int epb = h->epb > 0 ? h->epb : 4;
    const int blocks = (h->nelem + epb - 1) / epb;
    const int threads = std::min(cap(), cta_threads(epb * S::TPE, h->tile_div));
    const size_t smem = S::bytes(epb);
    StageArgs st{};
    st.member = h->d_member;
    st.xy = h->d_xy;
    st.t_rhs = t;
    if (mode == kModeStage) {
      set_stage(st, h->scheme, stage);
      st.t_member = h->d_mscal;
      st.dt = h->d_mscal + h->nmembers;
      st.max_speed = last ? h->d_mscal + 2 * h->nmembers : nullptr;
      st.sink = last && h->capturing_steps ? h->sink : nullptr;
      k_element<Phys, n, kModeStage, VOL><<<blocks, threads, smem, h->stream>>>(
          params_of<Phys>(h), h->basis, u, du, h->d_k, h->d_Ja, h->d_invJ, h->d_sfv, h->nelem,
          epb, st, h->d_status);
    } else {
      k_element<Phys, n, kModeRhs, VOL><<<blocks, threads, smem, h->stream>>>(
          params_of<Phys>(h), h->basis, u, du, h->d_k, h->d_Ja, h->d_invJ, h->d_sfv, h->nelem,
          epb, st, h->d_status);
    }
    TAG_CUDA(cudaGetLastError());
    return TAG_OK;
  }
  static int max_speed(tag_handle h, const double* u) {
    using K = MaxSpeedTile<n>;
    k_max_speed<Phys, n><<<(h->nelem + K::EPB - 1) / K::EPB, K::T, 0, h->stream>>>(
        params_of<Phys>(h), u, h->d_Ja, h->d_invJ, h->nelem, h->d_member,
        h->d_mscal + 2 * h->nmembers);
    TAG_CUDA(cudaGetLastError());
    return TAG_OK;
  }
  // opt the element kernels into the device's full dynamic shared memory once,
  // outside any stream capture
  static int init(int max_smem) {
    TAG_CUDA(cudaFuncSetAttribute(k_element<Phys, n, kModeStage, VOL>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
    TAG_CUDA(cudaFuncSetAttribute(k_element<Phys, n, kModeRhs, VOL>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
    return launch_thread_cap(k_element<Phys, n, kModeStage, VOL>, k_element<Phys, n, kModeRhs, VOL>,
                             cap());
  }
  static int& cap() {
    static int c = 1024;
    return c;
  }
  static int max_threads() { return cap(); }
  static size_t smem_bytes(int epb) { return S::bytes(epb); }
  static const Ops* get() {
    static const Ops ops{&interface, &element, &max_speed, nullptr, &init, &smem_bytes,
                         S::TPE, &max_threads};
    return &ops;
  }
};

template <class Phys, int VOL = kVolFluxDiff>
const Ops* ops_for_n(int n) {
  switch (n) {
    case 2: return OpsImpl<Phys, 2, VOL>::get();
    case 3: return OpsImpl<Phys, 3, VOL>::get();
    case 4: return OpsImpl<Phys, 4, VOL>::get();
    case 5: return OpsImpl<Phys, 5, VOL>::get();
    case 6: return OpsImpl<Phys, 6, VOL>::get();
    case 7: return OpsImpl<Phys, 7, VOL>::get();
    case 8: return OpsImpl<Phys, 8, VOL>::get();
    default: return nullptr;
  }
}

template <class Phys, int n>
struct OpsImpl3D {
  using S = ElemSmem3D<Phys, n>;
  static int interface(tag_handle h, const double* u) {
    const int total = (h->nif + h->nbd) * n * n;
    if (total == 0) return TAG_OK;
    k_interface3d<Phys, n><<<(total + 255) / 256, 256, 0, h->stream>>>(
        params_of<Phys>(h), u, h->d_Ja, h->d_invJ, h->d_if_e, h->d_if_f, h->d_if_flip, h->nif,
        h->d_bd_e, h->d_bd_f, h->nbd, h->d_sfv);
    TAG_CUDA(cudaGetLastError());
    return TAG_OK;
  }
  static int element(tag_handle h, int mode, double* u, double* du, int stage, bool last,
                     double) {
    const int epb = h->epb > 0 ? h->epb : 1;
    const int blocks = (h->nelem + epb - 1) / epb;
    const int threads = std::min(cap(), cta_threads(epb * S::TPE, h->tile_div));
    const size_t smem = S::bytes(epb);
    StageArgs st{};
    st.member = h->d_member;
    if (mode == kModeStage) {
      set_stage(st, h->scheme, stage);
      st.dt = h->d_mscal + h->nmembers;
      st.max_speed = last ? h->d_mscal + 2 * h->nmembers : nullptr;
      st.sink = last && h->capturing_steps ? h->sink : nullptr;
      k_element3d<Phys, n, kModeStage><<<blocks, threads, smem, h->stream>>>(
          params_of<Phys>(h), h->basis, u, du, h->d_k, h->d_Ja, h->d_invJ, h->d_sfv, h->nelem,
          epb, st, h->d_status);
    } else {
      k_element3d<Phys, n, kModeRhs><<<blocks, threads, smem, h->stream>>>(
          params_of<Phys>(h), h->basis, u, du, h->d_k, h->d_Ja, h->d_invJ, h->d_sfv, h->nelem,
          epb, st, h->d_status);
    }
    TAG_CUDA(cudaGetLastError());
    return TAG_OK;
  }
  static int max_speed(tag_handle h, const double* u) { return speeds(h, u, nullptr); }
  // the state from mapped host memory into the device copy, speeds on the way
  static int load_state(tag_handle h, const double* u_mapped) {
    return speeds(h, u_mapped, h->d_u);
  }
  static int speeds(tag_handle h, const double* u, double* copy_to) {
    const int threads = 256, warps = threads / 32;  // one warp per element
    k_max_speed3d<Phys, n><<<(h->nelem + warps - 1) / warps, threads, 0, h->stream>>>(
        params_of<Phys>(h), u, h->d_Ja, h->d_invJ, h->nelem, h->d_member,
        h->d_mscal + 2 * h->nmembers, copy_to);
    TAG_CUDA(cudaGetLastError());
    return TAG_OK;
  }
  static int init(int max_smem) {
    TAG_CUDA(cudaFuncSetAttribute(k_element3d<Phys, n, kModeStage>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
    TAG_CUDA(cudaFuncSetAttribute(k_element3d<Phys, n, kModeRhs>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
    return launch_thread_cap(k_element3d<Phys, n, kModeStage>, k_element3d<Phys, n, kModeRhs>,
                             cap());
  }
  static int& cap() {
    static int c = 1024;
    return c;
  }
  static int max_threads() { return cap(); }
  static size_t smem_bytes(int epb) { return S::bytes(epb); }
  static const Ops* get() {
    static const Ops ops{&interface, &element, &max_speed, &load_state, &init, &smem_bytes,
                         S::TPE, &max_threads};
    return &ops;
  }
};

template <class Phys>
const Ops* ops3d_for_n(int n) {
  switch (n) {
    case 3: return OpsImpl3D<Phys, 3>::get();
    case 4: return OpsImpl3D<Phys, 4>::get();
    case 5: return OpsImpl3D<Phys, 5>::get();
    case 6: return OpsImpl3D<Phys, 6>::get();
    case 7: return OpsImpl3D<Phys, 7>::get();
    case 8: return OpsImpl3D<Phys, 8>::get();
    default: return nullptr;
  }
}

template <class T>
int upload(T** dst, const T* src, size_t count, cudaStream_t s) {
  if (count == 0) return TAG_OK;
  TAG_CUDA(cudaMalloc(dst, count * sizeof(T)));
  if (src) {
    TAG_CUDA(cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, s));
  } else {
    TAG_CUDA(cudaMemsetAsync(*dst, 0, count * sizeof(T), s));
  }
  return TAG_OK;
}

// Julia column-major [n, n] -> row-major Dsplit[a * n + b] = derivative_split[a, b]
void load_basis(BasisDev& b, const double* dsplit_colmajor, const double* w, int n) {
  std::memset(&b, 0, sizeof(b));
  for (int a = 0; a < n; ++a)
    for (int c = 0; c < n; ++c) b.Ds[a * n + c] = dsplit_colmajor[a + n * c];
  b.winv0 = 1.0 / w[0];
  b.winvN = 1.0 / w[n - 1];
  // D_hat = -M^{-1} D^T M from D_split = 2 D - M^{-1} B:
  //   D[a][c] = (Ds[a][c] + (M^{-1} B)[a][c]) / 2,  D_hat[a][c] = -D[c][a] w_c / w_a
  for (int a = 0; a < n; ++a)
    for (int c = 0; c < n; ++c) {
      double dca = b.Ds[c * n + a];
      if (c == a && c == 0) dca -= 1.0 / w[0];
      if (c == a && c == n - 1) dca += 1.0 / w[n - 1];
      b.Dh[a * n + c] = -0.5 * dca * w[c] / w[a];
    }
}

MemberScalars member_scalars(tag_handle h) {
  return MemberScalars{h->d_mscal, h->d_mscal + h->nmembers, h->d_mscal + 2 * h->nmembers};
}

int begin_step(tag_handle h) {
  k_begin_step<<<(h->nmembers + 127) / 128, 128, 0, h->stream>>>(member_scalars(h), h->d_ctl,
                                                                  h->nmembers, h->dt_n);
  TAG_CUDA(cudaGetLastError());
  return TAG_OK;
}

int reset_and_reduce_speeds(tag_handle h) {
  TAG_CUDA(cudaMemsetAsync(h->d_mscal + 2 * h->nmembers, 0, sizeof(double) * h->nmembers,
                           h->stream));
  return h->ops->max_speed(h, h->d_u);
}

int stage_sequence(tag_handle h) {
  // one RK step: begin-step scalars, then one (interface, element) pair per stage
  int rc0 = begin_step(h);
  if (rc0) return rc0;
  const int ns = rk_stages(h->scheme);
  for (int s = 0; s < ns; ++s) {
    int rc = h->ops->interface(h, h->d_u);
    if (rc) return rc;
    // with a stage limiter the next step's CFL speed is taken from the
    // limited state, after the last Newton solve, not inside the element kernel
    rc = h->ops->element(h, kModeStage, h->d_u, nullptr, s, s == ns - 1 && !h->has_limiter, 0.0);
    if (rc) return rc;
    if (h->has_limiter) {
      // stage limiter: saturation Newton solve on every node (warm start)
      const long nodes = (long)h->nodes;
      NewtonArgs a = h->newton;
      a.learned = h->newton_start;
      a.mlp = h->d_mlp;
      a.iters = nullptr;
      a.counters = h->d_run_counters;
      a.sink = s == ns - 1 && h->capturing_steps ? h->sink : nullptr;  // the limited state
      TAG_CUDA(launch_newton_rainy(h->d_u, nodes, a, h->d_status, h->stream));
      if (s == ns - 1) {
        rc = h->ops->max_speed(h, h->d_u);
        if (rc) return rc;
      }
    }
  }
  return TAG_OK;
}

int build_graph(tag_handle h) {
  const int key = h->epb * 8 + h->tile_div;
  if (h->graph && h->graph_epb == key && h->graph_sink == h->sink) return TAG_OK;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  cudaGraph_t g;
  TAG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  h->capturing_steps = true;
  int rc = stage_sequence(h);
  h->capturing_steps = false;
  cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
  if (rc) return rc;
  if (e2 != cudaSuccess) return fail(TAG_E_CUDA, cudaGetErrorString(e2));
  TAG_CUDA(cudaGraphInstantiate(&h->graph, g, 0));
  cudaGraphDestroy(g);
  h->graph_epb = key;
  h->graph_sink = h->sink;
  return TAG_OK;
}

// Times the element kernel (rhs mode, on the state `u`) for candidate tiles
// and keeps the fastest: elements per CTA (the shared-memory tile, each
// element's state, metric terms and accumulators staged once) times threads
// per CTA (one or two work items per thread and phase).  The trial launches'
// status bits are discarded.
int autotune(tag_handle h, const double* u) {
  if (h->epb > 0) return TAG_OK;
  int dev;
  TAG_CUDA(cudaGetDevice(&dev));
  int max_smem = 0;
  TAG_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (!h->d_tmp_du) TAG_CUDA(cudaMalloc(&h->d_tmp_du, sizeof(double) * h->nodes * h->nv));
  cudaEvent_t a, b;
  TAG_CUDA(cudaEventCreate(&a));
  TAG_CUDA(cudaEventCreate(&b));
  int best = 1, best_div = 1;
  float best_ms = 1e30f;
  const int cands[] = {1, 2, 3, 4, 6, 8, 12, 16};
  for (int trial = 0; trial < 16; ++trial) {
    const int c = cands[trial >> 1], div = 1 + (trial & 1);
    if ((size_t)h->ops->smem_bytes(c) > (size_t)max_smem) continue;
    if (c * h->ops->threads_per_element > h->ops->max_threads() && c > 1) continue;
    if (div == 2 && c * h->ops->threads_per_element < 128) continue;
    h->epb = c;
    h->tile_div = div;
    double* uu = const_cast<double*>(u);
    int rc = h->ops->interface(h, uu);
    if (rc) return rc;
    for (int w = 0; w < 2; ++w) {
      rc = h->ops->element(h, kModeRhs, uu, h->d_tmp_du, 0, false, 0.0);
      if (rc) return rc;
    }
    TAG_CUDA(cudaEventRecord(a, h->stream));
    for (int r = 0; r < 5; ++r) h->ops->element(h, kModeRhs, uu, h->d_tmp_du, 0, false, 0.0);
    TAG_CUDA(cudaEventRecord(b, h->stream));
    TAG_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    TAG_CUDA(cudaEventElapsedTime(&ms, a, b));
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
      best_div = div;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  h->epb = best;
  h->tile_div = best_div;
  TAG_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned), h->stream));
  return TAG_OK;
}

__global__ void k_fp64_probe(double* out, int iters, double seed) {
  double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4,
         a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double b = 0.999999999, c = 1.0e-9;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// ---- covariant equations (element groups of possibly different degree) ------
int cov_interface(tag_handle h, const double* u) {
  if (h->cov_iblocks == 0) return TAG_OK;
  k_cov_interface<<<h->cov_iblocks, 256, 0, h->stream>>>(h->p_cov, h->d_groups, u, h->d_aux,
                                                         h->d_if_e, h->d_if_f, h->d_if_flip,
                                                         h->d_sfv);
  TAG_CUDA(cudaGetLastError());
  return TAG_OK;
}

int cov_element(tag_handle h, int mode, double* u, double* du, int stage, bool last, double) {
  StageArgs st{};
  st.member = h->d_member;
  if (mode == kModeStage) {
    set_stage(st, h->scheme, stage);
    st.t_member = h->d_mscal;
    st.dt = h->d_mscal + h->nmembers;
    st.max_speed = last ? h->d_mscal + 2 * h->nmembers : nullptr;
    st.sink = last && h->capturing_steps ? h->sink : nullptr;
    auto kern = h->p_cov.volume == 0 ? k_cov_element<kModeStage, 0> : k_cov_element<kModeStage, 1>;
    kern<<<h->cov_blocks, h->cov_threads, h->cov_smem, h->stream>>>(
        h->p_cov, h->d_groups, h->d_bases, u, du, h->d_k, h->d_pk, h->d_sfv, st, h->d_status);
  } else {
    auto kern = h->p_cov.volume == 0 ? k_cov_element<kModeRhs, 0> : k_cov_element<kModeRhs, 1>;
    kern<<<h->cov_blocks, h->cov_threads, h->cov_smem, h->stream>>>(
        h->p_cov, h->d_groups, h->d_bases, u, du, h->d_k, h->d_pk, h->d_sfv, st, h->d_status);
  }
  TAG_CUDA(cudaGetLastError());
  return TAG_OK;
}

int cov_max_speed(tag_handle h, const double* u) {
  k_cov_max_speed<<<(h->nelem + 127) / 128, 128, 0, h->stream>>>(
      h->p_cov, h->d_groups, u, h->d_pk, h->d_member, h->d_mscal + 2 * h->nmembers, h->nelem);
  TAG_CUDA(cudaGetLastError());
  return TAG_OK;
}

int cov_init(int max_smem) {
  TAG_CUDA(cudaFuncSetAttribute(k_cov_element<kModeStage, 0>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  TAG_CUDA(cudaFuncSetAttribute(k_cov_element<kModeRhs, 0>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  TAG_CUDA(cudaFuncSetAttribute(k_cov_element<kModeStage, 1>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  TAG_CUDA(cudaFuncSetAttribute(k_cov_element<kModeRhs, 1>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  return TAG_OK;
}

size_t cov_smem_bytes(int) { return 0; }
int cov_max_threads() { return 256; }

const Ops kCovOps{&cov_interface, &cov_element, &cov_max_speed, nullptr, &cov_init,
                  &cov_smem_bytes, 256, &cov_max_threads};

// Flux options of a covariant member configuration; returns the reason it is
// rejected, or null.
const char* cov_params(const tag_config* c, CovParams& P, double& omega) {
  if (c->equations != TAG_EQ_COVARIANT_SWE) return "every member must use the covariant equations";
  P = CovParams{};
  P.g = c->params[0];
  omega = c->params[1];
  P.split = c->params[2] != 0.0;
  P.vol_nc = (int)c->params[3];
  P.surf_nc = (int)c->params[4];
  switch (c->volume_flux) {
    case TAG_VF_WEAK_FORM: P.volume = 0; break;
    case TAG_VF_COV_CENTRAL: P.volume = 1; P.vol_sym = 0; break;
    case TAG_VF_COV_EC: P.volume = 1; P.vol_sym = 1; break;
    default: return "unsupported volume flux for the covariant equations";
  }
  switch (c->surface_flux) {
    case TAG_SF_LAX_FRIEDRICHS: P.surf_sym = 0; P.surf_diss = 1; break;
    case TAG_SF_COV_CENTRAL: P.surf_sym = 0; P.surf_diss = 0; break;
    case TAG_SF_COV_EC: P.surf_sym = 1; P.surf_diss = 0; break;
    case TAG_SF_COV_EC_LLF: P.surf_sym = 1; P.surf_diss = 1; break;
    default: return "unsupported surface flux for the covariant equations";
  }
  if (P.vol_nc < 0 || P.vol_nc > 1 || P.surf_nc < 0 || P.surf_nc > 2)
    return "unsupported nonconservative flux id";
  if ((P.vol_nc || P.surf_nc || P.vol_sym) && !P.split)
    return "flux_ec and the nonconservative fluxes need the split form";
  if (P.volume == 0 && P.vol_nc) return "the weak form has no nonconservative volume term";
  if (!(P.g > 0.0)) return "gravity must be positive";
  return nullptr;
}

int create_cov(const tag_config* cfgs, int m, tag_handle* out) {
  if (m < 1) return fail(TAG_E_INVALID, "no members");
  CovParams P;
  double omega = 0.0;
  if (const char* why = cov_params(&cfgs[0], P, omega)) return fail(TAG_E_INVALID, why);
  for (int k = 1; k < m; ++k) {
    CovParams Q;
    double om2;
    if (const char* why = cov_params(&cfgs[k], Q, om2)) return fail(TAG_E_INVALID, why);
    if (std::memcmp(&Q, &P, sizeof(P)) != 0 || om2 != omega)
      return fail(TAG_E_INVALID, "members must share equations and fluxes");
  }
  long nodes = 0, sf = 0;
  int nelem = 0, nif = 0, max_n = 0;
  for (int k = 0; k < m; ++k) {
    const tag_config* c = &cfgs[k];
    const int n = c->polydeg + 1;
    if (n < 2 || n > kMaxNodes) return fail(TAG_E_INVALID, "polydeg out of range 1..7");
    if (c->nelements <= 0 || c->ninterfaces < 0 || c->nboundaries != 0)
      return fail(TAG_E_INVALID, "bad mesh sizes (the covariant solver has no boundaries)");
    if (!c->derivative_split || !c->weights || !c->aux_node_vars || !c->node_coordinates)
      return fail(TAG_E_INVALID, "missing basis, aux_node_vars or node_coordinates");
    for (int i = 0; i < c->ninterfaces; ++i) {
      for (int sd = 0; sd < 2; ++sd) {
        const int e = c->interface_elements[2 * i + sd], f = c->interface_faces[2 * i + sd];
        if (e < 0 || e >= c->nelements || f < 0 || f > 3)
          return fail(TAG_E_INVALID, "interface index out of range");
      }
      const int o = c->interface_flip ? c->interface_flip[i] : 0;
      if (o < 0 || o > 1) return fail(TAG_E_INVALID, "interface orientation out of range");
    }
    nodes += (long)c->nelements * n * n;
    sf += (long)c->nelements * 4 * n * 3;
    nelem += c->nelements;
    nif += c->ninterfaces;
    max_n = std::max(max_n, n);
  }
  // groups: runs of members with the same degree
  CovGroups G{};
  std::vector<BasisDev> bases;
  std::vector<double> aux((size_t)nodes * 26), xyz((size_t)nodes * 3);
  std::vector<int> ie((size_t)2 * nif), ifc((size_t)2 * nif), ifl((size_t)nif), member(nelem);
  long node_off = 0, sf_off = 0;
  int e_off = 0, if_off = 0, blk = 0, iblk = 0;
  size_t smem = 0;
  for (int k = 0; k < m; ++k) {
    const tag_config* c = &cfgs[k];
    const int n = c->polydeg + 1, nn = n * n;
    if (G.count == 0 || G.g[G.count - 1].n != n) {
      if (G.count == kCovMaxGroups) return fail(TAG_E_INVALID, "too many degree runs (max 64)");
      CovGroup& g = G.g[G.count++];
      g.n = n;
      g.e0 = e_off;
      g.ne = 0;
      g.node0 = node_off;
      g.sf0 = sf_off;
      g.if0 = if_off;
      g.nif = 0;
      g.epb = std::max(1, 256 / nn);
      g.basis = (int)bases.size();
      BasisDev b;
      load_basis(b, c->derivative_split, c->weights, n);
      bases.push_back(b);
    }
    CovGroup& g = G.g[G.count - 1];
    const size_t q0 = (size_t)node_off;
    std::memcpy(&aux[q0 * 26], c->aux_node_vars, sizeof(double) * (size_t)c->nelements * nn * 26);
    std::memcpy(&xyz[q0 * 3], c->node_coordinates, sizeof(double) * (size_t)c->nelements * nn * 3);
    for (int i = 0; i < c->ninterfaces; ++i) {
      ie[2 * (if_off + i)] = c->interface_elements[2 * i] + e_off;
      ie[2 * (if_off + i) + 1] = c->interface_elements[2 * i + 1] + e_off;
      ifc[2 * (if_off + i)] = c->interface_faces[2 * i];
      ifc[2 * (if_off + i) + 1] = c->interface_faces[2 * i + 1];
      ifl[if_off + i] = c->interface_flip ? c->interface_flip[i] : 0;
    }
    for (int e = 0; e < c->nelements; ++e) member[e_off + e] = k;
    g.ne += c->nelements;
    g.nif += c->ninterfaces;
    node_off += (long)c->nelements * nn;
    sf_off += (long)c->nelements * 4 * n * 3;
    e_off += c->nelements;
    if_off += c->ninterfaces;
  }
  for (int k = 0; k < G.count; ++k) {
    CovGroup& g = G.g[k];
    g.blk0 = blk;
    blk += (g.ne + g.epb - 1) / g.epb;
    g.iblk0 = iblk;
    iblk += (g.nif * g.n + 255) / 256;
    smem = std::max(smem, sizeof(double) * (size_t)g.epb * cov_elem_doubles(g.n));
  }
  tag_handle h = new tag_handle_s();
  h->eq = TAG_EQ_COVARIANT_SWE;
  h->n = max_n;
  h->nelem = nelem;
  h->nif = nif;
  h->nbd = 0;
  h->nmembers = m;
  h->dim = 2;
  h->nface = 4;
  h->npe = max_n * max_n;
  h->jpn = 0;
  h->nodes = nodes;
  h->dt_n = 1;  // the kernels reduce n-scaled speeds
  h->nv = 3;
  h->na = 3;
  h->p_cov = P;
  h->h_groups = G;
  h->cov_blocks = blk;
  h->cov_iblocks = iblk;
  h->cov_threads = 256;
  h->cov_smem = smem + sizeof(BasisDev);
  h->epb = 1;  // tiling is per group; no autotuning
  h->ops = &kCovOps;
  auto cleanup = [&](int rc) {
    tag_destroy(h);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(fail(TAG_E_CUDA, "stream create failed"));
  int rc = TAG_OK;
  if ((rc = upload(&h->d_u, (const double*)nullptr, (size_t)nodes * 3, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_k, (const double*)nullptr, (size_t)nodes * 3, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_aux, aux.data(), aux.size(), h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_xy, xyz.data(), xyz.size(), h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_pk, (const double*)nullptr, (size_t)nodes * kPack, h->stream)))
    return cleanup(rc);
  if ((rc = upload(&h->d_sfv, (const double*)nullptr, (size_t)sf, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_if_e, ie.data(), ie.size(), h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_if_f, ifc.data(), ifc.size(), h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_if_flip, ifl.data(), ifl.size(), h->stream))) return cleanup(rc);
  if (m > 1)
    if ((rc = upload(&h->d_member, member.data(), member.size(), h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_groups, &h->h_groups, 1, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_bases, bases.data(), bases.size(), h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_mscal, (const double*)nullptr, (size_t)3 * m, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_ctl, (const StepCtl*)nullptr, 1, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_status, (const unsigned*)nullptr, 1, h->stream))) return cleanup(rc);
  if (cudaMallocHost(&h->h_pin, sizeof(double) * (3 * m + 2)) != cudaSuccess)
    return cleanup(fail(TAG_E_CUDA, "pinned alloc failed"));
  k_cov_pack<<<(unsigned)((nodes + 255) / 256), 256, 0, h->stream>>>(h->d_aux, h->d_xy, nodes,
                                                                      omega, h->d_pk);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess)
    return cleanup(fail(TAG_E_CUDA, "upload failed"));
  {
    int dev = 0, max_smem = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (h->cov_smem > (size_t)max_smem) return cleanup(fail(TAG_E_INVALID, "tile too large"));
    if ((rc = h->ops->init(max_smem))) return cleanup(rc);
  }
  *out = h;
  return TAG_OK;
}

// Supported (equations, volume flux, surface flux, source) combinations;
// returns the reason a configuration is rejected, or null.
const char* check_equations(const tag_config* cfg) {
  const int vf = cfg->volume_flux, sf = cfg->surface_flux;
  switch (cfg->equations) {
    case TAG_EQ_EULER_ENERGY_2D:
    case TAG_EQ_EULER_ENERGY_3D:
      if (vf != TAG_VF_RANOCHA_WARUSZEWSKI || sf != TAG_SF_LMARS)
        return "unsupported flux combination";
      return nullptr;
    case TAG_EQ_RAINY_2D: {
      if ((vf != TAG_VF_EC_RAIN && vf != TAG_VF_WEAK_FORM) ||
          (sf != TAG_SF_LAX_FRIEDRICHS && sf != TAG_SF_LMARS))
        return "unsupported flux combination for the rainy equations";
      const double k = cfg->params[0];
      if (k != TAG_SRC_RAINY && k != TAG_SRC_RAINY_CONVERGENCE && k != TAG_SRC_RAINY_NO_PHASE_CHANGE)
        return "unsupported source kind for the rainy equations";
      if (k == TAG_SRC_RAINY_CONVERGENCE && !cfg->node_coordinates)
        return "the convergence-test source needs node coordinates";
      return nullptr;
    }
    case TAG_EQ_MOIST_EULER_2D: {
      if ((vf != TAG_VF_CHANDRASHEKAR && vf != TAG_VF_WEAK_FORM) ||
          (sf != TAG_SF_LMARS && sf != TAG_SF_LAX_FRIEDRICHS && sf != TAG_SF_CHANDRASHEKAR))
        return "unsupported flux combination for the moist equations";
      const double k = cfg->params[6];
      if (k != 0 && k != TAG_SRC_GEOPOTENTIAL && k != TAG_SRC_MOIST_BUBBLE &&
          k != TAG_SRC_MOIST_CONVERGENCE_DRY && k != TAG_SRC_MOIST_CONVERGENCE &&
          k != TAG_SRC_MOIST_GRAVITY_WAVE)
        return "unsupported source kind for the moist equations";
      if ((k == TAG_SRC_MOIST_CONVERGENCE_DRY || k == TAG_SRC_MOIST_CONVERGENCE ||
           k == TAG_SRC_MOIST_GRAVITY_WAVE) && !cfg->node_coordinates)
        return "this source needs node coordinates";
      if (sf == TAG_SF_LMARS && !(cfg->params[5] > 0.0))
        return "FluxLMARS needs a positive speed of sound";
      return nullptr;
    }
    case TAG_EQ_POTENTIAL_TEMPERATURE_2D:
    case TAG_EQ_POTENTIAL_TEMPERATURE_3D: {
      const bool ec_surface =
          sf == TAG_SF_PT_EC && cfg->equations == TAG_EQ_POTENTIAL_TEMPERATURE_2D;
      const bool kg = vf == TAG_VF_PT_KG && cfg->equations == TAG_EQ_POTENTIAL_TEMPERATURE_3D;
      if ((vf != TAG_VF_PT_TEC && vf != TAG_VF_PT_EC && vf != TAG_VF_PT_ETEC && !kg) ||
          (sf != TAG_SF_LMARS && !ec_surface))
        return "unsupported flux combination for the potential-temperature equations";
      const double k = cfg->params[4];
      if (k != 0 && k != 1 && k != 2) return "unsupported nonconservative gravity term";
      if (ec_surface) {
        const double s = cfg->params[7];
        if (s != 0 && s != 1 && s != 2 && s != 3) return "unsupported surface gravity term";
      } else if (!(cfg->params[3] > 0.0)) {
        return "FluxLMARS needs a positive speed of sound";
      }
      return nullptr;
    }
    case TAG_EQ_INTERNAL_ENERGY_2D:
      if (vf != TAG_VF_IE_ETEC || sf != TAG_SF_IE_ES)
        return "unsupported flux combination for the internal-energy equations";
      return nullptr;
    default:
      return "unsupported equations id";
  }
}

bool boundary_kind_ok(int eq, int kind) {
  switch (eq) {
    case TAG_EQ_EULER_ENERGY_2D:
    case TAG_EQ_MOIST_EULER_2D:
    case TAG_EQ_POTENTIAL_TEMPERATURE_2D:
      return kind == TAG_BC_SLIP_WALL_STRUCTURED || kind == TAG_BC_SLIP_WALL_NORMAL ||
             kind == TAG_BC_DIRICHLET;
    case TAG_EQ_EULER_ENERGY_3D:
    case TAG_EQ_POTENTIAL_TEMPERATURE_3D: return kind == TAG_BC_SLIP_WALL_NORMAL;
    case TAG_EQ_RAINY_2D:
      return kind == TAG_BC_SIMPLE_SLIP_WALL || kind == TAG_BC_SLIP_WALL_STRUCTURED ||
             kind == TAG_BC_SLIP_WALL_NORMAL || kind == TAG_BC_DIRICHLET;
    case TAG_EQ_INTERNAL_ENERGY_2D:
      return kind == TAG_BC_SLIP_WALL_NORMAL || kind == TAG_BC_DIRICHLET;
    default: return false;
  }
}

// ---- analysis ---------------------------------------------------------------
int analysis_phys(tag_handle h) {
  switch (h->eq) {
    case TAG_EQ_EULER_ENERGY_2D: return kAnEnergy2D;
    case TAG_EQ_EULER_ENERGY_3D: return kAnEnergy3D;
    case TAG_EQ_RAINY_2D: return kAnRainy2D;
    case TAG_EQ_MOIST_EULER_2D: return kAnMoist2D;
    case TAG_EQ_POTENTIAL_TEMPERATURE_2D: return kAnPT2D;
    case TAG_EQ_POTENTIAL_TEMPERATURE_3D: return kAnPT3D;
    case TAG_EQ_INTERNAL_ENERGY_2D: return kAnIE2D;
    default: return kAnCov;
  }
}

const void* analysis_params(tag_handle h) {
  switch (h->eq) {
    case TAG_EQ_EULER_ENERGY_2D: return &h->p_energy;
    case TAG_EQ_EULER_ENERGY_3D: return &h->p_energy3d;
    case TAG_EQ_RAINY_2D: return &h->p_rainy;
    case TAG_EQ_MOIST_EULER_2D: return &h->p_moist;
    case TAG_EQ_POTENTIAL_TEMPERATURE_2D: return &h->p_pt;
    case TAG_EQ_POTENTIAL_TEMPERATURE_3D: return &h->p_pt3d;
    case TAG_EQ_INTERNAL_ENERGY_2D: return &h->p_ie;
    default: return &h->p_cov;
  }
}

// Node and element ranges of the members, rng[4][nmembers]: node begin,
// node end, element begin, element end (each member one contiguous range).
int member_ranges(tag_handle h, std::vector<long>& rng) {
  const bool cov = h->eq == TAG_EQ_COVARIANT_SWE;
  const int M = h->nmembers, E = h->nelem;
  std::vector<int> member(E, 0);
  if (h->d_member) {
    TAG_CUDA(cudaMemcpyAsync(member.data(), h->d_member, sizeof(int) * E, cudaMemcpyDeviceToHost,
                             h->stream));
    TAG_CUDA(cudaStreamSynchronize(h->stream));
  }
  std::vector<long> enode(E + 1);
  if (cov) {
    for (int k = 0; k < h->h_groups.count; ++k) {
      const CovGroup& g = h->h_groups.g[k];
      for (int e = g.e0; e < g.e0 + g.ne; ++e) enode[e] = g.node0 + (long)(e - g.e0) * g.n * g.n;
    }
  } else {
    for (int e = 0; e < E; ++e) enode[e] = (long)e * h->npe;
  }
  enode[E] = h->nodes;
  rng.assign(4 * (size_t)M, -1);
  long *nb = rng.data(), *ne_ = nb + M, *eb = nb + 2 * M, *ee = nb + 3 * M;
  for (int e = 0; e < E; ++e) {
    const int m = member[e];
    if (m < 0 || m >= M) return fail(TAG_E_INVALID, "element member out of range");
    if (eb[m] < 0)
      eb[m] = e;
    else if (ee[m] != e)
      return fail(TAG_E_INVALID, "each member must be one contiguous element range");
    ee[m] = e + 1;
  }
  for (int m = 0; m < M; ++m) {
    if (eb[m] < 0) return fail(TAG_E_INVALID, "a member has no elements");
    nb[m] = enode[eb[m]];
    ne_[m] = enode[ee[m]];
  }
  return TAG_OK;
}

// Member node / element ranges, quadrature weights x |J| per node, the
// analysis interpolation (Cartesian meshes) and reduction scratch; once per
// handle.
int analysis_setup(tag_handle h) {
  if (h->an_ready) return TAG_OK;
  const bool cov = h->eq == TAG_EQ_COVARIANT_SWE;
  const int M = h->nmembers, E = h->nelem;
  std::vector<long> rng;
  int rc = member_ranges(h, rng);
  if (rc) return rc;
  long lmax = 1;
  for (int m = 0; m < M; ++m) lmax = std::max(lmax, rng[M + m] - rng[m]);
  rc = upload(&h->d_an_rng, rng.data(), rng.size(), h->stream);
  if (rc) return rc;
  TAG_CUDA(cudaMalloc(&h->d_an_wj, sizeof(double) * h->nodes));
  std::vector<double*> tmp;
  auto solution_weights = [&](int n, double** dw) {
    std::vector<double> x(n), w(n);
    lgl_nodes_weights(n - 1, x.data(), w.data());
    *dw = nullptr;
    const int r = upload(dw, w.data(), (size_t)n, h->stream);
    tmp.push_back(*dw);
    return r;
  };
  if (cov) {
    for (int k = 0; k < h->h_groups.count && !rc; ++k) {
      const CovGroup& g = h->h_groups.g[k];
      double* dw;
      if ((rc = solution_weights(g.n, &dw))) break;
      rc = analysis_weights_covariant(h->d_aux, dw, g.n, g.node0, (long)g.ne * g.n * g.n,
                                      h->d_an_wj, h->stream);
    }
  } else {
    double* dw;
    if (!(rc = solution_weights(h->n, &dw)))
      rc = analysis_weights_cartesian(h->d_invJ, dw, h->n, h->dim, h->nodes, h->d_an_wj,
                                      h->stream);
    if (!rc) {
      const int n = h->n, m = 2 * n - 1;
      std::vector<double> xn(n), wn(n), xm(m), wm(m), V((size_t)m * n);
      lgl_nodes_weights(n - 1, xn.data(), wn.data());
      lgl_nodes_weights(m - 1, xm.data(), wm.data());
      interpolation_matrix(xn.data(), n, xm.data(), m, V.data());
      h->an_m = m;
      rc = upload(&h->d_an_V, V.data(), V.size(), h->stream);
      if (!rc) rc = upload(&h->d_an_wa, wm.data(), wm.size(), h->stream);
      if (!rc)
        rc = upload(&h->d_an_erows, (const double*)nullptr, (size_t)E * (2 * h->nv + 1),
                    h->stream);
    }
  }
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  for (double* p : tmp)
    if (p) cudaFree(p);
  if (rc) return rc;
  h->an_chunk = 8192;
  h->an_chunks = (int)((lmax + h->an_chunk - 1) / h->an_chunk);
  const size_t width = 2 * (size_t)h->nv + 1;
  if ((rc = upload(&h->d_an_rows, (const double*)nullptr, (size_t)M * h->an_chunks * width,
                   h->stream)))
    return rc;
  if ((rc = upload(&h->d_an_out, (const double*)nullptr, (size_t)M * width, h->stream))) return rc;
  h->an_ready = true;
  return TAG_OK;
}

AnalysisArgs analysis_args(tag_handle h, int quantity, const double* du) {
  AnalysisArgs a{};
  a.phys = analysis_phys(h);
  a.params = analysis_params(h);
  a.quantity = quantity;
  a.nmembers = h->nmembers;
  a.u = h->d_u;
  a.du = du;
  a.aux = h->eq == TAG_EQ_COVARIANT_SWE ? h->d_aux : nullptr;
  a.wj = h->d_an_wj;
  a.mbeg = h->d_an_rng;
  a.mend = h->d_an_rng + h->nmembers;
  return a;
}

}  // namespace

extern "C" {

const char* tag_last_error(void) { return g_last_error.c_str(); }

int tag_create(const tag_config* cfg, tag_handle* out) {
  if (!cfg || !out) return fail(TAG_E_INVALID, "null argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(TAG_E_NO_DEVICE, "no CUDA device visible");
  if (cfg->equations == TAG_EQ_COVARIANT_SWE) return create_cov(cfg, 1, out);
  const char* why = check_equations(cfg);
  if (why) return fail(TAG_E_INVALID, why);
  const int dim = (cfg->equations == TAG_EQ_EULER_ENERGY_3D ||
                   cfg->equations == TAG_EQ_POTENTIAL_TEMPERATURE_3D) ? 3 : 2;
  const int nface = 2 * dim;
  const bool rainy = cfg->equations == TAG_EQ_RAINY_2D;
  const bool moist = cfg->equations == TAG_EQ_MOIST_EULER_2D;
  const int n = cfg->polydeg + 1;
  if (n < 2 || n > kMaxNodes) return fail(TAG_E_INVALID, "polydeg out of range 1..7");
  if (dim == 3 && n < 3) return fail(TAG_E_INVALID, "3D meshes need polydeg >= 2");
  if (cfg->nelements <= 0 || cfg->ninterfaces < 0 || cfg->nboundaries < 0)
    return fail(TAG_E_INVALID, "bad mesh sizes");
  if (!cfg->derivative_split || !cfg->weights || !cfg->contravariant_vectors ||
      !cfg->inverse_jacobian)
    return fail(TAG_E_INVALID, "missing basis or geometry arrays");
  for (int k = 0; k < cfg->ninterfaces; ++k) {
    for (int s = 0; s < 2; ++s) {
      const int e = cfg->interface_elements[2 * k + s], f = cfg->interface_faces[2 * k + s];
      if (e < 0 || e >= cfg->nelements || f < 0 || f >= nface)
        return fail(TAG_E_INVALID, "interface index out of range");
    }
    const int o = cfg->interface_flip ? cfg->interface_flip[k] : 0;
    if (o < 0 || o > (dim == 3 ? 7 : 1))
      return fail(TAG_E_INVALID, "interface orientation out of range");
  }
  if (cfg->nmembers > 1) {
    if (!cfg->element_member) return fail(TAG_E_INVALID, "element_member missing");
    for (int e = 0; e < cfg->nelements; ++e)
      if (cfg->element_member[e] < 0 || cfg->element_member[e] >= cfg->nmembers)
        return fail(TAG_E_INVALID, "element_member out of range");
    for (int k = 0; k < cfg->ninterfaces; ++k)
      if (cfg->element_member[cfg->interface_elements[2 * k]] !=
          cfg->element_member[cfg->interface_elements[2 * k + 1]])
        return fail(TAG_E_INVALID, "an interface joins two ensemble members");
  }
  for (int k = 0; k < cfg->nboundaries; ++k) {
    const int e = cfg->boundary_elements[k], f = cfg->boundary_faces[k];
    const int kind = cfg->boundary_kinds ? cfg->boundary_kinds[k] : TAG_BC_SLIP_WALL_NORMAL;
    if (e < 0 || e >= cfg->nelements || f < 0 || f >= nface ||
        !boundary_kind_ok(cfg->equations, kind))
      return fail(TAG_E_INVALID, "boundary index or kind out of range");
  }

  tag_handle h = new tag_handle_s();
  h->eq = cfg->equations;
  h->n = n;
  h->nelem = cfg->nelements;
  h->nif = cfg->ninterfaces;
  h->nbd = cfg->nboundaries;
  h->nmembers = cfg->nmembers > 1 ? cfg->nmembers : 1;
  h->dim = dim;
  h->nface = nface;
  h->npe = dim == 3 ? n * n * n : n * n;
  h->nodes = (long)h->nelem * h->npe;
  h->dt_n = n;
  h->jpn = dim * dim;
  if (rainy) {
    h->nv = PhysRainy2D::NV;
    h->na = PhysRainy2D::NA;
    h->p_rainy = PhysRainy2D::make_params(cfg->params, cfg->surface_flux);
    h->ops = cfg->volume_flux == TAG_VF_WEAK_FORM ? ops_for_n<PhysRainy2D, kVolWeak>(n)
                                                  : ops_for_n<PhysRainy2D, kVolFluxDiff>(n);
    h->has_limiter = true;
  } else if (cfg->equations == TAG_EQ_POTENTIAL_TEMPERATURE_2D) {
    h->nv = PhysPT2D::NV;
    h->na = PhysPT2D::NA;
    double pp[8];
    for (int k = 0; k < 8; ++k) pp[k] = cfg->params[k];
    pp[5] = cfg->volume_flux == TAG_VF_PT_TEC ? 0 : cfg->volume_flux == TAG_VF_PT_EC ? 1 : 2;
    pp[6] = cfg->surface_flux == TAG_SF_PT_EC ? 1 : 0;
    if (cfg->surface_flux != TAG_SF_PT_EC) pp[7] = 0;  // flux_zero
    h->p_pt = PhysPT2D::make_params(pp);
    h->ops = ops_for_n<PhysPT2D, kVolFluxDiff>(n);
  } else if (moist) {
    h->nv = PhysMoist2D::NV;
    h->na = PhysMoist2D::NA;
    h->p_moist = PhysMoist2D::make_params(cfg->params);
    h->p_moist.surface = cfg->surface_flux;
    h->ops = cfg->volume_flux == TAG_VF_WEAK_FORM ? ops_for_n<PhysMoist2D, kVolWeak>(n)
                                                  : ops_for_n<PhysMoist2D, kVolFluxDiff>(n);
  } else if (cfg->equations == TAG_EQ_INTERNAL_ENERGY_2D) {
    h->nv = PhysIE2D::NV;
    h->na = PhysIE2D::NA;
    h->p_ie = PhysIE2D::make_params(cfg->params);
    h->ops = ops_for_n<PhysIE2D, kVolFluxDiff>(n);
  } else if (cfg->equations == TAG_EQ_POTENTIAL_TEMPERATURE_3D) {
    h->nv = PhysPT3D::NV;
    h->na = PhysPT3D::NA;
    double pp[8];
    for (int k = 0; k < 8; ++k) pp[k] = cfg->params[k];
    pp[5] = cfg->volume_flux == TAG_VF_PT_TEC  ? 0
            : cfg->volume_flux == TAG_VF_PT_EC ? 1
            : cfg->volume_flux == TAG_VF_PT_KG ? 3
                                               : 2;
    h->p_pt3d = PhysPT3D::make_params(pp);
    h->ops = ops3d_for_n<PhysPT3D>(n);
  } else if (dim == 3) {
    h->nv = PhysEnergy3D::NV;
    h->na = PhysEnergy3D::NA;
    h->p_energy3d = PhysEnergy3D::make_params(cfg->params);
    h->ops = ops3d_for_n<PhysEnergy3D>(n);
  } else {
    h->nv = PhysEnergy2D::NV;
    h->na = PhysEnergy2D::NA;
    h->p_energy = PhysEnergy2D::make_params(cfg->params);
    h->ops = ops_for_n<PhysEnergy2D>(n);
  }
  load_basis(h->basis, cfg->derivative_split, cfg->weights, n);
  auto cleanup = [&](int rc) {
    tag_destroy(h);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(fail(TAG_E_CUDA, "stream create failed"));
  const size_t nodes = (size_t)h->nodes;
  const size_t face_nodes = (size_t)h->nelem * nface * (dim == 3 ? n * n : n);
  int rc = TAG_OK;
  if ((rc = upload(&h->d_u, (const double*)nullptr, nodes * h->nv, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_k, (const double*)nullptr, nodes * h->na, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_Ja, cfg->contravariant_vectors, nodes * h->jpn, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_invJ, cfg->inverse_jacobian, nodes, h->stream))) return cleanup(rc);
  if (cfg->node_coordinates)
    if ((rc = upload(&h->d_xy, cfg->node_coordinates, nodes * dim, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_sfv, (const double*)nullptr, face_nodes * h->na, h->stream)))
    return cleanup(rc);
  if ((rc = upload(&h->d_if_e, cfg->interface_elements, (size_t)2 * h->nif, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_if_f, cfg->interface_faces, (size_t)2 * h->nif, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_if_flip, cfg->interface_flip, (size_t)h->nif, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_bd_e, cfg->boundary_elements, (size_t)h->nbd, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_bd_f, cfg->boundary_faces, (size_t)h->nbd, h->stream))) return cleanup(rc);
  if (cfg->boundary_kinds)
    if ((rc = upload(&h->d_bd_kind, cfg->boundary_kinds, (size_t)h->nbd, h->stream)))
      return cleanup(rc);
  for (int k = 0; cfg->boundary_kinds && k < h->nbd; ++k)
    h->need_bvals = h->need_bvals || cfg->boundary_kinds[k] == TAG_BC_DIRICHLET;
  if (h->need_bvals)
    if ((rc = upload(&h->d_bvals, (const double*)nullptr, (size_t)h->nbd * n * h->nv, h->stream)))
      return cleanup(rc);
  if (cfg->nmembers > 1)
    if ((rc = upload(&h->d_member, cfg->element_member, (size_t)h->nelem, h->stream)))
      return cleanup(rc);
  if ((rc = upload(&h->d_mscal, (const double*)nullptr, (size_t)3 * h->nmembers, h->stream)))
    return cleanup(rc);
  if ((rc = upload(&h->d_ctl, (const StepCtl*)nullptr, 1, h->stream))) return cleanup(rc);
  if ((rc = upload(&h->d_status, (const unsigned*)nullptr, 1, h->stream))) return cleanup(rc);
  if (rainy) {
    if ((rc = upload(&h->d_run_counters, (const unsigned long long*)nullptr, 4, h->stream)))
      return cleanup(rc);
    if ((rc = upload(&h->d_counters, (const unsigned long long*)nullptr, 4, h->stream)))
      return cleanup(rc);
    if ((rc = upload(&h->d_iters, (const int*)nullptr, nodes, h->stream))) return cleanup(rc);
  }
  if (cudaMallocHost(&h->h_pin, sizeof(double) * (3 * h->nmembers + 2)) != cudaSuccess)
    return cleanup(fail(TAG_E_CUDA, "pinned alloc failed"));
  if (cudaStreamSynchronize(h->stream) != cudaSuccess)
    return cleanup(fail(TAG_E_CUDA, "upload failed"));
  {
    int dev = 0, max_smem = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if ((rc = h->ops->init(max_smem))) return cleanup(rc);
  }
  *out = h;
  return TAG_OK;
}

int tag_create_ensemble(const tag_config* members, int32_t nmembers, tag_handle* out) {
  if (!members || !out || nmembers < 1) return fail(TAG_E_INVALID, "bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(TAG_E_NO_DEVICE, "no CUDA device visible");
  if (members[0].equations != TAG_EQ_COVARIANT_SWE)
    return fail(TAG_E_INVALID, "tag_create_ensemble supports the covariant equations");
  return create_cov(members, nmembers, out);
}

int tag_destroy(tag_handle h) {
  if (!h) return TAG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  double* dp[] = {h->d_u,       h->d_k,       h->d_Ja,         h->d_invJ,    h->d_xy,
                  h->d_sfv,     h->d_tmp_u,   h->d_tmp_du,     h->d_an_wj,   h->d_an_V,
                  h->d_an_wa,   h->d_an_rows, h->d_an_erows,   h->d_an_out,  h->d_an_uex,
                  h->d_an_x,    h->d_bvals,   h->d_u3,         h->d_err};
  for (double* p : dp)
    if (p) cudaFree(p);
  int* ip[] = {h->d_if_e, h->d_if_f, h->d_if_flip, h->d_bd_e, h->d_bd_f, h->d_bd_kind};
  for (int* p : ip)
    if (p) cudaFree(p);
  if (h->d_member) cudaFree(h->d_member);
  if (h->d_an_rng) cudaFree(h->d_an_rng);
  if (h->d_aux) cudaFree(h->d_aux);
  if (h->d_pk) cudaFree(h->d_pk);
  if (h->d_groups) cudaFree(h->d_groups);
  if (h->d_bases) cudaFree(h->d_bases);
  if (h->d_mlp) cudaFree(h->d_mlp);
  if (h->d_counters) cudaFree(h->d_counters);
  if (h->d_run_counters) cudaFree(h->d_run_counters);
  if (h->d_iters) cudaFree(h->d_iters);
  if (h->d_mscal) cudaFree(h->d_mscal);
  if (h->d_ctl) cudaFree(h->d_ctl);
  if (h->d_status) cudaFree(h->d_status);
  if (h->h_pin) cudaFreeHost(h->h_pin);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return TAG_OK;
}

int64_t tag_ndofs_total(tag_handle h) {
  return h ? (int64_t)h->nodes * h->nv : -1;
}

int tag_rhs(tag_handle h, const double* u, double* du, double t, int32_t on_device) {
  if (!h || !u || !du) return fail(TAG_E_INVALID, "null argument");
  const size_t bytes = sizeof(double) * (size_t)tag_ndofs_total(h);
  const double* ud = u;
  double* dud = du;
  if (!on_device) {
    if (!h->d_tmp_u) TAG_CUDA(cudaMalloc(&h->d_tmp_u, bytes));
    if (!h->d_tmp_du) TAG_CUDA(cudaMalloc(&h->d_tmp_du, bytes));
    TAG_CUDA(cudaMemcpyAsync(h->d_tmp_u, u, bytes, cudaMemcpyHostToDevice, h->stream));
    ud = h->d_tmp_u;
    dud = h->d_tmp_du;
  }
  NvtxRange r_rhs("rhs!");
  int rc = autotune(h, ud);
  if (rc) return rc;
  {
    NvtxRange r(kNvtxInterface);
    rc = h->ops->interface(h, ud);
  }
  if (rc) return rc;
  {
    NvtxRange r(kNvtxElement);
    rc = h->ops->element(h, kModeRhs, const_cast<double*>(ud), dud, 0, false, t);
  }
  if (rc) return rc;
  if (!on_device) TAG_CUDA(cudaMemcpyAsync(du, dud, bytes, cudaMemcpyDeviceToHost, h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  return TAG_OK;
}

int tag_set_state(tag_handle h, const double* u_host) {
  if (!h || !u_host) return fail(TAG_E_INVALID, "null argument");
  // pinned (mapped) host memory: one kernel reads the state over the host link,
  // stores it on the device and reduces the CFL speeds in the same pass
  cudaPointerAttributes attr{};
  const bool mapped = cudaPointerGetAttributes(&attr, u_host) == cudaSuccess &&
                      attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr;
  if (!mapped) cudaGetLastError();  // a pointer CUDA does not know is not an error here
  if (mapped && h->ops->load_state) {
    TAG_CUDA(cudaMemsetAsync(h->d_k, 0, sizeof(double) * (size_t)h->nodes * h->na, h->stream));
    TAG_CUDA(cudaMemsetAsync(h->d_mscal + 2 * h->nmembers, 0, sizeof(double) * h->nmembers,
                             h->stream));
    int rc = h->ops->load_state(h, static_cast<const double*>(attr.devicePointer));
    if (rc) return rc;
    TAG_CUDA(cudaStreamSynchronize(h->stream));
    h->speed_valid = true;
    return TAG_OK;
  }
  TAG_CUDA(cudaMemcpyAsync(h->d_u, u_host, sizeof(double) * (size_t)tag_ndofs_total(h),
                           cudaMemcpyHostToDevice, h->stream));
  TAG_CUDA(cudaMemsetAsync(h->d_k, 0, sizeof(double) * (size_t)h->nodes * h->na,
                           h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  h->speed_valid = false;
  return TAG_OK;
}

int tag_get_state(tag_handle h, double* u_host) {
  if (!h || !u_host) return fail(TAG_E_INVALID, "null argument");
  TAG_CUDA(cudaMemcpyAsync(u_host, h->d_u, sizeof(double) * (size_t)tag_ndofs_total(h),
                           cudaMemcpyDeviceToHost, h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  return TAG_OK;
}

int tag_solution_variables(tag_handle h, int32_t solution_variables, int32_t member,
                           int32_t* nvars, int64_t* nnodes, double* data) {
  if (!h || !nvars || !nnodes) return fail(TAG_E_INVALID, "null argument");
  const bool cov = h->eq == TAG_EQ_COVARIANT_SWE;
  const int kind = solution_variables;
  if (kind < TAG_SOLVAR_CONS2CONS || kind > TAG_SOLVAR_CONS2PRIM_AND_VORTICITY ||
      (!cov && kind != TAG_SOLVAR_CONS2CONS))
    return fail(TAG_E_INVALID, cov ? "solution_variables out of range 0..3"
                                   : "this equation system writes cons2cons only");
  if (member < -1 || member >= h->nmembers) return fail(TAG_E_INVALID, "member out of range");
  long q0 = 0, q1 = h->nodes;
  if (member >= 0 && h->nmembers > 1) {
    std::vector<long> rng;
    const int rc = member_ranges(h, rng);
    if (rc) return rc;
    q0 = rng[member];
    q1 = rng[h->nmembers + member];
  }
  const long nq = q1 - q0;
  const int nr = !cov ? h->nv : kind == TAG_SOLVAR_CONTRAVARIANT2GLOBAL ? 4
                 : kind == TAG_SOLVAR_CONS2PRIM_AND_VORTICITY ? 6 : 3;
  *nvars = nr;
  *nnodes = nq;
  if (!data) return TAG_OK;
  NvtxRange nv_("save_solution");
  double* d_out = nullptr;
  TAG_CUDA(cudaMallocAsync(&d_out, sizeof(double) * (size_t)nr * nq, h->stream));
  const unsigned blocks = (unsigned)((nq + 255) / 256);
  if (cov)
    k_cov_solution_rows<<<blocks, 256, 0, h->stream>>>(h->d_groups, h->d_bases, h->d_u, h->d_aux,
                                                       kind, q0, nq, d_out);
  else
    k_state_rows<<<blocks, 256, 0, h->stream>>>(h->d_u, h->nv, q0, nq, d_out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(data, d_out, sizeof(double) * (size_t)nr * nq, cudaMemcpyDeviceToHost,
                        h->stream);
  const cudaError_t ef = cudaFreeAsync(d_out, h->stream);
  const cudaError_t es = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = ef != cudaSuccess ? ef : es;
  if (e != cudaSuccess) return fail(TAG_E_CUDA, std::string("tag_solution_variables: ") +
                                                    cudaGetErrorString(e));
  return TAG_OK;
}

int tag_set_state_sink(tag_handle h, double* u_host) {
  if (!h) return fail(TAG_E_INVALID, "null handle");
  if (!u_host) {
    h->sink = nullptr;
    return TAG_OK;
  }
  cudaPointerAttributes attr{};
  const bool mapped = cudaPointerGetAttributes(&attr, u_host) == cudaSuccess &&
                      attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr;
  if (!mapped) {
    cudaGetLastError();
    return fail(TAG_E_INVALID, "the state sink must be pinned host memory mapped for the device");
  }
  h->sink = static_cast<double*>(attr.devicePointer);
  return TAG_OK;
}

int tag_state_device_ptr(tag_handle h, double** u_dev) {
  if (!h || !u_dev) return fail(TAG_E_INVALID, "null argument");
  *u_dev = h->d_u;
  h->speed_valid = false;  // the caller may write through the pointer
  return TAG_OK;
}

int tag_max_dt_members(tag_handle h, double* out) {
  if (!h || !out) return fail(TAG_E_INVALID, "null argument");
  int rc = reset_and_reduce_speeds(h);
  if (rc) return rc;
  TAG_CUDA(cudaMemcpyAsync(h->h_pin, h->d_mscal + 2 * h->nmembers, sizeof(double) * h->nmembers,
                           cudaMemcpyDeviceToHost, h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  for (int m = 0; m < h->nmembers; ++m) {
    double ms = h->h_pin[m];
    if (!(ms > 0.0)) ms = 4.9406564584124654e-324;
    out[m] = 2.0 / (h->dt_n * ms);
  }
  h->speed_valid = true;
  return TAG_OK;
}

int tag_max_dt(tag_handle h, double* out) {
  if (!h || !out) return fail(TAG_E_INVALID, "null argument");
  std::vector<double> v(h->nmembers);
  int rc = tag_max_dt_members(h, v.data());
  if (rc) return rc;
  *out = *std::min_element(v.begin(), v.end());
  return TAG_OK;
}

int tag_rk_steps(tag_handle h, int32_t nsteps, double cfl, double fixed_dt, double* t) {
  if (!h || !t || nsteps < 0) return fail(TAG_E_INVALID, "bad argument");
  if (nsteps == 0) return TAG_OK;
  int rc = autotune(h, h->d_u);
  if (rc) return rc;
  if (!h->speed_valid)
    if ((rc = reset_and_reduce_speeds(h))) return rc;
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  const int M = h->nmembers;
  for (int m = 0; m < M; ++m) {
    h->h_pin[m] = t[m];
    h->h_pin[M + m] = 0.0;
  }
  h->h_pin[3 * M] = cfl;
  h->h_pin[3 * M + 1] = fixed_dt;
  // t and dt (max_speed, the third array, is kept); then the control block
  TAG_CUDA(cudaMemcpyAsync(h->d_mscal, h->h_pin, sizeof(double) * 2 * M, cudaMemcpyHostToDevice,
                           h->stream));
  TAG_CUDA(cudaMemcpyAsync(h->d_ctl, h->h_pin + 3 * M, sizeof(StepCtl), cudaMemcpyHostToDevice,
                           h->stream));
  if ((rc = build_graph(h))) return rc;
  NvtxRange r_steps(h->has_limiter ? "RK steps (stages + nonlinear system solver)" : "RK steps");
  for (int s = 0; s < nsteps; ++s) TAG_CUDA(cudaGraphLaunch(h->graph, h->stream));
  if (h->has_limiter) h->run_node_solves += (long long)nsteps * rk_stages(h->scheme) * h->nodes;
  TAG_CUDA(cudaMemcpyAsync(h->h_pin, h->d_mscal, sizeof(double) * 2 * M, cudaMemcpyDeviceToHost,
                           h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  for (int m = 0; m < M; ++m) t[m] = h->h_pin[m] + h->h_pin[M + m];
  h->speed_valid = true;
  return TAG_OK;
}

}  // extern "C"

namespace {

constexpr int kErrBlocks = 512, kErrThreads = 256;

// Embedded error of one SSPRK43 step for every active variable:
//   e = (u_new - (2 u3 - u_prev)) / 2,
// u3 the stage value entering the last stage, taken before any stage limiter,
// so that 2 u3 - u_prev = u_prev/3 + 2/3 (u2 + dt/2 f(u2)) and e = u_new - u^
// with u^ the embedded second-order value; u_prev is the k register, which
// holds the step's starting state in the SSP form.  Sums of squares of
// e / (abstol + max(|u_prev|, |u_new|) reltol) per block, in a fixed order
// (a fixed grid), then summed in block order by k_err_total.  Passive
// variables do not change, so their terms are zero.
__global__ void __launch_bounds__(kErrThreads) k_ssp43_error(
    const double* __restrict__ u, const double* __restrict__ u3, const double* __restrict__ kprev,
    long nodes, int nv, int na, double abstol, double reltol, double* __restrict__ partial) {
  __shared__ double red[kErrThreads];
  double acc = 0.0;
  const long items = nodes * na;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < items;
       q += (long)gridDim.x * blockDim.x) {
    const long node = q / na;
    const int v = (int)(q % na);
    const double un = u[node * nv + v], up = kprev[q];
    const double e = 0.5 * (un - (2.0 * u3[node * nv + v] - up));
    const double x = e / (abstol + fmax(fabs(up), fabs(un)) * reltol);
    acc = fma(x, x, acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kErrThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_err_total(double* __restrict__ partial, int n) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < n; ++b) s += partial[b];
  partial[n] = s;
}

// A rejected step: the active variables return to the step's starting state.
__global__ void k_restore_active(double* __restrict__ u, const double* __restrict__ kprev,
                                 long nodes, int nv, int na) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nodes * na) return;
  u[(q / na) * nv + q % na] = kprev[q];
}

// Root mean square of x(q) over n entries, summed in index order.
template <class F>
double rms_host(long n, F&& x) {
  double s = 0.0;
  for (long q = 0; q < n; ++q) {
    const double v = x(q);
    s += v * v;
  }
  return std::sqrt(s / (double)n);
}

// du = rhs(u) on the device through the handle's kernels (time t).
int rhs_device(tag_handle h, double* u, double* du, double t) {
  int rc = h->ops->interface(h, u);
  if (rc) return rc;
  return h->ops->element(h, kModeRhs, u, du, 0, false, t);
}

}  // namespace

extern "C" {

int tag_rk_adaptive(tag_handle h, double* t, double t_end, double abstol, double reltol,
                    const double* stops, int32_t nstops, int64_t max_steps,
                    tag_adaptive_stats* stats) {
  if (!h || !t || !(t_end > *t) || !(abstol > 0.0) || !(reltol >= 0.0) || nstops < 0 ||
      (nstops > 0 && !stops) || max_steps <= 0)
    return fail(TAG_E_INVALID, "bad argument");
  if (h->nmembers != 1) return fail(TAG_E_INVALID, "adaptive steps integrate a single mesh");
  if (h->scheme != TAG_RK_SSPRK43)
    return fail(TAG_E_INVALID, "select SSPRK43 with tag_set_time_integrator first");
  for (int i = 1; i < nstops; ++i)
    if (!(stops[i] > stops[i - 1])) return fail(TAG_E_INVALID, "stops must increase");
  NvtxRange r_ad("adaptive SSPRK43");
  int rc = autotune(h, h->d_u);
  if (rc) return rc;
  const long nodes = (long)h->nodes;
  const int nv = h->nv, na = h->na;
  const size_t bytes = sizeof(double) * (size_t)nodes * nv;
  if (!h->d_u3) TAG_CUDA(cudaMalloc(&h->d_u3, bytes));
  if (!h->d_tmp_du) TAG_CUDA(cudaMalloc(&h->d_tmp_du, bytes));
  if (!h->d_err) TAG_CUDA(cudaMalloc(&h->d_err, sizeof(double) * (kErrBlocks + 1)));
  const long N = nodes * nv;  // the ODE state has every variable, passive ones included
  // controller constants (OrdinaryDiffEq's defaults for SSPRK43, order 3)
  const double beta1 = 7.0 / 30.0, beta2 = 2.0 / 15.0, qmin = 0.2, qmax = 10.0, gamma = 0.9,
               qoldinit = 1e-4;
  double tt = *t;
  // initial step (Hairer, Norsett, Wanner II.4, as OrdinaryDiffEq's
  // ode_determine_initdt): two rhs evaluations, norms on the host
  double dt;
  {
    std::vector<double> u0(N), f0(N), f1(N);
    if ((rc = rhs_device(h, h->d_u, h->d_tmp_du, tt))) return rc;
    TAG_CUDA(cudaMemcpyAsync(u0.data(), h->d_u, bytes, cudaMemcpyDeviceToHost, h->stream));
    TAG_CUDA(cudaMemcpyAsync(f0.data(), h->d_tmp_du, bytes, cudaMemcpyDeviceToHost, h->stream));
    TAG_CUDA(cudaStreamSynchronize(h->stream));
    auto sk = [&](long q) { return abstol + std::fabs(u0[q]) * reltol; };
    const double d0 = rms_host(N, [&](long q) { return u0[q] / sk(q); });
    const double d1 = rms_host(N, [&](long q) { return f0[q] / sk(q); });
    double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
    dt0 = std::min(dt0, t_end - tt);
    for (long q = 0; q < N; ++q) f1[q] = u0[q] + dt0 * f0[q];
    TAG_CUDA(cudaMemcpyAsync(h->d_u3, f1.data(), bytes, cudaMemcpyHostToDevice, h->stream));
    if ((rc = rhs_device(h, h->d_u3, h->d_tmp_du, tt + dt0))) return rc;
    TAG_CUDA(cudaMemcpyAsync(f1.data(), h->d_tmp_du, bytes, cudaMemcpyDeviceToHost, h->stream));
    TAG_CUDA(cudaStreamSynchronize(h->stream));
    const double d2 = rms_host(N, [&](long q) { return (f1[q] - f0[q]) / sk(q); }) / dt0;
    const double m = std::max(d1, d2);
    const double dt1 =
        m <= 1e-15 ? std::max(1e-6, dt0 * 1e-3) : std::pow(10.0, -(2.0 + std::log10(m)) / 3.0);
    dt = std::min(std::min(100.0 * dt0, dt1), t_end - tt);
  }
  tag_adaptive_stats out{};
  out.dt_first = dt;
  double qold = qoldinit;
  int next = 0;
  const int ns = rk_stages(h->scheme);
  while (tt < t_end) {
    if (out.accepted + out.rejected >= max_steps) {
      *t = tt;
      if (stats) *stats = out;
      return fail(TAG_E_INVALID, "adaptive steps: max_steps reached before t_end");
    }
    while (next < nstops && stops[next] <= tt) ++next;
    const double stop = next < nstops ? std::min(stops[next], t_end) : t_end;
    const double hdt = std::min(dt, stop - tt);
    h->h_pin[0] = tt;
    h->h_pin[1] = hdt;
    TAG_CUDA(cudaMemcpyAsync(h->d_mscal, h->h_pin, sizeof(double) * 2, cudaMemcpyHostToDevice,
                             h->stream));
    for (int s = 0; s < ns; ++s) {
      if ((rc = h->ops->interface(h, h->d_u))) return rc;
      if ((rc = h->ops->element(h, kModeStage, h->d_u, nullptr, s, false, 0.0))) return rc;
      if (s == ns - 2)
        TAG_CUDA(cudaMemcpyAsync(h->d_u3, h->d_u, bytes, cudaMemcpyDeviceToDevice, h->stream));
      if (h->has_limiter) {
        NewtonArgs a = h->newton;
        a.learned = h->newton_start;
        a.mlp = h->d_mlp;
        a.iters = nullptr;
        a.counters = h->d_run_counters;
        TAG_CUDA(launch_newton_rainy(h->d_u, nodes, a, h->d_status, h->stream));
        h->run_node_solves += nodes;
      }
    }
    k_ssp43_error<<<kErrBlocks, kErrThreads, 0, h->stream>>>(h->d_u, h->d_u3, h->d_k, nodes, nv,
                                                             na, abstol, reltol, h->d_err);
    TAG_CUDA(cudaGetLastError());
    k_err_total<<<1, 32, 0, h->stream>>>(h->d_err, kErrBlocks);
    TAG_CUDA(cudaGetLastError());
    TAG_CUDA(cudaMemcpyAsync(h->h_pin + 2, h->d_err + kErrBlocks, sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
    TAG_CUDA(cudaStreamSynchronize(h->stream));
    const double eest = std::sqrt(h->h_pin[2] / (double)N);
    if (!std::isfinite(eest)) {
      *t = tt;
      if (stats) *stats = out;
      return fail(TAG_E_INVALID, "adaptive steps: non-finite error estimate");
    }
    const double q11 = std::pow(eest, beta1);
    if (eest <= 1.0) {
      double q = eest == 0.0 ? 1.0 / qmax : q11 / std::pow(qold, beta2);
      if (eest != 0.0) q = std::max(1.0 / qmax, std::min(1.0 / qmin, q / gamma));
      tt = (hdt == stop - tt) ? stop : tt + hdt;
      qold = std::max(eest, qoldinit);
      dt = hdt / q;
      out.dt_last = hdt;
      ++out.accepted;
    } else {
      k_restore_active<<<(unsigned)((nodes * na + 255) / 256), 256, 0, h->stream>>>(
          h->d_u, h->d_k, nodes, nv, na);
      TAG_CUDA(cudaGetLastError());
      dt = hdt / std::min(1.0 / qmin, q11 / gamma);
      ++out.rejected;
    }
  }
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  h->speed_valid = false;
  *t = tt;
  if (stats) *stats = out;
  return TAG_OK;
}

int tag_time_kernels(tag_handle h, int32_t reps, double* ms_interface, double* ms_element) {
  if (!h || !ms_interface || !ms_element || reps <= 0) return fail(TAG_E_INVALID, "bad argument");
  int rc = autotune(h, h->d_u);
  if (rc) return rc;
  if ((rc = reset_and_reduce_speeds(h))) return rc;
  h->h_pin[0] = 1.0;  // cfl
  h->h_pin[1] = 0.0;
  TAG_CUDA(cudaMemcpyAsync(h->d_ctl, h->h_pin, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
  if ((rc = begin_step(h))) return rc;
  std::vector<cudaEvent_t> ev(3 * reps);
  for (auto& e : ev) TAG_CUDA(cudaEventCreate(&e));
  // warm-up stage
  if ((rc = h->ops->interface(h, h->d_u))) return rc;
  if ((rc = h->ops->element(h, kModeStage, h->d_u, nullptr, 0, false, 0.0))) return rc;
  for (int r = 0; r < reps; ++r) {
    TAG_CUDA(cudaEventRecord(ev[3 * r], h->stream));
    if ((rc = h->ops->interface(h, h->d_u))) return rc;
    TAG_CUDA(cudaEventRecord(ev[3 * r + 1], h->stream));
    if ((rc = h->ops->element(h, kModeStage, h->d_u, nullptr, (r + 1) % 5, false, 0.0))) return rc;
    TAG_CUDA(cudaEventRecord(ev[3 * r + 2], h->stream));
  }
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  double si = 0.0, se = 0.0;
  for (int r = 0; r < reps; ++r) {
    float a = 0.f, b = 0.f;
    TAG_CUDA(cudaEventElapsedTime(&a, ev[3 * r], ev[3 * r + 1]));
    TAG_CUDA(cudaEventElapsedTime(&b, ev[3 * r + 1], ev[3 * r + 2]));
    si += a;
    se += b;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  *ms_interface = si / reps;
  *ms_element = se / reps;
  h->speed_valid = false;
  return TAG_OK;
}

int tag_set_boundary_values(tag_handle h, const double* values) {
  if (!h || !values) return fail(TAG_E_INVALID, "bad argument");
  if (!h->need_bvals) return fail(TAG_E_INVALID, "the mesh has no Dirichlet boundary faces");
  const size_t bytes = (size_t)h->nbd * h->n * h->nv * sizeof(double);
  TAG_CUDA(cudaMemcpyAsync(h->d_bvals, values, bytes, cudaMemcpyHostToDevice, h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  h->bvals_set = true;
  return TAG_OK;
}

int tag_set_source(tag_handle h, int32_t kind, const double* params, int32_t nparams) {
  if (!h) return fail(TAG_E_INVALID, "bad argument");
  if (h->eq != TAG_EQ_POTENTIAL_TEMPERATURE_2D || kind != TAG_SRC_MOUNTAIN_WAVE)
    return fail(TAG_E_INVALID, "unsupported source for these equations");
  if (!params || nparams != 8) return fail(TAG_E_INVALID, "MountainWaveSetup needs 8 parameters");
  if (!h->d_xy) return fail(TAG_E_INVALID, "this source needs node coordinates");
  if (!(params[4] > params[3]) || !(params[6] > params[5]) || !(params[7] >= 0.0))
    return fail(TAG_E_INVALID, "bad damping layers");
  h->p_pt.mountain = 1;
  for (int k = 0; k < 8; ++k) h->p_pt.mw[k] = params[k];
  h->graph_epb = -2;  // the parameters are baked into the captured graph
  return TAG_OK;
}

int tag_set_time_integrator(tag_handle h, int32_t scheme) {
  if (!h) return fail(TAG_E_INVALID, "bad argument");
  if (scheme != TAG_RK_CK2N54 && scheme != TAG_RK_SSPRK43 && scheme != TAG_RK_SSPRK33)
    return fail(TAG_E_INVALID, "unknown time integrator");
  if (scheme != h->scheme) {
    h->scheme = scheme;
    h->graph_epb = -2;  // the stage sequence is baked into the captured graph
  }
  return TAG_OK;
}

int tag_set_newton(tag_handle h, int32_t mode, double tol, int32_t max_iterations,
                   int32_t polish) {
  if (!h || !h->has_limiter) return fail(TAG_E_INVALID, "not a rainy handle");
  if ((mode != 0 && mode != 1) || !(tol > 0.0) || max_iterations < 1 || polish < 0)
    return fail(TAG_E_INVALID, "bad Newton settings");
  h->newton.mode = mode;
  h->newton.tol = tol;
  h->newton.maxit = max_iterations;
  h->newton.polish = polish;
  h->graph_epb = -2;  // limiter settings are baked into the captured graph
  return TAG_OK;
}

int tag_set_newton_start(tag_handle h, int32_t start) {
  if (!h || !h->has_limiter) return fail(TAG_E_INVALID, "not a rainy handle");
  if (start < 0 || start > 3) return fail(TAG_E_INVALID, "start must be 0, 1, 2 or 3");
  if ((start == 1 || start == 3) && !h->d_mlp) return fail(TAG_E_INVALID, "no MLP parameters set");
  h->newton_start = start;
  h->graph_epb = -2;  // the limiter's arguments are baked into the captured graph
  return TAG_OK;
}

int tag_newton_counters(tag_handle h, int64_t* out, int32_t reset) {
  if (!h || !h->has_limiter || !out) return fail(TAG_E_INVALID, "bad argument");
  unsigned long long c[4];
  TAG_CUDA(cudaMemcpyAsync(c, h->d_run_counters, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  out[0] = (int64_t)c[0];
  out[1] = (int64_t)c[1];
  out[2] = (int64_t)c[2];
  out[3] = h->run_node_solves;
  if (reset) {
    TAG_CUDA(cudaMemsetAsync(h->d_run_counters, 0, sizeof(c), h->stream));
    TAG_CUDA(cudaStreamSynchronize(h->stream));
    h->run_node_solves = 0;
  }
  return TAG_OK;
}

int tag_set_mlp(tag_handle h, const float* params) {
  if (!h || !h->has_limiter || !params) return fail(TAG_E_INVALID, "bad argument");
  if (!h->d_mlp) TAG_CUDA(cudaMalloc(&h->d_mlp, sizeof(float) * kMlpParams));
  TAG_CUDA(cudaMemcpyAsync(h->d_mlp, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice,
                           h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  return TAG_OK;
}

int tag_newton_solve(tag_handle h, int32_t use_learned, int32_t* iters, tag_newton_stats* stats) {
  if (!h || !h->has_limiter) return fail(TAG_E_INVALID, "not a rainy handle");
  if (use_learned < 0 || use_learned > 3) return fail(TAG_E_INVALID, "start must be 0, 1, 2 or 3");
  NvtxRange r_solve("nonlinear system solver");
  if ((use_learned == 1 || use_learned == 3) && !h->d_mlp)
    return fail(TAG_E_INVALID, "no MLP parameters set");
  const long nodes = (long)h->nodes;
  NewtonArgs a = h->newton;
  a.learned = use_learned;
  a.mlp = h->d_mlp;
  a.iters = h->d_iters;
  a.counters = h->d_counters;
  TAG_CUDA(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * 4, h->stream));
  TAG_CUDA(launch_newton_rainy(h->d_u, nodes, a, h->d_status, h->stream));
  unsigned long long c[4];
  TAG_CUDA(cudaMemcpyAsync(c, h->d_counters, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
  if (iters)
    TAG_CUDA(cudaMemcpyAsync(iters, h->d_iters, sizeof(int) * nodes, cudaMemcpyDeviceToHost,
                             h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  if (stats) {
    stats->nodes = nodes;
    stats->updates = (int64_t)c[0];
    stats->fallbacks = (int64_t)c[1];
    stats->not_converged = (int64_t)c[2];
  }
  h->speed_valid = false;
  return TAG_OK;
}

int tag_status(tag_handle h, uint32_t* flags, int32_t clear) {
  if (!h || !flags) return fail(TAG_E_INVALID, "null argument");
  unsigned v = 0;
  TAG_CUDA(cudaMemcpyAsync(&v, h->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
  if (clear) TAG_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned), h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  *flags = v;
  return TAG_OK;
}

void* tag_stream(tag_handle h) { return h ? (void*)h->stream : nullptr; }

int tag_set_elements_per_block(tag_handle h, int32_t epb) {
  if (!h || epb < 0) return fail(TAG_E_INVALID, "bad argument");
  if (epb > 0) {
    int dev, max_smem = 0;
    TAG_CUDA(cudaGetDevice(&dev));
    TAG_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (h->ops->smem_bytes(epb) > (size_t)max_smem ||
        (epb > 1 && epb * h->ops->threads_per_element > h->ops->max_threads()))
      return fail(TAG_E_INVALID, "elements per block too large for one CTA");
  }
  h->epb = epb;
  h->tile_div = 1;
  return TAG_OK;
}

int tag_get_elements_per_block(tag_handle h, int32_t* epb) {
  if (!h || !epb) return fail(TAG_E_INVALID, "null argument");
  *epb = h->epb;
  return TAG_OK;
}

int tag_set_tile(tag_handle h, int32_t epb, int32_t items_per_thread) {
  if (!h || epb < 1 || items_per_thread < 1 || items_per_thread > 2)
    return fail(TAG_E_INVALID, "bad argument");
  int rc = tag_set_elements_per_block(h, epb);
  if (rc) return rc;
  h->tile_div = items_per_thread;
  return TAG_OK;
}

int tag_get_cta_threads(tag_handle h, int32_t* threads) {
  if (!h || !threads) return fail(TAG_E_INVALID, "null argument");
  const int epb = h->epb > 0 ? h->epb : 1;
  *threads = h->ops ? std::min(h->ops->max_threads(),
                               cta_threads(epb * h->ops->threads_per_element, h->tile_div))
                    : 0;
  return TAG_OK;
}

int tag_fp64_peak(double* flops_per_s) {
  if (!flops_per_s) return fail(TAG_E_INVALID, "null argument");
  int dev, sms = 0;
  TAG_CUDA(cudaGetDevice(&dev));
  TAG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256, blocks = sms * 8, iters = 1 << 14;
  double* out = nullptr;
  TAG_CUDA(cudaMalloc(&out, sizeof(double) * threads * blocks));
  cudaEvent_t a, b;
  TAG_CUDA(cudaEventCreate(&a));
  TAG_CUDA(cudaEventCreate(&b));
  k_fp64_probe<<<blocks, threads>>>(out, iters, 1.0);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    TAG_CUDA(cudaEventRecord(a));
    k_fp64_probe<<<blocks, threads>>>(out, iters, 1.0 + r);
    TAG_CUDA(cudaEventRecord(b));
    TAG_CUDA(cudaEventSynchronize(b));
    float ms;
    TAG_CUDA(cudaEventElapsedTime(&ms, a, b));
    best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  *flops_per_s = 2.0 * 8.0 * iters * (double)threads * blocks / (best * 1e-3);
  return TAG_OK;
}

int tag_analyze_integral(tag_handle h, int32_t quantity, int32_t normalize, double t,
                         double* out) {
  if (!h || !out) return fail(TAG_E_INVALID, "bad argument");
  const int nq = analysis_values(analysis_phys(h), quantity);
  if (nq < 0) return fail(TAG_E_INVALID, "quantity not defined for these equations");
  int rc = analysis_setup(h);
  if (rc) return rc;
  const double* du = nullptr;
  if (quantity == TAG_AQ_ENTROPY_TIMEDERIVATIVE) {
    if (!h->d_tmp_du) TAG_CUDA(cudaMalloc(&h->d_tmp_du, sizeof(double) * h->nodes * h->nv));
    if ((rc = h->ops->interface(h, h->d_u))) return rc;
    if ((rc = h->ops->element(h, kModeRhs, h->d_u, h->d_tmp_du, 0, false, t))) return rc;
    du = h->d_tmp_du;
  }
  const AnalysisArgs a = analysis_args(h, quantity, du);
  if ((rc = analysis_node_rows(a, h->an_chunks, h->an_chunk, h->d_an_rows, h->stream)))
    return fail(rc, "analysis launch failed");
  if ((rc = analysis_reduce_rows(h->d_an_rows, nq + 1, 0, 0, nullptr, nullptr, h->an_chunks,
                                 h->nmembers, h->d_an_out, h->stream)))
    return fail(rc, "analysis reduction failed");
  const int M = h->nmembers;
  std::vector<double> v((size_t)M * (nq + 1));
  TAG_CUDA(cudaMemcpyAsync(v.data(), h->d_an_out, sizeof(double) * v.size(),
                           cudaMemcpyDeviceToHost, h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  for (int m = 0; m < M; ++m) {
    const double* r = &v[(size_t)m * (nq + 1)];
    for (int q = 0; q < nq; ++q) out[(size_t)m * nq + q] = normalize ? r[q] / r[nq] : r[q];
  }
  return TAG_OK;
}

int tag_analysis_nodes(tag_handle h, int32_t* m, double* x) {
  if (!h || !m) return fail(TAG_E_INVALID, "bad argument");
  int rc = analysis_setup(h);
  if (rc) return rc;
  if (h->eq == TAG_EQ_COVARIANT_SWE) {
    *m = 0;
    if (x) {
      TAG_CUDA(cudaMemcpyAsync(x, h->d_xy, sizeof(double) * h->nodes * 3, cudaMemcpyDeviceToHost,
                               h->stream));
      TAG_CUDA(cudaStreamSynchronize(h->stream));
    }
    return TAG_OK;
  }
  *m = h->an_m;
  if (!x) return TAG_OK;
  if (!h->d_xy) return fail(TAG_E_INVALID, "tag_create was given no node_coordinates");
  const size_t ma = h->dim == 3 ? (size_t)h->an_m * h->an_m * h->an_m : (size_t)h->an_m * h->an_m;
  const size_t count = (size_t)h->nelem * ma * h->dim;
  if (!h->d_an_x) TAG_CUDA(cudaMalloc(&h->d_an_x, sizeof(double) * count));
  if ((rc = analysis_coordinates(h->dim, h->n, h->an_m, h->nelem, h->d_xy, h->d_an_V, h->d_an_x,
                                 h->stream)))
    return fail(rc, "analysis launch failed");
  TAG_CUDA(cudaMemcpyAsync(x, h->d_an_x, sizeof(double) * count, cudaMemcpyDeviceToHost,
                           h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  return TAG_OK;
}

int tag_analyze_errors(tag_handle h, const double* u_exact, double* l2, double* linf) {
  if (!h || !u_exact || !l2 || !linf) return fail(TAG_E_INVALID, "bad argument");
  int rc = analysis_setup(h);
  if (rc) return rc;
  const bool cov = h->eq == TAG_EQ_COVARIANT_SWE;
  const int nv = h->nv, nq = 2 * nv + 1, M = h->nmembers;
  const size_t ma =
      cov ? 0
          : (h->dim == 3 ? (size_t)h->an_m * h->an_m * h->an_m : (size_t)h->an_m * h->an_m);
  const size_t count = cov ? (size_t)h->nodes * nv : (size_t)h->nelem * ma * nv;
  if (h->an_uex_cap < count) {
    if (h->d_an_uex) cudaFree(h->d_an_uex);
    h->d_an_uex = nullptr;
    h->an_uex_cap = 0;
    TAG_CUDA(cudaMalloc(&h->d_an_uex, sizeof(double) * count));
    h->an_uex_cap = count;
  }
  TAG_CUDA(cudaMemcpyAsync(h->d_an_uex, u_exact, sizeof(double) * count, cudaMemcpyHostToDevice,
                           h->stream));
  if (cov) {
    const AnalysisArgs a = analysis_args(h, TAG_AQ_STATE, nullptr);
    if ((rc = analysis_node_error_rows(a, h->d_an_uex, h->an_chunks, h->an_chunk, h->d_an_rows,
                                       h->stream)))
      return fail(rc, "analysis launch failed");
    rc = analysis_reduce_rows(h->d_an_rows, nq, nv, 2 * nv, nullptr, nullptr, h->an_chunks, M,
                              h->d_an_out, h->stream);
  } else {
    if ((rc = analysis_element_error_rows(analysis_phys(h), h->dim, h->n, h->an_m, h->nelem,
                                          h->d_u, h->d_invJ, h->d_an_V, h->d_an_wa, h->d_an_uex,
                                          h->d_an_erows, h->stream)))
      return fail(rc, "analysis launch failed");
    rc = analysis_reduce_rows(h->d_an_erows, nq, nv, 2 * nv, h->d_an_rng + 2 * M,
                              h->d_an_rng + 3 * M, 0, M, h->d_an_out, h->stream);
  }
  if (rc) return fail(rc, "analysis reduction failed");
  std::vector<double> v((size_t)M * nq);
  TAG_CUDA(cudaMemcpyAsync(v.data(), h->d_an_out, sizeof(double) * v.size(),
                           cudaMemcpyDeviceToHost, h->stream));
  TAG_CUDA(cudaStreamSynchronize(h->stream));
  for (int m = 0; m < M; ++m) {
    const double* r = &v[(size_t)m * nq];
    for (int q = 0; q < nv; ++q) {
      l2[(size_t)m * nv + q] = std::sqrt(r[q] / r[2 * nv]);
      linf[(size_t)m * nv + q] = r[nv + q];
    }
  }
  return TAG_OK;
}

int tag_lgl_basis(int32_t polydeg, double* nodes, double* weights) {
  if (polydeg < 1 || polydeg > 64 || !nodes || !weights)
    return fail(TAG_E_INVALID, "bad argument");
  lgl_nodes_weights(polydeg, nodes, weights);
  return TAG_OK;
}

}  // extern "C"
