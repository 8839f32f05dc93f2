// tag_rhs_noalloc: the 2D dry-Euler right-hand side for callers that cannot
// allocate device memory themselves or through this library — for example a
// host program whose device memory is owned by an arena or memory pool that
// only it may carve up, or a Julia session whose GPU array allocator owns every
// buffer.  Such a caller passes device buffers for everything it owns (state,
// tendency, geometry, connectivity); the one buffer the kernels need beyond
// those — the surface-flux scratch between the interface kernel and the
// element kernel — lives in a fixed file-scope device array of this library.
//
// The scratch array is per device: each GPU that loads the library holds it
// (kNoallocScratchDoubles doubles = 8 MiB) until the process exits.  All calls
// on one device share it, so two calls whose kernels overlap in time on the
// same GPU (different streams, different host threads) race on it and give
// wrong results; callers must order such calls.
//
// The array's device address is looked up once per device and kept.  It
// belongs to the device's primary context (the one the CUDA runtime, PyTorch
// and Julia's CUDA.jl use): calls made under another context of the same
// device, or after cudaDeviceReset destroyed the primary context, would use a
// stale address and are not supported.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "dg2d_kernels.cuh"
#include "phys_euler_energy_2d.cuh"

using namespace tag;

namespace {

constexpr size_t kNoallocScratchDoubles = size_t(1) << 20;  // 8 MiB
constexpr int kMaxDevices = 64;

// Scratch for the outward surface fluxes sfv[e][face][l][NA] and the status word.
static __device__ __align__(256) double g_noalloc_sfv[kNoallocScratchDoubles];
static __device__ __align__(256) unsigned g_noalloc_status[64];

// Device addresses of the arrays above, looked up once per device (the host
// symbols are stand-ins, not device addresses).
std::mutex g_setup_mutex;
double* g_sfv_dev[kMaxDevices] = {};
unsigned* g_status_dev[kMaxDevices] = {};

int nfail(int code, const std::string& msg) {
  tag::set_last_error(msg);  // reported by tag_last_error()
  return code;
}

// Boundary kinds this entry point evaluates: the slip walls need nothing but
// the inner state; a Dirichlet face would need the per-face boundary states
// that only a tag_create handle owns (tag_set_boundary_values).
bool supported_boundary_kind(int32_t k) {
  return k == TAG_BC_SLIP_WALL_STRUCTURED || k == TAG_BC_SLIP_WALL_NORMAL;
}

// Reads the caller's boundary_kinds (device memory) in fixed-size pieces into
// a stack buffer, ordered on `s` after the caller's own work, and rejects any
// kind the kernels cannot evaluate without more data.
int check_boundary_kinds(const int32_t* kinds, int nbd, cudaStream_t s) {
  constexpr int kChunk = 1024;
  int32_t buf[kChunk];
  for (int off = 0; off < nbd; off += kChunk) {
    const int m = nbd - off < kChunk ? nbd - off : kChunk;
    cudaError_t e = cudaMemcpyAsync(buf, kinds + off, sizeof(int32_t) * m, cudaMemcpyDefault, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
      return nfail(TAG_E_CUDA, std::string("reading boundary_kinds: ") + cudaGetErrorString(e));
    for (int k = 0; k < m; ++k)
      if (!supported_boundary_kind(buf[k]))
        return nfail(TAG_E_INVALID,
                     "tag_rhs_noalloc evaluates slip walls only (TAG_BC_SLIP_WALL_STRUCTURED, "
                     "TAG_BC_SLIP_WALL_NORMAL); boundary face " + std::to_string(off + k) +
                         " has kind " + std::to_string(buf[k]));
  }
  return TAG_OK;
}

// Widest launch the element kernel allows (its register use bounds the
// threads per block); the kernel strides over its block, so a narrower
// block computes the same result.
template <int n>
int element_thread_cap(int& cap) {
  static int c = 0;
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    cudaFuncAttributes a;
    err = cudaFuncGetAttributes(&a, k_element<PhysEnergy2D, n, kModeRhs>);
    if (err == cudaSuccess) c = (a.maxThreadsPerBlock / 32) * 32;
  });
  if (err != cudaSuccess)
    return nfail(TAG_E_CUDA, std::string("cudaFuncGetAttributes: ") + cudaGetErrorString(err));
  cap = c;
  return TAG_OK;
}

int setup_device(int dev, double** sfv, unsigned** status) {
  if (dev < 0 || dev >= kMaxDevices) return nfail(TAG_E_INVALID, "device ordinal too large");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_sfv_dev[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sfv);
    if (e != cudaSuccess)
      return nfail(TAG_E_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    void* q = nullptr;
    e = cudaGetSymbolAddress(&q, g_noalloc_status);
    if (e != cudaSuccess)
      return nfail(TAG_E_CUDA, std::string("cudaGetSymbolAddress(status): ") + cudaGetErrorString(e));
    g_status_dev[dev] = static_cast<unsigned*>(q);
    g_sfv_dev[dev] = static_cast<double*>(p);
  }
  *sfv = g_sfv_dev[dev];
  *status = g_status_dev[dev];
  return TAG_OK;
}

template <int n>
int launch_noalloc(const tag_config* cfg, const PhysEnergy2D::Params& P, const BasisDev& basis,
                   const double* u, double* du, cudaStream_t s, double* sfv, unsigned* status) {
  using Phys = PhysEnergy2D;
  using S = ElemSmem<Phys, n>;
  const int nelem = cfg->nelements, nif = cfg->ninterfaces, nbd = cfg->nboundaries;
  const int total = (nif + nbd) * n;
  if (total > 0) {
    k_interface<Phys, n><<<(total + 255) / 256, 256, 0, s>>>(
        P, u, cfg->contravariant_vectors, cfg->inverse_jacobian, cfg->interface_elements,
        cfg->interface_faces, cfg->interface_flip, nif, cfg->boundary_elements,
        cfg->boundary_faces, cfg->boundary_kinds, nbd, sfv);
  }
  // elements per CTA: the largest count whose shared memory fits the default
  // 48 KB window (no attribute change needed)
  int cap = 0;
  int rc = element_thread_cap<n>(cap);
  if (rc) return rc;
  int epb = 1;
  while (epb < 16 && S::bytes(epb + 1) <= 48 * 1024 && (epb + 1) * S::TPE <= 1024) ++epb;
  const int threads = std::min(cap, epb * S::TPE);
  StageArgs st{};
  k_element<Phys, n, kModeRhs><<<(nelem + epb - 1) / epb, threads, S::bytes(epb), s>>>(
      P, basis, const_cast<double*>(u), du, nullptr, cfg->contravariant_vectors,
      cfg->inverse_jacobian, sfv, nelem, epb, st, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return nfail(TAG_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return TAG_OK;
}

}  // namespace

extern "C" {

int tag_rhs_noalloc(const tag_config* cfg, const double* u, double* du, void* stream,
                    uint32_t* status_out) {
  if (!cfg || !u || !du) return nfail(TAG_E_INVALID, "null argument");
  if (cfg->equations != TAG_EQ_EULER_ENERGY_2D || cfg->volume_flux != TAG_VF_RANOCHA_WARUSZEWSKI ||
      cfg->surface_flux != TAG_SF_LMARS)
    return nfail(TAG_E_INVALID, "tag_rhs_noalloc supports TAG_EQ_EULER_ENERGY_2D with "
                                "TAG_VF_RANOCHA_WARUSZEWSKI / TAG_SF_LMARS only");
  const int n = cfg->polydeg + 1;
  if (n < 2 || n > kMaxNodes) return nfail(TAG_E_INVALID, "polydeg out of range 1..7");
  if (cfg->nelements <= 0 || cfg->ninterfaces < 0 || cfg->nboundaries < 0)
    return nfail(TAG_E_INVALID, "bad mesh sizes");
  if (cfg->nmembers > 1) return nfail(TAG_E_INVALID, "tag_rhs_noalloc takes a single mesh");
  if (!cfg->derivative_split || !cfg->weights || !cfg->contravariant_vectors ||
      !cfg->inverse_jacobian || (cfg->ninterfaces > 0 && (!cfg->interface_elements ||
                                                           !cfg->interface_faces ||
                                                           !cfg->interface_flip)) ||
      (cfg->nboundaries > 0 && (!cfg->boundary_elements || !cfg->boundary_faces ||
                                !cfg->boundary_kinds)))
    return nfail(TAG_E_INVALID, "missing basis, geometry or connectivity array");
  const size_t need = (size_t)cfg->nelements * 4 * n * PhysEnergy2D::NA;
  if (need > kNoallocScratchDoubles)
    return nfail(TAG_E_INVALID,
                 "mesh too large for tag_rhs_noalloc: needs " + std::to_string(need) +
                     " scratch doubles, the fixed maximum is " +
                     std::to_string(kNoallocScratchDoubles) + " (nelements * 4 * (polydeg+1) * 4)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nfail(TAG_E_NO_DEVICE, cudaGetErrorString(e));
  double* sfv = nullptr;
  unsigned* status = nullptr;
  int rc = setup_device(dev, &sfv, &status);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cfg->nboundaries > 0 && (rc = check_boundary_kinds(cfg->boundary_kinds, cfg->nboundaries, s)))
    return rc;
  // the shared scratch keeps the previous call's contents: clear it (a well-
  // formed mesh lists every face as an interface side or a boundary face and
  // overwrites all of it; a face listed nowhere then reads zero flux rather
  // than another call's data; at most 8 MiB of writes, about 1 us)
  e = cudaMemsetAsync(sfv, 0, need * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return nfail(TAG_E_CUDA, cudaGetErrorString(e));
  const PhysEnergy2D::Params P = PhysEnergy2D::make_params(cfg->params);
  BasisDev basis{};
  for (int a = 0; a < n; ++a)
    for (int c = 0; c < n; ++c) basis.Ds[a * n + c] = cfg->derivative_split[a + n * c];
  basis.winv0 = 1.0 / cfg->weights[0];
  basis.winvN = 1.0 / cfg->weights[n - 1];
  switch (n) {
    case 2: rc = launch_noalloc<2>(cfg, P, basis, u, du, s, sfv, status); break;
    case 3: rc = launch_noalloc<3>(cfg, P, basis, u, du, s, sfv, status); break;
    case 4: rc = launch_noalloc<4>(cfg, P, basis, u, du, s, sfv, status); break;
    case 5: rc = launch_noalloc<5>(cfg, P, basis, u, du, s, sfv, status); break;
    case 6: rc = launch_noalloc<6>(cfg, P, basis, u, du, s, sfv, status); break;
    case 7: rc = launch_noalloc<7>(cfg, P, basis, u, du, s, sfv, status); break;
    default: rc = launch_noalloc<8>(cfg, P, basis, u, du, s, sfv, status); break;
  }
  if (rc) return rc;
  unsigned flags = 0;
  e = cudaMemcpyAsync(&flags, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return nfail(TAG_E_CUDA, cudaGetErrorString(e));
  if (status_out) *status_out = flags;
  return TAG_OK;
}

}  // extern "C"
