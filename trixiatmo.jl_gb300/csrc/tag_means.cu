// tag_eval_means: evaluates the device forms of the logarithmic and Stolarsky
// means (the kernels' own inline functions) on arrays of value pairs, so that
// they can be checked directly against exact values on both sides of every
// branch threshold.  Diagnostics only: no kernel of the right-hand side calls
// this path.
#include <cuda_runtime.h>

#include <string>

#include "phys_pt_2d.cuh"
#include "tag_common.cuh"

using namespace tag;

namespace {

int mfail(int code, const std::string& msg) {
  set_last_error(msg);
  return code;
}

// kind 0: ln_mean_pair (2D kernels: six-coefficient polynomials, logarithms inline)
// kind 1: ln_mean_pair with per-node logarithms and the four-term short form
// kind 2: ln_mean_pair_halved (3D energy kernel; halved inputs)
// kind 3: ln_mean_single / inv_ln_mean_single
// kind 4: Stolarsky mean of the potential-temperature kernels (out2 unused)
// kind 5: ln_mean_pair_halved with the pair as the ln_mean pair and (1, 1) as
//         the inv_ln_mean pair; kind 6 the other way round
// out1 = ln_mean(x, y) (kind 4: the Stolarsky mean), out2 = inv_ln_mean(x, y);
// kinds 5 and 6 return the means of their (x, y) and (1, 1) pairs.
__global__ void k_eval_means(int kind, long n, const double* __restrict__ x,
                             const double* __restrict__ y, PhysPT2D::Params pt,
                             double* __restrict__ out1, double* __restrict__ out2) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double a = x[q], b = y[q];
  double m = 0.0, im = 0.0;
  if (kind == 0) {
    ln_mean_pair<false>(a, b, a, b, 0.0, 0.0, 0.0, 0.0, m, im);
  } else if (kind == 1) {
    const double la = log(a), lb = log(b);
    ln_mean_pair<true>(a, b, a, b, la, lb, la, lb, m, im);
  } else if (kind == 2) {
    const double ha = 0.5 * a, hb = 0.5 * b;
    const double la = log(ha), lb = log(hb);
    ln_mean_pair_halved(ha, hb, ha, hb, la, lb, la, lb, m, im);
  } else if (kind == 5 || kind == 6) {
    const double ha = 0.5 * a, hb = 0.5 * b;
    const double la = log(ha), lb = log(hb), l1 = log(0.5);
    if (kind == 5)
      ln_mean_pair_halved(ha, hb, 0.5, 0.5, la, lb, l1, l1, m, im);
    else
      ln_mean_pair_halved(0.5, 0.5, ha, hb, l1, l1, la, lb, m, im);
  } else if (kind == 3) {
    m = ln_mean_single(a, b);
    im = inv_ln_mean_single(a, b);
  } else {
    const double ag = pow(a, pt.gamma), bg = pow(b, pt.gamma);
    m = PhysPT2D::stolarsky(pt, a, b, ag, ag / a, bg, bg / b);
  }
  out1[q] = m;
  out2[q] = im;
}

}  // namespace

extern "C" {

int tag_eval_means(int32_t kind, int64_t n, double gamma_cp, double gamma_cv, const double* x,
                   const double* y, double* out1, double* out2) {
  if (kind < 0 || kind > 6 || n < 0 || (n > 0 && (!x || !y || !out1 || !out2)))
    return mfail(TAG_E_INVALID, "tag_eval_means: bad argument");
  if (n == 0) return TAG_OK;
  const double pp[8] = {gamma_cp, gamma_cv, 9.81, 340.0, 0.0, 0.0, 0.0, 1.0};
  const PhysPT2D::Params pt = PhysPT2D::make_params(pp);
  double* d = nullptr;
  const size_t bytes = sizeof(double) * (size_t)n;
  cudaError_t e = cudaMalloc(&d, 4 * bytes);
  if (e != cudaSuccess) return mfail(TAG_E_CUDA, cudaGetErrorString(e));
  e = cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, y, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_eval_means<<<(unsigned)((n + 255) / 256), 256>>>(kind, n, d, d + n, pt, d + 2 * n, d + 3 * n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out1, d + 2 * n, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(out2, d + 3 * n, bytes, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return mfail(TAG_E_CUDA, cudaGetErrorString(e));
  return TAG_OK;
}

}  // extern "C"
