// Learned initial guess for the rainy saturation Newton solve: FP32 MLP
// 5 -> 32 -> 32 -> 1 (tanh), with hand-written CUDA kernels for inference
// (fused into k_newton_rainy), for the loss gradient and for Adam training.
//
// Training data are (state, converged temperature) pairs produced by the
// reference's Newton algorithm (k_newton_rainy run to a tight tolerance from
// the warm start, the same iteration as nonlinear_solve_dg2d.jl:6-44); on the
// nodes that are saturated at equilibrium the network predicts the normalised
// offset T* - T_unsat from the normalised inputs of mlp_inputs().  Gradients of one batch are accumulated per CTA in a fixed
// order and then summed over CTAs in a fixed order, so training is bitwise
// reproducible for a given seed.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "newton_rainy.cuh"

using namespace tag;

namespace {

constexpr int kSamplesPerBlock = 64;
constexpr int kGradThreads = 256;

#define MLP_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      tag::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));         \
      return TAG_E_CUDA;                                                                \
    }                                                                                   \
  } while (0)

// One CTA: forward + backward of up to kSamplesPerBlock samples (indices idx),
// then the CTA's partial gradient of the summed loss (d/dparams of
// sum_s (y_s - t_s)^2) into part[blockIdx.x][kMlpTrain], and its loss sum into
// lpart[blockIdx.x].
__global__ void __launch_bounds__(kGradThreads) k_mlp_grad(
    const float* __restrict__ P, const float* __restrict__ X, const float* __restrict__ T,
    const int* __restrict__ idx, int nbatch, float* __restrict__ part, float* __restrict__ lpart) {
  __shared__ float sp[kMlpParams];
  __shared__ float xs[kSamplesPerBlock][kMlpIn];
  __shared__ float h1[kSamplesPerBlock][kMlpH];
  __shared__ float h2[kSamplesPerBlock][kMlpH];
  __shared__ float d2[kSamplesPerBlock][kMlpH];
  __shared__ float d1[kSamplesPerBlock][kMlpH];
  __shared__ float dy[kSamplesPerBlock];
  for (int t = threadIdx.x; t < kMlpParams; t += blockDim.x) sp[t] = P[t];
  __syncthreads();
  const int s0 = blockIdx.x * kSamplesPerBlock;
  const int ns = min(kSamplesPerBlock, nbatch - s0);
  if (threadIdx.x < kSamplesPerBlock) {
    const int s = threadIdx.x;
    if (s < ns) {
      const int q = idx ? idx[s0 + s] : s0 + s;
      float x[kMlpIn];
#pragma unroll
      for (int k = 0; k < kMlpIn; ++k) {
        x[k] = (X[(size_t)q * kMlpIn + k] - sp[oInMean + k]) * sp[oInScale + k];
        xs[s][k] = x[k];
      }
      for (int o = 0; o < kMlpH; ++o) {
        float z = sp[oB1 + o];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) z = fmaf(sp[oW1 + o * kMlpIn + k], x[k], z);
        h1[s][o] = tanhf(z);
      }
      float y = sp[oB3];
      for (int o = 0; o < kMlpH; ++o) {
        float z = sp[oB2 + o];
        for (int k = 0; k < kMlpH; ++k) z = fmaf(sp[oW2 + o * kMlpH + k], h1[s][k], z);
        h2[s][o] = tanhf(z);
        y = fmaf(sp[oW3 + o], h2[s][o], y);
      }
      const float t = (T[q] - sp[oOutMean]) / sp[oOutScale];
      const float e = y - t;
      dy[s] = 2.0f * e;
      for (int o = 0; o < kMlpH; ++o) d2[s][o] = dy[s] * sp[oW3 + o] * (1.0f - h2[s][o] * h2[s][o]);
      for (int k = 0; k < kMlpH; ++k) {
        float a = 0.0f;
        for (int o = 0; o < kMlpH; ++o) a = fmaf(sp[oW2 + o * kMlpH + k], d2[s][o], a);
        d1[s][k] = a * (1.0f - h1[s][k] * h1[s][k]);
      }
    } else {
      dy[s] = 0.0f;
      for (int o = 0; o < kMlpH; ++o) {
        h1[s][o] = h2[s][o] = d2[s][o] = d1[s][o] = 0.0f;
      }
      for (int k = 0; k < kMlpIn; ++k) xs[s][k] = 0.0f;
    }
  }
  __syncthreads();
  float* g = part + (size_t)blockIdx.x * kMlpTrain;
  for (int p = threadIdx.x; p < kMlpTrain; p += blockDim.x) {
    float a = 0.0f;
    if (p < oB1) {                         // W1[o][k]
      const int o = p / kMlpIn, k = p % kMlpIn;
      for (int s = 0; s < kSamplesPerBlock; ++s) a = fmaf(d1[s][o], xs[s][k], a);
    } else if (p < oW2) {                  // b1[o]
      const int o = p - oB1;
      for (int s = 0; s < kSamplesPerBlock; ++s) a += d1[s][o];
    } else if (p < oB2) {                  // W2[o][k]
      const int o = (p - oW2) / kMlpH, k = (p - oW2) % kMlpH;
      for (int s = 0; s < kSamplesPerBlock; ++s) a = fmaf(d2[s][o], h1[s][k], a);
    } else if (p < oW3) {                  // b2[o]
      const int o = p - oB2;
      for (int s = 0; s < kSamplesPerBlock; ++s) a += d2[s][o];
    } else if (p < oB3) {                  // W3[o]
      const int o = p - oW3;
      for (int s = 0; s < kSamplesPerBlock; ++s) a = fmaf(dy[s], h2[s][o], a);
    } else {                               // b3
      for (int s = 0; s < kSamplesPerBlock; ++s) a += dy[s];
    }
    g[p] = a;
  }
  if (threadIdx.x == 0) {
    float l = 0.0f;
    for (int s = 0; s < kSamplesPerBlock; ++s) l += 0.25f * dy[s] * dy[s];
    lpart[blockIdx.x] = l;
  }
}

// Sum of the CTA partials in a fixed order, scaled by 1/nbatch (mean loss).
__global__ void k_mlp_reduce(const float* __restrict__ part, int nparts, float scale,
                             float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpTrain) return;
  float a = 0.0f;
  for (int b = 0; b < nparts; ++b) a += part[(size_t)b * kMlpTrain + p];
  grad[p] = a * scale;
}

// Adam (Kingma & Ba 2015) on the trainable parameters.
__global__ void k_mlp_adam(float* __restrict__ P, const float* __restrict__ grad,
                           float* __restrict__ m, float* __restrict__ v, float lr, float b1,
                           float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpTrain) return;
  const float gr = grad[p];
  const float mn = b1 * m[p] + (1.0f - b1) * gr;
  const float vn = b2 * v[p] + (1.0f - b2) * gr * gr;
  m[p] = mn;
  v[p] = vn;
  P[p] -= lr * (mn / c1) / (sqrtf(vn / c2) + eps);
}

__global__ void k_mlp_forward(const float* __restrict__ P, const float* __restrict__ X, long n,
                              float* __restrict__ Y) {
  __shared__ float sp[kMlpParams];
  for (int t = threadIdx.x; t < kMlpParams; t += blockDim.x) sp[t] = P[t];
  __syncthreads();
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  Y[q] = mlp_forward(sp, X + q * kMlpIn);
}

// Philox-free deterministic permutation (Fisher-Yates with a 64-bit LCG).
void permute(std::vector<int>& a, unsigned long long& st) {
  for (long i = (long)a.size() - 1; i > 0; --i) {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    const long j = (long)((st >> 33) % (unsigned long long)(i + 1));
    std::swap(a[i], a[j]);
  }
}

}  // namespace

extern "C" {

int tag_mlp_forward(const float* params, const float* x, int64_t n, float* y) {
  if (!params || !x || !y || n <= 0) {
    tag::set_last_error("bad argument");
    return TAG_E_INVALID;
  }
  float *dP = nullptr, *dX = nullptr, *dY = nullptr;
  MLP_CUDA(cudaMalloc(&dP, sizeof(float) * kMlpParams));
  MLP_CUDA(cudaMalloc(&dX, sizeof(float) * n * kMlpIn));
  MLP_CUDA(cudaMalloc(&dY, sizeof(float) * n));
  MLP_CUDA(cudaMemcpy(dP, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dX, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
  k_mlp_forward<<<(unsigned)((n + 255) / 256), 256>>>(dP, dX, (long)n, dY);
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemcpy(y, dY, sizeof(float) * n, cudaMemcpyDeviceToHost));
  cudaFree(dP);
  cudaFree(dX);
  cudaFree(dY);
  return TAG_OK;
}

int tag_mlp_loss_grad(const float* params, const float* x, const float* t, int64_t n,
                      float* grad, float* loss) {
  if (!params || !x || !t || !grad || !loss || n <= 0) {
    tag::set_last_error("bad argument");
    return TAG_E_INVALID;
  }
  const int nb = (int)((n + kSamplesPerBlock - 1) / kSamplesPerBlock);
  float *dP, *dX, *dT, *dPart, *dL, *dG;
  MLP_CUDA(cudaMalloc(&dP, sizeof(float) * kMlpParams));
  MLP_CUDA(cudaMalloc(&dX, sizeof(float) * n * kMlpIn));
  MLP_CUDA(cudaMalloc(&dT, sizeof(float) * n));
  MLP_CUDA(cudaMalloc(&dPart, sizeof(float) * nb * kMlpTrain));
  MLP_CUDA(cudaMalloc(&dL, sizeof(float) * nb));
  MLP_CUDA(cudaMalloc(&dG, sizeof(float) * kMlpTrain));
  MLP_CUDA(cudaMemcpy(dP, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dX, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dT, t, sizeof(float) * n, cudaMemcpyHostToDevice));
  k_mlp_grad<<<nb, kGradThreads>>>(dP, dX, dT, nullptr, (int)n, dPart, dL);
  k_mlp_reduce<<<(kMlpTrain + 255) / 256, 256>>>(dPart, nb, 1.0f / (float)n, dG);
  MLP_CUDA(cudaGetLastError());
  std::vector<float> lp(nb);
  MLP_CUDA(cudaMemcpy(grad, dG, sizeof(float) * kMlpTrain, cudaMemcpyDeviceToHost));
  MLP_CUDA(cudaMemcpy(lp.data(), dL, sizeof(float) * nb, cudaMemcpyDeviceToHost));
  double l = 0.0;
  for (float v : lp) l += v;
  *loss = (float)(l / (double)n);
  cudaFree(dP); cudaFree(dX); cudaFree(dT); cudaFree(dPart); cudaFree(dL); cudaFree(dG);
  return TAG_OK;
}

// Adam training on the GPU: `epochs` passes over the n samples in shuffled
// mini-batches of `batch` (a multiple of 64), learning rate lr decayed by
// cosine to lr/20.  params (kMlpParams floats, normalisation already set) are
// read and replaced; loss_per_epoch (may be null) receives the mean training
// loss of each epoch.
int tag_mlp_train(float* params, const float* x, const float* t, int64_t n, int32_t epochs,
                  int32_t batch, float lr, uint64_t seed, float* loss_per_epoch) {
  if (!params || !x || !t || n < batch || batch < kSamplesPerBlock || epochs <= 0 ||
      batch % kSamplesPerBlock) {
    tag::set_last_error("bad argument");
    return TAG_E_INVALID;
  }
  const int nb = batch / kSamplesPerBlock;
  float *dP, *dX, *dT, *dPart, *dL, *dG, *dM, *dV;
  int* dIdx;
  MLP_CUDA(cudaMalloc(&dP, sizeof(float) * kMlpParams));
  MLP_CUDA(cudaMalloc(&dX, sizeof(float) * n * kMlpIn));
  MLP_CUDA(cudaMalloc(&dT, sizeof(float) * n));
  MLP_CUDA(cudaMalloc(&dIdx, sizeof(int) * n));
  MLP_CUDA(cudaMalloc(&dPart, sizeof(float) * nb * kMlpTrain));
  MLP_CUDA(cudaMalloc(&dL, sizeof(float) * nb));
  MLP_CUDA(cudaMalloc(&dG, sizeof(float) * kMlpTrain));
  MLP_CUDA(cudaMalloc(&dM, sizeof(float) * kMlpTrain));
  MLP_CUDA(cudaMalloc(&dV, sizeof(float) * kMlpTrain));
  MLP_CUDA(cudaMemcpy(dP, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dX, x, sizeof(float) * n * kMlpIn, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(dT, t, sizeof(float) * n, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemset(dM, 0, sizeof(float) * kMlpTrain));
  MLP_CUDA(cudaMemset(dV, 0, sizeof(float) * kMlpTrain));
  std::vector<int> perm(n);
  for (long i = 0; i < n; ++i) perm[i] = (int)i;
  unsigned long long st = seed * 0x9E3779B97F4A7C15ull + 1;
  const long steps_per_epoch = n / batch;
  const long total = steps_per_epoch * epochs;
  long step = 0;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  std::vector<float> lp(nb);
  for (int ep = 0; ep < epochs; ++ep) {
    permute(perm, st);
    MLP_CUDA(cudaMemcpy(dIdx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    double lsum = 0.0;
    for (long b = 0; b < steps_per_epoch; ++b, ++step) {
      k_mlp_grad<<<nb, kGradThreads>>>(dP, dX, dT, dIdx + b * batch, batch, dPart, dL);
      k_mlp_reduce<<<(kMlpTrain + 255) / 256, 256>>>(dPart, nb, 1.0f / (float)batch, dG);
      const float frac = (float)step / (float)total;
      const float lr_t = lr * (0.05f + 0.95f * 0.5f * (1.0f + cosf(3.14159265f * frac)));
      const float c1 = 1.0f - powf(b1, (float)(step + 1));
      const float c2 = 1.0f - powf(b2, (float)(step + 1));
      k_mlp_adam<<<(kMlpTrain + 255) / 256, 256>>>(dP, dG, dM, dV, lr_t, b1, b2, eps, c1, c2);
      if (loss_per_epoch && (b % 16 == 0 || b == steps_per_epoch - 1)) {
        MLP_CUDA(cudaMemcpy(lp.data(), dL, sizeof(float) * nb, cudaMemcpyDeviceToHost));
        double l = 0.0;
        for (float v : lp) l += v;
        lsum = l / batch;  // latest sampled batch loss
      }
    }
    MLP_CUDA(cudaGetLastError());
    if (loss_per_epoch) loss_per_epoch[ep] = (float)lsum;
  }
  MLP_CUDA(cudaMemcpy(params, dP, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  cudaFree(dP); cudaFree(dX); cudaFree(dT); cudaFree(dIdx); cudaFree(dPart); cudaFree(dL);
  cudaFree(dG); cudaFree(dM); cudaFree(dV);
  return TAG_OK;
}

// Saturation Newton solve on `n` host states u[n][9] (slots 7-9 updated in
// place); see tag_newton_solve for the arguments.  mlp (host, may be null)
// selects the learned initial guess.
int tag_newton_solve_states(double* u, int64_t n, int32_t mode, double tol, int32_t max_iterations,
                            int32_t polish, const float* mlp, int32_t* iters,
                            tag_newton_stats* stats) {
  if (!u || n <= 0 || (mode != 0 && mode != 1) || !(tol > 0.0) || max_iterations < 1) {
    tag::set_last_error("bad argument");
    return TAG_E_INVALID;
  }
  double* dU;
  float* dP = nullptr;
  int* dI;
  unsigned long long* dC;
  unsigned* dS;
  MLP_CUDA(cudaMalloc(&dU, sizeof(double) * 9 * n));
  MLP_CUDA(cudaMalloc(&dI, sizeof(int) * n));
  MLP_CUDA(cudaMalloc(&dC, sizeof(unsigned long long) * 4));
  MLP_CUDA(cudaMalloc(&dS, sizeof(unsigned)));
  MLP_CUDA(cudaMemcpy(dU, u, sizeof(double) * 9 * n, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemset(dC, 0, sizeof(unsigned long long) * 4));
  MLP_CUDA(cudaMemset(dS, 0, sizeof(unsigned)));
  if (mlp) {
    MLP_CUDA(cudaMalloc(&dP, sizeof(float) * kMlpParams));
    MLP_CUDA(cudaMemcpy(dP, mlp, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
  }
  NewtonArgs a{mode, max_iterations, polish, mlp ? 1 : 0, 8, tol, dP, dI, dC};
  MLP_CUDA(launch_newton_rainy(dU, (long)n, a, dS, nullptr));
  unsigned long long c[4];
  MLP_CUDA(cudaMemcpy(u, dU, sizeof(double) * 9 * n, cudaMemcpyDeviceToHost));
  MLP_CUDA(cudaMemcpy(c, dC, sizeof(c), cudaMemcpyDeviceToHost));
  if (iters) MLP_CUDA(cudaMemcpy(iters, dI, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if (stats) {
    stats->nodes = n;
    stats->updates = (int64_t)c[0];
    stats->fallbacks = (int64_t)c[1];
    stats->not_converged = (int64_t)c[2];
  }
  cudaFree(dU); cudaFree(dI); cudaFree(dC); cudaFree(dS);
  if (dP) cudaFree(dP);
  return TAG_OK;
}

}  // extern "C"
