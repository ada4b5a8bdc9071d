// FP32 MLP of the learned kernel selection (tuner.h): 16 features -> 64 ReLU
// -> 64 ReLU -> kNumConfigs linear outputs (predicted log2 cost of each
// configuration relative to the fastest).  Forward, backward and the Adam
// update are hand-written kernels; every reduction runs in a fixed order, so
// training is deterministic for a given seed.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "common.h"
#include "tuner.h"

namespace vnec {
namespace {

constexpr int F = kNumFeatures, Hd = kHidden, C = kNumConfigs;
// Offsets of the parameter blocks.
constexpr int oW1 = 0, ob1 = oW1 + Hd * F, oW2 = ob1 + Hd, ob2 = oW2 + Hd * Hd, oW3 = ob2 + Hd, ob3 = oW3 + C * Hd;
static_assert(ob3 + C == kMlpParams, "parameter layout");

// Y[b, n] = act(sum_k X[b, k] W[n, k] + bias[n]).
__global__ void linear_fwd(const float* __restrict__ X, const float* __restrict__ W, const float* __restrict__ bias,
                           float* __restrict__ Y, int B, int K, int N, int relu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * N) return;
  const int b = i / N, n = i % N;
  float s = bias[n];
  for (int k = 0; k < K; ++k) s = fmaf(X[b * K + k], W[n * K + k], s);
  Y[i] = relu ? fmaxf(s, 0.f) : s;
}

// dX[b, k] = sum_n dY[b, n] W[n, k], times (H[b, k] > 0) when H is given.
__global__ void linear_bwd_input(const float* __restrict__ dY, const float* __restrict__ W,
                                 const float* __restrict__ H, float* __restrict__ dX, int B, int K, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * K) return;
  const int b = i / K, k = i % K;
  float s = 0.f;
  for (int n = 0; n < N; ++n) s = fmaf(dY[b * N + n], W[n * K + k], s);
  dX[i] = (H && H[i] <= 0.f) ? 0.f : s;
}

// dW[n, k] = sum_b dY[b, n] X[b, k]; db[n] = sum_b dY[b, n] (threads k == K).
__global__ void linear_bwd_weight(const float* __restrict__ dY, const float* __restrict__ X, float* __restrict__ dW,
                                  float* __restrict__ db, int B, int K, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * (K + 1)) return;
  const int n = i / (K + 1), k = i % (K + 1);
  float s = 0.f;
  if (k < K) {
    for (int b = 0; b < B; ++b) s = fmaf(dY[b * N + n], X[b * K + k], s);
    dW[n * K + k] = s;
  } else {
    for (int b = 0; b < B; ++b) s += dY[b * N + n];
    db[n] = s;
  }
}

// Masked mean squared error: dO = 2 M (O - T) / sum(M); per-sample partial
// losses into lossv[b] (summed on the host in order).
__global__ void mse_grad(const float* __restrict__ O, const float* __restrict__ T, const float* __restrict__ M,
                         float* __restrict__ dO, float* __restrict__ lossv, int B, float inv_count) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  float l = 0.f;
  for (int c = 0; c < C; ++c) {
    const int i = b * C + c;
    const float d = (O[i] - T[i]) * M[i];
    dO[i] = 2.f * d * inv_count;
    l = fmaf(d, d, l);
  }
  lossv[b] = l;
}

__global__ void adam_step(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                          float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float wd, float c1,
                          float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] + wd * p[i];
  m1[i] = b1 * m1[i] + (1.f - b1) * gi;
  m2[i] = b2 * m2[i] + (1.f - b2) * gi * gi;
  p[i] -= lr * (m1[i] * c1) / (sqrtf(m2[i] * c2) + eps);
}

__global__ void gather_rows(const float* __restrict__ src, const int* __restrict__ idx, float* __restrict__ dst, int n,
                            int w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * w) return;
  dst[i] = src[idx[i / w] * w + i % w];
}

inline unsigned blocks(int n) { return (unsigned)((n + 127) / 128); }

}  // namespace

struct MlpModel {
  DeviceBuffer params, grad, m1, m2;
  // Activations of the current batch (capacity `cap` rows).
  DeviceBuffer X, T, M, H1, H2, O, dO, dH2, dH1, lossv;
  int cap = 0;
  bool reserve(int n) {
    if (n <= cap) return true;
    const size_t f = sizeof(float);
    X.release(); T.release(); M.release(); H1.release(); H2.release(); O.release(); dO.release(); dH2.release();
    dH1.release(); lossv.release();
    if (!X.alloc(f * n * F) || !T.alloc(f * n * C) || !M.alloc(f * n * C) || !H1.alloc(f * n * Hd) ||
        !H2.alloc(f * n * Hd) || !O.alloc(f * n * C) || !dO.alloc(f * n * C) || !dH2.alloc(f * n * Hd) ||
        !dH1.alloc(f * n * Hd) || !lossv.alloc(f * n))
      return false;
    cap = n;
    return true;
  }
  bool forward(int n) {
    const float* P = params.as<float>();
    linear_fwd<<<blocks(n * Hd), 128>>>(X.as<float>(), P + oW1, P + ob1, H1.as<float>(), n, F, Hd, 1);
    linear_fwd<<<blocks(n * Hd), 128>>>(H1.as<float>(), P + oW2, P + ob2, H2.as<float>(), n, Hd, Hd, 1);
    linear_fwd<<<blocks(n * C), 128>>>(H2.as<float>(), P + oW3, P + ob3, O.as<float>(), n, Hd, C, 0);
    return VNEC_CUDA(cudaGetLastError());
  }
  // Loss and gradient of the batch in X/T/M (n rows) into `grad`.
  bool backward(int n, float mask_sum, float* loss) {
    const float* P = params.as<float>();
    float* G = grad.as<float>();
    mse_grad<<<blocks(n), 128>>>(O.as<float>(), T.as<float>(), M.as<float>(), dO.as<float>(), lossv.as<float>(), n,
                                 1.f / std::max(mask_sum, 1.f));
    linear_bwd_weight<<<blocks(C * (Hd + 1)), 128>>>(dO.as<float>(), H2.as<float>(), G + oW3, G + ob3, n, Hd, C);
    linear_bwd_input<<<blocks(n * Hd), 128>>>(dO.as<float>(), P + oW3, H2.as<float>(), dH2.as<float>(), n, Hd, C);
    linear_bwd_weight<<<blocks(Hd * (Hd + 1)), 128>>>(dH2.as<float>(), H1.as<float>(), G + oW2, G + ob2, n, Hd, Hd);
    linear_bwd_input<<<blocks(n * Hd), 128>>>(dH2.as<float>(), P + oW2, H1.as<float>(), dH1.as<float>(), n, Hd, Hd);
    linear_bwd_weight<<<blocks(Hd * (F + 1)), 128>>>(dH1.as<float>(), X.as<float>(), G + oW1, G + ob1, n, F, Hd);
    if (!VNEC_CUDA(cudaGetLastError())) return false;
    if (loss) {
      std::vector<float> lv((size_t)n);
      if (!VNEC_CUDA(cudaMemcpy(lv.data(), lossv.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost))) return false;
      double s = 0.0;
      for (float v : lv) s += v;
      *loss = (float)(s / std::max(mask_sum, 1.f));
    }
    return true;
  }
};

MlpModel* mlp_create(uint64_t seed) {
  auto* m = new MlpModel();
  if (!m->params.alloc(sizeof(float) * kMlpParams) || !m->grad.alloc(sizeof(float) * kMlpParams) ||
      !m->m1.alloc(sizeof(float) * kMlpParams) || !m->m2.alloc(sizeof(float) * kMlpParams)) {
    delete m;
    return nullptr;
  }
  // He-uniform initialisation, zero biases.
  std::vector<float> p(kMlpParams, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int fan_out, int fan_in) {
    const float a = std::sqrt(6.f / (float)fan_in);
    std::uniform_real_distribution<float> u(-a, a);
    for (int i = 0; i < fan_out * fan_in; ++i) p[(size_t)(off + i)] = u(rng);
  };
  fill(oW1, Hd, F);
  fill(oW2, Hd, Hd);
  fill(oW3, C, Hd);
  if (!mlp_set_params(m, p.data())) {
    delete m;
    return nullptr;
  }
  return m;
}

void mlp_destroy(MlpModel* m) { delete m; }

bool mlp_get_params(const MlpModel* m, float* out) {
  return VNEC_CUDA(cudaMemcpy(out, m->params.ptr, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
}

bool mlp_set_params(MlpModel* m, const float* in) {
  return VNEC_CUDA(cudaMemcpy(m->params.ptr, in, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice)) &&
         VNEC_CUDA(cudaMemset(m->m1.ptr, 0, sizeof(float) * kMlpParams)) &&
         VNEC_CUDA(cudaMemset(m->m2.ptr, 0, sizeof(float) * kMlpParams));
}

bool mlp_predict(MlpModel* m, const float* X, int n, float* out) {
  if (n <= 0) return true;
  if (!m->reserve(n) || !VNEC_CUDA(cudaMemcpy(m->X.ptr, X, sizeof(float) * n * F, cudaMemcpyHostToDevice)) ||
      !m->forward(n))
    return false;
  return VNEC_CUDA(cudaMemcpy(out, m->O.ptr, sizeof(float) * n * C, cudaMemcpyDeviceToHost));
}

bool mlp_loss_grad(MlpModel* m, const float* X, const float* T, const float* M, int n, float* loss, float* grad) {
  if (n <= 0 || !m->reserve(n)) return false;
  const size_t f = sizeof(float);
  if (!VNEC_CUDA(cudaMemcpy(m->X.ptr, X, f * n * F, cudaMemcpyHostToDevice)) ||
      !VNEC_CUDA(cudaMemcpy(m->T.ptr, T, f * n * C, cudaMemcpyHostToDevice)) ||
      !VNEC_CUDA(cudaMemcpy(m->M.ptr, M, f * n * C, cudaMemcpyHostToDevice)))
    return false;
  double ms = 0.0;
  for (int i = 0; i < n * C; ++i) ms += M[i];
  if (!m->forward(n) || !m->backward(n, (float)ms, loss)) return false;
  return !grad || VNEC_CUDA(cudaMemcpy(grad, m->grad.ptr, f * kMlpParams, cudaMemcpyDeviceToHost));
}

bool mlp_train(MlpModel* m, const float* X, const float* T, const float* M, int n, const MlpTrainParams& tp,
               float* loss_curve) {
  if (n <= 0 || tp.batch <= 0 || tp.epochs <= 0) {
    set_error("mlp_train: empty data or invalid parameters");
    return false;
  }
  const int bsz = std::min(tp.batch, n);
  const size_t f = sizeof(float);
  DeviceBuffer dX, dT, dM, didx;
  if (!dX.alloc(f * n * F) || !dT.alloc(f * n * C) || !dM.alloc(f * n * C) || !didx.alloc(sizeof(int) * bsz) ||
      !m->reserve(bsz) || !VNEC_CUDA(cudaMemcpy(dX.ptr, X, f * n * F, cudaMemcpyHostToDevice)) ||
      !VNEC_CUDA(cudaMemcpy(dT.ptr, T, f * n * C, cudaMemcpyHostToDevice)) ||
      !VNEC_CUDA(cudaMemcpy(dM.ptr, M, f * n * C, cudaMemcpyHostToDevice)))
    return false;
  std::vector<int> order((size_t)n);
  std::iota(order.begin(), order.end(), 0);
  std::mt19937_64 rng(tp.seed);
  std::vector<float> rowmask((size_t)n);
  for (int i = 0; i < n; ++i) {
    float s = 0.f;
    for (int c = 0; c < C; ++c) s += M[(size_t)i * C + c];
    rowmask[(size_t)i] = s;
  }
  int step = 0;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int ep = 0; ep < tp.epochs; ++ep) {
    std::shuffle(order.begin(), order.end(), rng);
    double ep_loss = 0.0, ep_mask = 0.0;
    for (int s0 = 0; s0 < n; s0 += bsz) {
      const int nb = std::min(bsz, n - s0);
      float msum = 0.f;
      for (int i = 0; i < nb; ++i) msum += rowmask[(size_t)order[(size_t)(s0 + i)]];
      if (!VNEC_CUDA(cudaMemcpy(didx.ptr, order.data() + s0, sizeof(int) * nb, cudaMemcpyHostToDevice))) return false;
      gather_rows<<<blocks(nb * F), 128>>>(dX.as<float>(), didx.as<int>(), m->X.as<float>(), nb, F);
      gather_rows<<<blocks(nb * C), 128>>>(dT.as<float>(), didx.as<int>(), m->T.as<float>(), nb, C);
      gather_rows<<<blocks(nb * C), 128>>>(dM.as<float>(), didx.as<int>(), m->M.as<float>(), nb, C);
      float loss = 0.f;
      if (!m->forward(nb) || !m->backward(nb, msum, loss_curve ? &loss : nullptr)) return false;
      ++step;
      const float c1 = 1.f / (1.f - std::pow(b1, (float)step)), c2 = 1.f / (1.f - std::pow(b2, (float)step));
      adam_step<<<blocks(kMlpParams), 128>>>(m->params.as<float>(), m->grad.as<float>(), m->m1.as<float>(),
                                             m->m2.as<float>(), kMlpParams, tp.lr, b1, b2, 1e-8f, tp.weight_decay, c1,
                                             c2);
      if (!VNEC_CUDA(cudaGetLastError())) return false;
      ep_loss += (double)loss * msum;
      ep_mask += msum;
    }
    if (loss_curve) loss_curve[ep] = (float)(ep_loss / std::max(ep_mask, 1.0));
  }
  return VNEC_CUDA(cudaDeviceSynchronize());
}

}  // namespace vnec
