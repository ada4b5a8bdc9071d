// Learned kernel selection: matrix features, the configuration space the
// autotuner searches, and the FP32 MLP (16 -> 64 -> 64 -> kNumConfigs) that
// predicts each configuration's cost from the features.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "vnec_gb300.h"

namespace vnec {

struct CsrView;

constexpr int kNumFeatures = 16;

// ---------------------------------------------------------------------------
// Configuration space: the kernel variant, its chunk size (merge-path items per
// thread, or the long-row chunk of the warp-task formats) and the row-level
// dense/sparse split threshold (dense-block fill, permille; 0 = every row in
// dense blocks, 1001 = every row sliced).
// ---------------------------------------------------------------------------
struct TuneConfig {
  int kernel;    // SpB_VNEC_KERNEL_L or SpB_VNEC_KERNEL_HYBRID
  int chunk;     // L: items per thread; HYBRID: long-row chunk length
  int permille;  // HYBRID: dense-block fill threshold
};
constexpr int kNumConfigs = 15;
const TuneConfig& tune_config(int i);
// Options of configuration i on top of `base` (precision etc. kept).
SpB_VNEC_options_ext config_options(int i, const SpB_VNEC_options_ext* base);
// Whether configuration i can be built for the matrix (dense blocks need sorted columns).
bool config_available(int i, bool sorted_cols);

// ---------------------------------------------------------------------------
// Features (features.cu): computed on the GPU from device CSR arrays.
//   0 log2(n_rows+1)/24        1 log2(n_cols+1)/24      2 log2(nnz+1)/32
//   3 log2(mean row len+1)/12  4 min(cv of row len, 8)/8 5 log2(max row len+1)/16
//   6..11 fraction of rows with length 0, [1,4), [4,16), [16,64), [64,1024), >= 1024
//   12 mean column span of non-empty rows / n_cols
//   13 nnz / (4 * aligned 4-column blocks)   (dense-block fill of the matrix)
//   14 fraction of non-empty rows with aligned-block fill >= 1/2
//   15 share of nonzeros in columns used at least 8x the mean column count
// ---------------------------------------------------------------------------
bool matrix_features_device(int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t* d_row_ptr,
                            const int32_t* d_col, float* out, cudaStream_t s);
bool matrix_features(const CsrView& v, float* out);

// ---------------------------------------------------------------------------
// MLP (mlp.cu).  Parameters in one FP32 array: W1[64x16] b1[64] W2[64x64]
// b2[64] W3[C x 64] b3[C], row-major (out x in).
// ---------------------------------------------------------------------------
constexpr int kHidden = 64;
constexpr int kMlpParams = kHidden * kNumFeatures + kHidden + kHidden * kHidden + kHidden +
                           kNumConfigs * kHidden + kNumConfigs;

struct MlpModel;
MlpModel* mlp_create(uint64_t seed);
void mlp_destroy(MlpModel* m);
bool mlp_get_params(const MlpModel* m, float* out);
bool mlp_set_params(MlpModel* m, const float* in);
// Forward pass for n host feature rows -> n x kNumConfigs host outputs.
bool mlp_predict(MlpModel* m, const float* X, int n, float* out);
// Loss (masked mean squared error) and gradient for one batch (host arrays).
bool mlp_loss_grad(MlpModel* m, const float* X, const float* T, const float* M, int n, float* loss, float* grad);
// Adam training over n samples; loss_curve (optional) gets one training loss per epoch.
struct MlpTrainParams {
  int epochs = 300;
  int batch = 64;
  float lr = 2e-3f;
  float weight_decay = 1e-4f;
  uint64_t seed = 1;
};
bool mlp_train(MlpModel* m, const float* X, const float* T, const float* M, int n, const MlpTrainParams& tp,
               float* loss_curve);

// The model shipped with the library (tuner_weights.inc); null if none.
const float* builtin_mlp_params();
// Feature range the built-in model was trained on (min, max per feature).
const float* builtin_feature_range();

}  // namespace vnec
