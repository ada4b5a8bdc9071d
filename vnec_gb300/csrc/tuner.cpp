// Kernel selection: the configuration space, the exhaustive autotuner, the
// reference's rule-based choice and the learned choice (features -> MLP ->
// cheapest predicted configuration, falling back to the exhaustive search for
// matrices outside the model's training range).

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "host.h"
#include "tuner.h"

namespace vnec {
namespace {

// Merge-path configurations: (items per thread, pipeline stages) with 256
// threads; ipt 4 runs the unpipelined kernel.  Warp-task configurations:
// long-row chunk x dense-block fill threshold (1: every row with a block goes
// dense, 1001: every row sliced).
const TuneConfig kConfigs[kNumConfigs] = {
    {SpB_VNEC_KERNEL_L, 4, 0},         {SpB_VNEC_KERNEL_L, 7, 0},         {SpB_VNEC_KERNEL_L, 12, 0},
    {SpB_VNEC_KERNEL_HYBRID, 256, 1},  {SpB_VNEC_KERNEL_HYBRID, 256, 500}, {SpB_VNEC_KERNEL_HYBRID, 256, 750},
    {SpB_VNEC_KERNEL_HYBRID, 256, 1001}, {SpB_VNEC_KERNEL_HYBRID, 1024, 1}, {SpB_VNEC_KERNEL_HYBRID, 1024, 500},
    {SpB_VNEC_KERNEL_HYBRID, 1024, 750}, {SpB_VNEC_KERNEL_HYBRID, 1024, 1001}, {SpB_VNEC_KERNEL_HYBRID, 4096, 1},
    {SpB_VNEC_KERNEL_HYBRID, 4096, 500}, {SpB_VNEC_KERNEL_HYBRID, 4096, 750}, {SpB_VNEC_KERNEL_HYBRID, 4096, 1001},
};

bool cols_sorted(const CsrView& v) {
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t r = 0; r < v.n_rows; ++r)
    for (int64_t q = v.row_begin(r) + 1; q < v.row_begin(r + 1); ++q)
      if (v.col_at(q) <= v.col_at(q - 1)) bad = 1;
  return !bad;
}

// `precision`: a precision form of the sliced kernel restricts the choice to
// the pure sliced configurations (the only plans that carry the forms).
bool available(int i, const CsrView& v, bool sorted, int precision = 0) {
  const TuneConfig& c = kConfigs[i];
  if (precision != 0) return c.kernel != SpB_VNEC_KERNEL_L && c.permille > 1000;
  if (c.kernel == SpB_VNEC_KERNEL_L) return c.chunk != 12 || v.type == SpB_FP64;
  // Rows in dense blocks need sorted columns; the pure-sliced configuration does not.
  return sorted || c.permille > 1000;
}

std::unique_ptr<Plan> build_config(int i, const CsrView& v, const SpB_VNEC_options_ext* base) {
  const SpB_VNEC_options_ext o = config_options(i, base);
  const TuneConfig& c = kConfigs[i];
  if (c.kernel == SpB_VNEC_KERNEL_L) return build_merge_path(v, &o);
  if (c.permille > 1000) return build_sliced(v, &o);
  return build_hybrid(v, &o);
}

// Times one plan: warm-up calls, then `reps` calls each after an L2 flush,
// median of the CUDA-event times (ms).
float time_plan(Plan* p, const void* dx, void* dy, void* flush, size_t flush_bytes, int reps, cudaStream_t s,
                cudaEvent_t e0, cudaEvent_t e1) {
  for (int w = 0; w < 2; ++w)
    if (!p->run(dx, dy, s)) return FLT_MAX;
  std::vector<float> t;
  for (int r = 0; r < reps; ++r) {
    if (flush && !VNEC_CUDA(cudaMemsetAsync(flush, r & 0xff, flush_bytes, s))) return FLT_MAX;
    if (!VNEC_CUDA(cudaEventRecord(e0, s)) || !p->run(dx, dy, s) || !VNEC_CUDA(cudaEventRecord(e1, s)) ||
        !VNEC_CUDA(cudaEventSynchronize(e1)))
      return FLT_MAX;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    t.push_back(ms);
  }
  std::sort(t.begin(), t.end());
  return t[t.size() / 2];
}

std::mutex g_model_mu;
MlpModel* builtin_model() {
  static MlpModel* m = nullptr;
  if (!m && builtin_mlp_params()) {
    m = mlp_create(0);
    if (m && !mlp_set_params(m, builtin_mlp_params())) {
      mlp_destroy(m);
      m = nullptr;
    }
  }
  return m;
}

}  // namespace

const TuneConfig& tune_config(int i) { return kConfigs[i]; }

SpB_VNEC_options_ext config_options(int i, const SpB_VNEC_options_ext* base) {
  SpB_VNEC_options_ext o;
  std::memset(&o, 0, sizeof(o));
  if (base) o = *base;
  const TuneConfig& c = kConfigs[i];
  o.kernel = c.kernel;
  if (c.kernel == SpB_VNEC_KERNEL_L) {
    o.threads_per_block = 256;
    o.items_per_thread = c.chunk;
    o.pipeline_stages = c.chunk == 4 ? 1 : 2;
  } else {
    o.threads_per_block = 0;
    o.items_per_thread = -1;  // sliced parts time their unroll on the matrix
    o.long_row_len = c.chunk;
    o.dense_fill_permille = c.permille;
  }
  return o;
}

bool config_available(int i, bool sorted_cols) {
  return kConfigs[i].kernel == SpB_VNEC_KERNEL_L || sorted_cols || kConfigs[i].permille > 1000;
}

// Exhaustive search: every available configuration built and timed; ms[i] =
// FLT_MAX for configurations that cannot be built.  Returns the fastest index.
// Times every available configuration (only those with only[i] != 0 when
// `only` is given); ms[i] = FLT_MAX for the rest.  Returns the fastest index.
int autotune_search(const CsrView& v, const SpB_VNEC_options_ext* base, int reps, float* ms,
                    const uint8_t* only = nullptr) {
  const bool sorted = cols_sorted(v);
  const size_t vb = v.value_bytes();
  DeviceBuffer dx, dy, flush;
  const size_t flush_bytes = (size_t)256 << 20;
  TimingStream ts;
  int best = -1;
  if (!dx.alloc(vb * (size_t)std::max<int64_t>(v.n_cols, 1)) || !dy.alloc(vb * (size_t)std::max<int64_t>(v.n_rows, 1)) ||
      !flush.alloc(flush_bytes) || !VNEC_CUDA(cudaMemset(dx.ptr, 0x3f, dx.bytes))) {
    for (int i = 0; i < kNumConfigs; ++i) ms[i] = FLT_MAX;
    return -1;
  }
  if (!ts.create()) {
    set_error("autotune: cannot create a stream or events");
    for (int i = 0; i < kNumConfigs; ++i) ms[i] = FLT_MAX;
    return -1;
  }
  for (int i = 0; i < kNumConfigs; ++i) {
    ms[i] = FLT_MAX;
    if (only && !only[i]) continue;
    if (!available(i, v, sorted, base ? base->precision : 0)) continue;
    std::unique_ptr<Plan> p = build_config(i, v, base);
    if (!p) continue;
    ms[i] = time_plan(p.get(), dx.ptr, dy.ptr, flush.ptr, flush_bytes, reps, ts.s, ts.e0, ts.e1);
    if (ms[i] < FLT_MAX && (best < 0 || ms[i] < ms[best])) best = i;
  }
  if (best < 0) set_error("autotune: no configuration could be built");
  return best;
}

// The reference harness's choice (test_spmv_vnec.cpp:197-245): VNEC-L for
// 3,000,000 rows or more, otherwise IRD_VNEC's choice between VNEC-D and
// VNEC-S — here the merge path, the pure dense-block configuration and the
// pure sliced configuration with their default chunk.
int rule_choice(const CsrView& v) {
  // VNEC-L: the merge-path configuration a default L plan takes at this size.
  if (v.n_rows >= 3000000) return v.nnz >= ((int64_t)1 << 26) ? 0 : 1;
  const IrdParams prm = ird_params(v.type);
  const float ird = ird_ratio(v, prm);
  const bool dense = ird >= prm.threshold && cols_sorted(v);
  return dense ? 7 : 10;
}

// Learned choice: the configuration with the lowest predicted cost among the
// available ones; *ood is set when a feature lies outside the training range
// (widened by 0.05 on each side).  Returns -1 when no model is built in.
int learned_choice(const CsrView& v, bool* ood, float* pred, int precision = 0) {
  float f[kNumFeatures];
  *ood = false;
  if (!builtin_mlp_params()) return -1;
  if (!matrix_features(v, f)) return -1;
  const float* range = builtin_feature_range();
  for (int i = 0; i < kNumFeatures; ++i)
    if (f[i] < range[2 * i] - 0.05f || f[i] > range[2 * i + 1] + 0.05f) *ood = true;
  float out[kNumConfigs];
  {
    std::lock_guard<std::mutex> g(g_model_mu);
    MlpModel* m = builtin_model();
    if (!m || !mlp_predict(m, f, 1, out)) return -1;
  }
  if (pred) std::copy(out, out + kNumConfigs, pred);
  const bool sorted = cols_sorted(v);
  int best = -1;
  for (int i = 0; i < kNumConfigs; ++i)
    if (available(i, v, sorted, precision) && (best < 0 || out[i] < out[best])) best = i;
  return best;
}

// Plans of kernel LEARNED / SEARCH / RULE.
std::unique_ptr<Plan> build_tuned(const CsrView& v, const SpB_VNEC_options_ext* opts) {
  if (!validate_csr(v, false)) return nullptr;
  const int kernel = opts ? opts->kernel : SpB_VNEC_KERNEL_LEARNED;
  int choice = -1, how = 0;
  const int precision = opts ? opts->precision : 0;
  if (kernel == SpB_VNEC_KERNEL_RULE) {
    if (precision != 0) {
      set_error("the reference rule chooses among FP64 kernels: ask LEARNED or SEARCH for a precision form");
      return nullptr;
    }
    choice = rule_choice(v);
    how = SpB_VNEC_CHOSEN_RULE;
  } else if (kernel == SpB_VNEC_KERNEL_LEARNED) {
    bool ood = false;
    choice = learned_choice(v, &ood, nullptr, precision);
    how = SpB_VNEC_CHOSEN_LEARNED;
    if (choice < 0 || ood) choice = -1;
  }
  if (choice < 0) {
    float ms[kNumConfigs];
    how = kernel == SpB_VNEC_KERNEL_SEARCH ? SpB_VNEC_CHOSEN_SEARCH : SpB_VNEC_CHOSEN_FALLBACK;
    choice = autotune_search(v, opts, 3, ms);
    if (choice < 0) return nullptr;
  }
  std::unique_ptr<Plan> p = build_config(choice, v, opts);
  if (p) {
    p->tune_config = choice;
    p->tune_how = how;
  }
  return p;
}

}  // namespace vnec

// ---------------------------------------------------------------------------
// C ABI of the tuner.
// ---------------------------------------------------------------------------

using namespace vnec;

extern "C" {

int SpB_VNEC_tune_configs_ext(int* kernel, int* chunk, int* permille, int cap) {
  for (int i = 0; i < kNumConfigs && i < cap; ++i) {
    if (kernel) kernel[i] = kConfigs[i].kernel;
    if (chunk) chunk[i] = kConfigs[i].chunk;
    if (permille) permille[i] = kConfigs[i].permille;
  }
  return kNumConfigs;
}

SpB_Info SpB_VNEC_features_ext(int64_t n_rows, int64_t n_cols, const int64_t* row_ptr, const int32_t* col,
                               float* features) {
  clear_error();
  CsrView v;
  // Values are not read: the column array stands in for the value pointer.
  if (!features || !view_from_arrays(SpB_FP64, n_rows, n_cols, row_ptr, col, col, &v)) {
    if (!features) set_error("SpB_VNEC_features_ext: NULL output");
    return SpB_FAILURE;
  }
  v.val = nullptr;
  if (!validate_csr(v, false)) return SpB_FAILURE;
  return matrix_features(v, features) ? SpB_SUCCESS : SpB_FAILURE;
}

int SpB_VNEC_autotune_ext(const SpB_VNEC_options_ext* base, SpB_Type type, int64_t n_rows, int64_t n_cols,
                          const int64_t* row_ptr, const int32_t* col, const void* val, int reps, float* ms) {
  clear_error();
  CsrView v;
  if (!ms || reps < 1 || !view_from_arrays(type, n_rows, n_cols, row_ptr, col, val, &v)) {
    if (!ms || reps < 1) set_error("SpB_VNEC_autotune_ext: invalid arguments");
    return -1;
  }
  if (!validate_csr(v, false)) return -1;
  return autotune_search(v, base, reps, ms);
}

int SpB_VNEC_time_configs_ext(const SpB_VNEC_options_ext* base, SpB_Type type, int64_t n_rows, int64_t n_cols,
                              const int64_t* row_ptr, const int32_t* col, const void* val, int reps,
                              const int* configs, int n_configs, float* ms) {
  clear_error();
  CsrView v;
  if (!ms || !configs || n_configs < 1 || reps < 1 ||
      !view_from_arrays(type, n_rows, n_cols, row_ptr, col, val, &v)) {
    if (!ms || !configs || n_configs < 1 || reps < 1) set_error("SpB_VNEC_time_configs_ext: invalid arguments");
    return -1;
  }
  if (!validate_csr(v, false)) return -1;
  uint8_t only[kNumConfigs] = {0};
  for (int i = 0; i < n_configs; ++i) {
    if (configs[i] < 0 || configs[i] >= kNumConfigs) {
      set_error("SpB_VNEC_time_configs_ext: configuration index out of range");
      return -1;
    }
    only[configs[i]] = 1;
  }
  float all[kNumConfigs];
  autotune_search(v, base, reps, all, only);
  for (int i = 0; i < n_configs; ++i) ms[i] = all[configs[i]];
  return 0;
}

int SpB_VNEC_rule_choice_ext(SpB_Type type, int64_t n_rows, int64_t n_cols, const int64_t* row_ptr,
                             const int32_t* col, const void* val) {
  clear_error();
  CsrView v;
  if (!view_from_arrays(type, n_rows, n_cols, row_ptr, col, val, &v) || !validate_csr(v, false)) return -1;
  return rule_choice(v);
}

int SpB_VNEC_learned_choice_ext(SpB_Type type, int64_t n_rows, int64_t n_cols, const int64_t* row_ptr,
                                const int32_t* col, const void* val, float* predicted, int* out_of_range) {
  clear_error();
  CsrView v;
  if (!view_from_arrays(type, n_rows, n_cols, row_ptr, col, val, &v) || !validate_csr(v, false)) return -1;
  bool ood = false;
  const int c = learned_choice(v, &ood, predicted);
  if (out_of_range) *out_of_range = ood ? 1 : 0;
  if (c < 0 && !builtin_mlp_params()) set_error("no learned model is built into this library");
  return c;
}

SpB_Info SpB_VNEC_plan_choice_ext(const void* plan, int* config, int* how) {
  clear_error();
  Plan* p = find_plan(plan);
  if (!p) {
    set_error("unknown plan");
    return SpB_FAILURE;
  }
  if (config) *config = p->tune_config;
  if (how) *how = p->tune_how;
  return SpB_SUCCESS;
}

void* SpB_VNEC_mlp_create_ext(uint64_t seed) {
  clear_error();
  return mlp_create(seed);
}

void SpB_VNEC_mlp_free_ext(void* model) { mlp_destroy(static_cast<MlpModel*>(model)); }

int SpB_VNEC_mlp_num_params_ext(void) { return kMlpParams; }

SpB_Info SpB_VNEC_mlp_params_ext(void* model, float* params, int set) {
  clear_error();
  if (!model || !params) {
    set_error("SpB_VNEC_mlp_params_ext: NULL argument");
    return SpB_FAILURE;
  }
  auto* m = static_cast<MlpModel*>(model);
  return (set ? mlp_set_params(m, params) : mlp_get_params(m, params)) ? SpB_SUCCESS : SpB_FAILURE;
}

SpB_Info SpB_VNEC_mlp_predict_ext(void* model, const float* X, int n, float* out) {
  clear_error();
  if (!model || (n > 0 && (!X || !out)) || n < 0) {
    set_error("SpB_VNEC_mlp_predict_ext: invalid arguments");
    return SpB_FAILURE;
  }
  return mlp_predict(static_cast<MlpModel*>(model), X, n, out) ? SpB_SUCCESS : SpB_FAILURE;
}

SpB_Info SpB_VNEC_mlp_grad_ext(void* model, const float* X, const float* T, const float* M, int n, float* loss,
                               float* grad) {
  clear_error();
  if (!model || n <= 0 || !X || !T || !M) {
    set_error("SpB_VNEC_mlp_grad_ext: invalid arguments");
    return SpB_FAILURE;
  }
  return mlp_loss_grad(static_cast<MlpModel*>(model), X, T, M, n, loss, grad) ? SpB_SUCCESS : SpB_FAILURE;
}

SpB_Info SpB_VNEC_mlp_train_ext(void* model, const float* X, const float* T, const float* M, int n, int epochs,
                                int batch, float lr, float weight_decay, uint64_t seed, float* loss_curve) {
  clear_error();
  if (!model || n <= 0 || !X || !T || !M) {
    set_error("SpB_VNEC_mlp_train_ext: invalid arguments");
    return SpB_FAILURE;
  }
  MlpTrainParams tp;
  tp.epochs = epochs;
  tp.batch = batch;
  tp.lr = lr;
  tp.weight_decay = weight_decay;
  tp.seed = seed;
  return mlp_train(static_cast<MlpModel*>(model), X, T, M, n, tp, loss_curve) ? SpB_SUCCESS : SpB_FAILURE;
}

int SpB_VNEC_builtin_model_ext(float* params, float* feature_range) {
  const float* p = builtin_mlp_params();
  if (!p) return 0;
  if (params) std::copy(p, p + kMlpParams, params);
  if (feature_range) std::copy(builtin_feature_range(), builtin_feature_range() + 2 * kNumFeatures, feature_range);
  return 1;
}

}  // extern "C"
