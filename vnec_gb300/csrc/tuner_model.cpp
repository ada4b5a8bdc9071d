// The kernel selection model built into the library (tuner_weights.inc is
// written by vnec_gb300/tuner/train.py after training on GPU timings).

#include "tuner.h"

namespace vnec {
namespace {
#include "tuner_weights.inc"
}  // namespace

const float* builtin_mlp_params() { return kHaveModel ? kModelParams : nullptr; }
const float* builtin_feature_range() { return kFeatureRange; }

}  // namespace vnec
