// Learned skeleton-rank predictor: a small MLP, 16 -> 64 -> 64 -> 1 (ReLU,
// ReLU, sigmoid), FP32, predicting a box's ID rank as a fraction of its
// active DOFs from geometric features of the box.  Trained on ranks the
// plain factorization produces; the FP32 factorization uses the prediction
// to size each box's randomized sketch (ell = 1.25 k_pred + 12 rows by
// default instead of n + 16), and falls back to the full sketch for any box whose rank test
// does not close inside the shorter sketch.  Training and inference are
// hand-written kernels (rank_model.cu).
#pragma once

#include <cuda_runtime.h>

#include "plan.hpp"

namespace rskel {

constexpr int kRankFeatures = 16;
constexpr int kRankHidden = 64;
// W1 (64 x 16, row major), b1 (64), W2 (64 x 64), b2 (64), w3 (64), b3 (1)
constexpr int kRankWeights = kRankHidden * kRankFeatures + kRankHidden +
                             kRankHidden * kRankHidden + kRankHidden + kRankHidden + 1;

// Writes tasks[i].ell (sketch rows) for every task from its features
// (num_tasks x 16, row major), and the same value to ell_by_slot[tasks[i].slot]:
// ell = ceil(headroom * ceil(y n)) + extra, within [12, n + 16].
cudaError_t rank_infer_ell(const float* weights, const float* features, IdTask* tasks,
                           int num_tasks, int* ell_by_slot, float headroom, int extra,
                           cudaStream_t st);
// out[i] = predicted rank fraction of sample i.
cudaError_t rank_predict(const float* weights, const float* features, int count, float* out,
                         cudaStream_t st);
// Gradient of the mean squared error of the rank fraction over `count`
// samples into grad (kRankWeights floats, overwritten) and the summed
// squared error into *loss_sum (device pointer, overwritten).  Bit-for-bit
// reproducible (no atomics).  scratch: rank_gradient_scratch(count) floats.
size_t rank_gradient_scratch(int count);
cudaError_t rank_gradient(const float* weights, const float* features, const float* targets,
                          int count, float* grad, float* loss_sum, float* scratch,
                          cudaStream_t st);
// One Adam step (step t >= 1) over the weights with moment buffers m, v.
cudaError_t rank_adam(float* weights, const float* grad, float* m, float* v, int t, float lr,
                      cudaStream_t st);

}  // namespace rskel
