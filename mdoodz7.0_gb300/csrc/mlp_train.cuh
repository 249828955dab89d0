// mlp_train.cuh -- device state and launch interface of the warm-start perceptron training.
#pragma once
#include <cuda_runtime.h>

#include "mlp.cuh"

namespace mdz {

// Device buffers of one training run (all device pointers).
struct MlpTrainState {
  float *W1, *W2, *W3, *b1, *b2, *b3;          // FP32 masters: [64][16], [64][64], [2][64], 64, 64, 16
  float *mW1, *mW2, *mW3, *mb1, *mb2, *mb3;    // Adam first moments
  float *vW1, *vW2, *vW3, *vb1, *vb2, *vb3;    // Adam second moments
  float *gW1, *gW2, *gW3, *gb1, *gb2, *gb3;    // gradient accumulators
  uint4 *tW1, *tW2, *tW3, *tW2t, *tW3t;        // BF16 K-major tiles (umma.cuh layout)
  float *loss;                                 // [2]: sum of squared errors (z, plastic)
  int *fault;
  float x_shift[kMlpIn], x_scale[kMlpIn];
  float z_shift, z_scale;
};

// One CTA's gradient sums, in this order: gW1 [64][16], gW2 [64][64], gW3 [2][64], gb1,
// gb2, gb3 [16].  Each CTA of a step writes its own block; k_mlp_reduce adds the blocks in
// CTA order into the gradient accumulators, so a step's gradient does not depend on the
// order in which its CTAs finish.
constexpr int kGradW1 = 0, kGradW2 = kGradW1 + kMlpHid * kMlpIn, kGradW3 = kGradW2 + kMlpHid * kMlpHid,
              kGradB1 = kGradW3 + 2 * kMlpHid, kGradB2 = kGradB1 + kMlpHid, kGradB3 = kGradB2 + kMlpHid,
              kGradCount = kGradB3 + 16;

struct MlpTrainArgs {
  MlpTrainState W;
  float *part;      // [CTAs of the step][kGradCount], zeroed once (entries no CTA writes stay 0)
  const float *X;   // [n][kMlpIn] raw features
  const float *Y;   // [n][2] raw targets
  const int *perm;  // sample order (may be null)
  long long n, offset;
  int n_feat;
  float inv_batch, w_pl;
};

struct MlpAdam {
  float lr, beta1, beta2, eps, bc1, bc2;  // bc = 1 / (1 - beta^t)
};

__global__ void k_mlp_step(const __grid_constant__ MlpTrainArgs a);
__global__ void k_mlp_reduce(const __grid_constant__ MlpTrainArgs a, int ctas);
__global__ void k_mlp_adam(const __grid_constant__ MlpTrainArgs a, const __grid_constant__ MlpAdam o);
__global__ void k_mlp_pack(const __grid_constant__ MlpTrainArgs a);
__global__ void k_mlp_predict(const __grid_constant__ MlpTrainArgs a, float *Yp);
size_t mlp_step_smem();
size_t mlp_predict_smem();

}  // namespace mdz
