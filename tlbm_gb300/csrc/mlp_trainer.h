// mlp_trainer.h -- the learned closure's training set and optimiser on one GPU.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "engine.h"

namespace tlbm {

class MlpTrainer {
 public:
  ~MlpTrainer();
  // n samples of 8 normalised features and 1 normalised target, shuffled once with `seed`
  static Status create(int64_t n, const float* feats, const float* targets, uint64_t seed,
                       int device, MlpTrainer** out);
  Status set_params(const float* params);  // FP32 master weights (mlp::kParams); resets Adam
  Status get_params(float* params);
  // mean loss and gradient over samples [first, first+count) in data-set order
  Status loss_grad(int64_t first, int64_t count, float* loss, float* grad);
  // Adam over minibatches of the shuffled order; epoch_loss[e] = mean minibatch loss (optional)
  Status train(int epochs, int64_t batch, float lr, float* epoch_loss);
  Status predict(int64_t n, const float* feats, float* y);
  std::string last_error;

 private:
  MlpTrainer() = default;
  Status init(const float* feats, const float* targets, uint64_t seed);
  Status check(cudaError_t e, const char* what);

  int64_t n_ = 0;
  int device_ = 0;
  int nblocks_ = 1;
  int step_ = 0;
  cudaStream_t stream_ = nullptr;
  float *d_x_ = nullptr, *d_t_ = nullptr;
  int64_t* d_index_ = nullptr;
  float *d_w_ = nullptr, *d_wbf_ = nullptr, *d_m_ = nullptr, *d_v_ = nullptr;
  float *d_grad_ = nullptr, *d_partial_ = nullptr;
};

}  // namespace tlbm
