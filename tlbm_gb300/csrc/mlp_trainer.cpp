// mlp_trainer.cpp -- on-GPU training of the learned closure (Adam on BF16-rounded weights).
#include "mlp_trainer.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>

#include "mlp.cuh"
#include "mlp_kernels.h"

namespace tlbm {

#define TLBM_TRY(expr)         \
  do {                         \
    Status _s = (expr);        \
    if (!_s.good()) return _s; \
  } while (0)
#define TLBM_CUDA(expr) TLBM_TRY(check((expr), #expr))

Status MlpTrainer::check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return Status::ok();
  return Status::err(TLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

MlpTrainer::~MlpTrainer() {
  if (stream_) cudaStreamSynchronize(stream_);
  cudaFree(d_x_);
  cudaFree(d_t_);
  cudaFree(d_index_);
  cudaFree(d_w_);
  cudaFree(d_wbf_);
  cudaFree(d_m_);
  cudaFree(d_v_);
  cudaFree(d_grad_);
  cudaFree(d_partial_);
  if (stream_) cudaStreamDestroy(stream_);
}

Status MlpTrainer::create(int64_t n, const float* feats, const float* targets, uint64_t seed,
                          int device, MlpTrainer** out) {
  *out = nullptr;
  if (n < 1 || !feats || !targets)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "need n >= 1 samples");
  MlpTrainer* t = new (std::nothrow) MlpTrainer();
  if (!t) return Status::err(TLBM_ERR_NO_MEMORY, "out of host memory");
  t->n_ = n;
  t->device_ = device;
  Status s = t->init(feats, targets, seed);
  if (!s.good()) {
    delete t;
    return s;
  }
  *out = t;
  return Status::ok();
}

Status MlpTrainer::init(const float* feats, const float* targets, uint64_t seed) {
  TLBM_CUDA(cudaSetDevice(device_));
  TLBM_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  const size_t n = static_cast<size_t>(n_);
  TLBM_CUDA(cudaMalloc(&d_x_, n * mlp::kIn * sizeof(float)));
  TLBM_CUDA(cudaMalloc(&d_t_, n * sizeof(float)));
  TLBM_CUDA(cudaMemcpy(d_x_, feats, n * mlp::kIn * sizeof(float), cudaMemcpyHostToDevice));
  TLBM_CUDA(cudaMemcpy(d_t_, targets, n * sizeof(float), cudaMemcpyHostToDevice));
  // one seeded shuffle of the sample order; minibatches are contiguous ranges of it
  std::vector<int64_t> idx(n);
  for (size_t i = 0; i < n; ++i) idx[i] = static_cast<int64_t>(i);
  std::mt19937_64 rng(seed);
  std::shuffle(idx.begin(), idx.end(), rng);
  TLBM_CUDA(cudaMalloc(&d_index_, n * sizeof(int64_t)));
  TLBM_CUDA(cudaMemcpy(d_index_, idx.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice));
  for (float** p : {&d_w_, &d_wbf_, &d_m_, &d_v_})
    TLBM_CUDA(cudaMalloc(p, mlp::kParams * sizeof(float)));
  TLBM_CUDA(cudaMalloc(&d_grad_, (mlp::kParams + 1) * sizeof(float)));
  int sms = 0;
  TLBM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
  nblocks_ = std::max(1, sms);
  TLBM_CUDA(cudaMalloc(&d_partial_, static_cast<size_t>(nblocks_) * (mlp::kParams + 1) *
                                        sizeof(float)));
  // Xavier-uniform initial weights, zero biases
  std::vector<float> w(mlp::kParams, 0.0f);
  std::uniform_real_distribution<float> u(-1.0f, 1.0f);
  const float a1 = std::sqrt(6.0f / (mlp::kIn + mlp::kHid));
  const float a2 = std::sqrt(6.0f / (mlp::kHid + mlp::kHid));
  const float a3 = std::sqrt(6.0f / (mlp::kHid + 1));
  for (int k = 0; k < mlp::kHid * mlp::kIn; ++k) w[mlp::oW1 + k] = a1 * u(rng);
  for (int k = 0; k < mlp::kHid * mlp::kHid; ++k) w[mlp::oW2 + k] = a2 * u(rng);
  for (int k = 0; k < mlp::kHid; ++k) w[mlp::oW3 + k] = a3 * u(rng);
  return set_params(w.data());
}

Status MlpTrainer::set_params(const float* params) {
  TLBM_CUDA(cudaSetDevice(device_));
  TLBM_CUDA(cudaMemcpyAsync(d_w_, params, mlp::kParams * sizeof(float), cudaMemcpyHostToDevice,
                            stream_));
  TLBM_CUDA(cudaMemsetAsync(d_m_, 0, mlp::kParams * sizeof(float), stream_));
  TLBM_CUDA(cudaMemsetAsync(d_v_, 0, mlp::kParams * sizeof(float), stream_));
  TLBM_CUDA(launch_mlp_round(d_w_, d_wbf_, stream_));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  step_ = 0;
  return Status::ok();
}

Status MlpTrainer::get_params(float* params) {
  TLBM_CUDA(cudaSetDevice(device_));
  TLBM_CUDA(cudaMemcpyAsync(params, d_w_, mlp::kParams * sizeof(float), cudaMemcpyDeviceToHost,
                            stream_));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status MlpTrainer::loss_grad(int64_t first, int64_t count, float* loss, float* grad) {
  TLBM_CUDA(cudaSetDevice(device_));
  if (first < 0 || count < 1 || first + count > n_)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "sample range outside the data set");
  TLBM_CUDA(launch_mlp_grad(d_wbf_, d_x_, d_t_, nullptr, first, count, d_partial_, nblocks_,
                            d_grad_, stream_));
  std::vector<float> g(mlp::kParams + 1);
  TLBM_CUDA(cudaMemcpyAsync(g.data(), d_grad_, g.size() * sizeof(float), cudaMemcpyDeviceToHost,
                            stream_));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  if (grad) std::memcpy(grad, g.data(), mlp::kParams * sizeof(float));
  if (loss) *loss = g[mlp::kParams];
  return Status::ok();
}

Status MlpTrainer::train(int epochs, int64_t batch, float lr, float* epoch_loss) {
  TLBM_CUDA(cudaSetDevice(device_));
  if (epochs < 1 || batch < 1 || lr <= 0.0f)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "epochs, batch and lr must be positive");
  batch = std::min(batch, n_);
  for (int e = 0; e < epochs; ++e) {
    double acc = 0.0;
    int nb = 0;
    for (int64_t first = 0; first + batch <= n_; first += batch) {
      TLBM_CUDA(launch_mlp_grad(d_wbf_, d_x_, d_t_, d_index_, first, batch, d_partial_, nblocks_,
                                d_grad_, stream_));
      ++step_;
      TLBM_CUDA(launch_mlp_adam(d_w_, d_wbf_, d_m_, d_v_, d_grad_, lr, step_, stream_));
      if (epoch_loss) {
        float l = 0.0f;
        TLBM_CUDA(cudaMemcpyAsync(&l, d_grad_ + mlp::kParams, sizeof(float),
                                  cudaMemcpyDeviceToHost, stream_));
        TLBM_CUDA(cudaStreamSynchronize(stream_));
        acc += l;
      }
      ++nb;
    }
    if (epoch_loss) epoch_loss[e] = nb ? static_cast<float>(acc / nb) : 0.0f;
  }
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status MlpTrainer::predict(int64_t n, const float* feats, float* y) {
  TLBM_CUDA(cudaSetDevice(device_));
  if (n < 1) return Status::ok();
  float *dx = nullptr, *dy = nullptr;
  TLBM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dx), n * mlp::kIn * sizeof(float),
                            stream_));
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&dy), n * sizeof(float), stream_);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dx, feats, n * mlp::kIn * sizeof(float), cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess) e = launch_mlp_predict(d_wbf_, dx, n, dy, stream_);
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, dy, n * sizeof(float), cudaMemcpyDeviceToHost, stream_);
  cudaFreeAsync(dx, stream_);
  if (dy) cudaFreeAsync(dy, stream_);
  TLBM_CUDA(e);
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

}  // namespace tlbm
