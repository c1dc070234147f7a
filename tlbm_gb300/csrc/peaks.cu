// peaks.cu -- measured FP64-pipe rate of this GPU, for the benchmark's compute roofline.
//
// Built as its own small library (libtlbm_peaks.so), not part of the engine's C ABI.  GB300
// retires two FP64 fused multiply-adds per SM per clock; the same pipe executes the int64 <->
// double conversions.  Both rates are measured here with independent dependency chains (eight
// per thread, enough to cover the pipe's latency) over a grid of 8 blocks of 256 threads per SM,
// timed with CUDA events after a warm-up launch, best of five.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_dfma(double* out, int iters, double b, double c) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// one int64 -> double conversion per step of each chain (plus an integer xor, on the ALU)
__global__ void __launch_bounds__(256) k_i2d(long long* out, int iters, long long m) {
  long long x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = threadIdx.x * 977 + k * 131 + 1;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < kChains; ++k)
      x[k] = (x[k] ^ __double_as_longlong(__ll2double_rn(x[k]))) & m;
  long long s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class F>
float best_ms(F launch, cudaEvent_t a, cudaEvent_t b) {
  launch();
  if (cudaDeviceSynchronize() != cudaSuccess) return -1.0f;
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(a);
    launch();
    cudaEventRecord(b);
    if (cudaEventSynchronize(b) != cudaSuccess) return -1.0f;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  return best;
}

}  // namespace

// out[0]: DFMA per second, out[1]: int64 -> double conversions per second (whole GPU).
// Returns 0 on success, 1 on a CUDA error.
extern "C" int tlbm_peaks_fp64(int device, double* out) {
  if (!out || cudaSetDevice(device) != cudaSuccess) return 1;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return 1;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  void* buf = nullptr;
  if (cudaMalloc(&buf, static_cast<size_t>(blocks) * threads * 8) != cudaSuccess) return 1;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const double ops = static_cast<double>(blocks) * threads * iters * kChains;
  const float t1 = best_ms([&] {
    k_dfma<<<blocks, threads>>>(static_cast<double*>(buf), iters, 1.0000001, 1e-9);
  }, a, b);
  const float t2 = best_ms([&] {
    k_i2d<<<blocks, threads>>>(static_cast<long long*>(buf), iters, 0x7fffffffffffll);
  }, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  if (t1 <= 0.0f || t2 <= 0.0f) return 1;
  out[0] = ops / (t1 * 1e-3);
  out[1] = ops / (t2 * 1e-3);
  return 0;
}
