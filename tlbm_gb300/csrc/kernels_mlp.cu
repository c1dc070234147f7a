// kernels_mlp.cu -- training and evaluation kernels of the learned closure, and the box
// filter that turns a fine-grid run into training data.
//
// Training is deterministic: each block accumulates the gradient of its samples into
// registers (one thread per group of parameters, samples staged in shared memory), writes one
// partial per block, and a second kernel folds the partials in a fixed order.  Forward and
// backward use the network of mlp.cuh (BF16 weights, BF16 act outputs, FP32 accumulation), so
// the gradient is the gradient of the network the collide kernel runs.
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.cuh"
#include "mlp_kernels.h"

namespace tlbm {
namespace {

using namespace mlp;

constexpr int kTile = 128;  // samples per tile = threads per block

struct Smem {
  float w[kParams];
  float x[kTile][kIn];
  float h1[kTile][kHid];
  float dz1[kTile][kHid];
  float h2[kTile][kHid];
  float dz2[kTile][kHid];
  float dy[kTile];
  float loss[kTile];
};

// forward + backward of one sample into the tile buffers; returns 1/2 (y - t)^2
__device__ float sample_fb(Smem& s, int r, const float* __restrict__ xin, float t) {
  const float* w = s.w;
  float x[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) {
    x[k] = bf16r(xin[k]);
    s.x[r][k] = x[k];
  }
  float h1[kHid];
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    float z = w[oB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; ++k) z = fmaf(w[oW1 + j * kIn + k], x[k], z);
    h1[j] = act(z);
    s.h1[r][j] = h1[j];
  }
  float h2[kHid];
  float y = w[oB3];
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    float z = w[oB2 + j];
#pragma unroll
    for (int k = 0; k < kHid; ++k) z = fmaf(w[oW2 + j * kHid + k], h1[k], z);
    h2[j] = act(z);
    s.h2[r][j] = h2[j];
    y = fmaf(w[oW3 + j], h2[j], y);
  }
  const float dy = y - t;
  s.dy[r] = dy;
  float dz2[kHid];
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    dz2[j] = dy * w[oW3 + j] * (1.0f - h2[j] * h2[j]);
    s.dz2[r][j] = dz2[j];
  }
#pragma unroll
  for (int k = 0; k < kHid; ++k) {
    float dh = 0.0f;
#pragma unroll
    for (int j = 0; j < kHid; ++j) dh = fmaf(w[oW2 + j * kHid + k], dz2[j], dh);
    s.dz1[r][k] = dh * (1.0f - h1[k] * h1[k]);
  }
  return 0.5f * dy * dy;
}

// gradient of parameter p summed over the `rows` samples of the tile
__device__ float tile_grad(const Smem& s, int p, int rows) {
  float g = 0.0f;
  if (p < oB1) {
    const int j = (p - oW1) / kIn, k = (p - oW1) % kIn;
    for (int r = 0; r < rows; ++r) g = fmaf(s.dz1[r][j], s.x[r][k], g);
  } else if (p < oW2) {
    const int j = p - oB1;
    for (int r = 0; r < rows; ++r) g += s.dz1[r][j];
  } else if (p < oB2) {
    const int j = (p - oW2) / kHid, k = (p - oW2) % kHid;
    for (int r = 0; r < rows; ++r) g = fmaf(s.dz2[r][j], s.h1[r][k], g);
  } else if (p < oW3) {
    const int j = p - oB2;
    for (int r = 0; r < rows; ++r) g += s.dz2[r][j];
  } else if (p < oB3) {
    const int j = p - oW3;
    for (int r = 0; r < rows; ++r) g = fmaf(s.dy[r], s.h2[r][j], g);
  } else {
    for (int r = 0; r < rows; ++r) g += s.dy[r];
  }
  return g;
}

constexpr int kPerThread = (kParams + kTile - 1) / kTile;  // 11

__global__ void __launch_bounds__(kTile) k_mlp_grad_partial(const float* __restrict__ wbf,
                                                            const float* __restrict__ feats,
                                                            const float* __restrict__ targets,
                                                            const int64_t* __restrict__ index,
                                                            int64_t first, int64_t count,
                                                            float* __restrict__ partial) {
  extern __shared__ float4 smem_raw[];
  Smem& s = *reinterpret_cast<Smem*>(smem_raw);
  for (int k = threadIdx.x; k < kParams; k += kTile) s.w[k] = wbf[k];
  float acc[kPerThread];
#pragma unroll
  for (int q = 0; q < kPerThread; ++q) acc[q] = 0.0f;
  float loss = 0.0f;
  __syncthreads();
  const int64_t ntiles = (count + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * kTile;
    const int rows = static_cast<int>(count - base < kTile ? count - base : kTile);
    if (threadIdx.x < rows) {
      const int64_t si = index ? index[first + base + threadIdx.x] : first + base + threadIdx.x;
      loss += sample_fb(s, threadIdx.x, feats + si * kIn, targets[si]);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kPerThread; ++q) {
      const int p = threadIdx.x + q * kTile;
      if (p < kParams) acc[q] += tile_grad(s, p, rows);
    }
    __syncthreads();
  }
  float* out = partial + static_cast<size_t>(blockIdx.x) * (kParams + 1);
#pragma unroll
  for (int q = 0; q < kPerThread; ++q) {
    const int p = threadIdx.x + q * kTile;
    if (p < kParams) out[p] = acc[q];
  }
  // block loss in a fixed order
  s.loss[threadIdx.x] = loss;
  __syncthreads();
  if (threadIdx.x == 0) {
    float l = 0.0f;
    for (int r = 0; r < kTile; ++r) l += s.loss[r];
    out[kParams] = l;
  }
}

// grad[p] = sum over blocks (fixed order) / count; grad[kParams] = mean loss
__global__ void k_mlp_grad_reduce(const float* __restrict__ partial, int nblocks, int64_t count,
                                  float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > kParams) return;
  float g = 0.0f;
  for (int b = 0; b < nblocks; ++b) g += partial[static_cast<size_t>(b) * (kParams + 1) + p];
  grad[p] = g / static_cast<float>(count);
}

// Adam on the FP32 master weights; the BF16-rounded copy is what the kernels use.  Biases are
// kept in FP32 (only weights are rounded).
__device__ __forceinline__ bool is_bias(int p) {
  return (p >= oB1 && p < oW2) || (p >= oB2 && p < oW3) || p == oB3;
}

__global__ void k_mlp_adam(float* __restrict__ w, float* __restrict__ wbf, float* __restrict__ m,
                           float* __restrict__ v, const float* __restrict__ grad, float lr,
                           float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float g = grad[p];
  const float mm = b1 * m[p] + (1.0f - b1) * g;
  const float vv = b2 * v[p] + (1.0f - b2) * g * g;
  m[p] = mm;
  v[p] = vv;
  const float nw = w[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  w[p] = nw;
  wbf[p] = is_bias(p) ? nw : bf16r(nw);
}

__global__ void k_mlp_round(const float* __restrict__ w, float* __restrict__ wbf) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kParams) wbf[p] = is_bias(p) ? w[p] : bf16r(w[p]);
}

// Inference exactly as the collide kernel runs it: the tensor-core forward pass of mlp.cuh,
// 32 samples per warp.
__global__ void __launch_bounds__(kTile) k_mlp_predict(const float* __restrict__ wbf,
                                                       const float* __restrict__ feats, int64_t n,
                                                       float* __restrict__ y) {
  __shared__ MmaWeights sw;
  __shared__ WarpScratch ws[kTile / 32];
  stage_mma_weights(wbf, sw, threadIdx.x, kTile);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * static_cast<int64_t>(kTile) + warp * 32; base < n;
       base += static_cast<int64_t>(gridDim.x) * kTile) {
    const int64_t i = base + lane;
    float x[kIn];
#pragma unroll
    for (int k = 0; k < kIn; ++k) x[k] = i < n ? feats[i * kIn + k] : 0.0f;
    const float v = forward_warp(sw, ws[warp], x, lane);
    if (i < n) y[i] = v;
  }
}

// Box filter by `f` in each direction of the fine macroscopic fields (float or double):
// out[10][coarse] = rho, ux, uy, uz, ux ux, uy uy, uz uz, ux uy, ux uz, uy uz (box means).
template <class T>
__global__ void k_box_filter(const T* __restrict__ ux, const T* __restrict__ uy,
                             const T* __restrict__ uz, const T* __restrict__ rho, int nx, int ny,
                             int nz, int f, T* __restrict__ out) {
  const int cx = nx / f, cy = ny / f, cz = nz / f;
  const int64_t nc = static_cast<int64_t>(cx) * cy * cz;
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int z = static_cast<int>(c / (static_cast<int64_t>(cx) * cy));
    const int r = static_cast<int>(c - static_cast<int64_t>(z) * cx * cy);
    const int y = r / cx, x = r - (r / cx) * cx;
    double s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int dz = 0; dz < f; ++dz)
      for (int dy = 0; dy < f; ++dy)
        for (int dx = 0; dx < f; ++dx) {
          const int64_t g = (static_cast<int64_t>(z * f + dz) * ny + (y * f + dy)) * nx +
                            (x * f + dx);
          const double a = ux[g], b = uy[g], cc = uz[g];
          s[0] += rho[g];
          s[1] += a;
          s[2] += b;
          s[3] += cc;
          s[4] += a * a;
          s[5] += b * b;
          s[6] += cc * cc;
          s[7] += a * b;
          s[8] += a * cc;
          s[9] += b * cc;
        }
    const double inv = 1.0 / (static_cast<double>(f) * f * f);
#pragma unroll
    for (int k = 0; k < 10; ++k) out[k * nc + c] = static_cast<T>(s[k] * inv);
  }
}

}  // namespace

size_t mlp_grad_smem() { return sizeof(Smem); }

cudaError_t launch_mlp_grad(const float* wbf, const float* feats, const float* targets,
                            const int64_t* index, int64_t first, int64_t count, float* partial,
                            int nblocks, float* grad, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_grad_partial,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sizeof(Smem)));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_mlp_grad_partial<<<nblocks, kTile, sizeof(Smem), s>>>(wbf, feats, targets, index, first,
                                                          count, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_mlp_grad_reduce<<<(kParams + 1 + 255) / 256, 256, 0, s>>>(partial, nblocks, count, grad);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* w, float* wbf, float* m, float* v, const float* grad, float lr,
                            int step, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, static_cast<float>(step));
  const float c2 = 1.0f - powf(b2, static_cast<float>(step));
  k_mlp_adam<<<(kParams + 255) / 256, 256, 0, s>>>(w, wbf, m, v, grad, lr, b1, b2, 1e-8f, c1, c2);
  return cudaGetLastError();
}

cudaError_t launch_mlp_round(const float* w, float* wbf, cudaStream_t s) {
  k_mlp_round<<<(kParams + 255) / 256, 256, 0, s>>>(w, wbf);
  return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const float* wbf, const float* feats, int64_t n, float* y,
                               cudaStream_t s) {
  int64_t b = (n + kTile - 1) / kTile;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  k_mlp_predict<<<static_cast<int>(b), kTile, 0, s>>>(wbf, feats, n, y);
  return cudaGetLastError();
}

cudaError_t launch_box_filter(const void* const macro[4], int bytes, int nx, int ny, int nz,
                              int f, void* out, cudaStream_t s) {
  const int64_t nc = static_cast<int64_t>(nx / f) * (ny / f) * (nz / f);
  int64_t b = (nc + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  if (bytes == 8)
    k_box_filter<double><<<static_cast<int>(b), 256, 0, s>>>(
        static_cast<const double*>(macro[0]), static_cast<const double*>(macro[1]),
        static_cast<const double*>(macro[2]), static_cast<const double*>(macro[3]), nx, ny, nz,
        f, static_cast<double*>(out));
  else
    k_box_filter<float><<<static_cast<int>(b), 256, 0, s>>>(
        static_cast<const float*>(macro[0]), static_cast<const float*>(macro[1]),
        static_cast<const float*>(macro[2]), static_cast<const float*>(macro[3]), nx, ny, nz, f,
        static_cast<float*>(out));
  return cudaGetLastError();
}

}  // namespace tlbm
