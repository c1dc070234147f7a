// mlp.cuh -- the learned eddy-viscosity closure: an 8-32-32-1 tanh MLP per fluid cell.
//
// Inputs (normalised x_k = (raw_k - shift_k) * scale_k):
//   raw = [Pi_xx, Pi_yy, Pi_zz, Pi_xy, Pi_xz, Pi_yz, rho - 1, |Pi|]
// where Pi_ab = sum_i e_ia e_ib (f_i - feq_i) is the non-equilibrium stress the Smagorinsky
// model of the reference also starts from (include/LatticeStructure.hpp:106-153), and |Pi| its
// Frobenius norm (the strain-rate norm up to the factor -2 rho c_s^2 tau).
// Output: nu_t = out_scale * y, tau_eff = max(3 (nu + nu_t) + 1/2, tau_min) with tau_min > 1/2;
// a non-finite output falls back to the Smagorinsky rate.
//
// Weights are BF16 (rounded from FP32 master copies), activations entering each layer are
// rounded to BF16, accumulation is FP32: training (kernels_mlp.cu) and inference (the fused
// collide kernel) round identically, so the network trained is the network run.
#pragma once

#include <cuda_bf16.h>

#include <cstring>

namespace tlbm {
namespace mlp {

constexpr int kIn = 8;
constexpr int kHid = 32;
constexpr int oW1 = 0;                   // [kHid][kIn]
constexpr int oB1 = oW1 + kHid * kIn;    // [kHid]
constexpr int oW2 = oB1 + kHid;          // [kHid][kHid]
constexpr int oB2 = oW2 + kHid * kHid;   // [kHid]
constexpr int oW3 = oB2 + kHid;          // [kHid]
constexpr int oB3 = oW3 + kHid;          // [1]
constexpr int kParams = oB3 + 1;         // 1377

// what the collide kernel needs besides the weights
struct Closure {
  const float* w;  // kParams values: weights already rounded to BF16, biases FP32
  float scale[kIn], shift[kIn];
  float out_scale;
  float tau_min;
};

__host__ __device__ __forceinline__ float bf16r(float v) {
#if defined(__CUDA_ARCH__)
  return __bfloat162float(__float2bfloat16_rn(v));
#else
  // round to nearest even on the top 16 bits (finite inputs)
  unsigned u;
  memcpy(&u, &v, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  u &= 0xFFFF0000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
#endif
}

__device__ __forceinline__ float tanh_fast(float x) {
  float r;
  asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// y = w3 . tanh(W2 tanh(W1 x + b1) + b2) + b3 with BF16 rounding of each layer's input.
// `w` points to kParams floats (BF16-valued weights); shared memory in the kernels.
__device__ __forceinline__ float forward(const float* __restrict__ w, const float (&xin)[kIn]) {
  float x[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) x[k] = bf16r(xin[k]);
  float h1[kHid];
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    float z = w[oB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; ++k) z = fmaf(w[oW1 + j * kIn + k], x[k], z);
    h1[j] = bf16r(tanh_fast(z));
  }
  float y = w[oB3];
#pragma unroll 4
  for (int j = 0; j < kHid; ++j) {
    float z = w[oB2 + j];
#pragma unroll
    for (int k = 0; k < kHid; ++k) z = fmaf(w[oW2 + j * kHid + k], h1[k], z);
    y = fmaf(w[oW3 + j], bf16r(tanh_fast(z)), y);
  }
  return y;
}

}  // namespace mlp
}  // namespace tlbm
