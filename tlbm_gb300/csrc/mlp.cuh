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

#include <cstdint>

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

// ---------------------------------------------------------------- tensor-core forward pass
// Inference inside the collide kernel runs on the tensor cores one warp at a time: the warp's
// 32 cells form two 16-row tiles, and mma.sync m16n8k16 (BF16 in, FP32 accumulate) computes
//   layer 1: H1[32 x 32] = X[32 x 16] W1^T  (K padded from 8 to 16 with zeros), 8 MMAs
//   layer 2: H2[32 x 32] = tanh(H1) W2^T,                                       16 MMAs
// The FP32 accumulator fragment of layer 1 has the layout of the BF16 A fragment of layer 2
// (rows g, g+8; columns 2t, 2t+1 of each 8-column tile), so tanh(H1) is packed to BF16 in
// registers and fed back without a trip through shared memory.  Layer 3 (32 -> 1) is a dot
// product on the accumulator fragments reduced over the 4 lanes of a row group.  Rounding
// points are those of `forward` (BF16 layer inputs, BF16 tanh outputs, FP32 accumulation).

constexpr int kW2Stride = 40;  // BF16 row stride of W2: fragment loads hit 32 distinct banks

struct MmaWeights {
  __nv_bfloat16 w1[kHid][kIn];
  __nv_bfloat16 w2[kHid][kW2Stride];
  float b1[kHid], b2[kHid], w3[kHid];
  float b3;
};

// all threads of the block: the network of `w` (kParams floats) into `s`
__device__ __forceinline__ void stage_mma_weights(const float* __restrict__ w, MmaWeights& s,
                                                  int tid, int nthreads) {
  for (int k = tid; k < kHid * kIn; k += nthreads)
    s.w1[k / kIn][k % kIn] = __float2bfloat16_rn(w[oW1 + k]);
  for (int k = tid; k < kHid * kHid; k += nthreads)
    s.w2[k / kHid][k % kHid] = __float2bfloat16_rn(w[oW2 + k]);
  for (int k = tid; k < kHid; k += nthreads) {
    s.b1[k] = w[oB1 + k];
    s.b2[k] = w[oB2 + k];
    s.w3[k] = w[oW3 + k];
  }
  if (tid == 0) s.b3 = w[oB3];
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
  uint32_t u;
  memcpy(&u, &v, 4);
  return u;
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The network output for this lane's cell.  All 32 lanes of the warp call it together
// (converged); xs / ys are the warp's scratch (32 x 4 words, 32 floats) in shared memory.
__device__ __forceinline__ float forward_warp(const MmaWeights& w, uint4* xs, float* ys,
                                              const float (&xin)[kIn], int lane) {
  xs[lane] = make_uint4(pack_bf16(xin[0], xin[1]), pack_bf16(xin[2], xin[3]),
                        pack_bf16(xin[4], xin[5]), pack_bf16(xin[6], xin[7]));
  __syncwarp();
  const int g = lane >> 2, t = lane & 3;
  const uint32_t* xw = reinterpret_cast<const uint32_t*>(xs);
  uint32_t a1[2][4];
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    a1[m][0] = xw[(16 * m + g) * 4 + t];      // row g,   k = 2t, 2t+1
    a1[m][1] = xw[(16 * m + g + 8) * 4 + t];  // row g+8
    a1[m][2] = 0u;                            // k = 8..15: padding
    a1[m][3] = 0u;
  }
  // layer 1, tanh, BF16: the A fragments of layer 2 (a2[m][kk] covers k = 16 kk .. 16 kk + 15)
  uint32_t a2[2][2][4];
#pragma unroll
  for (int n = 0; n < 4; ++n) {
    const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&w.w1[8 * n + g][2 * t]);
    const float c0 = w.b1[8 * n + 2 * t], c1 = w.b1[8 * n + 2 * t + 1];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      float d[4] = {c0, c1, c0, c1};
      mma_bf16(d, a1[m], b0, 0u);
      const int kk = n >> 1, half = (n & 1) * 2;
      a2[m][kk][half] = pack_bf16(tanh_fast(d[0]), tanh_fast(d[1]));
      a2[m][kk][half + 1] = pack_bf16(tanh_fast(d[2]), tanh_fast(d[3]));
    }
  }
  // layer 2 and the output dot product, one 8-column tile at a time
  float s[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
  for (int n = 0; n < 4; ++n) {
    const __nv_bfloat16* row = w.w2[8 * n + g];
    const uint32_t b00 = *reinterpret_cast<const uint32_t*>(row + 2 * t);
    const uint32_t b01 = *reinterpret_cast<const uint32_t*>(row + 2 * t + 8);
    const uint32_t b10 = *reinterpret_cast<const uint32_t*>(row + 16 + 2 * t);
    const uint32_t b11 = *reinterpret_cast<const uint32_t*>(row + 24 + 2 * t);
    const float c0 = w.b2[8 * n + 2 * t], c1 = w.b2[8 * n + 2 * t + 1];
    const float w30 = w.w3[8 * n + 2 * t], w31 = w.w3[8 * n + 2 * t + 1];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      float d[4] = {c0, c1, c0, c1};
      mma_bf16(d, a2[m][0], b00, b01);
      mma_bf16(d, a2[m][1], b10, b11);
      s[m][0] = fmaf(w30, bf16r(tanh_fast(d[0])), s[m][0]);
      s[m][0] = fmaf(w31, bf16r(tanh_fast(d[1])), s[m][0]);
      s[m][1] = fmaf(w30, bf16r(tanh_fast(d[2])), s[m][1]);
      s[m][1] = fmaf(w31, bf16r(tanh_fast(d[3])), s[m][1]);
    }
  }
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      s[m][h] += __shfl_xor_sync(0xFFFFFFFFu, s[m][h], 1);
      s[m][h] += __shfl_xor_sync(0xFFFFFFFFu, s[m][h], 2);
    }
  if (t == 0) {
    ys[g] = s[0][0];
    ys[g + 8] = s[0][1];
    ys[g + 16] = s[1][0];
    ys[g + 24] = s[1][1];
  }
  __syncwarp();
  const float y = ys[lane] + w.b3;
  __syncwarp();  // the scratch may be reused by the next call
  return y;
}

}  // namespace mlp
}  // namespace tlbm
