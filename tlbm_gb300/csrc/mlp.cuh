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
// Weights are BF16 (rounded from FP32 master copies), biases FP32, accumulation FP32.  The
// activation is act(z) = tanh of z rounded to BF16, evaluated by the special-function unit in
// BF16 (tanh.approx.bf16, two lanes per instruction in the packed form), so every layer input
// is a BF16 value.  Training (kernels_mlp.cu) and inference (the fused collide kernel) use the
// same act, so the network trained is the network run.
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

struct MmaWeights;

// what the collide kernel needs to evaluate the closure
struct Closure {
  const MmaWeights* w;  // the network, as the tensor-core pass reads it
  float scale[kIn], shift[kIn];
  float offset[kIn];  // -shift * scale: the normalisation is one FMA per input
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

// host-side BF16 bits of v (round to nearest even, finite v)
inline uint16_t bf16_bits_host(float v) {
  const float r = bf16r(v);
  unsigned u;
  memcpy(&u, &r, 4);
  return static_cast<uint16_t>(u >> 16);
}

#if defined(__CUDACC__)
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
  uint32_t u;
  memcpy(&u, &v, 4);
  return u;
}

// act on two values packed as BF16x2
__device__ __forceinline__ uint32_t act2(uint32_t zz) {
  uint32_t r;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(r) : "r"(zz));
  return r;
}

// act(z) for one value, as a float holding a BF16 value
__device__ __forceinline__ float act(float z) {
  const uint32_t r = act2(pack_bf16(z, 0.0f));
  return __uint_as_float(r << 16);
}
#endif

// ---------------------------------------------------------------- tensor-core forward pass
// Inference inside the collide kernel runs on the tensor cores one warp at a time: the warp's
// 32 cells form two 16-row tiles, and mma.sync m16n8k16 (BF16 in, FP32 accumulate) computes
//   layer 1: H1[32 x 32] = X[32 x 16] W1^T  (K padded from 8 to 16 with zeros), 8 MMAs
//   layer 2: H2[32 x 32] = act(H1) W2^T,                                        16 MMAs
//   layer 3: y[32]       = act(H2) w3,                                           4 MMAs
// The FP32 accumulator fragment of layer 1 has the layout of the BF16 A fragment of layer 2
// (rows g, g+8; columns 2t, 2t+1 of each 8-column tile), so act(H1) is packed to BF16 in
// registers and fed back without a trip through shared memory; layer 3 (32 -> 1) is one more
// pair of MMAs with w3 as column 0 of the B tile.

constexpr int kRowStride = 40;  // BF16 row stride of the 32-column tiles: ldmatrix rows hit
                                // 32 distinct banks (80-byte rows)

// The network as the tensor-core pass reads it, built on the host (build_mma_weights) and
// copied to shared memory with 16-byte loads.  Matrices are stored [output][input] (the
// col-major B operand of mma.m16n8k16), so ldmatrix hands out B fragments directly; w3 is
// row 0 of an otherwise zero 8-row tile (column 0 of the layer-3 B tile).
struct alignas(16) MmaWeights {
  uint16_t w1[kHid][kIn];          // BF16 bits, 16-byte rows
  uint16_t w2[kHid][kRowStride];   // BF16 bits, columns 32..39 unused
  uint16_t w3[8][kRowStride];      // row 0 = w3, rows 1..7 = 0
  float b1[kHid], b2[kHid];
  float b3;
};
static_assert(sizeof(MmaWeights) % 16 == 0, "copied as 16-byte words");

inline void build_mma_weights(const float* params, MmaWeights* out) {
  memset(out, 0, sizeof(*out));
  for (int j = 0; j < kHid; ++j) {
    for (int k = 0; k < kIn; ++k) out->w1[j][k] = bf16_bits_host(params[oW1 + j * kIn + k]);
    for (int k = 0; k < kHid; ++k) out->w2[j][k] = bf16_bits_host(params[oW2 + j * kHid + k]);
    out->w3[0][j] = bf16_bits_host(params[oW3 + j]);
    out->b1[j] = params[oB1 + j];
    out->b2[j] = params[oB2 + j];
  }
  out->b3 = params[oB3];
}

#if defined(__CUDACC__)
// all threads of the block: the image at `g` (global memory) into `s`
__device__ __forceinline__ void copy_mma_weights(const MmaWeights* __restrict__ g, MmaWeights& s,
                                                 int tid, int nthreads) {
  const uint4* src = reinterpret_cast<const uint4*>(g);
  uint4* dst = reinterpret_cast<uint4*>(&s);
  for (int k = tid; k < static_cast<int>(sizeof(MmaWeights) / 16); k += nthreads)
    dst[k] = __ldg(src + k);
}

// all threads of the block: the image of `w` (kParams floats, weights BF16-valued) into `s`
__device__ __forceinline__ void stage_mma_weights(const float* __restrict__ w, MmaWeights& s,
                                                  int tid, int nthreads) {
  auto bits = [](float v) {
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    uint16_t u;
    memcpy(&u, &b, 2);
    return u;
  };
  uint16_t* w3 = &s.w3[0][0];
  for (int k = tid; k < 8 * kRowStride; k += nthreads) w3[k] = 0;
  __syncthreads();
  for (int k = tid; k < kHid * kIn; k += nthreads) s.w1[k / kIn][k % kIn] = bits(w[oW1 + k]);
  for (int k = tid; k < kHid * kHid; k += nthreads)
    s.w2[k / kHid][k % kHid] = bits(w[oW2 + k]);
  for (int k = tid; k < kHid; k += nthreads) {
    s.w3[0][k] = bits(w[oW3 + k]);
    s.b1[k] = w[oB1 + k];
    s.b2[k] = w[oB2 + k];
  }
  if (tid == 0) s.b3 = w[oB3];
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// four 8x8 BF16 matrices; lane L gives the address of row L % 8 of matrix L / 8 and receives
// in r[j] the elements (row L / 4, columns 2 (L % 4), 2 (L % 4) + 1) of matrix j
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* row) {
  const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(row));
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

// The network output for this lane's cell.  All 32 lanes of the warp call it together
// (converged); xs / ys are the warp's scratch (32 x 4 words, 32 floats) in shared memory.
// The warp's two 16-row tiles go through the network one after the other (fewer live
// registers); per tile 4 + 8 + 2 MMAs.  The accumulator fragments of layers 1 and 2, packed to
// BF16x2 and passed through act2, are the A fragments of layers 2 and 3.
__device__ __forceinline__ float forward_warp(const MmaWeights& w, uint4* xs, float* ys,
                                              const float (&xin)[kIn], int lane) {
  xs[lane] = make_uint4(pack_bf16(xin[0], xin[1]), pack_bf16(xin[2], xin[3]),
                        pack_bf16(xin[4], xin[5]), pack_bf16(xin[6], xin[7]));
  __syncwarp();
  const int g = lane >> 2, t = lane & 3;
  const int lr = lane & 7, lm = lane >> 3;  // ldmatrix: row and matrix this lane addresses
  const uint32_t* xw = reinterpret_cast<const uint32_t*>(xs);
#pragma unroll 1
  for (int m = 0; m < 2; ++m) {
    const uint32_t a1[4] = {xw[(16 * m + g) * 4 + t], xw[(16 * m + g + 8) * 4 + t], 0u, 0u};
    uint32_t b1f[4];  // b1f[n]: W1 rows 8n .. 8n + 7
    ldsm_x4(b1f, &w.w1[lane][0]);
    uint32_t a2[2][4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const float2 bias = *reinterpret_cast<const float2*>(&w.b1[8 * n + 2 * t]);
      float d[4] = {bias.x, bias.y, bias.x, bias.y};
      mma_bf16(d, a1, b1f[n], 0u);
      a2[n >> 1][(n & 1) * 2] = act2(pack_bf16(d[0], d[1]));
      a2[n >> 1][(n & 1) * 2 + 1] = act2(pack_bf16(d[2], d[3]));
    }
    uint32_t a3[2][4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      uint32_t b[4];  // columns 0-7, 8-15, 16-23, 24-31 of W2 rows 8n .. 8n + 7
      ldsm_x4(b, &w.w2[8 * n + lr][8 * lm]);
      const float2 bias = *reinterpret_cast<const float2*>(&w.b2[8 * n + 2 * t]);
      float d[4] = {bias.x, bias.y, bias.x, bias.y};
      mma_bf16(d, a2[0], b[0], b[1]);
      mma_bf16(d, a2[1], b[2], b[3]);
      a3[n >> 1][(n & 1) * 2] = act2(pack_bf16(d[0], d[1]));
      a3[n >> 1][(n & 1) * 2 + 1] = act2(pack_bf16(d[2], d[3]));
    }
    uint32_t b3f[4];
    ldsm_x4(b3f, &w.w3[lr][8 * lm]);
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma_bf16(d, a3[0], b3f[0], b3f[1]);
    mma_bf16(d, a3[1], b3f[2], b3f[3]);
    if (t == 0) {  // column 0: rows g and g + 8 of tile m
      ys[16 * m + g] = d[0];
      ys[16 * m + g + 8] = d[2];
    }
  }
  __syncwarp();
  const float y = ys[lane] + w.b3;
  __syncwarp();  // the scratch may be reused by the next call
  return y;
}
#endif

}  // namespace mlp
}  // namespace tlbm
