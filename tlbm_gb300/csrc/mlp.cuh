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
// activation is act(z) = BF16(tanh(z)): the special-function unit's FP32 tanh (tanh.approx.f32,
// relative error below 2^-10.9) of the FP32 pre-activation, rounded to BF16 once, so every
// layer input is a BF16 value.  In the tensor-core pass the rounding is the pack of two
// activations into the BF16x2 word of an A fragment.  Training (kernels_mlp.cu) and inference
// (the fused collide kernel) use the same act, so the network trained is the network run.
#pragma once

#include <cuda_bf16.h>

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <type_traits>

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

// the special-function unit's tanh of an FP32 value
__device__ __forceinline__ float tanh_sfu(float z) {
  float r;
  asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(z));
  return r;
}

// act of two FP32 pre-activations, packed as the BF16x2 word (lo in the low half)
__device__ __forceinline__ uint32_t act2(float lo, float hi) {
  return pack_bf16(tanh_sfu(lo), tanh_sfu(hi));
}

// act(z) for one value, as a float holding a BF16 value
__device__ __forceinline__ float act(float z) {
  return __bfloat162float(__float2bfloat16_rn(tanh_sfu(z)));
}
#endif

// ---------------------------------------------------------------- tensor-core forward pass
// Inference inside the collide kernel runs on the tensor cores one warp at a time: the warp's
// 32 cells form two 16-row tiles, and mma.sync m16n8k16 (BF16 in, FP32 accumulate) computes
//   layer 1: H1[32 x 32] = [X 1 1 1 0..][W1 b1h b1m b1l 0..]^T,   8 MMAs
//   layer 2: H2[32 x 32] = act(H1) W2^T + b2,                    16 MMAs
//   layer 3: y[32]       = act(H2) w3 (+ b3 after the exchange),  4 MMAs
// Layer 1's K runs over the 8 inputs and, in the columns 8..10 the inputs leave free, over
// three constant ones that multiply the BF16 parts b1h + b1m + b1l = b1 of the FP32 bias (exact:
// three BF16 significands hold FP32's), so its bias costs no load.  The FP32 accumulator
// fragment of layer 1 has the layout of the BF16 A fragment of layer 2 (rows g, g+8; columns
// 2t, 2t+1 of each 8-column tile), so act(H1) is packed to BF16 in registers (two
// tanh.approx.f32 and one cvt per word) and fed back without a trip through shared memory;
// layer 3 (32 -> 1) is one more pair of MMAs with w3 as column 0 of the B tile.

// The network as the tensor-core pass reads it: every lane's B fragments, in fragment order,
// so one 16-byte load hands a lane four fragment registers.  Lane (g, t) = (lane / 4, lane % 4)
// holds, for column tile n (hidden units 8n .. 8n + 7):
//   layer 1 (K = 16): w1f[n / 2][lane].(2 (n % 2)) = (W1[8n+g][2t], W1[8n+g][2t+1]),
//                     w1f[n / 2][lane].(2 (n % 2) + 1) = columns 8 + 2t, 9 + 2t of the bias
//                     block: (b1h, b1m)[8n+g] for t = 0, (b1l, 0) for t = 1, zero otherwise
//   layer 2 (K = 32): w2f[n][lane].j = (W2[8n+g][8j+2t], W2[8n+g][8j+2t+1]), j = 0..3
//                     (j = 0, 1: the k16 step over inputs 0..15; j = 2, 3: inputs 16..31)
//   layer 3 (N = 1):  w3 is column 0 of the B tile: lanes with g = 0 hold w3f[t] = the pairs
//                     w3[2t..], w3[8+2t..], w3[16+2t..], w3[24+2t..]; the others the zero row
//                     w3f[4]
// and layer 2's bias as accumulator quads, b2q[n][t] = (b2[8n+2t], b2[8n+2t+1]) twice: the
// initial value of the fragment (rows g, g+8; columns 2t, 2t+1) of column tile n, loaded
// straight into the MMA's C operand.  Matrices W are [output][input]; weights are BF16 bits,
// biases FP32.  Both the collide kernel and the training pass read the image from shared
// memory.
struct alignas(16) MmaWeights {
  uint4 w1f[2][32];   // [n / 2][lane]
  uint4 w2f[4][32];   // [n][lane]
  float4 b2q[4][4];   // [n][t]
  uint4 w3f[5];       // [t], row 4 = 0
  float b3, pad[3];
};
static_assert(sizeof(MmaWeights) % 16 == 0, "copied as 16-byte words");

// A warp's scratch for the forward pass, in shared memory: the 32 cells' layer-1 A rows (the 8
// inputs, the three constant ones, zeros; BF16, 48-byte rows so that ldmatrix reads the 8 rows
// of each of its matrices from distinct banks) and the 32 outputs.
struct alignas(16) WarpScratch {
  uint4 x[32][3];  // [cell][16-byte column block], block 2 unused
  float y[32];
};

// the value of the BF16 bits bits(v), as a float
template <class Bits>
__host__ __device__ inline float bf16_value(float v, Bits bits) {
  const uint32_t u = static_cast<uint32_t>(bits(v)) << 16;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

// the image from kParams FP32 parameters (weights rounded to BF16 here); bits(v) gives the
// BF16 bits of v, so host and device build the same image
template <class Bits>
__host__ __device__ inline void mma_image_entry(const float* p, int k, MmaWeights& o, Bits bits) {
  auto word = [&](float lo, float hi) {  // (lo, hi) as one fragment word (lo in the low half)
    return static_cast<uint32_t>(bits(lo)) | (static_cast<uint32_t>(bits(hi)) << 16);
  };
  auto pair = [&](int i) { return word(p[i], p[i + 1]); };
  // k enumerates the 16-byte words of the image
  if (k < 64) {
    const int h = k >> 5, lane = k & 31, g = lane >> 2, t = lane & 3;
    uint32_t r[4];
    for (int j = 0; j < 2; ++j) {
      const int n = 2 * h + j;
      r[2 * j] = pair(oW1 + (8 * n + g) * kIn + 2 * t);
      // b1 = hi + mid + lo exactly: each part is the BF16 rounding of what is left
      const float b = p[oB1 + 8 * n + g];
      const float hi = bf16_value(b, bits), mid = bf16_value(b - hi, bits);
      const float lo = bf16_value(b - hi - mid, bits);
      r[2 * j + 1] = t == 0 ? word(hi, mid) : (t == 1 ? word(lo, 0.0f) : 0u);
    }
    o.w1f[h][lane] = {r[0], r[1], r[2], r[3]};
  } else if (k < 64 + 128) {
    const int n = (k - 64) >> 5, lane = (k - 64) & 31, g = lane >> 2, t = lane & 3;
    uint32_t r[4];
    for (int j = 0; j < 4; ++j) r[j] = pair(oW2 + (8 * n + g) * kHid + 8 * j + 2 * t);
    o.w2f[n][lane] = {r[0], r[1], r[2], r[3]};
  } else if (k < 192 + 16) {
    const int n = (k - 192) >> 2, t = (k - 192) & 3;
    const float* b = p + oB2 + 8 * n + 2 * t;
    o.b2q[n][t] = {b[0], b[1], b[0], b[1]};
  } else if (k < 208 + 4) {
    const int t = k - 208;
    o.w3f[t] = {pair(oW3 + 2 * t), pair(oW3 + 8 + 2 * t), pair(oW3 + 16 + 2 * t),
                pair(oW3 + 24 + 2 * t)};
  } else if (k == 212) {
    o.w3f[4] = {0u, 0u, 0u, 0u};
  } else if (k == 213) {
    o.b3 = p[oB3];
    o.pad[0] = o.pad[1] = o.pad[2] = 0.0f;
  }
}
constexpr int kImageWords = 214;
static_assert(kImageWords * 16 == sizeof(MmaWeights), "one entry per 16-byte word");

inline void build_mma_weights(const float* params, MmaWeights* out) {
  for (int k = 0; k < kImageWords; ++k) mma_image_entry(params, k, *out, bf16_bits_host);
}

#if defined(__CUDACC__)
// all threads of the block: the image at `g` (global memory) into `s`, 16 bytes per copy
__device__ __forceinline__ void copy_mma_weights(const MmaWeights* __restrict__ g, MmaWeights& s,
                                                 int tid, int nthreads) {
  const uint4* src = reinterpret_cast<const uint4*>(g);
  uint4* dst = reinterpret_cast<uint4*>(&s);
  for (int k = tid; k < kImageWords; k += nthreads) dst[k] = __ldg(src + k);
}

// all threads of the block: the image of `w` (kParams floats) into `s`
__device__ __forceinline__ void stage_mma_weights(const float* __restrict__ w, MmaWeights& s,
                                                  int tid, int nthreads) {
  auto bits = [](float v) {
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    uint16_t u;
    memcpy(&u, &b, 2);
    return u;
  };
  for (int k = tid; k < kImageWords; k += nthreads) mma_image_entry(w, k, s, bits);
}

// D += A B, m16n8k16 (BF16 in, FP32 accumulate)
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
// (row: a shared-memory address)
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], unsigned row) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(row));
}

// D = A B, m16n8k16 (the zero accumulator is set inside the statement, so no zero registers
// stay live outside it)
__device__ __forceinline__ void mma_bf16_z(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                           uint32_t b1) {
  asm volatile(
      "{\n\t"
      "mov.f32 %0, 0f00000000;\n\t"
      "mov.f32 %1, 0f00000000;\n\t"
      "mov.f32 %2, 0f00000000;\n\t"
      "mov.f32 %3, 0f00000000;\n\t"
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n\t"
      "}"
      : "=&f"(d[0]), "=&f"(d[1]), "=&f"(d[2]), "=&f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// D = A B + C, m16n8k16, with C read from a register quad the MMA does not overwrite
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1, const float4& c) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%10,%11,%12,%13};"
      : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(c.x), "f"(c.y),
        "f"(c.z), "f"(c.w));
}

// The 16-byte word kOff bytes past `base` in the image (shared memory).  The offset is an
// immediate of the load and the load is volatile, so that it stays where it is written: every
// tile reloads its fragments from three base addresses instead of holding the whole image in
// registers.
template <int kOff>
__device__ __forceinline__ uint4 image_ld(unsigned base) {
  uint4 r;
  asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4+%5];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "r"(base), "n"(kOff));
  return r;
}

template <int kOff>
__device__ __forceinline__ float4 image_ldf(unsigned base) {
  const uint4 r = image_ld<kOff>(base);
  return make_float4(__uint_as_float(r.x), __uint_as_float(r.y), __uint_as_float(r.z),
                     __uint_as_float(r.w));
}

// The network output for this lane's cell.  All 32 lanes of the warp call it together
// (converged); s is the warp's scratch and w the image, both in shared memory.  The warp's two
// 16-row tiles go through the network one after the other (fewer live registers); per tile
// 4 + 8 + 2 MMAs.  The accumulator fragments of layers 1 and 2, through act2 (tanh, then the
// BF16x2 pack), are the A fragments of layers 2 and 3; layer 2's bias quads are the C operands
// of each column tile's first MMA.  Fragment loads are volatile with immediate offsets
// (image_ld), and the zero accumulators are set inside the MMA statements, so the image and
// the constants stay out of the registers between uses.
__device__ __forceinline__ float forward_warp(const MmaWeights& w, WarpScratch& s,
                                              const float (&xin)[kIn], int lane) {
  // this cell's A row: inputs 0..7, then ones in columns 8, 9, 10 (BF16 1.0 = 0x3F80)
  s.x[lane][0] = make_uint4(pack_bf16(xin[0], xin[1]), pack_bf16(xin[2], xin[3]),
                            pack_bf16(xin[4], xin[5]), pack_bf16(xin[6], xin[7]));
  s.x[lane][1] = make_uint4(0x3F803F80u, 0x00003F80u, 0u, 0u);
  __syncwarp();
  const int g = lane >> 2, t = lane & 3;
  // ldmatrix rows: matrices 0..3 = (rows 0-7, columns 0-7), (8-15, 0-7), (0-7, 8-15), (8-15, 8-15)
  const unsigned arow = static_cast<unsigned>(
      __cvta_generic_to_shared(&s.x[(lane & 7) + ((lane >> 3) & 1) * 8][lane >> 4]));
  const unsigned img = static_cast<unsigned>(__cvta_generic_to_shared(&w));
  const unsigned lb = img + 16 * lane;               // this lane's fragment words
  const unsigned tb = img + 16 * t;                  // the bias quads of column pair 2t
  const unsigned w3b = img + 16 * (g == 0 ? t : 4);  // layer 3: w3 in column 0
  constexpr int kW1 = offsetof(MmaWeights, w1f), kW2 = offsetof(MmaWeights, w2f);
  constexpr int kB2 = offsetof(MmaWeights, b2q), kW3 = offsetof(MmaWeights, w3f);
#pragma unroll 1
  for (int m = 0; m < 2; ++m) {
    uint32_t a1[4];  // A of layer 1: rows 16m .. 16m + 15
    ldsm_x4(a1, arow + 16 * sizeof(s.x[0]) * m);
    uint32_t a2[2][4];
    auto layer1 = [&](auto hc) {
      constexpr int h = decltype(hc)::value;  // column tiles 2h, 2h + 1
      const uint4 b = image_ld<kW1 + h * 512>(lb);
      float d[4];
      mma_bf16_z(d, a1, b.x, b.y);
      a2[h][0] = act2(d[0], d[1]);
      a2[h][1] = act2(d[2], d[3]);
      mma_bf16_z(d, a1, b.z, b.w);
      a2[h][2] = act2(d[0], d[1]);
      a2[h][3] = act2(d[2], d[3]);
    };
    layer1(std::integral_constant<int, 0>());
    layer1(std::integral_constant<int, 1>());
    uint32_t a3[2][4];
    auto layer2 = [&](auto nc) {
      constexpr int n = decltype(nc)::value;
      const uint4 b = image_ld<kW2 + n * 512>(lb);
      float d[4];
      mma_bf16(d, a2[0], b.x, b.y, image_ldf<kB2 + n * 64>(tb));
      mma_bf16(d, a2[1], b.z, b.w);
      a3[n >> 1][(n & 1) * 2] = act2(d[0], d[1]);
      a3[n >> 1][(n & 1) * 2 + 1] = act2(d[2], d[3]);
    };
    layer2(std::integral_constant<int, 0>());
    layer2(std::integral_constant<int, 1>());
    layer2(std::integral_constant<int, 2>());
    layer2(std::integral_constant<int, 3>());
    const uint4 b3 = image_ld<kW3>(w3b);
    float y[4];
    mma_bf16_z(y, a3[0], b3.x, b3.y);
    mma_bf16(y, a3[1], b3.z, b3.w);
    if (t == 0) {  // column 0: rows g and g + 8 of tile m
      s.y[16 * m + g] = y[0];
      s.y[16 * m + g + 8] = y[2];
    }
  }
  __syncwarp();
  const float y = s.y[lane] + w.b3;
  __syncwarp();  // the scratch may be reused by the next call
  return y;
}
#endif

}  // namespace mlp
}  // namespace tlbm
