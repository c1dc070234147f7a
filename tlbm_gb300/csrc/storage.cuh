// storage.cuh -- how populations are held in HBM and what they are computed in.
//
//   kStoreF64  : double,          computed in double
//   kStoreF32  : float,           computed in float
//   kStoreBF16 : bfloat16 of f-w, computed in float (f = w + stored)
//   kStoreF16  : half of f-w,     computed in float
//   kStoreBF16M: bfloat16 of f - w (rho_s + e.(3 j_s)), computed in float, where rho_s and j_s
//                are the density and momentum of the populations the cell s that stored them
//                held after its collision; (rho_s, 3 j_s) follow the Q planes as one float4 per
//                cell.
//   kStoreFX   : FP64 populations as 64-bit fixed point Q1.62 (physics_fx.cuh), fluid nodes
//                collided in fixed point as stored, everything else computed in double after
//                a conversion to the nearest double (and back to the nearest Q1.62).
// Storing f_i - w_i keeps the 16-bit mantissa on the part that varies: at rest f_i == w_i and
// the stored value is 0, so the round-off scales with the deviation, not with w_i.  The
// moment shift also removes the first-order part w_i 3 e_i.j: the remainder is the second-order
// and non-equilibrium part (~1 % of w_i at |u| ~ 0.05), so BF16's 8 mantissa bits lose ~15x
// less.  Writer and reader form the shift with the same float operations from the same stored
// float4, so only the remainder is rounded.
//
// Store<K>::T is the per-population value a thread holds after loading (the memory type, or the
// reconstructed float for kStoreBF16M); Store<K>::P is the memory type.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kernels.h"
#include "lattice.cuh"

namespace tlbm {

template <int K>
struct Store;

template <>
struct Store<kStoreF64> {
  using T = double;
  using P = T;
  static constexpr bool kMoment = false;
  using C = double;
  static constexpr bool kShifted = false;
  static __device__ __forceinline__ C load(T v, C) { return v; }
  static __device__ __forceinline__ T save(C f, C) { return f; }
};

template <>
struct Store<kStoreF32> {
  using T = float;
  using P = T;
  static constexpr bool kMoment = false;
  using C = float;
  static constexpr bool kShifted = false;
  static __device__ __forceinline__ C load(T v, C) { return v; }
  static __device__ __forceinline__ T save(C f, C) { return f; }
};

template <>
struct Store<kStoreBF16> {
  using T = __nv_bfloat16;
  using P = T;
  static constexpr bool kMoment = false;
  using C = float;
  static constexpr bool kShifted = true;
  static __device__ __forceinline__ C load(T v, C w) { return w + __bfloat162float(v); }
  static __device__ __forceinline__ T save(C f, C w) { return __float2bfloat16_rn(f - w); }
  // the stored shift f - w itself
  static __device__ __forceinline__ C shift_of(T v) { return __bfloat162float(v); }
  static __device__ __forceinline__ T of_shift(C d) { return __float2bfloat16_rn(d); }
};

template <>
struct Store<kStoreF16> {
  using T = __half;
  using P = T;
  static constexpr bool kMoment = false;
  using C = float;
  static constexpr bool kShifted = true;
  static __device__ __forceinline__ C load(T v, C w) { return w + __half2float(v); }
  static __device__ __forceinline__ T save(C f, C w) { return __float2half_rn(f - w); }
  static __device__ __forceinline__ C shift_of(T v) { return __half2float(v); }
  static __device__ __forceinline__ T of_shift(C d) { return __float2half_rn(d); }
};

template <>
struct Store<kStoreFX> {
  using T = fx::i64;
  using P = T;
  static constexpr bool kMoment = false;
  using C = double;
  static constexpr bool kShifted = false;
  static __device__ __forceinline__ C load(T v, C) { return fx::f64_of_store(v); }
  static __device__ __forceinline__ T save(C f, C) { return fx::store_of_f64(f); }
};

template <>
struct Store<kStoreBF16M> {
  using T = float;          // reconstructed population
  using P = __nv_bfloat16;  // stored remainder
  using C = float;
  static constexpr bool kShifted = false;
  static constexpr bool kMoment = true;
  static __device__ __forceinline__ C load(T v, C) { return v; }
};

namespace moment {

// the per-cell float4 (rho, 3 jx, 3 jy, 3 jz) after the Q planes of a buffer
__host__ __device__ __forceinline__ size_t params_offset(int q, size_t n) {
  return ((n * q * 2 + 15) / 16) * 16;
}
__device__ __forceinline__ const float4* params(const void* f, int q, size_t n) {
  return reinterpret_cast<const float4*>(static_cast<const char*>(f) + params_offset(q, n));
}
__device__ __forceinline__ float4* params(void* f, int q, size_t n) {
  return reinterpret_cast<float4*>(static_cast<char*>(f) + params_offset(q, n));
}

// w_i (rho + e_i . (3 j)) for the float4 p = (rho, 3 jx, 3 jy, 3 jz), in a fixed order
template <class L>
__device__ __forceinline__ float shift(int i, float4 p) {
  float t = p.x;
  if (L::ex(i) > 0) t = __fadd_rn(t, p.y);
  if (L::ex(i) < 0) t = __fsub_rn(t, p.y);
  if (L::ey(i) > 0) t = __fadd_rn(t, p.z);
  if (L::ey(i) < 0) t = __fsub_rn(t, p.z);
  if (L::ez(i) > 0) t = __fadd_rn(t, p.w);
  if (L::ez(i) < 0) t = __fsub_rn(t, p.w);
  return __fmul_rn(static_cast<float>(L::wlit(i)), t);
}

// population i of a buffer at slot `cell` (which cell s stored), reconstructed
template <class L>
__device__ __forceinline__ float load(const __nv_bfloat16* __restrict__ planes,
                                      const float4* __restrict__ prm, size_t n, int i,
                                      int64_t cell) {
  return __fadd_rn(shift<L>(i, __ldg(prm + cell)),
                   __bfloat162float(__ldg(planes + i * n + cell)));
}

// the moments a cell stores with its populations f
template <class L>
__device__ __forceinline__ float4 moments_of(const float (&f)[L::Q]) {
  float rho = 0.f, jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    rho = __fadd_rn(rho, f[i]);
    if (L::ex(i) > 0) jx = __fadd_rn(jx, f[i]);
    if (L::ex(i) < 0) jx = __fsub_rn(jx, f[i]);
    if (L::ey(i) > 0) jy = __fadd_rn(jy, f[i]);
    if (L::ey(i) < 0) jy = __fsub_rn(jy, f[i]);
    if (L::ez(i) > 0) jz = __fadd_rn(jz, f[i]);
    if (L::ez(i) < 0) jz = __fsub_rn(jz, f[i]);
  }
  return make_float4(rho, __fmul_rn(3.f, jx), __fmul_rn(3.f, jy), __fmul_rn(3.f, jz));
}

// cell c stores f (its populations after collision) in the buffer `buf`
template <class L>
__device__ __forceinline__ void store(void* buf, size_t n, int64_t c, const float (&f)[L::Q]) {
  const float4 p = moments_of<L>(f);
  params(buf, L::Q, n)[c] = p;
  __nv_bfloat16* planes = static_cast<__nv_bfloat16*>(buf);
#pragma unroll
  for (int i = 0; i < L::Q; ++i)
    planes[i * n + c] = __float2bfloat16_rn(__fsub_rn(f[i], shift<L>(i, p)));
}

}  // namespace moment

}  // namespace tlbm
