// storage.cuh -- how populations are held in HBM and what they are computed in.
//
//   kStoreF64  : double,          computed in double
//   kStoreF32  : float,           computed in float
//   kStoreBF16 : bfloat16 of f-w, computed in float (f = w + stored)
//   kStoreF16  : half of f-w,     computed in float
// Storing f_i - w_i keeps the 16-bit mantissa on the part that varies: at rest f_i == w_i and
// the stored value is 0, so the round-off scales with the deviation, not with w_i.
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
  using C = double;
  static constexpr bool kShifted = false;
  static __device__ __forceinline__ C load(T v, C) { return v; }
  static __device__ __forceinline__ T save(C f, C) { return f; }
};

template <>
struct Store<kStoreF32> {
  using T = float;
  using C = float;
  static constexpr bool kShifted = false;
  static __device__ __forceinline__ C load(T v, C) { return v; }
  static __device__ __forceinline__ T save(C f, C) { return f; }
};

template <>
struct Store<kStoreBF16> {
  using T = __nv_bfloat16;
  using C = float;
  static constexpr bool kShifted = true;
  static __device__ __forceinline__ C load(T v, C w) { return w + __bfloat162float(v); }
  static __device__ __forceinline__ T save(C f, C w) { return __float2bfloat16_rn(f - w); }
};

template <>
struct Store<kStoreF16> {
  using T = __half;
  using C = float;
  static constexpr bool kShifted = true;
  static __device__ __forceinline__ C load(T v, C w) { return w + __half2float(v); }
  static __device__ __forceinline__ T save(C f, C w) { return __float2half_rn(f - w); }
};

}  // namespace tlbm
