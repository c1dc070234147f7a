// kernels_post.cu -- processTLBM.py on the device (python/processTLBM.py:52-186).
//
// processTLBM reads the float32 dump files, converts them to physical units in numpy float32
// arithmetic (every operand rounded to float32, every operation rounded once), puts them in
// global order and writes pressure - pRef, u, |u| and F.  The kernel below does the same
// operations in the same order with explicitly rounded intrinsics (no contraction into FMA),
// so its output is bit-identical to the script's on the same float32 inputs.
#include <cuda_runtime.h>

#include <cstdint>

#include "post.h"

namespace tlbm {
namespace {

constexpr int kThreads = 256;

template <class E>
__device__ __forceinline__ float as_f32(E v) {
  return static_cast<float>(v);  // double -> float: round to nearest
}

// p = rho * p_conv (processTLBM.py:86 / :159), after the division by Num_ts for time averages
template <class E>
__device__ __forceinline__ float pressure_of(E rho, const PostFactors& k) {
  float p = as_f32(rho);
  if (k.avg) p = __fdiv_rn(p, k.avg_div);  // pressure_i /= Num_ts (:153)
  return __fmul_rn(p, k.p_conv);
}

template <class E>
__device__ __forceinline__ float velocity_of(E u, const PostFactors& k) {
  float v = as_f32(u);
  if (k.avg) v = __fdiv_rn(v, k.avg_div);  // ux_i /= Num_ts (:150-152)
  return __fdiv_rn(v, k.u_conv);           // ux_i /= u_conv_fact (:83-85, :156-158)
}

// in: 7 fields (ux, uy, uz, rho, Fx, Fy, Fz; no forces for time averages) at input position i,
// scattered to global node order[i] (identity when order is null).  out: planes of n floats in
// the order of post.h, pressure in plane k.p_plane.
template <class E>
__global__ void k_post(PostInputs<E> in, const int32_t* order, int64_t n, int64_t p_ref_pos,
                       PostFactors k, float* out) {
  const float p_ref = pressure_of(in.rho[p_ref_pos], k);  // pRef = pressure[pRef_idx] (:95)
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = order ? static_cast<int64_t>(order[i]) : i;
    const float ux = velocity_of(in.ux[i], k);
    const float uy = velocity_of(in.uy[i], k);
    const float uz = velocity_of(in.uz[i], k);
    const float p = __fsub_rn(pressure_of(in.rho[i], k), p_ref);  // pressure -= pRef (:96)
    // velmag = sqrt(ux**2 + uy**2 + uz**2) (:98): three rounded squares, two rounded sums
    const float m = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)),
                                         __fmul_rn(uz, uz)));
    out[k.p_plane * n + g] = p;
    out[kPostUx * n + g] = ux;
    out[kPostUy * n + g] = uy;
    out[kPostUz * n + g] = uz;
    out[kPostVelmag * n + g] = m;
    if (in.fx) {  // Fx_i *= f_conv_fact (:107-109)
      out[kPostFx * n + g] = __fmul_rn(as_f32(in.fx[i]), k.f_conv);
      out[kPostFy * n + g] = __fmul_rn(as_f32(in.fy[i]), k.f_conv);
      out[kPostFz * n + g] = __fmul_rn(as_f32(in.fz[i]), k.f_conv);
    }
  }
}

int blocks_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : static_cast<int>(b);
}

}  // namespace

cudaError_t launch_post(const PostInputs<float>& in, const int32_t* order, int64_t n,
                        int64_t p_ref_pos, const PostFactors& k, float* out, cudaStream_t s) {
  k_post<float><<<blocks_for(n), kThreads, 0, s>>>(in, order, n, p_ref_pos, k, out);
  return cudaGetLastError();
}

cudaError_t launch_post(const PostInputs<double>& in, const int32_t* order, int64_t n,
                        int64_t p_ref_pos, const PostFactors& k, float* out, cudaStream_t s) {
  k_post<double><<<blocks_for(n), kThreads, 0, s>>>(in, order, n, p_ref_pos, k, out);
  return cudaGetLastError();
}

}  // namespace tlbm
