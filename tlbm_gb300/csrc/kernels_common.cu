// kernels_common.cu -- storage-generic kernels: initialisation, layout export, neighbour-table
// export, the deterministic FP64 mass reduction and the partition-order gather.
#include "grid.cuh"
#include "kernels.h"
#include "physics_ref.cuh"
#include "storage.cuh"

namespace tlbm {
namespace {

constexpr int kThreads = 256;

// grid-stride over all cells
#define TLBM_FOR_CELLS(c, n)                                                                \
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < (n);                 \
       c += (int64_t)gridDim.x * blockDim.x)

int blocks_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return static_cast<int>(b);
}

template <class L, int K>
__global__ void k_init_uniform(DevProblem pb, void* fv, double rho) {
  using S = Store<K>;
  using C = typename S::C;
  const size_t n = static_cast<size_t>(pb.n);
  auto* f = static_cast<typename S::P*>(fv);
  TLBM_FOR_CELLS(c, pb.n) {
    if constexpr (S::kMoment) {
      float fc[L::Q];
#pragma unroll
      for (int i = 0; i < L::Q; ++i) fc[i] = __fmul_rn(weight<L, float>(i), float(rho));
      moment::store<L>(fv, n, c, fc);
      continue;
    }
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      if constexpr (S::kShifted) {
        const C w = weight<L, float>(i);
        f[i * n + c] = S::save(w * static_cast<C>(rho), w);
      } else if constexpr (K == kStoreFX) {
        f[i * n + c] = S::save(weight<L, C>(i) * static_cast<C>(rho), C(0));
      } else if constexpr (!S::kMoment) {
        // w[spd]*rho in `real` (src/TLBM_Partition.cpp:462-463)
        f[i * n + c] = weight<L, C>(i) * static_cast<C>(rho);
      }
    }
  }
}

// restart: f = feq(u, rho) of each node (load_restart_data, src/TLBM_Partition.cpp:527-532),
// written to c - e_i so that the first pull returns it at node c
// the moment-shifted kind: the shift of slot s is formed from node s's own restart fields
template <class M>
__device__ __forceinline__ float4 restart_params(const M* ux, const M* uy, const M* uz,
                                                 const M* rho, int64_t s) {
  const float r = float(rho[s]);
  const float r3 = __fmul_rn(3.f, r);
  return make_float4(r, __fmul_rn(r3, float(ux[s])), __fmul_rn(r3, float(uy[s])),
                     __fmul_rn(r3, float(uz[s])));
}

template <class L, int K, class M>
__global__ void k_init_equilibrium(DevProblem pb, void* fv, const M* ux, const M* uy,
                                   const M* uz, const M* rho) {
  using S = Store<K>;
  using C = typename S::C;
  const size_t n = static_cast<size_t>(pb.n);
  auto* f = static_cast<typename S::P*>(fv);
  TLBM_FOR_CELLS(c, pb.n) {
    int x, y, z;
    decompose(static_cast<int>(c), pb.nx, pb.nxy, x, y, z);
    const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
    C feq[L::Q];
    ref::equilibrium<L, C>(static_cast<C>(ux[c]), static_cast<C>(uy[c]), static_cast<C>(uz[c]),
                           static_cast<C>(rho[c]), feq);
    if constexpr (S::kMoment) {
      moment::params(fv, L::Q, n)[c] = restart_params(ux, uy, uz, rho, c);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        const int s = nb.from<L>(i);
        const float sh = moment::shift<L>(i, restart_params(ux, uy, uz, rho, s));
        f[i * n + s] = __float2bfloat16_rn(__fsub_rn(feq[i], sh));
      }
    } else {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        const C w = S::kShifted ? weight<L, float>(i) : C(0);
        f[i * n + nb.from<L>(i)] = S::save(feq[i], w);
      }
    }
  }
}

template <class L, int K, class O>
__global__ void k_to_aos(DevProblem pb, const void* fv, int post_stream, O* out) {
  using S = Store<K>;
  using C = typename S::C;
  const size_t n = static_cast<size_t>(pb.n);
  const auto* f = static_cast<const typename S::P*>(fv);
  TLBM_FOR_CELLS(c, pb.n) {
    int x, y, z;
    decompose(static_cast<int>(c), pb.nx, pb.nxy, x, y, z);
    const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const int src = post_stream ? nb.from<L>(i) : static_cast<int>(c);
      if constexpr (S::kMoment) {
        out[c * L::Q + i] = static_cast<O>(
            moment::load<L>(f, moment::params(fv, L::Q, n), n, i, src));
      } else {
        const C w = S::kShifted ? weight<L, float>(i) : C(0);
        out[c * L::Q + i] = static_cast<O>(S::load(f[i * n + src], w));
      }
    }
  }
}

template <class L>
__global__ void k_adjacency(DevProblem pb, int32_t* out) {
  TLBM_FOR_CELLS(c, pb.n) {
    int x, y, z;
    decompose(static_cast<int>(c), pb.nx, pb.nxy, x, y, z);
    const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) out[c * L::Q + i] = nb.to<L>(i);
  }
}

// block-level deterministic double sum (fixed shuffle tree, fixed smem tree)
__device__ double block_sum(double v) {
  __shared__ double warp_part[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_part[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < kThreads / 32 ? warp_part[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

template <class L, int K>
__global__ void __launch_bounds__(kThreads) k_mass_partial(DevProblem pb, const void* fv,
                                                           double* partial) {
  using S = Store<K>;
  const size_t n = static_cast<size_t>(pb.n);
  const auto* f = static_cast<const typename S::P*>(fv);
  double acc = 0.0;
  TLBM_FOR_CELLS(c, pb.n) {
    double cell = 0.0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      if constexpr (S::kMoment)
        cell += static_cast<double>(moment::load<L>(f, moment::params(fv, L::Q, n), n, i, c));
      else if constexpr (S::kShifted)
        cell += static_cast<double>(weight<L, float>(i)) + static_cast<double>(f[i * n + c]);
      else if constexpr (K == kStoreFX)
        cell += S::load(f[i * n + c], 0.0);
      else
        cell += static_cast<double>(f[i * n + c]);
    }
    acc += cell;
  }
  const double b = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = b;
}

__global__ void __launch_bounds__(kThreads) k_mass_final(const double* partial, int nb,
                                                         double* out) {
  double acc = 0.0;
  for (int k = threadIdx.x; k < nb; k += kThreads) acc += partial[k];
  const double b = block_sum(acc);
  if (threadIdx.x == 0) *out = b;
}

template <class E>
__global__ void k_gather(const E* in, const int32_t* order, int64_t n, E* out) {
  TLBM_FOR_CELLS(k, n) out[k] = in[order[k]];
}

template <template <class, int> class Fn, class... A>
cudaError_t by_q_store(int q, int store, A&&... a) {
#define TLBM_CASE_K(QQ, KK) \
  if (q == QQ && store == KK) return Fn<Lattice<QQ>, KK>::run(a...);
  TLBM_CASE_K(15, kStoreF64) TLBM_CASE_K(15, kStoreF32) TLBM_CASE_K(15, kStoreBF16)
  TLBM_CASE_K(15, kStoreF16) TLBM_CASE_K(19, kStoreF64) TLBM_CASE_K(19, kStoreF32)
  TLBM_CASE_K(19, kStoreBF16) TLBM_CASE_K(19, kStoreF16) TLBM_CASE_K(27, kStoreF64)
  TLBM_CASE_K(27, kStoreF32) TLBM_CASE_K(27, kStoreBF16) TLBM_CASE_K(27, kStoreF16)
  TLBM_CASE_K(15, kStoreBF16M) TLBM_CASE_K(19, kStoreBF16M) TLBM_CASE_K(27, kStoreBF16M)
  TLBM_CASE_K(15, kStoreFX) TLBM_CASE_K(19, kStoreFX) TLBM_CASE_K(27, kStoreFX)
#undef TLBM_CASE_K
  return cudaErrorInvalidValue;
}

template <class L, int K>
struct InitUniform {
  static cudaError_t run(const DevProblem& pb, void* f, double rho, const Launch& l) {
    k_init_uniform<L, K><<<blocks_for(pb.n), kThreads, 0, l.stream>>>(pb, f, rho);
    return cudaGetLastError();
  }
};

template <class L, int K>
struct InitEq {
  static cudaError_t run(const DevProblem& pb, void* f, const void* const* m, int mb,
                         const Launch& l) {
    void* ff = f;
    if (mb == 8)
      k_init_equilibrium<L, K, double><<<blocks_for(pb.n), kThreads, 0, l.stream>>>(
          pb, ff, static_cast<const double*>(m[0]), static_cast<const double*>(m[1]),
          static_cast<const double*>(m[2]), static_cast<const double*>(m[3]));
    else
      k_init_equilibrium<L, K, float><<<blocks_for(pb.n), kThreads, 0, l.stream>>>(
          pb, ff, static_cast<const float*>(m[0]), static_cast<const float*>(m[1]),
          static_cast<const float*>(m[2]), static_cast<const float*>(m[3]));
    return cudaGetLastError();
  }
};

template <class L, int K>
struct ToAos {
  static cudaError_t run(const DevProblem& pb, const void* f, int post, void* out, int ob,
                         const Launch& l) {
    const void* ff = f;
    if (ob == 8)
      k_to_aos<L, K, double><<<blocks_for(pb.n), kThreads, 0, l.stream>>>(
          pb, ff, post, static_cast<double*>(out));
    else
      k_to_aos<L, K, float><<<blocks_for(pb.n), kThreads, 0, l.stream>>>(
          pb, ff, post, static_cast<float*>(out));
    return cudaGetLastError();
  }
};

template <class L, int K>
struct Mass {
  static cudaError_t run(const DevProblem& pb, const void* f, double* partial, int nb,
                         double* out, const Launch& l) {
    k_mass_partial<L, K><<<nb, kThreads, 0, l.stream>>>(pb, f, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_mass_final<<<1, kThreads, 0, l.stream>>>(partial, nb, out);
    return cudaGetLastError();
  }
};

}  // namespace

cudaError_t launch_init_uniform(int q, int store, const DevProblem& pb, void* f, double rho,
                                const Launch& l) {
  return by_q_store<InitUniform>(q, store, pb, f, rho, l);
}

cudaError_t launch_init_equilibrium(int q, int store, const DevProblem& pb, void* f,
                                    const void* const macro[4], int macro_bytes,
                                    const Launch& l) {
  return by_q_store<InitEq>(q, store, pb, f, macro, macro_bytes, l);
}

cudaError_t launch_to_aos(int q, int store, const DevProblem& pb, const void* f, int post_stream,
                          void* out, int out_bytes, const Launch& l) {
  return by_q_store<ToAos>(q, store, pb, f, post_stream, out, out_bytes, l);
}

cudaError_t launch_adjacency(int q, const DevProblem& pb, int32_t* out, const Launch& l) {
  const int b = blocks_for(pb.n);
  switch (q) {
    case 15: k_adjacency<Lattice<15>><<<b, kThreads, 0, l.stream>>>(pb, out); break;
    case 19: k_adjacency<Lattice<19>><<<b, kThreads, 0, l.stream>>>(pb, out); break;
    case 27: k_adjacency<Lattice<27>><<<b, kThreads, 0, l.stream>>>(pb, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int mass_blocks(const DevProblem& pb) { return blocks_for(pb.n); }

cudaError_t launch_mass(int q, int store, const DevProblem& pb, const void* f, double* partial,
                        int nblocks, double* out, const Launch& l) {
  return by_q_store<Mass>(q, store, pb, f, partial, nblocks, out, l);
}

struct CopyWords {
  const uint4* src[8];
  uint4* dst[8];
  int count;
  long long words;
};

__global__ void __launch_bounds__(256) k_copy_words(const CopyWords c) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const long long i0 = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (int k = 0; k < c.count; ++k) {
    const uint4* __restrict__ s = c.src[k];
    uint4* __restrict__ d = c.dst[k];
    for (long long i = i0; i < c.words; i += stride) d[i] = __ldg(s + i);
  }
}

cudaError_t launch_copy_words(const void* const* src, void* const* dst, int count, size_t bytes,
                              int blocks, const Launch& l) {
  if (count < 0 || count > 8 || bytes % 16 != 0 || blocks < 1) return cudaErrorInvalidValue;
  CopyWords c{};
  for (int k = 0; k < count; ++k) {
    if ((reinterpret_cast<uintptr_t>(src[k]) | reinterpret_cast<uintptr_t>(dst[k])) % 16 != 0)
      return cudaErrorInvalidValue;
    c.src[k] = static_cast<const uint4*>(src[k]);
    c.dst[k] = static_cast<uint4*>(dst[k]);
  }
  c.count = count;
  c.words = static_cast<long long>(bytes / 16);
  k_copy_words<<<blocks, 256, 0, l.stream>>>(c);
  return cudaGetLastError();
}

cudaError_t launch_gather(const void* in, const int32_t* order, int64_t n, int bytes, void* out,
                          const Launch& l) {
  const int b = blocks_for(n);
  if (bytes == 8)
    k_gather<double><<<b, kThreads, 0, l.stream>>>(static_cast<const double*>(in), order, n,
                                                  static_cast<double*>(out));
  else if (bytes == 4)
    k_gather<float><<<b, kThreads, 0, l.stream>>>(static_cast<const float*>(in), order, n,
                                                 static_cast<float*>(out));
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace tlbm
