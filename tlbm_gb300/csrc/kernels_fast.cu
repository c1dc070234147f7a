// kernels_fast.cu -- the fused stream-collide step for throughput (FMA, reassociated sums).
//
// Same data flow as kernels_ref.cu -- one thread per cell, pull Q populations from c - e_i,
// node-type branch, collide in registers, store at c -- for every storage kind of
// storage.cuh.  Solid nodes move the raw stored values (bounce-back needs no arithmetic, and
// opposite speeds share a weight, so the f - w shift of 16-bit storage carries over unchanged).
#include "kernels.h"
#include "step_fast.cuh"

namespace tlbm {
namespace {

// (no minimum of resident blocks: stating one, even 1, changes ptxas's register budget, e.g.
// 64 -> 96 registers for the moment-shifted BF16 step, 15 % slower)
template <class L, int K, int kClosure, bool kReg>
__global__ void __launch_bounds__(128) k_step_fast(StepArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= a.pb.nx || y >= a.pb.ny) return;
  cell_step<L, K, kClosure, kReg>(a, x, y, z);
}

// 16-bit storage of f - w (BF16, FP16).  These steps are bound by memory latency (2-byte loads:
// few bytes in flight per thread), so they state one resident block as their minimum, which
// leaves ptxas a larger register budget to hoist loads (measured 45.5 against 42.0 GLUPS at
// the default budget); TLBM_TWO_CELLS_16 gives each thread two cells (step_fast.cuh:
// cell_step2), a block of (bx, by) threads covering 2 by rows, thread row ty taking rows ty and
// ty + by of the block's band.
#ifndef TLBM_TWO_CELLS_16
#define TLBM_TWO_CELLS_16 1
#endif
template <class L, int K, int kClosure>
__global__ void __launch_bounds__(128, 1) k_step_fast16(StepArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= a.pb.nx || y >= a.pb.ny) return;
  cell_step<L, K, kClosure, false>(a, x, y, z);
}

template <class L, int K, int kClosure, bool kReg>
__global__ void __launch_bounds__(128, 1) k_step_fast2(StepArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y0 = blockIdx.y * blockDim.y * 2 + threadIdx.y;
  const int y1 = y0 + blockDim.y;
  const int z = blockIdx.z;
  if (x >= a.pb.nx || y0 >= a.pb.ny) return;
  cell_step2<L, K, kClosure, kReg>(a, x, y0, y1 < a.pb.ny ? y1 : -1, z);
}

// 16-bit storage, cells in x pairs (step_fast.cuh: pair_step): thread (tx, ty) of a block of
// (bx, by) takes cells 2 (bx * blockIdx.x + tx) and the next of row by * blockIdx.y + ty.  For
// lattices with nx even and steps without time averaging.
#ifndef TLBM_PAIRS_16
#define TLBM_PAIRS_16 1
#endif
#ifndef TLBM_PAIR_MIN_BLOCKS
#define TLBM_PAIR_MIN_BLOCKS 1
#endif
template <class L, int K, int kClosure>
__global__ void __launch_bounds__(128, TLBM_PAIR_MIN_BLOCKS)
    k_step_pair16(const __grid_constant__ PairArgs pa) {
  const int x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= pa.a.pb.nx || y >= pa.a.pb.ny) return;
  pair_step<L, K, kClosure>(pa, x, y, blockIdx.z);
}

// FP64 storage with the fluid collision in exact fixed point (step_fast.cuh: cell_step_fx).  The
// parameter is a __grid_constant__, so the out-of-line FP64 cold path takes it by reference
// without a per-thread copy.  The kernel is bound by integer issue and dependent-latency stalls:
// more resident warps per SM hide more of the latency (D3Q27 holds more state: more blocks would
// spill).
#ifndef TLBM_FX_MIN_BLOCKS
#define TLBM_FX_MIN_BLOCKS 5
#endif
template <class L>
constexpr int kFxMinBlocks = L::Q == 27 ? 4 : TLBM_FX_MIN_BLOCKS;

template <class L, int K, int kClosure>
__global__ void __launch_bounds__(128, kFxMinBlocks<L>)
    k_step_fast_fx(const __grid_constant__ StepArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= a.pb.nx || y >= a.pb.ny) return;
  cell_step_fx<L, K, kClosure>(a, x, y, z);
}

// Q1.62 storage, plane bases in the parameters (step_fast.cuh: cell_step_fxp)
template <class L, int kClosure>
__global__ void __launch_bounds__(128, kFxMinBlocks<L>)
    k_step_fast_fxp(const __grid_constant__ FxArgs fa) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= fa.a.pb.nx || y >= fa.a.pb.ny) return;
  cell_step_fxp<L, kClosure>(fa, x, y, z);
}

// an opaque copy: the compiler cannot reuse values computed from v before this point
__device__ __forceinline__ void launder(float& v) { asm volatile("" : "+f"(v)); }
__device__ __forceinline__ void launder(double& v) { asm volatile("" : "+d"(v)); }

// Learned closure.  The network runs on the tensor cores, one warp (32 cells) at a time
// (mlp::forward_warp); the closure's description arrives by value in the kernel parameters.
// Every lane of a warp reaches the warp-collective part, which a warp without fluid cells
// skips.  Across the network only f, rho, u and Pi:Pi stay live (and Pi for the regularised
// collision); the pair terms of the equilibrium are recomputed after it.
#ifndef TLBM_MLP_MIN_BLOCKS
#define TLBM_MLP_MIN_BLOCKS 8  // resident blocks per SM: 64 registers per thread
#endif
template <int K>
constexpr int kMlpMinBlocks = (K == kStoreF64 || K == kStoreFX) ? 4 : TLBM_MLP_MIN_BLOCKS;

// One cell of the learned-closure step; all 32 lanes of the warp call it together (the network
// is warp-collective), lanes outside the lattice included.  kReg: regularised (moment-space)
// collision, which also needs the stress after the network.
template <class L, int K, bool kReg>
__device__ __forceinline__ void mlp_cell(const StepArgs& a, const mlp::Closure& cl,
                                         const mlp::MmaWeights& sw, mlp::WarpScratch& ws, int x,
                                         int y, int z, int lane) {
  using S = Store<K>;
  using C = typename S::C;
  const DevProblem& pb = a.pb;
  const bool in = x < pb.nx && y < pb.ny;
  const int c = x + y * pb.nx + z * pb.nxy;
  bool fluid = false;
  C f[L::Q];
  C rho = 0, ux = 0, uy = 0, uz = 0, q2 = 0;
  C pi[kReg ? 6 : 1];
  float xin[mlp::kIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (in) {
    typename S::T raw[L::Q];
    load_raw<L, K>(a, x, y, z, c, raw);
    const uint8_t t = pb.nd_type[c];
    if (t == kFluid) {
      fluid = true;
      unpack<L, K>(raw, f);
      fast::FluidPre<L, C> st;
      fast::fluid_pre<L, C, true>(f, st);
      rho = st.rho;
      ux = st.ux;
      uy = st.uy;
      uz = st.uz;
      q2 = st.q2;
      if constexpr (kReg) {
#pragma unroll
        for (int k = 0; k < 6; ++k) pi[k] = st.pi[k];
      }
      if (relaxes(pb)) fast::closure_inputs<L, C>(st, cl, xin);
    } else {
      if (pb.cs > 0)
        boundary_node<L, K, true, kReg>(a, x, y, c, t, raw, rho, ux, uy, uz);
      else
        boundary_node<L, K, false, kReg>(a, x, y, c, t, raw, rho, ux, uy, uz);
      if (a.time_avg) accumulate_avg<C>(a, c, rho, ux, uy, uz);
    }
  }
  __syncthreads();  // the network is in shared memory
  float net = 0.f;
  if (__any_sync(0xFFFFFFFFu, fluid && relaxes(pb)))
    net = mlp::forward_warp(sw, ws, xin, lane);
  if (!fluid) return;
  if (relaxes(pb)) {
    launder(ux);
    launder(uy);
    launder(uz);
    fast::FluidPre<L, C> st;
    st.rho = rho;
    st.ux = ux;
    st.uy = uy;
    st.uz = uz;
    fast::fluid_pair_terms<L, C>(st);
    const C omega = fast::closure_omega<C>(net, cl, Par<C>::omega(pb), Par<C>::cs(pb),
                                           Par<C>::nu(pb), q2);
    if constexpr (kReg) {
#pragma unroll
      for (int k = 0; k < 6; ++k) st.pi[k] = pi[k];
      fast::fluid_relax_moment<L, C>(f, st, omega, Par<C>::ghost_omega(pb));
    } else {
      fast::fluid_relax<L, C>(f, st, omega);
    }
  }
  store_cell<L, K>(a, c, f);
  if (a.time_avg) accumulate_avg<C>(a, c, rho, ux, uy, uz);
}

// The learned-closure step: one thread per cell like k_step_fast.  The block copies the network
// image to shared memory while its cells load, and waits for the copy only before the network.
template <class L, int K, bool kReg>
__global__ void __launch_bounds__(128, kMlpMinBlocks<K>)
    k_step_fast_mlp(StepArgs a, const mlp::Closure cl) {
  __shared__ mlp::MmaWeights sw;
  __shared__ mlp::WarpScratch ws[4];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  mlp::copy_mma_weights(cl.w, sw, tid, blockDim.x * blockDim.y);
  const int warp = tid >> 5, lane = tid & 31;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  mlp_cell<L, K, kReg>(a, cl, sw, ws[warp], x, y, blockIdx.z, lane);
}

template <class L, int K>
__global__ void __launch_bounds__(128) k_macros_fast(DevProblem pb,
                                                    const void* __restrict__ src,
                                                    typename Store<K>::C* ux_o,
                                                    typename Store<K>::C* uy_o,
                                                    typename Store<K>::C* uz_o,
                                                    typename Store<K>::C* rho_o) {
  using C = typename Store<K>::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= pb.nx || y >= pb.ny) return;
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  const int c = nb.self();
  typename Store<K>::T raw[L::Q];
  load_cell<L, K>(src, static_cast<size_t>(pb.n), nb, raw);
  const uint8_t t = pb.nd_type[c];
  if constexpr (K == kStoreFX) {
    // Q1.62 populations within the collision's ranges: density and momentum as its exact
    // integer pair sums, so a node costs four conversions to double and the division instead
    // of Q conversions and the FP64 sums; inlet and outlet nodes and states outside the
    // ranges (the stored NaN included) take the FP64 code below
    fx::i64 rq, jx, jy, jz;
    if (t != kInlet && t != kOutlet && fx::in_q62_ranges<L>(raw)) {
      fx::pair_moments<L>(raw, rq, jx, jy, jz);
      const double rho = fx::to_f64_59(rq);
      rho_o[c] = rho;
      if (t == kSolid) {
        ux_o[c] = uy_o[c] = uz_o[c] = 0.0;
      } else {
        const double inv = 1.0 / rho;
        ux_o[c] = fx::to_f64_59(jx) * inv;
        uy_o[c] = fx::to_f64_59(jy) * inv;
        uz_o[c] = fx::to_f64_59(jz) * inv;
      }
      return;
    }
  }
  C f[L::Q];
  unpack<L, K>(raw, f);
  C rho, ux, uy, uz;
  node_macros<L, C>(t, f, Par<C>::u_in(pb, c % pb.nxy), Par<C>::rho_bc(pb), rho, ux, uy, uz);
  ux_o[c] = ux;
  uy_o[c] = uy;
  uz_o[c] = uz;
  rho_o[c] = rho;
}

template <class L, int K>
__global__ void k_quirk_fast(DevProblem pb, const void* __restrict__ src,
                             typename Store<K>::C* uy_out) {
  using C = typename Store<K>::C;
  const int c = threadIdx.x;
  if (c >= L::Q || c >= pb.n) return;
  int x, y, z;
  decompose(c, pb.nx, pb.nxy, x, y, z);
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  typename Store<K>::T raw[L::Q];
  load_cell<L, K>(src, static_cast<size_t>(pb.n), nb, raw);
  C f[L::Q];
  unpack<L, K>(raw, f);
  C rho, ux, uy, uz;
  node_macros<L, C>(pb.nd_type[c], f, Par<C>::u_in(pb, c % pb.nxy), Par<C>::rho_bc(pb), rho, ux,
                    uy, uz);
  uy_out[c] = uy;
}

// The boundary-link sums of calc_force (src/TLBM_Partition.cpp:174-208) for solid node c, in the
// storage kind's arithmetic: the fluid neighbour g = c + e_i adds (f_i arriving at c + f_bb(i)
// arriving at g) e_bb(i), i.e. the stored values of speed i at c - e_i and of speed bb(i) at
// c + 2 e_i.
template <class L, int K>
__device__ __forceinline__ void force_links(const DevProblem& pb, const void* __restrict__ fv,
                                            const Nbr& nb, const Nbr2& n2,
                                            typename Store<K>::C& fx, typename Store<K>::C& fy,
                                            typename Store<K>::C& fz) {
  using S = Store<K>;
  using C = typename S::C;
  const size_t n = static_cast<size_t>(pb.n);
  const auto* f = static_cast<const typename S::P*>(fv);
  // post-stream value of speed i at cell d: the slot (i, from) of the buffer
  auto pulled = [&](int i, int from) -> C {
    if constexpr (S::kMoment)
      return moment::load<L>(f, moment::params(fv, L::Q, n), n, i, from);
    else
      return S::load(f[i * n + from], fast::wgt<L, C>(i));
  };
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    if (pb.nd_type[nb.to<L>(i)] != kFluid) continue;
    const int b = L::bb(i);
    const C s = pulled(i, nb.from<L>(i)) + pulled(b, n2.to2<L>(nb, i));
    fx += C(L::ex(b)) * s;
    fy += C(L::ey(b)) * s;
    fz += C(L::ez(b)) * s;
  }
}

template <class L, int K>
__global__ void __launch_bounds__(128) k_force_fast(DevProblem pb,
                                                   const void* __restrict__ fv,
                                                   typename Store<K>::C* fx_o,
                                                   typename Store<K>::C* fy_o,
                                                   typename Store<K>::C* fz_o) {
  using C = typename Store<K>::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= pb.nx || y >= pb.ny) return;
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  const int c = nb.self();
  C fx = 0, fy = 0, fz = 0;
  if (pb.nd_type[c] == kSolid)
    force_links<L, K>(pb, fv, nb, Nbr2(nb, pb.nx, pb.ny, pb.nz, pb.nxy), fx, fy, fz);
  fx_o[c] = fx;
  fy_o[c] = fy;
  fz_o[c] = fz;
}

// the FP64 sums for a Q1.62 node the integer sums do not take (out of line: rare, and kept out
// of the integer kernel's register allocation)
template <class L>
__device__ __noinline__ void force_links_f64(const DevProblem& pb, const void* fv, const Nbr& nb,
                                             const Nbr2& n2, double& fx, double& fy, double& fz) {
  force_links<L, kStoreFX>(pb, fv, nb, n2, fx, fy, fz);
}

// Q1.62 storage: the link sums accumulate as integers (each value rounded once to 2^-58; Q5.58
// holds the 2 (Q - 1) values in [-1/2, 1/2) a node can gather), three conversions per node.  The
// work sits in the warps that hold solid surface nodes and is bound by load latency: 64 registers
// (eight resident blocks per SM, against three at the 138 the same sums took with the FP64
// fallback inline) and predicated loads that issue without waiting on each link's type test.  A
// value outside the range (the stored NaN included) sends the node to the FP64 sums.
template <class L>
__global__ void __launch_bounds__(128, 8) k_force_fx(const __grid_constant__ DevProblem pb,
                                                      const fx::i64* __restrict__ f,
                                                      double* fx_o, double* fy_o, double* fz_o) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= pb.nx || y >= pb.ny) return;
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  const int c = nb.self();
  double fx = 0, fy = 0, fz = 0;
  if (pb.nd_type[c] == kSolid) {
    const Nbr2 n2(nb, pb.nx, pb.ny, pb.nz, pb.nxy);
    const size_t n = static_cast<size_t>(pb.n);
    fx::i64 ax = 0, ay = 0, az = 0;
    unsigned out = 0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {  // a non-link adds zero
      const int b = L::bb(i);
      const bool link = pb.nd_type[nb.to<L>(i)] == kFluid;
      const fx::i64 v1 = link ? __ldg(f + i * n + nb.from<L>(i)) : 0;
      const fx::i64 v2 = link ? __ldg(f + b * n + n2.to2<L>(nb, i)) : 0;
      out |= fx::beyond_half(v1) | fx::beyond_half(v2);
      const fx::i64 s = fx::to58(v1) + fx::to58(v2);
      if (L::ex(b) > 0) ax += s;
      if (L::ex(b) < 0) ax -= s;
      if (L::ey(b) > 0) ay += s;
      if (L::ey(b) < 0) ay -= s;
      if (L::ez(b) > 0) az += s;
      if (L::ez(b) < 0) az -= s;
    }
    if (out == 0) {
      fx = fx::to_f64_58(ax);
      fy = fx::to_f64_58(ay);
      fz = fx::to_f64_58(az);
    } else {
      force_links_f64<L>(pb, f, nb, n2, fx, fy, fz);
    }
  }
  fx_o[c] = fx;
  fy_o[c] = fy;
  fz_o[c] = fz;
}

dim3 grid_of(const DevProblem& pb, const Launch& l) {
  return dim3((pb.nx + l.bx - 1) / l.bx, (pb.ny + l.by - 1) / l.by, pb.nz);
}

template <class L, int K>
cudaError_t step_lk(const StepArgs& a, const Launch& l) {
  const dim3 g = grid_of(a.pb, l), b(l.bx, l.by, 1);
  if (a.closure) {
    const mlp::Closure& cl = *static_cast<const mlp::Closure*>(a.closure);
    if (a.pb.mcoll)
      k_step_fast_mlp<L, K, true><<<g, b, 0, l.stream>>>(a, cl);
    else
      k_step_fast_mlp<L, K, false><<<g, b, 0, l.stream>>>(a, cl);
  } else if ((K == kStoreF64 || K == kStoreFX) && a.pb.fx && !a.pb.mcoll) {
    // FP64 storage (double or Q1.62): fluid nodes in exact fixed point (physics_fx.cuh)
    if constexpr (K == kStoreFX) {
      FxArgs fa{};
      fa.a = a;
      const size_t n = static_cast<size_t>(a.pb.n);
      for (int i = 0; i < L::Q; ++i) {
        fa.src[i] = static_cast<const fx::i64*>(a.src) + i * n;
        fa.dst[i] = static_cast<fx::i64*>(a.dst) + i * n;
      }
      if (a.pb.cs > 0)
        k_step_fast_fxp<L, fast::kClosureSmag><<<g, b, 0, l.stream>>>(fa);
      else
        k_step_fast_fxp<L, fast::kClosureNone><<<g, b, 0, l.stream>>>(fa);
    } else if constexpr (K == kStoreF64) {
      if (a.pb.cs > 0)
        k_step_fast_fx<L, K, fast::kClosureSmag><<<g, b, 0, l.stream>>>(a);
      else
        k_step_fast_fx<L, K, fast::kClosureNone><<<g, b, 0, l.stream>>>(a);
    }
  } else if ((K == kStoreBF16 || K == kStoreF16) && !a.pb.mcoll) {
    // 16-bit storage of f - w
    if constexpr (K == kStoreBF16 || K == kStoreF16) {
      if (TLBM_PAIRS_16 && a.pb.nx % 2 == 0 && !a.time_avg) {
        // a block row of bx pairs spans 2 bx cells: narrower blocks for narrow lattices
        int bx = l.bx;
        while (bx > 16 && 2 * bx > a.pb.nx) bx /= 2;
        const int by = (l.bx * l.by) / bx;
        const dim3 gp((a.pb.nx / 2 + bx - 1) / bx, (a.pb.ny + by - 1) / by, a.pb.nz),
            bp(bx, by, 1);
        PairArgs pa{};
        pa.a = a;
        const size_t words = static_cast<size_t>(a.pb.n) / 2;  // of one population plane
        for (int i = 0; i < L::Q; ++i) {
          pa.src[i] = static_cast<const uint32_t*>(a.src) + i * words;
          pa.dst[i] = static_cast<uint32_t*>(a.dst) + i * words;
        }
        if (a.pb.cs > 0)
          k_step_pair16<L, K, fast::kClosureSmag><<<gp, bp, 0, l.stream>>>(pa);
        else
          k_step_pair16<L, K, fast::kClosureNone><<<gp, bp, 0, l.stream>>>(pa);
      } else if (TLBM_TWO_CELLS_16) {
        const dim3 g2(g.x, (a.pb.ny + 2 * l.by - 1) / (2 * l.by), g.z);
        if (a.pb.cs > 0)
          k_step_fast2<L, K, fast::kClosureSmag, false><<<g2, b, 0, l.stream>>>(a);
        else
          k_step_fast2<L, K, fast::kClosureNone, false><<<g2, b, 0, l.stream>>>(a);
      } else if (a.pb.cs > 0) {
        k_step_fast16<L, K, fast::kClosureSmag><<<g, b, 0, l.stream>>>(a);
      } else {
        k_step_fast16<L, K, fast::kClosureNone><<<g, b, 0, l.stream>>>(a);
      }
    }
  } else if (a.pb.cs > 0 && a.pb.mcoll)
    k_step_fast<L, K, fast::kClosureSmag, true><<<g, b, 0, l.stream>>>(a);
  else if (a.pb.cs > 0)
    k_step_fast<L, K, fast::kClosureSmag, false><<<g, b, 0, l.stream>>>(a);
  else if (a.pb.mcoll)
    k_step_fast<L, K, fast::kClosureNone, true><<<g, b, 0, l.stream>>>(a);
  else
    k_step_fast<L, K, fast::kClosureNone, false><<<g, b, 0, l.stream>>>(a);
  return cudaGetLastError();
}

template <class L, int K>
cudaError_t macros_lk(const DevProblem& pb, const void* src, void* const out[4], const Launch& l) {
  using C = typename Store<K>::C;
  const dim3 g = grid_of(pb, l), b(l.bx, l.by, 1);
  k_macros_fast<L, K><<<g, b, 0, l.stream>>>(
      pb, src, static_cast<C*>(out[0]),
      static_cast<C*>(out[1]), static_cast<C*>(out[2]), static_cast<C*>(out[3]));
  return cudaGetLastError();
}

template <class L, int K>
cudaError_t quirk_lk(const DevProblem& pb, const void* src, void* out, const Launch& l) {
  using C = typename Store<K>::C;
  k_quirk_fast<L, K><<<1, 32, 0, l.stream>>>(pb, src,
                                              static_cast<C*>(out));
  return cudaGetLastError();
}

template <class L, int K>
cudaError_t force_lk(const DevProblem& pb, const void* f, void* const out[3], const Launch& l) {
  using C = typename Store<K>::C;
  const dim3 g = grid_of(pb, l), b(l.bx, l.by, 1);
  if constexpr (K == kStoreFX)
    k_force_fx<L><<<g, b, 0, l.stream>>>(pb, static_cast<const fx::i64*>(f),
                                         static_cast<C*>(out[0]), static_cast<C*>(out[1]),
                                         static_cast<C*>(out[2]));
  else
    k_force_fast<L, K><<<g, b, 0, l.stream>>>(pb, f, static_cast<C*>(out[0]),
                                               static_cast<C*>(out[1]), static_cast<C*>(out[2]));
  return cudaGetLastError();
}

#define TLBM_DISPATCH(FN, q, store, ...)                                            \
  do {                                                                              \
    switch (q * 10 + store) {                                                       \
      case 150: return FN<Lattice<15>, kStoreF64>(__VA_ARGS__);                     \
      case 151: return FN<Lattice<15>, kStoreF32>(__VA_ARGS__);                     \
      case 152: return FN<Lattice<15>, kStoreBF16>(__VA_ARGS__);                    \
      case 153: return FN<Lattice<15>, kStoreF16>(__VA_ARGS__);                     \
      case 190: return FN<Lattice<19>, kStoreF64>(__VA_ARGS__);                     \
      case 191: return FN<Lattice<19>, kStoreF32>(__VA_ARGS__);                     \
      case 192: return FN<Lattice<19>, kStoreBF16>(__VA_ARGS__);                    \
      case 193: return FN<Lattice<19>, kStoreF16>(__VA_ARGS__);                     \
      case 270: return FN<Lattice<27>, kStoreF64>(__VA_ARGS__);                     \
      case 271: return FN<Lattice<27>, kStoreF32>(__VA_ARGS__);                     \
      case 272: return FN<Lattice<27>, kStoreBF16>(__VA_ARGS__);                    \
      case 273: return FN<Lattice<27>, kStoreF16>(__VA_ARGS__);                     \
      case 154: return FN<Lattice<15>, kStoreBF16M>(__VA_ARGS__);                   \
      case 194: return FN<Lattice<19>, kStoreBF16M>(__VA_ARGS__);                   \
      case 274: return FN<Lattice<27>, kStoreBF16M>(__VA_ARGS__);                   \
      case 155: return FN<Lattice<15>, kStoreFX>(__VA_ARGS__);                      \
      case 195: return FN<Lattice<19>, kStoreFX>(__VA_ARGS__);                      \
      case 275: return FN<Lattice<27>, kStoreFX>(__VA_ARGS__);                      \
      default: return cudaErrorInvalidValue;                                        \
    }                                                                               \
  } while (0)

}  // namespace

cudaError_t launch_step_fast(int q, int store, const StepArgs& a, const Launch& l) {
  if (a.pb.has_type5) {
    cudaError_t e = [&]() -> cudaError_t {
      TLBM_DISPATCH(quirk_lk, q, store, a.pb, a.src, const_cast<void*>(a.uyq_cur), l);
    }();
    if (e != cudaSuccess) return e;
  }
  TLBM_DISPATCH(step_lk, q, store, a, l);
}

cudaError_t launch_macros_fast(int q, int store, const DevProblem& pb, const void* src,
                               void* const out[4], const Launch& l) {
  TLBM_DISPATCH(macros_lk, q, store, pb, src, out, l);
}

cudaError_t launch_force_fast(int q, int store, const DevProblem& pb, const void* dst,
                              void* const out[3], const Launch& l) {
  TLBM_DISPATCH(force_lk, q, store, pb, dst, out, l);
}

}  // namespace tlbm
