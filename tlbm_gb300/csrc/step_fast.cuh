// step_fast.cuh -- one cell of the fused stream-collide step in fast arithmetic.
//
// Shared by the single-lattice kernel (kernels_fast.cu) and the batched-ensemble kernel
// (kernels_ensemble.cu), so both compute every cell with the same instructions.  The cell
// pulls its Q populations from c - e_i (periodic), branches on its node type, collides in
// registers and stores at c:
//   fluid        -> pair-form BGK / Smagorinsky, optionally regularised (physics_fast.cuh:
//                   fluid_collide)
//   solid        -> bounce-back of the raw stored values, no collision
//   inlet/outlet -> the reference's density/velocity rule, non-equilibrium bounce-back of the
//                   unknown speeds, then BGK / Smagorinsky
//   moving wall  -> the reference's set_uz_bc nudge (uy of node number i, see physics_ref.cuh)
#pragma once

#include "kernels.h"
#include "physics_fast.cuh"
#include "storage.cuh"

namespace tlbm {

// the Q values a cell pulls from the buffer `src` (the moment-shifted kind: reconstructed)
template <class L, int K>
__device__ __forceinline__ void load_cell(const void* __restrict__ src, size_t n, const Nbr& nb,
                                          typename Store<K>::T (&raw)[L::Q]) {
  using S = Store<K>;
  const auto* p = static_cast<const typename S::P*>(src);
  if constexpr (S::kMoment) {
    const float4* prm = moment::params(src, L::Q, n);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) raw[i] = moment::load<L>(p, prm, n, i, nb.from<L>(i));
  } else {
#pragma unroll
    for (int i = 0; i < L::Q; ++i) raw[i] = __ldg(p + i * n + nb.from<L>(i));
  }
}

template <class L, int K>
__device__ __forceinline__ void unpack(const typename Store<K>::T (&raw)[L::Q],
                                       typename Store<K>::C (&f)[L::Q]) {
  using S = Store<K>;
  using C = typename S::C;
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = S::load(raw[i], fast::wgt<L, C>(i));
}

// node macroscopic values as the reference holds them after processing the node
template <class L, class C>
__device__ __forceinline__ void node_macros(uint8_t t, const C (&f)[L::Q], C u_bc, C rho_bc,
                                            C& rho, C& ux, C& uy, C& uz) {
  if (t == kSolid) {
    rho = fast::density<L, C>(f);
    ux = uy = uz = C(0);
  } else if (t == kInlet) {
    rho = fast::inlet_rho<L, C>(f, C(1) / (C(1) - u_bc));
    ux = uy = C(0);
    uz = u_bc;
  } else {
    fast::moments<L, C>(f, rho, ux, uy, uz);
    if (t == kOutlet) {
      rho = rho_bc;
      uz = fast::outlet_uz<L, C>(f, C(1) / rho_bc);
    }
  }
}

// the Q stored values cell c pulls (from c - e_i, periodic).  kWrapFree: cells on the x and y
// edges of a plane take the interior path too, their wrap folded into the offsets by selects
// (no divergent second path in the warps that hold an x edge: every warp of a narrow lattice);
// z-edge planes, uniform across a warp, and planes whose byte size does not fit the 32-bit
// offsets keep the neighbour-table path.  Same values either way.
template <class L, int K, bool kWrapFree = true>
__device__ __forceinline__ void load_raw(const StepArgs& a, int x, int y, int z, int c,
                                         typename Store<K>::T (&raw)[L::Q]) {
  using S = Store<K>;
  using P = typename S::P;
  const DevProblem& pb = a.pb;
  const P* __restrict__ src = static_cast<const P*>(a.src);
  if constexpr (kWrapFree && !S::kMoment) {
    constexpr int kMaxPlane = 0x7FFFFFFF / static_cast<int>(sizeof(P));
    if (z > 0 && z < pb.nz - 1 && pb.nxy <= kMaxPlane - pb.nx) {  // |wx + wy| fits an int
      // speed i pulls from x - ex_i: from the far edge when that leaves the plane
      constexpr int b = static_cast<int>(sizeof(P));
      const int wx_pos = x == 0 ? pb.nx * b : 0;               // ex > 0 at x = 0
      const int wx_neg = x == pb.nx - 1 ? -pb.nx * b : 0;      // ex < 0 at x = nx - 1
      const int wy_pos = y == 0 ? pb.nxy * b : 0;              // ey > 0 at y = 0
      const int wy_neg = y == pb.ny - 1 ? -pb.nxy * b : 0;     // ey < 0 at y = ny - 1
      const char* base = reinterpret_cast<const char*>(src + c);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        const int ex = L::ex(i), ey = L::ey(i);
        const int w = (ex > 0 ? wx_pos : (ex < 0 ? wx_neg : 0)) +
                      (ey > 0 ? wy_pos : (ey < 0 ? wy_neg : 0));
        raw[i] = __ldg(reinterpret_cast<const P*>(base + pb.pull_off[i] + w));
      }
      return;
    }
  }
  if (x > 0 && x < pb.nx - 1 && y > 0 && y < pb.ny - 1 && z > 0 && z < pb.nz - 1) {
    // interior cell: speed i comes from a fixed byte offset of the cell's own slot
    const char* base = reinterpret_cast<const char*>(src + c);
    if constexpr (S::kMoment) {
      // and its shift from the float4 of the cell it comes from, c - e_i
      const float4* prm = moment::params(a.src, L::Q, static_cast<size_t>(pb.n)) + c;
#pragma unroll
      for (int i = 0; i < L::Q; ++i)
        raw[i] = __fadd_rn(
            moment::shift<L>(i, __ldg(prm - pb.pull_cell[i])),
            __bfloat162float(__ldg(reinterpret_cast<const P*>(base + pb.pull_off[i]))));
    } else {
#pragma unroll
      for (int i = 0; i < L::Q; ++i)
        raw[i] = __ldg(reinterpret_cast<const P*>(base + pb.pull_off[i]));
    }
  } else {
    const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
    load_cell<L, K>(a.src, static_cast<size_t>(pb.n), nb, raw);
  }
}

template <class L, int K>
__device__ __forceinline__ void store_cell(const StepArgs& a, int c,
                                           const typename Store<K>::C (&f)[L::Q]) {
  using S = Store<K>;
  using C = typename S::C;
  const size_t n = static_cast<size_t>(a.pb.n);
  if constexpr (S::kMoment) {
    moment::store<L>(a.dst, n, c, f);
  } else {
    typename S::P* __restrict__ dst = static_cast<typename S::P*>(a.dst);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) dst[i * n + c] = S::save(f[i], fast::wgt<L, C>(i));
  }
}

// every node type but fluid: solid bounce-back, inlet/outlet reconstruction and relaxation,
// the moving-wall nudge.  kSmag: boundary nodes relax at the Smagorinsky rate; kReg: with the
// moment-space collision.
template <class L, int K, bool kSmag, bool kReg>
__device__ __forceinline__ void boundary_node(const StepArgs& a, int x, int y, int c, uint8_t t,
                                              const typename Store<K>::T (&raw)[L::Q],
                                              typename Store<K>::C& rho,
                                              typename Store<K>::C& ux,
                                              typename Store<K>::C& uy,
                                              typename Store<K>::C& uz) {
  using S = Store<K>;
  using C = typename S::C;
  const DevProblem& pb = a.pb;
  if (t == kSolid) {
    if constexpr (S::kMoment) {
      float sw[L::Q];
#pragma unroll
      for (int i = 0; i < L::Q; ++i) sw[i] = raw[L::bb(i)];
      store_cell<L, K>(a, c, sw);
    } else {
      typename S::P* __restrict__ dst = static_cast<typename S::P*>(a.dst);
      const size_t n = static_cast<size_t>(pb.n);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) dst[i * n + c] = raw[L::bb(i)];
    }
    if (a.time_avg) {
      C f[L::Q];
      unpack<L, K>(raw, f);
      rho = fast::density<L, C>(f);
    }
    return;
  }
  C f[L::Q];
  unpack<L, K>(raw, f);
  const C u_bc = (t == kInlet) ? Par<C>::u_in(pb, x + y * pb.nx) : Par<C>::u_bc(pb);
  node_macros<L, C>(t, f, u_bc, Par<C>::rho_bc(pb), rho, ux, uy, uz);
  if constexpr (S::kShifted) {
    // 16-bit storage: the inlet density and outlet velocity sums are taken in FP64
    if (t == kInlet || t == kOutlet) {
      double fd[L::Q];
#pragma unroll
      for (int i = 0; i < L::Q; ++i)
        fd[i] = static_cast<double>(fast::wgt<L, float>(i)) +
                static_cast<double>(S::load(raw[i], 0.0f));
      if (t == kInlet)
        rho = static_cast<C>(fast::inlet_rho<L, double>(
            fd, 1.0 / (1.0 - Par<double>::u_in(pb, x + y * pb.nx))));
      else
        uz = static_cast<C>(fast::outlet_uz<L, double>(fd, 1.0 / pb.rho_bc));
    }
  }
  if (pb.has_type5 && t == kMovingWall) {
    const C* cur = static_cast<const C*>(a.uyq_cur);
    const C* prev = static_cast<const C*>(a.uyq_prev);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const C uyq = i <= c ? cur[i] : prev[i];
      f[i] += C(3) * rho * fast::wgt<L, C>(i) *
              (C(L::ez(i)) * (u_bc - uz) - C(L::ex(i)) * ux - C(L::ey(i)) * uyq);
    }
  }
  C feq[L::Q];
  fast::equilibrium<L, C>(rho, ux, uy, uz, feq);
  if (t == kInlet) fast::nebb<L, C, true>(f, feq);
  if (t == kOutlet) fast::nebb<L, C, false>(f, feq);
  if (relaxes(pb)) {
    C om = Par<C>::omega(pb);
    if (kSmag) om = fast::smagorinsky_omega<L, C>(f, feq, Par<C>::cs(pb), Par<C>::nu(pb));
    if constexpr (kReg)
      fast::relax_moment<L, C>(f, feq, om, Par<C>::ghost_omega(pb));
    else
      fast::relax<L, C>(f, feq, om);
  }
  store_cell<L, K>(a, c, f);
}

template <class C>
__device__ __forceinline__ void accumulate_avg(const StepArgs& a, int c, C rho, C ux, C uy,
                                               C uz) {
  C* const* avg = reinterpret_cast<C* const*>(a.avg);
  avg[0][c] += ux;
  avg[1][c] += uy;
  avg[2][c] += uz;
  avg[3][c] += rho;
}

// kClosure: fast::kClosureNone (BGK) or kClosureSmag (the learned closure has its own kernel,
// kernels_fast.cu: k_step_fast_mlp); kReg: the moment-space collision (RBGK / MRT);
// kWrapFree: load_raw's branch-free x/y wrap; kFx: FP64 storage with the fixed-point fluid
// collision (the FP64 code remains for nodes outside its ranges and for boundary nodes)
template <class L, int K, int kClosure, bool kReg = false, bool kWrapFree = true,
          bool kFx = false>
__device__ __forceinline__ void cell_step(const StepArgs& a, int x, int y, int z);

// FP64 storage (double or Q1.62), the FP64 code for one cell, out of line: the fixed-point
// kernel sends here the nodes its hot path does not take (boundary nodes, fluid nodes outside
// the fixed-point ranges, runs that accumulate time averages), which reload their populations.
template <class L, int K, int kClosure>
__device__ __noinline__ void cell_step_f64_cold(const StepArgs& a, int x, int y, int z) {
  cell_step<L, K, kClosure, false, true, false>(a, x, y, z);
}

// FP64 storage with the fluid collision in exact fixed point (physics_fx.cuh): solid nodes swap
// and fluid nodes collide here; everything else goes to cell_step_f64_cold.  With Q1.62 storage
// (kStoreFX) the populations move between HBM and the collision as they are; with double
// storage each converts exactly in and to the nearest double out.  The hot path holds no FP64
// arithmetic, so it stays small for the instruction cache.
template <class L, int K, int kClosure>
__device__ __forceinline__ void cell_step_fx(const StepArgs& a, int x, int y, int z) {
  using T = typename Store<K>::T;
  const DevProblem& pb = a.pb;
  const int c = x + y * pb.nx + z * pb.nxy;
  T f[L::Q];
  load_raw<L, K, true>(a, x, y, z, c, f);
  const uint8_t t = pb.nd_type[c];
  if (!a.time_avg && pb.fx) {
    T* __restrict__ dst = static_cast<T*>(a.dst);
    const size_t n = static_cast<size_t>(pb.n);
    if (t == kSolid) {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) dst[i * n + c] = f[L::bb(i)];
      return;
    }
    fx::i64 rq, jq[3];
    if (t == kFluid && relaxes(pb) &&
        fx::fluid_collide<L, kClosure == fast::kClosureSmag>(f, pb.fxk, rq, jq)) {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) dst[i * n + c] = f[i];
      return;
    }
  }
  cell_step_f64_cold<L, K, kClosure>(a, x, y, z);
}

// The same step for Q1.62 storage with each population plane's first element in the kernel
// parameters (as the x-pair step): a load or store address is one multiply-add of a 32-bit cell
// index onto a parameter, where the one-buffer form adds a 64-bit byte offset per speed.
struct FxArgs {
  StepArgs a;
  const fx::i64* src[27];
  fx::i64* dst[27];
};

template <class L, int kClosure>
__device__ __forceinline__ void cell_step_fxp(const FxArgs& fa, int x, int y, int z) {
  const StepArgs& a = fa.a;
  const DevProblem& pb = a.pb;
  const int c = x + y * pb.nx + z * pb.nxy;
  fx::i64 f[L::Q];
  if (z > 0 && z < pb.nz - 1) {
    // speed i pulls from c - e_i; across an x or y edge from the far side of the plane
    const int wx_pos = x == 0 ? pb.nx : 0, wx_neg = x == pb.nx - 1 ? -pb.nx : 0;
    const int wy_pos = y == 0 ? pb.nxy : 0, wy_neg = y == pb.ny - 1 ? -pb.nxy : 0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const int ex = L::ex(i), ey = L::ey(i);
      const int w = (ex > 0 ? wx_pos : (ex < 0 ? wx_neg : 0)) +
                    (ey > 0 ? wy_pos : (ey < 0 ? wy_neg : 0));
      f[i] = __ldg(fa.src[i] + static_cast<unsigned>(c - pb.pull_cell[i] + w));
    }
  } else {
    const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) f[i] = __ldg(fa.src[i] + static_cast<unsigned>(nb.from<L>(i)));
  }
  const uint8_t t = pb.nd_type[c];
  if (!a.time_avg && pb.fx) {
    const unsigned cu = static_cast<unsigned>(c);
    if (t == kSolid) {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) fa.dst[i][cu] = f[L::bb(i)];
      return;
    }
    fx::i64 rq, jq[3];
    if (t == kFluid && relaxes(pb) &&
        fx::fluid_collide<L, kClosure == fast::kClosureSmag>(f, pb.fxk, rq, jq)) {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) fa.dst[i][cu] = f[i];
      return;
    }
  }
  cell_step_f64_cold<L, kStoreFX, kClosure>(a, x, y, z);
}

// the part of cell_step after the loads: node-type branch, collision, store
template <class L, int K, int kClosure, bool kReg>
__device__ __forceinline__ void cell_compute(const StepArgs& a, int x, int y, int c, uint8_t t,
                                             const typename Store<K>::T (&raw)[L::Q]) {
  using S = Store<K>;
  using C = typename S::C;
  const DevProblem& pb = a.pb;
  C rho = 0, ux = 0, uy = 0, uz = 0;
  if (t == kFluid) {
    if constexpr (S::kShifted && !kReg) {
      // 16-bit storage of f - w: collide the stored shifts themselves
      float d[L::Q];
#pragma unroll
      for (int i = 0; i < L::Q; ++i) d[i] = S::shift_of(raw[i]);
      fast::fluid_collide_shifted<L, kClosure>(d, Par<C>::omega(pb), Par<C>::cs(pb),
                                               Par<C>::nu(pb), relaxes(pb), rho, ux, uy, uz);
      typename S::P* __restrict__ dst = static_cast<typename S::P*>(a.dst);
      const size_t n = static_cast<size_t>(pb.n);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) dst[i * n + c] = S::of_shift(d[i]);
    } else {
      C f[L::Q];
      unpack<L, K>(raw, f);
      fast::fluid_collide<L, C, kClosure, kReg>(f, Par<C>::omega(pb), Par<C>::cs(pb),
                                                Par<C>::nu(pb), Par<C>::ghost_omega(pb),
                                                relaxes(pb), rho, ux, uy, uz);
      store_cell<L, K>(a, c, f);
    }
  } else {
    boundary_node<L, K, kClosure == fast::kClosureSmag, kReg>(a, x, y, c, t, raw, rho, ux, uy,
                                                              uz);
  }
  if (a.time_avg) accumulate_avg<C>(a, c, rho, ux, uy, uz);
}

template <class L, int K, int kClosure, bool kReg, bool kWrapFree, bool kFx>
__device__ __forceinline__ void cell_step(const StepArgs& a, int x, int y, int z) {
  if constexpr (kFx && (K == kStoreF64 || K == kStoreFX) && !kReg) {
    cell_step_fx<L, K, kClosure>(a, x, y, z);
  } else {
    const DevProblem& pb = a.pb;
    const int c = x + y * pb.nx + z * pb.nxy;
    typename Store<K>::T raw[L::Q];
    load_raw<L, K, kWrapFree>(a, x, y, z, c, raw);
    cell_compute<L, K, kClosure, kReg>(a, x, y, c, pb.nd_type[c], raw);
  }
}

// Two cells per thread, rows y0 and y1 of one x column: both cells' loads are issued before
// either is computed, so a thread keeps twice the bytes in flight (the 16-bit kinds move only
// 2 bytes per load and are otherwise bound by memory latency).  y1 < 0: one cell.
template <class L, int K, int kClosure, bool kReg>
__device__ __forceinline__ void cell_step2(const StepArgs& a, int x, int y0, int y1, int z) {
  const DevProblem& pb = a.pb;
  const int c0 = x + y0 * pb.nx + z * pb.nxy;
  typename Store<K>::T r0[L::Q];
  load_raw<L, K, true>(a, x, y0, z, c0, r0);
  const uint8_t t0 = pb.nd_type[c0];
  if (y1 < 0) {
    cell_compute<L, K, kClosure, kReg>(a, x, y0, c0, t0, r0);
    return;
  }
  const int c1 = x + y1 * pb.nx + z * pb.nxy;
  typename Store<K>::T r1[L::Q];
  load_raw<L, K, true>(a, x, y1, z, c1, r1);
  const uint8_t t1 = pb.nd_type[c1];
  cell_compute<L, K, kClosure, kReg>(a, x, y0, c0, t0, r0);
  cell_compute<L, K, kClosure, kReg>(a, x, y1, c1, t1, r1);
}

// ------------------------------------------------------------ 16-bit storage, cells in x pairs
// Cells (x, x + 1) of one row per thread, x even.  With nx even, each population of the pair
// is one aligned 32-bit word of its plane (cell x in the low half), so the pair moves with one
// load and one store per speed where two cells of their own take two of each, and one
// instruction converts both cells' results.  A speed with e_x = 0 pulls the word of its source
// row whole; e_x = +1 pulls cells (x - 1, x), the high half of the word before the pair's and
// the low half of the pair's own; e_x = -1 pulls (x + 1, x + 2), the high half of the pair's
// word and the low half of the one after.  The solid bounce-back swaps opposite shifts after
// widening them to float, which both 16-bit formats hold exactly, so it stays a bit copy.
template <int K>
struct Pair16;

template <>
struct Pair16<kStoreBF16> {
  static __device__ __forceinline__ float lo(uint32_t w) { return __uint_as_float(w << 16); }
  static __device__ __forceinline__ float hi(uint32_t w) {
    return __uint_as_float(w & 0xFFFF0000u);
  }
  // (a, b) rounded to nearest even, a in the low half
  static __device__ __forceinline__ uint32_t pack(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
  }
};

template <>
struct Pair16<kStoreF16> {
  static __device__ __forceinline__ float lo(uint32_t w) {
    return __half2float(__ushort_as_half(static_cast<unsigned short>(w & 0xFFFFu)));
  }
  static __device__ __forceinline__ float hi(uint32_t w) {
    return __half2float(__ushort_as_half(static_cast<unsigned short>(w >> 16)));
  }
  static __device__ __forceinline__ uint32_t pack(float a, float b) {
    const __half2 v = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
  }
};

// a pair with a node that is neither fluid nor solid (inlet, outlet, moving wall): each cell
// through the one-cell code, which loads its own values again
template <class L, int K, int kClosure>
__device__ __noinline__ void pair_cold(const StepArgs& a, int x, int y, int z) {
  cell_step<L, K, kClosure, false, true, false>(a, x, y, z);
  cell_step<L, K, kClosure, false, true, false>(a, x + 1, y, z);
}

// one cell's shifts d (f - w), fluid or solid, collided or bounced back in place
template <class L, int kClosure>
__device__ __forceinline__ void pair_cell(const DevProblem& pb, uint32_t t, float (&d)[L::Q]) {
  if (t == kFluid) {
    float rho, ux, uy, uz;
    fast::fluid_collide_shifted<L, kClosure>(d, Par<float>::omega(pb), Par<float>::cs(pb),
                                             Par<float>::nu(pb), relaxes(pb), rho, ux, uy, uz);
  } else {
    float s[L::Q];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) s[i] = d[L::bb(i)];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) d[i] = s[i];
  }
}

// The pair step's parameters: the step's, and each population plane's first word in both
// buffers, so that a word's address is one multiply-add of its index onto a parameter.
struct PairArgs {
  StepArgs a;
  const uint32_t* src[27];
  uint32_t* dst[27];
};

// The populations (one word per speed) and the two node types of cells (x, x + 1), row y,
// plane z.
template <class L>
__device__ __forceinline__ void pair_load(const PairArgs& pa, int x, int y, int z,
                                          uint32_t (&w)[L::Q], uint32_t& tt) {
  const DevProblem& pb = pa.a.pb;
  const int nx = pb.nx;
  // cell offsets of the source rows y - e_y and planes z - e_z (periodic)
  const int y0 = y * nx, z0 = z * pb.nxy;
  const int ym = (y == 0 ? pb.ny - 1 : y - 1) * nx, yp = (y == pb.ny - 1 ? 0 : y + 1) * nx;
  const int zm = (z == 0 ? pb.nz - 1 : z - 1) * pb.nxy;
  const int zp = (z == pb.nz - 1 ? 0 : z + 1) * pb.nxy;
  const int xl = x == 0 ? nx - 2 : x - 2;  // the word before the pair's (e_x = +1)
  const int xr = x + 2 == nx ? 0 : x + 2;  // the word after it (e_x = -1)
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    const int ex = L::ex(i), ey = L::ey(i), ez = L::ez(i);
    const int row = (ey > 0 ? ym : (ey < 0 ? yp : y0)) + (ez > 0 ? zm : (ez < 0 ? zp : z0));
    const uint32_t* __restrict__ pl = pa.src[i];
    const uint32_t mid = __ldg(pl + (static_cast<uint32_t>(row + x) >> 1));
    if (ex == 0)
      w[i] = mid;
    else if (ex > 0)
      w[i] = __byte_perm(__ldg(pl + (static_cast<uint32_t>(row + xl) >> 1)), mid, 0x5432);
    else
      w[i] = __byte_perm(mid, __ldg(pl + (static_cast<uint32_t>(row + xr) >> 1)), 0x5432);
  }
  tt = *reinterpret_cast<const uint16_t*>(pb.nd_type + x + y0 + z0);
}

// The rest of the step of cells (x, x + 1) from their loaded words and types.
template <class L, int K, int kClosure>
__device__ __forceinline__ void pair_finish(const PairArgs& pa, int x, int y, int z,
                                            const uint32_t (&w)[L::Q], uint32_t tt) {
  using PK = Pair16<K>;
  constexpr int Q = L::Q;
  const DevProblem& pb = pa.a.pb;
  const uint32_t t0 = tt & 0xFFu, t1 = tt >> 8;
  if (((t0 > kSolid) | (t1 > kSolid)) != 0) {
    pair_cold<L, K, kClosure>(pa.a, x, y, z);
    return;
  }
  float d0[Q], d1[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    d0[i] = PK::lo(w[i]);
    d1[i] = PK::hi(w[i]);
  }
  pair_cell<L, kClosure>(pb, t0, d0);
  pair_cell<L, kClosure>(pb, t1, d1);
  const uint32_t cw = static_cast<uint32_t>(x + y * pb.nx + z * pb.nxy) >> 1;
#pragma unroll
  for (int i = 0; i < Q; ++i) pa.dst[i][cw] = PK::pack(d0[i], d1[i]);
}

// The step of cells (x, x + 1) of row y, plane z, for launches without time averaging.
template <class L, int K, int kClosure>
__device__ __forceinline__ void pair_step(const PairArgs& pa, int x, int y, int z) {
  uint32_t w[L::Q], tt;
  pair_load<L>(pa, x, y, z, w, tt);
  pair_finish<L, K, kClosure>(pa, x, y, z, w, tt);
}

}  // namespace tlbm
