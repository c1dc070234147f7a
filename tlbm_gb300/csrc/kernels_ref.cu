// kernels_ref.cu -- the fused stream-collide step in the reference's exact arithmetic.
//
// Compiled with -fmad=false (no a*b+c contraction) so that, together with physics_ref.cuh,
// every value is bit-identical to the CPU reference built with `real` = R.  One thread owns one
// cell: it pulls its Q populations (the reference's push, stream_node_data,
// src/TLBM_Partition.cpp:826-837, read from the receiving side), runs the node-type branch of
// process_node_list (:742-812) in registers, and stores the post-collision populations at its
// own cell.  No neighbour table, no fEq array and no macroscopic arrays touch memory.
#include "kernels.h"
#include "physics_ref.cuh"

namespace tlbm {
namespace {

template <class L, class R>
__global__ void __launch_bounds__(128) k_step_ref(StepArgs a) {
  const DevProblem& pb = a.pb;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= pb.nx || y >= pb.ny) return;
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  const int c = nb.self();
  const size_t n = static_cast<size_t>(pb.n);
  const R* __restrict__ src = static_cast<const R*>(a.src);
  R* __restrict__ dst = static_cast<R*>(a.dst);

  R f[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = __ldg(src + i * n + nb.from<L>(i));

  const uint8_t t = pb.nd_type[c];
  const R u_bc = static_cast<R>(pb.u_bc);
  const R rho_bc = static_cast<R>(pb.rho_bc);
  R ux, uy, uz, rho;
  if (t == kSolid) {
    // moments (only rho survives), u = 0, bounce-back swap, no collision (:750-756)
    rho = ref::density(f);
    ux = 0;
    uy = 0;
    uz = 0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) dst[i * n + c] = f[L::bb(i)];
  } else {
    R feq[L::Q];
    if (t == kInlet) {
      ref::inlet_macro<L, R>(f, u_bc, ux, uy, uz, rho);
      ref::equilibrium<L, R>(ux, uy, uz, rho, feq);
      ref::nebb<L, R, true>(f, feq);
    } else {
      ref::moments<L, R>(f, ux, uy, uz, rho);
      if (t == kOutlet) {
        ref::outlet_macro<L, R>(f, rho_bc, uz, rho);
        ref::equilibrium<L, R>(ux, uy, uz, rho, feq);
        ref::nebb<L, R, false>(f, feq);
      } else if (pb.has_type5 && t == kMovingWall) {
        // uy[spd] of the reference: nodes already processed this step hold this step's value
        const R* cur = static_cast<const R*>(a.uyq_cur);
        const R* prev = static_cast<const R*>(a.uyq_prev);
        ref::set_uz<L, R>(f, ux, uz, rho, u_bc, [&](int i) { return i <= c ? cur[i] : prev[i]; });
        ref::equilibrium<L, R>(ux, uy, uz, rho, feq);
      } else {
        ref::equilibrium<L, R>(ux, uy, uz, rho, feq);
      }
    }
    R om = static_cast<R>(pb.omega);
    if (pb.cs > 0) om = ref::smagorinsky<L, R>(f, feq, om, static_cast<R>(pb.cs));
    if (pb.dynamics == 1) ref::relax<L, R>(f, feq, om);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) dst[i * n + c] = f[i];
  }
  if (a.time_avg) {  // update_time_avg (src/TLBM_Partition.cpp:815-824)
    R* const* avg = reinterpret_cast<R* const*>(a.avg);
    avg[0][c] += ux;
    avg[1][c] += uy;
    avg[2][c] += uz;
    avg[3][c] += rho;
  }
}

template <class L, class R>
__global__ void __launch_bounds__(128) k_macros_ref(DevProblem pb, const R* __restrict__ src,
                                                   R* ux_o, R* uy_o, R* uz_o, R* rho_o) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= pb.nx || y >= pb.ny) return;
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  const int c = nb.self();
  const size_t n = static_cast<size_t>(pb.n);
  R f[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = __ldg(src + i * n + nb.from<L>(i));
  R ux, uy, uz, rho;
  ref::node_macros<L, R>(pb.nd_type[c], f, static_cast<R>(pb.u_bc), static_cast<R>(pb.rho_bc), ux,
                         uy, uz, rho);
  ux_o[c] = ux;
  uy_o[c] = uy;
  uz_o[c] = uz;
  rho_o[c] = rho;
}

template <class L, class R>
__global__ void k_quirk_uy_ref(DevProblem pb, const R* __restrict__ src, R* uy_out) {
  const int c = threadIdx.x;
  if (c >= L::Q || c >= pb.n) return;
  int x, y, z;
  decompose(c, pb.nx, pb.nxy, x, y, z);
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  const size_t n = static_cast<size_t>(pb.n);
  R f[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = src[i * n + nb.from<L>(i)];
  R ux, uy, uz, rho;
  ref::node_macros<L, R>(pb.nd_type[c], f, static_cast<R>(pb.u_bc), static_cast<R>(pb.rho_bc), ux,
                         uy, uz, rho);
  uy_out[c] = uy;
}

// calc_force (src/TLBM_Partition.cpp:174-208) with make_force_calc_map's selection (:143-172):
// solid nodes, speeds whose push target is a fluid (type 0) node, in ascending speed order.
// Post-stream population (g, s) = post-collision population s of node g - e_s.
template <class L, class R>
__global__ void __launch_bounds__(128) k_force_ref(DevProblem pb, const R* __restrict__ f,
                                                  R* fx_o, R* fy_o, R* fz_o) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= pb.nx || y >= pb.ny) return;
  const Nbr nb(x, y, z, pb.nx, pb.ny, pb.nz, pb.nxy);
  const int c = nb.self();
  const size_t n = static_cast<size_t>(pb.n);
  R fx = 0, fy = 0, fz = 0;
  bool ax = false, ay = false, az = false;
  if (pb.nd_type[c] == kSolid) {
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const int g = nb.to<L>(i);
      if (pb.nd_type[g] != kFluid) continue;
      const int b = L::bb(i);
      int gx, gy, gz;
      decompose(g, pb.nx, pb.nxy, gx, gy, gz);
      const Nbr ng(gx, gy, gz, pb.nx, pb.ny, pb.nz, pb.nxy);
      const R f1 = f[i * n + nb.from<L>(i)];
      const R f2 = f[b * n + ng.from<L>(b)];
      const R s = f1 + f2;
      if (L::ex(b) != 0) {
        const R t = L::ex(b) > 0 ? s : -s;
        fx = ax ? fx + t : t;
        ax = true;
      }
      if (L::ey(b) != 0) {
        const R t = L::ey(b) > 0 ? s : -s;
        fy = ay ? fy + t : t;
        ay = true;
      }
      if (L::ez(b) != 0) {
        const R t = L::ez(b) > 0 ? s : -s;
        fz = az ? fz + t : t;
        az = true;
      }
    }
  }
  fx_o[c] = fx;
  fy_o[c] = fy;
  fz_o[c] = fz;
}

dim3 grid_of(const DevProblem& pb, const Launch& l) {
  return dim3((pb.nx + l.bx - 1) / l.bx, (pb.ny + l.by - 1) / l.by, pb.nz);
}

dim3 block_of(const Launch& l) { return dim3(l.bx, l.by, 1); }

template <class R>
cudaError_t step_ref_q(int q, const StepArgs& a, const Launch& l) {
  const dim3 g = grid_of(a.pb, l), b = block_of(l);
  switch (q) {
    case 15: k_step_ref<Lattice<15>, R><<<g, b, 0, l.stream>>>(a); break;
    case 19: k_step_ref<Lattice<19>, R><<<g, b, 0, l.stream>>>(a); break;
    case 27: k_step_ref<Lattice<27>, R><<<g, b, 0, l.stream>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t macros_ref_q(int q, const DevProblem& pb, const void* src, void* const out[4],
                         const Launch& l) {
  const dim3 g = grid_of(pb, l), b = block_of(l);
  const R* s = static_cast<const R*>(src);
  R* o[4] = {static_cast<R*>(out[0]), static_cast<R*>(out[1]), static_cast<R*>(out[2]),
             static_cast<R*>(out[3])};
  switch (q) {
    case 15: k_macros_ref<Lattice<15>, R><<<g, b, 0, l.stream>>>(pb, s, o[0], o[1], o[2], o[3]); break;
    case 19: k_macros_ref<Lattice<19>, R><<<g, b, 0, l.stream>>>(pb, s, o[0], o[1], o[2], o[3]); break;
    case 27: k_macros_ref<Lattice<27>, R><<<g, b, 0, l.stream>>>(pb, s, o[0], o[1], o[2], o[3]); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t quirk_ref_q(int q, const DevProblem& pb, const void* src, void* out, const Launch& l) {
  const R* s = static_cast<const R*>(src);
  R* o = static_cast<R*>(out);
  switch (q) {
    case 15: k_quirk_uy_ref<Lattice<15>, R><<<1, 32, 0, l.stream>>>(pb, s, o); break;
    case 19: k_quirk_uy_ref<Lattice<19>, R><<<1, 32, 0, l.stream>>>(pb, s, o); break;
    case 27: k_quirk_uy_ref<Lattice<27>, R><<<1, 32, 0, l.stream>>>(pb, s, o); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t force_ref_q(int q, const DevProblem& pb, const void* f, void* const out[3],
                        const Launch& l) {
  const dim3 g = grid_of(pb, l), b = block_of(l);
  const R* s = static_cast<const R*>(f);
  R* o[3] = {static_cast<R*>(out[0]), static_cast<R*>(out[1]), static_cast<R*>(out[2])};
  switch (q) {
    case 15: k_force_ref<Lattice<15>, R><<<g, b, 0, l.stream>>>(pb, s, o[0], o[1], o[2]); break;
    case 19: k_force_ref<Lattice<19>, R><<<g, b, 0, l.stream>>>(pb, s, o[0], o[1], o[2]); break;
    case 27: k_force_ref<Lattice<27>, R><<<g, b, 0, l.stream>>>(pb, s, o[0], o[1], o[2]); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_step_ref(int q, int rbytes, const StepArgs& a, const Launch& l) {
  return rbytes == 8 ? step_ref_q<double>(q, a, l) : step_ref_q<float>(q, a, l);
}

cudaError_t launch_macros_ref(int q, int rbytes, const DevProblem& pb, const void* src,
                              void* const out[4], const Launch& l) {
  return rbytes == 8 ? macros_ref_q<double>(q, pb, src, out, l)
                     : macros_ref_q<float>(q, pb, src, out, l);
}

cudaError_t launch_quirk_uy_ref(int q, int rbytes, const DevProblem& pb, const void* src,
                                void* uy_out, const Launch& l) {
  return rbytes == 8 ? quirk_ref_q<double>(q, pb, src, uy_out, l)
                     : quirk_ref_q<float>(q, pb, src, uy_out, l);
}

cudaError_t launch_force_ref(int q, int rbytes, const DevProblem& pb, const void* dst,
                             void* const out[3], const Launch& l) {
  return rbytes == 8 ? force_ref_q<double>(q, pb, dst, out, l)
                     : force_ref_q<float>(q, pb, dst, out, l);
}

}  // namespace tlbm
