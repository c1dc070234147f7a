// physics_ref.cuh -- per-node physics in the reference's exact arithmetic.
//
// These device functions compute what LatticeStructure<T> and its D3Q15/19/27 subclasses
// compute per node (include/LatticeStructure.hpp:70-177 and the lattice headers), with
//   * the same operation order (left-to-right sums over speeds 0..Q-1, divide after summing),
//   * the same C++ type promotions: `R` is the reference's `real`; double literals such as 3.0,
//     1. or 2. promote an R operand to double exactly where the reference's expressions do,
//   * no FMA contraction: the translation unit that instantiates them is compiled with
//     -fmad=false, and division and square root are the IEEE round-to-nearest operations,
// so results are bit-identical to the reference compiled for the CPU.
//
// Terms whose lattice coefficient is 0 are skipped and coefficients +-1 become additions and
// subtractions.  That changes no bit: the reference's running sums start at +0, x*(+-1) is exact,
// a + (-b) == a - b, and adding a signed zero to a sum that is never -0 leaves it unchanged.
#pragma once

#include "lattice.cuh"

namespace tlbm {
namespace ref {

#define TLBM_DEV __device__ __forceinline__

// sum_i c_i f_i over speeds in order, c_i in {-1,0,1}; +0 when every c_i is 0
template <class R, int Q, class Coef>
TLBM_DEV R signed_sum(const R (&f)[Q], Coef c) {
  R s = R(0);
  bool any = false;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const int e = c(i);
    if (e != 0) {
      const R t = e > 0 ? f[i] : -f[i];
      if (any) {
        s = s + t;
      } else {
        s = t;
        any = true;
      }
    }
  }
  return s;
}

// rho = sum f (the reference's rho_l starts at 0 and adds every speed)
template <class R, int Q>
TLBM_DEV R density(const R (&f)[Q]) {
  R r = f[0];
#pragma unroll
  for (int i = 1; i < Q; ++i) r = r + f[i];
  return r;
}

// compute_macroscopic_data (include/LatticeStructure.hpp:70-90)
template <class L, class R>
TLBM_DEV void moments(const R (&f)[L::Q], R& ux, R& uy, R& uz, R& rho) {
  rho = density(f);
  const R jx = signed_sum(f, [](int i) { return L::ex(i); });
  const R jy = signed_sum(f, [](int i) { return L::ey(i); });
  const R jz = signed_sum(f, [](int i) { return L::ez(i); });
  ux = jx / rho;
  uy = jy / rho;
  uz = jz / rho;
}

// ex*ux + ey*uy + ez*uz in R, zero terms skipped
template <class L, class R>
TLBM_DEV R edotu(int i, R ux, R uy, R uz) {
  R s = R(0);
  bool any = false;
  const int c[3] = {L::ex(i), L::ey(i), L::ez(i)};
  const R u[3] = {ux, uy, uz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (c[a] != 0) {
      const R t = c[a] > 0 ? u[a] : -u[a];
      if (any) {
        s = s + t;
      } else {
        s = t;
        any = true;
      }
    }
  }
  return s;
}

// compute_equilibrium (include/LatticeStructure.hpp:93-103)
template <class L, class R>
TLBM_DEV void equilibrium(R ux, R uy, R uz, R rho, R (&feq)[L::Q]) {
  const R usq = ux * ux + uy * uy + uz * uz;
  const double t15 = 3. / 2. * usq;
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    const R cu = 3.0 * edotu<L, R>(i, ux, uy, uz);
    const R wr = weight<L, R>(i) * rho;
    feq[i] = wr * (1.0 + cu + 0.5 * (cu * cu) - t15);
  }
}

// known-population sums of the inlet/outlet density/velocity formulas, literal order
template <int N, class R, int Q, class Idx>
TLBM_DEV R listed_sum(const R (&f)[Q], Idx idx) {
  R s = f[idx(0)];
#pragma unroll
  for (int k = 1; k < N; ++k) s = s + f[idx(k)];
  return s;
}

// set_inletW_bc_macro: Q15 :113-134, Q19 :108-132, Q27 :112-140
template <class L, class R>
TLBM_DEV void inlet_macro(const R (&f)[L::Q], R u_bc, R& ux, R& uy, R& uz, R& rho) {
  const R a = listed_sum<L::NBB>(f, [](int k) { return L::in_known(k); });
  const R b = listed_sum<L::NFLAT>(f, [](int k) { return L::zero(k); });
  ux = 0;
  uy = 0;
  uz = u_bc;
  if constexpr (L::kInletIntTwo) {
    const R s = 2 * a + b;
    rho = (1. / (1. - u_bc)) * s;
  } else {
    rho = (1. / (1. - u_bc)) * (2. * a + b);
  }
}

// set_outletE_bc_macro: Q15 :137-153, Q19 :135-155, Q27 :144-167 (ux, uy untouched)
template <class L, class R>
TLBM_DEV void outlet_macro(const R (&f)[L::Q], R rho_bc, R& uz, R& rho) {
  const R a = listed_sum<L::NBB>(f, [](int k) { return L::out_known(k); });
  const R b = listed_sum<L::NFLAT>(f, [](int k) { return L::zero(k); });
  rho = rho_bc;
  uz = -1. + (1. / rho_bc) * (2. * a + b);
}

// set_inletW_bc_micro / set_outletE_bc_micro: f[sp] = feq[sp] + f[bb] - feq[bb]
template <class L, class R, bool kInlet>
TLBM_DEV void nebb(R (&f)[L::Q], const R (&feq)[L::Q]) {
#pragma unroll
  for (int k = 0; k < L::NBB; ++k) {
    const int sp = kInlet ? L::in_sp(k) : L::in_bb(k);
    const int bp = kInlet ? L::in_bb(k) : L::in_sp(k);
    f[sp] = feq[sp] + f[bp] - feq[bp];
  }
}

// set_uz_bc (include/LatticeStructure.hpp:167-177).  `uyq(i)` is the uy of node number i --
// the reference indexes uy by the speed (uy[spd]), not by the node.
template <class L, class R, class UyQ>
TLBM_DEV void set_uz(R (&f)[L::Q], R ux, R uz, R rho, R u_bc, UyQ uyq) {
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    f[i] += 3. * rho * weight<L, R>(i) *
            (L::ez(i) * (u_bc - uz) + L::ex(i) * (0. - ux) + L::ey(i) * (0. - uyq(i)));
  }
}

// compute_strain_tensor + apply_turbulence_model (include/LatticeStructure.hpp:106-153)
template <class L, class R>
TLBM_DEV R smagorinsky(const R (&f)[L::Q], const R (&feq)[L::Q], R omega, R cs) {
  R d[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) d[i] = f[i] - feq[i];
  const R s0 = signed_sum(d, [](int i) { return L::ex(i) * L::ex(i); });
  const R s4 = signed_sum(d, [](int i) { return L::ey(i) * L::ey(i); });
  const R s8 = signed_sum(d, [](int i) { return L::ez(i) * L::ez(i); });
  const R s1 = signed_sum(d, [](int i) { return L::ex(i) * L::ey(i); });
  const R s2 = signed_sum(d, [](int i) { return L::ex(i) * L::ez(i); });
  const R s5 = signed_sum(d, [](int i) { return L::ey(i) * L::ez(i); });
  const R nu = ((1. / omega) - 0.5) / 3.0;
  R p = ::sqrt(s0 * s0 + s4 * s4 + s8 * s8 + 2.0 * (s1 * s1 + s2 * s2 + s5 * s5));
  p *= cs;
  // the reference's unqualified sqrt is the global double sqrt: widen, subtract in double
  p = ::sqrt(static_cast<double>(p + nu * nu)) - nu;
  const R nu_e = p / 6.;
  const R omega_r = 1. / (3. * (nu + nu_e) + 0.5);
  return omega_r;
}

// relax (include/LatticeStructure.hpp:156-163)
template <class L, class R>
TLBM_DEV void relax(R (&f)[L::Q], const R (&feq)[L::Q], R omega) {
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = f[i] - omega * (f[i] - feq[i]);
}

// The macroscopic values the reference holds for a node after processing it
// (src/TLBM_Partition.cpp:744-777): solid -> u = 0, inlet -> u = (0,0,u_bc) and its density,
// outlet -> rho = rho_bc and its uz, others -> the moments.
template <class L, class R>
TLBM_DEV void node_macros(uint8_t t, const R (&f)[L::Q], R u_bc, R rho_bc, R& ux, R& uy, R& uz,
                          R& rho) {
  if (t == kSolid) {
    rho = density(f);
    ux = 0;
    uy = 0;
    uz = 0;
  } else if (t == kInlet) {
    inlet_macro<L, R>(f, u_bc, ux, uy, uz, rho);
  } else {
    moments<L, R>(f, ux, uy, uz, rho);
    if (t == kOutlet) outlet_macro<L, R>(f, rho_bc, uz, rho);
  }
}

}  // namespace ref
}  // namespace tlbm
