// lattice.cuh -- D3Q15 / D3Q19 / D3Q27 velocity sets as compile-time tables (host + device).
//
// The tables carry the reference's exact numbering and values, because output parity depends
// on them: speed order, bounce-back partner bbSpd, weights (D3Q15/D3Q19 weights are float
// literals widened to `real`; D3Q27 weights are double literals), the speeds each inlet/outlet
// reconstruction treats as unknown, and the literal order of the known-population sums.
//   D3Q15: include/D3Q15LatticeStructure.hpp:39-45, :77-153
//   D3Q19: include/D3Q19LatticeStructure.hpp:40-47, :80-155
//   D3Q27: include/D3Q27LatticeStructure.hpp:40-53, :84-167
// Every accessor is constexpr so that fully unrolled speed loops fold to immediates.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define TLBM_HD __host__ __device__ __forceinline__
#else
#define TLBM_HD inline
#endif

namespace tlbm {

template <int Q_>
struct Lattice;

template <>
struct Lattice<15> {
  static constexpr int Q = 15;
  static constexpr int NBB = 5;   // unknown speeds at the inlet / outlet
  static constexpr int NFLAT = 5; // speeds with ez == 0
  static constexpr bool kInletIntTwo = false;
  TLBM_HD static constexpr int ex(int i) {
    constexpr int v[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int ey(int i) {
    constexpr int v[15] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int ez(int i) {
    constexpr int v[15] = {0, 0, 0, 0, 0, 1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int bb(int i) {
    constexpr int v[15] = {0, 2, 1, 4, 3, 6, 5, 14, 13, 12, 11, 10, 9, 8, 7};
    return v[i];
  }
  // reference weights: float literals
  TLBM_HD static constexpr float wlit(int i) {
    constexpr float v[15] = {2.f / 9.f,  1.f / 9.f,  1.f / 9,    1.f / 9.f,  1.f / 9.f,
                             1.f / 9.f,  1.f / 9.f,  1.f / 72.f, 1.f / 72.f, 1.f / 72.f,
                             1.f / 72.f, 1.f / 72.f, 1.f / 72.f, 1.f / 72.f, 1.f / 72.f};
    return v[i];
  }
  // inlet unknowns (ez > 0) and their partners -- z-mirror pairs, not bbSpd opposites
  TLBM_HD static constexpr int in_sp(int k) {
    constexpr int v[5] = {5, 7, 8, 9, 10};
    return v[k];
  }
  TLBM_HD static constexpr int in_bb(int k) {
    constexpr int v[5] = {6, 11, 12, 13, 14};
    return v[k];
  }
  // inlet density: known ez<0 speeds in the reference's literal order, then ez==0 speeds
  TLBM_HD static constexpr int in_known(int k) {
    constexpr int v[5] = {6, 11, 12, 13, 14};
    return v[k];
  }
  TLBM_HD static constexpr int out_known(int k) {
    constexpr int v[5] = {5, 7, 8, 9, 10};
    return v[k];
  }
  TLBM_HD static constexpr int zero(int k) {
    constexpr int v[5] = {0, 1, 2, 3, 4};
    return v[k];
  }
};

template <>
struct Lattice<19> {
  static constexpr int Q = 19;
  static constexpr int NBB = 5;
  static constexpr int NFLAT = 9;
  static constexpr bool kInletIntTwo = false;
  TLBM_HD static constexpr int ex(int i) {
    constexpr int v[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
    return v[i];
  }
  TLBM_HD static constexpr int ey(int i) {
    constexpr int v[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int ez(int i) {
    constexpr int v[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int bb(int i) {
    constexpr int v[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
    return v[i];
  }
  TLBM_HD static constexpr float wlit(int i) {
    constexpr float v[19] = {3.f / 9.f,  1.f / 18.f, 1.f / 18.f, 1.f / 18.f, 1.f / 18.f,
                             1.f / 18.f, 1.f / 18.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f,
                             1.f / 36.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f,
                             1.f / 36.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f};
    return v[i];
  }
  TLBM_HD static constexpr int in_sp(int k) {
    constexpr int v[5] = {5, 11, 12, 15, 16};
    return v[k];
  }
  TLBM_HD static constexpr int in_bb(int k) {
    constexpr int v[5] = {6, 14, 13, 18, 17};
    return v[k];
  }
  TLBM_HD static constexpr int in_known(int k) {
    constexpr int v[5] = {6, 13, 14, 17, 18};
    return v[k];
  }
  TLBM_HD static constexpr int out_known(int k) {
    constexpr int v[5] = {5, 11, 12, 15, 16};
    return v[k];
  }
  TLBM_HD static constexpr int zero(int k) {
    constexpr int v[9] = {0, 1, 2, 3, 4, 7, 8, 9, 10};
    return v[k];
  }
};

template <>
struct Lattice<27> {
  static constexpr int Q = 27;
  static constexpr int NBB = 9;
  static constexpr int NFLAT = 9;
  // the D3Q27 inlet density multiplies its unknown-side sum by the int 2 (the sum stays in
  // `real`), the other lattices by the double 2. (D3Q27LatticeStructure.hpp:294)
  static constexpr bool kInletIntTwo = true;
  TLBM_HD static constexpr int ex(int i) {
    constexpr int v[27] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1,
                           -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int ey(int i) {
    constexpr int v[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0,
                           0, 1, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int ez(int i) {
    constexpr int v[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1,
                           -1, 1, -1, 1, -1, 1, -1, 1, -1, 1, -1, 1, -1};
    return v[i];
  }
  TLBM_HD static constexpr int bb(int i) {
    constexpr int v[27] = {0,  2,  1,  4,  3,  6,  5,  10, 9,  8,  7,  14, 13, 12,
                           11, 18, 17, 16, 15, 26, 25, 24, 23, 22, 21, 20, 19};
    return v[i];
  }
  TLBM_HD static constexpr double wlit(int i) {
    constexpr double v[27] = {8. / 27.,  2. / 27.,  2. / 27.,  2. / 27.,  2. / 27.,  2. / 27.,
                              2. / 27.,  1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,
                              1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,
                              1. / 54.,  1. / 216., 1. / 216., 1. / 216., 1. / 216., 1. / 216.,
                              1. / 216., 1. / 216., 1. / 216.};
    return v[i];
  }
  TLBM_HD static constexpr int in_sp(int k) {
    constexpr int v[9] = {5, 11, 13, 15, 17, 19, 21, 23, 25};
    return v[k];
  }
  TLBM_HD static constexpr int in_bb(int k) {
    constexpr int v[9] = {6, 14, 12, 18, 16, 26, 24, 22, 20};
    return v[k];
  }
  TLBM_HD static constexpr int in_known(int k) {
    constexpr int v[9] = {6, 14, 12, 18, 16, 26, 24, 22, 20};
    return v[k];
  }
  TLBM_HD static constexpr int out_known(int k) {
    constexpr int v[9] = {5, 11, 13, 15, 17, 19, 21, 23, 25};
    return v[k];
  }
  TLBM_HD static constexpr int zero(int k) {
    constexpr int v[9] = {0, 1, 2, 3, 4, 7, 8, 9, 10};
    return v[k];
  }
};

// weight in the reference's `real` type R (float literal or double literal converted to R)
template <class L, class R>
TLBM_HD constexpr R weight(int i) {
  return static_cast<R>(L::wlit(i));
}

// node type codes (python/FluidChannel.py:1386-1397, :1217-1219)
enum : uint8_t { kFluid = 0, kSolid = 1, kInlet = 2, kOutlet = 3, kMovingWall = 5 };

}  // namespace tlbm
