// grid.cuh -- lattice geometry on the device and the periodic neighbour arithmetic.
//
// Populations are stored structure-of-arrays, f[speed][z][y][x] (x fastest), so a warp's 32
// consecutive x cells read and write 32 consecutive values of one speed.  The stream step is a
// pull: cell c gathers speed i from cell c - e_i, with periodic wrap on all three axes exactly
// like get_tgt_index (src/TLBM_Partition.cpp:691-712): the reference pushes to c + e_i, so
// pulling from c - e_i moves the same values.
#pragma once

#include <cstdint>

#include "lattice.cuh"
#include "physics_fx.cuh"

namespace tlbm {

struct DevProblem {
  int nx, ny, nz;
  int nxy;         // nx*ny
  int64_t n;       // nx*ny*nz (< 2^31 so cell offsets fit in int)
  const uint8_t* nd_type;
  double omega, cs, u_bc, rho_bc;  // the parsed `real` values, held exactly
  double nu;                        // (1/omega - 1/2)/3, the molecular viscosity
  // the same values rounded to float once on the host (a float kernel converting doubles per
  // thread would spend FP64-pipe slots on it)
  float omega_f, cs_f, u_bc_f, rho_bc_f, nu_f;
  int dynamics;
  // moment-space collision (fast arithmetic): dynamics 2 with the rbgk option (regularised
  // BGK, ghost rate 1) or dynamics 3 with the mrt option (ghost rate from the options)
  int mcoll;
  double ghost_omega;
  float ghost_omega_f;
  int has_type5;
  // byte offset, from a cell's own population of speed 0, of the population of speed i that an
  // interior cell (no face of the box) pulls: i*n*bytes - (ex + ey*nx + ez*nx*ny)*bytes
  long long pull_off[27];
  // the same offsets in cells, ex + ey*nx + ez*nx*ny (the pulled slot is c - pull_cell[i])
  int pull_cell[27];
  // optional inlet velocity per (x, y) of the z = 0 plane (nx*ny values; null: uniform u_bc)
  const double* inlet_d;
  const float* inlet_f;
  // FP64 storage, fast arithmetic: fluid nodes collide in exact fixed point (physics_fx.cuh)
  int fx;
  fx::Consts fxk;
};

// whether nodes relax: LBGK, or the regularised BGK of dynamics 2
TLBM_HD bool relaxes(const DevProblem& p) { return p.dynamics == 1 || p.mcoll; }

// problem parameters in the compute type
template <class C>
struct Par;
template <>
struct Par<double> {
  static TLBM_HD double omega(const DevProblem& p) { return p.omega; }
  static TLBM_HD double cs(const DevProblem& p) { return p.cs; }
  static TLBM_HD double u_bc(const DevProblem& p) { return p.u_bc; }
  static TLBM_HD double rho_bc(const DevProblem& p) { return p.rho_bc; }
  static TLBM_HD double nu(const DevProblem& p) { return p.nu; }
  static TLBM_HD double ghost_omega(const DevProblem& p) { return p.ghost_omega; }
  static TLBM_HD double u_in(const DevProblem& p, int xy) {
    return p.inlet_d ? p.inlet_d[xy] : p.u_bc;
  }
};
template <>
struct Par<float> {
  static TLBM_HD float omega(const DevProblem& p) { return p.omega_f; }
  static TLBM_HD float cs(const DevProblem& p) { return p.cs_f; }
  static TLBM_HD float u_bc(const DevProblem& p) { return p.u_bc_f; }
  static TLBM_HD float rho_bc(const DevProblem& p) { return p.rho_bc_f; }
  static TLBM_HD float nu(const DevProblem& p) { return p.nu_f; }
  static TLBM_HD float ghost_omega(const DevProblem& p) { return p.ghost_omega_f; }
  static TLBM_HD float u_in(const DevProblem& p, int xy) {
    return p.inlet_f ? p.inlet_f[xy] : p.u_bc_f;
  }
};

// fills the float copies and the interior pull offsets of `pb` for q speeds of `bytes` each
template <class L>
inline void fill_pull_offsets(DevProblem& pb, int bytes) {
  for (int i = 0; i < 27; ++i) {
    pb.pull_off[i] = 0;
    pb.pull_cell[i] = 0;
  }
  for (int i = 0; i < L::Q; ++i) {
    const long long d = L::ex(i) + static_cast<long long>(L::ey(i)) * pb.nx +
                        static_cast<long long>(L::ez(i)) * pb.nxy;
    pb.pull_off[i] = (static_cast<long long>(i) * pb.n - d) * bytes;
    pb.pull_cell[i] = static_cast<int>(d);
  }
}

inline void fill_derived(DevProblem& pb, int q, int bytes) {
  pb.omega_f = static_cast<float>(pb.omega);
  pb.cs_f = static_cast<float>(pb.cs);
  pb.u_bc_f = static_cast<float>(pb.u_bc);
  pb.rho_bc_f = static_cast<float>(pb.rho_bc);
  pb.nu_f = static_cast<float>(pb.nu);
  pb.ghost_omega_f = static_cast<float>(pb.ghost_omega);
  if (q == 15) fill_pull_offsets<Lattice<15>>(pb, bytes);
  if (q == 19) fill_pull_offsets<Lattice<19>>(pb, bytes);
  if (q == 27) fill_pull_offsets<Lattice<27>>(pb, bytes);
}

// offsets of a cell and its periodic neighbours along each axis
struct Nbr {
  int x0, xm, xp;  // x, x-1, x+1 (wrapped)
  int y0, ym, yp;  // row offsets y*nx, (y-1)*nx, (y+1)*nx (wrapped)
  int z0, zm, zp;  // plane offsets z*nxy, ...

  TLBM_HD Nbr(int x, int y, int z, int nx, int ny, int nz, int nxy) {
    x0 = x;
    xm = (x == 0) ? nx - 1 : x - 1;
    xp = (x == nx - 1) ? 0 : x + 1;
    y0 = y * nx;
    ym = ((y == 0) ? ny - 1 : y - 1) * nx;
    yp = ((y == ny - 1) ? 0 : y + 1) * nx;
    z0 = z * nxy;
    zm = ((z == 0) ? nz - 1 : z - 1) * nxy;
    zp = ((z == nz - 1) ? 0 : z + 1) * nxy;
  }
  TLBM_HD int self() const { return x0 + y0 + z0; }
  // cell c - e_i (where speed i streams from)
  template <class L>
  TLBM_HD int from(int i) const {
    const int ex = L::ex(i), ey = L::ey(i), ez = L::ez(i);
    return (ex > 0 ? xm : (ex < 0 ? xp : x0)) + (ey > 0 ? ym : (ey < 0 ? yp : y0)) +
           (ez > 0 ? zm : (ez < 0 ? zp : z0));
  }
  // cell c + e_i (where speed i streams to: the reference's adj[c*Q+i])
  template <class L>
  TLBM_HD int to(int i) const {
    const int ex = L::ex(i), ey = L::ey(i), ez = L::ez(i);
    return (ex > 0 ? xp : (ex < 0 ? xm : x0)) + (ey > 0 ? yp : (ey < 0 ? ym : y0)) +
           (ez > 0 ? zp : (ez < 0 ? zm : z0));
  }
};

// Cell c + 2 e_i (wrapped) from a cell's neighbour offsets: where the fluid neighbour
// g = c + e_i pulls speed bb(i) from (the second source of a boundary link's force term).
struct Nbr2 {
  int xpp, xmm, ypp, ymm, zpp, zmm;  // x+2, x-2, row offsets of y+2, y-2, plane offsets z+-2

  TLBM_HD Nbr2(const Nbr& b, int nx, int ny, int nz, int nxy) {
    xpp = (b.xp == nx - 1) ? 0 : b.xp + 1;
    xmm = (b.xm == 0) ? nx - 1 : b.xm - 1;
    ypp = (b.yp == (ny - 1) * nx) ? 0 : b.yp + nx;
    ymm = (b.ym == 0) ? (ny - 1) * nx : b.ym - nx;
    zpp = (b.zp == (nz - 1) * nxy) ? 0 : b.zp + nxy;
    zmm = (b.zm == 0) ? (nz - 1) * nxy : b.zm - nxy;
  }
  template <class L>
  TLBM_HD int to2(const Nbr& b, int i) const {
    const int ex = L::ex(i), ey = L::ey(i), ez = L::ez(i);
    return (ex > 0 ? xpp : (ex < 0 ? xmm : b.x0)) + (ey > 0 ? ypp : (ey < 0 ? ymm : b.y0)) +
           (ez > 0 ? zpp : (ez < 0 ? zmm : b.z0));
  }
};

// cell index -> (x, y, z)
TLBM_HD void decompose(int c, int nx, int nxy, int& x, int& y, int& z) {
  z = c / nxy;
  const int r = c - z * nxy;
  y = r / nx;
  x = r - y * nx;
}

}  // namespace tlbm
