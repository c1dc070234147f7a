/*
 * tlbm_oracle.c -- CPU restatement of the tLBM timestep path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the oracle the CUDA engine is checked against.  It is never linked into the
 * product: only the test suite, the smoke check and the CPU-baseline leg of the benchmark
 * load it (through ctypes).  It restates, in plain C, the reference's per-node physics and its
 * push-streaming data flow exactly as the reference executes them:
 *
 *   - array-of-structures populations f[node*Q + speed] in two ping-pong buffers
 *     (include/TLBM_Partition.h:57-60, src/TLBM_Partition.cpp:421-446, :910-920);
 *   - an int32 neighbour table adj[node*Q + speed] with periodic wrap in x, y and z
 *     (src/TLBM_Partition.cpp:254-271, :691-737);
 *   - nodes processed in ascending order (the interior list at one rank), each node doing
 *     macroscopic moments -> node-type branch -> optional Smagorinsky -> BGK relax -> push
 *     (src/TLBM_Partition.cpp:738-837, include/LatticeStructure.hpp:70-177,
 *      include/D3Q15LatticeStructure.hpp, D3Q19LatticeStructure.hpp, D3Q27LatticeStructure.hpp);
 *   - the same operation order and the same C/C++ type promotions (double literals such as
 *     3.0 or 1. promote float operands to double), so that with -ffp-contract=off the results
 *     are bit-identical to the reference compiled with `real` = float or double.
 *
 * Parity pin: tests/golden holds SHA-256 digests and fields of the reference's own outputs
 * (compiled from its sources by oracle/Makefile and run by tests/golden/make_golden.py); the
 * CPU test suite checks this oracle against them bit for bit.
 *
 * Precision is chosen at compile time, as in the reference: ORACLE_REAL_DOUBLE=1 -> double.
 */
#define _POSIX_C_SOURCE 200809L
#include <fcntl.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#if ORACLE_REAL_DOUBLE
typedef double real;
#define REAL_SCAN(s) strtod((s), NULL)
#else
typedef float real;
#define REAL_SCAN(s) strtof((s), NULL)
#endif

#define QMAX 27

typedef struct {
  int q;
  int ex[QMAX], ey[QMAX], ez[QMAX], bb[QMAX];
  real w[QMAX];
  /* inlet/outlet non-equilibrium bounce-back pairs (unknown speed, partner speed) */
  int nbb;
  int in_sp[9], in_bb[9], out_sp[9], out_bb[9];
} lattice_t;

/* Lattice tables: D3Q15 include/D3Q15LatticeStructure.hpp:39-45, D3Q19
 * include/D3Q19LatticeStructure.hpp:40-47, D3Q27 include/D3Q27LatticeStructure.hpp:40-53.
 * D3Q15/D3Q19 weights are float literals widened to `real`; D3Q27 weights are double literals. */
static void lattice_init(lattice_t* L, int q) {
  memset(L, 0, sizeof(*L));
  L->q = q;
  if (q == 15) {
    static const int ex[] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
    static const int ey[] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    static const int ez[] = {0, 0, 0, 0, 0, 1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    static const int bb[] = {0, 2, 1, 4, 3, 6, 5, 14, 13, 12, 11, 10, 9, 8, 7};
    static const float w[] = {2.f / 9.f, 1.f / 9.f, 1.f / 9, 1.f / 9.f, 1.f / 9.f,
                              1.f / 9.f, 1.f / 9.f, 1.f / 72.f, 1.f / 72.f, 1.f / 72.f,
                              1.f / 72.f, 1.f / 72.f, 1.f / 72.f, 1.f / 72.f, 1.f / 72.f};
    /* z-mirror pairs, not bbSpd opposites (D3Q15LatticeStructure.hpp:87-88, :101-102) */
    static const int isp[] = {5, 7, 8, 9, 10}, ibb[] = {6, 11, 12, 13, 14};
    for (int i = 0; i < q; ++i) {
      L->ex[i] = ex[i]; L->ey[i] = ey[i]; L->ez[i] = ez[i]; L->bb[i] = bb[i];
      L->w[i] = (real)w[i];
    }
    L->nbb = 5;
    for (int i = 0; i < 5; ++i) {
      L->in_sp[i] = isp[i]; L->in_bb[i] = ibb[i];
      L->out_sp[i] = ibb[i]; L->out_bb[i] = isp[i];
    }
  } else if (q == 19) {
    static const int ex[] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
    static const int ey[] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
    static const int ez[] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
    static const int bb[] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
    static const float w[] = {3.f / 9.f,  1.f / 18.f, 1.f / 18.f, 1.f / 18.f, 1.f / 18.f,
                              1.f / 18.f, 1.f / 18.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f,
                              1.f / 36.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f,
                              1.f / 36.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f};
    static const int isp[] = {5, 11, 12, 15, 16}, ibb[] = {6, 14, 13, 18, 17};
    for (int i = 0; i < q; ++i) {
      L->ex[i] = ex[i]; L->ey[i] = ey[i]; L->ez[i] = ez[i]; L->bb[i] = bb[i];
      L->w[i] = (real)w[i];
    }
    L->nbb = 5;
    for (int i = 0; i < 5; ++i) {
      L->in_sp[i] = isp[i]; L->in_bb[i] = ibb[i];
      L->out_sp[i] = ibb[i]; L->out_bb[i] = isp[i];
    }
  } else {
    static const int ex[] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1,
                             0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1};
    static const int ey[] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1,
                             1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1};
    static const int ez[] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1,
                             -1, 1, -1, 1, -1, 1, -1, 1, -1, 1, -1};
    static const int bb[] = {0,  2,  1,  4,  3,  6,  5,  10, 9,  8,  7,  14, 13, 12,
                             11, 18, 17, 16, 15, 26, 25, 24, 23, 22, 21, 20, 19};
    static const double w[] = {8. / 27.,  2. / 27.,  2. / 27.,  2. / 27.,  2. / 27.,
                               2. / 27.,  2. / 27.,  1. / 54.,  1. / 54.,  1. / 54.,
                               1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,
                               1. / 54.,  1. / 54.,  1. / 54.,  1. / 54.,  1. / 216.,
                               1. / 216., 1. / 216., 1. / 216., 1. / 216., 1. / 216.,
                               1. / 216., 1. / 216.};
    static const int isp[] = {5, 11, 13, 15, 17, 19, 21, 23, 25};
    static const int ibb[] = {6, 14, 12, 18, 16, 26, 24, 22, 20};
    for (int i = 0; i < q; ++i) {
      L->ex[i] = ex[i]; L->ey[i] = ey[i]; L->ez[i] = ez[i]; L->bb[i] = bb[i];
      L->w[i] = (real)w[i];
    }
    L->nbb = 9;
    for (int i = 0; i < 9; ++i) {
      L->in_sp[i] = isp[i]; L->in_bb[i] = ibb[i];
      L->out_sp[i] = ibb[i]; L->out_bb[i] = isp[i];
    }
  }
}

typedef struct oracle_state {
  lattice_t L;
  int dynamics;
  real cs, rho_lbm, u_lbm, omega;
  int nx, ny, nz;
  int64_t n;
  int32_t* nd_type;
  int32_t* adj;
  real *f_even, *f_odd, *f_eq, *f_in, *f_out;
  real *ux, *uy, *uz, *rho;
  real *u_avg, *v_avg, *w_avg, *rho_avg;
  int time_avg;
  int nthreads;
  /* force map: solid nodes next to fluid and, per node, a bitmask of speeds (ascending) */
  int64_t n_force;
  int32_t* force_nodes;
  uint32_t* force_mask;
} oracle_state;

/* get_tgt_index: periodic neighbour in direction (ex,ey,ez) (src/TLBM_Partition.cpp:691-737) */
static int32_t tgt_index(const oracle_state* s, int64_t g, int ex, int ey, int ez) {
  int64_t nxy = (int64_t)s->nx * s->ny;
  int z = (int)(g / nxy);
  int y = (int)((g - (int64_t)z * nxy) / s->nx);
  int x = (int)(g - (int64_t)z * nxy - (int64_t)y * s->nx);
  int tx = (x + ex) % s->nx, ty = (y + ey) % s->ny, tz = (z + ez) % s->nz;
  if (tx < 0) tx += s->nx;
  if (ty < 0) ty += s->ny;
  if (tz < 0) tz += s->nz;
  return (int32_t)(tx + (int64_t)ty * s->nx + (int64_t)tz * nxy);
}

int oracle_set_threads(oracle_state* s, int n) {
  s->nthreads = n > 0 ? n : 1;
  return s->nthreads;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int oracle_real_bytes(void) { return (int)sizeof(real); }

void oracle_destroy(oracle_state* s) {
  if (!s) return;
  free(s->nd_type); free(s->adj); free(s->f_even); free(s->f_odd); free(s->f_eq);
  free(s->ux); free(s->uy); free(s->uz); free(s->rho);
  free(s->u_avg); free(s->v_avg); free(s->w_avg); free(s->rho_avg);
  free(s->force_nodes); free(s->force_mask);
  free(s);
}

/* Build the problem state: neighbour table, f = w*rho in both buffers, force map.
 * (tlbm_initialize, src/TLBM_Partition.cpp:77-118; initialize_data_arrays :448-479;
 *  make_force_calc_map :143-172).  Returns NULL on an unknown lattice. */
oracle_state* oracle_create(int q, int dynamics, double cs, double rho_lbm, double u_lbm,
                            double omega, int nx, int ny, int nz, const int32_t* nd_type,
                            int time_avg) {
  if (q != 15 && q != 19 && q != 27) return NULL;
  oracle_state* s = (oracle_state*)calloc(1, sizeof(oracle_state));
  lattice_init(&s->L, q);
  s->dynamics = dynamics;
  s->cs = (real)cs; s->rho_lbm = (real)rho_lbm; s->u_lbm = (real)u_lbm; s->omega = (real)omega;
  s->nx = nx; s->ny = ny; s->nz = nz;
  s->n = (int64_t)nx * ny * nz;
  s->nthreads = 1;
  s->time_avg = time_avg;
  int64_t n = s->n;
  s->nd_type = (int32_t*)malloc(sizeof(int32_t) * n);
  memcpy(s->nd_type, nd_type, sizeof(int32_t) * n);
  s->adj = (int32_t*)malloc(sizeof(int32_t) * n * q);
  s->f_even = (real*)malloc(sizeof(real) * n * q);
  s->f_odd = (real*)malloc(sizeof(real) * n * q);
  s->f_eq = (real*)calloc((size_t)(n * q), sizeof(real));
  s->ux = (real*)calloc((size_t)n, sizeof(real));
  s->uy = (real*)calloc((size_t)n, sizeof(real));
  s->uz = (real*)calloc((size_t)n, sizeof(real));
  s->rho = (real*)calloc((size_t)n, sizeof(real));
  if (time_avg) {
    s->u_avg = (real*)calloc((size_t)n, sizeof(real));
    s->v_avg = (real*)calloc((size_t)n, sizeof(real));
    s->w_avg = (real*)calloc((size_t)n, sizeof(real));
    s->rho_avg = (real*)calloc((size_t)n, sizeof(real));
  }
  const lattice_t* L = &s->L;
  for (int64_t nd = 0; nd < n; ++nd)
    for (int i = 0; i < q; ++i) s->adj[nd * q + i] = tgt_index(s, nd, L->ex[i], L->ey[i], L->ez[i]);
  real r = s->rho_lbm;
  for (int64_t nd = 0; nd < n; ++nd)
    for (int i = 0; i < q; ++i) {
      s->f_even[nd * q + i] = L->w[i] * r;
      s->f_odd[nd * q + i] = L->w[i] * r;
    }
  /* force map */
  int64_t cnt = 0;
  for (int64_t nd = 0; nd < n; ++nd) {
    if (s->nd_type[nd] != 1) continue;
    uint32_t m = 0;
    for (int i = 0; i < q; ++i)
      if (s->nd_type[s->adj[nd * q + i]] == 0) m |= (1u << i);
    if (m) cnt++;
  }
  s->n_force = cnt;
  s->force_nodes = (int32_t*)malloc(sizeof(int32_t) * (cnt ? cnt : 1));
  s->force_mask = (uint32_t*)malloc(sizeof(uint32_t) * (cnt ? cnt : 1));
  cnt = 0;
  for (int64_t nd = 0; nd < n; ++nd) {
    if (s->nd_type[nd] != 1) continue;
    uint32_t m = 0;
    for (int i = 0; i < q; ++i)
      if (s->nd_type[s->adj[nd * q + i]] == 0) m |= (1u << i);
    if (m) { s->force_nodes[cnt] = (int32_t)nd; s->force_mask[cnt] = m; cnt++; }
  }
  s->f_in = s->f_odd;
  s->f_out = s->f_even;
  return s;
}

/* ------------------------------------------------------------------ per-node physics */

/* compute_macroscopic_data (include/LatticeStructure.hpp:70-90) */
static void macro(const oracle_state* s, const real* f, int64_t nd) {
  const lattice_t* L = &s->L;
  real ux_l = 0, uy_l = 0, uz_l = 0, rho_l = 0, v;
  for (int i = 0; i < L->q; ++i) {
    v = f[nd * L->q + i];
    rho_l += v;
    ux_l += v * L->ex[i];
    uy_l += v * L->ey[i];
    uz_l += v * L->ez[i];
  }
  ux_l /= rho_l;
  uy_l /= rho_l;
  uz_l /= rho_l;
  s->ux[nd] = ux_l; s->uy[nd] = uy_l; s->uz[nd] = uz_l; s->rho[nd] = rho_l;
}

/* compute_equilibrium (include/LatticeStructure.hpp:93-103) */
static void equilibrium(const oracle_state* s, real* feq, int64_t nd) {
  const lattice_t* L = &s->L;
  real cu;
  real ux = s->ux[nd], uy = s->uy[nd], uz = s->uz[nd], rho = s->rho[nd];
  for (int i = 0; i < L->q; ++i) {
    cu = 3.0 * (L->ex[i] * ux + L->ey[i] * uy + L->ez[i] * uz);
    feq[nd * L->q + i] = L->w[i] * rho *
        (1.0 + cu + 0.5 * (cu * cu) - 3. / 2. * (ux * ux + uy * uy + uz * uz));
  }
}

/* bounce_back: f[s] <- f[bb[s]] (D3Q19LatticeStructure.hpp:65-75 and siblings) */
static void bounce_back(const oracle_state* s, real* f, int64_t nd) {
  const lattice_t* L = &s->L;
  real tmp[QMAX];
  for (int i = 0; i < L->q; ++i) tmp[i] = f[nd * L->q + L->bb[i]];
  for (int i = 0; i < L->q; ++i) f[nd * L->q + i] = tmp[i];
}

#define F(k) f[nd * q + (k)]
/* set_inletW_bc_macro: D3Q15 :113-134, D3Q19 :108-132, D3Q27 :112-140 */
static void inlet_macro(const oracle_state* s, const real* f, int64_t nd) {
  const int q = s->L.q;
  real u_bc = s->u_lbm;
  s->ux[nd] = 0; s->uy[nd] = 0; s->uz[nd] = u_bc;
  if (q == 15) {
    s->rho[nd] = (1. / (1. - u_bc)) * (2. * (F(6) + F(11) + F(12) + F(13) + F(14)) +
                                      (F(0) + F(1) + F(2) + F(3) + F(4)));
  } else if (q == 19) {
    s->rho[nd] = (1. / (1. - u_bc)) * (2. * (F(6) + F(13) + F(14) + F(17) + F(18)) +
                                      (F(0) + F(1) + F(2) + F(3) + F(4) + F(7) + F(8) + F(9) + F(10)));
  } else {
    /* the D3Q27 coefficient is the int 2: the bracket stays in `real` */
    s->rho[nd] = (1. / (1. - u_bc)) *
                 (2 * (F(6) + F(14) + F(12) + F(18) + F(16) + F(26) + F(24) + F(22) + F(20)) +
                  (F(0) + F(1) + F(2) + F(3) + F(4) + F(7) + F(8) + F(9) + F(10)));
  }
}

/* set_outletE_bc_macro: D3Q15 :137-153, D3Q19 :135-155, D3Q27 :144-167.
 * ux and uy are left as computed from the moments. */
static void outlet_macro(const oracle_state* s, const real* f, int64_t nd) {
  const int q = s->L.q;
  real rho_bc = s->rho_lbm;
  s->rho[nd] = rho_bc;
  if (q == 15) {
    s->uz[nd] = -1.0 + (1.0 / rho_bc) * (2.0 * (F(5) + F(7) + F(8) + F(9) + F(10)) +
                                        (F(0) + F(1) + F(2) + F(3) + F(4)));
  } else if (q == 19) {
    s->uz[nd] = -1. + (1. / rho_bc) * (2. * (F(5) + F(11) + F(12) + F(15) + F(16)) +
                                      (F(0) + F(1) + F(2) + F(3) + F(4) + F(7) + F(8) + F(9) + F(10)));
  } else {
    s->uz[nd] = -1. + (1. / rho_bc) *
                          (2.0 * (F(5) + F(11) + F(13) + F(15) + F(17) + F(19) + F(21) + F(23) + F(25)) +
                           (F(0) + F(1) + F(2) + F(3) + F(4) + F(7) + F(8) + F(9) + F(10)));
  }
}
#undef F

/* non-equilibrium bounce-back of the unknown speeds: f[sp] = feq[sp] + f[bb] - feq[bb] */
static void nebb(const oracle_state* s, real* f, const real* feq, int64_t nd, const int* sp,
                 const int* bbp) {
  const int q = s->L.q;
  for (int k = 0; k < s->L.nbb; ++k)
    f[nd * q + sp[k]] = feq[nd * q + sp[k]] + f[nd * q + bbp[k]] - feq[nd * q + bbp[k]];
}

/* set_uz_bc (include/LatticeStructure.hpp:167-177): reads uy[spd] -- the uy of node number
 * `spd` -- where uy[nd] was presumably meant; restated as written. */
static void set_uz_bc(const oracle_state* s, real* f, int64_t nd) {
  const lattice_t* L = &s->L;
  real u_bc = s->u_lbm;
  for (int i = 0; i < L->q; ++i) {
    f[nd * L->q + i] += 3. * s->rho[nd] * L->w[i] *
                        (L->ez[i] * (u_bc - s->uz[nd]) + L->ex[i] * (0. - s->ux[nd]) +
                         L->ey[i] * (0. - s->uy[i]));
  }
}

/* compute_strain_tensor + apply_turbulence_model (include/LatticeStructure.hpp:106-153) */
static real smagorinsky(const oracle_state* s, const real* f, const real* feq, int64_t nd,
                        real omega) {
  const lattice_t* L = &s->L;
  real S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  real e[3];
  for (int i = 0; i < L->q; ++i) {
    e[0] = L->ex[i]; e[1] = L->ey[i]; e[2] = L->ez[i];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        S[a * 3 + b] += e[a] * e[b] * (f[nd * L->q + i] - feq[nd * L->q + i]);
  }
  real nu, nu_e, P;
  nu = ((1. / omega) - 0.5) / 3.0;
  P = sqrt(S[0] * S[0] + S[4] * S[4] + S[8] * S[8] + 2.0 * (S[1] * S[1] + S[2] * S[2] + S[5] * S[5]));
  P *= s->cs;
  /* The reference calls the unqualified global sqrt, i.e. sqrt(double), even for float
   * `real`: the argument is widened and the subtraction of nu happens in double. */
  P = sqrt(P + nu * nu) - nu;
  nu_e = P / 6.;
  return 1. / (3. * (nu + nu_e) + 0.5);
}

/* relax: BGK (include/LatticeStructure.hpp:156-163) */
static void relax(const oracle_state* s, real* f, const real* feq, int64_t nd, real omega) {
  const int q = s->L.q;
  for (int i = 0; i < q; ++i) {
    int64_t idx = nd * q + i;
    f[idx] = f[idx] - omega * (f[idx] - feq[idx]);
  }
}

/* one node of process_node_list (src/TLBM_Partition.cpp:742-812) */
static void process_node(const oracle_state* s, real* f_out, real* f_in, int64_t nd) {
  const lattice_t* L = &s->L;
  const int q = L->q;
  int t = s->nd_type[nd];
  macro(s, f_in, nd);
  if (t == 0) equilibrium(s, s->f_eq, nd);
  if (t == 1) {
    s->ux[nd] = 0; s->uy[nd] = 0; s->uz[nd] = 0;
    equilibrium(s, s->f_eq, nd);
    bounce_back(s, f_in, nd);
  }
  if (t != 1) {
    if (t == 2) {
      inlet_macro(s, f_in, nd);
      equilibrium(s, s->f_eq, nd);
      nebb(s, f_in, s->f_eq, nd, L->in_sp, L->in_bb);
    }
    if (t == 3) {
      outlet_macro(s, f_in, nd);
      equilibrium(s, s->f_eq, nd);
      nebb(s, f_in, s->f_eq, nd, L->out_sp, L->out_bb);
    }
    if (t == 5) {
      set_uz_bc(s, f_in, nd);
      equilibrium(s, s->f_eq, nd);
    }
    real omega = s->omega;
    if (s->cs > 0) omega = smagorinsky(s, f_in, s->f_eq, nd, omega);
    if (s->dynamics == 1) relax(s, f_in, s->f_eq, nd, omega);
    /* dynamics 2 computes a stress moment and does not relax (:800-804) */
  }
  /* stream_node_data: push (src/TLBM_Partition.cpp:826-837) */
  for (int i = 0; i < q; ++i) {
    int64_t idx = nd * q + i;
    f_out[(int64_t)s->adj[idx] * q + i] = f_in[idx];
  }
}

static int has_type5(const oracle_state* s) {
  for (int64_t nd = 0; nd < s->n; ++nd)
    if (s->nd_type[nd] == 5) return 1;
  return 0;
}

/* take_LBM_time_step (src/TLBM_Partition.cpp:910-947) at one rank. Nodes are independent
 * except through the type-5 quirk (uy of nodes 0..Q-1), so several threads are used only
 * when no type-5 node exists. */
void oracle_step(oracle_state* s, int is_even) {
  if (is_even) { s->f_in = s->f_even; s->f_out = s->f_odd; }
  else { s->f_in = s->f_odd; s->f_out = s->f_even; }
  real* fi = s->f_in;
  real* fo = s->f_out;
  int64_t n = s->n;
  int nt = s->nthreads;
  if (nt > 1 && has_type5(s)) nt = 1;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
  for (int64_t nd = 0; nd < n; ++nd) process_node(s, fo, fi, nd);
  if (s->time_avg) {
    for (int64_t nd = 0; nd < n; ++nd) {
      s->u_avg[nd] += s->ux[nd];
      s->v_avg[nd] += s->uy[nd];
      s->w_avg[nd] += s->uz[nd];
      s->rho_avg[nd] += s->rho[nd];
    }
  }
}

/* load_restart_data (src/TLBM_Partition.cpp:481-540): the restart fields are read as float
 * (NATIVE_FLOAT) into `real` macroscopic arrays, then both population buffers are set to
 * compute_equilibrium of them, node by node. */
void oracle_load_restart(oracle_state* s, const float* ux, const float* uy, const float* uz,
                         const float* rho) {
  for (int64_t nd = 0; nd < s->n; ++nd) {
    s->ux[nd] = ux[nd];
    s->uy[nd] = uy[nd];
    s->uz[nd] = uz[nd];
    s->rho[nd] = rho[nd];
  }
  for (int64_t nd = 0; nd < s->n; ++nd) {
    equilibrium(s, s->f_even, nd);
    equilibrium(s, s->f_odd, nd);
  }
}

/* run steps first_ts .. first_ts+nsteps-1 with take_LBM_time_step(ts % 2) */
void oracle_run(oracle_state* s, int first_ts, int nsteps) {
  for (int ts = first_ts; ts < first_ts + nsteps; ++ts) oracle_step(s, ts % 2);
}

/* calc_force on the populations of the last step (src/TLBM_Partition.cpp:174-208) */
void oracle_force(const oracle_state* s, real* Fx, real* Fy, real* Fz) {
  const lattice_t* L = &s->L;
  const int q = L->q;
  for (int64_t nd = 0; nd < s->n; ++nd) { Fx[nd] = 0; Fy[nd] = 0; Fz[nd] = 0; }
  const real* fo = s->f_out;
  for (int64_t k = 0; k < s->n_force; ++k) {
    int64_t nd = s->force_nodes[k];
    uint32_t m = s->force_mask[k];
    for (int i = 0; i < q; ++i) {
      if (!(m & (1u << i))) continue;
      int64_t idx = nd * q + i;
      int b = L->bb[i];
      int64_t ngb = s->adj[idx];
      real f1 = fo[idx];
      real f2 = fo[ngb * q + b];
      Fx[nd] += L->ex[b] * (f1 + f2);
      Fy[nd] += L->ey[b] * (f1 + f2);
      Fz[nd] += L->ez[b] * (f1 + f2);
    }
  }
}

void oracle_macros(const oracle_state* s, real* ux, real* uy, real* uz, real* rho) {
  size_t b = sizeof(real) * (size_t)s->n;
  if (ux) memcpy(ux, s->ux, b);
  if (uy) memcpy(uy, s->uy, b);
  if (uz) memcpy(uz, s->uz, b);
  if (rho) memcpy(rho, s->rho, b);
}

void oracle_time_avg(const oracle_state* s, real* u, real* v, real* w, real* r) {
  if (!s->time_avg) return;
  size_t b = sizeof(real) * (size_t)s->n;
  memcpy(u, s->u_avg, b); memcpy(v, s->v_avg, b); memcpy(w, s->w_avg, b); memcpy(r, s->rho_avg, b);
}

/* populations in reference layout: which=0 the buffer streamed into by the last step (fOut),
 * which=1 the other buffer (fIn, holding post-collision values) */
void oracle_populations(const oracle_state* s, int which, real* out) {
  memcpy(out, which == 0 ? s->f_out : s->f_in, sizeof(real) * (size_t)(s->n * s->L.q));
}

/* neighbour table adj[node*Q + speed] (global node numbers) */
void oracle_adjacency(const oracle_state* s, int32_t* out) {
  memcpy(out, s->adj, sizeof(int32_t) * (size_t)(s->n * s->L.q));
}

int64_t oracle_num_force_nodes(const oracle_state* s) { return s->n_force; }

/* ------------------------------------------------------------------ file-driven run */

/* Problem::load_input: 23 whitespace-separated tokens (src/Problem.cpp:5-32). */
typedef struct {
  char lattice[128];
  int dynamics, num_ts, ts_rep_freq, warmup_ts, plot_freq;
  real cs, rho_lbm, u_lbm, omega;
  int nx, ny, nz, restart, time_avg;
} oracle_params;

static int read_params(const char* dir, oracle_params* p) {
  char path[4096], tok[23][128];
  snprintf(path, sizeof(path), "%s/params.lbm", dir);
  FILE* fh = fopen(path, "r");
  if (!fh) return -1;
  int k = 0;
  while (k < 23 && fscanf(fh, "%127s", tok[k]) == 1) ++k;
  fclose(fh);
  if (k < 15) return -2;
  snprintf(p->lattice, sizeof(p->lattice), "%s", tok[0]);
  p->dynamics = atoi(tok[1]); p->num_ts = atoi(tok[2]); p->ts_rep_freq = atoi(tok[3]);
  p->warmup_ts = atoi(tok[4]); p->plot_freq = atoi(tok[5]);
  p->cs = REAL_SCAN(tok[6]); p->rho_lbm = REAL_SCAN(tok[7]); p->u_lbm = REAL_SCAN(tok[8]);
  p->omega = REAL_SCAN(tok[9]);
  p->nx = atoi(tok[10]); p->ny = atoi(tok[11]); p->nz = atoi(tok[12]);
  p->restart = atoi(tok[13]); p->time_avg = atoi(tok[14]);
  return 0;
}

static int32_t* read_ints(const char* dir, const char* name, int64_t n) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE* fh = fopen(path, "r");
  if (!fh) return NULL;
  int32_t* a = (int32_t*)calloc((size_t)n, sizeof(int32_t));
  int64_t i = 0;
  int v;
  while (i < n && fscanf(fh, "%d", &v) == 1) a[i++] = v;
  fclose(fh);
  return a;
}

/* MPI_File_write_at semantics at each rank's offset: create, no truncation */
static void write_at(const char* dir, const char* name, const void* buf, size_t bytes, size_t off) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  int fd = open(path, O_WRONLY | O_CREAT, 0644);
  if (fd < 0) return;
  ssize_t w = pwrite(fd, buf, bytes, (off_t)off);
  (void)w;
  close(fd);
}

/* Partition-major output order: nodes sorted by (partition id, global id); each rank writes
 * its nodes at writeOffset = sum of smaller partitions' sizes (src/TLBM_Partition.cpp:210-252,
 * :542-561, :608-683). */
static int64_t* output_order(const int32_t* parts, int64_t n, int nparts) {
  int64_t* count = (int64_t*)calloc((size_t)nparts + 1, sizeof(int64_t));
  for (int64_t g = 0; g < n; ++g) count[parts[g] + 1]++;
  for (int p = 0; p < nparts; ++p) count[p + 1] += count[p];
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  for (int64_t g = 0; g < n; ++g) order[count[parts[g]]++] = g;
  free(count);
  return order;
}

static void write_field(const char* dir, const char* name, const real* a, const int64_t* order,
                        int64_t n) {
  real* tmp = (real*)malloc(sizeof(real) * (size_t)n);
  for (int64_t k = 0; k < n; ++k) tmp[k] = a[order[k]];
  write_at(dir, name, tmp, sizeof(real) * (size_t)n, 0);
  free(tmp);
}

/* The tLBMexec flow (src/tLBM.cpp:7-88) driven by the files in `dir`: read inputs, write
 * ordering.b_dat, step num_ts times, dump on (ts+1)%plotFreq==0 && ts+1>warmupTs, write time
 * averages when the flag is set.  `nthreads` spreads the node loop over host cores.
 * Returns 0, or a negative code on input errors; *elapsed gets the step-loop wall time. */
int oracle_run_dir(const char* dir, int nthreads, double* elapsed) {
  oracle_params p;
  if (read_params(dir, &p)) return -1;
  int q = 0;
  if (!strcmp(p.lattice, "D3Q15")) q = 15;
  else if (!strcmp(p.lattice, "D3Q19")) q = 19;
  else if (!strcmp(p.lattice, "D3Q27")) q = 27;
  else return -2;
  int64_t n = (int64_t)p.nx * p.ny * p.nz;
  int32_t* nd = read_ints(dir, "ndType.lbm", n);
  int32_t* parts = read_ints(dir, "parts.lbm", n);
  if (!nd || !parts) { free(nd); free(parts); return -3; }
  int nparts = 1;
  for (int64_t g = 0; g < n; ++g) {
    if (parts[g] < 0) { free(nd); free(parts); return -4; }
    if (parts[g] + 1 > nparts) nparts = parts[g] + 1;
  }
  oracle_state* s = oracle_create(q, p.dynamics, p.cs, p.rho_lbm, p.u_lbm, p.omega, p.nx, p.ny,
                                  p.nz, nd, p.time_avg);
  oracle_set_threads(s, nthreads);
  if (p.restart) {
    /* restart fields as raw float32 files in global order (the reference's restart.h5 holds
     * the same datasets: velocity/x,y,z and density/rho) */
    static const char* names[4] = {"restart_ux.b_dat", "restart_uy.b_dat", "restart_uz.b_dat",
                                   "restart_rho.b_dat"};
    float* r[4] = {NULL, NULL, NULL, NULL};
    int ok = 1;
    for (int k = 0; k < 4; ++k) {
      char path[4096];
      snprintf(path, sizeof(path), "%s/%s", dir, names[k]);
      FILE* fh = fopen(path, "rb");
      r[k] = (float*)malloc(sizeof(float) * (size_t)n);
      if (!fh || fread(r[k], sizeof(float), (size_t)n, fh) != (size_t)n) ok = 0;
      if (fh) fclose(fh);
    }
    if (ok) oracle_load_restart(s, r[0], r[1], r[2], r[3]);
    for (int k = 0; k < 4; ++k) free(r[k]);
    if (!ok) {
      oracle_destroy(s);
      free(nd);
      free(parts);
      return -5;
    }
  }
  int64_t* order = output_order(parts, n, nparts);
  int32_t* ord32 = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  for (int64_t k = 0; k < n; ++k) ord32[k] = (int32_t)order[k];
  write_at(dir, "ordering.b_dat", ord32, sizeof(int32_t) * (size_t)n, 0);
  free(ord32);
  real *Fx = (real*)malloc(sizeof(real) * n), *Fy = (real*)malloc(sizeof(real) * n),
       *Fz = (real*)malloc(sizeof(real) * n);
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  int dump = 0;
  char name[256];
  for (int ts = 0; ts < p.num_ts; ++ts) {
    oracle_step(s, ts % 2);
    if (((ts + 1) % p.plot_freq == 0) && (ts + 1 > p.warmup_ts)) {
      snprintf(name, sizeof(name), "ux%d.b_dat", dump); write_field(dir, name, s->ux, order, n);
      snprintf(name, sizeof(name), "uy%d.b_dat", dump); write_field(dir, name, s->uy, order, n);
      snprintf(name, sizeof(name), "uz%d.b_dat", dump); write_field(dir, name, s->uz, order, n);
      snprintf(name, sizeof(name), "density%d.b_dat", dump); write_field(dir, name, s->rho, order, n);
      oracle_force(s, Fx, Fy, Fz);
      snprintf(name, sizeof(name), "Fx%d.b_dat", dump); write_field(dir, name, Fx, order, n);
      snprintf(name, sizeof(name), "Fy%d.b_dat", dump); write_field(dir, name, Fy, order, n);
      snprintf(name, sizeof(name), "Fz%d.b_dat", dump); write_field(dir, name, Fz, order, n);
      ++dump;
    }
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (elapsed) *elapsed = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  if (p.time_avg) {
    write_field(dir, "uAvg.b_dat", s->u_avg, order, n);
    write_field(dir, "vAvg.b_dat", s->v_avg, order, n);
    write_field(dir, "wAvg.b_dat", s->w_avg, order, n);
    write_field(dir, "rhoAvg.b_dat", s->rho_avg, order, n);
  }
  free(Fx); free(Fy); free(Fz); free(order); free(nd); free(parts);
  oracle_destroy(s);
  return 0;
}
