// fx_harness.cpp -- host check of physics_fx.cuh (the fixed-point FP64-storage collision).
//
//   fx_harness Q SMAG N SEED
//
// For N random near-equilibrium cells (rho in [0.6, 1.6], |u_a| <= 0.2, non-equilibrium parts up
// to 2e-3 w_i) it collides each cell with fx::fluid_collide and with a long-double evaluation of
// the reference's formulas (include/LatticeStructure.hpp:70-163: moments, equilibrium with the
// reference's weights, Smagorinsky rate, BGK relaxation), and prints the largest difference in
// ulps of the result and the share of results that are not the nearest double.  It also checks
// the exact double <-> Q4.59 conversions and the range guards.  Exit status 1 on a failed check.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../tlbm_gb300/csrc/grid.cuh"
#include "../tlbm_gb300/csrc/physics_fx.cuh"

using namespace tlbm;
using LD = long double;

template <class L>
LD w_of(int i) {
  return static_cast<LD>(static_cast<double>(L::wlit(i)));
}

// reference collision in long double, result rounded to double
template <class L>
void collide_exact(const double (&f)[L::Q], bool smag, double omega, double cs, double (&out)[L::Q]) {
  constexpr int Q = L::Q;
  LD rho = 0, jx = 0, jy = 0, jz = 0;
  for (int i = 0; i < Q; ++i) {
    rho += f[i];
    jx += L::ex(i) * static_cast<LD>(f[i]);
    jy += L::ey(i) * static_cast<LD>(f[i]);
    jz += L::ez(i) * static_cast<LD>(f[i]);
  }
  const LD ux = jx / rho, uy = jy / rho, uz = jz / rho;
  LD feq[Q];
  for (int i = 0; i < Q; ++i) {
    const LD cu = 3 * (L::ex(i) * ux + L::ey(i) * uy + L::ez(i) * uz);
    feq[i] = w_of<L>(i) * rho * (1 + cu + 0.5L * cu * cu - 1.5L * (ux * ux + uy * uy + uz * uz));
  }
  LD om = omega;
  if (smag) {
    LD s[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < Q; ++i) {
      const LD d = f[i] - feq[i];
      const int ex = L::ex(i), ey = L::ey(i), ez = L::ez(i);
      s[0] += ex * ex * d;
      s[1] += ey * ey * d;
      s[2] += ez * ez * d;
      s[3] += ex * ey * d;
      s[4] += ex * ez * d;
      s[5] += ey * ez * d;
    }
    const LD nu = (1 / static_cast<LD>(omega) - 0.5L) / 3;
    LD p = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] +
                     2 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]));
    p *= cs;
    p = std::sqrt(p + nu * nu) - nu;
    om = 1 / (3 * (nu + p / 6) + 0.5L);
  }
  for (int i = 0; i < Q; ++i) out[i] = static_cast<double>(f[i] - om * (f[i] - feq[i]));
}

double ulps(double a, double b) {
  if (a == b) return 0;
  const double u = std::nextafter(std::fabs(b), INFINITY) - std::fabs(b);
  return std::fabs(a - b) / u;
}

template <class L>
bool bgk(double (&f)[L::Q], const fx::Consts& k) {
  fx::i64 rq, jq[3];
  return fx::fluid_collide<L, false>(f, k, rq, jq);
}

template <class L>
bool smagorinsky(double (&f)[L::Q], const fx::Consts& k) {
  fx::i64 rq, jq[3];
  return fx::fluid_collide<L, true>(f, k, rq, jq);
}

int fails = 0;
#define CHECK(c, ...)                  \
  do {                                 \
    if (!(c)) {                        \
      std::printf("FAIL: " __VA_ARGS__); \
      std::printf("\n");               \
      ++fails;                         \
    }                                  \
  } while (0)

template <class L>
void run(bool smag, int n, unsigned seed) {
  constexpr int Q = L::Q;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const double omega = 1.9725868, cs = 0.1;
  const double nu = (1.0 / omega - 0.5) / 3.0;
  fx::Consts k;
  fx::fill_consts(k, omega, smag ? cs : 0.0, nu);
  double worst = 0;
  long not_nearest = 0, total = 0, rejected = 0;
  for (int c = 0; c < n; ++c) {
    const LD rho = 1.1L + 0.5L * U(rng);
    const LD u[3] = {0.2L * U(rng), 0.2L * U(rng), 0.2L * U(rng)};
    const LD usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    double f[Q], want[Q];
    for (int i = 0; i < Q; ++i) {
      const LD cu = 3 * (L::ex(i) * u[0] + L::ey(i) * u[1] + L::ez(i) * u[2]);
      const LD feq = w_of<L>(i) * rho * (1 + cu + 0.5L * cu * cu - 1.5L * usq);
      f[i] = static_cast<double>(feq * (1 + 2e-3L * U(rng)));
    }
    collide_exact<L>(f, smag, omega, cs, want);
    // the same populations held as Q1.62 (exact: every value is above 2^-10)
    fx::i64 F[Q];
    for (int i = 0; i < Q; ++i) F[i] = fx::store_of_f64(f[i]);
    fx::i64 rq, jq[3];
    const bool ok_q = smag ? fx::fluid_collide<L, true>(F, k, rq, jq)
                           : fx::fluid_collide<L, false>(F, k, rq, jq);
    const bool ok = smag ? smagorinsky<L>(f, k) : bgk<L>(f, k);
    // the only state the sampling can leave the ranges with: a corner speed's |e.j| near 1
    const double jsum = static_cast<double>(rho * (std::fabs(u[0]) + std::fabs(u[1]) +
                                                   std::fabs(u[2])));
    const bool corner_limit = fx::has_corners<L>() && jsum > 0.93;
    CHECK(ok || corner_limit, "D3Q%d cell %d outside the fixed-point ranges", Q, c);
    CHECK(ok_q == ok, "D3Q%d cell %d: the stored form's guards differ", Q, c);
    if (!ok) {
      ++rejected;
      continue;
    }
    // the stored form keeps the collided Q1.62 values; their nearest doubles are the double
    // form's results
    for (int i = 0; i < Q; ++i)
      CHECK(fx::f64_of_store(F[i]) == f[i], "D3Q%d cell %d speed %d: stored form", Q, c, i);
    for (int i = 0; i < Q; ++i) {
      const double e = ulps(f[i], want[i]);
      worst = e > worst ? e : worst;
      not_nearest += e != 0;
      ++total;
    }
  }
  std::printf("D3Q%d %s: %d cells, largest difference %.3g ulp, %.3g %% not the nearest double\n",
              Q, smag ? "Smagorinsky" : "BGK", n, worst, 100.0 * not_nearest / total);
  CHECK(worst <= 3.0, "D3Q%d %s: %.3g ulp", Q, smag ? "smag" : "bgk", worst);
  CHECK(rejected * 100 <= n, "D3Q%d: %ld of %d cells rejected", Q, rejected, n);
}

void conversions(unsigned seed) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  // doubles with at most 62 fractional bits convert exactly and back
  for (int t = 0; t < 1000000; ++t) {
    const double d = std::ldexp(U(rng), -static_cast<int>(rng() % 11));
    if (std::fabs(d) < 0x1p-10) continue;
    const double back = fx::to_f64(fx::from_f64(d));
    CHECK(back == d, "round trip %.17g -> %.17g", d, back);
    if (fails > 10) return;
  }
  // to_f64 rounds to nearest (ties to even): within half an ulp of the exact value
  for (int t = 0; t < 1000000; ++t) {
    const fx::i64 v = static_cast<fx::i64>(rng()) >> (1 + rng() % 62);
    const LD exact = std::ldexp(static_cast<LD>(v), -62);
    const double got = fx::to_f64(v);
    const LD ulp = static_cast<LD>(std::nextafter(std::fabs(got), INFINITY) - std::fabs(got));
    CHECK(std::fabs(static_cast<LD>(got) - exact) <= ulp / 2, "to_f64(%lld)", v);
    if (fails > 10) return;
  }
  CHECK(fx::from_f64(0.0) == 0 && fx::from_f64(-0.0) == 0 && fx::from_f64(1e-300) == 0, "zero");
  CHECK(fx::from_f64(1.5) == (static_cast<fx::i64>(3) << 61), "1.5");
  CHECK(fx::from_f64(-1.0) == -(static_cast<fx::i64>(1) << 62), "-1");
  // Q1.62 storage: exact above 2^-10 and back, nearest (ties to even) below, NaN marker
  for (int t = 0; t < 1000000; ++t) {
    const double d = std::ldexp(U(rng), -static_cast<int>(rng() % 40));
    const fx::i64 v = fx::store_of_f64(d);
    const LD err = std::fabs(std::ldexp(static_cast<LD>(v), -62) - static_cast<LD>(d));
    CHECK(err <= 0x1p-63L, "store_of_f64(%.17g)", d);
    if (err == 0x1p-63L) CHECK((v & 1) == 0, "store_of_f64 tie %.17g", d);
    if (std::fabs(d) >= 0x1p-10) CHECK(fx::f64_of_store(v) == d, "storage round trip %.17g", d);
    if (fails > 10) return;
  }
  CHECK(fx::store_of_f64(1.9999999999999998) == 0x7FFFFFFFFFFFFC00LL, "below 2");
  CHECK(fx::store_of_f64(-1.9999999999999998) == -0x7FFFFFFFFFFFFC00LL, "above -2");
  CHECK(fx::store_of_f64(2.0) == fx::kStoreNaN && fx::store_of_f64(-2.0) == fx::kStoreNaN &&
            fx::store_of_f64(NAN) == fx::kStoreNaN && fx::store_of_f64(INFINITY) == fx::kStoreNaN,
        "out of range -> NaN marker");
  CHECK(std::isnan(fx::f64_of_store(fx::kStoreNaN)), "NaN marker reads as NaN");
  CHECK(fx::f64_of_store(fx::store_of_f64(0.0)) == 0.0 && fx::store_of_f64(-0.0) == 0, "zero");
  // 1/(2 rho) to 2^-59 over the accepted density range
  for (int t = 0; t < 200000; ++t) {
    const fx::i64 rq = static_cast<fx::i64>(std::ldexp(1.25 + 0.75 * U(rng), 59));
    const LD r = std::ldexp(static_cast<LD>(fx::recip2_q63(rq)), -63);
    const LD want = 1 / (2 * std::ldexp(static_cast<LD>(rq), -59));
    CHECK(std::fabs(r - want) <= 0x1p-58L, "recip2 %lld", rq);
    if (fails > 10) return;
  }
  std::printf("conversions: checked\n");
}

template <class L>
void guards() {
  constexpr int Q = L::Q;
  fx::Consts k;
  fx::fill_consts(k, 1.5, 0.0, (1.0 / 1.5 - 0.5) / 3.0);
  double f[Q];
  for (int i = 0; i < Q; ++i) f[i] = static_cast<double>(L::wlit(i));
  f[0] = 1.0;  // the rest population at its limit
  CHECK(!bgk<L>(f, k) && f[0] == 1.0, "guard f_0 < 1");
  for (int i = 0; i < Q; ++i) f[i] = static_cast<double>(L::wlit(i));
  f[0] = -0.01;
  CHECK(!bgk<L>(f, k), "guard f_0 >= 0");
  for (int i = 0; i < Q; ++i) f[i] = static_cast<double>(L::wlit(i));
  f[1] = 0.5;  // a moving population at its limit
  CHECK(!bgk<L>(f, k), "guard |f_i| < 1/2");
  for (int i = 0; i < Q; ++i) f[i] = 0.3 * static_cast<double>(L::wlit(i));  // rho = 0.3
  CHECK(!bgk<L>(f, k), "guard rho >= 1/2");
  for (int i = 0; i < Q; ++i) f[i] = static_cast<double>(L::wlit(i));
  f[1] = NAN;
  CHECK(!bgk<L>(f, k), "guard NaN");
  for (int i = 0; i < Q; ++i) f[i] = static_cast<double>(L::wlit(i));
  f[1] += 0.4;  // speed 1 has ex = +1: jx = 0.4 > 0.234 rho (rho = 1.4)
  CHECK(!bgk<L>(f, k), "guard |j| < 0.234 rho");
  for (int i = 0; i < Q; ++i) f[i] = 1.5 * static_cast<double>(L::wlit(i));
  f[1] += 0.3;  // rho = 1.8, jx = 0.3 < 0.234 rho: accepted
  CHECK(bgk<L>(f, k), "|j| < 0.234 rho accepted at rho 1.8");
  for (int i = 0; i < Q; ++i) f[i] = static_cast<double>(L::wlit(i));
  f[0] = 0.9;  // rho ~ 1.57 with a rest population above 1/2: accepted
  CHECK(bgk<L>(f, k), "f_0 = 0.9 accepted");
  for (int i = 0; i < Q; ++i) f[i] = static_cast<double>(L::wlit(i));
  CHECK(bgk<L>(f, k), "state at rest accepted");
  // corner speeds: |j_x| + |j_y| + |j_z| < 0.94 (each component inside 0.234 rho)
  // rho = 1.8, j = 0.38 (1, 1, 1): +-0.19 on the axis speeds (each |j_a| < 0.234 rho = 0.42)
  for (int i = 0; i < Q; ++i) {
    f[i] = 1.8 * static_cast<double>(L::wlit(i));
    if (std::abs(L::ex(i)) + std::abs(L::ey(i)) + std::abs(L::ez(i)) == 1)
      f[i] += 0.19 * (L::ex(i) + L::ey(i) + L::ez(i));
  }
  CHECK(bgk<L>(f, k) == !fx::has_corners<L>(), "corner guard (D3Q%d)", Q);
  // the stored form's population guards
  fx::i64 F[Q], rq, jq[3];
  auto rest = [&]() {
    for (int i = 0; i < Q; ++i) F[i] = fx::store_of_f64(static_cast<double>(L::wlit(i)));
  };
  rest();
  F[0] = 1LL << 62;  // f_0 = 1
  CHECK(!(fx::fluid_collide<L, false>(F, k, rq, jq)) && F[0] == (1LL << 62), "stored f_0 < 1");
  rest();
  F[0] = -1;
  CHECK(!(fx::fluid_collide<L, false>(F, k, rq, jq)), "stored f_0 >= 0");
  rest();
  F[1] = 1LL << 61;  // 1/2
  CHECK(!(fx::fluid_collide<L, false>(F, k, rq, jq)), "stored |f_i| < 1/2");
  rest();
  F[2] = -(1LL << 61);
  CHECK(!(fx::fluid_collide<L, false>(F, k, rq, jq)), "stored |f_i| < 1/2 (negative)");
  rest();
  F[Q - 1] = fx::kStoreNaN;
  CHECK(!(fx::fluid_collide<L, false>(F, k, rq, jq)), "stored NaN marker");
  rest();
  CHECK((fx::fluid_collide<L, false>(F, k, rq, jq)), "stored state at rest accepted");
}

// The output fields' helpers: the half-range test, Q5.58 rounding, the pair moments against
// long-double sums, and the two-step neighbour offsets of the force terms against modular
// arithmetic on small lattices (where the wraps interact).
void output_helpers(unsigned seed) {
  std::mt19937_64 rng(seed);
  const fx::i64 half = 1LL << 61;
  const fx::i64 edges[] = {0, 1, -1, half - 1, half, -half, -half + 1, -half - 1, fx::kStoreNaN,
                           0x7FFFFFFFFFFFFFFFLL};
  for (fx::i64 v : edges) {
    const bool beyond = v >= half || v < -half;  // -1/2 <= f < 1/2 passes
    CHECK((fx::beyond_half(v) != 0) == beyond, "beyond_half(%lld)", v);
  }
  for (int t = 0; t < 1000000; ++t) {
    const fx::i64 v = static_cast<fx::i64>(rng()) >> (rng() % 64);
    const bool beyond = v >= half || v < -half;
    CHECK((fx::beyond_half(v) != 0) == beyond, "beyond_half(%lld)", v);
    if (!beyond) {  // nearest multiple of 16 (ties up)
      const fx::i64 r = fx::to58(v);
      CHECK(r * 16 - v >= -7 && r * 16 - v <= 8, "to58(%lld) = %lld", v, r);
    }
    if (fails > 10) return;
  }
  // pair moments of random in-range states: each pair sum rounded once to 2^-59
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  for (int t = 0; t < 100000; ++t) {
    using L = Lattice<19>;
    fx::i64 F[L::Q];
    LD rho = 0, jx = 0, jy = 0, jz = 0;
    for (int i = 0; i < L::Q; ++i) {
      F[i] = static_cast<fx::i64>(std::ldexp(i == 0 ? 0.5 + 0.49 * U(rng) : 0.49 * U(rng), 62));
      const LD v = std::ldexp(static_cast<LD>(F[i]), -62);
      rho += v;
      jx += L::ex(i) * v;
      jy += L::ey(i) * v;
      jz += L::ez(i) * v;
    }
    CHECK(fx::in_q62_ranges<L>(F), "in range");
    fx::i64 r, x, y, z;
    fx::pair_moments<L>(F, r, x, y, z);
    const LD tol = 10 * 0x1p-60L;  // one 2^-60 rounding per pair and the rest population
    CHECK(std::fabs(std::ldexp(static_cast<LD>(r), -59) - rho) <= tol, "rho");
    CHECK(std::fabs(std::ldexp(static_cast<LD>(x), -59) - jx) <= tol, "jx");
    CHECK(std::fabs(std::ldexp(static_cast<LD>(y), -59) - jy) <= tol, "jy");
    CHECK(std::fabs(std::ldexp(static_cast<LD>(z), -59) - jz) <= tol, "jz");
    CHECK(fx::to_f64_58(x) == std::ldexp(fx::to_f64_59(x), 1), "Q5.58 scaling");
    if (fails > 10) return;
  }
  const int sizes[] = {1, 2, 3, 5};
  for (int nx : sizes)
    for (int ny : sizes)
      for (int nz : sizes) {
        const int nxy = nx * ny;
        for (int zz = 0; zz < nz; ++zz)
          for (int yy = 0; yy < ny; ++yy)
            for (int xx = 0; xx < nx; ++xx) {
              const Nbr nb(xx, yy, zz, nx, ny, nz, nxy);
              const Nbr2 n2(nb, nx, ny, nz, nxy);
              for (int i = 0; i < 27; ++i) {
                using L = Lattice<27>;
                const int wx = ((xx + 2 * L::ex(i)) % nx + nx) % nx;
                const int wy = ((yy + 2 * L::ey(i)) % ny + ny) % ny;
                const int wz = ((zz + 2 * L::ez(i)) % nz + nz) % nz;
                CHECK(n2.to2<L>(nb, i) == wx + wy * nx + wz * nxy, "c + 2e_%d at (%d %d %d) of "
                      "%dx%dx%d", i, xx, yy, zz, nx, ny, nz);
              }
            }
        if (fails > 10) return;
      }
  std::printf("output helpers: checked\n");
}

int main(int argc, char** argv) {
  const int q = argc > 1 ? std::atoi(argv[1]) : 19;
  const bool smag = argc > 2 && std::atoi(argv[2]) != 0;
  const int n = argc > 3 ? std::atoi(argv[3]) : 20000;
  const unsigned seed = argc > 4 ? static_cast<unsigned>(std::atoi(argv[4])) : 1u;
  if (q == 0) {
    conversions(seed);
    output_helpers(seed);
    guards<Lattice<15>>();
    guards<Lattice<19>>();
    guards<Lattice<27>>();
  } else if (q == 15) {
    run<Lattice<15>>(smag, n, seed);
  } else if (q == 19) {
    run<Lattice<19>>(smag, n, seed);
  } else {
    run<Lattice<27>>(smag, n, seed);
  }
  return fails ? 1 : 0;
}
