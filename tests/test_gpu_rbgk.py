"""Regularised BGK (dynamics 2 with tlbm_options.rbgk): one collision on an all-fluid periodic
box against the projection computed in numpy, and the boundary path against plain BGK where
the two coincide (omega = 1)."""

import numpy as np
import pytest

import tlbm_gb300 as T
from tlbm_gb300 import build as B
from tlbm_gb300 import geometry as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    T.library()


def lattice_from_adjacency(part, nx, ny, q):
    c = 1 + nx + nx * ny
    n = part.n
    tgt = part.adjacency().reshape(n, q)[c]
    return np.stack([tgt % nx - 1, (tgt // nx) % ny - 1, tgt // (nx * ny) - 1], axis=1)


@pytest.mark.parametrize("q", [15, 19, 27])
@pytest.mark.parametrize("precision,tol", [("f64", 1e-14), ("f32", 2e-7)])
def test_regularized_collision_matches_numpy(q, precision, tol):
    nx, ny, nz = 32, 6, 5
    g = G.Geometry(nx, ny, nz, np.zeros(nx * ny * nz, np.int32))
    p = G.params_lattice_units(g, "D3Q%d" % q, 0.05, 60.0, 6.0, 10)
    p.omega, p.dynamics = 1.7, 2
    n = g.num_nodes
    part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision=precision,
                                       arithmetic="fast", rbgk=True)
    rng = np.random.default_rng(q)
    part.load_restart(rng.uniform(-0.04, 0.04, n), rng.uniform(-0.04, 0.04, n),
                      rng.uniform(-0.04, 0.04, n), rng.uniform(0.99, 1.01, n))
    part.run(0, 2)  # equilibrium start: the first collision leaves it, streaming does not
    f = part.populations(0).reshape(n, q).astype(np.float64)
    e = lattice_from_adjacency(part, nx, ny, q).astype(np.float64)
    e2 = (e * e).sum(1)
    w = {15: {0: 2 / 9, 1: 1 / 9, 3: 1 / 72}, 19: {0: 1 / 3, 1: 1 / 18, 2: 1 / 36},
         27: {0: 8 / 27, 1: 2 / 27, 2: 1 / 54, 3: 1 / 216}}[q]
    wt = np.array([w[int(k)] for k in e2])
    if q != 27:  # float literals widened (include/D3Q15LatticeStructure.hpp, D3Q19)
        wt = wt.astype(np.float32).astype(np.float64)
    rho = f.sum(1)
    u = (f @ e) / rho[:, None]
    eu = u @ e.T
    feq = wt[None, :] * rho[:, None] * (1 + 3 * eu + 4.5 * eu ** 2 - 1.5 * (u * u).sum(1)[:, None])
    d = f - feq
    pi = np.einsum("ni,ia,ib->nab", d, e, e)
    qdot = np.einsum("ia,ib,nab->ni", e, e, pi) - np.trace(pi, axis1=1, axis2=2)[:, None] / 3
    want = feq + (1 - p.omega) * 4.5 * wt[None, :] * qdot
    part.run(2, 1)
    got = part.populations(1).reshape(n, q).astype(np.float64)
    err = np.abs(got - want).max()
    plain_gap = np.abs(got - (f - p.omega * d)).max()  # distance to plain BGK
    print("D3Q%d %s: max |f - numpy| = %.2e (plain BGK differs by %.2e)"
          % (q, precision, err, plain_gap))
    assert err <= tol
    assert plain_gap > 100 * tol  # the projection changed the result


def test_regularized_equals_bgk_at_unit_omega():
    """At omega = 1 both collisions return feq, so a channel with inlet, outlet and walls must
    give the same fields whether dynamics 2 is regularised or dynamics 1 is plain BGK."""
    g = G.sphere_in_box(16, 12, 30, 3, 8, 6, 10, walls=True)
    p = G.params_lattice_units(g, "D3Q19", 0.05, 40.0, 6.0, 10)
    p.omega = 1.0
    a = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                    arithmetic="fast")
    p.dynamics = 2
    b = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                    arithmetic="fast", rbgk=True)
    a.run(0, 40)
    b.run(0, 40)
    for x, y in zip(a.macros(), b.macros()):
        assert np.allclose(x, y, rtol=0, atol=1e-13)


def test_regularized_needs_fast_arithmetic():
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    p = G.params_lattice_units(g, "D3Q19", 0.04, 20.0, 4.0, 10)
    p.dynamics = 2
    with pytest.raises(T.TLBMError) as e:
        T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                    arithmetic="reference", rbgk=True)
    assert e.value.status == T.ERR_UNSUPPORTED
