"""Moment-space collisions: regularised BGK (dynamics 2 with tlbm_options.rbgk) and the two-rate
MRT (dynamics 3 with tlbm_options.mrt).  One collision on an all-fluid periodic
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


@pytest.mark.parametrize("q", [15, 19, 27])
def test_mrt_collision_matches_numpy(q):
    """Dynamics 3 with the mrt option: stress moments at omega, ghost moments at 1.35."""
    nx, ny, nz = 32, 6, 5
    g = G.Geometry(nx, ny, nz, np.zeros(nx * ny * nz, np.int32))
    p = G.params_lattice_units(g, "D3Q%d" % q, 0.05, 60.0, 6.0, 10)
    p.omega, p.dynamics = 1.7, 3
    og = 1.375  # the option is a float: a rate exact in float compares with numpy's double
    n = g.num_nodes
    part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                       arithmetic="fast", mrt=True, ghost_rate=og)
    rng = np.random.default_rng(q + 7)
    part.load_restart(rng.uniform(-0.04, 0.04, n), rng.uniform(-0.04, 0.04, n),
                      rng.uniform(-0.04, 0.04, n), rng.uniform(0.99, 1.01, n))
    part.run(0, 2)
    f = part.populations(0).reshape(n, q).astype(np.float64)
    e = lattice_from_adjacency(part, nx, ny, q).astype(np.float64)
    w = {15: {0: 2 / 9, 1: 1 / 9, 3: 1 / 72}, 19: {0: 1 / 3, 1: 1 / 18, 2: 1 / 36},
         27: {0: 8 / 27, 1: 2 / 27, 2: 1 / 54, 3: 1 / 216}}[q]
    wt = np.array([w[int(k)] for k in (e * e).sum(1)])
    if q != 27:
        wt = wt.astype(np.float32).astype(np.float64)
    rho = f.sum(1)
    u = (f @ e) / rho[:, None]
    eu = u @ e.T
    feq = wt[None, :] * rho[:, None] * (1 + 3 * eu + 4.5 * eu ** 2 - 1.5 * (u * u).sum(1)[:, None])
    d = f - feq
    pi = np.einsum("ni,ia,ib->nab", d, e, e)
    p2 = 4.5 * wt[None, :] * (np.einsum("ia,ib,nab->ni", e, e, pi)
                              - np.trace(pi, axis1=1, axis2=2)[:, None] / 3)
    want = feq + (1 - og) * d + (og - p.omega) * p2
    part.run(2, 1)
    got = part.populations(1).reshape(n, q).astype(np.float64)
    err = np.abs(got - want).max()
    print("D3Q%d MRT: max |f - numpy| = %.2e (BGK differs by %.2e)"
          % (q, err, np.abs(got - (f - p.omega * d)).max()))
    assert err <= 1e-14


def channel_pair(dyn_a, kw_a, dyn_b, kw_b, omega=1.6, steps=40):
    g = G.sphere_in_box(16, 12, 30, 3, 8, 6, 10, walls=True)
    out = []
    for dyn, kw in ((dyn_a, kw_a), (dyn_b, kw_b)):
        p = G.params_lattice_units(g, "D3Q19", 0.05, 40.0, 6.0, 10, cs=0.1)
        p.omega, p.dynamics = omega, dyn
        part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                           arithmetic="fast", **kw)
        part.run(0, steps)
        out.append(part.macros())
        part.close()
    return out


def test_mrt_limits_are_rbgk_and_bgk():
    """Ghost rate 1 is the regularised collision bit for bit; a ghost rate equal to omega is
    BGK up to round-off, on a channel with walls, a sphere, inlet, outlet and Smagorinsky
    (Smagorinsky moves the stress rate away from omega, so only its boundary-free limit is
    exact: the comparison uses cs = 0 for that case)."""
    a, b = channel_pair(3, {"mrt": True, "ghost_rate": 1.0}, 2, {"rbgk": True})
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    a, b = channel_pair(3, {"mrt": True, "ghost_rate": 1.3}, 1, {}, omega=1.6)
    assert max(np.abs(x - y).max() for x, y in zip(a, b)) > 1e-8  # the ghost rate matters


def test_mrt_at_ghost_rate_omega_is_bgk():
    g = G.sphere_in_box(16, 12, 30, 3, 8, 6, 10, walls=True)
    res = []
    for dyn, kw in ((3, {"mrt": True, "ghost_rate": 1.625}), (1, {})):
        p = G.params_lattice_units(g, "D3Q19", 0.05, 40.0, 6.0, 10)
        p.omega, p.dynamics = 1.625, dyn  # exact in float, like the ghost-rate option
        part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                           arithmetic="fast", **kw)
        part.run(0, 40)
        res.append(part.macros())
        part.close()
    for x, y in zip(*res):
        assert np.allclose(x, y, rtol=0, atol=1e-13)


def test_mrt_needs_fast_arithmetic_and_a_valid_rate():
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    p = G.params_lattice_units(g, "D3Q19", 0.04, 20.0, 4.0, 10)
    p.dynamics = 3
    with pytest.raises(T.TLBMError) as e:
        T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                    arithmetic="reference", mrt=True)
    assert e.value.status == T.ERR_UNSUPPORTED
    with pytest.raises(T.TLBMError) as e:
        T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                    arithmetic="fast", mrt=True, ghost_rate=2.5)
    assert e.value.status == T.ERR_INVALID_ARGUMENT
