"""Batched ensembles (one persistent launch per step over many channels): every channel's
fields equal a single-lattice run of the same problem bit for bit, for any tile shape, and the
autotuner leaves the channels in their initial state."""

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


def channels(n=6, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx = int(rng.choice([12, 16, 33]))
        ny = int(rng.choice([9, 16]))
        nz = int(rng.integers(20, 41))
        lat = ["D3Q15", "D3Q19"][k % 2]
        g = G.sphere_in_box(nx, ny, nz, 3.0, nx / 2, ny / 2, nz / 3)
        cs = 0.1 if k % 3 == 0 else 0.0
        p = G.params_lattice_units(g, lat, 0.04, float(rng.uniform(30, 120)), 6.0, 30, cs=cs)
        out.append((g, p))
    return out


def single_runs(chs, steps, precision):
    res = []
    for g, p in chs:
        part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type,
                                           precision=precision, arithmetic="fast")
        part.run(0, steps)
        res.append(part.macros())
        part.close()
    return res


@pytest.mark.parametrize("precision", ["f32", "bf16", "f64"])
def test_ensemble_matches_single_runs(precision):
    chs = channels()
    ens = T.Ensemble([T.problem_from_params(p) for _, p in chs], [g.nd_type for g, _ in chs],
                     precision=precision)
    ens.run(0, 17)
    want = single_runs(chs, 17, precision)
    for k in range(len(chs)):
        for a, b in zip(ens.macros(k), want[k]):
            assert np.array_equal(a, b), k
    assert ens.cells == sum(g.num_nodes for g, _ in chs)
    ens.close()


@pytest.mark.parametrize("tiles", [(32, 4, 1), (64, 2, 2), (128, 1, 1), (32, 8, 3)])
def test_tile_shapes_do_not_change_results(tiles):
    chs = channels(seed=9)
    probs = [T.problem_from_params(p) for _, p in chs]
    nds = [g.nd_type for g, _ in chs]
    a = T.Ensemble(probs, nds)
    a.set_tiles(32, 4, 1)
    a.run(0, 11)
    b = T.Ensemble(probs, nds)
    b.set_tiles(*tiles)
    b.run(0, 11)
    for k in range(len(chs)):
        for x, y in zip(a.macros(k), b.macros(k)):
            assert np.array_equal(x, y)


def test_autotune_restores_initial_state():
    chs = channels(seed=5)
    probs = [T.problem_from_params(p) for _, p in chs]
    nds = [g.nd_type for g, _ in chs]
    a = T.Ensemble(probs, nds)
    bx, by, cpt = a.autotune(steps=4)
    assert bx % 32 == 0 and bx * by <= 256 and 1 <= cpt <= 8
    a.run(0, 9)
    want = single_runs(chs, 9, "f32")
    for k in range(len(chs)):
        for x, y in zip(a.macros(k), want[k]):
            assert np.array_equal(x, y)
    m = a.mass(0)
    assert np.isfinite(m) and m > 0


def test_ensemble_rejects_d3q27():
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    p = G.params_lattice_units(g, "D3Q27", 0.04, 20.0, 4.0, 10)
    with pytest.raises(T.TLBMError) as e:
        T.Ensemble([T.problem_from_params(p)], [g.nd_type])
    assert e.value.status == T.ERR_UNSUPPORTED
