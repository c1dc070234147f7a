"""The numpy input generator against the reference pipeline's files (SHA-256 in tests/golden)
and its own invariants (partition layout, sphere packing)."""

import hashlib
import os

import numpy as np
import pytest

from conftest import golden_cases
from tlbm_gb300 import geometry as G

CASES = golden_cases()


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def gen_case(name):
    spec = CASES[name]["spec"]
    g = spec["geom"]
    if g["kind"] == "sphere":
        geom = G.sphere_channel(g["Lx_p"], g["Ly_p"], g["Lz_p"], g["r"], g["xc"], g["yc"], g["zc"],
                                g["N_divs"], walls=tuple(g["walls"]))
    else:
        geom = G.lid_driven_cavity(n_divs=g["N_divs"])
        geom.p_ref_idx = 0
    p = G.params_from_physical(geom, spec["lattice"], spec["dynamics"], spec["num_ts"],
                               spec.get("ts_rep_freq", spec["num_ts"]), spec["warmup"],
                               spec["plot_freq"], spec["re"], spec["dt"], spec["cs"])
    if spec.get("rho1"):
        p.rho_lbm = 1.0
    return geom, p


@pytest.mark.parametrize("name", sorted(CASES))
def test_inputs_byte_identical_to_reference_pipeline(name, tmp_path):
    geom, p = gen_case(name)
    G.write_inputs(str(tmp_path), geom, p)
    want = CASES[name]["inputs"]
    for f in ("params.lbm", "ndType.lbm", "parts.lbm"):
        assert sha(os.path.join(str(tmp_path), f)) == want[f], f


def test_partition_1d_matches_geometric_rule():
    # z-slabs; Nz % p leading slabs get one more layer (python/partition_compare.py:49-95)
    p = G.partition_1d(3, 2, 10, 4).reshape(10, 2, 3)
    sizes = [int((p[:, 0, 0] == k).sum()) for k in range(4)]
    assert sizes == [3, 3, 2, 2]
    assert (p == p[:, :1, :1]).all()


def test_partition_3d_block_order():
    p = G.partition_geometric(4, 4, 4, 2, 2, 2).reshape(4, 4, 4)
    # x-blocks fastest, then y, then z
    assert p[0, 0, 0] == 0 and p[0, 0, 3] == 1 and p[0, 3, 0] == 2 and p[3, 0, 0] == 4


def test_random_sphere_pack_reaches_porosity():
    g = G.random_sphere_pack(64, 48, 96, 4, 8, porosity=0.7, seed=3)
    solid = (g.nd_type == G.SOLID).mean()
    assert abs(solid - 0.3) < 0.02
    assert g.meta["n_spheres"] > 3
    nd = g.nd_type.reshape(96, 48, 64)
    assert set(np.unique(nd[0])) <= {G.INLET, G.SOLID}
    assert set(np.unique(nd[-1])) <= {G.OUTLET, G.SOLID}
    # seeded: the same seed gives the same geometry
    g2 = G.random_sphere_pack(64, 48, 96, 4, 8, porosity=0.7, seed=3)
    assert np.array_equal(g.nd_type, g2.nd_type)


def test_params_text_roundtrip():
    g = G.channel_sphere_32x32x128()
    p = G.channel_sphere_32x32x128_params()
    toks = p.text().split()
    assert len(toks) == 23
    assert toks[0] == "D3Q19" and toks[8] == "0.05" and toks[9] == "1.69492"
    assert (int(toks[10]), int(toks[11]), int(toks[12])) == (32, 32, 128)
