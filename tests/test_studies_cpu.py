"""The precision study's error measures (tlbm_gb300/studies.py) on synthetic fields: the
relative velocity L2 over fluid nodes and the pressure drop between the planes next to the
inlet and the outlet.  No GPU."""

import numpy as np

from tlbm_gb300 import geometry as G
from tlbm_gb300 import studies as S


def geom_and_fields(nx=4, ny=3, nz=6):
    nd = np.zeros((nz, ny, nx), np.int32)
    nd[0] = G.INLET
    nd[-1] = G.OUTLET
    nd[2, 1, 1] = G.SOLID
    g = G.Geometry(nx, ny, nz, nd.reshape(-1))
    z = np.arange(nz, dtype=np.float64)[:, None, None] * np.ones((nz, ny, nx))
    rho = (1.0 + 0.01 * (nz - z)).reshape(-1)  # falls linearly along z
    ux = np.full(g.num_nodes, 0.01)
    uy = np.zeros(g.num_nodes)
    uz = np.full(g.num_nodes, 0.04)
    return g, {"ux": ux, "uy": uy, "uz": uz, "rho": rho}


def test_pressure_drop_between_the_planes_next_to_inlet_and_outlet():
    g, f = geom_and_fields()
    # planes z = 1 and z = nz - 2: rho 1.05 and 1.02; dp = c_s^2 (1.05 - 1.02)
    assert np.isclose(S.pressure_drop(f["rho"], g.nd_type, g.nx, g.ny, g.nz), 0.01)


def test_compare_measures_fluid_velocity_and_pressure_errors():
    g, ref = geom_and_fields()
    same = S.compare(ref, ref, g)
    assert same["u_l2_rel"] == 0.0 and same["dp_rel_err"] == 0.0 and same["finite"]
    res = {k: v.copy() for k, v in ref.items()}
    res["uz"] = res["uz"] * 1.01  # 1 % on uz everywhere
    solid = g.nd_type == G.SOLID
    res["ux"][solid] = 1e3  # solid nodes are not fluid: ignored
    c = S.compare(res, ref, g)
    want = 0.01 * 0.04 / np.sqrt(0.01 ** 2 + 0.04 ** 2)
    assert np.isclose(c["u_l2_rel"], want)
    res["rho"] = ref["rho"] * 1.0  # unchanged pressure drop
    assert S.compare(res, ref, g)["dp_rel_err"] == 0.0
    res["ux"][:] = np.nan
    assert not S.compare(res, ref, g)["finite"]
