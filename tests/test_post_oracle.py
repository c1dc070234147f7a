"""The post-processing oracle against processTLBM.py's own output (post_case.npz, written by
tests/golden/make_post_golden.py from the reference script)."""

import os

import numpy as np

import post_oracle as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "post_case.npz")


def case():
    z = np.load(GOLDEN)
    return z, P.parse_params(str(z["params"]))


def test_oracle_matches_processtlbm_bitwise():
    z, p = case()
    order = z["in:ordering.b_dat"]
    nd = (p["num_ts"] - p["warmup"]) // p["plot_freq"]
    for i in range(nd):
        f = {k: z["in:%s%d.b_dat" % (k, i)] for k in ("ux", "uy", "uz", "density", "Fx", "Fy", "Fz")}
        o = P.process(p, order, f["ux"], f["uy"], f["uz"], f["density"], f["Fx"], f["Fy"], f["Fz"])
        for k in P.DUMP_PLANES:
            want = z["out:out%d.h5:%s" % (i, P.H5_NAME[k])].reshape(-1)
            assert want.dtype == np.float32 and np.array_equal(o[k].view(np.uint32),
                                                               want.view(np.uint32)), (i, k)
    o = P.process(p, order, z["in:uAvg.b_dat"], z["in:vAvg.b_dat"], z["in:wAvg.b_dat"],
                  z["in:rhoAvg.b_dat"], time_avg=True)
    for k in P.AVG_PLANES:
        want = z["out:timeAvg.h5:%s" % P.H5_NAME[k]].reshape(-1)
        assert np.array_equal(o[k].view(np.uint32), want.view(np.uint32)), k


def test_xdmf_skeleton_strips_data_references_only():
    z, _ = case()
    t = str(z["xmf:data0.xmf"])
    s = P.xdmf_skeleton(t)
    assert "out0.h5" not in s and s.count("DATA") == 8
    assert 'Dimensions="4 5 6"' in s and "0.1 0.1 0.1" in s
