"""Post-processing on the GPU (processTLBM.py) and sub-space output: bit-exact against the
script's own output (post_case.npz) and against the oracle on real runs."""

import os
import shutil

import numpy as np
import pytest

import post_oracle as P
import tlbm_gb300 as T
from tlbm_gb300 import build as B
from tlbm_gb300 import geometry as G
from tlbm_gb300 import h5

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "post_case.npz")


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    T.library()


def bits(a):
    return np.ascontiguousarray(a, np.float32).reshape(-1).view(np.uint32)


def read_planes(path, names, n, shape=None):
    """The datasets of an out{n}.h5 / timeAvg.h5 file by plane name; pressure and |u| carry the
    script's (nz, ny, nx) shape, the others are flat."""
    out = {}
    for k in names:
        a = h5.read(str(path), P.H5_NAME[k])
        assert a.dtype == np.float32 and a.size == n
        if shape is not None:
            assert a.shape == (shape if k in ("pressure", "velmag") else (n,)), k
        out[k] = a.reshape(-1)
    return out


def test_process_output_dir_matches_processtlbm(tmp_path):
    z = np.load(GOLDEN)
    p = P.parse_params(str(z["params"]))
    (tmp_path / "params.lbm").write_text(str(z["params"]))
    for k in z.files:
        if k.startswith("in:"):
            z[k].tofile(tmp_path / k[3:])
    nd = T.process_output_dir(str(tmp_path))
    assert nd == (p["num_ts"] - p["warmup"]) // p["plot_freq"]
    n = p["nx"] * p["ny"] * p["nz"]
    shape = (p["nz"], p["ny"], p["nx"])
    for i in range(nd):
        got = read_planes(tmp_path / ("out%d.h5" % i), P.DUMP_PLANES, n, shape)
        for k in P.DUMP_PLANES:
            want = z["out:out%d.h5:%s" % (i, P.H5_NAME[k])]
            assert np.array_equal(bits(got[k]), bits(want)), (i, k)
        # the script's XDMF, character for character
        assert (tmp_path / ("data%d.xmf" % i)).read_text() == str(z["xmf:data%d.xmf" % i])
    got = read_planes(tmp_path / "timeAvg.h5", P.AVG_PLANES, n, shape)
    for k in P.AVG_PLANES:
        assert np.array_equal(bits(got[k]), bits(z["out:timeAvg.h5:%s" % P.H5_NAME[k]])), k
    assert (tmp_path / "timeAvg.xmf").read_text() == str(z["xmf:timeAvg.xmf"])


def test_process_output_dir_errors(tmp_path):
    with pytest.raises(T.TLBMError):
        T.process_output_dir(str(tmp_path))  # no params.lbm
    z = np.load(GOLDEN)
    (tmp_path / "params.lbm").write_text(str(z["params"]))
    z["in:ordering.b_dat"][:-1].tofile(tmp_path / "ordering.b_dat")  # wrong size
    with pytest.raises(T.TLBMError):
        T.process_output_dir(str(tmp_path))


def run_with_dumps(d, precision, ss_nodes=(), parts=None):
    rng = np.random.default_rng(5)
    nx, ny, nz = 10, 9, 16
    g = G.sphere_in_box(nx, ny, nz, 2, 5, 4, 6, walls=True)
    p = G.params_lattice_units(g, "D3Q19", 0.05, 40.0, 4.0, 30, cs=0.1, time_avg=1)
    p.num_ts, p.plot_freq, p.warmup_ts = 30, 10, 5
    p.t_conv, p.l_conv, p.p_conv = 0.0125, 0.002, 7.5
    p.lx_p = 0.3
    p.p_ref_idx = int(rng.integers(0, g.num_nodes))
    p.ss_flag = 1 if len(ss_nodes) else 0
    G.write_inputs(d, g, p, parts=parts, ss_nodes=ss_nodes)
    part = T.TLBMPartition(d, precision=precision, arithmetic="reference",
                           size=1 if parts is None else int(parts.max()) + 1)
    for ts in range(p.num_ts):
        part.take_LBM_time_step(ts % 2)
        if (ts + 1) % p.plot_freq == 0 and ts + 1 > p.warmup_ts:
            part.write_data()
            part.write_processed_data()
    part.write_time_avg_data()
    part.write_processed_data(time_avg=True)
    return part, g, p


def test_in_situ_equals_file_processing_and_oracle(tmp_path):
    d1, d2 = str(tmp_path / "run"), str(tmp_path / "files")
    part, g, p = run_with_dumps(d1, "f32")
    part.close()
    os.makedirs(d2)
    for f in os.listdir(d1):
        if f.endswith(".b_dat") or f == "params.lbm":
            shutil.copy(os.path.join(d1, f), d2)
    nd = T.process_output_dir(d2)
    assert nd == 2
    for f in ("out0.h5", "out1.h5", "timeAvg.h5", "data0.xmf", "data1.xmf", "timeAvg.xmf"):
        assert open(os.path.join(d1, f), "rb").read() == open(os.path.join(d2, f), "rb").read(), f
    # oracle on the dump files
    q = P.parse_params(open(os.path.join(d1, "params.lbm")).read())
    order = np.fromfile(os.path.join(d1, "ordering.b_dat"), np.int32)
    n = g.num_nodes

    def rd(name):
        return np.fromfile(os.path.join(d1, name), np.float32)

    for i in range(nd):
        o = P.process(q, order, *[rd("%s%d.b_dat" % (k, i)) for k in
                                  ("ux", "uy", "uz", "density", "Fx", "Fy", "Fz")])
        got = read_planes(os.path.join(d1, "out%d.h5" % i), P.DUMP_PLANES, n)
        for k in P.DUMP_PLANES:
            assert np.array_equal(bits(got[k]), bits(o[k])), (i, k)
    o = P.process(q, order, rd("uAvg.b_dat"), rd("vAvg.b_dat"), rd("wAvg.b_dat"),
                  rd("rhoAvg.b_dat"), time_avg=True)
    got = read_planes(os.path.join(d1, "timeAvg.h5"), P.AVG_PLANES, n)
    for k in P.AVG_PLANES:
        assert np.array_equal(bits(got[k]), bits(o[k])), k


def test_processed_fields_fp64_rounds_then_matches_oracle(tmp_path):
    part, g, p = run_with_dumps(str(tmp_path), "f64")
    ux, uy, uz, rho = part.macros()
    fx, fy, fz = part.force()
    q = P.parse_params(open(str(tmp_path / "params.lbm")).read())
    order = np.arange(g.num_nodes)
    o = P.process(q, order, *[np.asarray(a, np.float64).astype(np.float32)
                              for a in (ux, uy, uz, rho, fx, fy, fz)])
    got = part.processed_fields()
    for k in P.DUMP_PLANES:
        assert np.array_equal(bits(got[k]), bits(o[k])), k
    part.close()


def test_subspace_output_is_the_dump_at_listed_nodes(tmp_path):
    rng = np.random.default_rng(3)
    n = 10 * 9 * 16
    ss = np.sort(rng.choice(n, 37, replace=False))
    parts = (np.arange(n) * 3 // n).astype(np.int32)[::-1].copy()  # scrambled output order
    part, g, p = run_with_dumps(str(tmp_path), "f32", ss_nodes=ss, parts=parts)
    part.close()
    order = np.fromfile(str(tmp_path / "ordering.b_dat"), np.int32)
    for i in range(2):
        for f, s in (("ux", "ss_ux"), ("uy", "ss_uy"), ("uz", "ss_uz"), ("density", "ss_density")):
            dump = np.fromfile(str(tmp_path / ("%s%d.b_dat" % (f, i))), np.float32)
            glob = np.empty_like(dump)
            glob[order] = dump
            got = np.fromfile(str(tmp_path / ("%s%d.b_dat" % (s, i))), np.float32)
            assert np.array_equal(got, glob[ss]), (i, f)
