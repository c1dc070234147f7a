"""The oracle is pinned to the reference: its output files must be byte-identical to the files
the reference solver wrote on the same inputs (SHA-256 digests and fields in tests/golden)."""

import hashlib
import os

import numpy as np
import pytest

from conftest import golden_arrays, golden_cases
import oracle_lib
from tlbm_gb300 import geometry as G

CASES = golden_cases()
SMALL = [k for k, v in CASES.items() if not v["spec"].get("big")]
FIELDS = ("ux", "uy", "uz", "density", "Fx", "Fy", "Fz")


def sha(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def write_case_inputs(name, workdir):
    rec = CASES[name]
    os.makedirs(workdir, exist_ok=True)
    with open(os.path.join(workdir, "params.lbm"), "w") as fh:
        fh.write(rec["params_text"])
    arr = golden_arrays(name)
    nd = arr["ndType"].astype(np.int32)
    with open(os.path.join(workdir, "ndType.lbm"), "wb") as fh:
        fh.write(G._int_lines(nd))
    with open(os.path.join(workdir, "parts.lbm"), "wb") as fh:
        fh.write(G._int_lines(np.zeros_like(nd)))
    assert sha(os.path.join(workdir, "ndType.lbm")) == rec["inputs"]["ndType.lbm"]
    assert sha(os.path.join(workdir, "parts.lbm")) == rec["inputs"]["parts.lbm"]
    return rec


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference_files(name, prec, tmp_path):
    rec = write_case_inputs(name, str(tmp_path))
    oracle_lib.run_dir(str(tmp_path), prec)
    want = rec["outputs"][prec]
    got = {f: sha(os.path.join(str(tmp_path), f)) for f in os.listdir(str(tmp_path))
           if f.endswith(".b_dat")}
    assert sorted(got) == sorted(want)
    bad = [f for f in want if got[f] != want[f]]
    assert not bad, "oracle differs from the reference in %s" % bad


@pytest.mark.parametrize("name", ["q19_sphere_bgk", "q27_sphere_smag", "q19_cavity_lid"])
def test_oracle_fields_match_reference_fields(name):
    """Same check through the in-memory API: last dump's fields equal the reference's."""
    rec = CASES[name]
    spec = rec["spec"]
    arr = golden_arrays(name)
    toks = rec["params_text"].split()
    q = int(toks[0][3:])
    nx, ny, nz = int(toks[10]), int(toks[11]), int(toks[12])
    o = oracle_lib.Oracle(q, int(toks[1]), float(toks[6]), float(toks[7]), float(toks[8]),
                          float(toks[9]), nx, ny, nz, arr["ndType"])
    o.run(rec["last_dump_step"])
    ux, uy, uz, rho = o.macros()
    fx, fy, fz = o.force()
    for fn, a in zip(FIELDS, (ux, uy, uz, rho, fx, fy, fz)):
        np.testing.assert_array_equal(a, arr["f64_" + fn], err_msg=fn)


def test_channel32_inputs_match_reference_pipeline(tmp_path):
    """The numpy generator writes byte-identical inputs to the reference's Python pipeline for
    the 32x32x128 sphere channel."""
    rec = CASES["channel32_q19_2000"]
    g = G.channel_sphere_32x32x128()
    p = G.channel_sphere_32x32x128_params()
    G.write_inputs(str(tmp_path), g, p)
    for f in ("params.lbm", "ndType.lbm", "parts.lbm"):
        assert sha(os.path.join(str(tmp_path), f)) == rec["inputs"][f], f
    assert g.counts() == {0: 112505, 1: 16767, 2: 900, 3: 900}


def test_channel32_2000_steps_fp64_bit_exact(tmp_path):
    """2000 FP64 steps on the 32x32x128 channel: every output byte equals the reference's."""
    rec = CASES["channel32_q19_2000"]
    g = G.channel_sphere_32x32x128()
    G.write_inputs(str(tmp_path), g, G.channel_sphere_32x32x128_params())
    oracle_lib.run_dir(str(tmp_path), "f64", threads=os.cpu_count() or 1)
    for f, h in rec["outputs"]["f64"].items():
        assert sha(os.path.join(str(tmp_path), f)) == h, f
