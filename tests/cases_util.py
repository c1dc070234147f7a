"""Shared helpers: golden case inputs, file digests, field comparisons."""

import hashlib
import os

import numpy as np

from conftest import golden_arrays, golden_cases
from tlbm_gb300 import geometry as G

CASES = golden_cases()
SMALL = sorted(k for k, v in CASES.items() if not v["spec"].get("big"))
FIELDS = ("ux", "uy", "uz", "density", "Fx", "Fy", "Fz")


def sha(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def write_case_inputs(name, workdir):
    """The golden case's input files (verified against the reference pipeline's digests)."""
    rec = CASES[name]
    os.makedirs(workdir, exist_ok=True)
    if rec["spec"].get("big"):
        G.write_inputs(workdir, G.channel_sphere_32x32x128(), G.channel_sphere_32x32x128_params())
    else:
        with open(os.path.join(workdir, "params.lbm"), "w") as fh:
            fh.write(rec["params_text"])
        nd = golden_arrays(name)["ndType"].astype(np.int32)
        with open(os.path.join(workdir, "ndType.lbm"), "wb") as fh:
            fh.write(G._int_lines(nd))
        with open(os.path.join(workdir, "parts.lbm"), "wb") as fh:
            fh.write(G._int_lines(np.zeros_like(nd)))
    for f in ("params.lbm", "ndType.lbm", "parts.lbm"):
        assert sha(os.path.join(workdir, f)) == rec["inputs"][f], f
    return rec


def output_digests(workdir):
    return {f: sha(os.path.join(workdir, f)) for f in os.listdir(workdir) if f.endswith(".b_dat")}


def params_tokens(name):
    return CASES[name]["params_text"].split()


def rel_inf(a, b):
    """max |a-b| / max |b| (field-relative error)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))
