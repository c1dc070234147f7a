"""Output-file helpers: read dumps in global order, write restart data, and the gold-standard
check of python/gen_gold_standard.py and python/validate.py.

The solver writes each field in partition-major order with ``ordering.b_dat`` giving the global
node number of every position (src/TLBM_Partition.cpp:542-561, :608-683).  The reference's
``tLBM_create_restart.py`` (python/tLBM_create_restart.py:34-68) un-permutes dump n and stores
velocity/{x,y,z} and density/rho in ``restart.h5``; ``create_restart`` stores the same four
datasets as raw float32 files (``restart_{ux,uy,uz,rho}.b_dat``), which the engine reads when
params.lbm line 14 is 1 (HDF5 is not available to it).
"""

from __future__ import annotations

import os

import numpy as np


def read_dump(workdir: str, dump: int, dtype=np.float32, fields=("ux", "uy", "uz", "density")):
    """Fields of dump `dump` in global node order (the un-permutation of processTLBM.py)."""
    order = np.fromfile(os.path.join(workdir, "ordering.b_dat"), dtype=np.int32)
    out = {}
    for f in fields:
        a = np.fromfile(os.path.join(workdir, "%s%d.b_dat" % (f, dump)), dtype=dtype)
        g = np.zeros_like(a)
        g[order] = a
        out[f] = g
    return out


def create_restart(workdir: str, dump: int, out_dir: str | None = None, dtype=np.float32,
                   fmt: str = "h5"):
    """python/tLBM_create_restart.py: dump `dump` in global order as restart.h5
    (velocity/{x,y,z}, density/rho, float32) -- or, with fmt="raw", as
    restart_{ux,uy,uz,rho}.b_dat."""
    from . import h5

    out_dir = out_dir or workdir
    d = read_dump(workdir, dump, dtype)
    os.makedirs(out_dir, exist_ok=True)
    if fmt == "h5":
        path = os.path.join(out_dir, "restart.h5")
        if os.path.exists(path):  # h5py.File(..., 'w-') refuses an existing file
            raise FileExistsError(path)
        h5.write(path, {"velocity/x": d["ux"].astype(np.float32),
                        "velocity/y": d["uy"].astype(np.float32),
                        "velocity/z": d["uz"].astype(np.float32),
                        "density/rho": d["density"].astype(np.float32)})
        return out_dir
    for src, dst in (("ux", "ux"), ("uy", "uy"), ("uz", "uz"), ("density", "rho")):
        d[src].astype(np.float32).tofile(os.path.join(out_dir, "restart_%s.b_dat" % dst))
    return out_dir


def gold_standard(workdir: str, dump: int, dtype=np.float32) -> np.ndarray:
    """|u| of dump `dump` in global order, as python/gen_gold_standard.py:13-34 computes it
    (float32 squares and sum, float32 sqrt)."""
    d = read_dump(workdir, dump, dtype, fields=("ux", "uy", "uz"))
    return np.sqrt(d["ux"] ** 2 + d["uy"] ** 2 + d["uz"] ** 2)


def validate(workdir: str, dump: int, gold: np.ndarray, dtype=np.float32) -> dict:
    """python/validate.py:14-44: relative and absolute 1-norm differences of |u| of dump
    `dump` against a gold-standard array."""
    umag = gold_standard(workdir, dump, dtype)
    gold = np.asarray(gold)
    dif_abs = float(np.linalg.norm(umag - gold, ord=1))
    norm = float(np.linalg.norm(gold, ord=1))
    return {"l1_test": float(np.linalg.norm(umag, ord=1)), "l1_gold": norm,
            "rel": dif_abs / norm, "abs": dif_abs}
