"""Dump reading and restart-file writing (python/tLBM_create_restart.py:34-68) on a synthetic
partition-major dump."""

import numpy as np
import pytest

from tlbm_gb300 import h5
from tlbm_gb300 import io as TIO


def test_read_dump_unpermutes_and_create_restart_round_trips(tmp_path):
    rng = np.random.default_rng(4)
    n = 257
    order = rng.permutation(n).astype(np.int32)
    order.tofile(tmp_path / "ordering.b_dat")
    glob = {f: rng.normal(size=n).astype(np.float32) for f in ("ux", "uy", "uz", "density")}
    for f, g in glob.items():
        g[order].tofile(tmp_path / ("%s3.b_dat" % f))  # position i holds node order[i]
    d = TIO.read_dump(str(tmp_path), 3)
    for f in glob:
        assert np.array_equal(d[f], glob[f])
    out = tmp_path / "restart"
    TIO.create_restart(str(tmp_path), 3, str(out))  # restart.h5, as tLBM_create_restart.py
    for src, ds in (("ux", "velocity/x"), ("uy", "velocity/y"), ("uz", "velocity/z"),
                    ("density", "density/rho")):
        r = h5.read(str(out / "restart.h5"), ds)
        assert r.dtype == np.float32 and np.array_equal(r, glob[src])
    with pytest.raises(FileExistsError):  # h5py's mode 'w-'
        TIO.create_restart(str(tmp_path), 3, str(out))
    TIO.create_restart(str(tmp_path), 3, str(out), fmt="raw")
    for src, dst in (("ux", "ux"), ("uy", "uy"), ("uz", "uz"), ("density", "rho")):
        r = np.fromfile(out / ("restart_%s.b_dat" % dst), dtype=np.float32)
        assert np.array_equal(r, glob[src])
