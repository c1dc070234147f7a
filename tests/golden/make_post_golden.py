"""Golden vectors for post-processing: runs the reference's python/processTLBM.py on seeded
synthetic dump files and stores its inputs and outputs in post_case.npz.

processTLBM.py stores its results through h5py (python/hdf5Helper.py:1-56), which is not
installed; a stand-in ``h5py`` module records every dataset the script creates instead.  The
XDMF files the script writes are stored as text.  Run from the repository root:

    python tests/golden/make_post_golden.py /path/to/reference
"""

from __future__ import annotations

import os
import runpy
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

NX, NY, NZ = 6, 5, 4
PARAMS = dict(num_ts=40, ts_rep=10, warmup=10, plot_freq=10, time_avg=1, p_ref_idx=77,
              lx=0.5, ly=0.4, lz=0.3, t_conv=0.0123456789, l_conv=0.00217, p_conv=123.4567)


def params_text(p=PARAMS):
    vals = ["D3Q19", 1, p["num_ts"], p["ts_rep"], p["warmup"], p["plot_freq"], 0.1, 1, 0.05,
            1.7, NX, NY, NZ, 0, p["time_avg"], p["lx"], p["ly"], p["lz"], repr(p["t_conv"]),
            repr(p["l_conv"]), repr(p["p_conv"]), p["p_ref_idx"], 0]
    return "".join("%s \n" % v for v in vals)


def synthetic_inputs(seed=7):
    """Dump files of a run with a scrambled (partition-major) node order."""
    rng = np.random.default_rng(seed)
    n = NX * NY * NZ
    files = {"ordering.b_dat": rng.permutation(n).astype(np.int32)}
    ndumps = (PARAMS["num_ts"] - PARAMS["warmup"]) // PARAMS["plot_freq"]
    for i in range(ndumps):
        for f in ("ux", "uy", "uz"):
            files["%s%d.b_dat" % (f, i)] = rng.normal(0, 0.03, n).astype(np.float32)
        files["density%d.b_dat" % i] = (1 + rng.normal(0, 0.01, n)).astype(np.float32)
        for f in ("Fx", "Fy", "Fz"):
            a = rng.normal(0, 1e-3, n) * (rng.random(n) < 0.3)
            files["%s%d.b_dat" % (f, i)] = a.astype(np.float32)
    for f in ("uAvg", "vAvg", "wAvg"):
        files[f + ".b_dat"] = (rng.normal(0, 0.03, n) * PARAMS["num_ts"]).astype(np.float32)
    files["rhoAvg.b_dat"] = ((1 + rng.normal(0, 0.01, n)) * PARAMS["num_ts"]).astype(np.float32)
    return files


def fake_h5py(store):
    mod = types.ModuleType("h5py")

    class Group:
        def __init__(self, f, name):
            self.f, self.name = f, name

        def create_dataset(self, name, data):
            self.f.data["%s/%s" % (self.name, name)] = np.array(data)

    class File:
        def __init__(self, filename, mode):
            self.filename, self.data = filename, {}

        def create_group(self, name):
            return Group(self, name)

        def close(self):
            store[os.path.basename(self.filename)] = dict(self.data)

    mod.File = File
    return mod


def main(reference):
    script = os.path.join(reference, "python", "processTLBM.py")
    files = synthetic_inputs()
    store = {}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "params.lbm"), "w") as f:
            f.write(params_text())
        for name, a in files.items():
            a.tofile(os.path.join(d, name))
        saved = dict(sys.modules)
        sys.modules["h5py"] = fake_h5py(store)
        sys.path.insert(0, os.path.join(reference, "python"))
        try:
            os.chdir(d)
            runpy.run_path(script, run_name="__main__")
        finally:
            os.chdir(cwd)
            sys.path.pop(0)
            sys.modules.clear()
            sys.modules.update(saved)
        xmf = {n: open(os.path.join(d, n)).read() for n in sorted(os.listdir(d))
               if n.endswith(".xmf")}
    out = {"params": np.array(params_text())}
    for name, a in files.items():
        out["in:" + name] = a
    for h5, ds in store.items():
        for k, v in ds.items():
            out["out:%s:%s" % (h5, k)] = v
    for n, t in xmf.items():
        out["xmf:" + n] = np.array(t)
    np.savez_compressed(os.path.join(HERE, "post_case.npz"), **out)
    print("wrote %d arrays from %d h5 files and %d xmf files" % (len(out), len(store), len(xmf)))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TLBM_REFERENCE", "")
    if not os.path.isdir(os.path.join(ref, "python")):
        sys.exit("make_post_golden.py: pass the reference checkout (or set TLBM_REFERENCE)")
    main(ref)
