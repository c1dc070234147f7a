#!/usr/bin/env python3
"""Regenerate the golden fixtures in this directory from the reference itself.

Run with ``TLBM_REFERENCE`` naming a reference checkout (required), after
``make -C oracle ref REF=$TLBM_REFERENCE`` has built the reference solver (``oracle/_ref/tLBMexec_f32`` and ``tLBMexec_f64``) from its own sources.

For every case this script

1. builds the inputs with the reference's own pre-processing scripts
   (``FluidChannel`` -> ``write_mat_file``, ``tLBM_partition.py``, ``tLBM_write_params.py``),
   executed unmodified through two shims: an empty ``pyvista`` module (only used by STL
   obstacles) and ``scipy.io.loadmat(..., squeeze_me=True)`` (the scripts call ``float()`` on
   1x1 arrays, which numpy 2 rejects);
2. applies the case's edits to ``params.lbm`` (e.g. the density line set to 1);
3. runs the reference solver in FP32 and FP64 and records every output file.

Outputs: ``cases.json`` (case definitions, SHA-256 of every input and output file) and, for
the small cases, ``<case>.npz`` with the input files and the last dump's fields.
"""

from __future__ import annotations

import contextlib
import hashlib
import io
import json
import os
import runpy
import shutil
import subprocess
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("TLBM_REFERENCE", "")
if not os.path.isdir(os.path.join(REF, "python")):
    sys.exit("make_golden.py: set TLBM_REFERENCE to a reference checkout")
REF_PY = os.path.join(REF, "python")
EXE = {p: os.path.join(REPO, "oracle", "_ref", "tLBMexec_" + p) for p in ("f32", "f64")}

sys.dont_write_bytecode = True  # never leave __pycache__ inside the reference tree

# Each case: geometry call, partition args, write_params args, params edits, run sizes.
# write_params args: lattice dynamics style nprocs Num_ts ts_rep_freq Warmup_ts plot_freq Re dt Cs
#                    Restart TimeAvg SS
SMALL_SPHERE = dict(kind="sphere", Lx_p=11.0, Ly_p=11.0, Lz_p=31.0, r=3, xc=6, yc=6, zc=10,
                    N_divs=7, walls=["left", "right", "top", "bottom"])
CASES = {
    "q19_sphere_bgk": dict(geom=SMALL_SPHERE, lattice="D3Q19", dynamics=1, num_ts=300,
                           plot_freq=100, warmup=0, re=20.0, dt=0.05 / 6.0, cs=0.0, rho1=True),
    # D3Q15 plain BGK diverges near step 160 here (its inlet/outlet pair speeds by z-mirror):
    # stop while the fields are still finite.
    "q15_sphere_bgk": dict(geom=SMALL_SPHERE, lattice="D3Q15", dynamics=1, num_ts=120,
                           plot_freq=40, warmup=0, re=20.0, dt=0.05 / 6.0, cs=0.0, rho1=True),
    "q27_sphere_bgk": dict(geom=SMALL_SPHERE, lattice="D3Q27", dynamics=1, num_ts=300,
                           plot_freq=100, warmup=0, re=20.0, dt=0.05 / 6.0, cs=0.0, rho1=True),
    "q19_sphere_smag": dict(geom=SMALL_SPHERE, lattice="D3Q19", dynamics=1, num_ts=300,
                            plot_freq=150, warmup=100, re=200.0, dt=0.05 / 6.0, cs=0.1,
                            rho1=True),
    "q15_sphere_smag": dict(geom=SMALL_SPHERE, lattice="D3Q15", dynamics=1, num_ts=300,
                            plot_freq=150, warmup=100, re=200.0, dt=0.05 / 6.0, cs=0.1,
                            rho1=True),
    "q27_sphere_smag": dict(geom=SMALL_SPHERE, lattice="D3Q27", dynamics=1, num_ts=300,
                            plot_freq=150, warmup=100, re=200.0, dt=0.05 / 6.0, cs=0.1,
                            rho1=True),
    "q19_periodic_bgk": dict(geom=dict(SMALL_SPHERE, walls=[]), lattice="D3Q19", dynamics=1,
                             num_ts=200, plot_freq=200, warmup=0, re=20.0, dt=0.05 / 6.0,
                             cs=0.0, rho1=True),
    "q19_dyn2": dict(geom=SMALL_SPHERE, lattice="D3Q19", dynamics=2, num_ts=40, plot_freq=20,
                     warmup=0, re=20.0, dt=0.05 / 6.0, cs=0.0, rho1=True),
    "q19_water_rho": dict(geom=SMALL_SPHERE, lattice="D3Q19", dynamics=1, num_ts=100,
                          plot_freq=100, warmup=0, re=20.0, dt=0.05 / 6.0, cs=0.0, rho1=False),
    # The type-5 lid nudge grows without bound within ~20 steps: keep the run short.
    "q19_cavity_lid": dict(geom=dict(kind="cavity", N_divs=10), lattice="D3Q19", dynamics=1,
                           num_ts=12, plot_freq=6, warmup=0, re=100.0, dt=0.05 / 9.0,
                           cs=0.0, rho1=True),
    "q27_cavity_lid": dict(geom=dict(kind="cavity", N_divs=10), lattice="D3Q27", dynamics=1,
                           num_ts=12, plot_freq=6, warmup=0, re=100.0, dt=0.05 / 9.0,
                           cs=0.0, rho1=True),
    # The 32x32x128 sphere channel: D3Q19 BGK, Re=20, u=0.05, rho=1, 2000 steps.
    "channel32_q19_2000": dict(
        geom=dict(kind="sphere", Lx_p=31.0, Ly_p=31.0, Lz_p=127.0, r=6, xc=16, yc=16, zc=32,
                  N_divs=13, walls=["left", "right", "top", "bottom"]),
        lattice="D3Q19", dynamics=1, num_ts=2000, plot_freq=2000, warmup=0, re=20.0,
        dt=0.0041666666666667, cs=0.0, rho1=True, ts_rep_freq=500, big=True),
}

OUT_FIELDS = ("ux", "uy", "uz", "density", "Fx", "Fy", "Fz")


def sha(path: str) -> str:
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


@contextlib.contextmanager
def reference_python(workdir: str):
    """Import path and shims for running the reference's Python scripts in ``workdir``."""
    import scipy.io

    saved_path = list(sys.path)
    saved_mods = dict(sys.modules)
    saved_cwd = os.getcwd()
    saved_loadmat = scipy.io.loadmat
    sys.path.insert(0, REF_PY)
    sys.modules["pyvista"] = types.ModuleType("pyvista")

    def loadmat(name, *a, **k):
        k.setdefault("squeeze_me", True)
        return saved_loadmat(name, *a, **k)

    scipy.io.loadmat = loadmat
    os.chdir(workdir)
    try:
        yield
    finally:
        os.chdir(saved_cwd)
        scipy.io.loadmat = saved_loadmat
        sys.path[:] = saved_path
        for k in list(sys.modules):
            if k not in saved_mods:
                del sys.modules[k]


def run_script(name: str, argv: list[str]) -> None:
    saved = sys.argv
    sys.argv = [name] + argv
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            runpy.run_path(os.path.join(REF_PY, name), run_name="__main__")
    finally:
        sys.argv = saved


def make_inputs(case: dict, workdir: str) -> None:
    g = case["geom"]
    with reference_python(workdir):
        import FluidChannel as fc  # noqa: the reference's module

        with contextlib.redirect_stdout(io.StringIO()):
            if g["kind"] == "sphere":
                obst = fc.SphereObstruction(g["r"], g["xc"], g["yc"], g["zc"])
                ch = fc.FluidChannel(Lx_p=g["Lx_p"], Ly_p=g["Ly_p"], Lz_p=g["Lz_p"], obst=obst,
                                     N_divs=g["N_divs"], wallList=list(g["walls"]))
                ch.write_mat_file("geom")
            else:
                cav = fc.LidDrivenCavity(N_divs=g["N_divs"])
                # LidDrivenCavity.write_mat_file omits pRef_idx and ssNds, which
                # tLBM_write_params.py reads; store the full field set here instead.
                import scipy.io

                scipy.io.savemat("geom.mat", {
                    "Lx_p": cav.Lx_p, "Ly_p": cav.Ly_p, "Lz_p": cav.Lz_p, "Lo": cav.Lo,
                    "Ny_divs": cav.N_divs, "rho_p": cav.rho_p, "nu_p": cav.nu_p,
                    "ndType": list(cav.ndType[:]), "pRef_idx": 0, "ssNds": []})
        run_script("tLBM_partition.py", ["geom.mat", case["lattice"], "1D", "1"])
        run_script("tLBM_write_params.py", [
            "geom.mat", case["lattice"], str(case["dynamics"]), "1D", "1", str(case["num_ts"]),
            str(case.get("ts_rep_freq", case["num_ts"])), str(case["warmup"]),
            str(case["plot_freq"]), repr(case["re"]), repr(case["dt"]), repr(case["cs"]), "0",
            "0", "0"])
    if case.get("rho1"):
        path = os.path.join(workdir, "params.lbm")
        lines = open(path).read().splitlines(keepends=True)
        lines[7] = "1 \n"
        open(path, "w").write("".join(lines))


def run_reference(prec: str, src: str, dst: str) -> dict:
    os.makedirs(dst, exist_ok=True)
    for f in ("params.lbm", "ndType.lbm", "parts.lbm"):
        shutil.copy(os.path.join(src, f), dst)
    res = subprocess.run([EXE[prec]], cwd=dst, capture_output=True, text=True, check=True)
    return {"stdout": res.stdout}


def main() -> None:
    if not all(os.path.exists(e) for e in EXE.values()):
        sys.exit("build the reference first: make -C oracle ref")
    out = {"reference": "stu314159/tLBM", "cases": {}}
    only = set(sys.argv[1:])
    old = {}
    cj = os.path.join(HERE, "cases.json")
    if only and os.path.exists(cj):
        old = json.load(open(cj))["cases"]
    for name, case in CASES.items():
        if only and name not in only:
            if name in old:
                out["cases"][name] = old[name]
            continue
        print("case", name, flush=True)
        tmp = tempfile.mkdtemp(prefix="tlbm_golden_")
        try:
            inp = os.path.join(tmp, "in")
            os.makedirs(inp)
            make_inputs(case, inp)
            rec = {"spec": {k: v for k, v in case.items()}, "inputs": {}, "outputs": {}}
            for f in ("params.lbm", "ndType.lbm", "parts.lbm"):
                rec["inputs"][f] = sha(os.path.join(inp, f))
            rec["params_text"] = open(os.path.join(inp, "params.lbm")).read()
            arrays = {}
            if not case.get("big"):
                arrays["ndType"] = np.loadtxt(os.path.join(inp, "ndType.lbm"), dtype=np.int8)
            for prec in ("f64", "f32"):
                run_dir = os.path.join(tmp, prec)
                run_reference(prec, inp, run_dir)
                files = sorted(f for f in os.listdir(run_dir) if f.endswith(".b_dat"))
                rec["outputs"][prec] = {f: sha(os.path.join(run_dir, f)) for f in files}
                # dumps happen after step ts when (ts+1)%plotFreq==0 and ts+1>warmupTs
                # (src/tLBM.cpp:55-60); the npz keeps the last one
                ndumps = sum(1 for ts in range(case["num_ts"])
                             if (ts + 1) % case["plot_freq"] == 0 and ts + 1 > case["warmup"])
                last = ndumps - 1
                rec["last_dump_step"] = max(ts + 1 for ts in range(case["num_ts"])
                                            if (ts + 1) % case["plot_freq"] == 0
                                            and ts + 1 > case["warmup"])
                dt = np.float64 if prec == "f64" else np.float32
                fields = {fn: np.fromfile(os.path.join(run_dir, "%s%d.b_dat" % (fn, last)), dtype=dt)
                          for fn in OUT_FIELDS}
                rec.setdefault("summary", {})[prec] = {
                    "last_dump": last,
                    "uz_max": float(fields["uz"].max()),
                    "rho_sum": float(fields["density"].astype(np.float64).sum()),
                }
                if not case.get("big"):
                    for fn, a in fields.items():
                        arrays["%s_%s" % (prec, fn)] = a
                    arrays["ordering"] = np.fromfile(os.path.join(run_dir, "ordering.b_dat"),
                                                     dtype=np.int32)
            if arrays:
                np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
            out["cases"][name] = rec
        finally:
            shutil.rmtree(tmp)
    with open(cj, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("wrote", cj)


if __name__ == "__main__":
    main()
