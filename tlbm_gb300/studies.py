"""Accuracy studies of the reduced and fast storage forms against the FP64 reference path.

The FP64 run in the reference's exact arithmetic writes byte-identical results to the CPU
reference (checked by the GPU parity tests), so errors measured against it are errors against
the reference CPU solver.  Each form runs the same lattice for the same number of steps and is
compared on
  * velocity: relative L2 norm of (u - u_ref) over fluid nodes,
  * pressure drop: dp = c_s^2 (mean rho on the first fluid plane after the inlet - mean rho on
    the last plane before the outlet), relative error against the reference's dp,
  * mass: relative change of the FP64 total mass over the run.
"""

from __future__ import annotations

import time

import numpy as np

from . import TLBMPartition, problem_from_params
from . import geometry as G

FORMS = {
    "f64-reference": ("f64", "reference"),
    "f64-fast": ("f64", "fast"),
    "f64-fast-fp64": ("f64", "fast-fp64"),
    "f32": ("f32", "fast"),
    "f16": ("f16", "fast"),
    "bf16": ("bf16", "fast"),
    "bf16m": ("bf16m", "fast"),
}


def pressure_drop(rho: np.ndarray, nd: np.ndarray, nx: int, ny: int, nz: int) -> float:
    r = rho.reshape(nz, ny, nx).astype(np.float64)
    t = nd.reshape(nz, ny, nx)
    a = r[1][t[1] == G.FLUID].mean()
    b = r[nz - 2][t[nz - 2] == G.FLUID].mean()
    return (a - b) / 3.0


def run_form(geom, params, form: str, steps: int, device: int = 0) -> dict:
    prec, arith = FORMS[form]
    part = TLBMPartition.from_arrays(problem_from_params(params), geom.nd_type, precision=prec,
                                     arithmetic=arith, device=device)
    m0 = part.mass()
    t0 = time.perf_counter()
    ms = part.time_steps(0, steps)
    wall = time.perf_counter() - t0
    ux, uy, uz, rho = part.macros()
    m1 = part.mass()
    part.close()
    return {"ux": ux, "uy": uy, "uz": uz, "rho": rho, "ms": ms, "wall_s": wall,
            "mass_drift": (m1 - m0) / m0,
            "mlups": geom.num_nodes * steps / (ms / 1e3) / 1e6}


def compare(res: dict, ref: dict, geom) -> dict:
    fluid = geom.nd_type == G.FLUID
    du = [res[k].astype(np.float64)[fluid] - ref[k].astype(np.float64)[fluid]
          for k in ("ux", "uy", "uz")]
    un = [ref[k].astype(np.float64)[fluid] for k in ("ux", "uy", "uz")]
    l2 = float(np.sqrt(sum((d ** 2).sum() for d in du)) / np.sqrt(sum((u ** 2).sum() for u in un)))
    dp = pressure_drop(res["rho"], geom.nd_type, geom.nx, geom.ny, geom.nz)
    dp_ref = pressure_drop(ref["rho"], geom.nd_type, geom.nx, geom.ny, geom.nz)
    return {"u_l2_rel": l2, "dp": dp, "dp_ref": dp_ref,
            "dp_rel_err": abs(dp - dp_ref) / abs(dp_ref) if dp_ref else float("nan"),
            "finite": bool(np.isfinite(res["ux"]).all())}


def precision_study(geom, params, steps: int,
                    forms=("f64-fast", "f32", "f16", "bf16", "bf16m"),
                    reference: str = "f64-reference", device: int = 0) -> dict:
    """Run every form and the reference form; returns per-form errors, MLUPS and mass drift."""
    ref = run_form(geom, params, reference, steps, device)
    out = {reference: {"mlups": ref["mlups"], "mass_drift": ref["mass_drift"]}}
    for f in forms:
        r = run_form(geom, params, f, steps, device)
        c = compare(r, ref, geom)
        c.update({"mlups": r["mlups"], "mass_drift": r["mass_drift"]})
        out[f] = c
    return out


def sphere_pack_problem(nx=512, ny=256, nz=256, seed=2024, lattice="D3Q19", cs=0.1,
                        u_in=0.04, re=200.0, steps=5000):
    """The sphere-packed channel of the throughput benchmark (porosity 0.7, r ~ U[4, 12])."""
    g = G.random_sphere_pack(nx, ny, nz, 4.0, 12.0, 0.7, seed=seed, max_tries=3_000_000)
    p = G.params_lattice_units(g, lattice, u_in, re, g.lo, steps, cs=cs, rho_lbm=1.0)
    return g, p


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--seed", type=int, default=2024)
    a = ap.parse_args()
    g, p = sphere_pack_problem(a.nx, a.ny, a.nz, a.seed, steps=a.steps)
    res = precision_study(g, p, a.steps)
    print(json.dumps({"workload": "%dx%dx%d sphere pack D3Q19 BGK+Smagorinsky, %d steps"
                      % (a.nx, a.ny, a.nz, a.steps), "porosity": g.meta.get("porosity"),
                      "results": res}, indent=1))
