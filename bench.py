#!/usr/bin/env python3
"""Throughput benchmark: D3Q19 MLUPS of the fused stream-collide step and its HBM roofline.

Workload (default): 512x256x256 channel (z streamwise) packed with seeded non-overlapping spheres
of radius U[4,12] to porosity 0.7, periodic in x/y, Zou-He-style velocity inlet u_z=0.04 at z=0
and pressure outlet rho=1 at z=255, Re=200 on the mean sphere diameter, BGK + Smagorinsky
(cs=0.1), FP64 populations.  Inputs (10.2 GB of populations) are far larger than L2, so no L2
flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-timed (CUDA events around K graph-launched
steps on the engine's stream); `e2e` times the same metric through the C ABI from Python: the
lattice is uploaded from host arrays, each step is a tlbm_step call, and every 100 steps the
seven output fields of write_data are read back into page-locked host buffers (the copies
overlap the following steps; the timer stops after every step and copy has finished).  `cpu_baseline` times the CPU
restatement of the reference's timestep (oracle/, array-of-structures push with an int32
neighbour table, OpenMP over nodes) on the host cores on a slab of the same geometry.
"""

from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "D3Q19 MLUPS (% HBM roofline); BF16/learned vs plain FP64 at equal L2 error"
CPU_SAMPLE_NZ = 32


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=30)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--lattice", default="D3Q19")
    ap.add_argument("--precision", default="f64", choices=["f64", "f32", "bf16", "f16", "bf16m"])
    ap.add_argument("--arithmetic", default="fast", choices=["fast", "fast-fp64", "reference"])
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-extras", action="store_true", help="skip e2e, CPU and extra lines")
    return ap.parse_args()


# ----------------------------------------------------------------------------- distributed


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------------------- workload


def workload(args):
    from tlbm_gb300 import geometry as G

    key = "%d_%d_%d_%d" % (args.nx, args.ny, args.nz, args.seed)
    cache = os.path.join("/tmp", "tlbm_bench_geom_%s.npz" % hashlib.md5(key.encode()).hexdigest())
    if os.path.exists(cache):
        z = np.load(cache)
        g = G.Geometry(args.nx, args.ny, args.nz, z["nd"])
        g.meta = json.loads(str(z["meta"]))
        g.lo = g.meta["mean_diameter"]
    else:
        g = G.random_sphere_pack(args.nx, args.ny, args.nz, 4.0, 12.0, 0.7, seed=args.seed,
                                 max_tries=3_000_000)
        try:
            np.savez(cache, nd=g.nd_type.astype(np.int8), meta=json.dumps(g.meta))
        except OSError:
            pass
    g.nd_type = g.nd_type.astype(np.int32)
    p = G.params_lattice_units(g, args.lattice, 0.04, 200.0, g.lo, args.steps, cs=0.1,
                               rho_lbm=1.0, plot_freq=100)
    return g, p


def cpu_sample(g, p, planes=CPU_SAMPLE_NZ):
    """A z-slab of the workload for the CPU baseline: its first `planes` planes, inlet plane
    kept, last plane turned into the outlet."""
    nz = min(planes, g.nz)
    nd = g.nd_type.reshape(g.nz, g.ny, g.nx)[:nz].copy()
    nd[-1][nd[-1] != 1] = 3
    return nd.reshape(-1), nz


# ----------------------------------------------------------------------------- clocks


class ClockSampler:
    """nvidia-smi samples every 200 ms while running (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                if int(parts[0]) != self.index:
                    continue
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "power_w_max": max(power) if power else None,
            "samples": len(sm),
            "reasons": sorted(reasons),
        }


# ----------------------------------------------------------------------------- roofline


def peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cell_bytes(q, precision):
    """Algorithmic bytes of one cell update: read and write Q populations, read the node type;
    the moment-shifted BF16 form also reads and writes a float4 per cell."""
    sb = {"f64": 8, "f32": 4, "bf16": 2, "f16": 2, "bf16m": 2}[precision]
    return 2 * q * sb + 1 + (32 if precision == "bf16m" else 0)


def fp64_pipe_peak(device):
    """DFMA per second of this GPU (the FP64 pipe, which also executes the int64 <-> double
    conversions), measured by the microbenchmark in tlbm_gb300/csrc/peaks.cu; None if it fails."""
    import ctypes

    from tlbm_gb300 import build as B

    try:
        lib = ctypes.CDLL(B.PEAKS_LIB)
    except OSError:
        return None
    out = (ctypes.c_double * 2)()
    if lib.tlbm_peaks_fp64(ctypes.c_int(device), out) != 0:
        return None
    return {"dfma_per_s": float(out[0]), "i2d_per_s": float(out[1])}


def pipe_ops_per_cell(lattice, precision, arithmetic):
    """FP64-pipe thread instructions per cell-update of the step kernel (ncu
    sm__inst_executed_pipe_fp64 x 32 / cells, from the committed summary), if measured."""
    path = os.path.join(HERE, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    v = d.get("%s_%s_%s" % (lattice, precision, arithmetic))
    return None if v is None else v.get("fp64_pipe_ops_per_cell")


def traffic_per_cell(lattice, precision, arithmetic):
    """DRAM bytes per cell-update of the step kernel from the committed ncu summary, if any."""
    path = os.path.join(HERE, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    v = d.get("%s_%s_%s" % (lattice, precision, arithmetic)) or d.get("%s_%s" % (lattice, precision))
    return None if v is None else float(v["dram_bytes_per_cell"])


# ----------------------------------------------------------------------------- arms


def _time_port(g, p, nz, threads, seconds, chunk, warmup):
    """MLUPS of the C restatement of the reference timestep on the first nz planes of the
    workload (cpu_sample), `threads` OpenMP threads, whole chunks of steps until `seconds`."""
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import oracle_lib

    nd, nz = cpu_sample(g, p, nz)
    q = int(p.lattice[3:])
    o = oracle_lib.Oracle(q, 1, p.cs, p.rho_lbm, p.u_lbm, p.omega, g.nx, g.ny, nz, nd,
                          prec="f64", threads=threads)
    o.run(warmup)
    steps = 0
    t0 = time.perf_counter()
    while True:
        o.run(chunk)
        steps += chunk
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    o.close()
    return g.nx * g.ny * nz * steps / dt / 1e6, nz, steps, dt


def cpu_baseline(g, p, seconds=10.0, chunk=10, warmup=2):
    """The CPU restatement of the reference timestep on all host cores, on a z-slab of the
    workload, timed over whole chunks of steps until `seconds` of work have passed; and the same
    on one core (one MPI rank of the reference), on a thinner slab."""
    threads = os.cpu_count() or 1
    value, nz, steps, dt = _time_port(g, p, CPU_SAMPLE_NZ, threads, seconds, chunk, warmup)
    v1, nz1, steps1, dt1 = _time_port(g, p, 4, 1, seconds / 2, 2, 1)
    return {
        "value": round(value, 3),
        "unit": "MLUPS",
        "cores": threads,
        "kind": "port",
        "sample": "%dx%dx%d slab of the same sphere pack (%s FP64 BGK+Smagorinsky), %d warm-up + "
                  "%d timed steps (%.1f s) of the C restatement of the reference timestep "
                  "(AoS push, int32 neighbour table), OpenMP over nodes"
                  % (g.nx, g.ny, nz, p.lattice, warmup, steps, dt),
        "single_core": {"value": round(v1, 3), "unit": "MLUPS", "cores": 1,
                        "sample": "%dx%dx%d slab, 1 warm-up + %d timed steps (%.1f s), one thread"
                                  % (g.nx, g.ny, nz1, steps1, dt1)},
    }


def config_of(args, g, p, dist):
    """The workload both arms report: the sphere pack, its flow and its memory footprint."""
    n = g.num_nodes
    q = int(args.lattice[3:])
    return {
        "workload": "%dx%dx%d sphere-packed channel, %s BGK+Smagorinsky cs=0.1, %s %s "
                    "arithmetic" % (args.nx, args.ny, args.nz, args.lattice, args.precision,
                                    args.arithmetic),
        "cells": n,
        "porosity": round(g.meta.get("porosity", 0.0), 5),
        "spheres": g.meta.get("n_spheres"),
        "re": 200.0,
        "u_in": 0.04,
        "omega": round(p.omega, 6),
        "l2": "populations (%.1f GB) larger than L2; no flush" % (
            n * (cell_bytes(q, args.precision) - 1) / 1e9),
        "parallelism": "replicas only" if dist.world > 1 else "single GPU",
    }


def run_ours(args, dist):
    import tlbm_gb300 as T
    from tlbm_gb300 import build as B

    B.build()
    g, p = workload(args)
    n = g.num_nodes
    q = int(args.lattice[3:])
    prob = T.problem_from_params(p)
    part = T.TLBMPartition.from_arrays(prob, g.nd_type, precision=args.precision,
                                       arithmetic=args.arithmetic, device=dist.local)
    part.run(0, args.warmup)
    part.synchronize()
    dist.barrier()
    part.synchronize()
    clocks = ClockSampler(dist.local)
    clocks.start()
    l0 = part.kernel_launches()
    ms = part.time_steps(args.warmup, args.steps)
    launches = part.kernel_launches() - l0
    clock = clocks.stop()
    part.synchronize()
    dist.barrier()
    ms_max = dist.max(ms)
    mass = part.mass()
    part.close()

    bytes_per_cell = cell_bytes(q, args.precision)
    step_s = ms_max / 1e3 / args.steps
    value = n * args.steps * dist.world / (ms_max / 1e3) / 1e6
    peak, peak_kind = peaks()
    achieved = n * bytes_per_cell / step_s / 1e9
    tpc = traffic_per_cell(args.lattice, args.precision, args.arithmetic)
    pipe = fp64_pipe_peak(dist.local) if args.precision == "f64" else None
    ops = pipe_ops_per_cell(args.lattice, args.precision, args.arithmetic)
    out = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "MLUPS",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_max / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"f64": "f64", "f32": "f32", "bf16": "bf16-storage/f32", "bf16m":
                  "bf16-moment-shifted-storage/f32", "f16":
                  "f16-storage/f32"}[args.precision],
        "data": "synthetic",
        "config": config_of(args, g, p, dist),
        "roofline": {
            "bound": "hbm",
            "achieved": round(achieved, 1),
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "peak_kind": peak_kind,
            "bytes_per_cell": bytes_per_cell,
            "traffic": None if tpc is None else round(tpc * n),
        },
        "gpu_launches": launches,
        "clocks": clock,
        "final_mass": mass,
    }
    if pipe is not None:
        # the FP64 pipe (FMA, conversions): its measured rate and this kernel's use of it
        fp = {"unit": "op/s", "peak": pipe["dfma_per_s"], "peak_kind": "measured (peaks.cu)",
              "ops_per_cell": ops}
        if ops is not None:
            fp["achieved"] = ops * n / step_s
            fp["frac"] = round(fp["achieved"] / pipe["dfma_per_s"], 4)
        out["roofline"]["fp64_pipe"] = fp
    if not args.no_extras:
        out["e2e"] = e2e(args, g, p, dist)
        if dist.rank == 0 and dist.world == 1:
            out["cpu_baseline"] = cpu_baseline(g, p)
            out["extras"] = extras(args, g, p, dist)
    return out


def variant_line(g, p, lattice, precision, arithmetic, steps, device):
    """MLUPS and HBM fraction of one storage/lattice form on the same geometry."""
    import tlbm_gb300 as T
    from tlbm_gb300 import geometry as G

    pv = G.params_lattice_units(g, lattice, p.u_lbm, 200.0, g.lo, steps, cs=p.cs, rho_lbm=1.0)
    part = T.TLBMPartition.from_arrays(T.problem_from_params(pv), g.nd_type, precision=precision,
                                       arithmetic=arithmetic, device=device)
    part.run(0, 4)
    ms = part.time_steps(4, steps)
    part.close()
    q = int(lattice[3:])
    bpc = cell_bytes(q, precision)
    mlups = g.num_nodes * steps / (ms / 1e3) / 1e6
    peak, _ = peaks()
    return {"lattice": lattice, "precision": precision, "arithmetic": arithmetic,
            "mlups": round(mlups, 1),
            "hbm_frac": round(mlups * 1e6 * bpc / 1e9 / peak, 4)}


def ensemble_line(device, steps=200, seed=7):
    """The 64-channel batched ensemble (FP32, D3Q15/D3Q19 mix): autotuned tile shape, MLUPS."""
    import tlbm_gb300 as T
    from tlbm_gb300 import geometry as G

    chs = G.ensemble_channels(64, seed=seed, num_ts=2000)
    ens = T.Ensemble([T.problem_from_params(pp) for _, pp in chs], [gg.nd_type for gg, _ in chs],
                     precision="f32", device=device)
    tiles = ens.autotune(steps=20)
    ens.run(0, 4)
    l0 = ens.kernel_launches()
    ms = ens.time_steps(4, steps)
    launches = ens.kernel_launches() - l0
    cells = ens.cells
    bytes_step = sum(gg.num_nodes * (2 * int(pp.lattice[3:]) * 4 + 1) for gg, pp in chs)
    finite = all(np.isfinite(ens.mass(k)) for k in range(len(chs)))
    ens.close()
    peak, _ = peaks()
    return {"channels": len(chs), "cells": cells, "steps": steps, "tiles": list(tiles),
            "mlups": round(cells * steps / (ms / 1e3) / 1e6, 1),
            "hbm_frac": round(bytes_step * steps / (ms / 1e3) / 1e9 / peak, 4),
            "launches_per_step": launches / steps, "all_finite": finite}


def closure_line(g, p, device, steps=50, seed=3):
    """Cost per step of the learned closure (tensor-core MLP fused in collide, Smagorinsky floor)
    against plain Smagorinsky on the same geometry, FP32 storage."""
    import tlbm_gb300 as T
    from tlbm_gb300 import geometry as G
    from tlbm_gb300 import mlp_params

    pv = G.params_lattice_units(g, "D3Q19", p.u_lbm, 200.0, g.lo, steps, cs=p.cs, rho_lbm=1.0)
    nu = (1.0 / pv.omega - 0.5) / 3.0
    res = {}
    for name in ("smagorinsky", "learned"):
        part = T.TLBMPartition.from_arrays(T.problem_from_params(pv), g.nd_type, precision="f32",
                                           arithmetic="fast", device=device)
        if name == "learned":
            part.set_closure_mlp(mlp_params.xavier(seed), np.ones(8), np.zeros(8), 1e-4,
                                 3.0 * nu + 0.5 + 1e-6)
        part.run(0, 4)
        res[name] = part.time_steps(4, steps) / steps
        part.close()
    return {"precision": "f32", "ms_per_step": {k: round(v, 4) for k, v in res.items()},
            "learned_over_smagorinsky": round(res["learned"] / res["smagorinsky"], 3),
            "learned_mlups": round(g.num_nodes / (res["learned"] / 1e3) / 1e6, 1),
            "les": les_closure_cost(device)}


def les_closure_cost(device, steps=1000, warm=100):
    """The same comparison on the learned-closure LES itself: 128x64x64 D3Q19 FP32 channel,
    periodic in x/y, Zou-He jet inlet (1 % perturbation) and outlet, Re 3000; Smagorinsky
    cs = 0.1 against the closure with its floor cs = 0.05.  The lattice (80 MB of populations)
    stays in L2, so the Smagorinsky step runs above the HBM rate there."""
    import tlbm_gb300 as T
    from tlbm_gb300 import closure as CL
    from tlbm_gb300 import mlp_params

    cx, cy, cz, u_in, re = 128, 64, 64, 0.05, 3000.0
    res = {}
    for name, cs in (("smagorinsky", 0.1), ("learned", 0.05)):
        g, p = CL.channel(cx, cy, cz, u_in, re, cy, cs=cs)
        part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f32",
                                           arithmetic="fast", device=device)
        CL.start_uniform(part, cx * cy * cz, u_in)
        part.set_inlet_profile(CL.inlet_velocity(cx, cy, 1, u_in, 0.01, 0.5, 11))
        if name == "learned":
            nu = (1.0 / p.omega - 0.5) / 3.0
            part.set_closure_mlp(mlp_params.xavier(3), np.ones(8), np.zeros(8), 1e-4,
                                 3.0 * nu + 0.5 + 1e-6)
        part.run(0, warm)
        res[name] = part.time_steps(warm, steps) / steps
        part.close()
    return {"lattice": "128x64x64", "ms_per_step": {k: round(v, 5) for k, v in res.items()},
            "learned_over_smagorinsky": round(res["learned"] / res["smagorinsky"], 3)}


def extras(args, g, p, dist):
    from tlbm_gb300 import geometry as G
    from tlbm_gb300 import studies

    out = {"lines": []}
    for lat, prec in (("D3Q27", "f64"), ("D3Q19", "f32"), ("D3Q27", "f32"), ("D3Q19", "bf16"),
                      ("D3Q19", "f16"), ("D3Q19", "bf16m")):
        out["lines"].append(variant_line(g, p, lat, prec, "fast", 50, dist.local))
    out["lines"].append(variant_line(g, p, "D3Q19", "f64", "fast-fp64", 20, dist.local))
    out["lines"].append(variant_line(g, p, "D3Q27", "f64", "fast-fp64", 20, dist.local))
    out["lines"].append(variant_line(g, p, "D3Q19", "f64", "reference", 20, dist.local))
    out["ensemble"] = ensemble_line(dist.local)
    out["closure"] = closure_line(g, p, dist.local)
    # storage-precision error after 1000 steps on a 256x128x128 pack, against the FP64
    # reference-exact run (byte-identical to the CPU reference)
    gs = G.random_sphere_pack(256, 128, 128, 4.0, 12.0, 0.7, seed=args.seed)
    ps = G.params_lattice_units(gs, "D3Q19", 0.04, 200.0, gs.lo, 1000, cs=0.1, rho_lbm=1.0)
    res = studies.precision_study(gs, ps, 1000, forms=("f64-fast", "f64-fast-fp64", "f32", "f16",
                                                       "bf16", "bf16m"), device=dist.local)
    out["precision_1000_steps_256x128x128"] = {
        k: {kk: fmt_study(kk, vv) for kk, vv in v.items()} for k, v in res.items()}
    return out


def fmt_study(key, v):
    """Study values as 4 significant digits (errors down to 1e-16 stay visible); MLUPS to 0.1."""
    if not isinstance(v, float):
        return v
    if key == "mlups":
        return round(v, 1)
    return float("%.3e" % v)


def e2e(args, g, p, dist, plot_every=100):
    """Same metric end to end through the C ABI from host buffers: upload the lattice, step with
    one tlbm_step call per step, read the write_data fields back every `plot_every` steps."""
    import tlbm_gb300 as T

    n = g.num_nodes
    steps = args.steps
    # the caller's destinations for the read-back fields: page-locked host buffers, allocated
    # once before the timed region like the reference's own output buffers
    dtype = np.float64 if args.precision == "f64" else np.float32
    host = [T.host_empty(n, dtype) for _ in range(7)]
    dist.barrier()
    t0 = time.perf_counter()
    part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type,
                                       precision=args.precision, arithmetic=args.arithmetic,
                                       device=dist.local)
    t_create = time.perf_counter() - t0
    d2h = 0
    for ts in range(steps):
        part.take_LBM_time_step(ts % 2)
        if (ts + 1) % plot_every == 0 or ts == steps - 1:
            # the fields of this step, copied while the next steps run (the host link ramps
            # up slowly after a stretch without traffic: ~0.1 s for the first 1.9 GB); the
            # last step's fields are always read back, so every run ends with its result in
            # host memory whatever the step count
            fields = part.outputs_async(host)
            d2h += sum(a.nbytes for a in fields)
    part.synchronize()  # every step and every copy done
    dt = time.perf_counter() - t0
    part.close()
    dt = dist.max(dt)
    return {
        "value": round(n * steps * dist.world / dt / 1e6, 2),
        "unit": "MLUPS",
        "h2d_bytes_per_step": round(n / steps),  # the node types, narrowed to bytes on the host
        "d2h_bytes_per_step": round(d2h / steps),
        "seconds": {"total": round(dt, 4), "create": round(t_create, 4)},
        "definition": "the reference's Estimated LPU/s (src/tLBM.cpp:69-73: nodes x steps over "
                      "the time from construction to the end, dumps included), with the dumps "
                      "read back to host memory instead of written to files",
        "includes": "construction (the caller's int32 node types checked and narrowed to "
                    "bytes on the host, uploaded once per run) + %d tlbm_step calls + "
                    "write_data fields (7 x %d values) read back after every %dth step and after "
                    "the last one into page-locked host buffers, each copy overlapping the steps "
                    "after it" % (steps, n, plot_every),
    }


def run_reference(args, dist, budget_s=60.0):
    """The reference's CPU timestep on all host cores, on the whole workload: its C restatement
    in oracle/ (AoS push through an int32 neighbour table, OpenMP over nodes), pinned
    byte-identical to the reference's own build.  That build (oracle/_ref, compiled from the
    reference's sources where they exist) is built for the machine that compiled it; a machine
    of another architecture without those sources can neither run nor rebuild it.  The timed
    steps are the requested ones, or as many as fit `budget_s` seconds at the rate of the
    warm-up steps (a bounded sample of the same run)."""
    g, p = workload(args)
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import oracle_lib

    q = int(args.lattice[3:])
    threads = os.cpu_count() or 1
    o = oracle_lib.Oracle(q, 1, p.cs, p.rho_lbm, p.u_lbm, p.omega, g.nx, g.ny, g.nz, g.nd_type,
                          prec="f64", threads=threads)
    warm = min(args.warmup, 3)
    t0 = time.perf_counter()
    o.run(warm)
    per_step = (time.perf_counter() - t0) / warm
    steps = max(1, min(args.steps, int(budget_s / max(per_step, 1e-9))))
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    o.close()
    cells = g.num_nodes
    value = cells * steps / dt / 1e6
    sample = ("the whole %dx%dx%d sphere pack, FP64 BGK+Smagorinsky, %d warm-up + %d timed steps "
              "(%.1f s) of the C restatement of the reference timestep, OpenMP over nodes"
              % (g.nx, g.ny, g.nz, warm, steps, dt))
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "MLUPS",
        "n_gpus": dist.world,
        "steps": steps,
        "warmup": warm,
        "ms_per_step": round(dt * 1e3 / steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": config_of(args, g, p, dist),
        "cpu_baseline": {"value": round(value, 3), "unit": "MLUPS", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    args = parse_args()
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            if dist.rank == 0:
                print(json.dumps(run_reference(args, dist)), flush=True)
            return
        out = run_ours(args, dist)
        if dist.rank == 0:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
