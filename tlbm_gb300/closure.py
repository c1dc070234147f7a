"""Learned eddy-viscosity closure: training data from the solver's own fine-grid runs, GPU
training, and evaluation against Smagorinsky on the box-filtered fine solution.

Pipeline (all on the GPU except numpy bookkeeping on coarse-sized arrays):

1. A fine run (factor `f` finer in space and time) of a periodic-x/y box whose Zou-He inlet
   carries a plane jet (u_in (1 + 0.5 J(y)), tanh shear layers) times a seeded, smooth 1 %
   perturbation; snapshots of its macroscopic fields are box-filtered on the device
   (``tlbm_filtered_fields``) to the coarse grid: rho, u and the means of u_a u_b.  The fine
   run relaxes with a constant Smagorinsky coefficient fine_cs (default 0.05): plain BGK at
   the fine tau = 0.5128 of Re = 3000 diverges within ~700 fine steps, first at the
   non-equilibrium bounce-back outlet, once the inlet perturbation's pressure waves reach it
   (measured with and without the perturbation: without it the run stays steady).
2. Per coarse cell the least-squares eddy viscosity that makes the Boussinesq model reproduce
   the filtered sub-grid stress:  nu_t* = -(tau_sgs^dev : S) / (2 S : S),
   tau_sgs_ab = mean(u_a u_b) - mean(u_a) mean(u_b), S the strain rate of the filtered velocity
   (central differences, periodic in x/y).  Clipped to [0, nu_cap].
3. Features are what a coarse LBM node sees when it relaxes with tau* = 3 (nu + nu_t*) + 1/2:
   its non-equilibrium stress Pi_ab = -2 rho c_s^2 tau* S_ab (first-order Chapman-Enskog),
   rho - 1 and |Pi| -- the same quantities the fused collide kernel computes from f - feq.
4. The 8-32-32-1 network is trained on the GPU (``tlbm_mlp_*``: BF16 weights, FP32
   accumulation, Adam) and installed with ``tlbm_set_closure_mlp``; the collide kernel then
   evaluates it on the tensor cores (mlp.cuh: forward_warp).
5. The closure runs as nu_t = max(k out_scale y, nu_smag(cs_floor)): the reference's
   Smagorinsky model is its floor and fallback.  The a-priori target averages ~2 % of nu here
   and sits in the shear layers, while the coarse run at tau = 0.5032 diverges from the outlet
   (acoustic waves meeting the non-equilibrium bounce-back boundaries) unless every strained
   cell gets Smagorinsky-level viscosity (cs >~ 0.02; plain BGK and the regularised collision
   diverge).  ``calibrate`` picks (cs_floor, k) a posteriori against the filtered fine run at
   an earlier snapshot; the floor alone (k = 0) is reported next to the closure so the
   network's own share of the result is visible.
6. Coarse runs with Smagorinsky (cs = 0.1), the learned closure, its floor alone and plain BGK
   are compared with the filtered fine run at the held-out final step on the mean
   streamwise-velocity profile and on the 2-D energy spectrum of u_z in x-y planes.
"""

from __future__ import annotations

import numpy as np

from . import MlpTrainer, TLBMPartition, problem_from_params
from . import geometry as G

CS2 = 1.0 / 3.0


# ----------------------------------------------------------------------------- flow setup


def inlet_noise(nx: int, ny: int, factor: int = 1, modes: int = 24, seed: int = 11,
                kmax: int = 6) -> np.ndarray:
    """Smooth, periodic, zero-mean, unit-std perturbation on an (ny, nx) inlet plane, evaluated
    at cell centres of a grid `factor` times finer than (nx, ny) coarse cells, so the fine and
    coarse inlets carry the same field (the fine one box-filters to the coarse one up to the
    sub-cell variation)."""
    rng = np.random.default_rng(seed)
    fx, fy = nx * factor, ny * factor
    x = (np.arange(fx) + 0.5) / fx
    y = (np.arange(fy) + 0.5) / fy
    X, Y = np.meshgrid(x, y)
    out = np.zeros((fy, fx))
    for _ in range(modes):
        m = int(rng.integers(-kmax, kmax + 1))
        n = int(rng.integers(1, kmax + 1))
        out += rng.normal() * np.sin(2 * np.pi * (m * X + n * Y) + rng.uniform(0, 2 * np.pi))
    out -= out.mean()
    return out / out.std()


def jet_profile(nx: int, ny: int, factor: int = 1, ratio: float = 0.5,
                delta: float = 2.0) -> np.ndarray:
    """Relative inlet excess J(y) in [0, 1] of a plane jet: 1 in the middle half of the
    y-period, 0 outside, joined by tanh shear layers of width `delta` coarse cells; evaluated at
    the cell centres of a grid `factor` times finer.  The inlet velocity is
    u_in (1 + ratio J) (1 + noise)."""
    fy = ny * factor
    y = (np.arange(fy) + 0.5) / factor
    j = 0.5 * (np.tanh((y - ny / 4) / delta) - np.tanh((y - 3 * ny / 4) / delta))
    return ratio * np.tile(j[:, None], (1, nx * factor))


def inlet_velocity(cx, cy, factor, u_in, noise_amp, jet_ratio, seed):
    return (u_in * (1.0 + jet_profile(cx, cy, factor, jet_ratio)) *
            (1.0 + noise_amp * inlet_noise(cx, cy, factor, seed=seed)))


def channel(nx, ny, nz, u_in, re, length, lattice="D3Q19", cs=0.0, steps=1000, rbgk=False):
    """Periodic-x/y box with a z==0 inlet and z==nz-1 outlet (no obstacle); rbgk: dynamics 2,
    run as the regularised BGK collision."""
    nd = np.zeros((nz, ny, nx), np.int32)
    nd[0] = G.INLET
    nd[nz - 1] = G.OUTLET
    g = G.Geometry(nx, ny, nz, nd.reshape(-1))
    p = G.params_lattice_units(g, lattice, u_in, re, length, steps, cs=cs, rho_lbm=1.0)
    if rbgk:
        p.dynamics = 2
    return g, p


# ----------------------------------------------------------------------------- targets / features


def strain(ux, uy, uz):
    """S_ab of a (z, y, x) velocity field: central differences, periodic in x and y,
    one-sided at the z ends.  Returns (xx, yy, zz, xy, xz, yz)."""

    def d(a, axis):
        if axis in (1, 2):
            return 0.5 * (np.roll(a, -1, axis) - np.roll(a, 1, axis))
        return np.gradient(a, axis=0)

    dux = [d(ux, 2), d(ux, 1), d(ux, 0)]
    duy = [d(uy, 2), d(uy, 1), d(uy, 0)]
    duz = [d(uz, 2), d(uz, 1), d(uz, 0)]
    return (dux[0], duy[1], duz[2], 0.5 * (dux[1] + duy[0]), 0.5 * (dux[2] + duz[0]),
            0.5 * (duy[2] + duz[1]))


def sgs_eddy_viscosity(F: dict, nu_cap: float):
    u = [F["ux"].astype(np.float64), F["uy"].astype(np.float64), F["uz"].astype(np.float64)]
    S = strain(*u)
    t = [F["uxux"] - u[0] * u[0], F["uyuy"] - u[1] * u[1], F["uzuz"] - u[2] * u[2],
         F["uxuy"] - u[0] * u[1], F["uxuz"] - u[0] * u[2], F["uyuz"] - u[1] * u[2]]
    tr = (t[0] + t[1] + t[2]) / 3.0
    td = [t[0] - tr, t[1] - tr, t[2] - tr, t[3], t[4], t[5]]
    w = [1, 1, 1, 2, 2, 2]
    num = -sum(wk * a * b for wk, a, b in zip(w, td, S))
    den = 2.0 * sum(wk * b * b for wk, b in zip(w, S))
    nut = np.where(den > 1e-30, num / np.maximum(den, 1e-30), 0.0)
    return np.clip(nut, 0.0, nu_cap), S


def raw_features(F: dict, S, nu: float, nu_t):
    rho = F["rho"].astype(np.float64)
    tau = 3.0 * (nu + nu_t) + 0.5
    pi = [-2.0 * rho * CS2 * tau * s for s in S]
    q2 = pi[0] ** 2 + pi[1] ** 2 + pi[2] ** 2 + 2 * (pi[3] ** 2 + pi[4] ** 2 + pi[5] ** 2)
    return np.stack(pi + [rho - 1.0, np.sqrt(q2)], axis=-1).reshape(-1, 8)


# ----------------------------------------------------------------------------- evaluation


def mean_profile(uz, nd):
    """Mean u_z over each x-y plane (fluid and inlet/outlet nodes)."""
    return uz.reshape(nd.shape).mean(axis=(1, 2))


def spectrum(uz, z_planes):
    """Radially binned 2-D energy spectrum of u_z fluctuations, averaged over z planes."""
    nz, ny, nx = uz.shape
    kx = np.fft.fftfreq(nx) * nx
    ky = np.fft.fftfreq(ny) * ny
    K = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    kb = np.rint(K).astype(int)
    nk = int(min(nx, ny) // 2)
    e = np.zeros(nk + 1)
    for z in z_planes:
        a = uz[z] - uz[z].mean()
        p = np.abs(np.fft.fft2(a)) ** 2 / (nx * ny) ** 2
        e += np.bincount(kb.reshape(-1), p.reshape(-1), minlength=kb.max() + 1)[:nk + 1]
    return e / len(z_planes)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ----------------------------------------------------------------------------- study


def start_uniform(part, n, u_in):
    """Populations = equilibrium of u = (0, 0, u_in), rho = 1 everywhere.  Starting from the
    inlet velocity instead of rest avoids the impulsive start, whose pressure wave bounces
    between the Zou-He inlet and outlet and is barely damped at tau close to 1/2."""
    z = np.zeros(n, np.float32)
    part.load_restart(z, z, np.full(n, u_in, np.float32), np.ones(n, np.float32))


def run_fine(cx, cy, cz, factor, u_in, re, noise_amp, coarse_steps, snap_every, precision="f32",
             device=0, seed=11, fine_cs=0.05, jet_ratio=0.5, rbgk=False):
    """Fine run (BGK, or Smagorinsky with constant fine_cs); returns filtered snapshots keyed
    by coarse step."""
    g, p = channel(cx * factor, cy * factor, cz * factor, u_in, re, cy * factor, cs=fine_cs,
                   rbgk=rbgk)
    part = TLBMPartition.from_arrays(problem_from_params(p), g.nd_type, precision=precision,
                                     arithmetic="fast", device=device, rbgk=rbgk)
    start_uniform(part, g.nx * g.ny * g.nz, u_in)
    part.set_inlet_profile(inlet_velocity(cx, cy, factor, u_in, noise_amp, jet_ratio, seed))
    snaps = {}
    ts = 0
    for k in range(snap_every, coarse_steps + 1, snap_every):
        part.run(ts, factor * k - ts)
        ts = factor * k
        snaps[k] = part.filtered_fields(factor)
    part.close()
    return snaps, p.omega


def build_dataset(snaps, nu_c, nu_cap):
    """Features and targets of every snapshot; cells with non-finite values are dropped."""
    feats, targets = [], []
    for F in snaps.values():
        nut, S = sgs_eddy_viscosity(F, nu_cap)
        x = raw_features(F, S, nu_c, nut)
        t = nut.reshape(-1)
        ok = np.isfinite(x).all(axis=1) & np.isfinite(t)
        feats.append(x[ok])
        targets.append(t[ok])
    return np.concatenate(feats), np.concatenate(targets)


def normalise(raw, targets):
    shift = raw.mean(axis=0)
    scale = 1.0 / np.maximum(raw.std(axis=0), 1e-30)
    out_scale = max(float(targets.std()), 1e-12)
    return shift.astype(np.float32), scale.astype(np.float32), out_scale


def train_closure(raw, targets, epochs=30, batch=8192, lr=2e-3, seed=5, device=0):
    shift, scale, out_scale = normalise(raw, targets)
    x = ((raw - shift) * scale).astype(np.float32)
    t = (targets / out_scale).astype(np.float32)
    tr = MlpTrainer(x, t, seed=seed, device=device)
    loss0, _ = tr.loss_grad()
    losses = tr.train(epochs, batch, lr)
    params = tr.params()
    tr.close()
    return {"params": params, "shift": shift, "scale": scale, "out_scale": out_scale,
            "loss_initial": loss0, "losses": losses}


def run_coarse(cx, cy, cz, u_in, re, noise_amp, steps, closure=None, cs=0.0, precision="f32",
               device=0, seed=11, tau_min=None, jet_ratio=0.5, rbgk=False):
    g, p = channel(cx, cy, cz, u_in, re, cy, cs=cs, rbgk=rbgk)
    part = TLBMPartition.from_arrays(problem_from_params(p), g.nd_type, precision=precision,
                                     arithmetic="fast", device=device, rbgk=rbgk)
    start_uniform(part, cx * cy * cz, u_in)
    part.set_inlet_profile(inlet_velocity(cx, cy, 1, u_in, noise_amp, jet_ratio, seed))
    nu = (1.0 / p.omega - 0.5) / 3.0
    if closure is not None:
        part.set_closure_mlp(closure["params"], closure["scale"], closure["shift"],
                             closure["out_scale"], tau_min if tau_min else 3.0 * nu + 0.5 + 1e-6)
    ms = part.time_steps(0, steps) / steps
    ux, uy, uz, rho = part.macros()
    part.close()
    return {"uz": uz.reshape(cz, cy, cx), "ms": ms, "finite": bool(np.isfinite(uz).all()),
            "nd": g.nd_type.reshape(cz, cy, cx)}


def evaluate(run, ref_uz, z_planes):
    prof = rel_l2(mean_profile(run["uz"], run["nd"]), ref_uz.mean(axis=(1, 2)))
    e_run = spectrum(run["uz"], z_planes)[1:]
    e_ref = spectrum(ref_uz, z_planes)[1:]
    spec = rel_l2(np.log(e_run + 1e-30), np.log(e_ref + 1e-30))
    return {"profile_err": prof, "spectrum_log_err": spec, "finite": run["finite"],
            "ms_per_step": run["ms"]}


def calibrate(cl, snaps, cx, cy, cz, u_in, re, noise_amp, calib_step, zp, jet_ratio, device,
              seed, floors=(0.0, 0.02, 0.05), multipliers=(0.0, 1.0, 3.0, 10.0, 30.0, 100.0)):
    """A-posteriori level of the learned eddy viscosity.  The closure runs as
    nu_t = max(k * out_scale * y, nu_smag(cs_floor)); coarse runs to `calib_step` for every
    (cs_floor, k) are scored by profile + log-spectrum error against the filtered fine run at
    that step.  The network fixes where its viscosity goes; the calibration fixes its level and
    the Smagorinsky floor the coarse collision needs to stay stable (the a-priori target alone
    is far below it).  k = 0 is the floor alone.  Returns (best (cs_floor, k), scores)."""
    ref = snaps[calib_step]["uz"].astype(np.float64)
    scores = {}
    for fl in floors:
        for k in multipliers:
            c = dict(cl, out_scale=cl["out_scale"] * k)
            r = run_coarse(cx, cy, cz, u_in, re, noise_amp, calib_step, closure=c, cs=fl,
                           device=device, seed=seed, jet_ratio=jet_ratio)
            e = evaluate(r, ref, zp)
            scores[(fl, k)] = (e["profile_err"] + e["spectrum_log_err"] if e["finite"]
                               else float("inf"))
    best = min(scores, key=lambda key: scores[key])
    return best, scores


FLOORS = (0.0, 0.02, 0.03, 0.04, 0.05, 0.06, 0.07, 0.08)


def study(cx=128, cy=64, cz=64, factor=4, u_in=0.05, re=3000.0, noise_amp=0.01,
          coarse_steps=1024, snap_every=64, train_from=512, epochs=30, device=0, seed=11,
          fine_cs=0.05, jet_ratio=0.5, calib_step=None, floors=FLOORS,
          multipliers=(0.0, 1.0, 3.0, 10.0, 30.0)):
    """The learned-closure experiment; returns errors against the filtered fine run at
    `coarse_steps` (held out: training uses snapshots before it, calibration the one at
    `calib_step`) and costs per step of: Smagorinsky at cs = 0.1 (the reference's model at the
    configured coefficient), Smagorinsky at the cs that scores best on the calibration snapshot
    over the same grid of floors (the calibrated judge), the learned closure, its Smagorinsky
    floor alone, and plain BGK."""
    snaps, omega_f = run_fine(cx, cy, cz, factor, u_in, re, noise_amp, coarse_steps, snap_every,
                              device=device, seed=seed, fine_cs=fine_cs, jet_ratio=jet_ratio)
    nu_c = u_in * cy / re
    train = {k: v for k, v in snaps.items() if train_from <= k < coarse_steps}
    raw, nut = build_dataset(train, nu_c, nu_cap=50.0 * nu_c)
    cl = train_closure(raw, nut, epochs=epochs, device=device)
    ref = snaps[coarse_steps]["uz"].astype(np.float64)
    zp = list(range(cz // 2, cz - 2, max(1, cz // 16)))
    if calib_step is None:
        calib_step = max(k for k in snaps if k < coarse_steps)
    (floor, mult), scores = calibrate(cl, snaps, cx, cy, cz, u_in, re, noise_amp, calib_step,
                                      zp, jet_ratio, device, seed, floors, multipliers)
    cal = dict(cl, out_scale=cl["out_scale"] * mult, floor_cs=floor)
    # Smagorinsky alone, calibrated on the same snapshot over the same coefficients (k = 0 runs)
    smag_cs = min((fl for fl in floors if fl > 0), key=lambda fl: scores[(fl, 0.0)])
    out = {"samples": int(len(nut)), "nu_t_mean": float(nut.mean()), "nu": nu_c,
           "fine_finite": bool(np.isfinite(ref).all()),
           # the fine run is specified as plain BGK; at this Re and resolution BGK diverges
           # (fine tau 0.5128), so unless fine_cs = 0 it relaxes with a constant Smagorinsky cs
           "fine_run": {"collision": "smagorinsky" if fine_cs > 0 else "bgk",
                        "cs": fine_cs, "factor": factor,
                        "deviation": ("plain BGK specified; constant Smagorinsky cs = %g used "
                                      "because BGK diverges at this resolution" % fine_cs)
                        if fine_cs > 0 else None},
           "loss_initial": float(cl["loss_initial"]), "loss_final": float(cl["losses"][-1]),
           "calibration": {"step": calib_step, "floor_cs": floor, "multiplier": mult,
                           "smagorinsky_cs": smag_cs,
                           "scores": {"%g,%g" % k: v for k, v in scores.items()}}}
    for name, kw in (("smagorinsky", {"cs": 0.1}),
                     ("smagorinsky_calibrated", {"cs": smag_cs}),
                     ("learned", {"closure": cal, "cs": floor}),
                     ("floor_only", {"cs": floor}),
                     ("none", {})):
        r = run_coarse(cx, cy, cz, u_in, re, noise_amp, coarse_steps, device=device, seed=seed,
                       jet_ratio=jet_ratio, **kw)
        out[name] = evaluate(r, ref, zp)
    return out, cal
