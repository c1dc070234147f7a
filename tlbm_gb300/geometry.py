"""Input generation for the tLBM file contract: geometry, node types, parameters, partitions.

The solver reads three whitespace-separated text files from its working directory:

* ``params.lbm`` -- 23 tokens read in order by ``Problem::load_input``
  (src/Problem.cpp:5-32, fields at include/Problem.h:18-40);
* ``ndType.lbm`` -- one integer node type per lattice point, in global order
  ``g = x + y*Nx + z*Nx*Ny`` (src/TLBM_Partition.cpp:120-141, :730-737);
* ``parts.lbm`` -- one partition id per lattice point, same order
  (src/TLBM_Partition.cpp:210-252).

The reference produces them with ``FluidChannel`` (python/FluidChannel.py:1309-1397),
``tLBM_partition.py`` and ``tLBM_write_params.py`` (python/tLBM_write_params.py:60-168).
Those scripts build Python lists and dictionaries per node and cannot reach 10^7+ nodes,
so this module restates their arithmetic on whole numpy arrays:

* lattice coordinates are float32 ``linspace`` values and every geometric test is done in
  float32, because the reference's node classification (``x == 0``, ``x > Lx - dx/2``,
  ``dist < r**2``) depends on those exact float32 values;
* the physical-to-lattice conversion and the ``%g`` / ``%f`` / ``%15.14f`` text formats follow
  python/tLBM_write_params.py:81-98 and :138-166 token for token, so the solver parses the
  same values the reference pipeline would give it.

It adds what the reference lacks: a seeded random non-overlapping sphere packing to a target
porosity and direct lattice-unit parameter files for synthetic workloads.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# node type codes (python/FluidChannel.py:1386-1397, :1217-1219)
FLUID, SOLID, INLET, OUTLET, MOVING_WALL = 0, 1, 2, 3, 5

# fluid library (python/FluidChannel.py:1162-1177): name -> (density, kinematic viscosity)
FLUIDS = {
    "water": (1000.0, 1.0e-6),
    "glycol": (965.3, 0.06 / 965.3),
    "glycerin": (1260.0, 1.49 / 1260.0),
}

LATTICES = ("D3Q15", "D3Q19", "D3Q27")


@dataclass
class Geometry:
    """A box channel: lattice size, node types in global order, and its physical scales."""

    nx: int
    ny: int
    nz: int
    nd_type: np.ndarray  # int32[nx*ny*nz], index x + y*nx + z*nx*ny
    lx_p: float = 0.0
    ly_p: float = 0.0
    lz_p: float = 0.0
    lo: float = 1.0  # characteristic length of the obstacle (physical units)
    n_divs: int = 2
    rho_p: float = 1000.0
    nu_p: float = 1.0e-6
    p_ref_idx: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def num_nodes(self) -> int:
        return self.nx * self.ny * self.nz

    def counts(self) -> dict:
        vals, cnt = np.unique(self.nd_type, return_counts=True)
        return {int(v): int(c) for v, c in zip(vals, cnt)}


def lattice_dims(lx_p: float, ly_p: float, lz_p: float, lo: float, n_divs: int):
    """Points per axis: ceil((N_divs-1)*L/Lo)+1 (python/FluidChannel.py:1336-1338)."""
    nx = math.ceil((n_divs - 1) * (lx_p / lo)) + 1
    ny = math.ceil((n_divs - 1) * (ly_p / lo)) + 1
    nz = math.ceil((n_divs - 1) * (lz_p / lo)) + 1
    return int(nx), int(ny), int(nz)


def _axis(l_p: float, n: int) -> np.ndarray:
    return np.linspace(0.0, l_p, n).astype(np.float32)


def _plane_ids(nx: int, ny: int, nz: int, z: int) -> np.ndarray:
    return np.arange(nx * ny, dtype=np.int64) + np.int64(z) * nx * ny


def sphere_channel(
    lx_p: float,
    ly_p: float,
    lz_p: float,
    r: float,
    xc: float,
    yc: float,
    zc: float,
    n_divs: int,
    walls=("left", "right", "top", "bottom"),
    fluid: str = "water",
) -> Geometry:
    """Channel with one spherical obstacle, the semantics of
    ``FluidChannel(Lx_p, Ly_p, Lz_p, obst=SphereObstruction(r, xc, yc, zc), N_divs, wallList)``.

    Obstacle: ``(x-xc)^2+(y-yc)^2+(z-zc)^2 < r^2`` in float32 (python/FluidChannel.py:269-276),
    characteristic length ``Lo = 2r`` (:265). Walls: ``right`` is x==0, ``left`` is
    x > Lx-dx/2, ``bottom`` is y==0, ``top`` is y > Ly-dx/2 (:1517-1539). Inlet is the z==0
    plane and outlet the z==Lz plane, minus wall and obstacle nodes (:1358-1383).
    """
    lo = float(r) * 2.0
    return _channel(lx_p, ly_p, lz_p, lo, n_divs, walls, fluid, ("sphere", r, xc, yc, zc))


def empty_channel(lx_p, ly_p, lz_p, lo, n_divs, walls=("left", "right", "top", "bottom"),
                  fluid="water") -> Geometry:
    """``FluidChannel`` with ``EmptyChannel(Lo)`` (python/FluidChannel.py:80-101)."""
    return _channel(lx_p, ly_p, lz_p, float(lo), n_divs, walls, fluid, None)


def _channel(lx_p, ly_p, lz_p, lo, n_divs, walls, fluid, obst) -> Geometry:
    nx, ny, nz = lattice_dims(lx_p, ly_p, lz_p, lo, n_divs)
    x1, y1, z1 = _axis(lx_p, nx), _axis(ly_p, ny), _axis(lz_p, nz)
    # broadcast views in (z, y, x) order == global node order
    X = x1[None, None, :]
    Y = y1[None, :, None]
    Z = z1[:, None, None]
    dx = np.float32(x1[1] - x1[0])
    shape = (nz, ny, nx)

    solid = np.zeros(shape, dtype=bool)
    for w in walls:
        if w == "right":
            solid |= np.broadcast_to(X == 0.0, shape)
        elif w == "left":
            solid |= np.broadcast_to(X > (lx_p - dx / 2.0), shape)
        elif w == "top":
            solid |= np.broadcast_to(Y > (ly_p - dx / 2.0), shape)
        elif w == "bottom":
            solid |= np.broadcast_to(Y == 0.0, shape)

    obstacle = np.zeros(shape, dtype=bool)
    if obst is not None and obst[0] == "sphere":
        _, r, xc, yc, zc = obst
        dist = (X - xc) ** 2 + (Y - yc) ** 2 + (Z - zc) ** 2
        obstacle = np.broadcast_to(dist < r**2, shape)

    inlet = np.broadcast_to(Z == 0.0, shape)
    outlet = np.broadcast_to(Z == lz_p, shape)

    nd = np.zeros(shape, dtype=np.int32)
    nd[solid | obstacle] = SOLID
    nd[inlet & ~solid & ~obstacle] = INLET
    nd[outlet & ~solid & ~obstacle] = OUTLET
    rho_p, nu_p = FLUIDS[fluid]
    g = Geometry(nx, ny, nz, nd.reshape(-1), lx_p, ly_p, lz_p, lo, n_divs, rho_p, nu_p)
    g.p_ref_idx = _p_ref_index(x1, y1, z1, dx, lx_p / 2.0, ly_p / 2.0, 0.95 * lz_p, nx, ny)
    return g


def _p_ref_index(x1, y1, z1, dx, xr, yr, zr, nx, ny) -> int:
    """Smallest node index within dx/1.5 of the reference point
    (``set_pRef_indx``, python/FluidChannel.py:1450-1470)."""
    tol = dx / 1.5
    xs = np.nonzero(np.abs(x1 - xr) < tol)[0]
    ys = np.nonzero(np.abs(y1 - yr) < tol)[0]
    zs = np.nonzero(np.abs(z1 - zr) < tol)[0]
    if len(xs) == 0 or len(ys) == 0 or len(zs) == 0:
        return 0
    return int(xs[0] + ys[0] * nx + zs[0] * nx * ny)


def lid_driven_cavity(lx_p=1.0, ly_p=1.0, lz_p=1.0, n_divs=11, fluid="water") -> Geometry:
    """Cavity with solid walls and a moving lid of node type 5 on the y==Ly face
    (python/FluidChannel.py:1179-1251): walls at x==0, x==Lx, y==0, z==0, z==Lz. The lid
    face is written after the walls, so its edge nodes are type 5 too (:1218-1219, :1248)."""
    lo = ly_p
    nx, ny, nz = lattice_dims(lx_p, ly_p, lz_p, lo, n_divs)
    x1, y1, z1 = _axis(lx_p, nx), _axis(ly_p, ny), _axis(lz_p, nz)
    X = x1[None, None, :]
    Y = y1[None, :, None]
    Z = z1[:, None, None]
    dx = np.float32(x1[1] - x1[0])
    shape = (nz, ny, nx)
    solid = np.broadcast_to(X == 0.0, shape) | np.broadcast_to(X > (lx_p - dx / 2.0), shape)
    solid = solid | np.broadcast_to(Y == 0.0, shape)
    solid = solid | np.broadcast_to(Z == 0.0, shape) | np.broadcast_to(Z > (lz_p - dx / 2.0), shape)
    lid = np.broadcast_to(Y > (ly_p - dx / 2.0), shape)
    nd = np.zeros(shape, dtype=np.int32)
    nd[solid] = SOLID
    nd[lid] = MOVING_WALL
    rho_p, nu_p = FLUIDS[fluid]
    return Geometry(nx, ny, nz, nd.reshape(-1), lx_p, ly_p, lz_p, lo, n_divs, rho_p, nu_p)


def random_sphere_pack(
    nx: int,
    ny: int,
    nz: int,
    r_min: float = 4.0,
    r_max: float = 12.0,
    porosity: float = 0.7,
    seed: int = 0,
    z_margin: int | None = None,
    max_tries: int = 200000,
) -> Geometry:
    """Seeded random non-overlapping spheres (radii uniform in [r_min, r_max]) added until the
    fraction of solid lattice nodes reaches ``1 - porosity``. The box is periodic in x and y
    (no walls) with a z==0 inlet and z==nz-1 outlet; sphere nodes on those planes stay solid.
    Sphere centres keep ``z_margin`` nodes (default r_max) clear of the inlet/outlet planes.

    Lattice units: node (x, y, z) is solid when ``|p - c|^2 < r^2`` using periodic x/y
    distance. ``meta['mean_diameter']`` records the mean sphere diameter (the Re length).
    """
    rng = np.random.default_rng(seed)
    if z_margin is None:
        z_margin = int(math.ceil(r_max))
    target = (1.0 - porosity) * nx * ny * nz
    solid = np.zeros((nz, ny, nx), dtype=bool)
    centres = []
    n_solid = 0
    tries = 0
    # candidate spheres are drawn in seeded batches; overlap tests look only at the accepted
    # spheres hashed into the 27 grid cells (edge 2*r_max) around the candidate
    h = 2.0 * r_max
    gx, gy, gz = max(1, int(nx // h)), max(1, int(ny // h)), max(1, int(math.ceil(nz / h)))
    sx, sy, sz = nx / gx, ny / gy, nz / gz
    grid: dict = {}
    batch = 65536
    while n_solid < target and tries < max_tries:
        rs = rng.uniform(r_min, r_max, batch)
        cs = np.stack([rng.uniform(0, nx, batch), rng.uniform(0, ny, batch),
                       rng.uniform(z_margin, nz - 1 - z_margin, batch)], axis=1)
        for k in range(batch):
            if n_solid >= target or tries >= max_tries:
                break
            tries += 1
            r = float(rs[k])
            cx, cy, cz = float(cs[k, 0]), float(cs[k, 1]), float(cs[k, 2])
            ix, iy, iz = int(cx / sx) % gx, int(cy / sy) % gy, min(int(cz / sz), gz - 1)
            ok = True
            for dz in (-1, 0, 1):
                jz = iz + dz
                if jz < 0 or jz >= gz:
                    continue
                for dy in (-1, 0, 1):
                    jy = (iy + dy) % gy
                    for dx in (-1, 0, 1):
                        for (qx, qy, qz, qr) in grid.get(((ix + dx) % gx, jy, jz), ()):
                            ddx = abs(cx - qx)
                            ddx = min(ddx, nx - ddx)
                            ddy = abs(cy - qy)
                            ddy = min(ddy, ny - ddy)
                            ddz = cz - qz
                            if ddx * ddx + ddy * ddy + ddz * ddz < (r + qr) ** 2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                continue
            grid.setdefault((ix, iy, iz), []).append((cx, cy, cz, r))
            c = np.array([cx, cy, cz])
            n_solid += _rasterise_sphere(solid, c, r, nx, ny, nz)
            centres.append((c, r))
    nd = np.zeros((nz, ny, nx), dtype=np.int32)
    nd[0] = INLET
    nd[nz - 1] = OUTLET
    nd[solid] = SOLID
    g = Geometry(nx, ny, nz, nd.reshape(-1))
    diam = [2.0 * r for (_, r) in centres]
    g.lo = float(np.mean(diam)) if diam else 1.0
    g.meta = {
        "n_spheres": len(centres),
        "mean_diameter": g.lo,
        "porosity": 1.0 - float(solid.sum()) / solid.size,
        "seed": seed,
        "tries": tries,
    }
    return g


def _rasterise_sphere(solid, c, r, nx, ny, nz) -> int:
    """Mark |p - c|^2 < r^2 (periodic in x, y) solid; returns the number of new solid nodes."""
    rr = int(math.ceil(r))
    zs = np.arange(max(0, int(math.floor(c[2] - rr))), min(nz, int(math.ceil(c[2] + rr)) + 1))
    ys = np.arange(int(math.floor(c[1] - rr)), int(math.ceil(c[1] + rr)) + 1)
    xs = np.arange(int(math.floor(c[0] - rr)), int(math.ceil(c[0] + rr)) + 1)
    dz = (zs - c[2])[:, None, None]
    dy = (ys - c[1])[None, :, None]
    dxx = (xs - c[0])[None, None, :]
    ball = (dxx**2 + dy**2 + dz**2) < r * r
    idx = np.ix_(zs, ys % ny, xs % nx)
    sub = solid[idx]
    added = int((ball & ~sub).sum())
    solid[idx] = sub | ball
    return added


def sphere_in_box(nx, ny, nz, r, xc, yc, zc, walls=True) -> Geometry:
    """Lattice-unit channel with one sphere (|p-c|^2 < r^2), optional solid x/y walls, z==0
    inlet and z==nz-1 outlet; used for the per-channel geometries of ensembles."""
    z = np.arange(nz)[:, None, None]
    y = np.arange(ny)[None, :, None]
    x = np.arange(nx)[None, None, :]
    shape = (nz, ny, nx)
    solid = np.broadcast_to(((x - xc) ** 2 + (y - yc) ** 2 + (z - zc) ** 2) < r * r, shape).copy()
    if walls:
        solid |= np.broadcast_to((x == 0) | (x == nx - 1), shape)
        solid |= np.broadcast_to((y == 0) | (y == ny - 1), shape)
    nd = np.zeros(shape, dtype=np.int32)
    nd[0] = INLET
    nd[nz - 1] = OUTLET
    nd[solid] = SOLID
    return Geometry(nx, ny, nz, nd.reshape(-1), lo=2.0 * r)


# ----------------------------------------------------------------------------- partitions


def partition_geometric(nx: int, ny: int, nz: int, px: int, py: int, pz: int) -> np.ndarray:
    """Block partition of the lattice into px*py*pz boxes, partition ids ordered z-, y-, then
    x-block major; the first ``N % p`` blocks along an axis get one extra layer
    (``set_geometric_partition``, python/partition_compare.py:49-95)."""

    def edges(n, p):
        b = n // p
        sizes = [b + (1 if (n % p) > i else 0) for i in range(p)]
        owner = np.repeat(np.arange(p), sizes)
        return owner

    ox, oy, oz = edges(nx, px), edges(ny, py), edges(nz, pz)
    part = (oz[:, None, None] * (py * px) + oy[None, :, None] * px + ox[None, None, :])
    return part.astype(np.int32).reshape(-1)


def partition_1d(nx: int, ny: int, nz: int, nparts: int) -> np.ndarray:
    """'1D' style: z-slabs (python/pyPartition.py:178-179)."""
    return partition_geometric(nx, ny, nz, 1, 1, nparts)


# ----------------------------------------------------------------------------- parameters


@dataclass
class Params:
    """The 23 tokens of params.lbm in file order (src/Problem.cpp:10-32)."""

    lattice: str = "D3Q19"
    dynamics: int = 1
    num_ts: int = 100
    ts_rep_freq: int = 100
    warmup_ts: int = 0
    plot_freq: int = 100
    cs: float = 0.0
    rho_lbm: float = 1.0
    u_lbm: float = 0.05
    omega: float = 1.0
    nx: int = 1
    ny: int = 1
    nz: int = 1
    restart: int = 0
    time_avg: int = 0
    lx_p: float = 1.0
    ly_p: float = 1.0
    lz_p: float = 1.0
    t_conv: float = 1.0
    l_conv: float = 1.0
    p_conv: float = 1.0
    p_ref_idx: int = 0
    ss_flag: int = 0

    def text(self) -> str:
        """The exact text tLBM_write_params.py writes (python/tLBM_write_params.py:139-166)."""
        lines = [
            "%s \n" % self.lattice,
            "%d \n" % self.dynamics,
            "%d \n" % self.num_ts,
            "%d \n" % self.ts_rep_freq,
            "%d \n" % self.warmup_ts,
            "%d \n" % self.plot_freq,
            "%g \n" % self.cs,
            "%g \n" % self.rho_lbm,
            "%g \n" % self.u_lbm,
            "%g \n" % self.omega,
            "%d \n" % self.nx,
            "%d \n" % self.ny,
            "%d \n" % self.nz,
            "%d \n" % self.restart,
            "%d \n" % self.time_avg,
            "%f \n" % self.lx_p,
            "%f \n" % self.ly_p,
            "%f \n" % self.lz_p,
            "%15.14f \n" % self.t_conv,
            "%15.14f \n" % self.l_conv,
            "%g \n" % self.p_conv,
            "%d \n" % self.p_ref_idx,
            "%d \n" % self.ss_flag,
        ]
        return "".join(lines)


def params_from_physical(geom: Geometry, lattice: str, dynamics: int, num_ts: int,
                         ts_rep_freq: int, warmup_ts: int, plot_freq: int, re: float, dt: float,
                         cs: float, restart: int = 0, time_avg: int = 0, ss_flag: int = 0) -> Params:
    """Non-dimensionalisation of python/tLBM_write_params.py:81-98."""
    uo = geom.nu_p * re / geom.lo
    to = geom.lo / uo
    uavg = uo
    ud = (to / geom.lo) * uavg
    nu_d = 1.0 / re
    dx = 1.0 / (geom.n_divs - 1.0)
    u_lbm = (dt / dx) * ud
    nu_lbm = (dt / (dx**2)) * nu_d
    omega = 1.0 / (3.0 * nu_lbm + 0.5)
    t_conv = dt * to
    l_conv = dx * geom.lo
    p_conv = (((l_conv / t_conv) ** 2) * (1.0 / 3.0)) / (l_conv**3)
    rho_lbm = geom.rho_p * (l_conv**3)
    return Params(lattice, dynamics, num_ts, ts_rep_freq, warmup_ts, plot_freq, cs, rho_lbm,
                  u_lbm, omega, geom.nx, geom.ny, geom.nz, restart, time_avg, geom.lx_p,
                  geom.ly_p, geom.lz_p, t_conv, l_conv, p_conv, geom.p_ref_idx, ss_flag)


def params_lattice_units(geom: Geometry, lattice: str, u_lbm: float, re: float, length: float,
                         num_ts: int, cs: float = 0.0, rho_lbm: float = 1.0, dynamics: int = 1,
                         plot_freq: int | None = None, warmup_ts: int = 0,
                         ts_rep_freq: int | None = None, time_avg: int = 0) -> Params:
    """Parameters for a synthetic lattice-unit workload: nu = u*L/Re, omega = 1/(3 nu + 1/2)."""
    nu = u_lbm * length / re
    omega = 1.0 / (3.0 * nu + 0.5)
    pf = plot_freq if plot_freq is not None else num_ts
    rf = ts_rep_freq if ts_rep_freq is not None else num_ts
    return Params(lattice, dynamics, num_ts, rf, warmup_ts, pf, cs, rho_lbm, u_lbm, omega,
                  geom.nx, geom.ny, geom.nz, 0, time_avg, float(geom.nx - 1), float(geom.ny - 1),
                  float(geom.nz - 1), 1.0, 1.0, 1.0, geom.p_ref_idx, 0)


def omega_from_re(u_lbm: float, length: float, re: float) -> float:
    return 1.0 / (3.0 * (u_lbm * length / re) + 0.5)


# ----------------------------------------------------------------------------- file writers


def _int_lines(a: np.ndarray) -> bytes:
    """'%d \\n' per value, the reference's ndType.lbm / parts.lbm line format."""
    a = np.asarray(a, dtype=np.int64).reshape(-1)
    if a.size == 0:
        return b""
    if a.min() >= 0 and a.max() <= 9:
        # single-digit fast path: "d \n" per value
        out = np.empty((a.size, 3), dtype=np.uint8)
        out[:, 0] = a.astype(np.uint8) + ord("0")
        out[:, 1] = ord(" ")
        out[:, 2] = ord("\n")
        return out.tobytes()
    return "".join("%d \n" % int(v) for v in a).encode()


def write_inputs(workdir: str, geom: Geometry, params: Params, parts: np.ndarray | None = None,
                 ss_nodes=()) -> None:
    """Write params.lbm, ndType.lbm, parts.lbm (and ssNds.lbm) into ``workdir``."""
    os.makedirs(workdir, exist_ok=True)
    with open(os.path.join(workdir, "params.lbm"), "w") as fh:
        fh.write(params.text())
    with open(os.path.join(workdir, "ndType.lbm"), "wb") as fh:
        fh.write(_int_lines(geom.nd_type))
    if parts is None:
        parts = np.zeros(geom.num_nodes, dtype=np.int32)
    with open(os.path.join(workdir, "parts.lbm"), "wb") as fh:
        fh.write(_int_lines(parts))
    with open(os.path.join(workdir, "ssNds.lbm"), "w") as fh:
        fh.write("".join("%i \n" % int(s) for s in ss_nodes))


def read_int_file(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        return np.array(fh.read().split(), dtype=np.int32)


# ----------------------------------------------------------------------------- named workloads


def channel_sphere_32x32x128() -> Geometry:
    """32x32x128 channel (z streamwise), no-slip walls on the x/y faces, one sphere of radius 6
    centred at (16,16,32): ``FluidChannel(31, 31, 127, SphereObstruction(6,16,16,32), N_divs=13)``."""
    return sphere_channel(31.0, 31.0, 127.0, 6, 16, 16, 32, 13)


def channel_sphere_32x32x128_params(num_ts=2000, plot_freq=2000, lattice="D3Q19", cs=0.0,
                                    dynamics=1) -> Params:
    """Re=20 on the sphere diameter, u_lbm=0.05, rho_lbm=1: tLBM_write_params.py with
    ``Re=20 dt=0.0041666666666667`` and the density line set to 1."""
    g = channel_sphere_32x32x128()
    p = params_from_physical(g, lattice, dynamics, num_ts, 500, 0, plot_freq, 20.0,
                             0.0041666666666667, cs)
    p.rho_lbm = 1.0
    return p


def ensemble_channels(n: int = 64, seed: int = 7, u_in: float = 0.04, num_ts: int = 2000,
                      cs: float = 0.1):
    """The batched-ensemble workload: ``n`` independent channels, each with Nx = Ny drawn from
    {32, 48, 64}, Nz uniform in [64, 256], lattice D3Q15 or D3Q19, Re uniform in [50, 500] on
    the sphere diameter, one sphere of radius Nx/6 on the channel axis at a seeded height in
    [Nz/4, Nz/2], solid x/y walls, z==0 inlet (u_in) and z==Nz-1 outlet (rho = 1).  The
    channels relax with the Smagorinsky model (cs): at these Reynolds numbers tau is 0.503 to
    0.55, and plain BGK from rest diverges in 60 of the 64 channels within 2000 steps.
    Returns a list of (Geometry, Params)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.choice([32, 48, 64]))
        nz = int(rng.integers(64, 257))
        lattice = str(rng.choice(["D3Q15", "D3Q19"]))
        re = float(rng.uniform(50.0, 500.0))
        r = nx / 6.0
        zc = float(rng.uniform(nz / 4.0, nz / 2.0))
        g = sphere_in_box(nx, nx, nz, r, (nx - 1) / 2.0, (nx - 1) / 2.0, zc, walls=True)
        p = params_lattice_units(g, lattice, u_in, re, 2.0 * r, num_ts, cs=cs)
        out.append((g, p))
    return out
