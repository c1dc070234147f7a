"""ctypes access to the C oracle (oracle/tlbm_oracle.c) for the test suite.

The oracle is test infrastructure: it is loaded here, by ``__graft_entry__.smoke`` and by the
CPU-baseline leg of ``bench.py`` only, as the checker, never as the thing measured or shipped.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")


def build() -> None:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


_LIBS: dict = {}


def lib(prec: str = "f64"):
    """Load libtlbm_oracle_<prec>.so (building it if missing)."""
    if prec in _LIBS:
        return _LIBS[prec]
    path = os.path.join(ORACLE_DIR, "lib", "libtlbm_oracle_%s.so" % prec)
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    L.oracle_create.restype = vp
    L.oracle_create.argtypes = [i32, i32, dbl, dbl, dbl, dbl, i32, i32, i32, vp, i32]
    L.oracle_destroy.argtypes = [vp]
    L.oracle_step.argtypes = [vp, i32]
    L.oracle_run.argtypes = [vp, i32, i32]
    L.oracle_force.argtypes = [vp, vp, vp, vp]
    L.oracle_macros.argtypes = [vp, vp, vp, vp, vp]
    L.oracle_time_avg.argtypes = [vp, vp, vp, vp, vp]
    L.oracle_populations.argtypes = [vp, i32, vp]
    L.oracle_adjacency.argtypes = [vp, vp]
    L.oracle_set_threads.argtypes = [vp, i32]
    L.oracle_set_threads.restype = i32
    L.oracle_max_threads.restype = i32
    L.oracle_num_force_nodes.argtypes = [vp]
    L.oracle_num_force_nodes.restype = i64
    L.oracle_run_dir.argtypes = [ctypes.c_char_p, i32, ctypes.POINTER(dbl)]
    L.oracle_run_dir.restype = i32
    L.oracle_real_bytes.restype = i32
    L.oracle_load_restart.argtypes = [vp, vp, vp, vp, vp]
    _LIBS[prec] = L
    return L


def run_dir(workdir: str, prec: str = "f64", threads: int = 1) -> float:
    """Run the tLBMexec flow of the oracle in ``workdir``; returns the step-loop seconds."""
    el = ctypes.c_double(0.0)
    rc = lib(prec).oracle_run_dir(workdir.encode(), threads, ctypes.byref(el))
    if rc != 0:
        raise RuntimeError("oracle_run_dir failed with %d" % rc)
    return el.value


class Oracle:
    """One oracle problem held in memory (the reference's data layout)."""

    def __init__(self, q, dynamics, cs, rho, u, omega, nx, ny, nz, nd_type, prec="f64",
                 time_avg=0, threads=1):
        self.L = lib(prec)
        self.dtype = np.float64 if prec == "f64" else np.float32
        self.q, self.n = q, nx * ny * nz
        nd = np.ascontiguousarray(nd_type, dtype=np.int32)
        self.h = self.L.oracle_create(q, dynamics, cs, rho, u, omega, nx, ny, nz,
                                      nd.ctypes.data, time_avg)
        if not self.h:
            raise ValueError("oracle_create failed")
        self.L.oracle_set_threads(self.h, threads)
        self.ts = 0

    def load_restart(self, ux, uy, uz, rho) -> None:
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (ux, uy, uz, rho)]
        self.L.oracle_load_restart(self.h, *[a.ctypes.data for a in arrs])

    def run(self, nsteps: int) -> None:
        self.L.oracle_run(self.h, self.ts, nsteps)
        self.ts += nsteps

    def macros(self):
        out = [np.empty(self.n, self.dtype) for _ in range(4)]
        self.L.oracle_macros(self.h, *[a.ctypes.data for a in out])
        return out

    def force(self):
        out = [np.empty(self.n, self.dtype) for _ in range(3)]
        self.L.oracle_force(self.h, *[a.ctypes.data for a in out])
        return out

    def time_avg(self):
        out = [np.empty(self.n, self.dtype) for _ in range(4)]
        self.L.oracle_time_avg(self.h, *[a.ctypes.data for a in out])
        return out

    def populations(self, which: int = 0):
        out = np.empty(self.n * self.q, self.dtype)
        self.L.oracle_populations(self.h, which, out.ctypes.data)
        return out

    def adjacency(self):
        out = np.empty(self.n * self.q, np.int32)
        self.L.oracle_adjacency(self.h, out.ctypes.data)
        return out

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
