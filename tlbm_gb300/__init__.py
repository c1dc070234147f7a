"""tlbm_gb300 -- GB300 lattice-Boltzmann engine with the tLBM operator surface.

The engine is ``lib/libtlbm_gb300.so`` (hand-written sm_103a CUDA behind the C ABI of
``include/tlbm.h``).  This module binds that ABI with ctypes and mirrors the reference's
``TLBM_Partition`` class (include/TLBM_Partition.h:33-133) for Python callers:

    part = TLBMPartition(workdir)            # TLBM_Partition(rank, size, comm)
    for ts in range(part.get_num_ts()):
        part.take_LBM_time_step(ts % 2)      # take_LBM_time_step(bool isEven)
        if (ts + 1) % part.get_plot_freq() == 0 and ts + 1 > part.get_warmupTs():
            part.write_data()                # write_data()

Errors raise ``TLBMError`` carrying the C status and message (the reference throws).  There is
no CPU fallback: if the library is missing, importing the binding fails loudly.
"""

from __future__ import annotations

import ctypes
import os
import re
import weakref

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libtlbm_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "tlbm.h")

# status codes (include/tlbm.h)
OK, ERR_IO, ERR_INVALID_ARGUMENT, ERR_FORMAT, ERR_OUT_OF_RANGE, ERR_CUDA, ERR_NUMERIC, \
    ERR_UNSUPPORTED, ERR_TIMEOUT, ERR_NO_MEMORY = range(10)
PREC = {"f64": 0, "f32": 1, "bf16": 2, "f16": 3, "bf16m": 4}
ARITH = {"reference": 0, "fast": 1}


class TLBMError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status
        self.message = message


class Options(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_int), ("precision", ctypes.c_int),
                ("arithmetic", ctypes.c_int), ("closure", ctypes.c_int),
                ("block_x", ctypes.c_int), ("block_y", ctypes.c_int), ("device", ctypes.c_int),
                ("rbgk", ctypes.c_int), ("mrt", ctypes.c_int), ("mrt_ghost_rate", ctypes.c_float),
                ("f64_pipe", ctypes.c_int), ("reserved", ctypes.c_int * 5)]


class Problem(ctypes.Structure):
    _fields_ = [("lattice", ctypes.c_char * 8), ("dynamics", ctypes.c_int),
                ("num_ts", ctypes.c_int), ("ts_rep_freq", ctypes.c_int),
                ("warmup_ts", ctypes.c_int), ("plot_freq", ctypes.c_int),
                ("cs", ctypes.c_double), ("rho_lbm", ctypes.c_double),
                ("u_lbm", ctypes.c_double), ("omega", ctypes.c_double),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("restart_flag", ctypes.c_int), ("time_avg_flag", ctypes.c_int),
                ("lx_p", ctypes.c_double), ("ly_p", ctypes.c_double), ("lz_p", ctypes.c_double),
                ("t_conv", ctypes.c_double), ("l_conv", ctypes.c_double),
                ("p_conv", ctypes.c_double), ("p_ref_idx", ctypes.c_int),
                ("ss_data_flag", ctypes.c_int)]


_lib = None


def library(path: str = LIB_PATH):
    """Load the engine library (ctypes) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("tlbm_gb300 engine library not built (%s); run "
                          "`python -m tlbm_gb300.build`" % path)
    L = ctypes.CDLL(path)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
    H = ctypes.c_void_p
    PH = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "tlbm_default_options": (None, [ctypes.POINTER(Options)]),
        "tlbm_create": (i32, [ctypes.c_char_p, i32, i32, PH]),
        "tlbm_create_ex": (i32, [ctypes.c_char_p, i32, i32, ctypes.POINTER(Options), PH]),
        "tlbm_create_from_arrays": (i32, [ctypes.POINTER(Problem), vp, vp, ctypes.c_char_p,
                                          ctypes.POINTER(Options), PH]),
        "tlbm_destroy": (i32, [H]),
        "tlbm_step": (i32, [H, i32]),
        "tlbm_run": (i32, [H, i32, i32]),
        "tlbm_time_steps": (i32, [H, i32, i32, ctypes.POINTER(ctypes.c_float)]),
        "tlbm_synchronize": (i32, [H]),
        "tlbm_write_data": (i32, [H]),
        "tlbm_write_time_avg_data": (i32, [H]),
        "tlbm_get_num_ts": (i32, [H]),
        "tlbm_get_ts_rep_freq": (i32, [H]),
        "tlbm_get_plot_freq": (i32, [H]),
        "tlbm_get_warmup_ts": (i32, [H]),
        "tlbm_get_num_global_nodes": (i32, [H]),
        "tlbm_get_time_avg_flag": (i32, [H]),
        "tlbm_is_restart": (i32, [H]),
        "tlbm_get_cut_size": (i32, [H]),
        "tlbm_get_last_error": (ctypes.c_char_p, [H]),
        "tlbm_status_string": (ctypes.c_char_p, [i32]),
        "tlbm_output_bytes": (i32, [H]),
        "tlbm_get_options": (i32, [H, ctypes.POINTER(Options)]),
        "tlbm_num_speeds": (i32, [H]),
        "tlbm_copy_macros": (i32, [H, vp, vp, vp, vp]),
        "tlbm_copy_force": (i32, [H, vp, vp, vp]),
        "tlbm_copy_outputs_async": (i32, [H, vp, vp, vp, vp, vp, vp, vp]),
        "tlbm_host_alloc": (i32, [ctypes.c_size_t, PH]),
        "tlbm_host_free": (i32, [vp]),
        "tlbm_copy_populations": (i32, [H, i32, vp]),
        "tlbm_copy_adjacency": (i32, [H, vp]),
        "tlbm_mass": (i32, [H, ctypes.POINTER(ctypes.c_double)]),
        "tlbm_kernel_launches": (i64, [H]),
        "tlbm_load_restart": (i32, [H, vp, vp, vp, vp]),
        "tlbm_set_inlet_profile": (i32, [H, vp]),
        "tlbm_set_closure_mlp": (i32, [H, vp, vp, vp, ctypes.c_float, ctypes.c_float]),
        "tlbm_filtered_fields": (i32, [H, i32, vp]),
        "tlbm_processed_fields": (i32, [H, i32, vp]),
        "tlbm_write_processed_data": (i32, [H, i32]),
        "tlbm_process_output_dir": (i32, [ctypes.c_char_p, i32, ctypes.POINTER(i32)]),
        "tlbm_mlp_num_params": (i32, []),
        "tlbm_mlp_create": (i32, [i64, vp, vp, ctypes.c_uint64, i32, PH]),
        "tlbm_mlp_destroy": (i32, [H]),
        "tlbm_mlp_set_params": (i32, [H, vp]),
        "tlbm_mlp_get_params": (i32, [H, vp]),
        "tlbm_mlp_loss_grad": (i32, [H, i64, i64, ctypes.POINTER(ctypes.c_float), vp]),
        "tlbm_mlp_train": (i32, [H, i32, i64, ctypes.c_float, vp]),
        "tlbm_mlp_predict": (i32, [H, i64, vp, vp]),
        "tlbm_mlp_last_error": (ctypes.c_char_p, [H]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def host_empty(n: int, dtype) -> np.ndarray:
    """An uninitialised array of n values in page-locked host memory (tlbm_host_alloc): the
    destination of choice for macros(out=...) and force(out=...), whose copies then run at the
    host link's rate.  The memory is released when the array is garbage-collected."""
    L = library()
    dtype = np.dtype(dtype)
    nbytes = max(1, int(n) * dtype.itemsize)
    ptr = ctypes.c_void_p()
    st = L.tlbm_host_alloc(nbytes, ctypes.byref(ptr))
    if st != OK:
        raise TLBMError(st, L.tlbm_get_last_error(None).decode())
    buf = (ctypes.c_char * nbytes).from_address(ptr.value)
    weakref.finalize(buf, L.tlbm_host_free, ctypes.c_void_p(ptr.value))
    return np.frombuffer(buf, dtype=dtype, count=int(n))


def process_output_dir(workdir: str, device: int = 0) -> int:
    """processTLBM.py for a finished run directory, on the GPU; returns the dumps processed."""
    L = library()
    done = ctypes.c_int(0)
    st = L.tlbm_process_output_dir(workdir.encode(), device, ctypes.byref(done))
    if st != 0:
        raise TLBMError(st, L.tlbm_get_last_error(None).decode())
    return done.value


def declared_symbols(header: str = HEADER) -> list[str]:
    """Function names declared in include/tlbm.h."""
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tlbm_[a-z_0-9]+)\s*\(", text)))


def options(precision="f32", arithmetic=None, block_x=0, block_y=0, device=0,
            rbgk=False, mrt=False, ghost_rate=0.0) -> Options:
    o = Options()
    library().tlbm_default_options(ctypes.byref(o))
    o.precision = PREC[precision]
    if arithmetic is None:
        arithmetic = "fast" if precision in ("bf16", "f16", "bf16m") else "reference"
    if arithmetic == "fast-fp64":
        # FP64 storage, fast arithmetic with the fluid collision on the FP64 pipe (f64_pipe)
        arithmetic = "fast"
        o.f64_pipe = 1
    o.arithmetic = ARITH[arithmetic]
    o.block_x, o.block_y, o.device = block_x, block_y, device
    o.rbgk = int(bool(rbgk))
    o.mrt = int(bool(mrt))
    o.mrt_ghost_rate = float(ghost_rate)
    return o


def _check(status: int, handle=None) -> None:
    if status != OK:
        L = library()
        msg = L.tlbm_get_last_error(handle).decode()
        raise TLBMError(status, msg or L.tlbm_status_string(status).decode())


def _sized(a, dtype, n: int, what: str) -> np.ndarray:
    """`a` as a contiguous 1-D array of n values of dtype: the C ABI reads exactly n values
    through a bare pointer, so a wrong length is refused here instead of read out of bounds."""
    out = np.ascontiguousarray(a, dtype=dtype).reshape(-1)
    if out.size != n:
        raise ValueError("%s: %d values given, %d expected" % (what, out.size, n))
    return out


class TLBMPartition:
    """The reference's TLBM_Partition over the GPU engine (one process, whole lattice)."""

    def __init__(self, workdir: str = ".", rank: int = 0, size: int = 1 << 20,
                 precision: str | None = None, arithmetic: str | None = None,
                 block_x: int = 0, block_y: int = 0, device: int = 0, rbgk: bool = False,
                 mrt: bool = False, ghost_rate: float = 0.0, _handle=None):
        self._L = library()
        self._h = ctypes.c_void_p()
        self.workdir = workdir
        if _handle is not None:
            self._h = _handle
        elif precision is None and arithmetic is None:
            # like the reference binary: defaults, optionally overridden by workdir/tlbm.cfg
            _check(self._L.tlbm_create(workdir.encode(), rank, size, ctypes.byref(self._h)))
        else:
            o = options(precision or "f32", arithmetic, block_x, block_y, device, rbgk, mrt,
                        ghost_rate)
            _check(self._L.tlbm_create_ex(workdir.encode(), rank, size, ctypes.byref(o),
                                          ctypes.byref(self._h)))
        try:
            toks = open(os.path.join(workdir, "params.lbm")).read().split()
            self._dims = (int(toks[10]), int(toks[11]), int(toks[12]))
        except (OSError, IndexError, ValueError):
            pass
        self._init_meta()

    @classmethod
    def from_arrays(cls, problem: Problem, nd_type, parts=None, workdir=None,
                    precision="f64", arithmetic=None, block_x=0, block_y=0, device=0,
                    rbgk=False, mrt=False, ghost_rate=0.0):
        L = library()
        cells = int(problem.nx) * int(problem.ny) * int(problem.nz)
        if cells <= 0:
            raise ValueError("lattice %d x %d x %d" % (problem.nx, problem.ny, problem.nz))
        nd = _sized(nd_type, np.int32, cells, "nd_type")
        pp = None if parts is None else _sized(parts, np.int32, cells, "parts")
        o = options(precision, arithmetic, block_x, block_y, device, rbgk, mrt, ghost_rate)
        h = ctypes.c_void_p()
        _check(L.tlbm_create_from_arrays(ctypes.byref(problem), nd.ctypes.data,
                                         None if pp is None else pp.ctypes.data,
                                         None if workdir is None else workdir.encode(),
                                         ctypes.byref(o), ctypes.byref(h)))
        obj = cls.__new__(cls)
        obj._L = L
        obj._h = h
        obj.workdir = workdir
        obj._dims = (problem.nx, problem.ny, problem.nz)
        obj._init_meta()
        return obj

    def _init_meta(self):
        self.n = self._L.tlbm_get_num_global_nodes(self._h)
        self.q = self._L.tlbm_num_speeds(self._h)
        self.dtype = np.float64 if self._L.tlbm_output_bytes(self._h) == 8 else np.float32

    # -- the reference's public surface ---------------------------------------------------
    def take_LBM_time_step(self, is_even) -> None:
        _check(self._L.tlbm_step(self._h, int(bool(is_even))), self._h)

    def write_data(self) -> None:
        _check(self._L.tlbm_write_data(self._h), self._h)

    def write_time_avg_data(self) -> None:
        _check(self._L.tlbm_write_time_avg_data(self._h), self._h)

    def get_num_ts(self) -> int:
        return self._L.tlbm_get_num_ts(self._h)

    def get_ts_rep_freq(self) -> int:
        return self._L.tlbm_get_ts_rep_freq(self._h)

    def get_plot_freq(self) -> int:
        return self._L.tlbm_get_plot_freq(self._h)

    def get_warmupTs(self) -> int:
        return self._L.tlbm_get_warmup_ts(self._h)

    def get_num_global_nodes(self) -> int:
        return self._L.tlbm_get_num_global_nodes(self._h)

    def get_time_avg_flag(self) -> int:
        return self._L.tlbm_get_time_avg_flag(self._h)

    def is_restart(self) -> int:
        return self._L.tlbm_is_restart(self._h)

    def get_cut_size(self) -> int:
        return self._L.tlbm_get_cut_size(self._h)

    # -- engine extras -----------------------------------------------------------------------
    def run(self, first_ts: int, nsteps: int) -> None:
        _check(self._L.tlbm_run(self._h, first_ts, nsteps), self._h)

    def time_steps(self, first_ts: int, nsteps: int) -> float:
        ms = ctypes.c_float(0.0)
        _check(self._L.tlbm_time_steps(self._h, first_ts, nsteps, ctypes.byref(ms)), self._h)
        return ms.value

    def synchronize(self) -> None:
        _check(self._L.tlbm_synchronize(self._h), self._h)

    def _outputs(self, k, out):
        if out is None:
            return [np.empty(self.n, self.dtype) for _ in range(k)]
        out = list(out)
        if len(out) != k or any(a.dtype != self.dtype or a.size != self.n or
                                not a.flags.c_contiguous or not a.flags.writeable for a in out):
            raise ValueError("out: %d writeable contiguous %s arrays of %d values"
                             % (k, np.dtype(self.dtype).name, self.n))
        return out

    def macros(self, out=None):
        """ux, uy, uz, rho of the last step (global order); out: 4 arrays to fill, e.g. from
        host_empty (page-locked), instead of new ones."""
        out = self._outputs(4, out)
        _check(self._L.tlbm_copy_macros(self._h, *[a.ctypes.data for a in out]), self._h)
        return out

    def force(self, out=None):
        """Fx, Fy, Fz of the last step (global order); out as for macros."""
        out = self._outputs(3, out)
        _check(self._L.tlbm_copy_force(self._h, *[a.ctypes.data for a in out]), self._h)
        return out

    def outputs_async(self, out):
        """Start copying ux, uy, uz, rho, Fx, Fy, Fz of the last step into the 7 arrays `out`
        (page-locked: host_empty) while later steps run (tlbm_copy_outputs_async); they hold
        the values after synchronize()."""
        out = self._outputs(7, out)
        _check(self._L.tlbm_copy_outputs_async(self._h, *[a.ctypes.data for a in out]), self._h)
        return out

    def populations(self, which: int = 0):
        out = np.empty(self.n * self.q, self.dtype)
        _check(self._L.tlbm_copy_populations(self._h, which, out.ctypes.data), self._h)
        return out

    def adjacency(self):
        out = np.empty(self.n * self.q, np.int32)
        _check(self._L.tlbm_copy_adjacency(self._h, out.ctypes.data), self._h)
        return out

    def mass(self) -> float:
        m = ctypes.c_double(0.0)
        _check(self._L.tlbm_mass(self._h, ctypes.byref(m)), self._h)
        return m.value

    def kernel_launches(self) -> int:
        return self._L.tlbm_kernel_launches(self._h)

    def load_restart(self, ux, uy, uz, rho) -> None:
        """Populations = equilibrium of the given fields (load_restart_data)."""
        arrs = [_sized(a, np.float32, self.n, name)
                for a, name in ((ux, "ux"), (uy, "uy"), (uz, "uz"), (rho, "rho"))]
        _check(self._L.tlbm_load_restart(self._h, *[a.ctypes.data for a in arrs]), self._h)

    def set_inlet_profile(self, uz) -> None:
        """Inlet u_z per (x, y) of the z = 0 plane (None restores the uniform uLBM)."""
        if uz is None:
            _check(self._L.tlbm_set_inlet_profile(self._h, None), self._h)
            return
        nx, ny, _ = self._shape()
        self._inlet = _sized(uz, np.float64, nx * ny, "inlet profile")
        _check(self._L.tlbm_set_inlet_profile(self._h, self._inlet.ctypes.data), self._h)

    def set_closure_mlp(self, params, scale, shift, out_scale: float, tau_min: float) -> None:
        """Install the learned eddy-viscosity closure (None removes it)."""
        if params is None:
            _check(self._L.tlbm_set_closure_mlp(self._h, None, None, None, 0.0, 0.0), self._h)
            return
        p = _sized(params, np.float32, self._L.tlbm_mlp_num_params(), "params")
        s = _sized(scale, np.float32, 8, "scale")
        h = _sized(shift, np.float32, 8, "shift")
        _check(self._L.tlbm_set_closure_mlp(self._h, p.ctypes.data, s.ctypes.data, h.ctypes.data,
                                            float(out_scale), float(tau_min)), self._h)

    FILTERED = ("rho", "ux", "uy", "uz", "uxux", "uyuy", "uzuz", "uxuy", "uxuz", "uyuz")

    def filtered_fields(self, factor: int) -> dict:
        """Box-filtered (width `factor`) fields of the last step, as coarse (z, y, x) arrays."""
        p = self._shape()
        nc = (p[0] // factor) * (p[1] // factor) * (p[2] // factor)
        out = np.empty(10 * nc, self.dtype)
        _check(self._L.tlbm_filtered_fields(self._h, factor, out.ctypes.data), self._h)
        cz, cy, cx = p[2] // factor, p[1] // factor, p[0] // factor
        return {k: out[i * nc:(i + 1) * nc].reshape(cz, cy, cx)
                for i, k in enumerate(self.FILTERED)}

    PROCESSED = ("ux", "uy", "uz", "velmag", "Fx", "Fy", "Fz", "pressure")
    PROCESSED_AVG = ("ux", "uy", "uz", "velmag", "pressure")

    def processed_fields(self, time_avg: bool = False) -> dict:
        """processTLBM.py's fields (physical units, pressure - pRef, |u|, forces) of the last
        step, or of the time averages, computed on the GPU; (z, y, x) float32 arrays."""
        nx, ny, nz = self._shape()
        n = nx * ny * nz
        names = self.PROCESSED_AVG if time_avg else self.PROCESSED
        out = np.empty(len(names) * n, np.float32)
        _check(self._L.tlbm_processed_fields(self._h, int(bool(time_avg)), out.ctypes.data),
               self._h)
        return {k: out[i * n:(i + 1) * n].reshape(nz, ny, nx) for i, k in enumerate(names)}

    def write_processed_data(self, time_avg: bool = False) -> None:
        """out{k}.h5 + data{k}.xmf (or timeAvg.h5/.xmf) in the run directory."""
        _check(self._L.tlbm_write_processed_data(self._h, int(bool(time_avg))), self._h)

    def _shape(self):
        if not hasattr(self, "_dims"):
            raise TLBMError(ERR_INVALID_ARGUMENT, "lattice dimensions unknown for this handle")
        return self._dims

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._L.tlbm_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def problem_from_params(p) -> Problem:
    """ctypes Problem from a ``geometry.Params``."""
    pr = Problem()
    pr.lattice = p.lattice.encode()
    for f in ("dynamics", "num_ts", "ts_rep_freq", "warmup_ts", "plot_freq", "nx", "ny", "nz",
              "p_ref_idx"):
        setattr(pr, f, int(getattr(p, f)))
    pr.restart_flag = int(p.restart)
    pr.time_avg_flag = int(p.time_avg)
    pr.ss_data_flag = int(p.ss_flag)
    for f in ("cs", "rho_lbm", "u_lbm", "omega", "lx_p", "ly_p", "lz_p"):
        setattr(pr, f, float(getattr(p, f)))
    pr.t_conv, pr.l_conv, pr.p_conv = float(p.t_conv), float(p.l_conv), float(p.p_conv)
    return pr


def run_like_tlbmexec(part: TLBMPartition) -> None:
    """The reference's main loop (src/tLBM.cpp:45-61) over a partition."""
    nts, pf, wu = part.get_num_ts(), part.get_plot_freq(), part.get_warmupTs()
    for ts in range(nts):
        part.take_LBM_time_step(ts % 2)
        if (ts + 1) % pf == 0 and ts + 1 > wu:
            part.write_data()
    if part.get_time_avg_flag() == 1:
        part.write_time_avg_data()


class Ensemble:
    """A batch of independent channels advanced by one persistent launch per step
    (``tlbm_ensemble_*`` in include/tlbm.h)."""

    _SIG = {
        "tlbm_ensemble_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p,
                                                ctypes.POINTER(ctypes.c_void_p)]),
        "tlbm_ensemble_destroy": (ctypes.c_int, [ctypes.c_void_p]),
        "tlbm_ensemble_set_tiles": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_int] * 3),
        "tlbm_ensemble_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]
                                   + [ctypes.POINTER(ctypes.c_int)] * 3),
        "tlbm_ensemble_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
        "tlbm_ensemble_time_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                    ctypes.POINTER(ctypes.c_float)]),
        "tlbm_ensemble_copy_macros": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]
                                      + [ctypes.c_void_p] * 4),
        "tlbm_ensemble_mass": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_double)]),
        "tlbm_ensemble_cells": (ctypes.c_int64, [ctypes.c_void_p]),
        "tlbm_ensemble_kernel_launches": (ctypes.c_int64, [ctypes.c_void_p]),
        "tlbm_ensemble_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    }

    def __init__(self, problems, nd_types, precision="f32", device=0, block_x=0, block_y=0):
        L = library()
        for name, (res, args) in self._SIG.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        self._L = L
        n = len(problems)
        self._probs = (Problem * n)(*problems)
        if len(nd_types) != n:
            raise ValueError("%d problems and %d node-type arrays" % (n, len(nd_types)))
        self._nd = [_sized(a, np.int32, int(pr.nx) * int(pr.ny) * int(pr.nz), "nd_types[%d]" % k)
                    for k, (a, pr) in enumerate(zip(nd_types, problems))]
        ptrs = (ctypes.c_void_p * n)(*[a.ctypes.data for a in self._nd])
        o = options(precision, "fast", block_x, block_y, device)
        self._h = ctypes.c_void_p()
        st = L.tlbm_ensemble_create(n, ctypes.cast(self._probs, ctypes.c_void_p),
                                    ctypes.cast(ptrs, ctypes.c_void_p), ctypes.byref(o),
                                    ctypes.byref(self._h))
        if st != OK:
            raise TLBMError(st, L.tlbm_ensemble_last_error(None).decode())
        self.sizes = [p.nx * p.ny * p.nz for p in problems]
        self.dtype = np.float64 if precision == "f64" else np.float32

    def _check(self, st):
        if st != OK:
            raise TLBMError(st, self._L.tlbm_ensemble_last_error(self._h).decode())

    def set_tiles(self, bx, by, cells_per_thread=1):
        """bx * by threads per block (bx a multiple of 32, at most 256), each taking
        cells_per_thread cells: a tile is that many consecutive cells of one z-plane."""
        self._check(self._L.tlbm_ensemble_set_tiles(self._h, bx, by, cells_per_thread))

    def autotune(self, steps=20):
        v = [ctypes.c_int(0) for _ in range(3)]
        self._check(self._L.tlbm_ensemble_autotune(self._h, steps, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def run(self, first_ts, nsteps):
        self._check(self._L.tlbm_ensemble_run(self._h, first_ts, nsteps))

    def time_steps(self, first_ts, nsteps):
        ms = ctypes.c_float(0)
        self._check(self._L.tlbm_ensemble_time_steps(self._h, first_ts, nsteps, ctypes.byref(ms)))
        return ms.value

    def macros(self, channel):
        n = self.sizes[channel]
        out = [np.empty(n, self.dtype) for _ in range(4)]
        self._check(self._L.tlbm_ensemble_copy_macros(self._h, channel,
                                                      *[a.ctypes.data for a in out]))
        return out

    def mass(self, channel):
        m = ctypes.c_double(0)
        self._check(self._L.tlbm_ensemble_mass(self._h, channel, ctypes.byref(m)))
        return m.value

    @property
    def cells(self):
        return self._L.tlbm_ensemble_cells(self._h)

    def kernel_launches(self):
        return self._L.tlbm_ensemble_kernel_launches(self._h)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.tlbm_ensemble_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MlpTrainer:
    """GPU training set and Adam optimiser of the learned closure (``tlbm_mlp_*``)."""

    def __init__(self, features, targets, seed: int = 0, device: int = 0):
        L = library()
        self._L = L
        self.n_params = L.tlbm_mlp_num_params()
        self._x = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 8)
        self._t = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1)
        self.n = len(self._t)
        self._h = ctypes.c_void_p()
        st = L.tlbm_mlp_create(self.n, self._x.ctypes.data, self._t.ctypes.data, seed, device,
                               ctypes.byref(self._h))
        if st != OK:
            raise TLBMError(st, L.tlbm_mlp_last_error(None).decode())

    def _check(self, st):
        if st != OK:
            raise TLBMError(st, self._L.tlbm_mlp_last_error(self._h).decode())

    def set_params(self, p):
        p = _sized(p, np.float32, self.n_params, "params")
        self._check(self._L.tlbm_mlp_set_params(self._h, p.ctypes.data))

    def params(self):
        p = np.empty(self.n_params, np.float32)
        self._check(self._L.tlbm_mlp_get_params(self._h, p.ctypes.data))
        return p

    def loss_grad(self, first: int = 0, count: int | None = None):
        count = self.n - first if count is None else count
        loss = ctypes.c_float(0)
        g = np.empty(self.n_params, np.float32)
        self._check(self._L.tlbm_mlp_loss_grad(self._h, first, count, ctypes.byref(loss),
                                               g.ctypes.data))
        return loss.value, g

    def train(self, epochs: int, batch: int, lr: float):
        losses = np.empty(epochs, np.float32)
        self._check(self._L.tlbm_mlp_train(self._h, epochs, batch, lr, losses.ctypes.data))
        return losses

    def predict(self, features):
        x = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 8)
        y = np.empty(len(x), np.float32)
        self._check(self._L.tlbm_mlp_predict(self._h, len(x), x.ctypes.data, y.ctypes.data))
        return y

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.tlbm_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
