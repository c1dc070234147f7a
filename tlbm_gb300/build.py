"""Build the engine for sm_103a: libtlbm_gb300.so (C ABI) and the tLBMexec command line.

    python -m tlbm_gb300.build          # or tlbm_gb300.build.build()

Translation units compile in parallel with nvcc; objects go to tlbm_gb300/_build, the shared
library to tlbm_gb300/lib and the executable to tlbm_gb300/bin.  The reference-arithmetic
kernels are compiled with -fmad=false (no a*b+c contraction) so that they round exactly like
the CPU reference; the fast kernels are too, with every fused multiply-add written out, so the
single-lattice and ensemble kernels that inline the same cell code round identically.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIBDIR, "libtlbm_gb300.so")
# the benchmark's measurement of this GPU's FP64-pipe rate (not part of the engine's C ABI)
PEAKS_LIB = os.path.join(LIBDIR, "libtlbm_peaks.so")
EXE = os.path.join(BINDIR, "tLBMexec")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
          "-I" + os.path.join(REPO, "include")]

# (source, extra flags)
UNITS = [
    ("kernels_ref.cu", ["-fmad=false"]),
    ("kernels_common.cu", ["-fmad=false"]),
    ("kernels_fast.cu", ["-fmad=false"]),
    ("mass_static.cu", []),
    ("kernels_ensemble.cu", ["-fmad=false"]),
    ("ensemble.cpp", ["-x", "cu"]),
    ("kernels_mlp.cu", []),
    ("kernels_post.cu", ["-fmad=false"]),
    ("post.cpp", ["-x", "cu"]),
    ("h5lite.cpp", ["-x", "cu"]),
    ("mlp_trainer.cpp", ["-x", "cu"]),
    ("capi_mlp.cpp", ["-x", "cu"]),
    ("engine.cpp", ["-x", "cu"]),
    ("capi.cpp", ["-x", "cu"]),
]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tlbm_gb300")
    return p


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit (in parallel) and link; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "tlbm.h"))
    todo = []
    objs = []
    for src, extra in UNITS:
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [os.path.join(CSRC, src)] + headers):
            todo.append((src, extra))
    if todo:
        with ThreadPoolExecutor(max_workers=len(todo)) as ex:
            list(ex.map(lambda u: _compile(u[0], u[1], verbose), todo))
    if force or todo or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    peaks_src = os.path.join(CSRC, "peaks.cu")
    if force or _stale(PEAKS_LIB, [peaks_src]):
        obj = _compile("peaks.cu", [], verbose)
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", PEAKS_LIB, obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    main_src = os.path.join(CSRC, "tlbm_main.cpp")
    if force or _stale(EXE, [main_src, LIB, os.path.join(REPO, "include", "tlbm.h")]):
        cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(REPO, "include"), main_src,
               "-L" + LIBDIR, "-ltlbm_gb300", "-Wl,-rpath,$ORIGIN/../lib", "-o", EXE]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("tLBMexec link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
