"""The bindings a maintainer copies into the reference (tlbm_gb300/examples): the rewritten
driver compiles against include/tlbm.h and links against the engine library, and the ctypes
stub is valid Python.  Nothing is run (both would need a GPU)."""

import os
import shutil
import subprocess

import pytest

from tlbm_gb300 import build as B

EXAMPLES = os.path.join(B.HERE, "examples")


def test_cpp_driver_compiles_and_links(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    B.build()
    src = os.path.join(EXAMPLES, "tLBM_main_over_abi.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-I" + os.path.join(B.REPO, "include"),
                        src, "-L" + os.path.dirname(B.LIB), "-ltlbm_gb300",
                        "-o", str(tmp_path / "driver")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_python_stub_is_valid():
    path = os.path.join(EXAMPLES, "ctypes_stub.py")
    compile(open(path).read(), path, "exec")


def test_header_is_strict_c(tmp_path):
    """include/tlbm.h is a C header (cgo, ctypes and C callers): it compiles as pedantic C99
    and a C program links against the engine with it."""
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("gcc not available")
    B.build()
    f = tmp_path / "use.c"
    f.write_text('#include "tlbm.h"\n'
                 "int main(void) { tlbm_options o; tlbm_default_options(&o);\n"
                 "  return o.struct_size > 0 ? 0 : 1; }\n")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I" + os.path.join(B.REPO, "include"), str(f),
                        "-L" + os.path.dirname(B.LIB), "-ltlbm_gb300", "-o", str(tmp_path / "use")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
