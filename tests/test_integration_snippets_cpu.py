"""The bindings INTEGRATION.md shows a maintainer: its C++ driver compiles against
include/tlbm.h and links against the engine library, and its Python stub is valid Python.
Nothing is run (both would need a GPU)."""

import os
import re
import shutil
import subprocess

import pytest

from tlbm_gb300 import build as B

DOC = os.path.join(B.REPO, "INTEGRATION.md")


def blocks(lang):
    text = open(DOC).read()
    return re.findall(r"```%s\n(.*?)```" % lang, text, flags=re.S)


def test_cpp_driver_compiles_and_links(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    B.build()
    src = [b for b in blocks("cpp") if "int main" in b]
    assert src, "no C++ driver in INTEGRATION.md"
    f = tmp_path / "driver.cpp"
    f.write_text(src[0])
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-I" + os.path.join(B.REPO, "include"),
                        str(f), "-L" + os.path.dirname(B.LIB), "-ltlbm_gb300",
                        "-o", str(tmp_path / "driver")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_python_stub_is_valid():
    src = blocks("python")
    assert src
    for b in src:
        compile(b, "INTEGRATION.md", "exec")


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
