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
