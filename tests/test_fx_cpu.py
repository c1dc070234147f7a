"""The fixed-point FP64-storage collision (tlbm_gb300/csrc/physics_fx.cuh) compiled for the host:
random near-equilibrium cells collided by it and by a long-double evaluation of the reference's
formulas (moments, equilibrium with the reference's weights, Smagorinsky rate, BGK relaxation)
differ by at most 3 ulp of the result (2 ulp on D3Q19; the 3 ulp are the smallest D3Q15 and
D3Q27 populations, ~0.002, where one ulp is 4e-19), and most results are the nearest double.  The exact
double <-> fixed-point conversions, the integer reciprocal and the range guards are checked
too, and so are the output fields' helpers: the pair moments, the Q5.58 rounding of the force
sums and the two-step neighbour offsets of the force terms."""

import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("fx") / "fx_harness")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Wno-unknown-pragmas",
                        os.path.join(HERE, "fx_harness.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_conversions_reciprocal_and_guards(harness):
    r = subprocess.run([harness, "0"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:]


@pytest.mark.parametrize("smag", [0, 1])
@pytest.mark.parametrize("q,ulp", [(15, 3), (19, 2), (27, 3)])
def test_collision_within_ulps_of_exact(harness, q, ulp, smag):
    r = subprocess.run([harness, str(q), str(smag), "20000", str(q + smag)], capture_output=True,
                       text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:]
    m = re.search(r"largest difference ([0-9.e+-]+) ulp, ([0-9.e+-]+) % not the nearest", r.stdout)
    assert m, r.stdout
    assert float(m.group(1)) <= ulp
    assert float(m.group(2)) <= 20.0
