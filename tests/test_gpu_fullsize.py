"""The benchmark's own workload at full size: the 512x256x256 sphere pack (33.5 M cells, D3Q19
BGK + Smagorinsky cs = 0.1, Re 200, FP64), built by bench.workload. The headline form (fast
FP64: Q1.62 storage, fixed-point fluid collision) runs against the reference-arithmetic kernel,
whose files are byte-identical to the reference's own build on the golden cases. After 20 steps
the fields and the force agree to 1e-12 of each field's largest value, and the global FP64 mass
of the two runs agrees to 1e-13. The end-to-end read-back (tlbm_copy_outputs_async into
page-locked buffers, overlapping two more steps) returns exactly the synchronous copies' values."""

import os
import sys

import numpy as np
import pytest

import tlbm_gb300 as T
from cases_util import rel_inf

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STEPS = 20


@pytest.fixture(scope="module")
def workload():
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        lattice, nx, ny, nz, seed, steps = "D3Q19", 512, 256, 256, 2024, STEPS

    return bench.workload(Args())


def test_headline_form_matches_reference_arithmetic_at_full_size(workload):
    g, p = workload
    assert g.num_nodes == 512 * 256 * 256
    out, mass = {}, {}
    for arith in ("reference", "fast"):
        part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                           arithmetic=arith)
        part.run(0, STEPS)
        out[arith] = part.macros() + part.force()
        mass[arith] = part.mass()
        if arith == "fast":
            host = [T.host_empty(g.num_nodes, np.float64) for _ in range(7)]
            part.outputs_async(host)
            part.run(STEPS, 2)  # the copies overlap these steps
            part.synchronize()
            for name, a, b in zip("ux uy uz rho Fx Fy Fz".split(), host, out[arith]):
                assert np.array_equal(a, b), name
        part.close()
    errs = [rel_inf(a, b) for a, b in zip(out["fast"], out["reference"])]
    print("512x256x256 pack, %d steps: rel_inf ux %.2e uy %.2e uz %.2e rho %.2e Fx %.2e Fy %.2e "
          "Fz %.2e; mass %.17g vs %.17g" % (STEPS, *errs, mass["fast"], mass["reference"]))
    assert all(np.all(np.isfinite(a)) for a in out["fast"])
    assert max(np.abs(f).max() for f in out["reference"][4:]) > 1e-4  # the spheres carry a force
    assert max(errs) <= 1e-12, errs
    assert abs(mass["fast"] - mass["reference"]) <= 1e-13 * mass["reference"]
