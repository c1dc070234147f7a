"""tlbm_mass_static: the allocation-free FP64 mass reduction, through the C ABI.

It exists for callers that cannot allocate device memory while running (a whole-GPU memory
pool reserved up front, or a no-allocation-after-start-up policy).  These checks hand it a
population array and an output that the test owns in device memory and compare its result with
tlbm_mass (the allocating entry point) on the same populations, on two calls in a row: the
static scratch array keeps the first call's partial sums, and the second call must not depend
on them.  The file is named to be collected last.
"""

import ctypes

import numpy as np
import pytest

import tlbm_gb300 as T
from tlbm_gb300 import build as B
from tlbm_gb300 import geometry as G

pytestmark = pytest.mark.gpu


def entry():
    B.build()
    L = T.library()
    fn = L.tlbm_mass_static
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p]
    return fn


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_mass_static_matches_tlbm_mass_on_two_calls(precision):
    torch = pytest.importorskip("torch")
    fn = entry()
    g = G.sphere_in_box(40, 24, 30, 5, 20, 12, 10)
    p = G.params_lattice_units(g, "D3Q19", 0.05, 40.0, 10.0, 50, cs=0.1)
    part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision=precision,
                                       arithmetic="fast")
    n, q = g.num_nodes, 19
    dtype = torch.float64 if precision == "f64" else torch.float32
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    ts = 0
    for call in range(2):
        part.run(ts, 7 + call)
        ts += 7 + call
        want = part.mass()
        # the same post-collision populations, in the engine's layout, owned by the caller
        aos = part.populations(1).reshape(n, q)
        soa = torch.from_numpy(np.ascontiguousarray(aos.T)).to(device="cuda", dtype=dtype)
        torch.cuda.synchronize()
        st = fn(q, T.PREC[precision], n, soa.data_ptr(), out.data_ptr(), None)
        assert st == T.OK
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - want) <= 1e-12 * abs(want), (call, got, want)
    part.close()


# D3Q19 weights as the kernels hold them: float literals (include/D3Q19LatticeStructure.hpp)
W19 = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32).astype(np.float64)


@pytest.mark.parametrize("precision", ["bf16", "f16"])
def test_mass_static_shifted_storage_on_two_calls(precision):
    """16-bit kinds store f - w_i: the sum adds w_i back per population.  The caller's array
    holds the 16-bit remainders of a seeded non-equilibrium state; the result must equal the
    FP64 sum of float(stored) + w_i on two calls with different contents."""
    torch = pytest.importorskip("torch")
    fn = entry()
    q, n = 19, 40 * 24 * 30 + 7  # a partial last block
    dt = torch.bfloat16 if precision == "bf16" else torch.float16
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(5)
    for call in range(2):
        f = W19[:, None] * rng.uniform(0.9, 1.1, size=(q, n))
        stored = torch.from_numpy(f - W19[:, None]).to(dt)
        want = float((stored.to(torch.float64).numpy() + W19[:, None]).sum())
        dev = stored.to("cuda")
        torch.cuda.synchronize()
        assert fn(q, T.PREC[precision], n, dev.data_ptr(), out.data_ptr(), None) == T.OK
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - want) <= 1e-12 * abs(want), (call, got, want)


def test_mass_static_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    fn = entry()
    buf = torch.zeros(32, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    limit = 65536 * 1024
    assert fn(19, T.PREC["f64"], limit + 1, buf.data_ptr(), out.data_ptr(), None) == \
        T.ERR_OUT_OF_RANGE
    assert fn(19, T.PREC["f64"], 0, buf.data_ptr(), out.data_ptr(), None) == T.ERR_INVALID_ARGUMENT
    assert fn(20, T.PREC["f64"], 1, buf.data_ptr(), out.data_ptr(), None) == T.ERR_INVALID_ARGUMENT
