"""The C-ABI library without a GPU: it loads, exports every function include/tlbm.h declares,
and rejects malformed inputs (which it checks before touching the device) with the right
status -- the conditions where the reference throws or aborts."""

import ctypes
import os
import subprocess

import numpy as np
import pytest

import tlbm_gb300 as T
from tlbm_gb300 import build as B
from tlbm_gb300 import geometry as G


@pytest.fixture(scope="session")
def lib():
    B.build()
    return T.library()


def test_exports_every_declared_symbol(lib):
    declared = T.declared_symbols()
    assert len(declared) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", B.LIB], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        assert hasattr(lib, s)


def test_status_strings(lib):
    assert lib.tlbm_status_string(T.OK) == b"ok"
    assert lib.tlbm_status_string(T.ERR_FORMAT) == b"malformed input"


def test_default_options(lib):
    o = T.Options()
    lib.tlbm_default_options(ctypes.byref(o))
    assert o.struct_size == ctypes.sizeof(T.Options)
    assert o.precision == T.PREC["f32"] and o.arithmetic == 0


def small_inputs(tmp, lattice="D3Q19", nd=None, parts=None):
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    if nd is not None:
        g.nd_type = nd
    p = G.params_lattice_units(g, lattice, 0.05, 20.0, 4.0, 10)
    G.write_inputs(str(tmp), g, p, parts)
    return g, p


def create_status(lib, workdir, rank=0, size=1):
    h = ctypes.c_void_p()
    st = lib.tlbm_create(str(workdir).encode(), rank, size, ctypes.byref(h))
    return st, lib.tlbm_get_last_error(None).decode()


def test_missing_params(lib, tmp_path):
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_IO and "params.lbm" in msg


def test_invalid_lattice(lib, tmp_path):
    small_inputs(tmp_path)
    txt = open(tmp_path / "params.lbm").read().replace("D3Q19", "D3Q13")
    open(tmp_path / "params.lbm", "w").write(txt)
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_INVALID_ARGUMENT and "Invalid Lattice Structure" in msg


def test_malformed_params(lib, tmp_path):
    small_inputs(tmp_path)
    lines = open(tmp_path / "params.lbm").read().splitlines(True)
    lines[2] = "lots \n"
    open(tmp_path / "params.lbm", "w").write("".join(lines))
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_FORMAT


def test_truncated_params(lib, tmp_path):
    small_inputs(tmp_path)
    lines = open(tmp_path / "params.lbm").read().splitlines(True)
    open(tmp_path / "params.lbm", "w").write("".join(lines[:10]))
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_FORMAT and "15" in msg


def test_ndtype_wrong_length(lib, tmp_path):
    small_inputs(tmp_path)
    with open(tmp_path / "ndType.lbm", "a") as fh:
        fh.write("0 \n")
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_FORMAT and "ndType.lbm" in msg
    small_inputs(tmp_path)
    lines = open(tmp_path / "ndType.lbm").read().splitlines(True)
    open(tmp_path / "ndType.lbm", "w").write("".join(lines[:-5]))
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_FORMAT


def test_ndtype_bad_code(lib, tmp_path):
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    nd = g.nd_type.copy()
    nd[17] = 4
    small_inputs(tmp_path, nd=nd)
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_OUT_OF_RANGE and "type 4" in msg


def test_ndtype_bad_code_lowest_node_named(lib):
    """The node types are checked in chunks on several host threads; the error still names the
    lowest offending node, whichever chunk finds one first."""
    nx, ny, nz = 256, 128, 128  # 4.19 M nodes: four chunks of 2^20
    nd = np.zeros(nx * ny * nz, np.int32)
    nd[3_900_000] = 9
    nd[2_500_000] = 7
    nd[1_234_567] = -1
    st, msg = _create(_problem(nx, ny, nz), nd, precision="f64")
    assert st == T.ERR_OUT_OF_RANGE and "node 1234567 " in msg and "type -1" in msg
    nd[1_234_567] = 0
    st, msg = _create(_problem(nx, ny, nz), nd, precision="f64")
    assert st == T.ERR_OUT_OF_RANGE and "node 2500000 " in msg and "type 7" in msg
    # two bad codes in one chunk ([2^20, 2^21)): its branch-free pass only flags it, and the
    # rescan names the first
    nd[2_500_000] = nd[3_900_000] = 0
    nd[1_100_000] = 6
    nd[1_060_000] = 4
    st, msg = _create(_problem(nx, ny, nz), nd, precision="f64")
    assert st == T.ERR_OUT_OF_RANGE and "node 1060000 " in msg and "type 4" in msg


def test_parts_beyond_job_size(lib, tmp_path):
    parts = G.partition_1d(8, 8, 12, 3)
    small_inputs(tmp_path, parts=parts)
    st, msg = create_status(lib, tmp_path, size=2)
    assert st == T.ERR_OUT_OF_RANGE and "partition 2" in msg


def test_rank_must_be_zero(lib, tmp_path):
    small_inputs(tmp_path)
    st, msg = create_status(lib, tmp_path, rank=1)
    assert st == T.ERR_INVALID_ARGUMENT


def test_bad_config_file(lib, tmp_path):
    small_inputs(tmp_path)
    open(tmp_path / "tlbm.cfg", "w").write("precision f128\n")
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_INVALID_ARGUMENT and "precision" in msg


def test_bad_options_struct(lib, tmp_path):
    small_inputs(tmp_path)
    o = T.Options()
    lib.tlbm_default_options(ctypes.byref(o))
    o.struct_size = 3
    h = ctypes.c_void_p()
    st = lib.tlbm_create_ex(str(tmp_path).encode(), 0, 1, ctypes.byref(o), ctypes.byref(h))
    assert st == T.ERR_INVALID_ARGUMENT


def test_null_handle_calls(lib):
    assert lib.tlbm_step(None, 0) == T.ERR_INVALID_ARGUMENT
    assert lib.tlbm_get_num_ts(None) == -1
    assert lib.tlbm_destroy(None) == T.ERR_INVALID_ARGUMENT


def test_ensemble_input_validation(lib):
    """Ensemble inputs are checked before any device work: lattice and node types."""
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    p27 = G.params_lattice_units(g, "D3Q27", 0.04, 20.0, 4.0, 10)
    with pytest.raises(T.TLBMError) as e:
        T.Ensemble([T.problem_from_params(p27)], [g.nd_type])
    assert e.value.status == T.ERR_UNSUPPORTED
    p19 = G.params_lattice_units(g, "D3Q19", 0.04, 20.0, 4.0, 10)
    nd = g.nd_type.copy()
    nd[3] = 5
    with pytest.raises(T.TLBMError) as e:
        T.Ensemble([T.problem_from_params(p19)], [nd])
    assert e.value.status == T.ERR_OUT_OF_RANGE


def test_python_mirror_raises(lib, tmp_path):
    with pytest.raises(T.TLBMError) as e:
        T.TLBMPartition(str(tmp_path))
    assert e.value.status == T.ERR_IO


def _problem(nx, ny, nz, dynamics=1):
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    p = G.params_lattice_units(g, "D3Q19", 0.04, 20.0, 4.0, 10)
    prob = T.problem_from_params(p)
    prob.nx, prob.ny, prob.nz, prob.dynamics = nx, ny, nz, dynamics
    return prob


def _create(prob, nd, **kw):
    o = T.options(**kw)
    h = ctypes.c_void_p()
    st = T.library().tlbm_create_from_arrays(ctypes.byref(prob), nd.ctypes.data, None, None,
                                              ctypes.byref(o), ctypes.byref(h))
    return st, T.library().tlbm_get_last_error(None).decode()


@pytest.mark.parametrize("dims,status", [((65536, 65536, 1), T.ERR_UNSUPPORTED),  # >= 2^31 cells
                                         ((1, 1, 70000), T.ERR_UNSUPPORTED),      # nz > 65535
                                         ((0, 8, 8), T.ERR_FORMAT)])
def test_lattice_size_limits(lib, dims, status):
    """Sizes beyond what one device kernel grid addresses are refused before the node types are
    read or any memory is allocated (the node-type array here is a single value)."""
    st, msg = _create(_problem(*dims), np.zeros(1, np.int32), precision="f64")
    assert st == status and msg


@pytest.mark.parametrize("kw,dynamics,status", [
    ({"precision": "bf16", "arithmetic": "reference"}, 1, T.ERR_INVALID_ARGUMENT),
    ({"precision": "bf16m", "arithmetic": "reference"}, 1, T.ERR_INVALID_ARGUMENT),
    ({"precision": "f64", "arithmetic": "reference", "rbgk": True}, 2, T.ERR_UNSUPPORTED),
    ({"precision": "f64", "arithmetic": "reference", "mrt": True}, 3, T.ERR_UNSUPPORTED),
    ({"precision": "f64", "arithmetic": "fast", "mrt": True, "ghost_rate": 2.5}, 3,
     T.ERR_INVALID_ARGUMENT)])
def test_option_combinations_refused_before_the_device(lib, kw, dynamics, status):
    nd = np.zeros(8 * 8 * 12, np.int32)
    st, msg = _create(_problem(8, 8, 12, dynamics), nd, **kw)
    assert st == status and msg


def test_host_alloc_arguments(lib):
    """tlbm_host_alloc refuses a NULL out-pointer and a zero size before calling CUDA;
    tlbm_host_free(NULL) is a no-op."""
    assert lib.tlbm_host_alloc(16, None) == T.ERR_INVALID_ARGUMENT
    p = ctypes.c_void_p(1)
    assert lib.tlbm_host_alloc(0, ctypes.byref(p)) == T.ERR_INVALID_ARGUMENT
    assert p.value is None
    assert lib.tlbm_host_free(None) == T.OK


def test_get_options_arguments(lib):
    """tlbm_get_options refuses a NULL handle or a bad struct_size without touching the device."""
    o = T.Options()
    o.struct_size = ctypes.sizeof(T.Options)
    assert lib.tlbm_get_options(None, ctypes.byref(o)) == T.ERR_INVALID_ARGUMENT
    assert lib.tlbm_get_options(None, None) == T.ERR_INVALID_ARGUMENT


def test_host_empty_fails_loudly_without_a_device(lib):
    """Page-locked host memory needs the CUDA driver: without a GPU, host_empty raises."""
    import shutil
    smi = shutil.which("nvidia-smi")
    if smi and subprocess.run([smi], capture_output=True).returncode == 0:
        pytest.skip("a GPU is present")
    with pytest.raises(T.TLBMError):
        T.host_empty(16, np.float32)


@pytest.mark.parametrize("cfg,word", [("arithmetic exact\n", "arithmetic"),
                                      ("colour blue\n", "unknown key"),
                                      ("precision bf16\narithmetic reference\n", ""),
                                      ("precision bf16m\narithmetic reference\n", "")])
def test_config_file_refusals(lib, tmp_path, cfg, word):
    """tlbm.cfg is parsed and checked before any device work: unknown keys and values, and
    16-bit storage with the reference arithmetic (which has no 16-bit form), are refused."""
    small_inputs(tmp_path)
    open(tmp_path / "tlbm.cfg", "w").write(cfg)
    st, msg = create_status(lib, tmp_path)
    assert st == T.ERR_INVALID_ARGUMENT and msg
    assert word in msg


def test_python_mirror_checks_array_sizes_before_the_abi(lib):
    """The C ABI reads a fixed number of values through each pointer; the Python mirror refuses
    arrays of the wrong length before any call (a short array would be read out of bounds)."""
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    p = G.params_lattice_units(g, "D3Q19", 0.04, 20.0, 4.0, 10)
    prob = T.problem_from_params(p)
    with pytest.raises(ValueError, match="nd_type"):
        T.TLBMPartition.from_arrays(prob, g.nd_type[:-1])
    with pytest.raises(ValueError, match="parts"):
        T.TLBMPartition.from_arrays(prob, g.nd_type, parts=np.zeros(5, np.int32))
    with pytest.raises(ValueError, match="nd_types"):
        T.Ensemble([prob, prob], [g.nd_type, g.nd_type[:10]])
    with pytest.raises(ValueError, match="node-type arrays"):
        T.Ensemble([prob, prob], [g.nd_type])
    a = T._sized(np.arange(6).reshape(2, 3), np.float32, 6, "x")
    assert a.shape == (6,) and a.dtype == np.float32 and a.flags.c_contiguous


def test_create_from_arrays_null_arguments(lib):
    g = G.sphere_in_box(8, 8, 12, 2, 4, 4, 5)
    p = G.params_lattice_units(g, "D3Q19", 0.04, 20.0, 4.0, 10)
    prob = T.problem_from_params(p)
    o = T.options("f64")
    h = ctypes.c_void_p()
    assert lib.tlbm_create_from_arrays(ctypes.byref(prob), None, None, None, ctypes.byref(o),
                                       ctypes.byref(h)) == T.ERR_INVALID_ARGUMENT
    assert h.value is None
    assert lib.tlbm_create_from_arrays(None, g.nd_type.ctypes.data, None, None, ctypes.byref(o),
                                       ctypes.byref(h)) == T.ERR_INVALID_ARGUMENT
    assert b"NULL" in lib.tlbm_get_last_error(None)
