"""The HDF5 subset for restart.h5 and out{n}.h5 (no HDF5 library in this image): the engine's
C++ writer/reader (tlbm_gb300/csrc/h5lite.cpp, through tests/h5_harness.cpp) and the package's
numpy writer/reader (tlbm_gb300/h5.py) are separate implementations of the file format
specification's layouts, and each reads what the other writes.  The two writers also make
different valid choices (symbol-table node size, a local-heap free block, extra header
messages, data placed beside or after the metadata), so each reader sees more than its own
writer's habits."""

import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from tlbm_gb300 import h5

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("h5") / "h5_harness")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", os.path.join(HERE, "h5_harness.cpp"),
                        os.path.join(HERE, "..", "tlbm_gb300", "csrc", "h5lite.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def cpp_read(harness, path, name):
    r = subprocess.run([harness, "read", path, name], capture_output=True, text=True, timeout=60)
    if r.returncode != 0:
        raise ValueError(r.stdout.strip())
    lines = r.stdout.split("\n")
    dims = tuple(int(t) for t in lines[0].split()[1:])
    vals = np.array([float.fromhex(t) for t in lines[1:] if t], np.float32)
    return vals.reshape(dims)


NAMES = ["velocity/x", "velocity/y", "velocity/z", "density/rho", "pres_group/presmag", "top"]


def test_cpp_writer_read_by_numpy_reader(harness, tmp_path):
    f = str(tmp_path / "a.h5")
    n = 64
    r = subprocess.run([harness, "write", f, str(n)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    for d, name in enumerate(NAMES):
        a = h5.read(f, name)
        want = (d + np.arange(n) / 8.0).astype(np.float32)
        assert a.dtype == np.float32
        assert a.shape == ((2, 2, n // 4) if d == 4 else (n,))
        assert np.array_equal(a.reshape(-1), want), name
    with pytest.raises(KeyError):
        h5.read(f, "velocity/w")


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_numpy_writer_read_by_cpp_reader(harness, tmp_path, dtype):
    f = str(tmp_path / "b.h5")
    rng = np.random.default_rng(5)
    data = {"velocity/x": rng.standard_normal(1000).astype(dtype),
            "velocity/y": rng.standard_normal(1000).astype(dtype),
            "velocity/z": rng.standard_normal(1000).astype(dtype),
            "density/rho": (1 + 0.01 * rng.standard_normal((5, 10, 20))).astype(dtype),
            "a/b/c/deep": np.arange(7, dtype=dtype)}
    h5.write(f, data)
    for name, a in data.items():
        got = cpp_read(harness, f, name)
        assert got.shape == a.shape
        # float64 data read as NATIVE_FLOAT: rounded to nearest float32
        assert np.array_equal(got, a.astype(np.float32)), name
        back = h5.read(f, name)
        assert back.dtype == a.dtype and np.array_equal(back, a)
    with pytest.raises(ValueError, match="no object named"):
        cpp_read(harness, f, "density/pressure")


def test_writer_round_trips_and_sizes(harness, tmp_path):
    """Each implementation reads its own files; an empty group list and many groups work."""
    f = str(tmp_path / "c.h5")
    data = {"g%d/v" % k: np.full(3, k, np.float32) for k in range(8)}
    h5.write(f, data)
    for name, a in data.items():
        assert np.array_equal(h5.read(f, name), a)
        assert np.array_equal(cpp_read(harness, f, name), a)
    with pytest.raises(ValueError):
        h5.write(str(tmp_path / "d.h5"), {"g/v%d" % k: np.zeros(1) for k in range(17)})


def test_unsupported_layouts_are_reported(harness, tmp_path):
    """A chunked layout and a filter pipeline are refused by both readers, not misread."""
    f = str(tmp_path / "e.h5")
    h5.write(f, {"x": np.arange(4, dtype=np.float32)})
    raw = bytearray(open(f, "rb").read())
    # the dataset's layout message (type 8, version 3, class 1): make it chunked (class 2)
    i = raw.find(struct.pack("<HH", 8, 24))
    assert i > 0 and raw[i + 8] == 3 and raw[i + 9] == 1
    raw[i + 9] = 2
    g = str(tmp_path / "f.h5")
    open(g, "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="chunked"):
        h5.read(g, "x")
    with pytest.raises(ValueError, match="chunked"):
        cpp_read(harness, g, "x")
    # the NIL padding message turned into a filter pipeline message (type 11)
    raw[i + 9] = 1
    j = raw.find(struct.pack("<HH", 0, 8), i)
    assert j > 0
    raw[j:j + 2] = struct.pack("<H", 11)
    open(g, "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="filtered"):
        h5.read(g, "x")
    with pytest.raises(ValueError, match="filtered"):
        cpp_read(harness, g, "x")
    with pytest.raises(ValueError, match="not an HDF5 file"):
        open(g, "wb").write(b"plain text, not HDF5 at all" * 4)
        cpp_read(harness, g, "x")


def _library_file():
    """An HDF5 file written by the HDF5 library itself (MATLAB 7.3 format: a 512-byte user
    block, superblock 0, a version-2 layout message, float64 data), shipped with scipy's test
    data; its dataset testdouble holds 0, pi/4, ..., 2 pi as a 9 x 1 array."""
    try:
        import scipy.io.matlab as m
    except ImportError:
        return None
    path = os.path.join(os.path.dirname(m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    return path if os.path.exists(path) else None


def test_readers_read_a_file_written_by_the_hdf5_library(harness):
    path = _library_file()
    if path is None:
        pytest.skip("scipy's HDF5-based MAT test file is not installed")
    want = np.arange(9) * np.pi / 4
    a = h5.read(path, "testdouble")
    assert a.dtype == np.float64 and a.shape == (9, 1)
    assert np.allclose(a.reshape(-1), want, rtol=1e-15, atol=1e-15)
    b = cpp_read(harness, path, "testdouble")
    assert b.shape == (9, 1) and np.array_equal(b, a.astype(np.float32))


def _v2_file(path):
    """A file in HDF5's newer layouts, assembled by hand from the specification: superblock
    version 2, version-2 object headers ("OHDR", with a continuation chunk "OCHK"), a root group
    held as link messages, version-2 dataspaces, and one compact and one contiguous float32
    dataset.  Checksums are left zero (neither reader verifies them)."""
    img = bytearray(48)  # superblock, written last

    def put(b):
        at = len(img)
        img.extend(b)
        return at

    def ohdr(messages):
        body = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in messages)
        return b"OHDR" + struct.pack("<BBI", 2, 2, len(body)) + body + b"\0" * 4

    space = lambda dims: struct.pack("<BBBB", 2, len(dims), 0, 1) + b"".join(
        struct.pack("<Q", d) for d in dims)
    f32 = struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 31, 0, 4, 0, 32, 23, 8, 0, 23, 127)
    small = np.array([1.5, -2.25, 3.0], np.float32)
    big = np.arange(12, dtype=np.float32).reshape(3, 4) / 4
    compact = ohdr([(1, space([3])), (3, f32),
                    (8, struct.pack("<BBH", 3, 0, small.nbytes) + small.tobytes())])
    a_small = put(compact)
    data = put(big.tobytes())
    a_big = put(ohdr([(1, space([3, 4])), (3, f32),
                      (8, struct.pack("<BBQQ", 3, 1, data, big.nbytes))]))

    def link(name, addr):
        return (6, struct.pack("<BBB", 1, 0, len(name)) + name.encode() + struct.pack("<Q", addr))

    cont = [link("big", a_big)]
    cbody = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in cont)
    a_chunk = put(b"OCHK" + cbody + b"\0" * 4)
    root = put(ohdr([link("small", a_small),
                     (0x10, struct.pack("<QQ", a_chunk, 4 + len(cbody) + 4))]))
    sb = b"\x89HDF\r\n\x1a\n" + struct.pack("<BBBB", 2, 8, 8, 0)
    sb += struct.pack("<QQQQ", 0, h5.UNDEF, len(img), root) + b"\0" * 4
    img[0:48] = sb
    open(path, "wb").write(bytes(img))
    return small, big


def test_readers_take_newer_layouts(harness, tmp_path):
    f = str(tmp_path / "v2.h5")
    small, big = _v2_file(f)
    for name, want in (("small", small), ("big", big)):
        a = h5.read(f, name)
        assert a.shape == want.shape and np.array_equal(a, want), name
        b = cpp_read(harness, f, name)
        assert b.shape == want.shape and np.array_equal(b, want), name
    with pytest.raises(KeyError):
        h5.read(f, "missing")
