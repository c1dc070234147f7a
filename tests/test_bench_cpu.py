"""bench.py without a GPU: every name a function uses is defined (a stale reference would only
fail at run time on the GPU), the per-cell byte counts, and the argument defaults."""

import builtins
import os
import symtable
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def undefined_globals(path):
    src = open(path).read()
    top = symtable.symtable(src, path, "exec")
    defined = {s.get_name() for s in top.get_symbols()
               if s.is_assigned() or s.is_imported() or s.is_namespace()}
    bad = []

    def walk(t):
        for s in t.get_symbols():
            name = s.get_name()
            if (s.is_global() and s.is_referenced() and name not in defined
                    and not hasattr(builtins, name) and name not in ("__file__", "__name__")):
                bad.append((t.get_name(), name))
        for ch in t.get_children():
            walk(ch)

    walk(top)
    return bad


def test_bench_has_no_undefined_names():
    assert undefined_globals(os.path.join(ROOT, "bench.py")) == []


def test_cell_bytes_and_defaults():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.cell_bytes(19, "f64") == 305
    assert bench.cell_bytes(19, "f32") == 153
    assert bench.cell_bytes(19, "bf16") == 77
    assert bench.cell_bytes(19, "bf16m") == 109
    assert bench.cell_bytes(27, "f64") == 433
    sys.argv = ["bench.py"]
    a = bench.parse_args()
    assert (a.gpus, a.precision, a.lattice, a.nx, a.ny, a.nz) == (1, "f64", "D3Q19", 512, 256, 256)
    assert a.warmup >= 3
