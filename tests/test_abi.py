"""The C-ABI library loads and exports every entry point include/rampack_gb300.h declares,
and the ctypes mirrors of its structs have the C layout (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rampack_gb300.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(rp_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_entry_point(engine):
    lib = C.CDLL(engine.LIB_PATH)
    names = declared()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares each of them
    assert set(names) <= set(engine.SIGNATURES)


def test_struct_layouts_match_header(engine, tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "rampack_gb300.h"\nint main(void){printf("%zu %zu %zu %zu %zu\\n",'
                   ' sizeof(rp_move), sizeof(rp_shape_desc), sizeof(rp_grid_info), sizeof(rp_sweep_params),'
                   ' sizeof(rp_sweep_stats)); return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [engine.MOVE_DTYPE.itemsize, C.sizeof(engine.ShapeDesc), C.sizeof(engine.GridInfo),
                     C.sizeof(engine.SweepParams), C.sizeof(engine.SweepStats)]


def test_oracle_exports(oracle):
    lib = C.CDLL(oracle.ORACLE_SO)
    for name in ("rpo_create", "rpo_replay", "rpo_count_overlaps", "rpo_try_scaling", "rpo_draw_moves",
                 "rpo_sim_run"):
        assert hasattr(lib, name)
    assert lib.rpo_move_size() == 120


def test_engine_refuses_to_import_without_library(tmp_path):
    from rampack_gb300 import _lib
    with pytest.raises(ImportError):
        _lib.load(str(tmp_path / "missing.so")) if _lib._LIB is None else (_ for _ in ()).throw(ImportError())
