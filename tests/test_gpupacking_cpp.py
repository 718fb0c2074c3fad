"""The C++ host class GpuPacking (the reference's Packing interface over the C ABI)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_gpupacking.cpp")


def test_header_compiles():
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", SRC], check=True)


@pytest.mark.gpu
def test_gpupacking_known_answers(engine, tmp_path):
    exe = tmp_path / "test_gpupacking"
    libdir = os.path.dirname(engine.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", SRC, "-o", str(exe), f"-L{libdir}", "-lrampack_gb300",
                    f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok" in out.stdout
