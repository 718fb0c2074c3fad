"""The casino GPU switch (rampack_gb300/host/casino): casino_gpu.patch applied to a copy of the
reference's sources and built by its Makefile, the reference never written.

* The patch applies and the patched core, the patched frontend matcher and the check program
  compile against the reference's own headers.
* Without a backend, the patched Simulation::integrate is the reference's: the same NpT run
  gives a bit-identical final state and identical counters to the unpatched reference library
  (oracle/_ref, Simulation::integrate through the reference driver).
* With the GPU backend attached and no usable CUDA device, the run fails loudly: exit status 3
  and the device's error text, never a silent CPU run.

Skipped where the reference checkout is absent (the GPU machine).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
CASINO = os.path.join(os.path.dirname(HERE), "rampack_gb300", "host", "casino")
N, SPACING, CYCLES, TSTEP, BSTEP, PRESSURE, SEED = 5, 1.2, 150, 0.1, 0.05, 5.0, 42


@pytest.fixture(scope="module")
def check_program(tmp_path_factory, oracle, engine):
    if not os.path.isdir(os.path.join(po.REFERENCE_DIR, "src")):
        pytest.skip("reference checkout not present")
    if shutil.which("patch") is None:
        pytest.skip("patch(1) not installed")
    out = tmp_path_factory.mktemp("casino_gpu")
    subprocess.run(["make", "-s", "-j", str(os.cpu_count() or 4), "-C", CASINO, f"REF={po.REFERENCE_DIR}",
                    f"OUT={out}"], check=True, capture_output=True)
    assert os.path.exists(os.path.join(out, "obj", "frontend", "matchers", "RampackMatcher.o"))
    return os.path.join(out, "casino_gpu_check")


def run(program, mode, adjust):
    args = [program, mode, str(N), str(SPACING), str(CYCLES), str(int(adjust)), str(TSTEP), str(BSTEP),
            str(PRESSURE), str(SEED)]
    return subprocess.run(args, capture_output=True, text=True, timeout=600)


def lattice():
    pos = np.array([[(i + 0.5) * SPACING, (j + 0.5) * SPACING, (k + 0.5) * SPACING]
                    for i in range(N) for j in range(N) for k in range(N)])
    rot = np.tile(np.eye(3).reshape(9), (len(pos), 1))
    box = np.diag([N * SPACING] * 3).reshape(9)
    return pos, rot, box


@pytest.mark.parametrize("adjust", [True, False])
def test_patched_simulation_without_backend_is_the_reference(check_program, adjust):
    if not po.reference_available():
        pytest.skip("reference library not built here")
    res = run(check_program, "cpu", adjust)
    assert res.returncode == 0, res.stderr
    lines = res.stdout.splitlines()
    values = np.array([float.fromhex(x) for x in lines if not x.startswith("#")])
    counters = {ln.split()[1]: (int(ln.split()[2]), int(ln.split()[3])) for ln in lines if ln.startswith("#")}
    box, pos = values[:9], values[9:].reshape(-1, 3)

    ref = po.CpuPacking("reference", po.SPHERE, np.array([0.5]), *lattice(), threads=1)
    st = po.run_cycles(ref, CYCLES, translation_step=TSTEP, box_kind=1, box_step=BSTEP, pressure=PRESSURE,
                       temperature=1.0, seed=SEED, adjust_steps=adjust)
    rp, _, rb = ref.state()
    ref.close()
    assert np.array_equal(box, np.asarray(rb).reshape(9))
    assert np.array_equal(pos, rp)
    assert counters["translation"] == (st.moves[0], st.accepted[0])
    assert counters["scaling"] == (st.scalings, st.scalings_accepted)
    assert 0 < st.scalings_accepted < st.scalings


def test_gpu_backend_fails_loudly_without_a_device(check_program):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    res = run(check_program, "gpu", True)
    assert res.returncode == 3, (res.returncode, res.stdout[-500:], res.stderr)
    assert "GPU backend: rp_create" in res.stderr and "device" in res.stderr, res.stderr
    assert res.stdout == ""
