"""The oracle's cycle loop against the reference's own Simulation::integrate, compiled here
from the reference's sources (oracle/Makefile `ref`): identical seeds must give identical
acceptance counts and bit-identical final states.  Skipped where the reference library is
not built (the GPU machine); there the committed golden fixtures carry the same pin."""
import numpy as np
import pytest

import pyoracle as po
from rampack_gb300 import workloads as W

BANANA = dict(arc_radius=0.6 / (2 * np.sin(np.radians(15))), arc_angle=np.radians(120), n_spheres=5)

RUNS = {
    "hs_log_volume": (lambda: W.hard_spheres(6, 0.30), 30,
                      dict(translation_step=0.1, box_kind=2, box_step=0.01 / 3, pressure=10.0)),
    "sc_delta_triclinic": (lambda: W.spherocylinders((6, 6, 6), 0.35, 2.0, 0.5, aspect=(1, 1, 3)), 20,
                           dict(translation_step=0.2, rotation_step=0.2, box_kind=1, box_step=0.005, pressure=1.5)),
    "sc_delta_volume": (lambda: W.spherocylinders((6, 6, 3), 0.2, 3.0, 0.5, aspect=(1, 1, 3)), 30,
                        dict(translation_step=0.5, rotation_step=1.0, box_kind=3, box_step=3.0, pressure=0.5)),
    "banana_triclinic": (lambda: W.bananas((6, 8, 4), 0.35, **BANANA), 10,
                         dict(translation_step=0.2, rotation_step=0.2, box_kind=1, box_step=0.005, pressure=1.5)),
    "sc_domains_8_threads": (lambda: W.spherocylinders((8, 8, 8), 0.35, 2.0, 0.5, aspect=(1, 1, 3)), 10,
                             dict(translation_step=0.2, rotation_step=0.2, box_kind=1, box_step=0.005, pressure=1.5,
                                  domains=(2, 2, 2), threads=8)),
    "bent_rods_triclinic": (lambda: W.bent_rods((5, 7, 7)), 12,
                            dict(translation_step=0.15, rotation_step=0.15, box_kind=1, box_step=0.005,
                                 pressure=2.0)),
    "bent_rods_dense_nvt": (lambda: W.bent_rods((4, 6, 6), spacing=(1.9, 0.6, 0.92)), 6,
                                   dict(translation_step=0.2, rotation_step=0.3)),
    "sc_step_adaptation": (lambda: W.spherocylinders((6, 6, 6), 0.35, 2.0, 0.5, aspect=(1, 1, 3)), 200,
                           dict(translation_step=0.05, rotation_step=0.05, box_kind=1, box_step=0.05,
                                pressure=1.5, adjust_steps=True)),
}


@pytest.mark.parametrize("name", sorted(RUNS))
def test_cycle_loop_matches_reference(oracle, name):
    if not po.reference_available():
        pytest.skip("reference library not built here")
    build, cycles, kw = RUNS[name]
    kind, prm, pos, rot, box = build()
    threads = kw.get("threads", 1)
    out = {}
    for which in ("oracle", "reference"):
        pk = po.CpuPacking(which, kind, prm, pos, rot, box, threads=threads)
        st = po.run_cycles(pk, cycles, seed=4321, **kw)
        out[which] = (list(st.moves), list(st.accepted), st.scalings, st.scalings_accepted, list(st.steps),
                      st.box_step, pk.state())
        pk.close()
    a, b = out["oracle"], out["reference"]
    assert a[:6] == b[:6]
    for x, y in zip(a[6], b[6]):
        assert np.array_equal(x, y)
