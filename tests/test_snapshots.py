"""Snapshot (RAMSNAP) and trajectory (RAMTRJ) formats on the host: the oracle restatement and
the engine's writers and readers against files written and read by the reference itself
(tests/golden/io_sc.ramsnap, io_sc.ramtrj, io.npz — tests/golden/make_golden.py io)."""
import os

import numpy as np
import pytest

import snapshots as S
from rampack_gb300 import snapshots as RS
from rampack_gb300._lib import EngineError

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SNAP = os.path.join(GOLD, "io_sc.ramsnap")
TRJ = os.path.join(GOLD, "io_sc.ramtrj")


@pytest.fixture(scope="module")
def io(engine):
    return np.load(os.path.join(GOLD, "io.npz"))


def aux_of(io):
    return dict(zip([str(k) for k in io["aux_keys"]], [str(v) for v in io["aux_values"]]))


def states_of(io):
    return [(io["trj_pos"][k], io["trj_rot"][k], io["trj_box"][k]) for k in range(len(io["trj_pos"]))]


def read(path):
    with open(path, "rb") as f:
        return f.read()


# ---- the oracle, pinned to the reference's files ----

def test_oracle_ramsnap_bytes(io):
    assert S.ramsnap_bytes(io["pos"], io["rot"], io["box"], aux_of(io)) == read(SNAP)


def test_oracle_ramtrj_bytes(io):
    assert S.ramtrj_bytes(states_of(io), int(io["trj_cycle_step"])) == read(TRJ)


def test_oracle_readers(io):
    pos, rot, box, aux = S.parse_ramsnap(read(SNAP))
    assert np.array_equal(pos, io["read_pos"]) and np.array_equal(rot, io["read_rot"])
    assert np.array_equal(box, io["read_box"]) and aux == aux_of(io)
    head, snaps = S.parse_ramtrj(read(TRJ))
    assert head == {"num_particles": 40, "snapshots": 3, "cycle_step": 50, "version": (1, 1)}
    for k, (p, r, b) in enumerate(snaps):
        assert np.array_equal(p, io[f"play{k}_pos"]) and np.array_equal(r, io[f"play{k}_rot"])
        assert np.array_equal(b, io[f"play{k}_box"])


# ---- the engine's host entry points (no GPU involved) ----

def test_engine_ramsnap_writer(io, tmp_path):
    f = tmp_path / "a.ramsnap"
    RS.write_ramsnap(f, io["pos"], io["rot"], io["box"], aux_of(io))
    assert read(f) == read(SNAP)


def test_engine_ramsnap_writer_refuses_keys_with_whitespace(io, tmp_path):
    with pytest.raises(EngineError, match="whitespace"):
        RS.write_ramsnap(tmp_path / "a.ramsnap", io["pos"], io["rot"], io["box"], {"two words": "x"})


def test_engine_ramsnap_reader(io):
    pos, rot, box, aux = RS.read_ramsnap(SNAP)
    assert np.array_equal(pos, io["read_pos"]) and np.array_equal(rot, io["read_rot"])
    assert np.array_equal(box, io["read_box"]) and aux == aux_of(io)
    # written numbers read back bit for bit, signs of zeros included
    assert np.array_equal(pos.view(np.uint64), io["pos"].view(np.uint64))
    assert np.array_equal(rot.view(np.uint64), io["rot"].view(np.uint64))


CASES = ["old_box", "old_box_trailing", "number_forms", "aux_values", "no_aux", "singular_box", "truncated",
         "bad_dimensions", "eight_dimensions", "bad_size", "bad_aux", "empty", "infinity", "overflow"]


@pytest.mark.parametrize("name", CASES)
def test_engine_ramsnap_reader_cases(io, tmp_path, name):
    # the reference's outcome on each input: its values, or its exception text
    f = tmp_path / name
    f.write_bytes(io[f"case_{name}_input"].tobytes())
    err = str(io[f"case_{name}_error"])
    if err:
        with pytest.raises(EngineError) as e:
            RS.read_ramsnap(f)
        assert str(e.value).split(": ", 1)[1] == err
    else:
        pos, rot, box, aux = RS.read_ramsnap(f)
        assert np.array_equal(pos, io[f"case_{name}_pos"]) and np.array_equal(rot, io[f"case_{name}_rot"])
        assert np.array_equal(box, io[f"case_{name}_box"])
        assert sorted(f"{k}\t{v}" for k, v in aux.items()) == [str(x) for x in io[f"case_{name}_aux"]]


def test_engine_ramtrj_recorder(io, tmp_path):
    f = tmp_path / "t.ramtrj"
    with RS.RamtrjRecorder(f, 40, 50) as rec:
        for k, st in enumerate(states_of(io)):
            rec.record_host(*st, cycle=50 * (k + 1))
        assert rec.snapshots() == 3
    assert read(f) == read(TRJ)


def test_engine_ramtrj_append(io, tmp_path):
    f = tmp_path / "t.ramtrj"
    st = states_of(io)
    with RS.RamtrjRecorder(f, 40, 50) as rec:
        rec.record_host(*st[0], cycle=50)
    with RS.RamtrjRecorder(f, 40, 50, append=True) as rec:
        assert rec.snapshots() == 1
        rec.record_host(*st[1], cycle=100)
        rec.record_host(*st[2], cycle=150)
    assert read(f) == read(TRJ)
    with pytest.raises(EngineError, match="unmatching"):
        RS.RamtrjRecorder(f, 40, 25, append=True)
    # a truncated trajectory cannot be continued
    g = tmp_path / "cut.ramtrj"
    g.write_bytes(read(TRJ)[:-8])
    with pytest.raises(EngineError, match="broken snapshot structure"):
        RS.RamtrjRecorder(g, 40, 50, append=True)


def test_engine_ramtrj_preconditions(io, tmp_path):
    st = states_of(io)
    with RS.RamtrjRecorder(tmp_path / "t.ramtrj", 40, 50) as rec:
        with pytest.raises(EngineError, match="cycle"):
            rec.record_host(*st[0], cycle=100)       # must be 50
        bad = st[0][1].copy()
        bad[7] *= 1.001                               # not a rotation: EulerAngles refuses it
        with pytest.raises(EngineError, match="not a rotation"):
            rec.record_host(st[0][0], bad, st[0][2], cycle=50)
        rec.record_host(*st[0], cycle=50)
        assert rec.snapshots() == 1


def test_engine_ramtrj_reader(io, tmp_path):
    assert RS.ramtrj_info(TRJ) == {"num_particles": 40, "snapshots": 3, "cycle_step": 50, "version": (1, 1)}
    for k in range(3):
        p, r, b = RS.read_ramtrj(TRJ, k)
        assert np.array_equal(p, io[f"play{k}_pos"]) and np.array_equal(r, io[f"play{k}_rot"])
        assert np.array_equal(b, io[f"play{k}_box"])
    with pytest.raises(EngineError, match="out of range"):
        RS.read_ramtrj(TRJ, 3)
    g = tmp_path / "cut.ramtrj"
    g.write_bytes(read(TRJ)[:-1])
    with pytest.raises(EngineError, match="broken snapshot structure"):
        RS.ramtrj_info(g)
    h = tmp_path / "magic.ramtrj"
    h.write_bytes(b"RAMTRX\n" + read(TRJ)[7:])
    with pytest.raises(EngineError, match="magic"):
        RS.ramtrj_info(h)
