"""Generates the golden fixtures in this directory from the REFERENCE'S OWN CODE.

Run in a checkout where the reference sources are present:

    make -C oracle ref            # compiles the reference's hot-path sources in place
    python tests/golden/make_golden.py        # every fixture
    python tests/golden/make_golden.py io     # the snapshot / trajectory files only
    python tests/golden/make_golden.py box    # the box-move proposal streams only
    python tests/golden/make_golden.py flips  # the FlipSampler moves only
    python tests/golden/make_golden.py walls  # the hard-wall packings only
    python tests/golden/make_golden.py correlation  # the pair-correlation observables only
    python tests/golden/make_golden.py nematic  # the nematic order of orientation sets only

Every expected value below is produced by the reference library (oracle/_ref/librpref.so:
rampack's Packing, NeighbourGrid, SpherocylinderTraits, samplers and Simulation compiled
from its sources with -ffp-contract=off).  Inputs are seeded synthetic configurations.
The fixtures pin the oracle restatement (tests/test_oracle_golden.py) and the GPU engine
(tests/test_gpu_golden.py) to the reference bit for bit.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pyoracle as po  # noqa: E402
from rampack_gb300 import workloads as W  # noqa: E402


def rand_rot(rng, n):
    """Random rotation matrices via the reference's Rodrigues formula (host libm)."""
    out = np.zeros((n, 9))
    for i in range(n):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        out[i] = po.rotation("reference", ax, rng.uniform(-np.pi, np.pi))
    return out


def gen_pairs(rng):
    """Pair overlap decisions near contact for spheres and spherocylinders."""
    recs = []
    shapes = [(po.SPHERE, [0.5]), (po.SPHEROCYLINDER, [2.0, 0.5]), (po.SPHEROCYLINDER, [5.0, 0.5]),
              (po.SPHEROCYLINDER, [0.0, 0.5]), (po.SPHEROCYLINDER, [3.0, 2.0])]
    for kind, prm in shapes:
        prm = np.array(prm)
        rng_len = 2 * prm[-1] + (prm[0] if kind == po.SPHEROCYLINDER else 0)
        for k in range(1500):
            r1 = rand_rot(rng, 1)[0]
            if k % 5 == 0:   # near-parallel partner
                r2 = po.rotation("reference", [1, 0, 0], rng.normal() * 1e-3).reshape(3, 3) @ r1.reshape(3, 3)
                r2 = r2.reshape(9)
            else:
                r2 = rand_rot(rng, 1)[0]
            p1 = rng.uniform(0, 10, size=3)
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            p2 = p1 + d * rng.uniform(0.0, 1.1) * rng_len
            t = rng.normal(size=3) * 3 if k % 3 == 0 else np.zeros(3)
            ov = po.pair_overlap("reference", kind, prm, p1, r1, p2 - t, r2, translation=t)
            recs.append((kind, prm[0], prm[-1], p1, r1, p2 - t, r2, t, ov))
    kinds = np.array([r[0] for r in recs], dtype=np.int32)
    prm = np.array([[r[1], r[2]] for r in recs])
    p1 = np.array([r[3] for r in recs])
    r1 = np.array([r[4] for r in recs])
    p2 = np.array([r[5] for r in recs])
    r2 = np.array([r[6] for r in recs])
    t = np.array([r[7] for r in recs])
    ov = np.array([r[8] for r in recs], dtype=np.int8)
    np.savez_compressed(os.path.join(HERE, "pairs.npz"), kind=kinds, params=prm, p1=p1, r1=r1, p2=p2, r2=r2,
                        translation=t, overlap=ov)
    print("pairs:", len(ov), "overlapping", int(ov.sum()))


def gen_geometry(rng):
    boxes = []
    for _ in range(40):
        b = np.diag(rng.uniform(5, 50, size=3)) + rng.uniform(-3, 3, size=(3, 3)) * (rng.uniform() < 0.7)
        boxes.append(b.reshape(9))
    boxes = np.array(boxes)
    inv, hts, vol = [], [], []
    for b in boxes:
        i, h, v = po.box_info("reference", b)
        inv.append(i)
        hts.append(h)
        vol.append(v)
    axes = rng.normal(size=(40, 3))
    angles = rng.uniform(-3, 3, size=40)
    rots = np.array([po.rotation("reference", a, ang) for a, ang in zip(axes, angles)])
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), boxes=boxes, inv=np.array(inv), heights=np.array(hts),
                        volume=np.array(vol), axes=axes, angles=angles, rotations=rots)
    print("geometry:", len(boxes), "boxes")


def grid_cells(pos, box, range_, shift):
    """Checkerboard cells of the GPU engine's grid rule (cells at least one range high and
    at most max(4096, 8 N) of them; an odd count above 3 drops one cell), restated in numpy
    to pick each cell's particles; particles within 1e-9 (relative) of a cell face are left
    out of the per-cell lists so the membership never hinges on rounding."""
    b = box.reshape(3, 3)
    s = [b[:, 0], b[:, 1], b[:, 2]]
    vol = abs(np.dot(np.cross(s[0], s[1]), s[2]))
    h = [vol / np.linalg.norm(np.cross(s[1], s[2])), vol / np.linalg.norm(np.cross(s[2], s[0])),
         vol / np.linalg.norm(np.cross(s[0], s[1]))]
    dims = []
    cell_min = max(range_, (vol / max(4096.0, 8.0 * len(pos))) ** (1 / 3)) * (1 + 1e-9)
    for d in range(3):
        n = max(1, int(np.floor(h[d] / cell_min)))
        dims.append(n - 1 if n > 3 and n % 2 else n)
    rel = pos @ np.linalg.inv(b).T
    u = (rel - np.array(shift)) % 1.0
    un = u * np.array(dims)
    c = np.minimum(un.astype(int), np.array(dims) - 1)
    frac = un - c
    safe = np.all((frac > 1e-9) & (frac < 1 - 1e-9), axis=1)
    cell = c[:, 0] + dims[0] * (c[:, 1] + dims[1] * c[:, 2])
    bounds = np.zeros((dims[0] * dims[1] * dims[2], 6))
    for idx in range(len(bounds)):
        cc = (idx % dims[0], (idx // dims[0]) % dims[1], idx // (dims[0] * dims[1]))
        for d in range(3):
            if dims[d] == 1:
                lo, hi = -np.inf, np.inf
            else:
                lo = shift[d] + cc[d] / dims[d]
                lo = lo - 1 if lo >= 1 else lo
                hi = shift[d] + (cc[d] + 1) / dims[d]
                hi = hi - 1 if hi >= 1 else hi
            bounds[idx, d], bounds[idx, 3 + d] = lo, hi
    return dims, cell, safe, bounds


def gen_system(name, cfg, trans, rot, rng, nshift=2, seed=77):
    """Snapshot, overlap counts, a replayed move stream and box moves, all from the reference."""
    import systems
    kind, prm, pos, rotm, box = cfg
    out = {"kind": kind, "params": prm, "pos": pos, "rot": rotm, "box": box}
    ref = po.CpuPacking("reference", kind, prm, pos, rotm, box)
    out["count"] = ref.count_overlaps(False)
    out["count_early"] = ref.count_overlaps(True)
    comp = systems.compressed(cfg, 0.96)
    rc = po.CpuPacking("reference", *comp)
    out["comp_pos"], out["comp_box"] = comp[2], comp[4]
    out["comp_count"] = rc.count_overlaps(False)
    out["comp_count_early"] = rc.count_overlaps(True)
    rc.close()
    # move stream: per phase, per active cell, moves drawn by the reference's samplers
    rng_h = ref.rng(seed)
    range_ = 2 * prm[-1] + (prm[0] if kind == po.SPHEROCYLINDER else 0)
    all_moves, all_bounds, off = [], [], 0
    for sh in range(nshift):
        shift = rng.uniform(0, 1, size=3) if sh else np.zeros(3)
        cur_pos, _, cur_box = ref.state()
        dims, cell, safe, bounds = grid_cells(cur_pos, cur_box, range_, shift)
        chunk = []
        from rampack_gb300.packing import cell_phase
        phase = [cell_phase(dims, ci) for ci in range(len(bounds))]
        for ph in sorted(set(phase)):
            for ci in range(len(bounds)):
                if phase[ci] != ph:
                    continue
                idx = np.nonzero((cell == ci) & safe)[0]
                if len(idx) == 0:
                    continue
                nt = (trans > 0) + (rot > 0)
                mv = ref.draw_moves(rng_h, trans, rot, idx, len(idx), nt * len(idx), domain=off + ci)
                chunk.append(mv)
        mv = np.concatenate(chunk)
        codes, _ = ref.replay(mv, np.concatenate(all_bounds + [bounds]) if all_bounds else bounds)
        all_moves.append((mv, codes, shift))
        all_bounds.append(bounds)
        off += len(bounds)
    ref.rng_free(rng_h)
    out["moves"] = np.concatenate([m[0] for m in all_moves])
    out["codes"] = np.concatenate([m[1] for m in all_moves])
    out["shifts"] = np.array([m[2] for m in all_moves])
    out["bounds"] = np.concatenate(all_bounds)
    out["chunk_moves"] = np.array([len(m[0]) for m in all_moves])
    out["chunk_cells"] = np.array([len(b) for b in all_bounds])
    out["move_pos"], out["move_rot"], out["move_box"] = ref.state()
    # box moves from the post-move state
    boxes, dEs = [], []
    for k in range(10):
        _, _, b = ref.state()
        bb = b.reshape(3, 3)
        nb = (bb * (1 + rng.uniform(-0.03, 0.01)) if k % 2 else bb + rng.uniform(-0.04, 0.04, size=(3, 3)))
        nb = nb.reshape(9)
        dE = ref.try_scaling(nb)
        if dE > 0:
            ref.revert_scaling()
        boxes.append(nb)
        dEs.append(dE)
    out["scale_boxes"] = np.array(boxes)
    out["scale_dE"] = np.array(dEs)
    out["final_pos"], out["final_rot"], out["final_box"] = ref.state()
    ref.close()
    np.savez_compressed(os.path.join(HERE, f"system_{name}.npz"), **out)
    acc = int(np.count_nonzero(out["codes"] & 0x80))
    print(f"system {name}: N={len(pos)} count={out['count']} comp={out['comp_count']} moves={len(out['moves'])} "
          f"accepted={acc} box dE={list(out['scale_dE'])}")


def gen_sim(name, cfg, cycles, **kw):
    """A short NpT run of the reference's Simulation::integrate from a lattice."""
    kind, prm, pos, rotm, box = cfg
    ref = po.CpuPacking("reference", kind, prm, pos, rotm, box, threads=kw.get("threads", 1))
    st = po.run_cycles(ref, cycles, **kw)
    p, r, b = ref.state()
    np.savez_compressed(os.path.join(HERE, f"sim_{name}.npz"), kind=kind, params=prm, pos=pos, rot=rotm, box=box,
                        final_pos=p, final_rot=r, final_box=b, cycles=cycles,
                        moves=np.array(list(st.moves)), accepted=np.array(list(st.accepted)),
                        params_json=repr(kw))
    print(f"sim {name}: moves {list(st.moves)} accepted {list(st.accepted)}")


def gen_proposals():
    """Proposal streams drawn by the reference's TranslationSampler / RotationSampler."""
    kind, prm, pos, rotm, box = W.spherocylinders((6, 6, 6), 0.3, 2.0, 0.5, aspect=(1, 1, 3))
    ref = po.CpuPacking("reference", kind, prm, pos, rotm, box)
    r = ref.rng(4242)
    idx = np.arange(0, len(pos), 3)
    mv = ref.draw_moves(r, 0.2, 0.3, idx, 50, 500, domain=5)
    ref.rng_free(r)
    np.savez_compressed(os.path.join(HERE, "proposals.npz"), moves=mv, idx=idx, box=box, seed=4242,
                        trans=0.2, rot=0.3, per_type=50)
    print("proposals:", len(mv))


# RAMSNAP inputs whose parse (or error) the reference fixes: old and new box formats,
# number forms, aux entries, and broken files
IO_CASES = {
    "old_box": b"1\nk v\n10 11 12\n2\n1 2 3        1 0 0 0 1 0 0 0 1\n4 5 6 1 0 0 0 1 0 0 0 1\n",
    "old_box_trailing": b"1\nk v\n10 11 12   \n1\n1 2 3 1 0 0 0 1 0 0 0 1\n",
    "number_forms": b"1\nk v\n1e1 0 0 0 +10 0 0 0 10.\n1\n.5 +2.5e-1 3E0 1 0 0 0 1 0 0 0 1\n",
    "aux_values": b"3\nb  two words \na x\nc\n\ny\n10 0 0 0 10 0 0 0 10\n1\n1 2 3 1 0 0 0 1 0 0 0 1\n",
    "no_aux": b"0\n10 0 0 0 10 0 0 0 10\n1\n1 2 3        1 0 0 0 1 0 0 0 1\n",
    "singular_box": b"1\nk v\n10 0 0 0 0 0 0 0 10\n1\n1 2 3 1 0 0 0 1 0 0 0 1\n",
    "truncated": b"1\nk v\n10 0 0 0 10 0 0 0 10\n3\n1 2 3 1 0 0 0 1 0 0 0 1\n4 5 6 1 0 0\n",
    "bad_dimensions": b"1\nk v\n10 x 0 0 10 0 0 0 10\n1\n1 2 3 1 0 0 0 1 0 0 0 1\n",
    "eight_dimensions": b"1\nk v\n10 0 0 0 10 0 0 0\n1\n1 2 3 1 0 0 0 1 0 0 0 1\n",
    "bad_size": b"1\nk v\n10 0 0 0 10 0 0 0 10\nx\n",
    "bad_aux": b"2\nk v\n",
    "empty": b"",
    "infinity": b"1\nk v\n10 0 0 0 10 0 0 0 10\n1\ninf 2 3 1 0 0 0 1 0 0 0 1\n",
    "overflow": b"1\nk v\n10 0 0 0 10 0 0 0 10\n1\n1e999 2 3 1 0 0 0 1 0 0 0 1\n",
}


def gen_io(rng):
    """RAMSNAP and RAMTRJ files written by the reference's own writers, the reference's
    reading of them, and its outcome (values or exception text) on edge-case inputs."""
    import tempfile
    import systems
    kind, prm, pos, rot, box = systems.sc_l2()
    sel = np.arange(0, len(pos), 25)  # 40 particles, enough to cover every number form
    pos, rot = pos[sel], rot[sel]
    box = box.copy()
    box[1], box[2], box[5] = 0.125, -0.0625, 1e-17  # triclinic, one tiny entry
    pos[0] = [1.0, 1.0, 1.0]
    rot[0] = [1.0, 5e-324, 0.0, 1e-300, 1.0, 0.0, 0.0, 0.0, 1.0]  # denormals
    pos[1] = [2.0, 1.0 / 3.0 + 1.0, 2.0 / 3.0 + 1.0]
    rot[1] = [1.0, 0.0, -0.0, -0.0, 1.0, 0.0, 0.0, -0.0, 1.0]     # negative zeros
    aux = {"cycles": "12000", "comment": "a value  with spaces", "a.key": "x", "zz": "trailing "}
    d = tempfile.mkdtemp()
    snap = os.path.join(HERE, "io_sc.ramsnap")
    po.ref_ramsnap_write(snap, kind, prm, pos, rot, box, aux)
    states = []
    for k in range(3):
        p = pos + rng.normal(scale=0.05, size=pos.shape)
        r = rand_rot(rng, len(pos))
        b = box * (1 + 0.01 * k)
        states.append((p, r, b))
    trj = os.path.join(HERE, "io_sc.ramtrj")
    po.ref_ramtrj_write(trj, kind, prm, states, 50)
    out = {"kind": kind, "params": prm, "pos": pos, "rot": rot, "box": box,
           "aux_keys": np.array(list(aux.keys())), "aux_values": np.array(list(aux.values())),
           "trj_pos": np.stack([s[0] for s in states]), "trj_rot": np.stack([s[1] for s in states]),
           "trj_box": np.stack([s[2] for s in states]), "trj_cycle_step": 50}
    # the reference's reading of its own files
    rp, rr, rb, ra = po.ref_ramsnap_read(snap, kind, prm)
    out.update(read_pos=rp, read_rot=rr, read_box=rb)
    for k in range(3):
        p, r, b = po.ref_ramtrj_read(trj, kind, prm, k, len(pos))
        out.update({f"play{k}_pos": p, f"play{k}_rot": r, f"play{k}_box": b})
    # edge cases
    for name, data in IO_CASES.items():
        f = os.path.join(d, name)
        with open(f, "wb") as fh:
            fh.write(data)
        out[f"case_{name}_input"] = np.frombuffer(data, dtype=np.uint8)
        try:
            p, r, b, a = po.ref_ramsnap_read(f, po.SPHERE, [0.5])
            out[f"case_{name}_pos"], out[f"case_{name}_rot"], out[f"case_{name}_box"] = p, r, b
            out[f"case_{name}_aux"] = np.array([f"{k}\t{v}" for k, v in sorted(a.items())])
            out[f"case_{name}_error"] = np.array("")
        except ValueError as e:
            out[f"case_{name}_error"] = np.array(str(e))
    np.savez_compressed(os.path.join(HERE, "io.npz"), **out)
    print("io: ramsnap", os.path.getsize(snap), "B, ramtrj", os.path.getsize(trj), "B,", len(IO_CASES), "cases")


# box scalers: (kind, scale together, axis groups, independent, step); kinds as rp_box_scaler_desc
SCALERS = [(1, 1, [], 0, 0.005), (1, 0, [], 0, 0.05), (2, 0, [7], 0, 0.01), (2, 0, [1, 2, 4], 1, 0.01),
           (2, 0, [3, 4], 0, 0.02), (2, 0, [3, 4], 1, 0.02), (3, 0, [7], 0, 0.1), (3, 0, [1, 2, 4], 1, 0.1),
           (4, 0, [], 0, 5.0)]


def gen_box_proposals():
    """Box-move proposals and Metropolis draws of the reference's scalers and generator."""
    box = np.array([10.0, 0.3, -0.2, 0.1, 11.0, 0.05, -0.0, -0.4, 12.5])
    out = {"box": box}
    for i, (kind, tog, groups, ind, step) in enumerate(SCALERS):
        b, u = po.ref_box_proposals(kind, tog, groups, ind, step, 1234 + i, box, 40)
        out[f"s{i}_spec"] = np.array([kind, tog, ind] + (groups + [0, 0, 0])[:3] + [len(groups)])
        out[f"s{i}_step"] = np.array(step)
        out[f"s{i}_boxes"], out[f"s{i}_uniforms"] = b, u
    np.savez_compressed(os.path.join(HERE, "box_proposals.npz"), **out)
    print("box proposals:", len(SCALERS), "scalers")


def gen_flips():
    """FlipSampler moves of the reference's own sampler (spherocylinders: flips about the
    body y axis, the primary axis z crossed with x)."""
    import systems
    cfg = systems.sc_l2()
    ref = po.CpuPacking("reference", *cfg)
    idx = np.arange(0, len(cfg[2]), 3)
    r = ref.rng(2468)
    mv = ref.draw_flips(r, idx, 300)
    ref.rng_free(r)
    np.savez_compressed(os.path.join(HERE, "flips.npz"), moves=mv, idx=idx, rot=cfg[3], seed=2468)
    print("flips:", len(mv))


def state_digest(pos, rot) -> np.ndarray:
    import hashlib
    h = hashlib.sha256(np.ascontiguousarray(pos, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(rot, dtype=np.float64).tobytes())
    return np.frombuffer(h.digest(), dtype=np.uint8)


# hard walls: (system, wall mask, translation step, rotation step)
WALLS = [("hs_small", 1, 0.1, 0.0), ("sc_l2", 5, 0.2, 0.2), ("poly_banana", 2, 0.2, 0.2), ("sc_l2_dense", 7, 0.2, 0.2),
         ("psc_bent", 3, 0.15, 0.15)]


def gen_walls():
    """Packings with hard walls (Packing::toggleWalls) through the reference: overlap counts,
    a replayed move list (no ActiveDomain), a box move, and the same moves in counting mode."""
    import systems
    out = {}
    for i, (name, mask, t, r) in enumerate(WALLS):
        cfg = systems.ALL[name]()
        kind, prm, pos, rot, box = cfg
        ref = po.CpuPacking("reference", *cfg)
        ref.set_walls(mask)
        out[f"w{i}_counts"] = np.array([ref.count_overlaps(False), ref.count_overlaps(True)])
        rng = ref.rng(500 + i)
        n = len(pos)
        mv = ref.draw_moves(rng, t, r, np.arange(n), n, 800)
        ref.rng_free(rng)
        codes, _ = ref.replay(mv)
        p1, r1, b1 = ref.state()
        nb = (b1.reshape(3, 3) * 0.995).reshape(9)
        out[f"w{i}_moves"], out[f"w{i}_codes"] = mv, codes
        # final states as SHA-256 digests of their bytes (the arrays would be megabytes)
        out[f"w{i}_state"] = state_digest(p1, r1)
        out[f"w{i}_box_dE"] = np.array(ref.try_scaling(nb))
        out[f"w{i}_box_state"] = state_digest(*ref.state()[:2])
        cnt = po.CpuPacking("reference", *cfg)
        cnt.set_walls(mask)
        cnt.set_counting(True)
        c2, d2 = cnt.replay(mv)
        out[f"w{i}_count_codes"], out[f"w{i}_count_deltas"] = c2, d2
        out[f"w{i}_count_final"] = np.array(cnt.cached_overlaps())
    np.savez_compressed(os.path.join(HERE, "walls.npz"), **out)
    print("walls:", len(WALLS), "systems")


def gen_correlation():
    """PairDensityCorrelation / PairAveragedCorrelation of the reference over two snapshots
    of each system (as thermalised, and compressed by 3%), printed at full precision, and the
    reference's named points of the shapes."""
    import systems
    from correlation_cases import CORRELATIONS, NAMED_POINTS, POLY_AXES
    out = {}
    for i, (name, en, lax, mil, fn, ax, focal, max_r, nb) in enumerate(CORRELATIONS):
        cfg = systems.ALL[name]()
        kind, prm = cfg[0], cfg[1]
        states = [cfg[2:5], systems.compressed(cfg, 0.97)[2:5]]
        d = po.pair_desc(enumerator=en, linear_axis=lax, miller=mil, function=fn, axis=ax, num_bins=nb,
                         max_r=max_r)
        prim, sec = POLY_AXES if kind == po.POLYSPHERE else (None, None)
        x, y, c = po.ref_pair_correlation(kind, prm, states, d, focal, primary=prim, secondary=sec)
        out[f"c{i}_x"], out[f"c{i}_y"], out[f"c{i}_count"] = x, y, c
    for i, (name, point) in enumerate(NAMED_POINTS):
        cfg = systems.ALL[name]()
        out[f"p{i}"] = po.ref_named_point(cfg[0], cfg[1], point)
    np.savez_compressed(os.path.join(HERE, "correlation.npz"), **out)
    print("correlation:", len(CORRELATIONS), "observables")


def nematic_orientations(rng):
    """Orientation sets of spherocylinders for the nematic-order fixture: aligned, isotropic,
    near-aligned along z, nematic along a tilted director, and a thermalised packing."""
    import systems
    sets = {}
    sets["aligned"] = np.tile(np.eye(3).reshape(9), (100, 1))
    sets["isotropic"] = rand_rot(rng, 1000).reshape(-1, 9)
    small = []
    for _ in range(500):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        small.append(po.rotation("reference", ax, float(rng.uniform(-0.3, 0.3))))
    sets["near_z"] = np.array(small)
    t3 = np.asarray(po.rotation("reference", np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0), 0.9)).reshape(3, 3)
    sets["tilted"] = np.array([(t3 @ m.reshape(3, 3)).reshape(9) for m in small[:300]])
    sets["sc_l2"] = np.asarray(systems.sc_l2()[3], dtype=np.float64).reshape(-1, 9)
    return sets


def gen_nematic(rng):
    """NematicOrder of the reference (core/observables/NematicOrder.cpp:9-28) on the sets above."""
    out = {}
    for name, rot in nematic_orientations(rng).items():
        n = len(rot)
        pos = np.zeros((n, 3))
        box = np.eye(3).reshape(9) * 50.0
        pk = po.CpuPacking("reference", po.SPHEROCYLINDER, np.array([2.0, 0.5]), pos, rot, box)
        q, p2 = pk.nematic_order()
        pk.close()
        out[f"{name}_rot"] = rot
        out[f"{name}_q"] = q
        out[f"{name}_p2"] = np.array([p2])
    np.savez_compressed(os.path.join(HERE, "nematic.npz"), names=np.array(sorted(k[:-4] for k in out if k.endswith("_rot"))),
                        **out)
    print("nematic:", len(out) // 3, "orientation sets")


def gen_convex():
    """XenoCollideTraits::overlapBetween of the reference's GenericXenoCollideTraits on random
    pairs around contact for every test body (tests/convex_bodies.py), 400 pairs each."""
    import convex_bodies as CB
    out = {}
    for i, (name, script) in enumerate(sorted(CB.BODIES.items())):
        p1, r1, p2, r2 = CB.random_pairs(np.random.default_rng(3000 + i), 400)
        dec = np.array([po.convex_overlap("reference", script, p1[k], r1[k], p2[k], r2[k]) for k in range(len(p1))])
        out[f"{name}_r1"], out[f"{name}_p2"], out[f"{name}_r2"], out[f"{name}_overlap"] = r1, p2, r2, dec
    np.savez_compressed(os.path.join(HERE, "convex.npz"), names=np.array(sorted(CB.BODIES)), **out)
    print("convex:", len(CB.BODIES), "bodies")


def main():
    if not po.reference_available():
        po.build(reference=True)
    if sys.argv[1:] == ["walls"]:
        gen_walls()
        return
    if sys.argv[1:] == ["correlation"]:
        gen_correlation()
        return
    if sys.argv[1:] == ["flips"]:
        gen_flips()
        return
    if sys.argv[1:] == ["io"]:
        gen_io(np.random.default_rng(20261204))
        return
    if sys.argv[1:] == ["box"]:
        gen_box_proposals()
        return
    if sys.argv[1:] == ["nematic"]:
        gen_nematic(np.random.default_rng(20261205))
        return
    if sys.argv[1:] == ["convex"]:
        gen_convex()
        return
    rng = np.random.default_rng(20241203)
    gen_pairs(rng)
    gen_geometry(rng)
    gen_proposals()
    import systems
    gen_system("hs", systems.hs_small(), 0.1, 0.0, rng)
    gen_system("sc_l2", systems.sc_l2(), 0.2, 0.2, rng)
    gen_system("sc_l5", systems.sc_l5(), 0.2, 0.2, rng, nshift=1)
    gen_sim("hs1000", W.config_hs_1000(), 60, translation_step=0.1, box_kind=2, box_step=0.01 / 3, pressure=10.0,
            adjust_steps=True)
    gen_sim("sc_dd", W.spherocylinders((12, 12, 12), 0.35, 2.0, 0.5, aspect=(1, 1, 3)), 8, translation_step=0.2,
            rotation_step=0.2, box_kind=1, box_step=0.005, pressure=1.5, domains=(2, 2, 2), threads=8)
    gen_io(np.random.default_rng(20261204))
    gen_box_proposals()
    gen_flips()
    gen_walls()
    gen_correlation()
    gen_nematic(np.random.default_rng(20261205))
    gen_convex()


if __name__ == "__main__":
    main()
