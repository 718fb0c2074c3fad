#!/usr/bin/env python3
"""Benchmark of the hard-particle Monte Carlo move-and-overlap path.

Workload (one "step" = one Monte Carlo cycle): hard spherocylinders l=2, r=0.5 (L/D=2),
N = 100^3 = 1,000,000 started aligned on an orthorhombic lattice (cell aspect 1:1:3) at
packing fraction 0.50 in a box that the isotension moves make triclinic; each cycle is
2N particle moves (translation step 0.2 and rotation step 0.2, half each, in
checkerboard domains) plus one box move, alternately an isotension move (every box-matrix
entry perturbed by up to 0.005) and an isotropic volume move (ln V uniform in +-1e-6), at
p* = 1.5, T = 1, whose overlap check rescales, rebuilds the cell grid and recounts all
overlaps.  The default line also compares the learned test ordering with the plain scan
on the same state ("ordering").  Synthetic seeded input; no dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W]           GPU engine (this repo)
  python bench.py --impl reference [--steps K] [--warmup W]     CPU implementation of the path
  python bench.py --ordering [--steps K]                        learned test ordering vs plain scan

Metric: attempted particle moves per second (higher is better).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "moves/sec at N=1e6"
UNIT = "moves/s"
TRANS_STEP, ROT_STEP, BOX_STEP, PRESSURE, TEMPERATURE = 0.2, 0.2, 0.005, 1.5, 1.0
# isotropic volume move of the headline: ln V uniform in +-VOL_STEP (LogScalingFactorSampler on
# X & Y & Z, VOL_STEP / 3 per side), the acceptance window at N = 1e6 and p* = 1.5
VOL_STEP = 1e-6
WORKLOAD = ("hard spherocylinders l=2 r=0.5 (L/D=2), N={n:,}, aligned orthorhombic start at phi=0.50 "
            "(cell aspect 1:1:3), triclinic box; per cycle 2N moves (translation 0.2, rotation 0.2) "
            "+ 1 box move, alternating an isotension move (TriclinicDeltaScaler, delta 0.005) and an "
            "isotropic volume move (log scaling of X & Y & Z, ln V uniform in +-1e-6); p*=1.5, T=1")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--n-side", type=int, default=100, help="particles per lattice side (default 100 -> 1e6)")
    ap.add_argument("--workload", default="sc-1e6", choices=sorted(WORKLOADS),
                    help="sc-1e6: the headline system; the others are further systems of the same path")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--bulk-staging", type=int, default=-1, choices=[-1, 0, 1],
                    help="stage neighbourhoods with bulk asynchronous copies (1) or per-lane loads (0); "
                         "-1: the engine's default")
    ap.add_argument("--cell-order", type=int, default=-1, choices=[-1, 0, 1],
                    help="sweep each phase's cells largest first (1) or in index order (0); -1: the engine's default")
    ap.add_argument("--cells-per-warp", type=int, default=0, choices=[0, 1, 2],
                    help="plain sweeps: 1 = a warp per cell, 2 = a cell per half-warp (0: the library default)")
    ap.add_argument("--no-ordering", action="store_true",
                    help="skip the learned-ordering comparison of the headline line")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--tuning", default=None,
                    help="replicas-64: fixed launch shape 'cell_factor,warps_per_block' instead of autotuning")
    ap.add_argument("--ordering", action="store_true",
                    help="compare the plain scan with centre-distance and learned partner ordering")
    ap.add_argument("--correlation", action="store_true",
                    help="time the pair density correlation g(r) of the workload's packing")
    ap.add_argument("--corr-max-r", type=float, default=8.0)
    ap.add_argument("--corr-bins", type=int, default=200)
    ap.add_argument("--corr-enumerator", default="radial", choices=["radial", "linear-z", "layerwise-z10"],
                    help="RadialEnumerator, LinearEnumerator(z) or LayerwiseRadialEnumerator((0, 0, 10))")
    ap.add_argument("--io", action="store_true",
                    help="snapshot files of the workload: RAMSNAP store / restore time and the cost of recording "
                         "a RAMTRJ snapshot every cycle while sweeping")
    return ap.parse_args()


def _sc_1e6(args):
    from rampack_gb300 import workloads as W
    n_side = args.n_side
    return W.spherocylinders((n_side, n_side, n_side), 0.50, 2.0, 0.5, aspect=(1.0, 1.0, 3.0))


def _banana_1e5(args):
    from rampack_gb300 import workloads as W
    return W.config_banana_1e5()


def _bent_rods_1e5(args):
    from rampack_gb300 import workloads as W
    return W.config_bent_rods_1e5()


def _sc_64000(args):
    from rampack_gb300 import workloads as W
    return W.config_sc_64000()


def _soft_wca(args):
    from rampack_gb300 import workloads as W
    return W.hard_spheres(46, 0.40)


def _convex_262144(args):
    from rampack_gb300 import workloads as W
    return W.config_convex(64)


# name -> (builder, description, metric)
WORKLOADS = {
    "sc-1e6": (_sc_1e6, WORKLOAD, METRIC),
    "banana-1e5": (_banana_1e5, "bent 5-sphere chains (sphere r=0.5, bond 0.6, 30 degrees between bonds: arc "
                   "120 degrees), N={n:,} (50x80x25), aligned orthorhombic start at phi=0.45, triclinic box; per "
                   "cycle 2N moves (translation 0.2, rotation 0.2) + 1 isotension box move (delta 0.005, p*=1.5, "
                   "T=1)", "moves/sec, bent chains N=1e5"),
    "replicas-64": (None, "64 replicas: 32 hard-sphere (r=0.5) and 32 spherocylinder (l=3, r=0.5) systems, "
                    "N_i = round(exp(U(ln 500, ln 20000))) (seeded; {n:,} particles in all), pressures log-spaced "
                    "on [1, 20], lattice start at phi=0.30, triclinic boxes; per cycle one translation (0.2) per "
                    "sphere, a translation (0.2) and a rotation (0.2) per spherocylinder, one isotension box move "
                    "(delta 0.005, T=1) per replica", "moves/sec, 64 replicas"),
    "bent-rods-1e5": (_bent_rods_1e5, "bent rods of two hard spherocylinders (r=0.25, half axes (0.3, 0, +-0.15) "
                      "at x=-+0.35: a 60 degree kink), N={n:,} (25x40x100), aligned orthorhombic start at phi~0.33, "
                      "triclinic box; per cycle 2N moves (translation 0.2, rotation 0.2) + 1 isotension box move "
                      "(delta 0.005, p*=1.5, T=1)", "moves/sec, bent spherocylinder rods N=1e5"),
    "soft-wca-97336": (_soft_wca, "WCA fluid: spheres of sigma=1 with the repulsive Lennard-Jones "
                       "(RepulsiveLennardJonesInteraction, eps=1, cut at 2^(1/6) sigma) and no hard core, N={n:,} "
                       "(46^3), simple-cubic start at phi=0.40, triclinic box; per cycle N translations (0.2) "
                       "decided in FP64 with the Metropolis test at T=1 + 1 isotension box move (delta 0.005, p*=1.5) "
                       "with the total-energy change", "moves/sec, WCA fluid N=97336"),
    "convex-262144": (_convex_262144, "generic convex bodies (XCBodyBuilder 'cuboid 1 1 2; sphere 0.1; sum': "
                      "rounded 1x1x2 boxes, XenoCollide pair tests: FP32 portal refinement with FP64 certificates, "
                      "exact FP64 refinement otherwise), N={n:,} (64^3), aligned orthorhombic start at phi~0.55, "
                      "triclinic box; per cycle 2N moves (translation 0.2, rotation 0.2) + 1 isotension box move "
                      "(delta 0.005, p*=1.5, T=1)", "moves/sec, convex bodies N=262144"),
    "sc-64000": (_sc_64000, "hard spherocylinders l=5 r=0.5, N={n:,} (40^3), aligned orthorhombic start at "
                 "phi=0.35 (cell aspect 1:1:6), triclinic box; per cycle 2N moves (translation 0.2, rotation "
                 "0.2) + 1 isotension box move (delta 0.005, p*=1.5, T=1)", "moves/sec, spherocylinders N=64000"),
}


# per-workload overrides: the rotation step (0: translations only) and a soft part
# (kind, epsilon, sigma, with the hard core) set on the packing before the run
EXTRA = {"soft-wca-97336": {"rotation_step": 0.0, "soft": (1, 1.0, 1.0, False)}}


def rot_step(args) -> float:
    return EXTRA.get(args.workload, {}).get("rotation_step", ROT_STEP)


def workload(args):
    return WORKLOADS[args.workload][0](args)


def describe(args, n):
    return WORKLOADS[args.workload][1].format(n=n)


def metric(args):
    return WORKLOADS[args.workload][2]


# ----------------------------------------------------------------------------------
# clocks sampled during the timed region
# ----------------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu=timestamp,{self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, t0: float, t1: float) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = time.mktime(time.strptime(parts[0].split(".")[0], "%Y/%m/%d %H:%M:%S"))
                frac = float("0." + parts[0].split(".")[1]) if "." in parts[0] else 0.0
                rows.append((ts + frac, parts))
            except Exception:
                continue
        os.unlink(self.path)
        inside = [p for ts, p in rows if t0 - 0.15 <= ts <= t1 + 0.15]
        if not inside and rows:  # timed region shorter than the sampling period: nearest samples
            rows.sort(key=lambda r: abs(r[0] - 0.5 * (t0 + t1)))
            inside = [p for _, p in rows[:3]]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(p[2]) for p in inside if p[2].replace(".", "").isdigit()]
        mx = [float(p[3]) for p in inside if p[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for p in inside for k in range(4) if p[6 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside)}


# ----------------------------------------------------------------------------------
# CPU implementation (the oracle port of the reference's path; all host threads)
# ----------------------------------------------------------------------------------
def cpu_domains(threads: int):
    """Domain divisions for the CPU run: the largest product <= threads, z (the long axis) first."""
    best = (1, 1, 1)
    for dz in range(1, threads + 1):
        for dy in range(1, threads + 1):
            for dx in range(1, threads + 1):
                p = dx * dy * dz
                if p <= threads and dx <= dy <= dz and p > best[0] * best[1] * best[2]:
                    best = (dx, dy, dz)
    return best


def cpu_run(cfg, cycles: int, warmup: int, threads: int, seed: int, volume_moves: bool = False,
            rotation_step: float = ROT_STEP, soft=None):
    """The oracle's cycle loop on all host threads; with ``volume_moves`` the box move of odd
    cycles is the isotropic log-volume move instead of isotension (the headline's cycle)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    kind, prm, pos, rot, box = cfg
    pk = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=threads)
    if soft is not None:
        pk.set_soft(*soft)
    dom = cpu_domains(threads)
    kw = dict(translation_step=TRANS_STEP, rotation_step=rotation_step, box_kind=1, box_step=BOX_STEP,
              pressure=PRESSURE, temperature=TEMPERATURE, domains=dom, threads=threads, seed=seed)
    kw_vol = dict(kw, box_kind=2, box_step=VOL_STEP / 3)
    if warmup:
        po.run_cycles(pk, warmup, **kw)
    times = []
    for c in range(cycles):
        t = time.perf_counter()
        st = po.run_cycles(pk, 1, **dict(kw_vol if volume_moves and c % 2 else kw, seed=seed + 1000 + c))
        times.append(time.perf_counter() - t)
    pk.close()
    moves = (2 if rotation_step > 0 else 1) * len(pos)
    return moves, times, dom, list(st.domains)


def main_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    cfg = workload(args)
    moves, times, dom, dom_used = cpu_run(cfg, max(1, args.steps), max(0, args.warmup), threads, args.seed,
                                          volume_moves=args.workload == "sc-1e6", rotation_step=rot_step(args),
                                          soft=EXTRA.get(args.workload, {}).get("soft"))
    total = sum(times)
    value = moves * len(times) / total
    line = {
        "impl": "reference", "metric": metric(args), "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": len(times), "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": describe(args, len(cfg[2])), "n": len(cfg[2]), "moves_per_step": moves,
                   "parallelism": f"OpenMP domain decomposition {dom_used}"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{len(times)} full cycles of the N={len(cfg[2]):,} system after "
                                   f"{args.warmup} warm-up cycles; oracle/ restatement of the reference's "
                                   f"Simulation/Packing (reference sources are not present on this host)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------------
# GPU engine
# ----------------------------------------------------------------------------------
def propose_box(box, rng):
    """Isotension proposal: every box-matrix entry + U(-0.005, 0.005) (TriclinicDeltaScaler)."""
    return box + rng.uniform(-BOX_STEP, BOX_STEP, size=9)


def box_volume(box):
    return abs(np.linalg.det(box.reshape(3, 3)))


def cycle(g, k, seed, rng, stats=False):
    """One Monte Carlo cycle: a device sweep of 2N moves, then one box move whose Metropolis
    pre-check runs first on the host (core/Simulation.cpp:512-530)."""
    st = g.sweep(TRANS_STEP, ROT_STEP, seed=seed, counter=k, stats=stats)
    box = g.box
    nb = propose_box(box, rng)
    v0, v1 = box_volume(box), box_volume(nb)
    expo = g.n * math.log(v1 / v0) - PRESSURE * (v1 - v0) / TEMPERATURE
    u = rng.uniform()
    accepted = False
    if u <= math.exp(min(expo, 700.0)):
        if g.try_scaling(nb) > 0:
            g.revert_scaling()
        else:
            g.box = nb
            accepted = True
    return st, accepted


PROFILES = {"sc-1e6": "k_sweep_sc_n1e6.md", "banana-1e5": "k_sweep_banana_n1e5.md",
            "bent-rods-1e5": "k_sweep_bent_rods_n1e5.md",
            "replicas-64": "k_b_sweep_replicas_64.md", "soft-wca-97336": "k_soft_sweep_wca_n97336.md",
            "convex-262144": "k_soft_sweep_convex_n262144.md"}
REBUILD_PROFILES = {"sc-1e6": "rebuild_sc_n1e6.md"}


def read_profile_traffic(workload, key="traffic_bytes_per_launch", profiles=None):
    """Per-launch DRAM traffic of the workload's sweep kernel (or, with another key and table,
    per rebuild of the cell grid) from its committed ncu summary, if any."""
    name = (profiles or PROFILES).get(workload)
    path = os.path.join(ROOT, "profiles", name) if name else ""
    if not name or not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def read_profile_note(workload, key, profiles=None):
    """A one-line finding (e.g. the limiter of the sweep kernel) from the workload's committed
    ncu summary, if any."""
    name = (profiles or PROFILES).get(workload)
    path = os.path.join(ROOT, "profiles", name) if name else ""
    if not name or not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith(key + ":"):
            return line.split(":", 1)[1].strip()
    return None


def reduce_max(value: float, dist=None, device=None) -> float:
    """Maximum of a per-rank value over all ranks (the job's time is its slowest rank's)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main_gpu(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)

    from rampack_gb300 import build as rb
    rb.build()
    from rampack_gb300 import _lib
    from rampack_gb300.packing import GpuPacking

    cfg = workload(args)
    kind, prm, pos, rot, box = cfg
    n = len(pos)
    g = GpuPacking(kind, prm, pos, rot, box, device=local)
    if "soft" in EXTRA.get(args.workload, {}):
        g.set_soft(*EXTRA[args.workload]["soft"])
    if args.cells_per_warp:
        g.set_cells_per_warp(args.cells_per_warp)
    if args.bulk_staging >= 0:
        g.set_bulk_staging(args.bulk_staging == 1)
    if args.cell_order >= 0:
        g.set_cell_order(args.cell_order == 1)
    g.box = np.array(box, dtype=np.float64)
    stream = torch.cuda.ExternalStream(g.stream(), device=local)
    seed = args.seed + 7919 * rank

    # the native cycle loop (rp_sim): one device sweep, then one box move pre-checked on the
    # host: an isotension move (TriclinicDeltaScaler, every entry +- 0.005, std::mt19937) and,
    # on the headline, on every other cycle an isotropic log-volume move (ln V +- VOL_STEP),
    # each simulation with its own generator and Philox key
    from rampack_gb300 import simulation as SIM
    sims = [SIM.Simulation(g, TRANS_STEP, rot_step(args), seed, SIM.delta_triclinic(BOX_STEP, True))]
    if args.workload == "sc-1e6":
        sims.append(SIM.Simulation(g, TRANS_STEP, ROT_STEP, seed + 104729, SIM.log_volume(VOL_STEP / 3)))
    for sm in sims:
        sm.set_conditions(TEMPERATURE, PRESSURE)
    state = {"k": 0}

    def run_cycles(k):
        for _ in range(k):
            sims[state["k"] % len(sims)].run(1)
            state["k"] += 1

    def box_counts():
        out = []
        for sm in sims:
            st = sm.stats()
            out.append((st["box_moves"], st["accepted_box_moves"]))
        return out

    run_cycles(max(3, args.warmup))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    s0 = g.stats()
    b0 = box_counts()
    gc0 = g.grid_counters()
    g.set_timing(True)
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0 = time.time()
    ev0.record(stream)
    run_cycles(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    t1 = time.time()
    b1 = box_counts()
    box_names = ["isotension", "isotropic_volume"]
    box_moves = {box_names[i]: {"moves": b1[i][0] - b0[i][0], "accepted": b1[i][1] - b0[i][1]}
                 for i in range(len(sims))}
    box_acc = sum(v["accepted"] for v in box_moves.values())
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop(t0, t1)
    timing = g.timing()
    g.set_timing(False)
    s1 = g.stats()
    gc1 = g.grid_counters()
    if dist:
        ms = reduce_max(ms, dist, device=f"cuda:{local}")
        dist.barrier()

    moves = s1["moves"] - s0["moves"]
    value = moves * world / (ms / 1e3)
    acc_rate = (s1["accepted"] - s0["accepted"]) / max(1, moves)
    pairs = s1["pair_tests"] - s0["pair_tests"]
    fp64 = s1["fp64_pairs"] - s0["fp64_pairs"]
    launches = s1["kernel_launches"] - s0["kernel_launches"]

    # ---- roofline of the dominant kernel (the checkerboard sweep, one launch per phase) ----
    sweep_ms, sweep_launches = timing["sweep"]
    info, _, _ = g.grid()
    phases = 1
    for d in info["dims"]:
        phases *= 1 if d == 1 else (3 if d == 3 else 2)  # colours per grid dimension
    ncell = info["num_cells"]
    moves_per_sweep = (2 if rot_step(args) > 0 else 1) * n
    # algorithmic bytes per sweep: each phase streams every particle's FP32 record (28 B) and
    # cell index (4 B) and the cell offsets; every move reads the mover's FP64 state (96 B)
    # and an accepted move writes FP64 (96 B) and FP32 (28 B) state back.  Polyspheres of K
    # centres add per particle K FP32 centres (16 B each) to the record, K FP64 rotated
    # centres (24 B each) to the mover's read, and K rotated + K absolute FP64 centres and
    # K FP32 centres to an accepted move's write.
    kcen = int(prm[0]) if kind == 2 else 0
    rec32, s64, w64 = 28 + 16 * kcen, 96 + 24 * kcen, 96 + 28 + 64 * kcen
    # soft parts and convex bodies move through the FP64 sweep (k_soft_sweep): each phase reads
    # every particle's FP64 position (24 B; convex bodies also the orientation, 72 B) and grid
    # slot (4 B) through the movers' neighbourhoods; an accepted move writes the FP64 state
    fp64_sweep = kind == _lib.SHAPE_CONVEX or "soft" in EXTRA.get(args.workload, {})
    if fp64_sweep:
        rec32, s64, w64 = 24 + (72 if kind == _lib.SHAPE_CONVEX else 0), 96, 96
    b_sweep = phases * n * (rec32 + 4) + phases * (ncell + 1) * 4 + moves_per_sweep * (s64 + acc_rate * w64)
    b_launch = b_sweep / phases
    avg_launch_ms = sweep_ms / max(1, sweep_launches)
    achieved = b_launch / (avg_launch_ms / 1e3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = json.load(open(peaks_path))["hbm_gbs"], "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    traffic = read_profile_traffic(args.workload)
    # the cell-grid rebuild (k_assign, the scan, k_scatter, k_cell_finish): algorithmic bytes
    # per rebuild N (12 + 12) + 2 (C + 1) 4 -- per particle a position (12 B) in and its cell,
    # slot and rank indices (12 B) out, plus the cell histogram and offsets -- against its
    # CUDA-event time per rebuild
    rebuild_ms, rebuild_groups = timing["rebuild"]
    rebuilds = gc1["rebuilds"] - gc0["rebuilds"]
    b_rebuild = n * 24 + 2 * (ncell + 1) * 4
    rebuild_avg_ms = rebuild_ms / max(1, rebuild_groups)
    rebuild_achieved = b_rebuild / (rebuild_avg_ms / 1e3) / 1e9 if rebuild_groups else 0.0
    roofline_rebuild = {"bound": "hbm", "achieved": rebuild_achieved, "peak": peak, "unit": "GB/s",
                        "frac": rebuild_achieved / peak,
                        "traffic": read_profile_traffic(args.workload, "traffic_bytes_per_rebuild", REBUILD_PROFILES),
                        "kernel": "cell-grid rebuild (k_assign, k_scan_blocks, k_scan_sums, k_scan_add, k_scatter, "
                                  "k_cell_finish)",
                        "avg_rebuild_ms": rebuild_avg_ms, "bytes_per_rebuild": b_rebuild,
                        "rebuilds": rebuilds, "box_moves_on_kept_grid": gc1["remaps"] - gc0["remaps"]}
    # bytes every cycle touches: the FP64 state (96 B), the FP32 mirror (32 B) and the cell
    # lists the rebuild writes (slot, particle, cell and rank indices and the by-particle FP32
    # position: 32 B) per particle, plus the polysphere centres
    state_mb = n * (96 + 32 + 32 + 64 * kcen) / 1e6
    l2_note = (f"inputs larger than L2: every cycle touches {state_mb:.0f} MB of device state (FP64 state, "
               f"FP32 mirror, cell lists; L2 129 MB)" if state_mb > 129
               else f"inputs smaller than L2 ({state_mb:.0f} MB of state; no flush between steps)")

    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    if not args.no_e2e:
        hpos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        hrot = torch.empty((n, 9), dtype=torch.float64, pin_memory=True).numpy()
        hbox = torch.empty(9, dtype=torch.float64, pin_memory=True).numpy()
        g.state(out=(hpos, hrot, hbox))
        torch.cuda.synchronize()
        e_steps = max(1, args.steps)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        m0 = g.stats()["moves"]
        f0.record(stream)
        for _ in range(e_steps):
            g.upload(hpos, hrot, hbox)   # H2D of the step's input state (pinned)
            run_cycles(1)
            g.state(out=(hpos, hrot, hbox))  # D2H of the step's result into the same pinned buffers
        f1.record(stream)
        f1.synchronize()
        e_ms = f0.elapsed_time(f1)
        e_moves = g.stats()["moves"] - m0
        if dist:
            e_ms = reduce_max(e_ms, dist, device=f"cuda:{local}")
        e2e = {"value": e_moves * world / (e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": int(n * 12 * 8),
               "d2h_bytes_per_step": int(n * 12 * 8),
               "step": "rp_upload_state (pinned host -> device) + one cycle + rp_download_state (device -> pinned host)"}

    # ---- learned test ordering against the plain scan on the same state (rank 0, headline) ----
    ordering = None
    if rank == 0 and args.workload == "sc-1e6" and not args.no_ordering:
        ordering = ordering_compare(g, args, sweeps=max(4, min(args.steps, 8)),
                                    variants=[("plain", 0, 1), ("distance", 2, 16), ("mlp", 1, 64)])
    if rank == 0 and args.workload == "banana-1e5" and not args.no_ordering:
        # the bent chains of the learned-ordering configuration: the network trained on 10^7
        # logged pair outcomes
        ordering = ordering_compare(g, args, sweeps=max(4, min(args.steps, 8)), pairs=10_000_000, every_move=1,
                                    epochs=2, variants=[("plain", 0, 1), ("distance", 2, 4), ("mlp", 1, 4),
                                                        ("mlp", 1, 16)])

    # ---- CPU baseline (rank 0, N=1 only) ----
    cpu_base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cmoves, ctimes, dom, dom_used = cpu_run(cfg, 2, 1, threads, args.seed, volume_moves=args.workload == "sc-1e6",
                                                rotation_step=rot_step(args), soft=EXTRA.get(args.workload, {}).get("soft"))
        cpu_base = {"value": cmoves * len(ctimes) / sum(ctimes), "unit": UNIT, "cores": threads, "kind": "port",
                    "sample": f"2 full cycles of the same N={n:,} system after 1 warm-up cycle, OpenMP domain "
                              f"decomposition {dom_used} (oracle/ restatement of the reference's path)"}

    for sm in sims:
        sm.close()
    g.close()
    if rank == 0:
        line = {
            "metric": metric(args), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": describe(args, n), "n": n, "moves_per_step": moves_per_sweep,
                       "variant": "plain (unordered FP32 filter + FP64 guard band)",
                       "l2": l2_note,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "grid_dims": list(info["dims"]), "box_moves_accepted": box_acc,
                       "box_moves": box_moves},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": ("k_soft_sweep (FP64 moves; one launch per checkerboard phase)" if fp64_sweep
                                    else "k_sweep (one launch per checkerboard phase)"),
                         "limiter": read_profile_note(args.workload, "limiter"),
                         "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                         else "fallback 6.8 TB/s",
                         "avg_launch_ms": avg_launch_ms, "bytes_per_launch": b_launch},
            "roofline_rebuild": roofline_rebuild,
            "kernel_ms": {kname: {"ms": v[0], "groups": v[1]} for kname, v in timing.items()},
            "acceptance": acc_rate, "guard_band": {"pair_tests": pairs, "fp64_pairs": fp64,
                                                   "rate": fp64 / max(1, pairs)},
            "gpu_launches": launches, "clocks": clk,
            "e2e": e2e, "cpu_baseline": cpu_base,
        }
        if ordering is not None:
            line["ordering"] = ordering
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def ordering_compare(g, args, sweeps: int, variants, pairs: int = 4_000_000, every_move: int = 16,
                     epochs: int = 4):
    """Sweeps from the packing's current state with the plain neighbourhood scan, with partners
    ranked by centre distance and with partners ranked by the network trained (on the device,
    by the engine's own kernels) on pair outcomes the sweep itself logs.  Every ordering must
    leave the FP64 state bit-identical to the plain sweep's.  Per variant: device time of the
    move sweep and of the ranking per sweep (CUDA events), candidate pairs examined per move;
    ``speedup_vs_plain`` = plain total / variant total, ``speedup_ranking_free`` = plain sweep /
    variant sweep (the ceiling of the ordering with its ranking made free)."""
    from rampack_gb300 import _lib
    start = g.state()
    # training data: the pairs reaching the exact pair stage in every `every_move`-th move,
    # logged over as many sweeps as it takes to collect `pairs` outcomes
    g.pair_log_enable(pairs, every_move)
    training_sweeps = 0
    while g.pair_log_count() < pairs and training_sweeps < 40:
        g.sweep(TRANS_STEP, ROT_STEP, seed=args.seed + 1, counter=training_sweeps, stats=False)
        training_sweeps += 1
    feats, labels = g.pair_log()
    _, loss0 = g.mlp_gradient(feats[:200_000], labels[:200_000])
    g.set_timing(True)
    t0 = time.perf_counter()
    loss = g.mlp_train(epochs=epochs, batch=1024, lr=2e-3, seed=args.seed)
    train_s = time.perf_counter() - t0
    train_ms = g.timing()["mlp"][0]
    g.set_timing(False)
    _, loss1 = g.mlp_gradient(feats[:200_000], labels[:200_000])
    g.pair_log_enable(0)
    modes = {"plain": _lib.ORDER_OFF, "distance": _lib.ORDER_DISTANCE, "mlp": _lib.ORDER_MLP}
    rows, ref_state = [], None
    for label, _, every in variants:
        g.upload(*start)
        g.set_ordering(modes[label], every)
        g.set_timing(True)
        pairs = moves = 0
        for c in range(sweeps):
            st = g.sweep(TRANS_STEP, ROT_STEP, seed=args.seed + 2, counter=c)
            pairs += st["pair_tests"]
            moves += st["moves"]
        t = g.timing()
        g.set_timing(False)
        state = g.state()
        if ref_state is None:
            ref_state = state
        same = bool(np.array_equal(state[0], ref_state[0]) and np.array_equal(state[1], ref_state[1]))
        sweep_ms = (t["sweep"][0] + t["overflow"][0]) / sweeps
        order_ms = t["order"][0] / sweeps
        rows.append({"ordering": label, "rerank_every": every, "sweep_ms": round(sweep_ms, 4),
                     "ranking_ms": round(order_ms, 4), "total_ms": round(sweep_ms + order_ms, 4),
                     "pairs_per_move": round(pairs / moves, 2), "state_identical_to_plain": same})
    g.set_ordering(_lib.ORDER_OFF, 1)
    g.upload(*start)
    base, base_sweep = rows[0]["total_ms"], rows[0]["sweep_ms"]
    for r in rows:
        r["speedup_vs_plain"] = round(base / r["total_ms"], 3)
        r["speedup_ranking_free"] = round(base_sweep / r["sweep_ms"], 3)
    learned = [r for r in rows if r["ordering"] == "mlp"]
    best = max(learned or rows, key=lambda r: r["speedup_vs_plain"])
    return {"speedup_vs_plain": best["speedup_vs_plain"], "rerank_every": best["rerank_every"],
            "speedup_ranking_free": max(r["speedup_ranking_free"] for r in rows),
            "state_identical_to_plain": all(r["state_identical_to_plain"] for r in rows),
            "sweeps": sweeps, "unit": "ms per sweep (CUDA events)",
            "training": {"pairs": int(len(feats)), "logged_over_sweeps": training_sweeps,
                         "positive_fraction": round(float(labels.mean()), 4),
                         "epochs": epochs, "batch": 1024, "loss_before": round(loss0, 4),
                         "loss_after": round(loss1, 4), "last_epoch_loss": round(loss, 4),
                         "device_ms": round(train_ms, 1), "wall_s": round(train_s, 2)},
            "rows": rows}


def main_ordering(args):
    """The ordering comparison alone, with more variants: sweeps of the bench workload with the
    plain neighbourhood scan, with partners ranked by centre distance, and with partners ranked
    by the trained network, each re-ranked every 1, 16 or 64 sweeps."""
    from rampack_gb300 import build as rb
    rb.build()
    from rampack_gb300.packing import GpuPacking

    kind, prm, pos, rot, box = workload(args)
    g = GpuPacking(kind, prm, pos, rot, box)
    for c in range(20):
        g.sweep(TRANS_STEP, ROT_STEP, seed=args.seed, counter=c, stats=False)
    res = ordering_compare(g, args, sweeps=max(args.steps, 4),
                           variants=[("plain", 0, 1), ("distance", 0, 1), ("distance", 0, 16), ("mlp", 0, 1),
                                     ("mlp", 0, 16), ("mlp", 0, 64)])
    g.close()
    print(json.dumps(dict({"metric": "learned ordering vs plain scan", "workload": describe(args, len(pos))}, **res)))
    return 0


def _replica_cpu(job):
    """One replica of the CPU baseline (spawned worker): `cycles` timed cycles after one."""
    kind, prm, pos, rot, box, pressure, cycles, seed = job
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    pk = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    kw = dict(translation_step=TRANS_STEP, rotation_step=ROT_STEP if kind == 1 else 0.0, box_kind=1,
              box_step=BOX_STEP, pressure=pressure, temperature=TEMPERATURE)
    po.run_cycles(pk, 1, seed=seed, **kw)
    t = time.perf_counter()
    po.run_cycles(pk, cycles, seed=seed + 1, **kw)
    dt = time.perf_counter() - t
    pk.close()
    return (2 if kind == 1 else 1) * len(pos) * cycles, dt


def main_replicas(args):
    """64 replicas in two batches (one per shape), every step of a batch one launch for all
    its replicas; box moves proposed and pre-checked on the host per replica (isotension
    delta 0.005, each replica at its own pressure), overlap checks batched.  The launch shape
    (cell factor x warps per block) is autotuned first."""
    import multiprocessing as mp
    from rampack_gb300 import workloads as W
    reps = W.config_replicas_64(args.seed)
    # the CPU baseline first, in spawned workers, before this process touches the GPU
    cpu_base = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = list(range(0, 64, 4))
        jobs = [tuple(reps[i][:5]) + (reps[i][5], 2, args.seed + i) for i in sample]
        ctx = mp.get_context("spawn")
        t0 = time.perf_counter()
        with ctx.Pool(min(threads, len(jobs))) as pool:
            res = pool.map(_replica_cpu, jobs)
        wall = time.perf_counter() - t0
        moves = sum(m for m, _ in res)
        busy = max(d for _, d in res)
        cpu_base = {"value": moves / busy, "unit": UNIT, "cores": min(threads, len(jobs)), "kind": "port",
                    "sample": f"16 of the 64 replicas (every 4th), one per spawned process, 2 timed cycles after 1; "
                              f"value = their moves / the slowest replica's time (wall {wall:.1f} s incl. start-up)"}

    from rampack_gb300 import build as rb
    rb.build()
    from rampack_gb300.packing import BatchPacking
    groups = {k: [i for i in range(64) if reps[i][0] == k] for k in (0, 1)}
    batches = {k: BatchPacking(k, reps[idx[0]][1], [reps[i][2:5] for i in idx]) for k, idx in groups.items()}
    steps = {0: (TRANS_STEP, 0.0), 1: (TRANS_STEP, ROT_STEP)}
    boxes = {k: np.array([reps[i][4] for i in idx], dtype=np.float64) for k, idx in groups.items()}
    sizes = {k: np.array([len(reps[i][2]) for i in idx], dtype=np.float64) for k, idx in groups.items()}
    press = {k: np.array([reps[i][5] for i in idx]) for k, idx in groups.items()}
    rng = np.random.default_rng(args.seed)
    moves_per_cycle = int(sizes[0].sum() + 2 * sizes[1].sum())
    state = {"k": 0, "box_acc": 0}

    def one_cycle():
        k = state["k"]
        for kind, b in batches.items():
            b.sweep(*steps[kind], seed=args.seed + kind, counter=k, stats=False)
        for kind, b in batches.items():
            # every replica's isotension proposal and Metropolis pre-check, vectorised
            old = boxes[kind]
            new = old + rng.uniform(-BOX_STEP, BOX_STEP, size=old.shape)
            v0 = np.abs(np.linalg.det(old.reshape(-1, 3, 3)))
            v1 = np.abs(np.linalg.det(new.reshape(-1, 3, 3)))
            expo = sizes[kind] * np.log(v1 / v0) - press[kind] * (v1 - v0) / TEMPERATURE
            prop = (rng.uniform(size=b.R) <= np.exp(np.minimum(expo, 700.0))).astype(np.uint8)
            dE = b.try_scaling(np.where(prop[:, None] == 1, new, old), prop)
            bad = (prop == 1) & (dE > 0)
            b.revert_scaling(bad.astype(np.uint8))
            keep = (prop == 1) & ~bad
            boxes[kind][keep] = new[keep]
            state["box_acc"] += int(keep.sum())
        state["k"] += 1

    # autotune the launch shape: cell factor x warps per block
    tune = []
    grid = [(cf, wpb) for cf in (1.0, 1.1, 1.25) for wpb in (2, 4, 8)]
    if args.tuning:
        cf, wpb = args.tuning.split(",")
        grid = [(float(cf), int(wpb))]
    for cf, wpb in grid:
        for b in batches.values():
            b.set_tuning(cf, wpb)
        one_cycle()
        t = time.perf_counter()
        for _ in range(3):
            one_cycle()
        tune.append({"cell_factor": cf, "warps_per_block": wpb, "ms_per_cycle": (time.perf_counter() - t) / 3 * 1e3})
    best = min(tune, key=lambda x: x["ms_per_cycle"])
    for b in batches.values():
        b.set_tuning(best["cell_factor"], best["warps_per_block"])
    for _ in range(max(3, args.warmup)):
        one_cycle()
    s0 = {k: b.sweep(*steps[k], seed=args.seed + 99, counter=0, stats=True) for k, b in batches.items()}
    acc = sum(x["accepted"] for v in s0.values() for x in v) / max(1, sum(x["moves"] for v in s0.values() for x in v))
    state["box_acc"] = 0
    # per-launch sweep bytes of the dominant batch (the spherocylinders, k_b_sweep<1,4>): the
    # single-system formula per replica, summed, P·n·(28+4) + P·(C+1)·4 + M·(96 + a·(96+28))
    # with P the replica's phases, C its cells, M its moves, a the batch's acceptance; over
    # the batch's phase launches per sweep (its largest P)
    sc = batches[1]
    acc_sc = sum(x["accepted"] for x in s0[1]) / max(1, sum(x["moves"] for x in s0[1]))
    b_cycle, maxph = 0.0, 0
    for r in range(sc.R):
        info, _, _ = sc.grid(r)
        P = int(np.prod([1 if d == 1 else (3 if d == 3 else 2) for d in info["dims"]]))
        maxph = max(maxph, P)
        m = 2 * sc.sizes[r]
        b_cycle += P * sc.sizes[r] * 32 + P * (info["num_cells"] + 1) * 4 + m * (96 + acc_sc * 124)
    for b in batches.values():
        b.set_timing(True)
    launches0 = sum(b.timing()[1] for b in batches.values())
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.3)
    import torch
    torch.cuda.synchronize()
    t0 = time.time()
    tp = time.perf_counter()
    for _ in range(args.steps):
        one_cycle()
    torch.cuda.synchronize()
    dt = time.perf_counter() - tp
    clk = clocks.stop(t0, time.time())
    value = moves_per_cycle * args.steps / dt
    n = sum(len(r[2]) for r in reps)
    timing = {}
    launches = -launches0
    sc_sweep = None
    for kind, b in batches.items():
        t, l = b.timing()
        launches += l
        if kind == 1:
            sc_sweep = t["sweep"]
        for name, (ms_, g) in t.items():
            a = timing.setdefault(name, [0.0, 0])
            a[0] += ms_
            a[1] += g
        b.set_timing(False)
    avg_launch_ms = sc_sweep[0] / max(1, sc_sweep[1])
    b_launch = b_cycle / maxph
    achieved = b_launch / (avg_launch_ms / 1e3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = json.load(open(peaks_path))["hbm_gbs"], "measured (MEASURED_PEAKS.json hbm_gbs)"
    else:
        peak, peak_src = 6800.0, "fallback 6.8 TB/s"
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": read_profile_traffic("replicas-64"),
                "kernel": "k_b_sweep<1,4> (the spherocylinder batch: one launch per checkerboard phase)",
                "peak_source": peak_src,
                "avg_launch_ms": avg_launch_ms, "bytes_per_launch": b_launch}

    # ---- end to end through the C ABI: every replica's state from pinned host buffers,
    # one cycle, every state back into the same buffers ----
    e2e = None
    if not args.no_e2e:
        host = {}
        for kind, b in batches.items():
            tot = sum(b.sizes)
            host[kind] = (torch.empty((tot, 3), dtype=torch.float64, pin_memory=True).numpy(),
                          torch.empty((tot, 9), dtype=torch.float64, pin_memory=True).numpy(),
                          torch.empty((b.R, 9), dtype=torch.float64, pin_memory=True).numpy())
            b.states(out=host[kind])
            boxes[kind][:] = host[kind][2]
        torch.cuda.synchronize()
        tp = time.perf_counter()
        for _ in range(args.steps):
            for kind, b in batches.items():
                b.upload_all(*host[kind])
            one_cycle()
            for kind, b in batches.items():
                b.states(out=host[kind])
        torch.cuda.synchronize()
        e_dt = time.perf_counter() - tp
        nbytes = sum(h[0].nbytes + h[1].nbytes + h[2].nbytes for h in host.values())
        e2e = {"value": moves_per_cycle * args.steps / e_dt, "unit": UNIT, "h2d_bytes_per_step": int(nbytes),
               "d2h_bytes_per_step": int(nbytes),
               "step": "rp_batch_upload_states (pinned host -> device, both batches) + one cycle + "
                       "rp_batch_download_states (device -> pinned host)"}
    for b in batches.values():
        b.close()
    print(json.dumps({
        "metric": "moves/sec, 64 replicas", "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS["replicas-64"][1].format(n=n), "n": n, "moves_per_step": moves_per_cycle,
                   "timing": "host wall clock per cycle (both batches, host box-move pre-checks and the batched "
                             "overlap checks; each cycle ends in a device synchronisation)",
                   "autotune": tune, "tuning": best, "box_moves_accepted": state["box_acc"],
                   "l2": "inputs smaller than L2 (no flush between steps)"},
        "acceptance": acc, "roofline": roofline,
        "kernel_ms": {name: {"ms": v[0], "groups": v[1]} for name, v in timing.items()},
        "gpu_launches": launches, "e2e": e2e, "clocks": clk, "cpu_baseline": cpu_base,
    }))
    return 0


def main_io(args):
    """Snapshot files of the workload's packing: RAMSNAP store (device state -> text file) and
    restore (file -> device) wall time, and the sweep rate with a RAMTRJ snapshot recorded
    every cycle (asynchronous: device-side copy, side-stream download, host writer thread)
    against the same cycles without recording."""
    import tempfile
    import torch
    from rampack_gb300 import build as rb
    rb.build()
    from rampack_gb300.packing import GpuPacking
    from rampack_gb300.snapshots import RamtrjRecorder
    kind, prm, pos, rot, box = workload(args)
    n = len(pos)
    g = GpuPacking(kind, prm, pos, rot, box)
    t, r = (0.2, 0.2)
    k = 0
    for _ in range(max(3, args.warmup)):
        g.sweep(t, r, seed=args.seed, counter=k, stats=False)
        k += 1
    torch.cuda.synchronize()
    out = {}
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "s.ramsnap")
        t0 = time.perf_counter()
        g.store(f, {"cycles": str(k)})
        out["store_s"] = time.perf_counter() - t0
        out["ramsnap_mb"] = os.path.getsize(f) / 1e6
        t0 = time.perf_counter()
        g.restore(f)
        torch.cuda.synchronize()
        out["restore_s"] = time.perf_counter() - t0
        os.remove(f)
        steps = max(4, args.steps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            g.sweep(t, r, seed=args.seed, counter=k, stats=False)
            k += 1
        torch.cuda.synchronize()
        plain = (time.perf_counter() - t0) / steps
        rec_rate = {}
        for every in (1, 10):
            tf = os.path.join(d, f"t{every}.ramtrj")
            cycles = steps * every
            with RamtrjRecorder(tf, n, every) as rec:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for c in range(1, cycles + 1):
                    g.sweep(t, r, seed=args.seed, counter=k, stats=False)
                    k += 1
                    if c % every == 0:
                        rec.record(g, c)
                torch.cuda.synchronize()
                rec.flush()
                rec_rate[every] = 2 * n * cycles / (time.perf_counter() - t0)
            os.remove(tf)
        out["ramtrj_mb_per_snapshot"] = (9 * 8 + n * 48) / 1e6
    g.close()
    moves = 2 * n
    print(json.dumps({
        "metric": f"snapshot files, {args.workload}", "unit": "s / moves/s", "n": n,
        "ramsnap": {"store_s": out["store_s"], "restore_s": out["restore_s"], "mb": out["ramsnap_mb"],
                    "store_mb_per_s": out["ramsnap_mb"] / out["store_s"]},
        "ramtrj": {"moves_per_s_plain": moves / plain, "moves_per_s_recording_every_cycle": rec_rate[1],
                   "moves_per_s_recording_every_10_cycles": rec_rate[10],
                   "mb_per_snapshot": out["ramtrj_mb_per_snapshot"], "snapshots": steps,
                   "note": "host wall clock incl. the final flush; files in the default temporary directory"},
    }))
    return 0


def main_correlation(args):
    """Pair density correlation g(r) (PairDensityCorrelation over a RadialEnumerator) of the
    workload's packing: snapshots per second on the GPU (cell grid, FP32 pre-filter, FP64
    decisions, bins exact), against the oracle's restatement of the reference's all-pairs loop
    timed on a bounded sample and scaled by the number of pairs."""
    import torch
    from rampack_gb300 import build as rb
    rb.build()
    from rampack_gb300 import correlation as K
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = workload(args)
    n = len(pos)
    max_r, bins = args.corr_max_r, args.corr_bins
    g = GpuPacking(kind, prm, pos, rot, box)
    for c in range(3):   # a disordered state (the lattice's distances sit far from the bin edges)
        g.sweep(0.2, 0.2, seed=args.seed, counter=c, stats=False)
    enum = {"radial": K.RadialEnumerator(), "linear-z": K.LinearEnumerator("z"),
            "layerwise-z10": K.LayerwiseRadialEnumerator((0, 0, 10))}[args.corr_enumerator]
    obs = K.PairDensityCorrelation(enum, max_r, bins)
    for _ in range(max(3, args.warmup)):
        obs.add_snapshot(g)
    torch.cuda.synchronize()
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        obs.add_snapshot(g)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    counts, _ = obs.last_snapshot()
    tested = obs.info()["pairs_tested"]
    obs.close()
    g.close()
    line = {
        "metric": f"pair density correlation snapshots/s ({args.workload}, {args.corr_enumerator}, r <= {max_r}, "
                  f"{bins} bins)", "value": 1.0 / dt,
        "unit": "snapshots/s", "n_gpus": 1, "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": dt * 1e3,
        "higher_is_better": True, "dtype": "f32 binning, f64 guard band", "data": "synthetic",
        "config": {"workload": args.workload, "particles": n, "max_r": max_r, "bins": bins,
                   "observable": f"PairDensityCorrelation({type(enum).__name__})"},
        "pairs_in_range": int(counts.sum()), "pairs_decided_fp64": tested,
        "pairs_in_range_per_s": float(counts.sum()) / dt,
        "timing": "host wall clock per addSnapshot (device work synchronous inside)",
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as po
        po.build()
        ns = min(n, 20000)
        d = po.pair_desc(enumerator={"radial": 0, "linear-z": 1, "layerwise-z10": 2}[args.corr_enumerator],
                         linear_axis=2, miller=(0, 0, 10), function=0, num_bins=bins, max_r=max_r)
        c = po.OracleCorrelation(d)
        t0 = time.perf_counter()
        c.add_snapshot(pos[:ns], rot[:ns], box)
        cpu = time.perf_counter() - t0
        per_pair = cpu / (ns * (ns + 1) / 2)
        full = per_pair * n * (n + 1) / 2
        line["cpu_baseline"] = {"value": 1.0 / full, "unit": "snapshots/s", "cores": 1, "kind": "port",
                                "sample": f"all {ns * (ns + 1) // 2} pairs of the first {ns} particles "
                                          f"({cpu:.1f} s), scaled to the N(N+1)/2 pairs of one snapshot"}
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return main_reference(args)
    if args.io:
        return main_io(args)
    if args.correlation:
        return main_correlation(args)
    if args.ordering:
        return main_ordering(args)
    if args.workload == "replicas-64":
        return main_replicas(args)
    return main_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
