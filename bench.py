#!/usr/bin/env python
"""Benchmark of the many-body MD hot path: fcc Cu, 80^3 cells (2,048,000 atoms), Cleri-Rosato
TB-SMA, sigma 0.05 A, 600 K, NVE velocity Verlet dt = 1 fs, skin trigger 0.15 A.

One step = fused corrector/predictor + skin check (+ device list rebuild when triggered) +
density pass + force pass, all on one GPU.  Prints one JSON line (see the keys below).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64|ff]
                  [--impl ours|reference]

--impl reference times the CPU restatement of the reference's serial path (the oracle, the
reference's CUDA Fortran cannot be built here) with all host threads on the same workload.
With N > 1 (torchrun) every rank runs an independent replica (the path does not shard on
one box); value sums the ranks and the time is the max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s FP64 vs mixed @1e-6 force err; batched boxes/s; HVP cost/force"
UNIT = "atom-steps/s"
NCELL, SIGMA, TEMP, SEED, DT = 80, 0.05, 600.0, 2024, 1.0
MXKVOIS = 64
OUTER_SKIN = 1.0      # two-level list: candidates within rc_nl + 1 A (lists are the same sets)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def reduce_max(value, dist=None):
    """Max of a float over the ranks of the default process group (identity without one)."""
    if dist is None or not dist.is_initialized():
        return float(value)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(atoms_per_rank, steps, ms_max, world):
    """Whole-job atom-steps/s of `world` independent replicas timed by the slowest rank."""
    return world * atoms_per_rank * steps / (ms_max / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload_config(ncell, n):
    """The workload entry of `config`, identical in both arms."""
    return {"workload": "fcc Cu %dx%dx%d cells, %d atoms, Cleri-Rosato, sigma 0.05 A, 600 K, NVE dt=1fs, "
                        "skin 0.3 A (rebuild at 0.15 A)" % (ncell, ncell, ncell, n),
            "atoms": n}


def workload(ncell=NCELL):
    from msmpscu_gb300 import lattice as lt
    pos, vel, L = lt.cu_config(ncell, SIGMA, TEMP, SEED)
    return pos, vel, L


def precision_compare(e, box, pos, vel, steps):
    """FP64 form and float-float form on the same state: their atom-steps/s, and the mixed
    and float-float force errors against the FP64 forces (norm-wise and max-abs, relative).
    Both are parity-checked against the oracle at 1e-10 by the GPU tests."""
    e.copyin(box, pos, vel)
    e.set_precision("fp64")
    e.calforce()
    f64 = e.get_force()
    out = {}
    for prec in ("mixed", "ff"):
        e.set_precision(prec)
        e.calforce()
        d = e.get_force() - f64
        out[prec + "_force_err_norm"] = float(np.linalg.norm(d) / np.linalg.norm(f64))
        out[prec + "_force_err_max"] = float(np.abs(d).max() / np.abs(f64).max())
    for prec in ("fp64", "ff"):
        e.copyin(box, pos, vel)
        e.set_precision(prec)
        e.run_steps(3, DT)
        ms, _ = e.time_steps(steps, DT)
        out[prec + "_value"] = len(pos) * steps / (ms / 1e3)
        out[prec + "_pass_ms"] = {k: v for k, v in e.time_passes(3).items() if k != "fused"}
    e.set_precision("mixed")
    e.copyin(box, pos, vel)
    return out


def batched_uneven_boxes(steps, steps_perbox, device=0):
    """512 independent periodic Cu boxes, edge uniform in 4..12 fcc cells, 0-3 vacancies,
    300-1200 K: all boxes in one context (one launch per pass over every box, the whole step
    one CUDA graph) against one context per box (512 graphs per step, each on its own
    stream so they may overlap).  Metric: box-steps per second."""
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    boxes = lt.uneven_batch(512, seed=512)
    pos = np.vstack([b[0] for b in boxes])
    vel = np.vstack([b[1] for b in boxes])
    desc = [(len(b[0]), (0, 0, 0), tuple(b[2]), (1, 1, 1)) for b in boxes]
    table = ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC)
    out = {"boxes": len(boxes), "atoms": int(len(pos)),
           "box_atoms_min": int(min(len(b[0]) for b in boxes)),
           "box_atoms_max": int(max(len(b[0]) for b in boxes))}

    def wall(e, k):
        """host wall clock around k steps (enqueued, then finished; device synchronised on
        both sides): the clock the per-box contexts are timed with"""
        e.synchronize()
        t0 = time.perf_counter()
        e.enqueue_steps(k, DT)
        e.finish_steps(DT)
        return time.perf_counter() - t0

    for prec in ("mixed", "ff", "fp64"):
        e = Engine(len(pos), lt.CU_RC_NL, max_boxes=len(boxes), mxkvois=MXKVOIS, skin_trigger=0.15,
                   precision=prec, device=device)
        e.init_forcetable(table)
        e.set_masses([lt.CU_MASS])
        e.copyin(desc, pos, vel)
        e.run_steps(3, DT)
        l0, g0 = e.launches, e.graph_launches
        ms, reb = e.time_steps(steps, DT)
        out["batched_%s_box_steps_per_s" % prec] = len(boxes) * steps / (ms / 1e3)
        out["batched_%s_atom_steps_per_s" % prec] = len(pos) * steps / (ms / 1e3)
        out["batched_%s_ms_per_step" % prec] = ms / steps
        out["batched_%s_launches_per_step" % prec] = (e.launches - l0) / steps
        out["batched_%s_graph_launches_per_step" % prec] = (e.graph_launches - g0) / steps
        if prec == "mixed":
            out["batched_mixed_wall_box_steps_per_s"] = len(boxes) * steps_perbox / wall(e, steps_perbox)
            # ten steps per graph launch
            e.set_steps_per_graph(10)
            e.run_steps(10, DT)
            g0 = e.graph_launches
            t = wall(e, steps_perbox)
            out["batched_mixed_k10_wall_box_steps_per_s"] = len(boxes) * steps_perbox / t
            out["batched_mixed_k10_graph_launches_per_step"] = (e.graph_launches - g0) / steps_perbox
        e.close()
    engines = []
    for (p, v, L), d in zip(boxes, desc):
        e = Engine(len(p), lt.CU_RC_NL, max_boxes=1, mxkvois=MXKVOIS, skin_trigger=0.15,
                   precision="mixed", device=device)
        e.init_forcetable(table)
        e.set_masses([lt.CU_MASS])
        e.copyin([d], p, v)
        e.run_steps(2, DT)
        engines.append(e)
    for e in engines:
        e.synchronize()
    t0 = time.perf_counter()
    for e in engines:
        e.enqueue_steps(steps_perbox, DT)
    for e in engines:
        e.finish_steps(DT)
    t1 = time.perf_counter()
    for e in engines:
        e.close()
    out["perbox_mixed_box_steps_per_s"] = len(boxes) * steps_perbox / (t1 - t0)
    out["perbox_graph_launches_per_step"] = len(boxes)
    # both sides on the host wall clock (the device-time figure is kept beside it)
    out["batched_vs_perbox"] = out["batched_mixed_wall_box_steps_per_s"] / out["perbox_mixed_box_steps_per_s"]
    out["batched_vs_perbox_device_vs_wall"] = (out["batched_mixed_box_steps_per_s"] /
                                               out["perbox_mixed_box_steps_per_s"])
    out["batched_k10_vs_perbox"] = out["batched_mixed_k10_wall_box_steps_per_s"] / out["perbox_mixed_box_steps_per_s"]
    out["perbox_timing"] = ("host wall clock around %d steps of 512 contexts and around %d steps of the "
                            "batched context (device synchronised both sides)" % (steps_perbox, steps_perbox))
    return out


def hvp_w_dumbbell(device=0):
    """bcc W 20^3 cells + <111> dumbbell (16,001 atoms), Marinica EAM2: device time of one
    HVP against one FP64 force call on the same state."""
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    pos, L = lt.w_sia_config(20, 0.0, 1)
    e = Engine(len(pos), lt.W_RC_NL, mxkvois=96, device=device)
    e.init_forcetable(ForceTable.marinica_eam2())
    e.copyin([(len(pos), (0, 0, 0), tuple(L), (1, 1, 1))], pos)
    v = np.random.default_rng(0).normal(size=pos.shape)
    v /= np.linalg.norm(v)
    ms_hvp, ms_force = e.time_hvp(v, reps=20)
    e.close()
    return {"atoms": len(pos), "hvp_ms": ms_hvp, "force_call_ms": ms_force,
            "hvp_cost_force_calls": ms_hvp / ms_force}


def hvp_cu_large(device=0):
    """fcc Cu 80^3 cells (2,048,000 atoms, sigma 0.05 A), Cleri-Rosato: device time of one HVP
    against one FP64 force call, and the size of the HVP's pair buffer."""
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    pos, _, L = lt.cu_config(80, 0.05, 600.0, 5)
    e = Engine(len(pos), lt.CU_RC_NL, mxkvois=64, device=device)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.copyin([(len(pos), (0, 0, 0), tuple(L), (1, 1, 1))], pos)
    v = np.random.default_rng(0).normal(size=pos.shape)
    v /= np.linalg.norm(v)
    ms_hvp, ms_force = e.time_hvp(v, reps=5)
    e.close()
    return {"atoms": len(pos), "hvp_ms": ms_hvp, "force_call_ms": ms_force,
            "hvp_cost_force_calls": ms_hvp / ms_force, "pair_buffer_bytes": 40 * 64 * len(pos)}


def adjoint_cu_snapshots(device=0):
    """64 fcc Cu snapshots of 4,000 atoms (sigma 0.1 A), targets from parameters x 1.02:
    wall time of one adjoint call (FP64 forces + adjoint passes + host derivative tables)
    against one FP64 force call with copy-out."""
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    from msmpscu_gb300 import _lib as L
    snaps = [lt.cu_config(10, 0.1, 300.0, 1000 + s) for s in range(64)]
    pos = np.vstack([s[0] for s in snaps])
    desc = [(len(s[0]), (0, 0, 0), tuple(s[2]), (1, 1, 1)) for s in snaps]
    prm = np.array([lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")])
    e = Engine(len(pos), lt.CU_RC_NL, max_boxes=64, mxkvois=MXKVOIS, device=device)
    e.init_forcetable(ForceTable(L.POT_CR, prm * 1.02, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
    e.copyin(desc, pos)
    e.calforce()
    ft = e.get_force()
    e.init_forcetable(ForceTable(L.POT_CR, prm, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
    e.param_adjoint(prm, ft)
    t0 = time.perf_counter()
    for _ in range(5):
        loss, grad = e.param_adjoint(prm, ft)
    t1 = time.perf_counter()
    for _ in range(5):
        e.calforce()
        e.get_force()
    t2 = time.perf_counter()
    e.close()
    return {"atoms": len(pos), "adjoint_ms": (t1 - t0) / 5 * 1e3, "force_call_ms": (t2 - t1) / 5 * 1e3,
            "adjoint_cost_force_calls": (t1 - t0) / (t2 - t1), "loss": loss,
            "grad": [float(g) for g in grad]}


def make_engine(n, precision, device=0, outer_skin=None):
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    e = Engine(n, lt.CU_RC_NL, mxkvois=MXKVOIS, skin_trigger=0.15, precision=precision, device=device,
               outer_skin=OUTER_SKIN if outer_skin is None else outer_skin)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


def steady_state(pos, vel, L, steps=1000, device=0):
    """The whole 1,000-step NVE run of the 2,048,000-atom Cu workload in each precision, from
    the copied-in state (list built at the copy-in), timed with CUDA events over all steps:
    atom-steps/s, list rebuilds inside the run (all and full ones) and the whole-step roofline
    of the run.  The mixed/FP64 and float-float/FP64 ratios come from these same runs."""
    n = len(pos)
    box = [(n, (0, 0, 0), tuple(L), (1, 1, 1))]
    hbm, _ = peaks()
    out = {"steps": steps}
    for prec in ("mixed", "ff", "fp64"):
        e = make_engine(n, prec, device)
        e.copyin(box, pos, vel)
        rc0 = e.rebuild_counts()        # the list, first forces, tuning and graphs: untimed
        ms, reb = e.time_steps(steps, DT)
        rc1 = e.rebuild_counts()
        _, kmean = e.list_stats()
        v = n * steps / (ms / 1e3)
        b = bytes_model(kmean)["step"]
        out[prec] = {"value": v, "ms_per_step": ms / steps, "rebuilds": rc1[0] - rc0[0],
                     "full_rebuilds": rc1[1] - rc0[1],
                     "step_roofline_frac": b * v / 1e9 / hbm, "bytes_per_atom_step": b}
        e.close()
    out["mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["ff_vs_fp64"] = out["ff"]["value"] / out["fp64"]["value"]
    return out


def bytes_model(kmean):
    """Algorithmic bytes per atom and launch (design-independent): int32 list entries read
    once per pass, own FP64 position (24 B), F'(rho) write/read (8 B each), force write
    (24 B); integrator reads x, v, F and writes x, v (5 x 24 B) and reads the build-time
    position for the skin check (24 B)."""
    dens = 4.0 * kmean + 24.0 + 8.0
    force = 4.0 * kmean + 24.0 + 8.0 + 24.0
    vv = 5 * 24.0 + 24.0
    # fused force pass + integrator: the force it writes is not read back
    return dict(density=dens, force=force, vv=vv, fused=force + vv - 24.0, step=dens + force + vv)


def oracle_parity(pos, vel, L, device=0, sample=200000):
    """Part of the CPU leg: the full 2,048,000-atom system against the oracle (OpenMP),
    relative force error of each precision (max abs difference over the max magnitude, and
    norm-wise), and the neighbour sets of a random sample of atoms compared as sets."""
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    from oracle import pyoracle as po
    n = len(pos)
    tabs = po.make_tables(po.POT_CR, [lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")],
                          lt.CU_RC, 10000, 10000, 20.0, want_embed=False)
    t = po.Tables(tabs, po.FS, lt.CU_RC)
    box = po.make_box([0, 0, 0], L)
    ones = np.ones(n, np.int32)
    okv, oind = po.nlist(pos, ones, box, lt.CU_RC_NL, 80)
    ref = po.force(pos, ones, ones, box, okv, oind, t, want_virial=False, want_epot=False)["f"]
    out = {"atoms": n}
    for prec in ("fp64", "ff", "mixed"):
        e = Engine(n, lt.CU_RC_NL, mxkvois=MXKVOIS, precision=prec, device=device)
        e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
        e.copyin([(n, (0, 0, 0), tuple(L), (1, 1, 1))], pos, vel)
        e.calforce()
        d = e.get_force() - ref
        out[prec + "_force_err_max"] = float(np.abs(d).max() / np.abs(ref).max())
        out[prec + "_force_err_norm"] = float(np.linalg.norm(d) / np.linalg.norm(ref))
        if prec == "fp64":
            kv, ind = e.get_neighborelist()
            rng = np.random.default_rng(1)
            idx = rng.choice(n, min(sample, n), replace=False)
            same = sum(1 for i in idx if np.array_equal(np.sort(ind[:kv[i], i]), np.sort(oind[:okv[i], i])))
            out["nl_atoms_checked"] = int(len(idx))
            out["nl_sets_identical"] = int(same)
        e.close()
    return out


def reference_output(device=0):
    """Forces and per-atom energies against the reference's own output: the step-0 records of
    its NEB example (2,000 W + 1 H, Bonny EAM1; tests/golden/neb_w2000h1_bonny_eam1.npz) with
    that run's parameters (RU = 1.9 lattice units, neighbour cutoff NB_RM = 1.2 RU, 10,000
    table points up to NB_RM as the version that wrote the records had them).  Per precision,
    over both records: the largest |F - F_ref| and |E - E_ref|, and the largest of each over
    the tolerance of its printed digits (half a unit in the 9th significant digit; forces at
    least 1e-11 eV/LU): a ratio up to 1 reproduces the printed value."""
    from msmpscu_gb300 import Engine, forcelib, lattice as lt
    d = np.load(os.path.join(ROOT, "tests", "golden", "neb_w2000h1_bonny_eam1.npz"))

    def half_unit(v):
        a = np.abs(v)
        return 0.5005 * 10.0 ** (np.floor(np.log10(np.where(a > 0.0, a, 1.0))) - 8)

    out = {"records": 2, "atoms": int(len(d["c0_typ"])), "potential": "EAM_WHeH_Bonny_JPCM26_2014 EAM1"}
    for prec in ("fp64", "ff", "mixed"):
        w = {"f_max_eV_per_A": 0.0, "e_atom_max_eV": 0.0, "f_over_printed_digits": 0.0, "e_over_printed_digits": 0.0}
        for k in range(2):
            latt = float(d["c%d_latt" % k])
            ru = 1.9 * latt
            typ = d["c%d_typ" % k]
            pos = d["c%d_pos" % k] * latt
            f_lu, pot = d["c%d_force" % k], d["c%d_pot" % k]
            n = len(typ)
            ft = forcelib.create("EAM_WHeH_Bonny_JPCM26_2014", ru=ru, rmax=1.2 * ru,
                                 ptype=np.array([[1, 2], [4, 5]], np.int32), subtype="EAM1")
            e = Engine(n, 1.2 * ru, mxkvois=160, precision=prec, device=device)
            e.init_forcetable(ft)
            e.set_masses(np.array([183.84, 1.008]) * lt.AMU)
            e.copyin([(n, tuple(d["c%d_boxlow" % k] * latt), tuple(d["c%d_boxsize" % k] * latt), (1, 1, 1))],
                     pos, ityp=typ)
            e.calforce()
            f = e.get_force() * latt            # eV/LU, as printed
            e.calepot()
            ep = -e.get_epot()                  # printed as -EPOT
            e.close()
            df, de = np.abs(f - f_lu), np.abs(ep - pot)
            w["f_max_eV_per_A"] = max(w["f_max_eV_per_A"], float(df.max() / latt))
            w["e_atom_max_eV"] = max(w["e_atom_max_eV"], float(de.max()))
            w["f_over_printed_digits"] = max(w["f_over_printed_digits"],
                                             float(np.max(df / np.maximum(half_unit(f_lu), 1e-11))))
            w["e_over_printed_digits"] = max(w["e_over_printed_digits"], float(np.max(de / half_unit(pot))))
        out[prec] = w
    return out


def nve_drift(device=0, steps=20000, every=2000):
    """Total-energy drift of NVE runs (Cu 10^3 cells, 4,000 atoms, 600 K, sigma 0.05 A,
    dt = 1 fs, skin trigger) in each precision: (E(end) - E(0)) per atom per ns and the largest
    excursion |E(t) - E(0)| per atom seen at the checkpoints.  Energies from the FP64 passes."""
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    pos, vel, L = lt.cu_config(10, SIGMA, TEMP, 7)
    n = len(pos)
    box = [(n, (0, 0, 0), tuple(L), (1, 1, 1))]
    out = {"atoms": n, "steps": steps, "dt_fs": DT}

    def energy(e):
        _, v, _, _ = e.get_state()
        prec = e.precision
        e.set_precision("fp64")
        e.calepot()
        pe = float(e.get_epot().sum())
        e.set_precision(prec)
        return pe + 0.5 * lt.CU_MASS * float((v * v).sum())

    for prec in ("fp64", "ff", "mixed"):
        e = Engine(n, lt.CU_RC_NL, mxkvois=MXKVOIS, skin_trigger=0.15, precision=prec, device=device)
        e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
        e.set_masses([lt.CU_MASS])
        e.copyin(box, pos, vel)
        e0 = energy(e)
        excursion = 0.0
        for _ in range(steps // every):
            e.run_steps(every, DT)
            excursion = max(excursion, abs(energy(e) - e0))
        e1 = energy(e)
        out[prec + "_drift_eV_per_atom_per_ns"] = (e1 - e0) / n / (steps * DT * 1e-6)
        out[prec + "_max_excursion_eV_per_atom"] = excursion / n
        e.close()
    return out


def cpu_baseline(pos, vel, L, nthreads, sample_steps=2):
    """Oracle (C restatement of the reference's serial CPU path) on the full workload:
    per-step time = (T(k steps) - T(0 steps)) / k, both runs including the initial list
    build and force."""
    from msmpscu_gb300 import lattice as lt
    from oracle import pyoracle as po
    n = len(pos)
    tabs = po.make_tables(po.POT_CR, [lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")],
                          lt.CU_RC, 10000, 10000, 20.0, want_embed=False)
    t = po.Tables(tabs, po.FS, lt.CU_RC)
    box = po.make_box([0, 0, 0], L)
    ones = np.ones(n, np.int32)
    cm = np.array([lt.CU_MASS])
    t0 = time.perf_counter()
    po.md(pos, vel, ones, ones, box, t, cm, DT, 0, lt.CU_RC_NL, skin_trigger=0.15, mxkvois=80,
          nthreads=nthreads)
    t1 = time.perf_counter()
    po.md(pos, vel, ones, ones, box, t, cm, DT, sample_steps, lt.CU_RC_NL, skin_trigger=0.15,
          mxkvois=80, nthreads=nthreads)
    t2 = time.perf_counter()
    per_step = max((t2 - t1) - (t1 - t0), 1e-9) / sample_steps
    return n / per_step, per_step


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    pos, vel, L = workload(args.ncell)
    n = len(pos)
    threads = os.cpu_count() or 1
    from msmpscu_gb300 import lattice as lt
    from oracle import pyoracle as po
    tabs = po.make_tables(po.POT_CR, [lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")],
                          lt.CU_RC, 10000, 10000, 20.0, want_embed=False)
    t = po.Tables(tabs, po.FS, lt.CU_RC)
    box = po.make_box([0, 0, 0], L)
    ones = np.ones(n, np.int32)
    cm = np.array([lt.CU_MASS])
    # warm-up: W steps (list build + forces), then the timed K steps run as one NVE segment,
    # capped at a time budget so the whole run ends within a few minutes
    p1, v1, _, _, _ = po.md(pos, vel, ones, ones, box, t, cm, DT, args.warmup, lt.CU_RC_NL,
                            skin_trigger=0.15, mxkvois=80, nthreads=threads)
    t0 = time.perf_counter()
    po.md(p1, v1, ones, ones, box, t, cm, DT, 0, lt.CU_RC_NL, skin_trigger=0.15, mxkvois=80,
          nthreads=threads)
    t_setup = time.perf_counter() - t0
    per_step_guess = None
    done = 0
    budget = args.ref_budget_s
    chunk = max(1, min(args.steps, 5))
    t_total = 0.0
    while done < args.steps:
        k = min(chunk, args.steps - done)
        ta = time.perf_counter()
        p1, v1, _, _, _ = po.md(p1, v1, ones, ones, box, t, cm, DT, k, lt.CU_RC_NL,
                                skin_trigger=0.15, mxkvois=80, nthreads=threads)
        dt = time.perf_counter() - ta - t_setup
        t_total += max(dt, 1e-9)
        done += k
        if t_total > budget:
            break
    value = n * done / t_total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded fcc Cu lattice)",
            "config": dict(workload_config(args.ncell, n), parallelism="host threads (OpenMP over atoms)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d of %d NVE steps of the full %d-atom system "
                                       "(oracle, OpenMP over atoms)" % (done, args.steps, n)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_case(args):
    """One differentiation kernel pair on its own, for a profiler capture or a quick timing:
    `hvp` on bcc W ncell^3 cells with the <111> dumbbell (Marinica EAM2, ncell 20 = the 16,001-atom
    case), `adjoint` on `snapshots` fcc Cu boxes of ncell^3 cells (Cleri-Rosato, sigma 0.1 A,
    targets from the parameters x 1.02; ncell 10 and 64 snapshots = the 64 x 4,000-atom case).
    Prints one JSON line with the device or wall times."""
    from msmpscu_gb300 import build as lib_build
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    from msmpscu_gb300 import _lib as L
    lib_build.build()
    if args.case == "hvp":
        pos, box_len = lt.w_sia_config(args.ncell, 0.0, 1)
        e = Engine(len(pos), lt.W_RC_NL, mxkvois=96)
        e.init_forcetable(ForceTable.marinica_eam2())
        e.copyin([(len(pos), (0, 0, 0), tuple(box_len), (1, 1, 1))], pos)
        v = np.random.default_rng(0).normal(size=pos.shape)
        v /= np.linalg.norm(v)
        ms_hvp, ms_force = e.time_hvp(v, reps=args.steps)
        e.close()
        out = {"case": "hvp", "atoms": len(pos), "hvp_ms": ms_hvp, "force_call_ms": ms_force,
               "hvp_cost_force_calls": ms_hvp / ms_force}
    else:
        snaps = [lt.cu_config(args.ncell, 0.1, 300.0, 1000 + s) for s in range(args.snapshots)]
        pos = np.vstack([s[0] for s in snaps])
        desc = [(len(s[0]), (0, 0, 0), tuple(s[2]), (1, 1, 1)) for s in snaps]
        prm = np.array([lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")])
        e = Engine(len(pos), lt.CU_RC_NL, max_boxes=len(snaps), mxkvois=MXKVOIS)
        e.init_forcetable(ForceTable(L.POT_CR, prm * 1.02, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
        e.copyin(desc, pos)
        e.calforce()
        ft = e.get_force()
        e.init_forcetable(ForceTable(L.POT_CR, prm, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
        e.param_adjoint(prm, ft)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e.param_adjoint(prm, ft)
        t1 = time.perf_counter()
        e.close()
        out = {"case": "adjoint", "atoms": len(pos), "snapshots": len(snaps),
               "adjoint_wall_ms": (t1 - t0) / args.steps * 1e3}
    print(json.dumps(out), flush=True)


def run_ours(args):
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if ws > 1 else 0
    from msmpscu_gb300 import build as lib_build
    lib_build.build()
    pos, vel, L = workload(args.ncell)
    n = len(pos)
    prec = args.precision
    e = make_engine(n, prec, device, args.outer_skin)
    if args.steps_per_graph > 1:
        e.set_steps_per_graph(args.steps_per_graph)
    box = [(n, (0, 0, 0), tuple(L), (1, 1, 1))]
    e.copyin(box, pos, vel)
    if args.pin:
        d, f, u = (int(v) for v in args.pin.split(","))
        e.set_tuning(density=d, force=f, fused=u)
    e.run_steps(args.warmup, DT)
    if dist:
        dist.barrier()
    l0 = e.launches
    rc0 = e.rebuild_counts()
    with Clocks(device) as clk:
        ms, rebuilds = e.time_steps(args.steps, DT)
    launches = e.launches - l0
    full_rebuilds = e.rebuild_counts()[1] - rc0[1]
    ms = reduce_max(ms, dist)
    value = replica_value(n, args.steps, ms, ws)
    kmax, kmean = e.list_stats()
    passes = e.time_passes(5)
    rbt = e.time_rebuilds(3)
    passes["nlist_full"], passes["nlist_reselect"] = rbt["full"], rbt["inner"]
    tune = e.tuning() if prec == "mixed" else None
    bm = bytes_model(kmean)
    hbm, peak_kind = peaks()
    cands = ["density", "fused"] if passes.get("fused", 0.0) > 0.0 else ["density", "force"]
    dom = max(cands, key=lambda k: passes[k])
    achieved = bm[dom] * n / (passes[dom] * 1e-3) / 1e9
    traffic = read_traffic(prec, dom)
    # every kernel of the step, the dominant one above (the two passes lie within a few %)
    roof_all = {k: {"ms": passes[k], "algorithmic_bytes_per_atom": bm[k],
                    "achieved": bm[k] * n / (passes[k] * 1e-3) / 1e9,
                    "frac": bm[k] * n / (passes[k] * 1e-3) / 1e9 / hbm,
                    "traffic": read_traffic(prec, k)} for k in cands}

    # e2e: the reference-facing C-ABI with pinned host buffers: copy-in of the state, the K
    # steps, copy-out of positions, velocities and forces, all inside the timed region
    xp, xp1, ty, st, fo, xo, vo = pinned_buffers(n)
    xp[:] = np.ascontiguousarray(pos.T).reshape(-1)
    xp1[:] = np.ascontiguousarray(vel.T).reshape(-1)
    ty[:] = 1
    st[:] = 1
    barr = e.pack_boxes(box)
    e.synchronize()
    t0 = time.perf_counter()
    e.copyin_raw(barr, 1, ty, st, xp, xp1)
    e.run_steps(args.steps, DT)
    e.copyout_raw(xo, vo, fo)
    t1 = time.perf_counter()
    e2e = n * args.steps / (t1 - t0)
    h2d = n * (24 + 24 + 4 + 4) / args.steps
    d2h = n * (24 + 24 + 24) / args.steps

    cmp = None
    if prec == "mixed" and not args.no_compare:
        pc = precision_compare(e, box, pos, vel, max(3, min(args.steps, 40)))
        cmp = {"fp64_value": pc["fp64_value"], "mixed_value": value / ws,
               "speedup": value / ws / pc["fp64_value"],
               "mixed_force_err_norm": pc["mixed_force_err_norm"], "mixed_force_err_max": pc["mixed_force_err_max"],
               "ff_value": pc["ff_value"], "ff_speedup_vs_fp64": pc["ff_value"] / pc["fp64_value"],
               "ff_force_err_norm": pc["ff_force_err_norm"], "ff_force_err_max": pc["ff_force_err_max"],
               "fp64_pass_ms": pc["fp64_pass_ms"], "ff_pass_ms": pc["ff_pass_ms"]}

    extras = {}
    if not args.no_extras:
        e.close()
        extras["batched_boxes"] = batched_uneven_boxes(max(10, min(args.steps, 100)), 20, device)
        extras["hvp"] = hvp_w_dumbbell(device)
        extras["hvp_cu_2048k"] = hvp_cu_large(device)
        extras["adjoint"] = adjoint_cu_snapshots(device)
        extras["nve_drift"] = nve_drift(device)
        extras["reference_output"] = reference_output(device)
        extras["steady_state_1000"] = steady_state(pos, vel, L, 1000, device)
        e = None

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cv, per = cpu_baseline(pos, vel, L, threads, sample_steps=args.cpu_steps)
        # the reference's CPU path is serial: the same sample on one thread
        cv1, per1 = cpu_baseline(pos, vel, L, 1, sample_steps=1)
        cpu = {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d NVE steps of the full 2,048,000-atom system (oracle, OpenMP over "
                         "atoms), per-step time %.2f s" % (args.cpu_steps, per),
               "serial_value": cv1, "serial_sample": "1 NVE step of the same system on one thread, "
                                                     "per-step time %.2f s" % per1}
        # the CPU leg also runs the oracle as the checker of the device passes on the full system
        if not args.no_extras:
            extras["oracle_parity"] = oracle_parity(pos, vel, L, device)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f32+f64",
                "data": "synthetic (seeded fcc Cu lattice, Gaussian displacements, Maxwell-Boltzmann velocities)",
                "config": {**workload_config(args.ncell, n), "precision": prec, "parallelism": "replicas" if ws > 1 else "single GPU",
                           "l2": "inputs larger than L2 (~0.9 GB touched per step)",
                           "rebuilds_in_timed_steps": rebuilds, "full_rebuilds_in_timed_steps": full_rebuilds,
                           "outer_skin": args.outer_skin, "pinned_variants": args.pin, "mean_neighbours": kmean,
                           "max_neighbours": kmax},
                "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                             "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                             "peak_kind": peak_kind,
                             "algorithmic_bytes_per_atom": bm[dom]},
                "roofline_per_kernel": roof_all,
                "step_roofline": {"achieved": bm["step"] * value / ws / 1e9, "peak": hbm, "unit": "GB/s",
                                  "frac": bm["step"] * value / ws / 1e9 / hbm,
                                  "bytes_per_atom_step": bm["step"]},
                "pass_ms": passes,
                "autotune": tune,
                "precision_compare": cmp,
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "cpu_baseline": cpu,
                **extras,
                "clocks": clk.summary(),
                "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    if e is not None:
        e.close()
    if dist:
        dist.destroy_process_group()


def pinned_buffers(n):
    """Page-locked host arrays for the end-to-end leg: positions, velocities, types and status
    going in; forces, positions and velocities coming out."""
    try:
        import torch
        if torch.cuda.is_available():
            mk = lambda k, dt: torch.empty(k, dtype=dt, pin_memory=True).numpy()
            return (mk(3 * n, torch.float64), mk(3 * n, torch.float64), mk(n, torch.int32),
                    mk(n, torch.int32), mk(3 * n, torch.float64), mk(3 * n, torch.float64),
                    mk(3 * n, torch.float64))
    except Exception:
        pass
    return (np.empty(3 * n), np.empty(3 * n), np.empty(n, np.int32), np.empty(n, np.int32),
            np.empty(3 * n), np.empty(3 * n), np.empty(3 * n))


def read_traffic(prec, kernel):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        for line in open(path):
            p = line.split()
            if len(p) >= 3 and not line.startswith("#") and p[0] == prec and p[1] == kernel:
                return float(p[2])
    except OSError:
        pass
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "ff"])
    ap.add_argument("--ncell", type=int, default=NCELL,
                    help="fcc cells per edge (80 = the benchmark; smaller for profiling captures)")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-box, HVP and adjoint measurements")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--outer-skin", type=float, default=OUTER_SKIN,
                    help="two-level list: candidates within rc_nl + this skin (0: single-level)")
    ap.add_argument("--pin", default=None,
                    help="mixed passes: kernel variant codes density,force,fused instead of the tuner's")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--steps-per-graph", type=int, default=1,
                    help="MD steps captured per CUDA graph launch (msmgb_set_steps_per_graph)")
    ap.add_argument("--case", default="md", choices=["md", "hvp", "adjoint"],
                    help="hvp / adjoint: only that differentiation call (profiling captures)")
    ap.add_argument("--snapshots", type=int, default=64, help="--case adjoint: number of Cu boxes")
    ap.add_argument("--ref-budget-s", type=float, default=150.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.case != "md":
        run_case(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
