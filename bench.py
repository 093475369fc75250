#!/usr/bin/env python
"""Benchmark: particle-updates/s of the explicit-MPM double-pass step on GB300.

Workload (default, "batch"): 256 independent square-honeycomb specimens, each
with its own grid, crushed in-plane by rigid platens on the contact path and
advanced together by one engine: walls U(0.4, 1.2) mm, pitch U(4, 8) mm,
4-10 cells per side, h = 0.25 mm, 8 particles per cell, particle counts
log-uniform in 10k-500k (about 40.7M particles in total, 59M nodes), platen
speed U(1, 10) m/s per specimen, von Mises hardening steel (E 200 GPa, nu 0.3,
rho 7850, yield 250 MPa, H 2 GPa), fixed floor with Coulomb friction 0.1.
The chosen form (FP32 transfers and grid, FP64 positions and energies, the
batch in one engine, autotuned launch shapes) is timed against the plain FP64
form run the reference's way, one specimen per engine; the batched FP64 rate
is reported beside it.  "--workload block" is the single J2 block crushed by a
platen (0.08 x 0.08 x 0.04 m, h = 1 mm, 2,074,896 particles).

One particle-update = one particle advanced through one full step.  Inputs are
synthetic (seeded generators), resident in HBM and larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--form fp64|fp32]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path has no exchange step); value = all ranks' updates / max rank time.
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
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-updates/s on 1 GB300: chosen vs plain FP64 GPU at <=1% stress err"
UNIT = "particle-updates/s"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

# Algorithmic bytes per particle-update per sweep (plain FP64 / FP32 transfers),
# fields read and written once per sweep, shape weights recomputed.
ALG_BYTES = {
    "fp64": {"p2g": 136, "pass1_remap": 80, "pass2": 532},
    "fp32": {"p2g": 80, "pass1_remap": 52, "pass2": 324},
}
# Grid bytes per active node of each sweep: P2G writes mass, momentum and force
# (7 values), pass 1 + remap reads f and m and writes the remap sum (4 + 3),
# pass 2 reads momentum, velocity and mass (3 + 3 + 1).
ALG_GRID_BYTES = {
    "fp64": {"p2g": 56, "pass1_remap": 56, "pass2": 56},
    "fp32": {"p2g": 28, "pass1_remap": 28, "pass2": 28},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="fp32", choices=["fp64", "fp32"],
                    help="fp32: the chosen form, timed beside the plain FP64 form; fp64: the plain form alone")
    ap.add_argument("--workload", default="batch", choices=["batch", "block", "foam", "bar"])
    ap.add_argument("--accuracy-steps", type=int, default=-1,
                    help="steps of the accuracy leg (chosen form against the plain FP64 form), independent of "
                         "--steps; default: the workload's configured horizon (batch 3000, block 5000, "
                         "foam 10000, bar 2000); 0 skips the leg")
    ap.add_argument("--specimens", type=int, default=256, help="batch workload: specimen count")
    ap.add_argument("--total", type=float, default=40.0e6, help="batch workload: target particle count")
    ap.add_argument("--block", default="0.08,0.08,0.04", help="block workload: block size in m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain FP64 form beside the chosen one")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cell-sort", type=int, default=-1, choices=(-1, 0, 1),
                    help="FP32 form: 1 sorts the particles by cell every step, 0 takes the storage order "
                         "(the engine's default when -1)")
    ap.add_argument("--host-scenes", action="store_true",
                    help="build the cellular scene bodies with numpy on the host (as the reference arm does) instead "
                         "of on the GPU; the particles are the same bit for bit")
    ap.add_argument("--no-network", action="store_true",
                    help="run the chosen form without the learned return map (and skip its isolated benchmark)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[5 + j].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def workload(args):
    """(specimen states, config record).  One state for the block workload."""
    from code_mpm_gb300 import scenes

    # the GPU arm builds the cellular bodies on the device (same bits); the reference arm stays on the host
    device = getattr(args, "impl", "gb300") != "reference" and not getattr(args, "host_scenes", False)
    if args.workload == "foam":
        st = scenes.graded_foam(device=device)  # 800 x 800 x 400 cells, 8 x 8 graded cells of 5 mm, platen -20 m/s
        cfg = {"workload": "density-graded square-cell foam crushed by a rigid platen, contact path, single instance",
               "block_m": [0.2, 0.2, 0.1], "h_m": 0.25e-3, "grid_cells": [800, 800, 400],
               "cells_per_side": 8, "pitch_m": 5.0e-3, "wall_m": [0.3e-3, 1.0e-3], "wall_perturbation": 0.1,
               "n_particles": st.n_particles, "n_nodes": st.n_nodes, "platen_speed_mps": 20.0,
               "floor_friction": 0.2, "dt_s": st.dt_max,
               "material": "von Mises hardening aluminium E=70GPa nu=0.33 rho=2700 yield=120MPa H=700MPa",
               "l2_policy": "inputs larger than L2 (~6 GB particle state)"}
        return [st], cfg
    if args.workload == "bar":
        st = scenes.bar()  # 50 x 10 x 10 cells of 1 mm plus one padding cell per side, 8 particles per cell
        cfg = {"workload": "elastic cuboid bar, first-mode vibration, fixed end, non-contact path, single instance",
               "bar_m": [0.05, 0.01, 0.01], "h_m": 1.0e-3, "grid_cells": [int(c) for c in st.cells],
               "particles_per_cell": 8, "n_particles": st.n_particles, "n_nodes": st.n_nodes, "dt_s": st.dt_max,
               "material": "linear elastic E=70GPa nu=0.3 rho=2700", "initial_velocity": "v_x = sin(pi x / 2L) m/s",
               "l2_policy": "inputs smaller than L2 (40,000 particles, ~20 MB): the rate is launch- and "
                            "latency-bound, not a bandwidth figure"}
        return [st], cfg
    if args.workload == "block":
        size = [float(v) for v in args.block.split(",")]
        st = scenes.platen_block(size=size)  # h = 1 mm, 8 ppc, platen -5 m/s, friction 0.1
        cfg = {"workload": "J2 block crushed by rigid platen, contact path", "block_m": size,
               "h_m": 1.0e-3, "particles_per_cell": 8, "n_particles": st.n_particles, "n_nodes": st.n_nodes,
               "material": "von Mises hardening E=200GPa nu=0.3 rho=7850 yield=250MPa H=2GPa",
               "platen_speed_mps": 5.0, "floor_friction": 0.1, "dt_s": st.dt_max,
               "l2_policy": "inputs larger than L2 (~0.8 GB particle state)"}
        return [st], cfg
    sts = scenes.honeycomb_batch(n=args.specimens, total=args.total, device=device)
    counts = [st.n_particles for st in sts]
    cfg = {"workload": f"{len(sts)} square-honeycomb specimens crushed by rigid platens, one grid each, "
                       "contact path, batched in one engine",
           "n_specimens": len(sts), "n_particles": int(sum(counts)), "n_nodes": int(sum(st.n_nodes for st in sts)),
           "particles_per_specimen": [int(min(counts)), int(max(counts))], "h_m": 0.25e-3, "particles_per_cell": 8,
           "wall_m": [0.4e-3, 1.2e-3], "pitch_m": [4.0e-3, 8.0e-3], "cells_per_side": [4, 10],
           "platen_speed_mps": [1.0, 10.0], "floor_friction": 0.1, "dt_s": sts[0].dt_max,
           "material": "von Mises hardening E=200GPa nu=0.3 rho=7850 yield=250MPa H=2GPa",
           "l2_policy": "inputs larger than L2 (~10 GB particle state)"}
    return sts, cfg


def subset(sts, k):
    """k specimens spread over the size distribution (quantiles of the particle count)."""
    if len(sts) <= k:
        return list(range(len(sts)))
    order = sorted(range(len(sts)), key=lambda i: sts[i].n_particles)
    return sorted({order[round(q * (len(sts) - 1) / (k - 1))] for q in range(k)})


def cpu_rate(sts, idx, contact, floor, budget_s, max_steps=50):
    """The CPU restatement (OpenMP, all host threads) over specimens idx: steps until the budget is spent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    threads = os.cpu_count() or 1
    work = [sts[i].copy() for i in idx]
    n = sum(s.n_particles for s in work)
    steps_done, secs = 0, 0.0
    t0 = time.perf_counter()
    while True:
        for s in work:
            secs += pyoracle.advance(s, 1, contact, floor_friction=floor, threads=threads, omp=True)
        steps_done += 1
        if time.perf_counter() - t0 > budget_s or steps_done >= max_steps:
            break
    return n * steps_done / secs, steps_done, secs, n, threads


def cpu_sample(args, sts):
    """(states, indices, description) of the CPU legs' bounded sample: 16 specimens spread over the size range,
    or for the foam a reduced foam of the same generator (its 257M-node grid needs ~60 GB of host memory in the
    CPU restatement)."""
    if getattr(args, "workload", "batch") == "foam":
        from code_mpm_gb300 import scenes

        st = scenes.graded_foam(ncell=2, block=(0.02, 0.02, 0.012), seed=5)
        return [st], [0], f"a reduced foam of the same generator (2 x 2 cells, {st.n_particles} particles)"
    if len(sts) == 1:
        return sts, [0], f"the whole workload ({sts[0].n_particles} particles)"
    idx = subset(sts, 16)
    n = sum(sts[i].n_particles for i in idx)
    return sts, idx, f"{len(idx)} of the {len(sts)} specimens ({n} particles, spread over the size range)"


def cpu_baseline(args, sts, contact, floor, budget_s=12.0):
    sts_, idx, what = cpu_sample(args, sts)
    rate, steps, secs, n, threads = cpu_rate(sts_, idx, contact, floor, budget_s)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} full steps of {what}, OpenMP restatement with per-node locks, {threads} threads, "
                      f"{secs:.2f} s"}


def make_engine(sts, pk, form):
    from code_mpm_gb300 import engine

    if pk is None:
        return engine.Engine.from_state(sts[0], form)
    e = engine.Engine(None, None, form, grids=pk.grids)
    e.upload_state(pk.state)
    return e


def apply_tune(e, tune):
    from code_mpm_gb300 import engine

    if tune:
        # the pair-reduced P2G (modes 5, 6) exists in the FP32 form only; an FP64 engine given such a tuning takes
        # the shared-memory cell runs
        red = tune["p2g_reduce"]
        e.set_option(engine.OPT_P2G_REDUCE, 3 if red >= 5 and e.form == engine.FORM_FP64 else red)
        e.set_option(engine.OPT_P2G_BLOCK, tune["p2g_block"])
        e.set_option(engine.OPT_PASS_BLOCK, tune["pass_block"])
        # the staged pass 2 (mode 2) exists in the FP32 form only; an FP64 engine given an FP32 tuning gathers
        # one corner at a time
        gather = tune["gather_batch"]
        e.set_option(engine.OPT_GATHER, 0 if gather == 2 and e.form == engine.FORM_FP64 else gather)
        e.set_option(engine.OPT_PASS1_CORNERS, tune["pass1_corners"])
        e.set_option(engine.OPT_PASS1_BLOCK, tune["pass1_block"])


def timed(e, steps, warmup, dt, contact, dist):
    """Warm up and time `steps` steps of engine e (CUDA events on its stream); (ms, launches, clocks)."""
    e.advance(warmup, dt, contact)
    e.synchronize()
    dist.barrier()
    clocks = Clocks(dist.local)
    clocks.start()
    time.sleep(0.25)
    l0 = e.launch_count()
    ms = e.advance_timed(steps, dt, contact)
    launches = e.launch_count() - l0
    rec = clocks.stop()
    dist.barrier()
    return dist.max(ms), launches, rec


def plain_per_specimen(sts, args, dist, contact, floor, steps):
    """The plain FP64 form run the reference's way: one engine per specimen, launched one after the other."""
    from code_mpm_gb300 import engine

    big = max(range(len(sts)), key=lambda i: sts[i].n_particles)
    with engine.Engine.from_state(sts[big], engine.FORM_FP64) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, floor)
        tune = None if args.no_autotune else e.autotune(steps=2, dt=sts[big].dt_max, contact=bool(contact))
    dist.barrier()
    clocks = Clocks(dist.local)
    clocks.start()
    ms, launches, n_upd = 0.0, 0, 0
    for st in sts:
        with engine.Engine.from_state(st, engine.FORM_FP64) as e:
            e.set_option(engine.OPT_FLOOR_FRICTION, floor)
            apply_tune(e, tune)
            e.advance(min(args.warmup, 3), st.dt_max, contact)
            l0 = e.launch_count()
            ms += e.advance_timed(steps, st.dt_max, contact)
            launches += e.launch_count() - l0
            n_upd += st.n_particles * steps
    rec = clocks.stop()
    ms = dist.max(ms)
    return {"value": n_upd * dist.world / (ms / 1e3), "ms_per_step": ms / steps, "steps": steps, "dtype": "f64",
            "gpu_launches": launches, "clocks": rec, "autotune": tune,
            "how": f"one FP64 engine per specimen, {steps} timed steps each after warm-up, device times summed "
                   "over specimens (engine creation and upload excluded); launch shapes autotuned on the "
                   "largest specimen"}


ACC_FIELDS = {"pos": 3, "vel": 3, "stress": 6, "e_strain": 1, "e_plastic": 1}
ACC_STEPS = {"batch": 3000, "block": 5000, "foam": 10000, "bar": 2000}


def download_fields(e, n, names=ACC_FIELDS):
    import numpy as np

    out = {k: np.empty((n, c) if c > 1 else (n,), dtype=np.float64) for k, c in names.items()}
    e.download_particles(out)
    return out


def perturbed(st, rel, seed=1):
    """A copy of st with every particle position scaled by 1 + U(-rel, rel)."""
    import numpy as np

    s = st.copy()
    rng = np.random.Generator(np.random.PCG64(seed))
    s["pos"][:] *= 1.0 + rng.uniform(-rel, rel, size=s["pos"].shape)
    return s


def energy_mask(st, contact):
    """The particles whose energy is counted: all but the displacement-controlled platen."""
    import numpy as np

    from code_mpm_gb300 import snapshot

    if contact:
        return (st["pflags"] & snapshot.PF_DC_SKIP) == 0
    m = np.ones(st.n_particles, dtype=bool)
    m[st["dc_list"].astype(np.int64)] = False
    return m


def accuracy_leg(states, what, steps, contact, floor, tune, net, cell_sort=-1):
    """The chosen form (launch shapes, FP64 fallback and network as timed) against the plain FP64 form on the same
    specimens for `steps` steps: von Mises stress errors per specimen in two norms, and the FP64 energy balance
    (kinetic + strain energy against the boundary work) at six checkpoints.  conditioning floor: the plain FP64
    form against itself with positions perturbed by 1e-7 relative (the size of an FP32 rounding)."""
    import numpy as np

    from code_mpm_gb300 import batch, engine, metrics

    pk = batch.pack(states) if len(states) > 1 else None
    src = pk.state if pk is not None else states[0]
    grids = pk.grids if pk is not None else [(src.length, src.cells)]
    poff = pk.particle_offsets if pk is not None else np.array([0, src.n_particles], dtype=np.int64)
    n, dt = src.n_particles, src.dt_max
    mask = energy_mask(src, contact)
    e0 = float(0.5 * np.sum(src["mass"][mask] * np.sum(src["vel"][mask] ** 2, axis=1)) +
               np.sum(src["e_strain"][mask]))
    checkpoints = sorted({max(1, round(steps * k / 6)) for k in range(1, 7)})

    def run(form, state, with_net):
        e = engine.Engine(None, None, form, grids=grids)
        e.upload_state(state)
        e.set_option(engine.OPT_FLOOR_FRICTION, floor)
        apply_tune(e, tune)
        if form == engine.FORM_FP32 and cell_sort >= 0:
            e.set_option(engine.OPT_CELL_SORT, cell_sort)
        if form == engine.FORM_FP32 and with_net and net is not None:
            e.attach_surrogate(net, band=0.02, recheck=0.01)
        e.upload_monitor_mask(mask.astype(np.uint8) * engine.MON_ENERGY)
        series, done = [], 0
        for c in checkpoints:
            e.advance(c - done, dt, contact)
            done = c
            m = e.monitors()
            en = m["kinetic"] + m["strain_energy"]
            series.append({"step": c, "kinetic": m["kinetic"], "strain_energy": m["strain_energy"],
                           "plastic_energy": m["plastic_energy"], "platen_work": m["platen_work"],
                           "friction_work": m["friction_work"],
                           "residual": en - e0 - m["platen_work"] - m["friction_work"]})
        out = download_fields(e, n)
        sg = e.surrogate_stats() if (form == engine.FORM_FP32 and with_net and net is not None) else None
        e.close()
        return out, series, sg

    t0 = time.perf_counter()
    chosen, ser_c, sg = run(engine.FORM_FP32, src, True)
    plain, ser_p, _ = run(engine.FORM_FP64, src, False)
    pert, ser_f, _ = run(engine.FORM_FP64, perturbed(src, 1e-7), False)
    nonet = run(engine.FORM_FP32, src, False) if net is not None else None
    secs = time.perf_counter() - t0

    def cut(d, i):
        return {k: v[poff[i]:poff[i + 1]] for k, v in d.items()}

    per, floor_per = [], []
    for i in range(len(poff) - 1):
        per.append(dict(metrics.form_errors(cut(chosen, i), cut(plain, i)), specimen=i,
                        n_particles=int(poff[i + 1] - poff[i])))
        floor_per.append(metrics.form_errors(cut(pert, i), cut(plain, i)))
    keys = ("vm_stress_rel_l2", "vm_stress_rel", "strain_energy_rel", "plastic_energy_rel", "pos_abs_max",
            "vel_rel")
    worst = {k: max(p[k] for p in per) for k in keys}

    def total(r):
        return r["kinetic"] + r["strain_energy"]

    def drift(a, b):
        return abs(total(a) - total(b)) / abs(total(b)) if total(b) != 0 else abs(total(a))

    scale = max(abs(ser_p[-1]["platen_work"]) + abs(ser_p[-1]["friction_work"]), abs(e0), 1e-300)
    energy = {
        "energy_drift_rel": drift(ser_c[-1], ser_p[-1]),
        "energy_drift_rel_series": [drift(a, b) for a, b in zip(ser_c, ser_p)],
        "work_rel": (abs(ser_c[-1]["platen_work"] - ser_p[-1]["platen_work"]) / abs(ser_p[-1]["platen_work"])
                     if ser_p[-1]["platen_work"] != 0 else None),
        "balance_residual_rel": {"chosen": ser_c[-1]["residual"] / scale, "plain_fp64": ser_p[-1]["residual"] / scale},
        "conditioning_floor_energy_drift_rel": drift(ser_f[-1], ser_p[-1]),
        "initial_energy": e0,
        "series": {"chosen": ser_c, "plain_fp64": ser_p},
        "definition": "E = kinetic + strain energy of the specimen particles (the platen excluded); the strain "
                      "energy is the stress work, plastic dissipation included.  energy_drift_rel = "
                      "|E_chosen - E_plain| / |E_plain| at the last checkpoint; balance residual = E - E_0 - "
                      "platen work - friction work (FP64 sums on the device), over the boundary work",
    }
    without_network = None
    if nonet is not None:  # the FP32 form alone: how much of the error is the network's
        errs = [metrics.form_errors(cut(nonet[0], i), cut(plain, i)) for i in range(len(poff) - 1)]
        without_network = {k: max(e[k] for e in errs) for k in keys}
        without_network["energy_drift_rel"] = drift(nonet[1][-1], ser_p[-1])
    bars = {"vm_stress_rel_l2": 1e-2, "energy_drift_rel": 5e-3}
    got = {"vm_stress_rel_l2": worst["vm_stress_rel_l2"], "energy_drift_rel": energy["energy_drift_rel"]}
    return dict(worst, steps=steps, specimens=per, energy=energy, bars=bars,
                bar_norms="the stress bar is the relative L2 norm of the von Mises stress over each specimen's "
                          "particles (worst specimen); the max-norm (vm_stress_rel) is reported beside the "
                          "conditioning floor, the same FP64 run perturbed by 1e-7",
                within_bars=all(got[k] <= v for k, v in bars.items()),
                conditioning_floor={k: max(p[k] for p in floor_per) for k in keys},
                network_in_run=sg, without_network=without_network, seconds=secs,
                versus=f"plain FP64 GPU form (itself within 1e-9 of the FP64 oracle) on {what}, same steps; "
                       "worst over the specimens")


def peaks_bf16():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


# algorithmic FLOPs of one sample through 13 -> 128 -> 128 -> 128 -> 7
NET_FLOPS = 2 * (13 * 128 + 128 * 128 + 128 * 128 + 128 * 7)


def harvest_run(e, rows, cap, steps, dt, contact, every=4):
    """Advance engine e by `steps` steps, recording the return-map inputs of every plastic von Mises hardening
    particle in one step out of `every` into the device rows (n x 13), up to cap rows; returns the rows written.
    Sampling the whole run keeps its late states in the training set."""
    n, done = 0, 0
    while done < steps:
        k = min(every - 1, steps - done)
        if k:
            e.advance(k, dt, contact)
            done += k
        if done >= steps:
            break
        if n < cap:
            e.harvest_begin(rows.data_ptr() + 4 * 13 * n, cap - n, mat_mask=1, band=0.0)
            e.advance(1, dt, contact)
            n += min(e.harvest_end(), cap - n)
        else:
            e.advance(1, dt, contact)
        done += 1
    return n


def deps_scale(rows, n):
    """Input scale of the strain increments: the standard deviation, raised so that the largest increments
    (the 99.9th percentile of |de| over a sample of the rows) sit within three scales."""
    import torch

    d = rows[:n, 7:]
    std = float(d.std().item())
    sample = d[torch.randint(0, n, (min(n, 200_000),), device=d.device)].abs().flatten()
    return max(std, float(torch.quantile(sample, 0.999).item()) / 3.0)


def network_for_batch(args, contact, floor, steps):
    """The learned return map for the batch: trained on the return-map inputs that the plain FP64 method meets on
    a pilot batch (16 other specimens drawn with another seed), labelled by the exact FP64 map."""
    import torch

    from code_mpm_gb300 import batch, engine, scenes

    pilot = scenes.honeycomb_batch(n=16, seed=99, total=2.5e6)
    ppk = batch.pack(pilot)
    cap = 16_000_000
    rows = torch.zeros((cap, 13), dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    e = engine.Engine(None, None, engine.FORM_FP64, grids=ppk.grids)
    e.upload_state(ppk.state)
    e.set_option(engine.OPT_FLOOR_FRICTION, floor)
    n = harvest_run(e, rows, cap, steps, pilot[0].dt_max, contact)
    e.close()
    t1 = time.perf_counter()
    dsig = deps_scale(rows, n)
    bsz = 8192
    epochs = int(max(20, math.ceil(5000 * bsz / max(n, 1))))  # about 5000 Adam steps
    net = engine.Net(E=200.0e9, nu=0.3, yield_=250.0e6, C0=2.0e-3, C1=1.0e12, n_samples=1000, epochs=epochs,
                     batch=bsz, deps_sigma=dsig, lr=4.0e-3)
    rep = net.train_rows(rows.data_ptr(), n)
    del rows
    info = {"pilot": f"16 honeycomb specimens (seed 99, {ppk.state.n_particles} particles), plain FP64, {steps} steps "
                     "(inputs of one step in four)",
            "harvested_rows": n, "seconds_pilot": t1 - t0, "training": rep}
    return net, info


def network_for_foam(args, contact, floor, steps):
    """The learned return map for the foam's aluminium: trained on the return-map inputs the plain FP64 method
    meets on a reduced foam (2 x 2 cells, another seed)."""
    import torch

    from code_mpm_gb300 import engine, scenes

    pilot = scenes.graded_foam(ncell=2, block=(0.02, 0.02, 0.012), seed=9)
    cap = 8_000_000
    rows = torch.zeros((cap, 13), dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    with engine.Engine.from_state(pilot, engine.FORM_FP64) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, floor)
        n = harvest_run(e, rows, cap, steps, pilot.dt_max, contact)
    t1 = time.perf_counter()
    dsig = deps_scale(rows, n)
    bsz = 8192
    epochs = int(max(20, math.ceil(5000 * bsz / max(n, 1))))
    net = engine.Net(E=70.0e9, nu=0.33, yield_=120.0e6, C0=700.0e6 / 1.0e12, C1=1.0e12, n_samples=1000,
                     epochs=epochs, batch=bsz, deps_sigma=dsig, lr=4.0e-3)
    rep = net.train_rows(rows.data_ptr(), n)
    return net, {"pilot": f"reduced foam 2 x 2 cells (seed 9, {pilot.n_particles} particles), plain FP64, "
                          f"{steps} steps (inputs of one step in four)", "harvested_rows": n, "seconds_pilot": t1 - t0, "training": rep}


def network_isolated(contact_unused=None):
    """The network as stated for the isolated return map: 20M samples (stress U(+-1.5 yield), R from epbar
    U(0, 0.2), strain increment N(0, 2e-4)), batch 65536, 20 epochs; inference on 16M samples per call (tensor cores)
    against the exact FP32 map on the same samples."""
    import torch

    from code_mpm_gb300 import engine

    net = engine.Net(E=200.0e9, nu=0.3, yield_=250.0e6, C0=2.0e-3, C1=1.0e12, n_samples=20_000_000, epochs=20,
                     batch=65536, lr=4.0e-3)
    rep = net.train()
    n = 16 * 1024 * 1024
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    Y = 250.0e6
    x = torch.empty((n, 13), dtype=torch.float32, device="cuda")
    x[:, :6] = (torch.rand((n, 6), generator=g, device="cuda") * 3.0 - 1.5) * Y
    ep = torch.rand((n,), generator=g, device="cuda") * 0.2
    x[:, 6] = (math.sqrt(2.0 / 3.0) * 1.0e12 * (1.0 - torch.exp(-2.0e-3 * ep.double()))).float()
    x[:, 7:] = torch.randn((n, 6), generator=g, device="cuda") * 2.0e-4
    out = torch.empty((n, 7), dtype=torch.float32, device="cuda")
    times = {}
    for name, k in (("network_tcgen05", engine.INFER_TC), ("exact_map_fp32", engine.INFER_EXACT)):
        for _ in range(3):
            net.infer_device(x.data_ptr(), out.data_ptr(), n, k)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(10):
            net.infer_device(x.data_ptr(), out.data_ptr(), n, k)
        b.record()
        b.synchronize()
        times[name] = a.elapsed_time(b) / 10
    peak, kind = peaks_bf16()
    achieved = NET_FLOPS * n / (times["network_tcgen05"] / 1e3) / 1e12
    net.close()
    return {"samples_per_call": n, "ms_per_call": times,
            "samples_per_s": {k: n / (v / 1e3) for k, v in times.items()},
            "network_over_exact_speed": times["exact_map_fp32"] / times["network_tcgen05"],
            "roofline": {"bound": "tensor", "kernel": "k_mlp_tc", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak, "peak_kind": f"{kind} cuBLAS bf16 burst",
                         "flops_per_sample": NET_FLOPS},
            "training": rep}


def kernel_table(e, steps, dt, contact):
    from code_mpm_gb300 import engine

    e.set_option(engine.OPT_PROFILE, 1)
    e.profile_reset()
    e.advance(steps, dt, contact)
    prof = e.profile()
    e.set_option(engine.OPT_PROFILE, 0)
    total = sum(v["ms"] for v in prof.values())
    kernels = {k: {"launches": v["launches"], "avg_us": 1e3 * v["ms"] / max(1, v["launches"]),
                   "share": v["ms"] / total if total else 0.0} for k, v in prof.items()}
    return prof, kernels


def active_nodes(e, n_nodes):
    import numpy as np

    from code_mpm_gb300 import engine

    state = np.zeros(n_nodes, dtype=np.uint8)
    nd = engine.Nodes(state=state.ctypes.data)
    e._check(e._L.mpm_download_nodes(e._h, engine.C.byref(nd)))
    return int(np.count_nonzero(state & 1))


def roofline_of(prof, formkey, n, n_active, workload_name):
    hbm, peak_kind = peaks()
    alg, galg = ALG_BYTES[formkey], ALG_GRID_BYTES[formkey]
    top = max(prof.items(), key=lambda kv: kv[1]["ms"])[0]
    dom = top if top in alg else max(alg, key=lambda k: prof.get(k, {"ms": 0})["ms"])
    tj = {}
    tfile = os.path.join(ROOT, "profiles", f"traffic_{workload_name}_{formkey}.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            tj = json.load(f)
    per = {}
    for k in alg:
        if k not in prof or not prof[k]["launches"]:
            continue
        avg_s = prof[k]["ms"] / prof[k]["launches"] / 1e3
        bytes_ = alg[k] * n + galg[k] * n_active
        per[k] = {"achieved": bytes_ / avg_s / 1e9, "frac": bytes_ / avg_s / 1e9 / hbm, "avg_us": avg_s * 1e6,
                  "alg_bytes": bytes_,
                  "traffic": tj[k]["bytes_per_particle"] * n if k in tj else None}
    d = per[dom]
    return {"bound": "hbm", "kernel": dom, "achieved": d["achieved"], "peak": hbm, "unit": "GB/s",
            "frac": d["frac"], "traffic": d["traffic"], "peak_kind": f"{peak_kind} copy bandwidth",
            "alg_bytes_per_launch": d["alg_bytes"],
            "alg_bytes_formula": f"{alg[dom]} B x particles + {galg[dom]} B x active nodes",
            "n_active_nodes": n_active, "top_kernel_by_time": top, "per_kernel": per}


def e2e_leg(e, pk, sts, n, k_e2e, dt, contact, dist):
    """The drop-in call with host buffers: H2D of the full particle state from pinned memory, k steps, D2H of the
    full particle state, on one stream, timed with CUDA events."""
    import torch

    src = pk.state if pk is not None else sts[0]
    fields = {"pos": 3, "vel": 3, "fext": 3, "mass": 1, "vol": 1, "vol0": 1, "F": 9, "stress": 6, "strain": 6,
              "eps_p": 6, "e_strain": 1, "e_strain_max": 1, "e_strain_ti": 1, "e_plastic": 1, "backstress": 1,
              "mp_mass_gradient": 3, "strain_rate": 6}
    host = {}
    for k, c in fields.items():
        t = torch.empty((n, c) if c > 1 else (n,), dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = src[k]
        host[k] = t
    for k, dt_ in (("material", torch.int32), ("pflags", torch.uint8), ("dc_mult", torch.float32)):
        t = torch.empty((n,), dtype=dt_, pin_memory=True)
        t.numpy()[...] = src[k]
        host[k] = t
    views = {k: v.numpy() for k, v in host.items()}
    if pk is not None:
        t = torch.empty((n,), dtype=torch.int32, pin_memory=True)
        t.numpy()[...] = pk.state["specimen"]
        host["specimen"] = t
        views["specimen"] = t.numpy()
    stream = torch.cuda.Stream()
    e.set_stream(stream.cuda_stream)
    h2d = sum(v.nbytes for v in views.values())
    outs = {k: views[k] for k in fields}
    d2h = sum(v.nbytes for v in outs.values())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    e.upload_particles(views, n)
    e.advance(k_e2e, dt, contact)
    e.download_particles(outs)
    ev1.record(stream)
    ev1.synchronize()
    ms = dist.max(ev0.elapsed_time(ev1))
    return {"value": n * k_e2e * dist.world / (ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d / k_e2e,
            "d2h_bytes_per_step": d2h / k_e2e, "steps_per_call": k_e2e,
            "how": "one drop-in call: H2D of the full particle state from pinned host memory, "
                   f"{k_e2e} steps, D2H of the full particle state; CUDA events on the call's stream"}


def run_gb300(args, dist: Dist):
    from code_mpm_gb300 import batch, build, engine

    if dist.rank == 0 or not os.path.exists(build.LIB):
        build.build()
    dist.barrier()
    sts, cfg = workload(args)
    pk = batch.pack(sts) if len(sts) > 1 else None
    # the bar vibrates freely on the non-contact path; the other workloads are platen crushes on the contact path
    contact, floor = (0, 0) if args.workload == "bar" else (1, 1)
    n = sum(st.n_particles for st in sts)
    n_nodes = sum(st.n_nodes for st in sts)
    dt = sts[0].dt_max
    chosen_form = engine.FORM_FP64 if args.form == "fp64" else engine.FORM_FP32
    formkey = "fp64" if chosen_form == engine.FORM_FP64 else "fp32"
    compare = chosen_form != engine.FORM_FP64 and not args.no_plain

    # plain FP64 form: the reference method on the GPU (parity-pinned to the oracle)
    plain, plain_batched = None, None
    if compare and pk is not None:
        plain = plain_per_specimen(sts, args, dist, contact, floor, steps=max(1, min(args.steps, 20)))
        with make_engine(sts, pk, engine.FORM_FP64) as ep:
            ep.set_option(engine.OPT_FLOOR_FRICTION, floor)
            tune_b = None if args.no_autotune else ep.autotune(steps=2, dt=dt, contact=bool(contact))
            kb = max(1, min(args.steps, 20))
            ms_b, launches_b, clocks_b = timed(ep, kb, args.warmup, dt, contact, dist)
        plain_batched = {"value": n * kb * dist.world / (ms_b / 1e3), "ms_per_step": ms_b / kb, "steps": kb,
                         "dtype": "f64", "gpu_launches": launches_b, "clocks": clocks_b, "autotune": tune_b,
                         "how": "the plain FP64 form with every specimen in one engine"}

    # the learned return map (chosen form, batch workload): trained on a pilot batch's plain-method samples
    net, net_info = None, None
    use_net = compare and not args.no_network and args.workload in ("batch", "foam")
    acc_steps = ACC_STEPS[args.workload] if args.accuracy_steps < 0 else args.accuracy_steps
    if use_net:
        # the pilot covers every state the network will serve: the timed steps and the accuracy horizon
        pilot_steps = max(args.warmup + args.steps, acc_steps)
        if args.workload == "foam":
            net, net_info = network_for_foam(args, contact, floor, steps=pilot_steps)
        else:
            net, net_info = network_for_batch(args, contact, floor, steps=pilot_steps)

    e = make_engine(sts, pk, chosen_form)
    e.set_option(engine.OPT_FLOOR_FRICTION, floor)
    if args.cell_sort >= 0:
        e.set_option(engine.OPT_CELL_SORT, args.cell_sort)
    if net is not None:
        e.attach_surrogate(net, band=0.02, recheck=0.01)
    tune = None if args.no_autotune else e.autotune(steps=2, dt=dt, contact=bool(contact))
    if net is not None:
        e.surrogate_stats(reset=True)
    ms, launches, clocks_rec = timed(e, args.steps, args.warmup, dt, contact, dist)
    value = n * args.steps * dist.world / (ms / 1e3)
    if net is not None:
        net_info["in_step"] = e.surrogate_stats()

    accuracy = None
    if compare:
        if acc_steps > 0:
            if args.workload == "foam":
                from code_mpm_gb300 import scenes

                red = scenes.graded_foam(ncell=2, block=(0.02, 0.02, 0.012), seed=5)
                acc_states = [red]
                what = f"a reduced foam of the same generator (2 x 2 cells, {red.n_particles} particles)"
            elif pk is not None:
                idx = subset(sts, 8)
                acc_states = [sts[i] for i in idx]
                what = (f"{len(idx)} of the {len(sts)} specimens spread over the size range "
                        f"({sum(s.n_particles for s in acc_states)} particles), batched in both forms")
            else:
                acc_states = sts
                what = f"the workload itself ({n} particles)"
            accuracy = accuracy_leg(acc_states, what, acc_steps, contact, floor, tune, net, args.cell_sort)
        if pk is None:  # single instance: the plain form timed on the same state (fewer steps for the foam)
            kp = args.steps if args.workload in ("block", "bar") else max(1, min(args.steps, 20))
            with make_engine(sts, pk, engine.FORM_FP64) as ep:
                ep.set_option(engine.OPT_FLOOR_FRICTION, floor)
                tune_p = None if args.no_autotune else ep.autotune(steps=2, dt=dt, contact=bool(contact))
                ms_p, launches_p, clocks_p = timed(ep, kp, min(args.warmup, 3), dt, contact, dist)
            plain = {"value": n * kp * dist.world / (ms_p / 1e3), "ms_per_step": ms_p / kp,
                     "steps": kp, "dtype": "f64", "gpu_launches": launches_p, "clocks": clocks_p,
                     "autotune": tune_p}

    prof_steps = min(args.steps, 30)
    prof, kernels = kernel_table(e, prof_steps, dt, contact)
    # launch gaps: the kernels' own time (each launch bracketed by events, graph off) against the graph-replayed step
    kernel_ms = sum(v["ms"] for v in prof.values()) / prof_steps
    launch_gaps = {"kernel_ms_per_step": kernel_ms, "step_ms": ms / args.steps,
                   "busy_fraction": kernel_ms / (ms / args.steps),
                   "launches_per_step": sum(v["launches"] for v in prof.values()) / prof_steps,
                   "how": f"sum of per-kernel CUDA-event times over {prof_steps} profiled steps (graph off) per step, "
                          "over the timed step (graph replay)"}
    n_active = active_nodes(e, n_nodes)
    roofline = roofline_of(prof, formkey, n, n_active, args.workload)
    without_net = None
    if net is not None:  # the same engine with the network detached
        e.attach_surrogate(None)
        k2 = max(1, min(args.steps, 300))
        ms2, l2, c2 = timed(e, k2, 2, dt, contact, dist)
        without_net = {"value": n * k2 * dist.world / (ms2 / 1e3), "ms_per_step": ms2 / k2, "steps": k2,
                       "gpu_launches": l2}
        e.attach_surrogate(net, band=0.02, recheck=0.01)  # the e2e call runs the chosen form as timed

    e2e = None
    if args.no_e2e:
        e2e = {"value": None, "unit": UNIT, "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
               "error": "skipped (--no-e2e)"}
    else:
        try:
            e2e = e2e_leg(e, pk, sts, n, max(1, min(args.steps, 50)), dt, contact, dist)
        except Exception as ex:  # reported, not hidden
            e2e = {"value": None, "unit": UNIT, "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                   "error": f"{type(ex).__name__}: {ex}"}
    e.close()

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if formkey == "fp64" else "f32+f64",
           "data": "synthetic (seeded scene generators)",
           "config": dict(cfg, form=("plain FP64" if formkey == "fp64" else "chosen: FP32 transfers/grid, FP64 "
                                     "positions and energies, batched, autotuned" +
                                     (", learned return map with 2% fallback band and 1% recheck" if use_net
                                      else "")),
                          parallelism=f"replicas x{dist.world}"),
           "clocks": clocks_rec, "gpu_launches": launches, "autotune": tune, "roofline": roofline,
           "kernels": kernels, "launch_gaps": launch_gaps, "e2e": e2e}
    if plain is not None:
        out["plain_fp64"] = plain
        out["chosen_over_plain"] = value / plain["value"]
    if plain_batched is not None:
        out["plain_fp64_batched"] = plain_batched
        out["chosen_over_plain_batched"] = value / plain_batched["value"]
    if accuracy is not None:
        out["accuracy"] = accuracy
    if net_info is not None:
        out["network"] = net_info
        out["chosen_without_network"] = without_net
        net.close()
    if dist.rank == 0 and dist.world == 1 and use_net:
        out["network_isolated"] = network_isolated()
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, sts, contact, floor)
    return out


def run_reference(args, dist: Dist):
    """The reference's CPU implementation of the path (the restatement of it), all host threads, on a bounded
    sample of the workload: the same specimens every step, steps capped to about two minutes."""
    if dist.rank != 0:
        return None
    sts, cfg = workload(args)
    sts_, idx, what = cpu_sample(args, sts)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    threads = os.cpu_count() or 1
    work = [sts_[i].copy() for i in idx]
    n = sum(s.n_particles for s in work)
    contact, floor = (0, 0) if args.workload == "bar" else (1, 1)

    def step():
        return sum(pyoracle.advance(s, 1, contact, floor_friction=floor, threads=threads, omp=True) for s in work)

    # warm-up as asked (each step is a bounded sample); timed steps as asked unless they would pass two minutes
    w = max(1, args.warmup)
    t0 = time.perf_counter()
    for _ in range(w):
        step()
    one = (time.perf_counter() - t0) / w
    k = max(1, min(args.steps, int(120.0 / max(one, 1e-3))))
    secs = sum(step() for _ in range(k))
    rate = n * k / secs
    sample = (f"{k} timed steps (+{w} warm-up) of {what}; CPU restatement of the reference path, OpenMP with "
              f"per-node locks, {threads} threads")
    return {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": dist.world, "steps": k, "warmup": w,
            "ms_per_step": 1e3 * secs / k, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded scene generators)", "config": dict(cfg, form="reference-cpu"),
            "impl": "reference",
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    dist = Dist()
    try:
        out = run_reference(args, dist) if args.impl == "reference" else run_gb300(args, dist)
        if out is not None and dist.rank == 0:
            print(json.dumps(out))
            sys.stdout.flush()
    finally:
        dist.close()


if __name__ == "__main__":
    main()
