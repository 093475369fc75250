#!/usr/bin/env python
"""Benchmark: particle-updates/s of the explicit-MPM double-pass step on GB300.

Workload: the J2 block crushed by a rigid platen on the contact path (the
configuration the headline metric is quoted on): block 0.08 x 0.08 x 0.04 m,
h = 1 mm, 8 particles per cell (2,048,000 block particles) plus a one-layer
platen (26,896 particles) moving at -5 m/s, von Mises hardening steel
(E 200 GPa, nu 0.3, rho 7850, yield 250 MPa, H 2 GPa), fixed floor with
Coulomb friction 0.1.  One particle-update = one particle advanced through
one full step; a step is one pass of every kernel of the step over the
whole particle set.  Inputs are synthetic (seeded generators), resident in
HBM and larger than L2 (~0.8 GB of particle state).

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
    "fp64": {"p2g": 136, "pass1_remap": 80, "pass2": 580},
    "fp32": {"p2g": 80, "pass1_remap": 52, "pass2": 348},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="fp32", choices=["fp64", "fp32"],
                    help="fp32: the chosen form, timed beside the plain FP64 form; fp64: the plain form alone")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain FP64 form beside the chosen one")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--block", default="0.08,0.08,0.04",
                    help="block size in m (smaller blocks only for profiling captures; the metric uses the default)")
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


def workload(block="0.08,0.08,0.04"):
    from code_mpm_gb300 import scenes

    size = [float(v) for v in block.split(",")]
    st = scenes.platen_block(size=size)  # default 0.08 x 0.08 x 0.04 m, h = 1 mm, 8 ppc, platen -5 m/s, friction 0.1
    cfg = {"workload": "J2 block crushed by rigid platen, contact path", "block_m": size,
           "h_m": 1.0e-3, "particles_per_cell": 8, "n_particles": st.n_particles, "n_nodes": st.n_nodes,
           "material": "von Mises hardening E=200GPa nu=0.3 rho=7850 yield=250MPa H=2GPa",
           "platen_speed_mps": 5.0, "floor_friction": 0.1, "dt_s": st.dt_max,
           "l2_policy": "inputs larger than L2 (~0.8 GB particle state)"}
    return st, cfg


def cpu_baseline(st, contact: int, floor_friction: int, budget_s: float = 12.0):
    """The CPU restatement (OpenMP, all host threads) on a bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    threads = os.cpu_count() or 1
    s = st.copy()
    steps_done, secs = 0, 0.0
    t0 = time.perf_counter()
    while True:
        secs += pyoracle.advance(s, 1, contact, floor_friction=floor_friction, threads=threads, omp=True)
        steps_done += 1
        if time.perf_counter() - t0 > budget_s or steps_done >= 50:
            break
    rate = st.n_particles * steps_done / secs
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps_done} full steps of the same workload ({st.n_particles} particles), "
                      f"OpenMP restatement with per-node locks, {threads} threads, {secs:.2f} s"}


def timed_form(st, form, args, dist, contact, floor, tune=True):
    """Autotune, warm up and time one form on `st`; returns (engine, ms, launches, clocks, tune result)."""
    from code_mpm_gb300 import engine

    e = engine.Engine.from_state(st, form)
    e.set_option(engine.OPT_FLOOR_FRICTION, floor)
    dt = st.dt_max
    tune_res = e.autotune(steps=2, dt=dt, contact=bool(contact)) if (tune and not args.no_autotune) else None
    e.advance(args.warmup, dt, contact)
    e.synchronize()
    dist.barrier()
    clocks = Clocks(dist.local)
    clocks.start()
    time.sleep(0.25)
    l0 = e.launch_count()
    ms = e.advance_timed(args.steps, dt, contact)
    launches = e.launch_count() - l0
    rec = clocks.stop()
    dist.barrier()
    return e, dist.max(ms), launches, rec, tune_res


def run_gb300(args, dist: Dist):
    from code_mpm_gb300 import build, engine, metrics

    if dist.rank == 0 or not os.path.exists(build.LIB):
        build.build()
    dist.barrier()
    st, cfg = workload(args.block)
    contact, floor = 1, 1
    n = st.n_particles
    dt = st.dt_max
    chosen_form = engine.FORM_FP64 if args.form == "fp64" else engine.FORM_FP32

    # plain FP64 form: the reference method on the GPU (parity-pinned to the oracle)
    plain = None
    plain_state = None
    if chosen_form != engine.FORM_FP64 and not args.no_plain:
        ep, ms_p, launches_p, clocks_p, tune_p = timed_form(st, engine.FORM_FP64, args, dist, contact, floor)
        plain_state = ep.download_state(st)
        ep.close()
        plain = {"value": n * args.steps * dist.world / (ms_p / 1e3), "ms_per_step": ms_p / args.steps,
                 "dtype": "f64", "gpu_launches": launches_p, "clocks": clocks_p, "autotune": tune_p}

    e, ms, launches, clocks_rec, tune = timed_form(st, chosen_form, args, dist, contact, floor)
    value = n * args.steps * dist.world / (ms / 1e3)
    accuracy = None
    if plain_state is not None:
        err = metrics.form_errors(e.download_state(st), plain_state)
        accuracy = dict(err, steps=args.warmup + args.steps,
                        versus="plain FP64 GPU form after the same steps (itself within 1e-9 of the FP64 oracle)",
                        bars={"vm_stress_rel": 1e-2, "strain_energy_rel": 5e-3})

    # per-kernel device times (CUDA events on the engine's stream), separate pass
    kprof = min(args.steps, 30)
    e.set_option(engine.OPT_PROFILE, 1)
    e.profile_reset()
    e.advance(kprof, dt, contact)
    prof = e.profile()
    e.set_option(engine.OPT_PROFILE, 0)
    total = sum(v["ms"] for v in prof.values())
    kernels = {k: {"launches": v["launches"], "avg_us": 1e3 * v["ms"] / max(1, v["launches"]),
                   "share": v["ms"] / total if total else 0.0} for k, v in prof.items()}
    top = max(prof.items(), key=lambda kv: kv[1]["ms"])[0]
    hbm, peak_kind = peaks()
    formkey = "fp64" if chosen_form == engine.FORM_FP64 else "fp32"
    alg = ALG_BYTES[formkey]
    dom = top if top in alg else max(alg, key=lambda k: prof.get(k, {"ms": 0})["ms"])
    avg_s = prof[dom]["ms"] / prof[dom]["launches"] / 1e3
    achieved = alg[dom] * n / avg_s / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", f"traffic_{formkey}.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            tj = json.load(f)
        if dom in tj:
            traffic = tj[dom]["bytes_per_particle"] * n
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic, "peak_kind": f"{peak_kind} copy bandwidth",
                "alg_bytes_per_particle": alg[dom], "top_kernel_by_time": top}

    # end to end through the C ABI with host buffers: H2D of the particle state,
    # K steps, D2H of the particle state, on one stream, timed with CUDA events.
    e2e = None
    try:
        if args.no_e2e:
            raise RuntimeError("skipped (--no-e2e)")
        import torch

        fields = {"pos": 3, "vel": 3, "fext": 3, "mass": 1, "vol": 1, "vol0": 1, "F": 9, "stress": 6, "strain": 6,
                  "eps_p": 6, "e_strain": 1, "e_strain_max": 1, "e_strain_ti": 1, "e_plastic": 1, "backstress": 1,
                  "mp_mass_gradient": 3, "strain_rate": 6}
        host = {}
        for k, c in fields.items():
            t = torch.empty((n, c) if c > 1 else (n,), dtype=torch.float64, pin_memory=True)
            a = t.numpy()
            a[...] = st[k]
            host[k] = (t, a)
        for k, dt_ in (("material", torch.int32), ("pflags", torch.uint8), ("dc_mult", torch.float32)):
            t = torch.empty((n,), dtype=dt_, pin_memory=True)
            a = t.numpy()
            a[...] = st[k]
            host[k] = (t, a)
        stream = torch.cuda.Stream()
        e.set_stream(stream.cuda_stream)
        k_e2e = max(1, min(args.steps, 50))
        views = {k: v[1] for k, v in host.items()}
        h2d = sum(v.nbytes for v in views.values())
        d2h = sum(views[k].nbytes for k in fields)
        outs = {k: views[k] for k in fields}
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        e.upload_particles(views, n)
        e.advance(k_e2e, dt, contact)
        e.download_particles(outs)
        ev1.record(stream)
        ev1.synchronize()
        e2e_ms = dist.max(ev0.elapsed_time(ev1))
        e2e = {"value": n * k_e2e * dist.world / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d / k_e2e,
               "d2h_bytes_per_step": d2h / k_e2e, "steps_per_call": k_e2e,
               "how": "one drop-in call: H2D of the full particle state from pinned host memory, "
                      f"{k_e2e} steps, D2H of the full particle state; CUDA events on the call's stream"}
    except Exception as ex:  # reported, not hidden
        e2e = {"value": None, "unit": UNIT, "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
               "error": f"{type(ex).__name__}: {ex}"}
    e.close()

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if formkey == "fp64" else "f32+f64",
           "data": "synthetic (seeded scene generator, reference scene conventions)",
           "config": dict(cfg, form=("plain FP64" if formkey == "fp64" else "chosen: FP32 transfers/grid, FP64 "
                                     "positions and energies"), parallelism=f"replicas x{dist.world}"),
           "clocks": clocks_rec, "gpu_launches": launches, "autotune": tune, "roofline": roofline,
           "kernels": kernels, "e2e": e2e}
    if plain is not None:
        out["plain_fp64"] = plain
        out["chosen_over_plain"] = value / plain["value"]
        out["accuracy"] = accuracy
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(st, contact, floor)
    return out


def run_reference(args, dist: Dist):
    """The reference's CPU implementation of the path (the restatement of it), all host threads."""
    if dist.rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    st, cfg = workload(args.block)
    threads = os.cpu_count() or 1
    s = st.copy()
    # bounded: warm-up and timed steps on the full workload, at most ~a few minutes in total
    w = min(args.warmup, 1)
    pyoracle.advance(s, w, 1, floor_friction=1, threads=threads, omp=True)
    one = pyoracle.advance(s, 1, 1, floor_friction=1, threads=threads, omp=True)
    k = max(1, min(args.steps, int(120.0 / max(one, 1e-3))))
    secs = pyoracle.advance(s, k, 1, floor_friction=1, threads=threads, omp=True)
    rate = st.n_particles * k / secs
    sample = (f"{k} timed steps (+{w + 1} warm-up) of the full workload ({st.n_particles} particles); "
              f"CPU restatement of the reference path, OpenMP with per-node locks, {threads} threads")
    return {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": dist.world, "steps": k, "warmup": w + 1,
            "ms_per_step": 1e3 * secs / k, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded scene generator)", "config": dict(cfg, form="reference-cpu"),
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
