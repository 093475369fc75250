"""Times the GPU voxel canvas on a ring-array cross-section like the reference's Shim scenes.

    python -m code_mpm_gb300.canvasbench [--cells N] [--offset M] [--reps R]

An N x N array of rings (outer radius 4.5 mm, inner 3.8 mm, pitch 9.5 mm,
…Shim_Square.cpp:197-214's drawRing per ring) on a canvas of offset M (default
12.5 um: 7,600 x 7,600 = 57.8M voxels for N = 8).  Prints one JSON line: GPU
milliseconds per full drawing pass and per extraction of the active voxels
(centres, ids, surface flags to device memory), voxels per second, and the CPU
restatement (oracle/canvas_oracle.py, numpy, one core) timed on a 1/16 area
sample of the same canvas when the oracle is present (test infrastructure,
timed here only as the CPU baseline).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time


def ring_ops(cells: int):
    pitch, ro, ri = 0.0095, 0.0045, 0.0038
    return [("ring", 0.005 + pitch * i, 0.005 + pitch * j, ro, ri) for i in range(cells) for j in range(cells)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=8)
    ap.add_argument("--offset", type=float, default=12.5e-6)
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args()

    import torch

    from . import build, canvas

    build.build()
    size = 0.0095 * a.cells + 0.0005
    ops = ring_ops(a.cells)
    ms_apply, ms_extract = [], []
    n_active = 0
    for _ in range(a.reps):
        with canvas.Canvas2D((size, size), a.offset) as cv:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cv.apply_ops(ops)
            n_active = cv.getCount_Active()  # applies the queued pass
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            cv.getVoxels_Active(device=True)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            nx, ny = cv.u2_Size
        ms_apply.append((t1 - t0) * 1e3)
        ms_extract.append((t2 - t1) * 1e3)
    nvox = nx * ny
    best_apply, best_extract = min(ms_apply), min(ms_extract)
    out = {"metric": "canvas voxels drawn per second", "voxels": nvox, "rings": len(ops), "active": n_active,
           "ms_draw_and_count": best_apply, "ms_extract_to_device": best_extract,
           "voxels_per_s": nvox / (best_apply / 1e3), "ring_voxel_tests_per_s": nvox * len(ops) / (best_apply / 1e3)}
    oracle = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
    if os.path.exists(os.path.join(oracle, "canvas_oracle.py")):
        sys.path.insert(0, oracle)
        import canvas_oracle

        sx, sy = nx // 4, ny // 4
        t0 = time.perf_counter()
        canvas_oracle.apply(sx, sy, a.offset, ops)
        sec = time.perf_counter() - t0
        out["cpu_restatement"] = {"voxels_per_s": sx * sy / sec, "sample": f"{sx} x {sy} voxels, numpy, 1 core",
                                  "seconds": sec}
        out["gpu_over_cpu"] = out["voxels_per_s"] / out["cpu_restatement"]["voxels_per_s"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
