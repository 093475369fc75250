"""Regenerates the golden MPM states under tests/golden/ from the reference itself.

Needs the reference checkout ($MPM_REFERENCE_DIR, else a checkout named
`reference` beside this repository): it builds the reference's own physics sources headless
(oracle/build_ref.sh) and advances each seeded input scene with the
one-thread build (oracle/_ref/ref_seq), whose scatter-add and overwrite order
is particle index order; the large-strain case uses the same build with the
large-strain pass 2 switched on (oracle/_ref/ref_seq_ls).  The canvas cases
run the reference's 2D voxel canvas (oracle/_ref/ref_canvas) and store its
voxel flags with the operations as .npz.  Each case stores
the input state and the reference's state after k steps as gzip-compressed
MPMSNAP1 files.

    python tests/golden/gen_golden.py [case ...]
"""
from __future__ import annotations

import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from code_mpm_gb300 import scenes, snapshot  # noqa: E402

# name -> (scene factory, contact path, steps, reference build)
CASES = {
    "mixed": (lambda: scenes.mixed_small(seed=1), 0, (1, 25), "ref_seq"),
    "mixed_contactpath": (lambda: scenes.mixed_small(seed=3), 1, (3,), "ref_seq"),
    "contact": (lambda: scenes.contact_small(seed=2), 1, (1, 25), "ref_seq"),
    "bar": (lambda: scenes.bar(cells_len=10, cells_w=2, seed=4), 0, (60,), "ref_seq"),
    "largestrain": (lambda: scenes.mixed_small(seed=5), 0, (1, 25), "ref_seq_ls"),
}


# The reference's 2D voxel canvas (Canvas2D_CC.cpp): name -> (width, height, offset, operations)
def _canvas_cases():
    rings = [("ring", 0.005 + 0.0095 * i, 0.005 + 0.0095 * j, 0.0045, 0.0038) for i in range(4) for j in range(4)]
    cells = [("rect", 0.02, 0.02, 0.032, 0.032, 0.0)]
    cells += [("cutrect", 0.0055 + 0.0072 * i, 0.0055 + 0.0072 * j, 0.0062, 0.0062, 0.0) for i in range(4)
              for j in range(4)]
    shapes = [("circle", 0.012, 0.013, 0.006), ("rect", 0.028, 0.012, 0.012, 0.005, 0.3),
              ("prism", 0.02, 0.03, 0.016, 0.006, 0.002, -0.7), ("cutcircle", 0.012, 0.013, 0.0025),
              ("cutrect", 0.028, 0.012, 0.004, 0.002, 1.1), ("ring", 0.03, 0.03, 0.006, 0.003),
              ("ring", 0.033, 0.03, 0.005, 0.002)]
    return {"canvas_rings": (0.04, 0.04, 0.000125, rings), "canvas_cells": (0.04, 0.04, 0.0002, cells),
            "canvas_shapes": (0.045, 0.04, 0.00025, shapes)}


def _canvas(name: str, exe: str, td: str) -> None:
    import json

    import numpy as np

    w, h, off, ops = _canvas_cases()[name]
    src = os.path.join(td, f"{name}.ops")
    with open(src, "w") as f:
        f.write(f"canvas {w!r} {h!r} {off!r}\n")
        for op in ops:
            f.write(" ".join([op[0]] + [repr(float(v)) for v in op[1:]]) + "\n")
    out = os.path.join(td, f"{name}.bin")
    subprocess.check_call([exe, src, out], stdout=subprocess.DEVNULL)
    raw = open(out, "rb").read()
    nx, ny = np.frombuffer(raw[:8], dtype="<u4")
    flags = np.frombuffer(raw[8:], dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), flags=flags, nx=nx, ny=ny, width=w, height=h, offset=off,
                        ops=json.dumps(ops))
    print(name, int(nx), "x", int(ny), "voxels,", int((flags & 1).sum()), "active,", int((flags & 2).sum() // 2),
          "surface")


def _gz(src: str, dst: str) -> None:
    with open(src, "rb") as f, open(dst, "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
            shutil.copyfileobj(f, g)


def main() -> None:
    ref = os.environ.get("MPM_REFERENCE_DIR") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), ref])
    wanted = sys.argv[1:] or list(CASES) + list(_canvas_cases())
    with tempfile.TemporaryDirectory() as td:
        for name in [w for w in wanted if w in _canvas_cases()]:
            _canvas(name, os.path.join(ROOT, "oracle", "_ref", "ref_canvas"), td)
        for name in [w for w in wanted if w in CASES]:
            make, contact, steps, build = CASES[name]
            exe = os.path.join(ROOT, "oracle", "_ref", build)
            st = make()
            src = os.path.join(td, f"{name}_in.snap")
            snapshot.save(src, st)
            _gz(src, os.path.join(HERE, f"{name}_in.snap.gz"))
            for k in steps:
                out = os.path.join(td, f"{name}_ref{k}.snap")
                subprocess.check_call([exe, src, out, str(k), str(contact)], stdout=subprocess.DEVNULL)
                _gz(out, os.path.join(HERE, f"{name}_ref{k}.snap.gz"))
            print(name, st.n_particles, "particles", st.n_nodes, "nodes", "steps", steps)


if __name__ == "__main__":
    main()
