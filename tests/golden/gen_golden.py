"""Regenerates the golden MPM states under tests/golden/ from the reference itself.

Needs the reference checkout (default /root/reference; override with
MPM_REFERENCE_DIR): it builds the reference's own physics sources headless
(oracle/build_ref.sh) and advances each seeded input scene with the
one-thread build (oracle/_ref/ref_seq), whose scatter-add and overwrite order
is particle index order.  Each case stores the input state and the reference's
state after k steps as gzip-compressed MPMSNAP1 files.

    python tests/golden/gen_golden.py
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

# name -> (scene factory, contact path, steps)
CASES = {
    "mixed": (lambda: scenes.mixed_small(seed=1), 0, (1, 25)),
    "mixed_contactpath": (lambda: scenes.mixed_small(seed=3), 1, (3,)),
    "contact": (lambda: scenes.contact_small(seed=2), 1, (1, 25)),
    "bar": (lambda: scenes.bar(cells_len=10, cells_w=2, seed=4), 0, (60,)),
}


def _gz(src: str, dst: str) -> None:
    with open(src, "rb") as f, open(dst, "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
            shutil.copyfileobj(f, g)


def main() -> None:
    ref = os.environ.get("MPM_REFERENCE_DIR", "/root/reference")
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), ref])
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_seq")
    with tempfile.TemporaryDirectory() as td:
        for name, (make, contact, steps) in CASES.items():
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
