"""Regenerates the golden MPM states under tests/golden/ from the reference itself.

Needs the reference checkout (default /root/reference; override with
MPM_REFERENCE_DIR): it builds the reference's own physics sources headless
(oracle/build_ref.sh) and advances each seeded input scene with the
one-thread build (oracle/_ref/ref_seq), whose scatter-add and overwrite order
is particle index order; the large-strain case uses the same build with the
large-strain pass 2 switched on (oracle/_ref/ref_seq_ls).  Each case stores
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


def _gz(src: str, dst: str) -> None:
    with open(src, "rb") as f, open(dst, "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
            shutil.copyfileobj(f, g)


def main() -> None:
    ref = os.environ.get("MPM_REFERENCE_DIR", "/root/reference")
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), ref])
    wanted = sys.argv[1:] or list(CASES)
    with tempfile.TemporaryDirectory() as td:
        for name in wanted:
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
