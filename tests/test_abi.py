"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every entry point of include/*.h."""
import ctypes
import os
import re

import pytest

from code_mpm_gb300 import build, engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h") or not f.startswith("mpm_"):
            continue
        src = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, f)).read(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:int|void|int64_t|const char\*)\s+(mpm_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


@pytest.fixture(scope="module")
def so():
    return build.build()


def test_header_declares_the_solver_entry_points():
    names = declared_functions()
    for must in ("mpm_create", "mpm_destroy", "mpm_upload_particles", "mpm_upload_nodes", "mpm_advance", "mpm_run",
                 "mpm_download_particles", "mpm_download_nodes", "mpm_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(so):
    lib = ctypes.CDLL(so)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header(so):
    engine.lib()  # loads and sets every signature
    names = declared_functions()
    src = "".join(open(os.path.join(ROOT, "code_mpm_gb300", f)).read() for f in ("engine.py", "canvas.py"))
    unbound = [n for n in names if f'"{n}"' not in src]
    assert not unbound, unbound


def test_built_for_sm_103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
