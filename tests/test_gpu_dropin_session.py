"""The C++ drop-in session (code_mpm_gb300/dropin/mpm_dropin.hpp) on stand-in objects.

tests/csrc/dropin_standin.cpp declares its own particle, node and material types carrying the member names of
MaterialPoint_BC / GridPoint / Material_BC, builds them from a snapshot, and drives the session the way the drop-in
translation unit does (one call per step, each attaching first).  Checked here:
  * AoS -> device -> AoS after 0 steps returns every mapped field bit for bit;
  * after 25 calls of one step the objects equal the reference's own golden states (1e-9 normwise, active sets and
    contact flags exact), for the non-contact and the contact loop;
  * the context stays resident: one upload for all calls, and a position edited between calls makes the next
    call upload again.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from code_mpm_gb300 import snapshot

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIELDS = ("pos", "vel", "stress", "strain", "eps_p", "F", "vol", "backstress", "e_strain", "e_plastic", "e_strain_ti",
          "e_strain_max", "mp_mass_gradient", "strain_rate", "g_mass", "g_mom", "g_vel", "g_force", "g_force_temp",
          "g_mass_gradient")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from code_mpm_gb300 import build

    build.build()
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_standin")
    lib = os.path.join(ROOT, "code_mpm_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
           "-I", os.path.join(ROOT, "code_mpm_gb300", "dropin"), os.path.join(ROOT, "tests", "csrc", "dropin_standin.cpp"),
           "-o", exe, "-L", lib, "-lmpm_gb300", f"-Wl,-rpath,{lib}"]
    subprocess.check_call(cmd)
    return exe


def _run(driver, tmp_path, st, steps, contact):
    src, dst = str(tmp_path / "in.snap"), str(tmp_path / "out.snap")
    snapshot.save(src, st)
    out = subprocess.run([driver, src, dst, str(steps), str(contact)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    return snapshot.load(dst), json.loads(out.stdout.strip().splitlines()[-1])


def relerr(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max() if b.size else 0.0
    d = np.abs(a - b).max() if b.size else 0.0
    return d / scale if scale > 0 else d


def test_round_trip_is_exact(driver, tmp_path, golden):
    st = golden("contact_ref1")  # a state with nonzero stresses, node values and contact flags
    out, info = _run(driver, tmp_path, st, 0, 1)
    for k in FIELDS + ("g_state", "fext", "mass", "vol0"):
        assert np.array_equal(out[k], st[k]), k
    assert info["uploads_run"] == 1


@pytest.mark.parametrize("name,contact", [("mixed", 0), ("contact", 1)])
def test_session_matches_reference_golden(driver, tmp_path, golden, name, contact):
    st = golden(f"{name}_in")
    ref = golden(f"{name}_ref25")
    out, info = _run(driver, tmp_path, st, 25, contact)
    bad = {k: relerr(out[k], ref[k]) for k in FIELDS}
    assert all(v <= 1e-9 for v in bad.values()), bad
    assert np.array_equal(out["g_state"], ref["g_state"])
    assert out.step == ref.step
    # resident: 25 calls, one upload; a moved particle triggers the next
    assert info["uploads_run"] == 1 and info["uploads_after_edit"] == 2 and info["rc"] == 0, info
