"""The FP32 form's integer/float-float helpers (code_mpm_gb300/csrc/fpsplit.h) on the CPU: the cell key decided
in float-float arithmetic equals the floor of the IEEE quotient whenever it decides, float-to-double by moving
bit fields equals the conversion, and the float mass threshold compares like the double one.  The same header
is compiled into the kernels."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
@pytest.mark.parametrize("seed", [1, 2])
def test_fpsplit_helpers_exact(tmp_path, seed):
    exe = str(tmp_path / "fps_check")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "csrc", "fps_check.c"), "-lm"],
                   check=True)
    r = subprocess.run([exe, "20000000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
    assert float(r.stdout.split("decided=")[1]) > 0.3
