"""The C++ drop-in translation unit compiles and links against the reference's own sources.

code_mpm_gb300/dropin/PhysicsEngine_runSimulation_GB300.cpp replaces the two
runSimulation_Classic_DoublePass_MPLocks{,_Contact}.cpp translation units of
code_MPM; build_dropin.sh links it with the rest of the reference physics and
libmpm_gb300.so.  Needs the reference checkout (skipped where it is absent).
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MPM_REFERENCE_DIR") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "PhysicsEngine.h")), reason="reference checkout absent")
def test_dropin_links_with_reference_sources():
    from code_mpm_gb300 import build

    build.build()
    out = subprocess.run([os.path.join(ROOT, "code_mpm_gb300", "dropin", "build_dropin.sh"), REF],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_gb300")
    assert os.path.exists(exe)
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    # the solver entry points come from the drop-in, and the engine is reached through the C ABI
    assert "PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks(double)" in syms
    assert "PhysicsEngine::runSimulation_Classic_DoublePass_MPLocks_Contact(double)" in syms
    assert " U mpm_advance" in syms and " U mpm_create" in syms
    # the reference's CPU phase functions are not linked in
    assert "runSimulation_M2G" not in syms
