"""The FMA-corrected quotient used by the kernels equals IEEE division on the operands they divide.

The kernels replace x/h by q = RN(x*y), r = fma(-q, h, x), q' = fma(r, y, q)
with y = RN(1/h) (Markstein's correction step).  oracle/div_check.c checks
q' == x/h bit for bit on positions, near-integer quotients (a few ulps either
side of k*h), cell offsets and shape-value products, for the cell sizes of the
scenes and random ones.
"""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_corrected_quotient_is_correctly_rounded():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")], stdout=subprocess.DEVNULL)
    out = subprocess.run([os.path.join(ROOT, "oracle", "_build", "div_check"), "200000", "3"], capture_output=True,
                         text=True)
    assert out.returncode == 0, out.stdout + out.stderr[:2000]
    assert out.stdout.startswith("mismatches 0 of ")
