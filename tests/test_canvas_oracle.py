"""The canvas restatement (oracle/canvas_oracle.py) against the reference's own 2D voxel canvas.

The golden voxel flags were made by the reference's Canvas2D_CC.cpp compiled headless
(tests/golden/gen_golden.py, oracle/_ref/ref_canvas); membership and surface flags must agree bit for bit.
"""
import json
import os

import numpy as np
import pytest

import canvas_oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return z, json.loads(str(z["ops"]))


@pytest.mark.parametrize("name", ["canvas_rings", "canvas_cells", "canvas_shapes"])
def test_canvas_oracle_matches_reference(name):
    z, ops = load(name)
    nx, ny = canvas_oracle.size(float(z["width"]), float(z["height"]), float(z["offset"]))
    assert (nx, ny) == (int(z["nx"]), int(z["ny"]))
    flags = canvas_oracle.apply(nx, ny, float(z["offset"]), ops)
    assert np.array_equal(flags, z["flags"])


def test_canvas_cases_cover_every_operation():
    kinds = set()
    for name in ("canvas_rings", "canvas_cells", "canvas_shapes"):
        z, ops = load(name)
        kinds |= {op[0] for op in ops}
        assert (z["flags"] & 1).any()
    assert kinds == {"ring", "rect", "cutrect", "circle", "cutcircle", "prism"}
    z, _ = load("canvas_shapes")
    assert (z["flags"] & 2).any()  # overlapping rings keep some surface voxels
