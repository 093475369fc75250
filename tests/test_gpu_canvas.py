"""The GPU voxel canvas (include/mpm_canvas.h) against the reference's own canvas.

Voxel flags must equal the golden flags made by the reference's Canvas2D_CC.cpp (tests/golden/canvas_*.npz) bit
for bit, and the active voxels must come back in voxel order with the reference's centres.
"""
import json
import os

import numpy as np
import pytest

import canvas_oracle
from code_mpm_gb300 import canvas

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["canvas_rings", "canvas_cells", "canvas_shapes"]


def load(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return z, json.loads(str(z["ops"]))


@pytest.mark.parametrize("name", CASES)
def test_gpu_canvas_matches_reference(name):
    z, ops = load(name)
    with canvas.Canvas2D((float(z["width"]), float(z["height"])), float(z["offset"])) as cv:
        assert cv.u2_Size == (int(z["nx"]), int(z["ny"]))
        cv.apply_ops(ops)
        assert np.array_equal(cv.flags(), z["flags"])


@pytest.mark.parametrize("name", CASES)
def test_gpu_canvas_active_voxels_in_voxel_order(name):
    z, ops = load(name)
    flags = z["flags"]
    nx, ny, off = int(z["nx"]), int(z["ny"]), float(z["offset"])
    with canvas.Canvas2D((float(z["width"]), float(z["height"])), off) as cv:
        cv.apply_ops(ops)
        v = cv.getVoxels_Active()
        assert cv.getCount_Active() == int((flags & 1).sum())
        dv = cv.getVoxels_Active(device=True)
    ids = np.nonzero(flags & 1)[0]
    assert np.array_equal(v["ids"], ids.astype(np.uint32))
    assert np.array_equal(v["xy"], canvas_oracle.positions(nx, ny, off)[ids])
    assert np.array_equal(v["surface"], (flags[ids] >> 1) & 1)
    assert np.array_equal(dv["xy"].cpu().numpy(), v["xy"]) and np.array_equal(dv["surface"].cpu().numpy(), v["surface"])


def test_gpu_canvas_queues_across_reads():
    """Operations queued after a read apply on top of the earlier ones, as on the reference's canvas."""
    z, ops = load("canvas_shapes")
    off = float(z["offset"])
    with canvas.Canvas2D((float(z["width"]), float(z["height"])), off) as cv:
        cv.apply_ops(ops[:3])
        first = cv.flags()
        cv.apply_ops(ops[3:])
        assert np.array_equal(cv.flags(), z["flags"])
    nx, ny = int(z["nx"]), int(z["ny"])
    assert np.array_equal(first, canvas_oracle.apply(nx, ny, off, ops[:3]))
