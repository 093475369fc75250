"""The synthetic scene generators' stated geometry (CPU): the graded foam's grading and boundary conditions, the
honeycomb batch's count range."""
import numpy as np

from code_mpm_gb300 import scenes
from code_mpm_gb300.snapshot import NF_FIX_Z, PF_DC_SKIP, PF_SURFACE


def test_graded_foam_small():
    st = scenes.graded_foam(ncell=2, block=(0.02, 0.02, 0.012), perturb=0.0)
    body = (st["pflags"] & PF_DC_SKIP) == 0
    z = st["pos"][body, 2]
    lo, hi = np.quantile(z, [0.05, 0.95])
    # walls thicken with z: more particles per layer near the top than near the floor
    n_lo = np.count_nonzero(np.abs(z - lo) < 0.5e-4)
    n_hi = np.count_nonzero(np.abs(z - hi) < 0.5e-4)
    assert n_hi > 1.5 * n_lo
    # floor plane fixed in z with friction; node arrays besides the boundary conditions are not held
    nn = st.cells + 1
    floor = 2 * nn[0] * nn[1] + np.arange(nn[0] * nn[1])
    assert np.all(st["fixed"][floor] & NF_FIX_Z) and np.all(st["friction"][floor] == 0.2)
    assert len(st["g_mass"]) == st.n_nodes and len(st["fixed"]) == st.n_nodes
    # large grids keep only the boundary conditions on the host
    from code_mpm_gb300.snapshot import empty_state
    bc = empty_state(st.length, st.cells, 10, st.dt_max, node_fields="bc")
    assert len(bc["g_mass"]) == 0 and len(bc["fixed"]) == bc.n_nodes and len(bc["friction"]) == bc.n_nodes
    assert 0.2 < np.mean((st["pflags"][body] & PF_SURFACE) != 0) < 0.9
    # platen: displacement-controlled, moving down
    assert np.all(st["dc_mult"][~body] < 0) and len(st["dc_list"]) == np.count_nonzero(~body)


def test_honeycomb_batch_counts():
    sts = scenes.honeycomb_batch(n=12, total=1.2e6)
    counts = np.array([np.count_nonzero((s["pflags"] & PF_DC_SKIP) == 0) for s in sts])
    assert counts.min() >= 5000 and counts.max() <= 600_000
    assert abs(counts.sum() - 1.2e6) < 0.25 * 1.2e6
