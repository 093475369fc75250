"""Particles stored in cell order (FP32 form, MPM_OPT_REORDER): results, downloads, lists and the cell order stay
in the caller's numbering and agree with the unordered run up to FP32 summation order."""
import numpy as np
import pytest

import pyoracle
from code_mpm_gb300 import engine, metrics, scenes

pytestmark = pytest.mark.gpu


def run(st, steps, contact, reorder, floor=0, graph=1, cell_sort=1, p2g=None):
    with engine.Engine.from_state(st, engine.FORM_FP32) as e:
        e.set_option(engine.OPT_REORDER, reorder)
        e.set_option(engine.OPT_GRAPH, graph)
        e.set_option(engine.OPT_CELL_SORT, cell_sort)
        if p2g is not None:
            e.set_option(engine.OPT_P2G_REDUCE, p2g)
        if floor:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(steps, st.dt_max, contact)
        return e.download_state(st)


def close(a, b, keys=("pos", "vel", "stress", "strain", "F", "e_strain", "g_mass", "g_vel"), rel=1e-4):
    for k in keys:
        scale = np.abs(b[k]).max()
        assert np.abs(a[k] - b[k]).max() <= rel * scale + 1e-30, k


@pytest.mark.parametrize("interval", [0, 7])
def test_reordered_run_matches_unordered(interval):
    st = scenes.contact_small(seed=2)
    a = run(st, 30, 1, interval)
    b = run(st, 30, 1, -1)
    close(a, b)
    assert np.array_equal(a["material"], b["material"]) and np.array_equal(a["pflags"], b["pflags"])
    assert np.array_equal(a["dc_mult"], b["dc_mult"])
    assert np.array_equal(a["g_state"] & 1, b["g_state"] & 1)
    ref = st.copy()
    pyoracle.advance(ref, 30, 1)
    err = metrics.form_errors(a, ref)
    assert err["vm_stress_rel"] <= 1e-2 and err["strain_energy_rel"] <= 5e-3, err


def test_cell_order_in_caller_numbering():
    st = scenes.mixed_small(seed=1)
    with engine.Engine.from_state(st, engine.FORM_FP32) as e:
        e.advance(3, st.dt_max, False)
        keys, order = e.cell_order()
        pos = e.download_state(st)["pos"]
    # keys of the positions before the last step's sort are those of the state after two steps
    with engine.Engine.from_state(st, engine.FORM_FP32) as e2:
        e2.set_option(engine.OPT_REORDER, -1)
        e2.advance(3, st.dt_max, False)
        keys2, order2 = e2.cell_order()
    assert np.array_equal(keys, keys2)
    assert np.array_equal(order, np.argsort(keys, kind="stable"))
    assert np.array_equal(order, order2)


def test_lists_uploaded_after_a_reorder():
    st = scenes.platen_block(size=(0.006, 0.006, 0.004), h=1.0e-3, speed=20.0, friction=0.0)
    n = st.n_particles
    mask = np.zeros(n, dtype=np.uint8)
    mask[::3] = engine.MON_ENERGY | engine.MON_STRESS
    outs, mons = [], []
    for reorder in (0, -1):
        with engine.Engine.from_state(st, engine.FORM_FP32) as e:
            e.set_option(engine.OPT_REORDER, reorder)
            e.advance(4, st.dt_max, True)
            # re-upload the platen list and a monitor mask in the caller's numbering after the reorder
            dcl = np.ascontiguousarray(st["dc_list"], dtype=np.uint32)
            e._check(e._L.mpm_upload_dc_list(e._h, engine._ptr(dcl), len(dcl)))
            e.upload_monitor_mask(mask)
            e.advance(6, st.dt_max, True)
            outs.append(e.download_state(st))
            mons.append(e.monitors())
    close(outs[0], outs[1])
    for k in ("strain_energy", "plastic_energy"):
        assert abs(mons[0][k] - mons[1][k]) <= 1e-4 * abs(mons[1][k]) + 1e-30, k
    assert mons[0]["count"] == mons[1]["count"]


@pytest.mark.parametrize("reorder,p2g", [(0, 2), (7, 3), (-1, 2), (-1, 4), (0, 5), (7, 6), (-1, 6)])
def test_sort_free_run_matches_sorted(reorder, p2g):
    """Without the per-step sort the cell-run kernels take the slots in storage order: cell order after a
    reorder, the caller's (unordered) order with reorders off, where nearly every cell splits into many runs."""
    st = scenes.contact_small(seed=2)
    a = run(st, 30, 1, reorder, cell_sort=0, p2g=p2g)
    b = run(st, 30, 1, -1)
    close(a, b)
    st = scenes.mixed_small(seed=1)
    a = run(st, 20, 0, reorder, floor=1, cell_sort=0, p2g=p2g)
    b = run(st, 20, 0, -1, floor=1)
    close(a, b)


def test_sort_free_cell_order_is_the_sorted_runs():
    """The cell order reported after steps without the sort: the keys of the positions before the last step and
    their stable order, the same as with the per-step sort."""
    st = scenes.mixed_small(seed=1)
    got = []
    for cs in (1, 0):
        with engine.Engine.from_state(st, engine.FORM_FP32) as e:
            e.set_option(engine.OPT_CELL_SORT, cs)
            e.advance(3, st.dt_max, False)
            got.append(e.cell_order())
    (k1, o1), (k0, o0) = got
    assert np.mean(k1 == k0) > 0.999
    assert np.array_equal(o0, np.argsort(k0, kind="stable"))


@pytest.mark.parametrize("contact,floor", [(1, 0), (0, 1)])
def test_steps_of_one_advance_match_output_steps(contact, floor):
    """Inside one advance only the last step is an output step (the others zero their nodes instead of a grid
    reset and skip the contact detection); one step per call makes every step an output step.  Both agree to
    FP32 summation order."""
    st = scenes.contact_small(seed=2) if contact else scenes.mixed_small(seed=1)
    a = run(st, 30, contact, 0, floor=floor, cell_sort=0)
    with engine.Engine.from_state(st, engine.FORM_FP32) as e:
        e.set_option(engine.OPT_CELL_SORT, 0)
        if floor:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        for _ in range(30):
            e.advance(1, st.dt_max, bool(contact))
        b = e.download_state(st)
    close(a, b)
    assert np.array_equal(a["g_state"] & 1, b["g_state"] & 1)
