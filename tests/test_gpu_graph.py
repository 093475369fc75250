"""The two-step CUDA graph that mpm_advance replays in the steady state: the same results, clock and launch count
as launching every kernel, for the plain form against the oracle, the platen timeline and the drop-in's chunked run."""
import time

import numpy as np
import pytest

import pyoracle
from code_mpm_gb300 import engine, scenes

pytestmark = pytest.mark.gpu


def run(st, steps, contact, form, graph, floor=0):
    with engine.Engine.from_state(st, form) as e:
        e.set_option(engine.OPT_GRAPH, graph)
        if floor:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        l0 = e.launch_count()
        e.advance(steps, st.dt_max, contact)
        launches = e.launch_count() - l0
        return e.download_state(st), launches


@pytest.mark.parametrize("name,contact", [("contact", 1), ("mixed", 0)])
def test_graph_replay_keeps_plain_parity(golden, name, contact):
    st = golden(f"{name}_in")
    ref = golden(f"{name}_ref25")
    g, lg = run(st, 25, contact, engine.FORM_FP64, 1)
    p, lp = run(st, 25, contact, engine.FORM_FP64, 0)
    # the graph also runs the two clock kernels of each replayed step: 22 of the 25 (the first step runs plainly,
    # and so does the last, the output step with the contact detection and the node values the caller sees, and
    # the one before it, which the two-step graph cannot take alone)
    assert lg - lp == 2 * 22
    for out in (g, p):
        for k in ("pos", "vel", "stress", "F", "g_vel", "g_mom"):
            scale = np.abs(ref[k]).max()
            assert np.abs(out[k] - ref[k]).max() <= 1e-9 * scale, k
        assert np.array_equal(out["g_state"], ref["g_state"])
        assert out.time == ref.time and out.step == ref.step


def test_graph_replay_platen_timeline_fp32():
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0)
    g, _ = run(st, 41, 1, engine.FORM_FP32, 1, floor=1)
    p, _ = run(st, 41, 1, engine.FORM_FP32, 0, floor=1)
    assert g.time == p.time and g.step == p.step
    for k in ("pos", "vel", "stress"):
        scale = np.abs(p[k]).max()
        assert np.abs(g[k] - p[k]).max() <= 1e-5 * scale, k
    plat = (st["pflags"] & 8) != 0
    assert np.array_equal(g["pos"][plat], p["pos"][plat])  # the timeline moves the platen identically


def test_chunked_run_through_graphs():
    st = scenes.contact_small(seed=2)
    with engine.Engine.from_state(st) as e:
        e.set_sim(time=0.0, dt_max=st.dt_max)
        done = e.runSimulation_Classic_DoublePass_MPLocks_Contact(6.5 * st.dt_max)
        out = e.download_state(st)
    # 6 full steps and one half step
    assert out.step == 7 and done == 0
    assert abs(out.time - 6.5 * st.dt_max) <= 1e-15


def test_graph_speeds_up_a_small_scene():
    st = scenes.bar()  # 40,000 particles: launch-bound
    times = {}
    for graph in (0, 1):
        with engine.Engine.from_state(st, engine.FORM_FP32) as e:
            e.set_option(engine.OPT_GRAPH, graph)
            e.advance(10, st.dt_max, False)
            ms = e.advance_timed(400, st.dt_max, False)
            times[graph] = ms / 400
    print({"ms_per_step_plain": times[0], "ms_per_step_graph": times[1]})
    assert times[1] <= times[0] * 1.05


@pytest.mark.parametrize("form", [engine.FORM_FP64, engine.FORM_FP32])
def test_advances_of_odd_length_replay_the_right_graph(form):
    """Each step flips the cell-key buffers, so a captured two-step graph is valid only at the parity it was
    captured with; advances of odd length change the parity between replays.  Runs of odd advances equal the
    run without graphs (the oracle for the plain form)."""
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0)
    chunks = [5, 7, 3, 25, 9, 4, 11]
    outs = {}
    for graph in (1, 0):
        with engine.Engine.from_state(st, form) as e:
            e.set_option(engine.OPT_GRAPH, graph)
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
            for k in chunks:
                e.advance(k, st.dt_max, True)
            outs[graph] = e.download_state(st)
    tol = 1e-9 if form == engine.FORM_FP64 else 1e-5
    for k in ("pos", "vel", "stress", "g_mass", "g_mom"):
        scale = np.abs(outs[0][k]).max()
        assert np.abs(outs[1][k] - outs[0][k]).max() <= tol * scale, k
    assert np.array_equal(outs[1]["g_state"], outs[0]["g_state"])
    if form == engine.FORM_FP64:
        ref = st.copy()
        pyoracle.advance(ref, sum(chunks), 1, floor_friction=1)
        for k in ("pos", "vel", "stress"):
            scale = np.abs(ref[k]).max()
            assert np.abs(outs[1][k] - ref[k]).max() <= 1e-9 * scale, k
