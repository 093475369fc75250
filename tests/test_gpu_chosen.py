"""The chosen (FP32-transfer) form against the FP64 oracle, and the autotuner.

Accuracy bars of the chosen form (stated per result, from the path's target):
  * von Mises stress: max |vm_fp32 - vm_fp64| / max vm_fp64 <= 1e-2;
  * strain energy (sum over particles): relative error <= 5e-3;
  * positions: max |x_fp32 - x_fp64| <= 1e-4 h (positions are accumulated in FP64).
"""
import numpy as np
import pytest

import pyoracle
from code_mpm_gb300 import engine, metrics, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from code_mpm_gb300 import build

    build.build()
    engine.lib()


def run(st, steps, contact, form, floor=0):
    with engine.Engine.from_state(st, form) as e:
        if floor:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(steps, st.dt_max, contact)
        return e.download_state(st)


CASES = [("mixed", lambda: scenes.mixed_small(seed=1), 0, 25, 0),
         ("contact", lambda: scenes.contact_small(seed=2), 1, 25, 0),
         ("bar", lambda: scenes.bar(), 0, 400, 0),
         ("block", lambda: scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0, yield_=120.0e6), 1, 150, 1)]


@pytest.mark.parametrize("name,make,contact,steps,floor", CASES)
def test_chosen_form_within_stated_error(name, make, contact, steps, floor):
    st = make()
    ref = st.copy()
    pyoracle.advance(ref, steps, contact, floor_friction=floor)
    out = run(st, steps, contact, engine.FORM_FP32, floor)
    err = metrics.form_errors(out, ref)
    h = float((st.length / st.cells).min())
    assert err["vm_stress_rel"] <= 1e-2, err
    assert err["strain_energy_rel"] <= 5e-3, err
    assert err["pos_abs_max"] <= 1e-4 * h, err


@pytest.mark.parametrize("form", [engine.FORM_FP64, engine.FORM_FP32])
def test_autotune_restores_state_and_picks_valid_options(golden, form):
    st = golden("contact_in")
    with engine.Engine.from_state(st, form) as e:
        before = e.download_state(st)
        res = e.autotune(steps=2, contact=True)
        after = e.download_state(st)
        # P2G stage 15, pass-1 stage 9 (cell-run P2G only), pass-2 stage 6 (FP64) or 9 (FP32: also the staged mode)
        ncand = (21, 30) if form == engine.FORM_FP64 else (30, 39)
        modes = (0, 1) if form == engine.FORM_FP64 else (0, 1, 2)
        assert res["candidates"] in ncand and res["pass1_corners"] in (1, 2, 4) and res["pass1_block"] in (128, 256, 512) and res["gather_batch"] in modes and res["p2g_block"] in (128, 256, 512) and res["pass_block"] in (128, 256, 512)
        assert res["best_ms_per_step"] <= res["worst_ms_per_step"]
        for k in ("pos", "vel", "stress", "F", "g_mass", "g_state"):
            assert np.array_equal(before[k], after[k]), k
        assert after.time == before.time and after.step == before.step


def test_plain_form_parity_holds_for_every_launch_configuration(golden):
    st = golden("contact_in")
    ref = golden("contact_ref25")
    for red in (0, 1, 2, 3, 4):
        for blk in (128, 512):
            with engine.Engine.from_state(st) as e:
                e.set_option(engine.OPT_GATHER, 1 if blk == 512 else 0)
                e.set_option(engine.OPT_P2G_REDUCE, red)
                e.set_option(engine.OPT_PASS1_CORNERS, {2: 1, 3: 2, 4: 4}.get(red, 1))
                e.set_option(engine.OPT_PASS1_BLOCK, blk)
                e.set_option(engine.OPT_P2G_BLOCK, blk)
                e.set_option(engine.OPT_PASS_BLOCK, blk)
                e.advance(25, st.dt_max, True)
                out = e.download_state(st)
            for k in ("pos", "vel", "stress"):
                scale = np.abs(ref[k]).max()
                assert np.abs(out[k] - ref[k]).max() / scale <= 1e-9, (red, blk, k)
            assert np.array_equal(out["g_state"], ref["g_state"])


def test_chosen_form_p2g_modes_agree():
    """The P2G reductions (per-particle atomics, lane runs, shared-memory cell runs with 1, 2 or 4 corners per
    thread, runs reduced in registers by lane pairs with the tile read from global memory or staged by bulk
    copies) sum the same contributions in different orders; with the contact path they also carry the FP32 mass
    gradient.  At 128 threads the pair kernel's tiles are 512 slots: the first two of this scene stage, the last
    (partial) one reads global memory."""
    st = scenes.contact_small(seed=2)
    outs = []
    for red in (0, 1, 2, 3, 4, 5, 6):
        for blk in ((128, 512) if red >= 2 else (256,)):
            with engine.Engine.from_state(st, engine.FORM_FP32) as e:
                e.set_option(engine.OPT_P2G_REDUCE, red)
                e.set_option(engine.OPT_P2G_BLOCK, blk)
                e.set_option(engine.OPT_PASS1_CORNERS, {2: 1, 3: 2, 4: 4}.get(red, 1))
                e.set_option(engine.OPT_PASS1_BLOCK, {128: 512, 512: 128}.get(blk, 128))
                e.advance(10, st.dt_max, True)
                outs.append(((red, blk), e.download_state(st)))
    (_, a) = outs[0]
    for cfg, b in outs[1:]:
        for k in ("g_mass", "g_mom", "g_mass_gradient", "stress", "vel"):
            scale = np.abs(a[k]).max()
            assert np.abs(b[k] - a[k]).max() <= 1e-4 * scale, (cfg, k)
        assert np.array_equal(a["g_state"] & 1, b["g_state"] & 1), cfg


def test_pair_modes_through_the_sort_permutation():
    """P2G modes 5 and 6 (and their pass 1) read particles through the per-step sort's permutation when the
    particles are sorted every step (MPM_OPT_CELL_SORT 1); mode 6 then reads global memory."""
    st = scenes.mixed_small(seed=3)
    outs = {}
    for red in (3, 5, 6):
        with engine.Engine.from_state(st, engine.FORM_FP32) as e:
            e.set_option(engine.OPT_CELL_SORT, 1)
            e.set_option(engine.OPT_REORDER, -1)
            e.set_option(engine.OPT_P2G_REDUCE, red)
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
            e.advance(12, st.dt_max, False)
            outs[red] = e.download_state(st)
    for red in (5, 6):
        for k in ("g_mass", "g_mom", "stress", "vel", "pos"):
            scale = np.abs(outs[3][k]).max()
            assert np.abs(outs[red][k] - outs[3][k]).max() <= 1e-4 * scale, (red, k)
        assert np.array_equal(outs[3]["g_state"] & 1, outs[red]["g_state"] & 1), red


PASS2_FIELDS = ("pos", "vel", "stress", "strain", "eps_p", "F", "vol", "backstress", "e_strain", "e_plastic")


@pytest.mark.parametrize("scene", ["mixed", "batch"])
def test_staged_pass2_reads_the_same_fields(scene):
    """Pass-2 mode 2 brings each block's particle fields into shared memory with bulk copies before the particle
    update; mode 0 reads them from global memory.  From the same state, one step of each agrees in every particle
    field to FP32 rounding (the only difference between two runs is the order of P2G's FP32 atomics), at each
    pass-2 block size; a misplaced component or particle would show as an O(1) difference.  "batch" covers the
    specimen ids (several specimens) and the contact path, "mixed" the non-contact path."""
    if scene == "mixed":
        sts, contact = [scenes.mixed_small(seed=1, ncell=(16, 14, 8))], False
    else:
        sts = [scenes.honeycomb(0.8e-3, 3e-3, 2, 3000, 8.0, h=0.5e-3),
               scenes.honeycomb(0.6e-3, 2.5e-3, 3, 5000, 4.0, h=0.5e-3)]
        contact = True
    assert sum(s.n_particles for s in sts) > 2 * (512 + 16)  # blocks of every size stage

    def one(mode, blk):
        make = (lambda: engine.Engine.from_state(sts[0], engine.FORM_FP32)) if len(sts) == 1 else \
            (lambda: engine.Engine.from_batch(sts, engine.FORM_FP32))
        with make() as e:
            e.set_option(engine.OPT_GATHER, mode)
            e.set_option(engine.OPT_PASS_BLOCK, blk)
            e.advance(1, sts[0].dt_max, contact)
            return e.download_state(sts[0]) if len(sts) == 1 else e.download_batch(sts)

    for blk in (128, 256, 512):
        a = one(0, blk)
        a = a if isinstance(a, list) else [a]
        for mode in (2,):
            b = one(mode, blk)
            b = b if isinstance(b, list) else [b]
            for x, y in zip(a, b):
                for k in PASS2_FIELDS:
                    d = x[k] - y[k] if k != "pos" else (x[k] - y[k]) / float((sts[0].length / sts[0].cells).min())
                    scale = max(np.abs(x[k]).max(), 1e-300) if k != "pos" else 1.0
                    assert np.abs(d).max() <= 1e-5 * scale, (mode, blk, k)


def test_staged_pass2_only_in_the_fp32_form():
    st = scenes.mixed_small(seed=1)
    with engine.Engine.from_state(st) as e:
        with pytest.raises(engine.MPMError):
            e.set_option(engine.OPT_GATHER, 2)
