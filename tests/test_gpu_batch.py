"""Batches of independent specimens (mpm_create_batch) and platen/body cell sharing.

A batch packs several scenes, each with its own grid, into one engine; each
specimen must evolve exactly as it does alone: against the oracle run on that
specimen alone, normwise 1e-9 for the real fields and bit-exact active sets
and contact flags (plain FP64 form), the chosen-form bars for the FP32 form.
"""
import numpy as np
import pytest

import pyoracle
from code_mpm_gb300 import engine, metrics, scenes

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "stress", "strain", "eps_p", "F", "vol", "backstress", "e_strain", "e_plastic",
          "g_mass", "g_mom", "g_vel", "g_force")


def relerr(a, b):
    scale = np.abs(b).max()
    return np.abs(a - b).max() / scale if scale > 0 else np.abs(a - b).max()


def specimens():
    out = [scenes.honeycomb(0.8e-3, 3e-3, 2, 3000, 8.0, h=0.5e-3),
           scenes.honeycomb(0.6e-3, 2.5e-3, 3, 5000, 4.0, h=0.5e-3),
           scenes.honeycomb(1.0e-3, 4e-3, 2, 2000, 9.0, h=0.5e-3)]
    rng = np.random.Generator(np.random.PCG64(3))
    for st in out:  # give the walls some motion so they yield within a few steps
        body = (st["pflags"] & 8) == 0
        st["vel"][body] += rng.normal(0.0, 20.0, size=(int(body.sum()), 3))
    return out


@pytest.mark.parametrize("form", [engine.FORM_FP64, engine.FORM_FP32])
def test_batch_each_specimen_as_alone(form):
    sts = specimens()
    steps = 20
    with engine.Engine.from_batch(sts, form) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(steps, sts[0].dt_max, True)
        outs = e.download_batch(sts)
        offs = e.batch_info()
    assert list(offs) == list(np.cumsum([0] + [s.n_nodes for s in sts]))
    for st, out in zip(sts, outs):
        ref = st.copy()
        pyoracle.advance(ref, steps, 1, floor_friction=1)
        if form == engine.FORM_FP64:
            bad = {k: relerr(out[k], ref[k]) for k in FIELDS if not relerr(out[k], ref[k]) <= 1e-9}
            assert not bad, bad
            assert np.array_equal(out["g_state"], ref["g_state"])
        else:
            err = metrics.form_errors(out, ref)
            assert err["vm_stress_rel"] <= 1e-2 and err["strain_energy_rel"] <= 5e-3, err
            assert np.array_equal(out["g_state"] & 1, ref["g_state"] & 1)


def test_platen_sharing_cells_with_the_body():
    """Platen particles (skipped by G2P) sorted last in a cell shared with body particles: the cell's remap sum
    must still reach the nodes."""
    st = scenes.platen_block(size=(0.006, 0.006, 0.004), h=1.0e-3, speed=20.0, friction=0.0)
    body = (st["pflags"] & 8) == 0
    top = st["pos"][body, 2].max()
    st["pos"][~body, 2] = top - 0.1e-3  # platen layer inside the body's top cells
    ref = st.copy()
    pyoracle.advance(ref, 5, 1)
    with engine.Engine.from_state(st) as e:
        e.advance(5, st.dt_max, True)
        out = e.download_state(st)
    for k in ("pos", "vel", "stress", "g_vel", "g_mom"):
        assert relerr(out[k], ref[k]) <= 1e-9, k
    assert np.array_equal(out["g_state"], ref["g_state"])


def test_upload_rejects_a_specimen_id_out_of_range_and_changes_nothing():
    """Specimen ids are checked on the device during the upload: an id outside the batch fails the upload with
    the first offending particle named, before any particle array is touched."""
    from code_mpm_gb300 import batch

    sts = specimens()[:2]
    with engine.Engine.from_batch(sts, engine.FORM_FP32) as e:
        e.advance(2, sts[0].dt_max, True)
        before = e.download_batch(sts)
        bad = batch.pack(sts).state
        bad["specimen"][[7, 11]] = [2, -1]
        with pytest.raises(engine.MPMError, match="particle 7: specimen 2 out of range"):
            e.upload_state(bad)
        e.packed = batch.pack(sts)
        after = e.download_batch(sts)
    for b, a in zip(before, after):
        for k in ("pos", "vel", "stress"):
            assert np.array_equal(b[k], a[k]), k
