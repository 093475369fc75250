"""Full-size workloads through size-independent properties: the 256-specimen honeycomb batch (40.7M particles)
and the graded foam (22.6M particles on an 800 x 800 x 400 grid).  After one step: every cell key equals the
IEEE floor(x/h) of the step's starting positions (numpy), the cell order is the stable argsort of the keys,
the grid holds exactly the mass of the particles whose corners are all in range, and the platen follows its
timeline; after more steps the state stays finite."""
import numpy as np
import pytest

from code_mpm_gb300 import engine, scenes

pytestmark = pytest.mark.gpu


def keys_of(st):
    h = st.length / st.cells
    b = np.floor(st["pos"] / h).astype(np.int64)  # IEEE division, as glm::floor(x / h)
    kd = st.cells.astype(np.int64) + 2
    ok = np.all((b >= -1) & (b <= st.cells.astype(np.int64)), axis=1)
    key = (b[:, 0] + 1) + kd[0] * ((b[:, 1] + 1) + kd[1] * (b[:, 2] + 1))
    return np.where(ok, key, np.prod(kd)), b


def check_one_step(e, st):
    keys, order = e.cell_order()
    ref, b = keys_of(st)
    assert np.array_equal(keys.astype(np.int64), ref)
    assert np.array_equal(order, np.argsort(keys, kind="stable"))
    # grid mass = mass of particles with every corner node in range (interior particles here)
    nn = st.cells + 1
    inside = np.all((b >= 0) & (b <= st.cells - 1), axis=1)
    mass = np.zeros(int(np.prod(nn.astype(np.int64))), dtype=np.float64)
    nd = engine.Nodes(mass=mass.ctypes.data)
    e._check(e._L.mpm_download_nodes(e._h, engine.C.byref(nd)))
    assert abs(mass.sum() - st["mass"][inside].sum()) <= 1e-5 * st["mass"][inside].sum()


def test_graded_foam_full_size():
    st = scenes.graded_foam()
    assert st.n_particles > 20_000_000 and st.n_nodes == 801 * 801 * 401
    with engine.Engine.from_state(st, engine.FORM_FP32) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(1, st.dt_max, True)
        check_one_step(e, st)
        e.advance(19, st.dt_max, True)
        out = {k: np.empty((st.n_particles, 3)) for k in ("pos", "vel")}
        e.download_particles(out)
        t = e.get_sim()["time"]
    plat = (st["pflags"] & 8) != 0
    assert np.all(np.isfinite(out["pos"])) and np.all(np.isfinite(out["vel"]))
    # the platen moved at -20 m/s (advected by its timeline velocity on the contact path)
    dz = out["pos"][plat, 2] - st["pos"][plat, 2]
    assert np.allclose(dz, -20.0 * t, rtol=1e-9, atol=1e-15)


def test_honeycomb_batch_full_size():
    sts = scenes.honeycomb_batch()
    with engine.Engine.from_batch(sts, engine.FORM_FP32) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(1, sts[0].dt_max, True)
        keys, order = e.cell_order()
        pk = e.packed
        n = pk.state.n_particles
        assert keys.shape == (n,)
        # keys per specimen: each specimen's own grid, offset by the keys of the specimens before it
        off = 0
        for i, st in enumerate(sts):
            lo, hi = pk.particle_offsets[i], pk.particle_offsets[i + 1]
            ref, _ = keys_of(st)
            kmax = int(np.prod(st.cells.astype(np.int64) + 2))
            ref = np.where(ref < kmax, ref + off, -1)
            got = keys[lo:hi].astype(np.int64)
            valid = ref >= 0
            assert np.array_equal(got[valid], ref[valid]), i
            off += kmax
        assert np.array_equal(order, np.argsort(keys, kind="stable"))


def test_reduced_foam_parity():
    """The foam generator's reduced case against the oracle: plain form at 1e-9 with exact active sets and contact
    flags (floor friction on), chosen form within its bars."""
    import pyoracle
    from code_mpm_gb300 import metrics

    st = scenes.graded_foam(ncell=2, block=(0.012, 0.012, 0.008), seed=3)
    ref = st.copy()
    pyoracle.advance(ref, 8, 1, floor_friction=1)
    with engine.Engine.from_state(st, engine.FORM_FP64) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(8, st.dt_max, True)
        out = e.download_state(st)
    for k in ("pos", "vel", "stress", "F"):
        scale = np.abs(ref[k]).max()
        assert np.abs(out[k] - ref[k]).max() <= 1e-9 * scale, k
    with engine.Engine.from_state(st, engine.FORM_FP32) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(8, st.dt_max, True)
        o32 = e.download_state(st)
    err = metrics.form_errors(o32, ref)
    assert err["vm_stress_rel_l2"] <= 1e-2 and err["strain_energy_rel"] <= 5e-3, err
