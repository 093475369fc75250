"""Parity of the CUDA engine (plain FP64 form) with the reference.

Tolerances (from the parity contract of this path):
  * cell keys, the stable cell order, active-node sets and contact flags: bit-exact;
  * particle position, velocity and stress (and the other real fields): normwise
    relative error max|gpu - ref| / max|ref| <= 1e-9 per field; the only source
    of difference is the order of floating-point atomic additions (and FMA
    contraction) in the scatter phases.
"""
import numpy as np
import pytest

import pyoracle
from code_mpm_gb300 import engine, scenes, snapshot

pytestmark = pytest.mark.gpu

TOL = 1.0e-9
REAL_PARTICLE = ("pos", "vel", "stress", "strain", "eps_p", "F", "vol", "backstress", "e_strain", "e_plastic",
                 "e_strain_ti", "e_strain_max", "mp_mass_gradient", "strain_rate")
REAL_NODE = ("g_mass", "g_mom", "g_vel", "g_force", "g_force_temp", "g_mass_gradient")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from code_mpm_gb300 import build

    build.build()
    engine.lib()


def run_gpu(st, steps, contact, form=engine.FORM_FP64, floor_friction=0):
    with engine.Engine.from_state(st, form) as e:
        if floor_friction:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.advance(steps, st.dt_max, contact)
        e.synchronize()
        return e.download_state(st)


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max() if b.size else 0.0
    diff = np.abs(a - b).max() if b.size else 0.0
    return diff / scale if scale > 0 else diff


def assert_parity(gpu, ref, tol=TOL, fields=REAL_PARTICLE + REAL_NODE, exact_state=True):
    bad = {k: relerr(gpu[k], ref[k]) for k in fields}
    bad = {k: v for k, v in bad.items() if not v <= tol}
    assert not bad, f"fields over tolerance {tol}: {bad}"
    if exact_state:
        assert np.array_equal(gpu["g_state"], ref["g_state"]), "active set / contact flags differ"
    assert gpu.time == ref.time and gpu.step == ref.step


CASES = [("mixed", 0, 1), ("mixed", 0, 25), ("mixed_contactpath", 1, 3), ("contact", 1, 1), ("contact", 1, 25),
         ("bar", 0, 60)]


@pytest.mark.parametrize("name,contact,steps", CASES)
def test_gpu_matches_reference_golden(golden, name, contact, steps):
    st = golden(f"{name}_in")
    ref = golden(f"{name}_ref{steps}")
    gpu = run_gpu(st, steps, contact)
    assert_parity(gpu, ref)


@pytest.mark.parametrize("steps", [1, 25])
def test_gpu_large_strain_matches_reference_golden(golden, steps):
    """The large-strain pass 2 (MPM_OPT_LARGE_STRAIN) against the reference built with that pass switched on."""
    st = golden("largestrain_in")
    ref = golden(f"largestrain_ref{steps}")
    with engine.Engine.from_state(st, engine.FORM_FP64) as e:
        e.set_option(engine.OPT_LARGE_STRAIN, 1)
        e.advance(steps, st.dt_max, False)
        e.synchronize()
        gpu = e.download_state(st)
    fields = tuple(k for k in REAL_PARTICLE + REAL_NODE if k not in ("e_strain_ti", "e_strain_max", "strain_rate",
                                                                      "mp_mass_gradient", "g_mass_gradient"))
    assert_parity(gpu, ref, fields=fields + (snapshot.FE_FIELD,))


def test_large_strain_option_is_fp64_only():
    st = scenes.mixed_small(seed=5)
    with engine.Engine.from_state(st, engine.FORM_FP32) as e:
        with pytest.raises(engine.MPMError):
            e.set_option(engine.OPT_LARGE_STRAIN, 1)


def test_cell_keys_and_order_bit_exact(golden):
    st = golden("mixed_in")
    with engine.Engine.from_state(st) as e:
        e.advance(1, st.dt_max, False)
        keys, perm = e.cell_order()
    h = st.length / st.cells
    b = np.floor(st["pos"] / h[None, :])  # IEEE quotient, as glm::floor(x / h)
    kd = st.cells.astype(np.int64) + 2
    ok = np.all((b >= -1) & (b <= st.cells[None, :]), axis=1)
    want = ((b[:, 0] + 1) + kd[0] * ((b[:, 1] + 1) + kd[1] * (b[:, 2] + 1))).astype(np.int64)
    want[~ok] = int(np.prod(kd))
    assert np.array_equal(keys.astype(np.int64), want)
    assert np.array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))


@pytest.mark.parametrize("contact", [0, 1])
def test_gpu_matches_oracle_medium(contact):
    """~20k particles, 12 steps, against the CPU restatement."""
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), h=1.0e-3, speed=20.0, yield_=120.0e6) if contact else \
        scenes.bar(cells_len=16, cells_w=6, v0=30.0)
    ref = st.copy()
    pyoracle.advance(ref, 12, contact)
    gpu = run_gpu(st, 12, contact)
    assert_parity(gpu, ref)


def test_floor_friction_extension_matches_oracle():
    st = scenes.platen_block(size=(0.006, 0.006, 0.004), h=1.0e-3, speed=40.0, friction=0.3)
    st["vel"][:, 0] += 3.0  # sliding on the floor
    ref = st.copy()
    pyoracle.advance(ref, 10, 1, floor_friction=1)
    gpu = run_gpu(st, 10, 1, floor_friction=1)
    assert_parity(gpu, ref)


def test_run_chunks_like_the_reference_loop(golden):
    """runSimulation_*(T) takes steps of dt_max and a shortened last step (…MPLocks.cpp:449-458)."""
    st = golden("mixed_in")
    T = 3.5 * st.dt_max
    ref = st.copy()
    with engine.Engine.from_state(st, time_end=st.time + 3.0 * st.dt_max) as e:
        done = e.runSimulation_Classic_DoublePass_MPLocks(T)
        gpu = e.download_state(st)
    assert done == 1 and gpu.step == 4
    assert gpu.time == st.time + st.dt_max + st.dt_max + st.dt_max + 0.5 * st.dt_max or abs(gpu.time - (st.time + T)) < 1e-20
    del ref


def test_empty_particle_set():
    st = scenes.mixed_small()
    e = engine.Engine(st.length, st.cells)
    empty = snapshot.empty_state(st.length, st.cells, 0, st.dt_max, n_materials=1)
    e.upload_state(empty)
    e.advance(3, st.dt_max, False)
    out = e.download_state(empty)
    assert out.step == 3 and not (out["g_state"] & snapshot.NS_ACTIVE).any()
    e.close()


def test_nonfinite_position_is_reported():
    st = scenes.mixed_small()
    st["pos"][5, 1] = np.nan
    with engine.Engine.from_state(st) as e:
        e.advance(1, st.dt_max, False)
        with pytest.raises(engine.MPMError) as ei:
            e.synchronize()
        assert ei.value.code == -4


def test_bad_arguments_fail_loudly():
    st = scenes.mixed_small()
    with engine.Engine.from_state(st) as e:
        with pytest.raises(engine.MPMError):
            e.advance(1, -1.0, False)
        bad = np.array([1, 1], dtype=np.uint32)
        with pytest.raises(engine.MPMError):
            e._check(e._L.mpm_upload_dc_list(e._h, bad.ctypes.data, 2))


def test_full_size_block_properties():
    """The contact-path workload at full size (~2.07M particles): size-independent properties."""
    st = scenes.platen_block()
    with engine.Engine.from_state(st) as e:
        e.advance(2, st.dt_max, True)
        keys, perm = e.cell_order()
        out = e.download_state(st)
    # the cell order is the stable CPU sort of the keys
    assert np.array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))
    # partition of unity: every particle is inside the grid, so grid mass = particle mass
    assert abs(out["g_mass"].sum() - st["mass"].sum()) <= 1e-12 * st["mass"].sum()
    # the platen moved by 2 dt v (x += v dt twice: rounding of x ~ 0.04 m is ~1e-17 m per add)
    dc = st["dc_list"]
    dz = out["pos"][dc, 2] - st["pos"][dc, 2]
    assert np.allclose(dz, -2 * st.dt_max * 5.0, rtol=0, atol=1e-16)
    assert np.isfinite(out["stress"]).all()
