"""GPU console monitors against a restatement of PhysicsEngine::reportConsole (PhysicsEngine.cpp:40-183).

The expected values are computed from the oracle's state after the same steps
(sums in FP64; the GPU reduction order differs, so sums agree to 1e-12
relative, maxima and counts exactly where the inputs agree).
"""
import numpy as np
import pytest

import pyoracle
from code_mpm_gb300 import engine, scenes

pytestmark = pytest.mark.gpu


def principal_abs_max(s):
    """getPrincipal (ConstitutiveRelation_calculateState.cpp:160-196), max |value|; NaN rows and Q > 0 give 0."""
    s = np.asarray(s, dtype=np.float64)
    I1 = s[:, 0] + s[:, 1] + s[:, 2]
    I2 = s[:, 0] * s[:, 1] + s[:, 1] * s[:, 2] + s[:, 0] * s[:, 2] - s[:, 3] ** 2 - s[:, 4] ** 2 - s[:, 5] ** 2
    m = np.stack([s[:, 0], s[:, 3], s[:, 5], s[:, 3], s[:, 1], s[:, 4], s[:, 5], s[:, 4], s[:, 2]], 1)
    I3 = (m[:, 0] * (m[:, 4] * m[:, 8] - m[:, 7] * m[:, 5]) - m[:, 3] * (m[:, 1] * m[:, 8] - m[:, 7] * m[:, 2]) +
          m[:, 6] * (m[:, 1] * m[:, 5] - m[:, 4] * m[:, 2]))
    Q = (3.0 * I2 - I1 * I1) / 9.0
    R = (2.0 * I1 ** 3 - 9.0 * I1 * I2 + 27.0 * I3) / 54.0
    with np.errstate(all="ignore"):
        T = np.clip(R / np.sqrt(-Q * Q * Q), -1.0, 1.0)
        th = np.arccos(T)
        pi = 3.14159265359
        vals = np.stack([np.abs(2.0 * np.sqrt(-Q) * np.cos((th + 2.0 * k * pi) / 3.0) + I1 / 3.0) for k in range(3)], 1)
    vals[~np.isfinite(vals)] = 0.0
    vals[Q > 0] = 0.0
    return vals.max(1)


@pytest.mark.parametrize("contact", [0, 1])
def test_monitors_match_report_console(contact):
    st = scenes.contact_small(seed=5) if contact else scenes.mixed_small(seed=6)
    rng = np.random.Generator(np.random.PCG64(7))
    mask = rng.integers(0, 32, size=st.n_particles).astype(np.uint8)
    ref = st.copy()
    pyoracle.advance(ref, 8, contact)
    with engine.Engine.from_state(st) as e:
        e.upload_monitor_mask(mask)
        e.advance(8, st.dt_max, bool(contact))
        mon = e.monitors()
    sel = lambda bit: (mask & bit) > 0  # noqa: E731
    d = sel(engine.MON_DISPLACEMENT)
    assert mon["count"] == [int(sel(b).sum()) for b in (1, 2, 4, 8, 16)]
    np.testing.assert_allclose(mon["position_mean"], ref["pos"][d].mean(0), rtol=1e-12)
    np.testing.assert_allclose(mon["force_sum"], ref["g_force_temp"].sum(0), rtol=1e-9, atol=1e-9)
    mm = sel(engine.MON_MOMENTUM)
    np.testing.assert_allclose(mon["momentum"], (ref["vel"][mm] * ref["mass"][mm, None]).sum(0), rtol=1e-9,
                               atol=1e-15)
    pp = sel(engine.MON_PRINCIPAL)
    np.testing.assert_allclose(mon["stress_p_max"], principal_abs_max(ref["stress"][pp]).max(), rtol=1e-9)
    np.testing.assert_allclose(mon["strain_p_max"], principal_abs_max(ref["strain"][pp]).max(), rtol=1e-9)
    ss = sel(engine.MON_STRESS)
    np.testing.assert_allclose(mon["stress_mean"], ref["stress"][ss, :3].mean(0), rtol=1e-9, atol=1e-3)
    np.testing.assert_allclose(mon["strain_mean"], ref["strain"][ss, :3].mean(0), rtol=1e-9, atol=1e-18)
    ee = sel(engine.MON_ENERGY)
    ke = (0.5 * ref["mass"][ee] * np.linalg.norm(ref["vel"][ee], axis=1) ** 2).sum()
    np.testing.assert_allclose(mon["kinetic"], ke, rtol=1e-9)
    np.testing.assert_allclose(mon["strain_energy"], ref["e_strain"][ee].sum(), rtol=1e-9)
    np.testing.assert_allclose(mon["plastic_energy"], ref["e_plastic"][ee].sum(), rtol=1e-9, atol=1e-20)


@pytest.mark.parametrize("contact", [0, 1])
def test_boundary_work_matches_restatement(contact):
    """Platen (displacement-control) and friction work against the oracle's restatement of the same sums
    (oracle/mpm_oracle.c, dc_work_* and friction_work): FP64 form to summation order, FP32 form to 1e-4."""
    if contact:
        st = scenes.platen_block(size=(0.01, 0.01, 0.006), speed=20.0)  # floor friction 0.1, platen at 20 m/s
    else:
        st = scenes.mixed_small(seed=6)  # platen particles on the list, x-wall friction
    steps = 40
    ref = st.copy()
    w = pyoracle.advance_work(ref, steps, contact, floor_friction=1)
    assert w[0] != 0.0
    for form, rtol in ((engine.FORM_FP64, 1e-9), (engine.FORM_FP32, 1e-4)):
        with engine.Engine.from_state(st, form) as e:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
            e.upload_monitor_mask(np.full(st.n_particles, 31, dtype=np.uint8))
            e.advance(steps, st.dt_max, bool(contact))
            mon = e.monitors()
        np.testing.assert_allclose(mon["platen_work"], w[0], rtol=rtol)
        np.testing.assert_allclose(mon["friction_work"], w[1], rtol=rtol, atol=rtol * abs(w[0]))
    if contact:
        assert w[1] < 0.0  # the floor friction dissipates
