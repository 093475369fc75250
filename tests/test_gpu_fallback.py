"""The chosen form's FP64 fallback: von Mises hardening particles near or past the yield surface that the
network does not take run the exact return map (…_VonMisesHardening.cpp:4-92) in FP64 on their FP32 state.

* the FP64 map kernel (the fallback's arithmetic, cr_increment_wide) against the float64 restatement of the map
  in oracle/mlp_oracle.py, outputs rounded to float: equal to float rounding;
* in an FP32 step, every plastic particle's new stress and back stress are its FP32 state plus the FP64
  increment rounded to float (inputs harvested in the same step), and MPM_OPT_FP64_FALLBACK 0 changes them.
"""
import numpy as np
import pytest

import mlp_oracle
from code_mpm_gb300 import engine, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
MAT = dict(E=200.0e9, nu=0.3, yield_=250.0e6, C0=2.0e-3, C1=1.0e12)


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from code_mpm_gb300 import build

    build.build()
    engine.lib()


def _rows_near_surface(n, seed=3):
    """Inputs whose trial states straddle the yield surface (the fallback band and beyond)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Y, k0 = MAT["yield_"], MAT["yield_"] / np.sqrt(3.0)
    dev = rng.normal(size=(n, 6))
    dev[:, :3] -= dev[:, :3].mean(1, keepdims=True)
    j2 = ((dev[:, 0] - dev[:, 1]) ** 2 + (dev[:, 1] - dev[:, 2]) ** 2 + (dev[:, 2] - dev[:, 0]) ** 2) / 6.0 + \
        (dev[:, 3:] ** 2).sum(1)
    ep = rng.uniform(0, 0.05, size=n)
    R = np.sqrt(2 / 3) * MAT["C1"] * (1 - np.exp(-MAT["C0"] * ep))
    rad = k0 + R / np.sqrt(2.0)
    sig = dev * (rng.uniform(0.9, 1.02, size=n) * rad / np.sqrt(j2))[:, None]
    sig[:, :3] += rng.uniform(-1, 1, size=(n, 1)) * Y
    de = rng.normal(0, 1e-4, size=(n, 6))
    return np.concatenate([sig, R[:, None], de], axis=1).astype(np.float32)


def _infer(net, x32, kernel):
    d_in = torch.tensor(x32, device="cuda").contiguous()
    d_out = torch.zeros((x32.shape[0], 7), dtype=torch.float32, device="cuda")
    net.infer_device(d_in.data_ptr(), d_out.data_ptr(), x32.shape[0], kernel)
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


def _ulps(a, b):
    a = np.asarray(a, dtype=np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, dtype=np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def test_fp64_map_kernel_equals_float64_restatement():
    net = engine.Net(**MAT, n_samples=1000)
    x = _rows_near_surface(200_000)
    wide = _infer(net, x, engine.INFER_EXACT_FP64)
    fp32 = _infer(net, x, engine.INFER_EXACT)
    x64 = x.astype(np.float64)
    ds, dR, f = mlp_oracle.vmh_return_map(x64[:, :6], x64[:, 6], x64[:, 7:], **MAT)
    want = np.concatenate([ds, dR[:, None]], axis=1).astype(np.float32)
    plastic = f > 0
    assert 0.2 < plastic.mean() < 0.8
    # the FP64 map rounded once: equal to the float64 restatement rounded, up to the last bit of a few outputs
    # (the two differ in association order far below float resolution)
    u = _ulps(wide, want)
    assert u.max() <= 1 and (u > 0).mean() < 1e-3, (u.max(), (u > 0).mean())
    # the FP32 map is measurably less exact on the plastic rows
    u32 = _ulps(fp32[plastic], want[plastic])
    assert u32.max() > 4
    net.close()


def _state_arrays(e, n):
    out = {"stress": np.empty((n, 6)), "backstress": np.empty(n)}
    e.download_particles(out)
    return out


def _one_step_with_inputs(st, fallback):
    """60 steps into plastic flow, then one step whose plastic particles' return-map inputs are harvested:
    (harvested rows, the particle of each row, state after the step)."""
    n = st.n_particles
    with engine.Engine.from_state(st, engine.FORM_FP32) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.set_option(engine.OPT_FP64_FALLBACK, fallback)
        e.advance(60, st.dt_max, True)
        before = _state_arrays(e, n)
        rows = torch.zeros((n, 13), dtype=torch.float32, device="cuda")
        e.harvest_begin(rows.data_ptr(), n, mat_mask=1, band=0.0)  # plastic trial states of the next step
        e.advance(1, st.dt_max, True)
        k = min(e.harvest_end(), n)
        after = _state_arrays(e, n)
        r = rows[:k].cpu().numpy()
    assert k > 100
    # harvested inputs -> particle, by its (unique) stress before the step
    key = {}
    for i in range(n):
        key.setdefault(before["stress"][i].astype(np.float32).tobytes(), []).append(i)
    idx = np.array([(lambda v: v[0] if v and len(v) == 1 else -1)(key.get(r[j, :6].tobytes())) for j in range(k)])
    ok = idx >= 0
    assert ok.mean() > 0.9
    return r[ok].astype(np.float64), idx[ok], after


def _expected(r):
    ds, dR, f = mlp_oracle.vmh_return_map(r[:, :6], r[:, 6], r[:, 7:], **MAT)
    # the kernel adds the FP64 increment, rounded to float, to the float state in float arithmetic
    return r[:, :6].astype(np.float32) + ds.astype(np.float32), r[:, 6].astype(np.float32) + dR.astype(np.float32)


def test_plastic_particles_take_the_fp64_map_in_the_step():
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0)
    r, idx, after = _one_step_with_inputs(st, 1)
    want_sig, want_R = _expected(r)
    assert _ulps(after["stress"][idx], want_sig).max() <= 1
    assert _ulps(after["backstress"][idx], want_R).max() <= 1
    # with the fallback off the step runs the FP32 map: its plastic particles miss the FP64 result
    r0, idx0, after0 = _one_step_with_inputs(st, 0)
    want_sig0, _ = _expected(r0)
    assert np.any(_ulps(after0["stress"][idx0], want_sig0) > 1)
