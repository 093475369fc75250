"""The learned von Mises hardening return map (include/mpm_surrogate.h).

* the training kernels' loss and gradient against the float64 CPU oracle (oracle/mlp_oracle.py);
* the BF16 tcgen05 inference kernel against the oracle's BF16 arithmetic and the FP32 kernels;
* training on samples of the exact map reduces the held-out error;
* what the network gains: its throughput and error against the exact return map on the same samples;
* in the step: clearly plastic particles go through the network, the band stays exact, rechecks are counted.
"""
import json
import os

import numpy as np
import pytest

import mlp_oracle
from code_mpm_gb300 import engine, metrics, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
MAT = dict(E=200.0e9, nu=0.3, yield_=250.0e6, C0=2.0e-3, C1=1.0e12)


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from code_mpm_gb300 import build

    build.build()
    engine.lib()


def random_params(seed=0, scale=1.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = []
    for s in mlp_oracle.SHAPES:
        fan = s[1] if len(s) == 2 else 128
        a = rng.uniform(-1, 1, size=s) * scale / np.sqrt(fan)
        if s == (128, 16):
            a[:, 13:] = 0.0
        parts.append(a.ravel())
    return np.concatenate(parts).astype(np.float32)


def samples(n, seed=1):
    """Physical inputs like the training distribution: stress U(+-1.5 yield), R, strain increment N(0, 2e-4)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Y = MAT["yield_"]
    sig = rng.uniform(-1.5, 1.5, size=(n, 6)) * Y
    ep = rng.uniform(0, 0.2, size=n)
    R = np.sqrt(2 / 3) * MAT["C1"] * (1 - np.exp(-MAT["C0"] * ep))
    de = rng.normal(0, 2e-4, size=(n, 6))
    return np.concatenate([sig, R[:, None], de], axis=1)


def test_gradient_matches_cpu_oracle():
    net = engine.Net(**MAT, n_samples=1000)
    theta = random_params(3)
    net.set_params(theta)
    rng = np.random.Generator(np.random.PCG64(5))
    n = 777
    x = np.zeros((n, 16))
    x[:, :13] = rng.normal(0, 1, size=(n, 13))
    t = np.zeros((n, 8))
    t[:, :7] = rng.normal(0, 1, size=(n, 7))
    loss_gpu, g_gpu = net.loss_grad(x, t)
    loss_ref, g_ref = mlp_oracle.loss_and_grad(theta.astype(np.float64), x.astype(np.float32).astype(np.float64),
                                               t.astype(np.float32).astype(np.float64))
    assert abs(loss_gpu - loss_ref) <= 1e-5 * abs(loss_ref)
    o = 0
    for s in mlp_oracle.SHAPES:
        k = int(np.prod(s))
        a, b = g_gpu[o:o + k].astype(np.float64), g_ref[o:o + k]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b) + 1e-12, (s, np.linalg.norm(a - b) / np.linalg.norm(b))
        o += k


def _infer(net, x_phys, kernel):
    d_in = torch.tensor(x_phys, dtype=torch.float32, device="cuda").contiguous()
    d_out = torch.zeros((x_phys.shape[0], 7), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    net.infer_device(d_in.data_ptr(), d_out.data_ptr(), x_phys.shape[0], kernel)
    torch.cuda.synchronize()
    return d_out.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("n", [128, 1000, 70001])
def test_tcgen05_inference_matches_bf16_oracle_and_fp32(n):
    net = engine.Net(**MAT, n_samples=1000)
    theta = random_params(11, scale=2.0)
    net.set_params(theta)
    x = samples(n, seed=n)
    in_scale, out_scale, out_shift = net.scales()
    y_tc = _infer(net, x, engine.INFER_TC)
    y_32 = _infer(net, x, engine.INFER_FP32)
    xn = np.zeros((n, 16))
    xn[:, :13] = (x.astype(np.float32) * (1.0 / in_scale).astype(np.float32)).astype(np.float64)
    pred = np.zeros((n, 7))
    pred[:, :6] = mlp_oracle.elastic_predictor(x[:, 7:], MAT["E"], MAT["nu"])  # the kernels add D de
    y_ref = mlp_oracle.forward_bf16(theta.astype(np.float64), xn)[:, :7] * out_scale + out_shift + pred
    y_f64, _ = mlp_oracle.forward(theta.astype(np.float64), xn)
    y_f64 = y_f64[:, :7] * out_scale + out_shift + pred
    scale = np.sqrt(np.mean(y_f64 ** 2))
    # FP32 kernels: float rounding only
    assert np.abs(y_32 - y_f64).max() <= 1e-4 * scale
    # tensor cores: BF16 operands (8-bit significands), FP32 sums, BF16 activations
    rms = np.sqrt(np.mean((y_tc - y_ref) ** 2))
    assert rms <= 1e-2 * scale, rms / scale
    assert np.abs(y_tc - y_ref).max() <= 8e-2 * scale
    assert np.sqrt(np.mean((y_tc - y_f64) ** 2)) <= 3e-2 * scale


def _train(n_samples, epochs, seed=7, **kw):
    net = engine.Net(**MAT, n_samples=n_samples, epochs=epochs, seed=seed, **kw)
    rep = net.train()
    return net, rep


def test_training_reduces_held_out_error():
    net, rep = _train(2_000_000, 3)
    assert rep["steps"] == (2_000_000 // 65536) * 3
    assert rep["loss_last"] < 0.2 * rep["loss_first"], rep
    assert rep["val_rms_dsig_outside"] < 0.2, rep  # dstress / yield, after 3 short epochs
    y = samples(4096, seed=9)
    ex = _infer(net, y, engine.INFER_EXACT)
    ds, dR, f = mlp_oracle.vmh_return_map(y[:, :6], y[:, 6], y[:, 7:], MAT["E"], MAT["nu"], MAT["yield_"], MAT["C0"],
                                          MAT["C1"])
    # the FP32 exact kernel (the method without the network) agrees with the float64 restatement
    assert np.abs(ex[:, :6] - ds).max() <= 1e-5 * MAT["yield_"] * 10
    assert np.abs(ex[:, 6] - dR).max() <= 1e-5 * MAT["yield_"]


def test_what_the_network_gains(tmp_path):
    """Time the network (tensor cores and FP32) and the exact FP32 map on the same 4M samples and compare their
    dstress.  The record is printed and written beside the test's temporaries; the assertions only check that each
    path ran and that the network's error outside the band is that of its training."""
    net, rep = _train(4_000_000, 4)
    n = 4_000_000
    x = samples(n, seed=21)
    d_in = torch.tensor(x, dtype=torch.float32, device="cuda").contiguous()
    outs = {}
    times = {}
    for name, k in (("network_tcgen05", engine.INFER_TC), ("network_fp32", engine.INFER_FP32),
                    ("exact_map_fp32", engine.INFER_EXACT)):
        d_out = torch.zeros((n, 7), dtype=torch.float32, device="cuda")
        for _ in range(2):
            net.infer_device(d_in.data_ptr(), d_out.data_ptr(), n, k)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        reps = 5
        for _ in range(reps):
            net.infer_device(d_in.data_ptr(), d_out.data_ptr(), n, k)
        b.record()
        b.synchronize()
        times[name] = a.elapsed_time(b) / reps
        outs[name] = d_out.cpu().numpy().astype(np.float64)
    ds, dR, f = mlp_oracle.vmh_return_map(x[:, :6], x[:, 6], x[:, 7:], MAT["E"], MAT["nu"], MAT["yield_"], MAT["C0"],
                                          MAT["C1"])
    k0 = MAT["yield_"] / np.sqrt(3)
    outside = f >= 0.02 * k0
    err = {k: float(np.sqrt(np.mean(((v[outside, :6] - ds[outside]) / MAT["yield_"]) ** 2))) for k, v in outs.items()}
    rec = {"samples": n, "ms_per_call": times, "samples_per_s": {k: n / (v / 1e3) for k, v in times.items()},
           "network_over_exact_speed": times["exact_map_fp32"] / times["network_tcgen05"],
           "rms_dsig_over_yield_outside_band": err, "fraction_outside_band": float(outside.mean()), "training": rep}
    print(json.dumps(rec))
    (tmp_path / "network_gain.json").write_text(json.dumps(rec))
    assert all(t > 0 for t in times.values())
    assert err["exact_map_fp32"] <= 1e-5
    assert err["network_tcgen05"] <= 0.1 and err["network_fp32"] <= 0.1


def harvest(st, steps, cap=4_000_000):
    """Return-map inputs the plain FP64 method meets on a run of st (device rows, count)."""
    rows = torch.zeros((cap, 13), dtype=torch.float32, device="cuda")
    with engine.Engine.from_state(st, engine.FORM_FP64) as e:
        e.set_option(engine.OPT_FLOOR_FRICTION, 1)
        e.harvest_begin(rows.data_ptr(), cap, mat_mask=1, band=0.0)
        e.advance(steps, st.dt_max, True)
        n = min(e.harvest_end(), cap)
    return rows, n


def test_harvest_leaves_the_run_unchanged():
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0)
    outs = []
    for on in (False, True):
        rows = torch.zeros((100000, 13), dtype=torch.float32, device="cuda")
        with engine.Engine.from_state(st, engine.FORM_FP64) as e:
            if on:
                e.harvest_begin(rows.data_ptr(), rows.shape[0], mat_mask=1, band=0.0)
            e.advance(20, st.dt_max, True)
            n = e.harvest_end()
            outs.append(e.download_state(st))
    assert n > 0
    for k in ("pos", "vel", "stress"):  # the same run up to the order of atomic sums
        scale = np.abs(outs[0][k]).max()
        assert np.abs(outs[0][k] - outs[1][k]).max() <= 1e-12 * scale, k
    r = rows[:min(n, rows.shape[0])].cpu().numpy().astype(np.float64)
    ds, dR, f = mlp_oracle.vmh_return_map(r[:, :6], r[:, 6], r[:, 7:], MAT["E"], MAT["nu"], MAT["yield_"], MAT["C0"],
                                          MAT["C1"])
    assert (f >= -1e-3 * MAT["yield_"]).all()  # only plastic trial states (float rounding aside)


def test_network_in_the_step():
    """A network trained on the return-map inputs the plain method meets in a pilot run (platen at 15 m/s) runs in
    the step of another (20 m/s): clearly plastic particles go through it, the band stays exact, rechecks are kept."""
    pilot = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=15.0)
    rows, n = harvest(pilot, 150)
    dsig = float(rows[:n, 7:].std().item())
    net = engine.Net(**MAT, n_samples=1000, epochs=40, batch=8192, deps_sigma=dsig, lr=4.0e-3)
    rep = net.train_rows(rows.data_ptr(), n)
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0)
    steps = 60
    ref = st.copy()
    import pyoracle

    pyoracle.advance(ref, steps, 1, floor_friction=1)
    outs = {}
    for use in (False, True):
        with engine.Engine.from_state(st, engine.FORM_FP32) as e:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
            if use:
                e.attach_surrogate(net, band=0.02, recheck=0.01)
            e.advance(steps, st.dt_max, True)
            outs[use] = e.download_state(st)
            if use:
                stats = e.surrogate_stats()
    assert stats["queued"] > 0 and stats["rechecked"] > 0, stats
    err_net = metrics.form_errors(outs[True], ref)
    err_exact = metrics.form_errors(outs[False], ref)
    print(json.dumps({"harvested_rows": n, "training": rep, "with_network": err_net, "exact": err_exact,
                      "stats": stats}))
    assert err_exact["vm_stress_rel_l2"] <= 1e-3
    # the chosen form's bars hold with the network in the loop
    assert err_net["vm_stress_rel_l2"] <= 1e-2 and err_net["strain_energy_rel"] <= 5e-3, err_net


def test_guard_replaces_implausible_network_results():
    """A network with random weights (its results are not radial returns) in the step: the guard rejects every
    result and the exact FP64 map takes its place, so the run equals the run without the network (the same
    FP64 map, applied by the finishing kernel instead of pass 2: equal to float rounding); with the guard off
    (MPM_OPT_SURROGATE_GUARD 0) the same network leaves the queued particles off the yield surface."""
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0)
    net = engine.Net(**MAT, n_samples=1000)
    net.set_params(random_params(11))
    steps = 40
    outs = {}
    for mode in ("none", "guard", "off"):
        with engine.Engine.from_state(st, engine.FORM_FP32) as e:
            e.set_option(engine.OPT_FLOOR_FRICTION, 1)
            if mode != "none":
                e.attach_surrogate(net, band=0.02, recheck=0.01)
            if mode == "off":
                e.set_option(engine.OPT_SURROGATE_GUARD, 0.0)
            e.advance(steps, st.dt_max, True)
            outs[mode] = e.download_state(st)
            if mode == "guard":
                stats = e.surrogate_stats()
    assert stats["queued"] > 0 and stats["rejected"] == stats["queued"], stats
    for k in ("pos", "vel", "stress", "backstress", "e_strain", "e_plastic"):
        scale = np.abs(outs["none"][k]).max()
        assert np.abs(outs["guard"][k] - outs["none"][k]).max() <= 1e-6 * scale, k
    scale = np.abs(outs["none"]["stress"]).max()
    assert np.abs(outs["off"]["stress"] - outs["none"]["stress"]).max() > 1e-3 * scale
    net.close()
