"""Train the learned return map on the stated sample distribution and time its inference against the exact map.

    python -m code_mpm_gb300.netbench [--train-samples N] [--epochs E] [--samples M] [--reps R]

Prints one JSON line: training report, milliseconds per call of the BF16 tcgen05 network, the FP32 network and the
exact FP32 return map on the same M samples (stress U(+-1.5 yield), R from epbar U(0, 0.2), strain increment
N(0, 2e-4); von Mises hardening steel E 200 GPa, nu 0.3, yield 250 MPa, H 2 GPa).
"""
from __future__ import annotations

import argparse
import json
import math


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-samples", type=int, default=2_000_000)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--samples", type=int, default=4 * 1024 * 1024)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--fp32", action="store_true", help="also time the FP32 network")
    a = ap.parse_args()

    import torch

    from . import build, engine

    build.build()
    net = engine.Net(n_samples=a.train_samples, epochs=a.epochs)
    rep = net.train()
    n = a.samples
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    Y = 250.0e6
    x = torch.empty((n, 13), dtype=torch.float32, device="cuda")
    x[:, :6] = (torch.rand((n, 6), generator=g, device="cuda") * 3.0 - 1.5) * Y
    ep = torch.rand((n,), generator=g, device="cuda").double() * 0.2
    x[:, 6] = (math.sqrt(2.0 / 3.0) * 1.0e12 * (1.0 - torch.exp(-2.0e-3 * ep))).float()
    x[:, 7:] = torch.randn((n, 6), generator=g, device="cuda") * 2.0e-4
    out = torch.empty((n, 7), dtype=torch.float32, device="cuda")
    kernels = [("network_tcgen05", engine.INFER_TC), ("exact_map_fp32", engine.INFER_EXACT)]
    if a.fp32:
        kernels.append(("network_fp32", engine.INFER_FP32))
    ms = {}
    for name, k in kernels:
        net.infer_device(x.data_ptr(), out.data_ptr(), n, k)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(a.reps):
            net.infer_device(x.data_ptr(), out.data_ptr(), n, k)
        e.record()
        e.synchronize()
        ms[name] = s.elapsed_time(e) / a.reps
    flops = 2 * (13 * 128 + 128 * 128 + 128 * 128 + 128 * 7)
    print(json.dumps({"samples": n, "ms_per_call": ms, "tflops_network": flops * n / (ms["network_tcgen05"] / 1e3) / 1e12,
                      "training": rep}))


if __name__ == "__main__":
    main()
