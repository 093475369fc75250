"""CPU oracle for the return-map surrogate network (test infrastructure only).

Only tests and the bench's checks use this file.  It restates the network
that code_mpm_gb300/csrc/surrogate.cu trains and runs, in float64 numpy:
13 inputs padded to 16, three hidden layers of 128 with ReLU, 8 outputs
(7 used).  The weight layout is the kernels' own: W[out][in] row-major,
packed as W1, b1, W2, b2, W3, b3, W4, b4.  Inputs and targets are in the
network's normalised units (the caller applies the scalings).

It also restates the von Mises hardening return map in the form the
surrogate learns (ConstitutiveRelation_calculateIncrement_VonMisesHardening.cpp:4-92):
inputs (stress[6], R, strain increment[6]), outputs (dstress[6], dR).
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 16, 128, 8
SHAPES = [(HID, IN), (HID,), (HID, HID), (HID,), (HID, HID), (HID,), (OUT, HID), (OUT,)]
N_PARAMS = int(sum(np.prod(s) for s in SHAPES))


def unpack(theta):
    out, o = [], 0
    for s in SHAPES:
        k = int(np.prod(s))
        out.append(np.asarray(theta[o:o + k], dtype=np.float64).reshape(s))
        o += k
    return out


def relu(z):
    return np.maximum(z, 0.0)


def drelu(z):
    return (z > 0.0).astype(np.float64)


def forward(theta, x):
    """x: n x 16 -> (y n x 8, cache)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(theta)
    z1 = x @ W1.T + b1
    h1 = relu(z1)
    z2 = h1 @ W2.T + b2
    h2 = relu(z2)
    z3 = h2 @ W3.T + b3
    h3 = relu(z3)
    y = h3 @ W4.T + b4
    return y, (x, z1, h1, z2, h2, z3, h3)


def loss_and_grad(theta, x, t, used=7):
    """Mean over samples and the `used` outputs of (y - t)^2, and its gradient in the packed layout."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(theta)
    y, (x, z1, h1, z2, h2, z3, h3) = forward(theta, x)
    n = x.shape[0]
    d = np.zeros_like(y)
    d[:, :used] = y[:, :used] - t[:, :used]
    loss = float(np.sum(d * d) / (n * used))
    dy = 2.0 * d / (n * used)
    gW4, gb4 = dy.T @ h3, dy.sum(0)
    dz3 = (dy @ W4) * drelu(z3)
    gW3, gb3 = dz3.T @ h2, dz3.sum(0)
    dz2 = (dz3 @ W3) * drelu(z2)
    gW2, gb2 = dz2.T @ h1, dz2.sum(0)
    dz1 = (dz2 @ W2) * drelu(z1)
    gW1, gb1 = dz1.T @ x, dz1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4)])
    return loss, g


def bf16(a):
    """Round float64 values to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_bf16(theta, x):
    """The inference kernel's arithmetic: bf16 weights, biases and activations, exact products, float sums (the
    hidden biases are summed with the products); each hidden layer's sum through ReLU, rounded to bf16 once."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(theta)
    h = bf16(x)
    for W, b in ((W1, b1), (W2, b2), (W3, b3)):
        h = bf16(relu(h @ bf16(W).T + bf16(b)))
    return h @ bf16(W4).T + b4


def elastic_predictor(deps, E, nu):
    """D de (isotropic, Voigt engineering shear; …_Elastic.cpp:4-18)."""
    C = E / (1.0 + nu) / (1.0 - 2.0 * nu)
    e = deps
    d = np.empty_like(e)
    d[:, 0] = C * ((1.0 - nu) * e[:, 0] + nu * e[:, 1] + nu * e[:, 2])
    d[:, 1] = C * ((1.0 - nu) * e[:, 1] + nu * e[:, 0] + nu * e[:, 2])
    d[:, 2] = C * ((1.0 - nu) * e[:, 2] + nu * e[:, 0] + nu * e[:, 1])
    d[:, 3:] = C * ((0.5 - nu) * e[:, 3:])
    return d


def vmh_return_map(sig, R, deps, E, nu, yield_, C0, C1):
    """Closed-form radial return with explicit saturating hardening, vectorised over rows."""
    C = E / (1.0 + nu) / (1.0 - 2.0 * nu)
    a, hb = 1.0 - nu, 0.5 - nu
    e = deps
    d = np.empty_like(e)
    d[:, 0] = C * (a * e[:, 0] + nu * e[:, 1] + nu * e[:, 2])
    d[:, 1] = C * (a * e[:, 1] + nu * e[:, 0] + nu * e[:, 2])
    d[:, 2] = C * (a * e[:, 2] + nu * e[:, 0] + nu * e[:, 1])
    d[:, 3:] = C * (hb * e[:, 3:])
    tr = sig + d
    hyd = (tr[:, 0] + tr[:, 1] + tr[:, 2]) / 3.0
    J2 = ((tr[:, 0] - tr[:, 1]) ** 2 + (tr[:, 1] - tr[:, 2]) ** 2 + (tr[:, 2] - tr[:, 0]) ** 2) / 6.0 + \
        (tr[:, 3:] ** 2).sum(1)
    rad = yield_ / np.sqrt(3.0) + R / np.sqrt(2.0)
    plastic = J2 > rad * rad
    sc = np.where(plastic, rad / np.sqrt(np.maximum(J2, 1e-300)), 1.0)
    dev = tr.copy()
    dev[:, :3] -= hyd[:, None]
    dsig = np.where(plastic[:, None], dev * sc[:, None] - sig, d)
    dsig[:, :3] += np.where(plastic, hyd, 0.0)[:, None]
    G = 0.5 * E / (1.0 + nu)
    ee = np.empty_like(dsig)
    ee[:, 0] = dsig[:, 0] / E - dsig[:, 1] * nu / E - dsig[:, 2] * nu / E
    ee[:, 1] = dsig[:, 1] / E - dsig[:, 0] * nu / E - dsig[:, 2] * nu / E
    ee[:, 2] = dsig[:, 2] / E - dsig[:, 0] * nu / E - dsig[:, 1] * nu / E
    ee[:, 3:] = dsig[:, 3:] / G
    deps_p = np.where(plastic[:, None], e - ee, 0.0)
    ep = np.sqrt((deps_p ** 2).sum(1) * 2.0 / 3.0)
    sat = np.sqrt(2.0 / 3.0) * C1 - R
    dR = np.where(plastic & (sat > 0), C0 * sat * ep, 0.0)
    ftrial = np.sqrt(J2) - rad
    return dsig, dR, ftrial
