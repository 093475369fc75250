"""The network's CPU oracle (oracle/mlp_oracle.py) pinned on its own: central finite differences of the loss
against its analytic gradient, and the return map restatement against the von Mises hardening invariants
(ConstitutiveRelation_calculateIncrement_VonMisesHardening.cpp:4-92): a plastic state returns onto the yield
surface k0 + R/sqrt 2, an elastic one gets D de, dR follows the hardening law."""
import numpy as np

import mlp_oracle


def test_gradient_by_finite_differences():
    rng = np.random.Generator(np.random.PCG64(0))
    theta = rng.normal(0, 0.2, size=mlp_oracle.N_PARAMS)
    x = np.zeros((9, 16))
    x[:, :13] = rng.normal(size=(9, 13))
    t = rng.normal(size=(9, 8))
    _, g = mlp_oracle.loss_and_grad(theta, x, t)
    for i in rng.choice(mlp_oracle.N_PARAMS, size=60, replace=False):
        h = 1e-6
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (mlp_oracle.loss_and_grad(tp, x, t)[0] - mlp_oracle.loss_and_grad(tm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_return_map_invariants():
    rng = np.random.Generator(np.random.PCG64(1))
    E, nu, Y, C0, C1 = 200e9, 0.3, 250e6, 2e-3, 1e12
    n = 2000
    sig = rng.uniform(-1.5, 1.5, size=(n, 6)) * Y
    R = rng.uniform(0, 0.3, size=n) * Y
    de = rng.normal(0, 2e-4, size=(n, 6))
    ds, dR, f = mlp_oracle.vmh_return_map(sig, R, de, E, nu, Y, C0, C1)
    s = sig + ds
    J2 = ((s[:, 0] - s[:, 1]) ** 2 + (s[:, 1] - s[:, 2]) ** 2 + (s[:, 2] - s[:, 0]) ** 2) / 6 + (s[:, 3:] ** 2).sum(1)
    rad = Y / np.sqrt(3) + R / np.sqrt(2)
    pl = f > 0
    assert pl.any() and (~pl).any()
    np.testing.assert_allclose(np.sqrt(J2[pl]), rad[pl], rtol=1e-12)
    C = E / (1 + nu) / (1 - 2 * nu)
    D = np.zeros((6, 6))
    D[:3, :3] = C * nu
    np.fill_diagonal(D[:3, :3], C * (1 - nu))
    D[3:, 3:] = np.eye(3) * C * (0.5 - nu)
    np.testing.assert_allclose(ds[~pl], de[~pl] @ D.T, rtol=1e-12, atol=1e-6)
    assert (dR[~pl] == 0).all() and (dR[pl] >= 0).all()
