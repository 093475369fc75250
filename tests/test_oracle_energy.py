"""The boundary-work restatement closes the energy balance of the oracle's own runs (no GPU).

Kinetic + strain energy of the specimen (the strain energy is the stress work, plastic dissipation included)
minus its initial value equals the platen's work plus the friction work up to the method's own error, which is
a small fraction of the work done, and is positive work into the specimen.
"""
import numpy as np

import pyoracle
from code_mpm_gb300 import scenes


def _energy(st, mask):
    return float(0.5 * np.sum(st["mass"][mask] * np.sum(st["vel"][mask] ** 2, axis=1)) + np.sum(st["e_strain"][mask]))


def test_platen_crush_energy_balance():
    st = scenes.platen_block(size=(0.012, 0.012, 0.008), speed=20.0)
    mask = (st["pflags"] & 8) == 0  # the specimen, without the platen
    e0 = _energy(st, mask)
    w = pyoracle.advance_work(st, 300, 1, floor_friction=1)
    resid = _energy(st, mask) - e0 - w[0] - w[1]
    assert w[0] > 0.0 and w[1] < 0.0
    assert abs(resid) < 0.05 * w[0], (resid, w)


def test_free_bar_conserves_energy():
    st = scenes.bar(cells_len=12, cells_w=4)
    mask = np.ones(st.n_particles, dtype=bool)
    e0 = _energy(st, mask)
    w = pyoracle.advance_work(st, 400, 0)
    assert w == [0.0, 0.0]  # a fixed end does no work
    assert abs(_energy(st, mask) - e0) < 0.02 * e0
