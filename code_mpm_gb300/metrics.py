"""Error measures between two states of the same scene (chosen form vs FP64 reference)."""
from __future__ import annotations

from typing import Dict

import numpy as np

from .snapshot import State


def von_mises(stress: np.ndarray) -> np.ndarray:
    """Von Mises equivalent stress of Voigt stresses (xx, yy, zz, xy, yz, zx), n x 6."""
    s = np.asarray(stress, dtype=np.float64)
    return np.sqrt(0.5 * ((s[:, 0] - s[:, 1]) ** 2 + (s[:, 1] - s[:, 2]) ** 2 + (s[:, 2] - s[:, 0]) ** 2) +
                   3.0 * (s[:, 3] ** 2 + s[:, 4] ** 2 + s[:, 5] ** 2))


def form_errors(out: State, ref: State) -> Dict[str, float]:
    """Normwise errors of `out` against `ref`: von Mises stress (max-norm and relative L2 over the particles),
    strain and plastic energy, positions, velocity."""
    vo, vr = von_mises(out["stress"]), von_mises(ref["stress"])
    vmax = float(vr.max()) if vr.size else 0.0
    vl2 = float(np.linalg.norm(vr))
    es_o, es_r = float(np.sum(out["e_strain"])), float(np.sum(ref["e_strain"]))
    ep_o, ep_r = float(np.sum(out["e_plastic"])), float(np.sum(ref["e_plastic"]))
    vel_scale = float(np.abs(ref["vel"]).max()) if ref["vel"].size else 0.0
    return {
        "vm_stress_rel": float(np.abs(vo - vr).max() / vmax) if vmax > 0 else 0.0,
        "vm_stress_rel_l2": float(np.linalg.norm(vo - vr) / vl2) if vl2 > 0 else 0.0,
        "strain_energy_rel": abs(es_o - es_r) / abs(es_r) if es_r != 0 else abs(es_o),
        "plastic_energy_rel": abs(ep_o - ep_r) / abs(ep_r) if ep_r != 0 else abs(ep_o),
        "pos_abs_max": float(np.abs(out["pos"] - ref["pos"]).max()) if ref["pos"].size else 0.0,
        "vel_rel": float(np.abs(out["vel"] - ref["vel"]).max() / vel_scale) if vel_scale > 0 else 0.0,
    }
